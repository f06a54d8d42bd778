// A complex-double type for the complex-step build of the FP64 path
// (the role of the reference's complexified build, libidwarp_cs, that
// idwarp/UnstructuredMesh_C.py loads).
//
// Arithmetic follows the usual complex rules; comparisons, as in a
// complexified Fortran code, look at real parts only (re()).  The elementary
// functions are the ones the nodal properties use:
//   sqrt  principal square root, t = sqrt((|x| + |z|) / 2) with |z| from
//         hypot; for x >= 0 the result is t + i y / (2 t), for x < 0
//         |y| / (2 t) + i sign(y) t;
//   acos  acos(x) - i y / sqrt(1 - x^2): the first-order analytic
//         continuation, which is what a complex step with an imaginary part
//         of 1e-40 can resolve (the closed form -i log(z + i sqrt(1 - z^2))
//         loses the imaginary part to rounding: |z + i sqrt(1 - z^2)| = 1 +
//         O(y) rounds to 1);
//   sin, cos  sin x cosh y + i cos x sinh y, cos x cosh y - i sin x sinh y;
//   division  Smith's algorithm (R. L. Smith, CACM 5(8), 1962), scaling by
//         the larger of |c|, |d| of the divisor c + i d.
#pragma once
#include <cmath>
#ifndef __CUDACC__
// compiled as plain C++ (the host check of these functions)
#define __host__
#define __device__
#endif

namespace idw {

struct cplx {
    double re, im;
    __host__ __device__ cplx() : re(0.0), im(0.0) {}
    __host__ __device__ cplx(double r) : re(r), im(0.0) {}
    __host__ __device__ cplx(double r, double i) : re(r), im(i) {}
};

__host__ __device__ inline cplx operator+(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ inline cplx operator-(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ inline cplx operator-(cplx a) { return {-a.re, -a.im}; }
__host__ __device__ inline cplx operator*(cplx a, cplx b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__host__ __device__ inline cplx operator*(double s, cplx a) { return {s * a.re, s * a.im}; }
__host__ __device__ inline cplx operator*(cplx a, double s) { return {a.re * s, a.im * s}; }
__host__ __device__ inline cplx operator/(cplx a, double s) { return {a.re / s, a.im / s}; }
__host__ __device__ inline cplx operator/(cplx a, cplx b) {
    if (fabs(b.re) >= fabs(b.im)) {
        const double r = b.im / b.re, d = b.re + b.im * r;
        return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
    }
    const double r = b.re / b.im, d = b.re * r + b.im;
    return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}
__host__ __device__ inline cplx operator/(double s, cplx b) { return cplx(s) / b; }
__host__ __device__ inline cplx &operator+=(cplx &a, cplx b) {
    a = a + b;
    return a;
}
__host__ __device__ inline cplx &operator-=(cplx &a, cplx b) {
    a = a - b;
    return a;
}
__host__ __device__ inline cplx &operator/=(cplx &a, double s) {
    a = a / s;
    return a;
}
__host__ __device__ inline cplx &operator/=(cplx &a, cplx b) {
    a = a / b;
    return a;
}

// real part (the value comparisons use)
__host__ __device__ inline double re(double x) { return x; }
__host__ __device__ inline double re(cplx z) { return z.re; }

__host__ __device__ inline double sqrt_(double x) { return sqrt(x); }
__host__ __device__ inline cplx sqrt_(cplx z) {
    if (z.re == 0.0 && z.im == 0.0) return cplx(0.0, 0.0);
    const double t = sqrt(0.5 * (fabs(z.re) + hypot(z.re, z.im)));
    if (z.re >= 0.0) return cplx(t, z.im / (2.0 * t));
    return cplx(fabs(z.im) / (2.0 * t), z.im < 0.0 ? -t : t);
}

__host__ __device__ inline double acos_(double x) { return acos(x); }
__host__ __device__ inline cplx acos_(cplx z) {
    // d acos / dx = -1 / sqrt(1 - x^2); no imaginary part at x = +-1
    const double q = 1.0 - z.re * z.re;
    return cplx(acos(z.re), q > 0.0 ? -z.im / sqrt(q) : 0.0);
}

__host__ __device__ inline double sin_(double x) { return sin(x); }
__host__ __device__ inline cplx sin_(cplx z) { return cplx(sin(z.re) * cosh(z.im), cos(z.re) * sinh(z.im)); }
__host__ __device__ inline double cos_(double x) { return cos(x); }
__host__ __device__ inline cplx cos_(cplx z) { return cplx(cos(z.re) * cosh(z.im), -sin(z.re) * sinh(z.im)); }

}  // namespace idw
