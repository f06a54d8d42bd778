// Shared device-side definitions of the GB300 IDW warping kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace idw {

// 32-byte aligned quadruple of doubles (one 256-bit load).
struct __align__(32) dbl4 {
    double x, y, z, w;
};
__host__ __device__ __forceinline__ dbl4 mk_dbl4(double x, double y, double z, double w) {
    dbl4 r;
    r.x = x;
    r.y = y;
    r.z = z;
    r.w = w;
    return r;
}

// Read-only-cache load of a dbl4.
__device__ __forceinline__ dbl4 ldg4(const dbl4 *p) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
    double2 a = __ldg(q), b = __ldg(q + 1);
    return mk_dbl4(a.x, a.y, b.x, b.y);
}

constexpr int kNerr = 12;
constexpr int kMaxSym = 6;
constexpr int kMaxFacePts = 32;  // the reference caps faces at 20 points (kd_tree.F90:1590)
constexpr unsigned kFull = 0xffffffffu;

// Error-table radii (src/modules/kd_tree.F90:34-35) and their reciprocal gaps.
__constant__ static double c_rstar[kNerr] = {2.0, 3.0, 4.0, 5.0, 7.5, 10.0, 20.0, 40.0, 80.0, 160.0, 320.0, 640.0};

// Weight law w = A * ((L/d)^a + alpha^b (L/d)^b) of src/modules/kd_tree.F90:680-689.
// Integer exponents (the common case, 3 and 5) use repeated multiplication;
// any other exponent falls back to pow().
struct WeightLaw {
    double Ldef, alphaToBexp, aExp, bExp;
    int ia, ib;     // integer exponents when isInt
    int isInt;
};

__device__ __forceinline__ double ipow(double x, int n) {
    double r = 1.0;
    double b = x;
    while (n > 0) {
        if (n & 1) r *= b;
        n >>= 1;
        if (n) b *= b;
    }
    return r;
}

__device__ __forceinline__ float ipowf(float x, int n) {
    float r = 1.0f;
    float b = x;
    while (n > 0) {
        if (n & 1) r *= b;
        n >>= 1;
        if (n) b *= b;
    }
    return r;
}

// (L/d)^a + alpha^b (L/d)^b for a given LdefoDist = L/d, FP64.
__device__ __forceinline__ double law64(const WeightLaw &w, double LoD) {
    if (w.isInt) {
        double ta = ipow(LoD, w.ia);
        double tb = ta * ipow(LoD, w.ib - w.ia);
        return ta + w.alphaToBexp * tb;
    }
    return pow(LoD, w.aExp) + w.alphaToBexp * pow(LoD, w.bExp);
}

// Linear interpolation of the error table (src/modules/kd_tree.F90:882-906).
__device__ __forceinline__ double get_error64(const double *err, double dOvrR) {
    double e = err[kNerr - 1];
#pragma unroll
    for (int i = 0; i < kNerr - 1; ++i) {
        if (dOvrR < c_rstar[i + 1]) {
            double fact = (dOvrR - c_rstar[i]) * (1.0 / (c_rstar[i + 1] - c_rstar[i]));
            return (1.0 - fact) * err[i] + fact * err[i + 1];
        }
    }
    return e;
}

// FP64 fast-walk decision at interior node `node` (kd_tree.F90:636-660):
// returns 1 to approximate (dist set), 0 to open.  Shared by the FP64 walk and
// the mixed walk's guarded fallback so both take bit-identical decisions.
__device__ __forceinline__ int decide64(const dbl4 &g, const double *err, const double *r, double tolDen,
                                        double &dist) {
    dist = sqrt((r[0] - g.x) * (r[0] - g.x) + (r[1] - g.y) * (r[1] - g.y) + (r[2] - g.z) * (r[2] - g.z));
    double dOvrR = dist * g.w;
    if (dOvrR < 2.0) return 0;
    return get_error64(err, dOvrR) < tolDen ? 1 : 0;
}

// Symmetry-plane reflections (src/warp/initializeWarping.F90:533-601): loop
// index kk (0-based here) selects the planes j with bit j set.
struct SymPlanes {
    int n;
    int nLoop;
    double p[kMaxSym][3];
    double nrm[kMaxSym][3];
};

__device__ __forceinline__ void mirror_point(const SymPlanes &s, int kk, const double *pt, double *r) {
    r[0] = pt[0];
    r[1] = pt[1];
    r[2] = pt[2];
    for (int j = 0; j < s.n; ++j) {
        if ((kk >> j) & 1) {
            double d0 = r[0] - s.p[j][0], d1 = r[1] - s.p[j][1], d2 = r[2] - s.p[j][2];
            double dp = d0 * s.nrm[j][0] + d1 * s.nrm[j][1] + d2 * s.nrm[j][2];
            r[0] -= 2.0 * s.nrm[j][0] * dp;
            r[1] -= 2.0 * s.nrm[j][1] * dp;
            r[2] -= 2.0 * s.nrm[j][2] * dp;
        }
    }
}

// Reflect a vector (no translation) through the same planes, in plane order.
template <class T>
__device__ __forceinline__ void mirror_vector(const SymPlanes &s, int kk, T *v) {
    for (int j = 0; j < s.n; ++j) {
        if ((kk >> j) & 1) {
            T dp = v[0] * T(s.nrm[j][0]) + v[1] * T(s.nrm[j][1]) + v[2] * T(s.nrm[j][2]);
            v[0] -= T(2) * dp * T(s.nrm[j][0]);
            v[1] -= T(2) * dp * T(s.nrm[j][1]);
            v[2] -= T(2) * dp * T(s.nrm[j][2]);
        }
    }
}

// Transpose of mirror_vector: the same reflections in reverse plane order.
__device__ __forceinline__ void mirror_vector_t(const SymPlanes &s, int kk, double *v) {
    for (int j = s.n - 1; j >= 0; --j) {
        if ((kk >> j) & 1) {
            double dp = v[0] * s.nrm[j][0] + v[1] * s.nrm[j][1] + v[2] * s.nrm[j][2];
            v[0] -= 2.0 * dp * s.nrm[j][0];
            v[1] -= 2.0 * dp * s.nrm[j][1];
            v[2] -= 2.0 * dp * s.nrm[j][2];
        }
    }
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

}  // namespace idw
