// Geometry of the nodal properties, written once for a scalar type T:
// double (the FP64 path) or cplx (the complex-step build of the same path).
//   getElementProps     src/warp/getElementProps.F90:1-46
//   getRotationMatrix3d src/utils/vectorUtils.f90:31-103
//   node normals        src/modules/kd_tree.F90:1603-1625
// Comparisons use real parts (re()); with T = double every expression is the
// plain FP64 one.
#pragma once
#include "idw_cplx.cuh"
#include "idw_kernels.h"

namespace idw {

template <class A, class B, class C>
__device__ __forceinline__ void cross3(const A *a, const B *b, C *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// Area and unit normal of one polygonal face (fan of cross products of the
// centre-relative vertex vectors).
template <class T>
__device__ void element_props(const T *Xu, const int *conn, int np, T &area, T *normal) {
    T c[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < np; ++k) {
        const T *p = Xu + 3 * conn[k];
        c[0] += p[0];
        c[1] += p[1];
        c[2] += p[2];
    }
    c[0] /= double(np);
    c[1] /= double(np);
    c[2] /= double(np);
    T nrm[3] = {0.0, 0.0, 0.0};
    T a = 0.0;
    const T *p0 = Xu + 3 * conn[0];
    T rv0[3] = {p0[0] - c[0], p0[1] - c[1], p0[2] - c[2]};
    T rvi[3] = {rv0[0], rv0[1], rv0[2]};
    for (int k = 0; k < np; ++k) {
        T rvj[3];
        if (k < np - 1) {
            const T *pj = Xu + 3 * conn[k + 1];
            rvj[0] = pj[0] - c[0];
            rvj[1] = pj[1] - c[1];
            rvj[2] = pj[2] - c[2];
        } else {
            rvj[0] = rv0[0];
            rvj[1] = rv0[1];
            rvj[2] = rv0[2];
        }
        T cr[3];
        cross3(rvi, rvj, cr);
        T cn = sqrt_(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2] + 1e-15);
        a += 0.5 * cn;
        nrm[0] += cr[0] / cn;
        nrm[1] += cr[1] / cn;
        nrm[2] += cr[2] / cn;
        rvi[0] = rvj[0];
        rvi[1] = rvj[1];
        rvi[2] = rvj[2];
    }
    T m = sqrt_(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    normal[0] = nrm[0] / m;
    normal[1] = nrm[1] / m;
    normal[2] = nrm[2] / m;
    area = a;
}

template <class T>
__device__ __forceinline__ T mag_eps(const T *v) {
    return sqrt_(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + 1e-30);
}

constexpr double kRotTol = 1.4901161193847656e-08;

// Rodrigues rotation taking direction v1 (normals0, fixed) to direction v2
// (row-major M).
template <class T>
__device__ void rotation_matrix(const double *v1, const T *v2, T *M) {
    double mag1 = mag_eps(v1);
    T mag2 = mag_eps(v2);
    T ax[3];
    cross3(v1, v2, ax);
    T axm = mag_eps(ax);
    T s, omc;
    if (re(axm) < kRotTol) {
        ax[0] = 1.0;
        ax[1] = 0.0;
        ax[2] = 0.0;
        s = 0.0;
        omc = 0.0;
    } else {
        ax[0] /= axm;
        ax[1] /= axm;
        ax[2] /= axm;
        T d = (v1[0] / mag1) * (v2[0] / mag2) + (v1[1] / mag1) * (v2[1] / mag2) + (v1[2] / mag1) * (v2[2] / mag2);
        T arg = (1.0 > re(d)) ? d : T(1.0);
        T ang = acos_(arg);
        s = sin_(ang);
        omc = 1.0 - cos_(ang);
    }
    T A[9] = {0.0, -ax[2], ax[1], ax[2], 0.0, -ax[0], -ax[1], ax[0], 0.0};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T C = A[3 * i] * A[j] + A[3 * i + 1] * A[3 + j] + A[3 * i + 2] * A[6 + j];
            M[3 * i + j] = (i == j ? 1.0 : 0.0) + s * A[3 * i + j] + omc * C;
        }
}

// Area-weighted node normal from the node's faces (kd_tree.F90:1603-1625).
template <class T>
__device__ void node_normal(const SurfaceDev &s, const T *Xu, int i, T &sumArea, T *sumNormal) {
    sumArea = 0.0;
    sumNormal[0] = sumNormal[1] = sumNormal[2] = 0.0;
    for (int e = s.n2ePtr[i]; e < s.n2ePtr[i + 1]; ++e) {
        int f = s.n2e[e];
        int f0 = s.facePtr[f], np = s.facePtr[f + 1] - f0;
        T area, fn[3];
        element_props(Xu, s.faceConn + f0, np, area, fn);
        T dA = area / double(np);
        sumArea += dA;
        sumNormal[0] += dA * fn[0];
        sumNormal[1] += dA * fn[1];
        sumNormal[2] += dA * fn[2];
    }
}

}  // namespace idw
