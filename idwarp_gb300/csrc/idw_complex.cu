// Complex-step build of the FP64 nodal properties (the counterpart of the
// reference's complexified library libidwarp_cs, idwarp/UnstructuredMesh_C.py).
//
// In warpMesh only the nodal properties depend on the surface coordinates:
// the weights come from the initial surface (Xu0, A_i, Ldef0) and the
// volume nodes, and the decisions from real quantities.  With complex surface
// coordinates X + i Y the warped grid is therefore
//   Xv = Xv0 + sum w (M r + b - r) / sum w,   M, b complex,
// whose real part is the ordinary warp of X and whose imaginary part is
//   sum w (Im M r + Im b) / sum w,
// the same walk applied to (Im M, Im b) as a tangent walk (motions M r + b:
// an imaginary part of 1e-40 next to the identity, as in M r + b - r, would
// round away).  This file computes M and b in complex arithmetic from the complex
// coordinates (computeNodalProperties, kd_tree.F90:1580-1664) with the
// templated geometry of idw_nodal_math.cuh; the walk is the FP64 one.
#include "idw_common.cuh"
#include "idw_kernels.h"
#include "idw_nodal_math.cuh"

namespace idw {

namespace {

// Xu (complex, tree order) from the caller's interleaved complex coordinates.
__global__ void k_gather_xu_cs(int n, const int *xuInd, const double *xsC, cplx *xu) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = xuInd[i];
#pragma unroll
    for (int a = 0; a < 3; ++a) xu[3 * i + a] = cplx(xsC[2 * (3 * j + a)], xsC[2 * (3 * j + a) + 1]);
}

// M_i, b_i in complex arithmetic; writes their imaginary parts, 12 doubles
// per node.
__global__ void k_nodal_cs(SurfaceDev s, const cplx *Xu, const dbl4 *xa, const double *normals0, const double *Ai,
                           const int *isCorner, int useRotations, double *ptMBim) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    cplx M[9] = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
    cplx b[3] = {0.0, 0.0, 0.0};
    if (Ai[i] != 0.0) {
        if (useRotations && !isCorner[i]) {
            cplx sa, sn[3];
            node_normal(s, Xu, i, sa, sn);
            const cplx nrm[3] = {sn[0] / sa, sn[1] / sa, sn[2] / sa};
            rotation_matrix(normals0 + 3 * i, nrm, M);
        }
        const dbl4 q = xa[i];
        const double x0[3] = {q.x, q.y, q.z};
        for (int a = 0; a < 3; ++a) b[a] = Xu[3 * i + a] - (M[3 * a] * x0[0] + M[3 * a + 1] * x0[1] + M[3 * a + 2] * x0[2]);
    }
    double *o = ptMBim + 12 * i;
#pragma unroll
    for (int k = 0; k < 9; ++k) o[k] = M[k].im;
    o[9] = b[0].im;
    o[10] = b[1].im;
    o[11] = b[2].im;
}

// out[2 k] = re[k], out[2 k + 1] = im[k]
__global__ void k_interleave(int64_t n, const double *re, const double *im, double *out) {
    const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n) return;
    out[2 * k] = re[k];
    out[2 * k + 1] = im[k];
}

// re[k] = in[2 k], im[k] = in[2 k + 1]
__global__ void k_split(int64_t n, const double *in, double *re, double *im) {
    const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n) return;
    re[k] = in[2 * k];
    im[k] = in[2 * k + 1];
}

inline int blocks(int64_t n, int b) { return int((n + b - 1) / b); }

}  // namespace

void launch_nodal_cs(const SurfaceDev &s, const int *xuInd, const double *xsC, cplx *xu, const dbl4 *xa,
                     const double *normals0, const double *Ai, const int *isCorner, int useRotations, double *ptMBim,
                     cudaStream_t st) {
    if (s.n <= 0) return;
    k_gather_xu_cs<<<blocks(s.n, 256), 256, 0, st>>>(s.n, xuInd, xsC, xu);
    k_nodal_cs<<<blocks(s.n, 128), 128, 0, st>>>(s, xu, xa, normals0, Ai, isCorner, useRotations, ptMBim);
}

void launch_interleave(int64_t n, const double *re, const double *im, double *out, cudaStream_t st) {
    if (n > 0) k_interleave<<<blocks(n, 256), 256, 0, st>>>(n, re, im, out);
}

void launch_split(int64_t n, const double *in, double *re, double *im, cudaStream_t st) {
    if (n > 0) k_split<<<blocks(n, 256), 256, 0, st>>>(n, in, re, im);
}

}  // namespace idw
