// Per-surface-node properties on the GPU (FP64):
//   forward  computeNodalProperties   src/modules/kd_tree.F90:1580-1664
//            getElementProps          src/warp/getElementProps.F90:1-46
//            getRotationMatrix3d      src/utils/vectorUtils.f90:31-103
//            determineCorners         src/modules/kd_tree.F90:1666-1715
//            setData                  src/modules/kd_tree.F90:595-617
//   reverse  COMPUTENODALPROPERTIES_B src/modules/kd_tree.F90:1057-1162
//            setData_b                src/modules/kd_tree.F90:1033-1051
//   tangent  COMPUTENODALPROPERTIES_D src/modules/kd_tree.F90:1250-1356
//            GETELEMENTPROPS_D        src/adjoint/outputForward/getElementProps_d.f90
//            GETROTATIONMATRIX3D_D    src/adjoint/outputForward/vectorUtils_d.f90:7-119
// The reverse kernels recompute the forward intermediates of each node in
// registers instead of replaying a tape.
#include "idw_common.cuh"
#include "idw_kernels.h"
#include "idw_land.cuh"
#include "idw_nodal_math.cuh"

namespace idw {

namespace {

// Adjoint of element_props: accumulate d(area)*areab + d(normal).normalb into
// Xub of the face's vertices (atomically: vertices are shared between nodes).
template <bool DET>
__device__ void element_props_b(const double *Xu, const int *conn, int np, double areab, const double *normalb,
                                double *Xub) {
    double c[3] = {0, 0, 0};
    for (int k = 0; k < np; ++k) {
        const double *p = Xu + 3 * conn[k];
        c[0] += p[0];
        c[1] += p[1];
        c[2] += p[2];
    }
    c[0] /= double(np);
    c[1] /= double(np);
    c[2] /= double(np);
    auto rv = [&](int k, double *o) {
        const double *p = Xu + 3 * conn[k];
        o[0] = p[0] - c[0];
        o[1] = p[1] - c[1];
        o[2] = p[2] - c[2];
    };
    // forward pass: the un-normalised normal sum
    double ns[3] = {0, 0, 0};
    for (int k = 0; k < np; ++k) {
        double a[3], b[3], cr[3];
        rv(k, a);
        rv(k < np - 1 ? k + 1 : 0, b);
        cross3(a, b, cr);
        double cn = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2] + 1e-15);
        ns[0] += cr[0] / cn;
        ns[1] += cr[1] / cn;
        ns[2] += cr[2] / cn;
    }
    double t = ns[0] * ns[0] + ns[1] * ns[1] + ns[2] * ns[2];
    double t0 = sqrt(t);
    double dotb = ns[0] * normalb[0] + ns[1] * normalb[1] + ns[2] * normalb[2];
    double tb = (t == 0.0) ? 0.0 : -(dotb / (2.0 * t0 * t0 * t0));
    double nsb[3] = {normalb[0] / t0 + 2 * ns[0] * tb, normalb[1] / t0 + 2 * ns[1] * tb,
                     normalb[2] / t0 + 2 * ns[2] * tb};
    double rvb[kMaxFacePts][3];
    for (int k = 0; k < np; ++k) rvb[k][0] = rvb[k][1] = rvb[k][2] = 0.0;
    for (int k = np - 1; k >= 0; --k) {
        int j = k < np - 1 ? k + 1 : 0;
        double a[3], b[3], cr[3];
        rv(k, a);
        rv(j, b);
        cross3(a, b, cr);
        double cn = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2] + 1e-15);
        double crb[3] = {nsb[0] / cn, nsb[1] / cn, nsb[2] / cn};
        double cnb = 0.5 * areab - (cr[0] * nsb[0] + cr[1] * nsb[1] + cr[2] * nsb[2]) / (cn * cn);
        double q = cnb / (2.0 * cn);
        crb[0] += 2 * cr[0] * q;
        crb[1] += 2 * cr[1] * q;
        crb[2] += 2 * cr[2] * q;
        double tmp[3];
        cross3(b, crb, tmp);  // d(a x b)/da applied to crb
        rvb[k][0] += tmp[0];
        rvb[k][1] += tmp[1];
        rvb[k][2] += tmp[2];
        cross3(crb, a, tmp);  // d(a x b)/db applied to crb
        rvb[j][0] += tmp[0];
        rvb[j][1] += tmp[1];
        rvb[j][2] += tmp[2];
    }
    double cb[3] = {0, 0, 0};
    for (int k = 0; k < np; ++k) {
        cb[0] -= rvb[k][0];
        cb[1] -= rvb[k][1];
        cb[2] -= rvb[k][2];
    }
    cb[0] /= double(np);
    cb[1] /= double(np);
    cb[2] /= double(np);
    for (int k = 0; k < np; ++k) {
        double *o = Xub + 3 * conn[k];
        land_add<DET>(o + 0, rvb[k][0] + cb[0]);
        land_add<DET>(o + 1, rvb[k][1] + cb[1]);
        land_add<DET>(o + 2, rvb[k][2] + cb[2]);
    }
}

// Adjoint of rotation_matrix with respect to v2 (v1 = normals0 is fixed).
// Zero when the rotation axis is degenerate (axisMag < tol) or the acos
// argument was clamped, as the reference's derivative
// (src/adjoint/outputReverse/vectorUtils_b.f90:7-154).
__device__ void rotation_matrix_b(const double *v1, const double *v2, const double *Mb, double *v2b) {
    double mag1 = mag_eps(v1), mag2 = mag_eps(v2);
    double ax0[3];
    cross3(v1, v2, ax0);
    double axm = mag_eps(ax0);
    if (axm < kRotTol) return;
    double ax[3] = {ax0[0] / axm, ax0[1] / axm, ax0[2] / axm};
    double vv1[3] = {v1[0] / mag1, v1[1] / mag1, v1[2] / mag1};
    double d = vv1[0] * (v2[0] / mag2) + vv1[1] * (v2[1] / mag2) + vv1[2] * (v2[2] / mag2);
    bool clamped = !(1.0 > d);
    double arg = clamped ? 1.0 : d;
    double ang = acos(arg);
    double s = sin(ang), c = cos(ang);
    double A[9] = {0.0, -ax[2], ax[1], ax[2], 0.0, -ax[0], -ax[1], ax[0], 0.0};
    double angb = 0.0;
    double Ab[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double C = A[3 * i] * A[j] + A[3 * i + 1] * A[3 + j] + A[3 * i + 2] * A[6 + j];
            angb += c * A[3 * i + j] * Mb[3 * i + j] + s * C * Mb[3 * i + j];
            Ab[3 * i + j] = s * Mb[3 * i + j];
        }
    const double w = 1.0 - c;  // Cb = w * Mb; Ab += Cb A^T + A^T Cb
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < 3; ++k) acc += Mb[3 * i + k] * A[3 * j + k] + A[3 * k + i] * Mb[3 * k + j];
            Ab[3 * i + j] += w * acc;
        }
    double axb[3] = {Ab[7] - Ab[5], Ab[2] - Ab[6], Ab[3] - Ab[1]};
    double argb = (arg == 1.0 || arg == -1.0) ? 0.0 : -(angb / sqrt(1.0 - arg * arg));
    double vv2b[3] = {0, 0, 0};
    if (!clamped) {
        vv2b[0] = vv1[0] * argb;
        vv2b[1] = vv1[1] * argb;
        vv2b[2] = vv1[2] * argb;
    }
    double mag2b = -(v2[0] * vv2b[0] + v2[1] * vv2b[1] + v2[2] * vv2b[2]) / (mag2 * mag2);
    double axmb = -(ax0[0] * axb[0] + ax0[1] * axb[1] + ax0[2] * axb[2]) / (axm * axm);
    double ax0b[3] = {axb[0] / axm + ax0[0] * axmb / axm, axb[1] / axm + ax0[1] * axmb / axm,
                      axb[2] / axm + ax0[2] * axmb / axm};
    double tmp[3];
    cross3(ax0b, v1, tmp);  // ax0 = v1 x v2
    v2b[0] += vv2b[0] / mag2 + tmp[0] + v2[0] * mag2b / mag2;
    v2b[1] += vv2b[1] / mag2 + tmp[1] + v2[1] * mag2b / mag2;
    v2b[2] += vv2b[2] / mag2 + tmp[2] + v2[2] * mag2b / mag2;
}

// Area and unit normal of every face of the current surface, once per face
// (the node kernels read them instead of recomputing each face per node).
__global__ void k_face_props(SurfaceDev s, const double *Xu) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= s.nFaces) return;
    const int f0 = s.facePtr[f], np = s.facePtr[f + 1] - f0;
    double area, fn[3];
    element_props(Xu, s.faceConn + f0, np, area, fn);
    double *o = s.faceScratch + 4 * int64_t(f);
    o[0] = area;
    o[1] = fn[0];
    o[2] = fn[1];
    o[3] = fn[2];
}

// Area-weighted node normal from the stored face properties, summed over the
// node's faces in the order of node_normal.
__device__ void node_normal_f(const SurfaceDev &s, int i, double &sumArea, double *sumNormal) {
    sumArea = 0.0;
    sumNormal[0] = sumNormal[1] = sumNormal[2] = 0.0;
    for (int e = s.n2ePtr[i]; e < s.n2ePtr[i + 1]; ++e) {
        const int f = s.n2e[e];
        const int np = s.facePtr[f + 1] - s.facePtr[f];
        const double *fp = s.faceScratch + 4 * int64_t(f);
        const double dA = fp[0] / double(np);
        sumArea += dA;
        sumNormal[0] += dA * fp[1];
        sumNormal[1] += dA * fp[2];
        sumNormal[2] += dA * fp[3];
    }
}

__global__ void k_gather_xu(int n, const int *xuInd, const double *Xs, double *Xu) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int j = xuInd[i];
    Xu[3 * i + 0] = Xs[3 * j + 0];
    Xu[3 * i + 1] = Xs[3 * j + 1];
    Xu[3 * i + 2] = Xs[3 * j + 2];
}

// Initial pass: normals0 and the node areas Ai (kd_tree.F90:1630-1636).
__global__ void k_nodal_init(SurfaceDev s, const double *Xu, double *normals0, double *Ai) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    double sa, sn[3];
    node_normal(s, Xu, i, sa, sn);
    normals0[3 * i + 0] = sn[0] / sa;
    normals0[3 * i + 1] = sn[1] / sa;
    normals0[3 * i + 2] = sn[2] / sa;
    Ai[i] = sa;
}

__global__ void k_corners(SurfaceDev s, const double *Xu, const double *normals0, double threshold, int enabled,
                          int *isCorner) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    int flag = 0;
    if (enabled) {
        for (int e = s.n2ePtr[i]; e < s.n2ePtr[i + 1]; ++e) {
            int f = s.n2e[e];
            int f0 = s.facePtr[f], np = s.facePtr[f + 1] - f0;
            double area, fn[3];
            element_props(Xu, s.faceConn + f0, np, area, fn);
            double dp = fn[0] * normals0[3 * i] + fn[1] * normals0[3 * i + 1] + fn[2] * normals0[3 * i + 2];
            if (fabs(dp) < threshold) flag = 1;
        }
    }
    isCorner[i] = flag;
}

// Per warp: Mi, Bi of every node (kd_tree.F90:1637-1663), stored as 12
// doubles per node (M row-major, then b).
__global__ void k_nodal(SurfaceDev s, const double *Xu, const dbl4 *xa, const double *normals0, const double *Ai,
                        const int *isCorner, int useRotations, double *ptMB) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    double M[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    double b[3] = {0, 0, 0};
    if (Ai[i] != 0.0) {
        if (useRotations && !isCorner[i]) {
            double sa, sn[3];
            node_normal_f(s, i, sa, sn);
            double nrm[3] = {sn[0] / sa, sn[1] / sa, sn[2] / sa};
            rotation_matrix(normals0 + 3 * i, nrm, M);
        }
        const dbl4 q = xa[i];
        const double x0[3] = {q.x, q.y, q.z};
        for (int a = 0; a < 3; ++a)
            b[a] = Xu[3 * i + a] - (M[3 * a] * x0[0] + M[3 * a + 1] * x0[1] + M[3 * a + 2] * x0[2]);
    }
    double *o = ptMB + 12 * i;
#pragma unroll
    for (int q = 0; q < 9; ++q) o[q] = M[q];
    o[9] = b[0];
    o[10] = b[1];
    o[11] = b[2];
}

// setData: unweighted mean of the 12 node values over each interior node's
// range (kd_tree.F90:595-617), bottom-up: a leaf sums its own points, and the
// second child to finish adds the two child sums into the parent and carries
// on towards the root (the first one stops).  Every point is read once.
__global__ void k_set_data(TreeDev t, const double *ptMB, double *nodeMB, double *sum, unsigned *flags) {
    const int q0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (q0 >= t.nNodes) return;
    const int4 inf = t.info[q0];
    if (!inf.w) return;
    double acc[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) acc[c] = 0.0;
    for (int i = inf.x; i <= inf.y; ++i) {
        const double2 *p = reinterpret_cast<const double2 *>(ptMB + 12 * i);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const double2 v = __ldg(p + c);
            acc[2 * c] += v.x;
            acc[2 * c + 1] += v.y;
        }
    }
#pragma unroll
    for (int c = 0; c < 12; ++c) sum[12 * q0 + c] = acc[c];
    int q = q0;
    while (true) {
        const int p = t.parent[q];
        if (p < 0) break;
        __threadfence();
        if (atomicAdd(flags + p, 1u) == 0u) break;  // the sibling is not done yet
        const int a = p + 1, b = t.info[a].z;
        const int4 pi = t.info[p];
        const double cnt = double(pi.y - pi.x + 1);
#pragma unroll
        for (int c = 0; c < 12; ++c) {
            const double s = __ldcg(sum + 12 * a + c) + __ldcg(sum + 12 * b + c);
            sum[12 * p + c] = s;
            nodeMB[12 * p + c] = s / cnt;
        }
        q = p;
    }
}

__global__ void k_tree_parents(TreeDev t, int *parent) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= t.nNodes) return;
    if (q == 0) parent[0] = -1;
    const int4 inf = t.info[q];
    if (inf.w) return;
    parent[q + 1] = q;
    parent[t.info[q + 1].z] = q;
}

// setData_b: push the cluster adjoints down to the member points
// (kd_tree.F90:1033-1051).  One thread per point walks its ancestors.
__global__ void k_set_data_b(TreeDev t, const double *nodeAdj, double *ptAdj, int nPts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nPts) return;
    double acc[12];
#pragma unroll
    for (int c = 0; c < 12; ++c) acc[c] = 0.0;
    int q = 0;
    while (q < t.nNodes) {
        int4 inf = t.info[q];
        if (inf.w) break;
        double ovrN = 1.0 / double(inf.y - inf.x + 1);
        const double *a = nodeAdj + 12 * q;
#pragma unroll
        for (int c = 0; c < 12; ++c) acc[c] += a[c] * ovrN;
        int left = q + 1;
        int4 li = t.info[left];
        q = (i <= li.y) ? left : li.z;
    }
    double *o = ptAdj + 12 * i;
#pragma unroll
    for (int c = 0; c < 12; ++c) o[c] += acc[c];
}

// Reverse nodal properties: point adjoints (Mib, Bib) -> Xub; one thread per
// node, scatter to face vertices with atomics.
// relative = 1: ptAdj's first nine entries already hold Mib - Xu0 (x) Bib
// (the mixed adjoint accumulates them that way).
// Reverse nodal properties, node part (COMPUTENODALPROPERTIES_B): Xub += Bb;
// for a rotating node, Mb through the Rodrigues adjoint to the node normal,
// and from it the adjoints of the face areas and normals it was summed from,
// added per face (the face part then runs each face's element adjoint once:
// element_props_b is linear in those adjoints).
template <bool DET>
__global__ void k_nodal_b_nodes(SurfaceDev s, const dbl4 *xa, const double *normals0, const int *isCorner,
                                int useRotations, const double *ptAdj, int relative, double *Xub) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    const double *adj = ptAdj + 12 * i;
    double Mb[9];
    double Bb[3] = {adj[9], adj[10], adj[11]};
    Xub[3 * i + 0] += Bb[0];
    Xub[3 * i + 1] += Bb[1];
    Xub[3 * i + 2] += Bb[2];
    if (!(useRotations && !isCorner[i])) return;
    const int e0 = s.n2ePtr[i], e1 = s.n2ePtr[i + 1];
    if (e1 == e0) return;
    const dbl4 q = xa[i];
    const double x0[3] = {q.x, q.y, q.z};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int k = 0; k < 3; ++k) Mb[3 * a + k] = relative ? adj[3 * a + k] : adj[3 * a + k] - x0[k] * Bb[a];
    double sa, sn[3];
    node_normal_f(s, i, sa, sn);
    double nrm[3] = {sn[0] / sa, sn[1] / sa, sn[2] / sa};
    double nb[3] = {0, 0, 0};
    rotation_matrix_b(normals0 + 3 * i, nrm, Mb, nb);
    double snb[3] = {nb[0] / sa, nb[1] / sa, nb[2] / sa};
    double sab = -(sn[0] * nb[0] + sn[1] * nb[1] + sn[2] * nb[2]) / sa / sa;
    double *faceAdj = s.faceScratch + 4 * int64_t(s.nFaces);
    for (int e = e1 - 1; e >= e0; --e) {
        const int f = s.n2e[e];
        const int np = s.facePtr[f + 1] - s.facePtr[f];
        const double *fp = s.faceScratch + 4 * int64_t(f);
        const double dA = fp[0] / double(np);
        const double dAb = sab + fp[1] * snb[0] + fp[2] * snb[1] + fp[3] * snb[2];
        double *fa = faceAdj + 4 * int64_t(f);
        land_add<DET>(fa + 0, dAb / double(np));
        land_add<DET>(fa + 1, dA * snb[0]);
        land_add<DET>(fa + 2, dA * snb[1]);
        land_add<DET>(fa + 3, dA * snb[2]);
    }
}

// Reverse nodal properties, face part: each face's element adjoint with the
// summed area and normal adjoints of its nodes, into Xub of its vertices.
template <bool DET>
__global__ void k_nodal_b_faces(SurfaceDev s, const double *Xu, double *Xub) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= s.nFaces) return;
    const double *fa = s.faceScratch + 4 * int64_t(s.nFaces) + 4 * int64_t(f);
    const double areab = fa[0], nb[3] = {fa[1], fa[2], fa[3]};
    if (areab == 0.0 && nb[0] == 0.0 && nb[1] == 0.0 && nb[2] == 0.0) return;
    const int f0 = s.facePtr[f], np = s.facePtr[f + 1] - f0;
    element_props_b<DET>(Xu, s.faceConn + f0, np, areab, nb, Xub);
}

// dXs[XuInd[i]] = Xub[i]: only the first caller occurrence of a unique point
// receives the gradient (kd_tree.F90:1155-1159); dXs is pre-zeroed.
__global__ void k_scatter_dxs(int n, const int *xuInd, const double *Xub, double *dXs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int j = xuInd[i];
    dXs[3 * j + 0] = Xub[3 * i + 0];
    dXs[3 * j + 1] = Xub[3 * i + 1];
    dXs[3 * j + 2] = Xub[3 * i + 2];
}

// ---- tangent (forward-mode) nodal properties ----

// element_props and its directional derivative along Xud.
__device__ void element_props_d(const double *Xu, const double *Xud, const int *conn, int np, double &area,
                                double &aread, double *normal, double *normald) {
    double c[3] = {0, 0, 0}, cd[3] = {0, 0, 0};
    for (int k = 0; k < np; ++k) {
        const double *p = Xu + 3 * conn[k];
        const double *pd = Xud + 3 * conn[k];
        for (int a = 0; a < 3; ++a) {
            c[a] += p[a];
            cd[a] += pd[a];
        }
    }
    for (int a = 0; a < 3; ++a) {
        c[a] /= double(np);
        cd[a] /= double(np);
    }
    double nrm[3] = {0, 0, 0}, nrmd[3] = {0, 0, 0};
    double ar = 0, ard = 0;
    for (int k = 0; k < np; ++k) {
        const int j = k < np - 1 ? k + 1 : 0;
        const double *pi = Xu + 3 * conn[k], *pj = Xu + 3 * conn[j];
        const double *pid = Xud + 3 * conn[k], *pjd = Xud + 3 * conn[j];
        double a[3], b[3], ad[3], bd[3];
        for (int q = 0; q < 3; ++q) {
            a[q] = pi[q] - c[q];
            b[q] = pj[q] - c[q];
            ad[q] = pid[q] - cd[q];
            bd[q] = pjd[q] - cd[q];
        }
        double cr[3], t1[3], t2[3];
        cross3(a, b, cr);
        cross3(ad, b, t1);
        cross3(a, bd, t2);
        const double crd[3] = {t1[0] + t2[0], t1[1] + t2[1], t1[2] + t2[2]};
        const double cn = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2] + 1e-15);
        const double cnd = (cr[0] * crd[0] + cr[1] * crd[1] + cr[2] * crd[2]) / cn;
        ar += 0.5 * cn;
        ard += 0.5 * cnd;
        for (int q = 0; q < 3; ++q) {
            nrm[q] += cr[q] / cn;
            nrmd[q] += (crd[q] - cr[q] * cnd / cn) / cn;
        }
    }
    const double m = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    const double md = (nrm[0] * nrmd[0] + nrm[1] * nrmd[1] + nrm[2] * nrmd[2]) / m;
    for (int q = 0; q < 3; ++q) {
        normal[q] = nrm[q] / m;
        normald[q] = (nrmd[q] - nrm[q] * md / m) / m;
    }
    area = ar;
    aread = ard;
}

// rotation_matrix and its derivative along v2d (v1 = normals0 is fixed).
// The derivative is zero when the axis is degenerate, and the angle carries
// none when the acos argument was clamped or is +-1, as GETROTATIONMATRIX3D_D.
__device__ void rotation_matrix_d(const double *v1, const double *v2, const double *v2d, double *M, double *Md) {
    const double mag1 = mag_eps(v1), mag2 = mag_eps(v2);
    const double mag2d = (v2[0] * v2d[0] + v2[1] * v2d[1] + v2[2] * v2d[2]) / mag2;
    double ax[3], axd[3];
    cross3(v1, v2, ax);
    cross3(v1, v2d, axd);
    const double axm = mag_eps(ax);
    double s, omc, sd, omcd;
    if (axm < kRotTol) {
        ax[0] = 1.0;
        ax[1] = ax[2] = 0.0;
        axd[0] = axd[1] = axd[2] = 0.0;
        s = omc = sd = omcd = 0.0;
    } else {
        const double axmd = (ax[0] * axd[0] + ax[1] * axd[1] + ax[2] * axd[2]) / axm;
        for (int q = 0; q < 3; ++q) {
            axd[q] = (axd[q] - ax[q] * axmd / axm) / axm;
            ax[q] /= axm;
        }
        double d = 0.0, dd = 0.0;
        for (int q = 0; q < 3; ++q) {
            const double vv1 = v1[q] / mag1;
            d += vv1 * (v2[q] / mag2);
            dd += vv1 * ((v2d[q] - v2[q] * mag2d / mag2) / mag2);
        }
        double arg = d, argd = dd;
        if (!(1.0 > d)) {
            arg = 1.0;
            argd = 0.0;
        }
        const double angd = (arg == 1.0 || arg == -1.0) ? 0.0 : -(argd / sqrt(1.0 - arg * arg));
        const double ang = acos(arg);
        s = sin(ang);
        omc = 1.0 - cos(ang);
        sd = cos(ang) * angd;
        omcd = s * angd;
    }
    const double A[9] = {0.0, -ax[2], ax[1], ax[2], 0.0, -ax[0], -ax[1], ax[0], 0.0};
    const double Ad[9] = {0.0, -axd[2], axd[1], axd[2], 0.0, -axd[0], -axd[1], axd[0], 0.0};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double C = 0.0, Cd = 0.0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                C += A[3 * i + k] * A[3 * k + j];
                Cd += Ad[3 * i + k] * A[3 * k + j] + A[3 * i + k] * Ad[3 * k + j];
            }
            M[3 * i + j] = (i == j ? 1.0 : 0.0) + s * A[3 * i + j] + omc * C;
            Md[3 * i + j] = sd * A[3 * i + j] + s * Ad[3 * i + j] + omcd * C + omc * Cd;
        }
}

__global__ void k_nodal_d(SurfaceDev s, const double *Xu, const double *Xud, const dbl4 *xa, const double *normals0,
                          const double *Ai, const int *isCorner, int useRotations, int plusIdentity, double *ptMBd) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    double Md[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double bd[3] = {0, 0, 0};
    // nodes without faces keep M = I, b = 0 and carry no derivative
    if (Ai[i] != 0.0) {
        if (useRotations && !isCorner[i]) {
            double sa = 0.0, sad = 0.0, sn[3] = {0, 0, 0}, snd[3] = {0, 0, 0};
            for (int e = s.n2ePtr[i]; e < s.n2ePtr[i + 1]; ++e) {
                const int f = s.n2e[e];
                const int f0 = s.facePtr[f], np = s.facePtr[f + 1] - f0;
                double area, aread, fn[3], fnd[3];
                element_props_d(Xu, Xud, s.faceConn + f0, np, area, aread, fn, fnd);
                const double dA = area / double(np), dAd = aread / double(np);
                sa += dA;
                sad += dAd;
                for (int q = 0; q < 3; ++q) {
                    sn[q] += dA * fn[q];
                    snd[q] += dAd * fn[q] + dA * fnd[q];
                }
            }
            double nrm[3], nrmd[3], M[9];
            for (int q = 0; q < 3; ++q) {
                nrm[q] = sn[q] / sa;
                nrmd[q] = (snd[q] * sa - sn[q] * sad) / (sa * sa);
            }
            rotation_matrix_d(normals0 + 3 * i, nrm, nrmd, M, Md);
        }
        const dbl4 q = xa[i];
        const double x0[3] = {q.x, q.y, q.z};
        for (int a = 0; a < 3; ++a)
            bd[a] = Xud[3 * i + a] - (Md[3 * a] * x0[0] + Md[3 * a + 1] * x0[1] + Md[3 * a + 2] * x0[2]);
    }
    double *o = ptMBd + 12 * i;
#pragma unroll
    for (int q = 0; q < 9; ++q) o[q] = Md[q] + ((plusIdentity && (q % 4 == 0)) ? 1.0 : 0.0);
    o[9] = bd[0];
    o[10] = bd[1];
    o[11] = bd[2];
}

inline int blocks(int64_t n, int b) { return int((n + b - 1) / b); }

}  // namespace

void launch_gather_xu(int n, const int *xuInd, const double *Xs, double *Xu, cudaStream_t st) {
    if (n > 0) k_gather_xu<<<blocks(n, 256), 256, 0, st>>>(n, xuInd, Xs, Xu);
}
void launch_nodal_init(const SurfaceDev &s, const double *Xu, double *normals0, double *Ai, cudaStream_t st) {
    if (s.n > 0) k_nodal_init<<<blocks(s.n, 128), 128, 0, st>>>(s, Xu, normals0, Ai);
}
void launch_corners(const SurfaceDev &s, const double *Xu, const double *normals0, double threshold, int enabled,
                    int *isCorner, cudaStream_t st) {
    if (s.n > 0) k_corners<<<blocks(s.n, 128), 128, 0, st>>>(s, Xu, normals0, threshold, enabled, isCorner);
}
void launch_nodal(const SurfaceDev &s, const double *Xu, const dbl4 *xa, const double *normals0,
                  const double *Ai, const int *isCorner, int useRotations, double *ptMB, cudaStream_t st) {
    if (s.n <= 0) return;
    if (useRotations && s.nFaces > 0) k_face_props<<<blocks(s.nFaces, 128), 128, 0, st>>>(s, Xu);
    k_nodal<<<blocks(s.n, 128), 128, 0, st>>>(s, Xu, xa, normals0, Ai, isCorner, useRotations, ptMB);
}
void launch_set_data(const TreeDev &t, const double *ptMB, double *nodeMB, const SetDataScratch &sc, cudaStream_t st) {
    if (t.nNodes <= 0) return;
    cudaMemsetAsync(sc.flags, 0, sizeof(unsigned) * size_t(t.nNodes), st);
    k_set_data<<<blocks(t.nNodes, 128), 128, 0, st>>>(t, ptMB, nodeMB, sc.sum, sc.flags);
}
void launch_tree_parents(const TreeDev &t, int *parent, cudaStream_t st) {
    if (t.nNodes > 0) k_tree_parents<<<blocks(t.nNodes, 128), 128, 0, st>>>(t, parent);
}
void launch_set_data_b(const TreeDev &t, const double *nodeAdj, double *ptAdj, int nPts, cudaStream_t st) {
    if (nPts > 0) k_set_data_b<<<blocks(nPts, 128), 128, 0, st>>>(t, nodeAdj, ptAdj, nPts);
}
void launch_nodal_b(const SurfaceDev &s, const double *Xu, const dbl4 *xa, const double *normals0,
                    const int *isCorner, int useRotations, const double *ptAdj, int relative, double *Xub,
                    cudaStream_t st, int faceProps) {
    if (s.n <= 0) return;
    if (useRotations && s.nFaces > 0) {
        if (faceProps) k_face_props<<<blocks(s.nFaces, 128), 128, 0, st>>>(s, Xu);
        cudaMemsetAsync(s.faceScratch + 4 * size_t(s.nFaces), 0, 4 * sizeof(double) * size_t(s.nFaces), st);
    }
    k_nodal_b_nodes<false>
        <<<blocks(s.n, 128), 128, 0, st>>>(s, xa, normals0, isCorner, useRotations, ptAdj, relative, Xub);
    if (useRotations && s.nFaces > 0) k_nodal_b_faces<false><<<blocks(s.nFaces, 128), 128, 0, st>>>(s, Xu, Xub);
}
void launch_nodal_b_nodes(const SurfaceDev &s, const double *Xu, const dbl4 *xa, const double *normals0,
                          const int *isCorner, int useRotations, const double *ptAdj, int relative, double *Xub,
                          cudaStream_t st, int faceProps, int det) {
    if (s.n <= 0) return;
    if (useRotations && s.nFaces > 0) {
        if (faceProps) k_face_props<<<blocks(s.nFaces, 128), 128, 0, st>>>(s, Xu);
        cudaMemsetAsync(s.faceScratch + 4 * size_t(s.nFaces), 0, 4 * sizeof(double) * size_t(s.nFaces), st);
    }
    if (det)
        k_nodal_b_nodes<true>
            <<<blocks(s.n, 128), 128, 0, st>>>(s, xa, normals0, isCorner, useRotations, ptAdj, relative, Xub);
    else
        k_nodal_b_nodes<false>
            <<<blocks(s.n, 128), 128, 0, st>>>(s, xa, normals0, isCorner, useRotations, ptAdj, relative, Xub);
}
void launch_nodal_b_faces(const SurfaceDev &s, const double *Xu, int useRotations, double *Xub, cudaStream_t st,
                          int det) {
    if (!(s.n > 0 && useRotations && s.nFaces > 0)) return;
    if (det) k_nodal_b_faces<true><<<blocks(s.nFaces, 128), 128, 0, st>>>(s, Xu, Xub);
    else k_nodal_b_faces<false><<<blocks(s.nFaces, 128), 128, 0, st>>>(s, Xu, Xub);
}
void launch_nodal_d(const SurfaceDev &s, const double *Xu, const double *Xud, const dbl4 *xa, const double *normals0,
                    const double *Ai, const int *isCorner, int useRotations, int plusIdentity, double *ptMBd,
                    cudaStream_t st) {
    if (s.n > 0)
        k_nodal_d<<<blocks(s.n, 128), 128, 0, st>>>(s, Xu, Xud, xa, normals0, Ai, isCorner, useRotations,
                                                    plusIdentity, ptMBd);
}
void launch_scatter_dxs(int n, const int *xuInd, const double *Xub, double *dXs, cudaStream_t st) {
    if (n > 0) k_scatter_dxs<<<blocks(n, 256), 256, 0, st>>>(n, xuInd, Xub, dXs);
}

IDW_LAND_SETTER(land_set_nodal)

}  // namespace idw
