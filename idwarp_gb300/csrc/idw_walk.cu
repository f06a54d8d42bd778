// Per-volume-node evaluation of the IDW sums, FP64 form.
//   fast walk   evalNode / evalNodeApprox     src/modules/kd_tree.F90:619-662, 692-713
//   exact       evalNodeExact (on the root)   src/modules/kd_tree.F90:664-690
//   driver      warpMesh                      src/warp/warpMesh.F90:37-70
//   tangent     evalNode_d / evalNodeExact_d / evalNodeApprox_d  kd_tree.F90:1164-1236,
//               driven as warpDerivFwd        src/warp/warpDerivFwd.F90:58-97
//               (the walk is the forward one with (M, b) replaced by
//               (Md + I, bd), so that S = Md r + bd)
//   adjoint     evalNode_b / evalNodeExact_b / evalNodeApprox_b  kd_tree.F90:942-1031,
//               driven as warpDeriv           src/warp/warpDeriv.F90:71-88
//
// Traversal.  Each warp takes 32 volume nodes that are adjacent in Morton
// order and walks the preorder tree together: the current tree node is the
// same for the whole warp, every lane decides for itself (open /
// approximate / leaf) exactly as the reference recursion would, a lane that
// approximated a cluster idles until the walk leaves that cluster's subtree
// (its escape index), and the warp descends when any lane opens.  Each lane
// therefore sees precisely the reference's sequence of nodes, in the
// reference's order (left before right), while the tree data it reads is the
// same for all 32 lanes (broadcast loads).
#include "idw_common.cuh"
#include "idw_kernels.h"
#include "idw_land.cuh"

namespace idw {

namespace {

struct Counters {
    unsigned long long leafPairs = 0, approx = 0, visited = 0, fallback = 0;
    __device__ void flush(unsigned long long *dst) {
        if (!dst) return;
        unsigned long long a = warp_sum(leafPairs), b = warp_sum(approx), c = warp_sum(visited),
                           d = warp_sum(fallback);
        if ((threadIdx.x & 31) == 0) {
            if (a) atomicAdd(dst + 0, a);
            if (b) atomicAdd(dst + 1, b);
            if (c) atomicAdd(dst + 2, c);
            if (d) atomicAdd(dst + 3, d);
        }
    }
};

__device__ __forceinline__ void load12(const double *src, double *d) {
    const double2 *s2 = reinterpret_cast<const double2 *>(src);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        double2 v = __ldg(s2 + c);
        d[2 * c] = v.x;
        d[2 * c + 1] = v.y;
    }
}

// One exact pair (kd_tree.F90:677-688).  tangent: the pair's motion is
// M r + b (the tangent's Md r + bd, warpDerivFwd.F90), without the - r of
// the warp's M r + b - r.
__device__ __forceinline__ void pair64(const EvalConsts &k, const dbl4 &x, const double *mb, const double *r,
                                       int tangent, double *num, double &den) {
    double r0 = r[0] - x.x, r1 = r[1] - x.y, r2 = r[2] - x.z;
    double LoD = k.law.Ldef / sqrt(r0 * r0 + r1 * r1 + r2 * r2 + 1e-15);
    double W = x.w * law64(k.law, LoD);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double S = mb[3 * a] * r[0] + mb[3 * a + 1] * r[1] + mb[3 * a + 2] * r[2] + mb[9 + a];
        if (!tangent) S -= r[a];
        num[a] += W * S;
    }
    den += W;
}

__global__ void __launch_bounds__(128) k_walk64(TreeDev t, PointsDev p, VolumeDev v, const double *nodeMB,
                                                EvalConsts k, int exact, int nPts, WalkOut o) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = gid < v.nVol;
    const int vi = valid ? v.perm[gid] : 0;
    const double x0[3] = {v.xv0[3 * vi], v.xv0[3 * vi + 1], v.xv0[3 * vi + 2]};
    const double approxDen = v.den0[vi];
    const double tolDen = k.errTol * approxDen;
    double numer[3] = {0, 0, 0}, denom = 0.0;
    Counters cnt;
    for (int kk = 0; kk < k.sym.nLoop; ++kk) {
        double r[3];
        mirror_point(k.sym, kk, x0, r);
        double num[3] = {0, 0, 0}, den = 0.0;
        if (exact) {
            for (int i = 0; i < nPts; ++i) {
                double mb[12];
                load12(p.mb + 12 * i, mb);
                pair64(k, ldg4(p.xa + i), mb, r, o.tangent, num, den);
            }
            cnt.leafPairs += valid ? nPts : 0;
            cnt.visited += valid ? 1 : 0;
        } else {
            int node = 0, skip = 0;
            while (node < t.nNodes) {
                const int4 inf = t.info[node];
                const bool active = valid && node >= skip;
                if (inf.w) {
                    if (active) {
                        for (int i = inf.x; i <= inf.y; ++i) {
                            double mb[12];
                            load12(p.mb + 12 * i, mb);
                            pair64(k, ldg4(p.xa + i), mb, r, o.tangent, num, den);
                        }
                        cnt.leafPairs += inf.y - inf.x + 1;
                        cnt.visited++;
                    }
                    node = inf.z;
                } else {
                    bool open = false;
                    if (active) {
                        cnt.visited++;
                        double dist;
                        if (decide64(t.geom[node], t.err + kNerr * node, r, tolDen, dist)) {
                            double LoD = k.law.Ldef / dist;
                            double W = t.ai[node] * law64(k.law, LoD);
                            double mb[12];
                            load12(nodeMB + 12 * node, mb);
#pragma unroll
                            for (int a = 0; a < 3; ++a) {
                                double S = mb[3 * a] * r[0] + mb[3 * a + 1] * r[1] + mb[3 * a + 2] * r[2] + mb[9 + a];
                                if (!o.tangent) S -= r[a];
                                num[a] += W * S;
                            }
                            den += W;
                            skip = inf.z;
                            cnt.approx++;
                        } else {
                            open = true;
                        }
                    }
                    node = __any_sync(kFull, open) ? node + 1 : inf.z;
                }
            }
        }
        mirror_vector(k.sym, kk, num);
        numer[0] += num[0];
        numer[1] += num[1];
        numer[2] += num[2];
        denom += den;
    }
    if (valid) {
        if (o.tangent) {
            // warpDerivFwd.F90:91-97: the derivative numerator over the last
            // warpMesh's denominator
            const double oden = 1.0 / o.denIn[vi];
            o.xv[3 * vi + 0] = numer[0] * oden;
            o.xv[3 * vi + 1] = numer[1] * oden;
            o.xv[3 * vi + 2] = numer[2] * oden;
        } else {
            double oden = 1.0 / denom;
            if (o.xv) {
                o.xv[3 * vi + 0] = x0[0] + numer[0] * oden;
                o.xv[3 * vi + 1] = x0[1] + numer[1] * oden;
                o.xv[3 * vi + 2] = x0[2] + numer[2] * oden;
            }
            if (o.den) o.den[vi] = denom;
        }
    }
    cnt.flush(o.counters);
}

// Sum `val` over the lanes of the warp and add it to *dst from lane 0.
template <bool DET>
__device__ __forceinline__ void warp_atomic_add(double *dst, double val, bool any) {
    if (!any) return;
    double s = warp_sum(val);
    if ((threadIdx.x & 31) == 0 && s != 0.0) land_add<DET>(dst, s);
}


// Reverse walk for nSeeds seeds at once: the weights are computed once per
// pair and shared by all seeds.  Point adjoints are 12 values per point per
// seed (Mib row-major then Bib), cluster adjoints likewise per tree node.
template <int NS, bool DET = false>
__global__ void __launch_bounds__(128) k_walk_adj64(TreeDev t, PointsDev p, VolumeDev v, EvalConsts k, int exact,
                                                    int nPts, const double *dxv, const double *den, int64_t seedStride,
                                                    double *ptAdj, double *nodeAdj, int64_t ptStride,
                                                    int64_t nodeStride, unsigned long long *counters) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = gid < v.nVol;
    const int vi = valid ? v.perm[gid] : 0;
    const double x0[3] = {v.xv0[3 * vi], v.xv0[3 * vi + 1], v.xv0[3 * vi + 2]};
    const double tolDen = k.errTol * v.den0[vi];
    const double oden = valid ? 1.0 / den[vi] : 0.0;
    Counters cnt;
    for (int kk = 0; kk < k.sym.nLoop; ++kk) {
        double r[3];
        mirror_point(k.sym, kk, x0, r);
        double numb[NS][3];
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            const double *d = dxv + s * seedStride + 3 * int64_t(vi);
            numb[s][0] = valid ? d[0] * oden : 0.0;
            numb[s][1] = valid ? d[1] * oden : 0.0;
            numb[s][2] = valid ? d[2] * oden : 0.0;
            mirror_vector_t(k.sym, kk, numb[s]);
        }
        int node = exact ? -1 : 0, skip = 0;
        const int nNodes = exact ? 0 : t.nNodes;
        // exact mode: a single pass over all points as if the root were a leaf
        bool exactPass = exact;
        while (exactPass || node < nNodes) {
            int4 inf;
            bool isLeaf;
            if (exactPass) {
                inf = make_int4(0, nPts - 1, nNodes, 1);
                isLeaf = true;
            } else {
                inf = t.info[node];
                isLeaf = inf.w != 0;
            }
            const bool active = valid && (exactPass || node >= skip);
            if (isLeaf) {
                const bool any = __any_sync(kFull, active);
                if (any) {
                    for (int i = inf.x; i <= inf.y; ++i) {
                        double W = 0.0;
                        if (active) {
                            dbl4 x = ldg4(p.xa + i);
                            double r0 = r[0] - x.x, r1 = r[1] - x.y, r2 = r[2] - x.z;
                            double dist = sqrt(r0 * r0 + r1 * r1 + r2 * r2 + 1e-15);
                            W = x.w * law64(k.law, k.law.Ldef / dist);
                        }
#pragma unroll
                        for (int s = 0; s < NS; ++s) {
                            double *dst = ptAdj + s * ptStride + 12 * int64_t(i);
                            double sib[3] = {W * numb[s][0], W * numb[s][1], W * numb[s][2]};
#pragma unroll
                            for (int a = 0; a < 3; ++a) {
#pragma unroll
                                for (int c = 0; c < 3; ++c) warp_atomic_add<DET>(dst + 3 * a + c, r[c] * sib[a], true);
                                warp_atomic_add<DET>(dst + 9 + a, sib[a], true);
                            }
                        }
                    }
                    if (active) {
                        cnt.leafPairs += inf.y - inf.x + 1;
                        cnt.visited++;
                    }
                }
                if (exactPass) {
                    exactPass = false;
                    node = nNodes;
                } else {
                    node = inf.z;
                }
            } else {
                bool open = false, approx = false;
                double W = 0.0;
                if (active) {
                    cnt.visited++;
                    double dist;
                    if (decide64(t.geom[node], t.err + kNerr * node, r, tolDen, dist)) {
                        W = t.ai[node] * law64(k.law, k.law.Ldef / dist);
                        approx = true;
                        skip = inf.z;
                        cnt.approx++;
                    } else {
                        open = true;
                    }
                }
                if (__any_sync(kFull, approx)) {
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        double *dst = nodeAdj + s * nodeStride + 12 * int64_t(node);
                        double sib[3] = {W * numb[s][0], W * numb[s][1], W * numb[s][2]};
#pragma unroll
                        for (int a = 0; a < 3; ++a) {
#pragma unroll
                            for (int c = 0; c < 3; ++c) warp_atomic_add<DET>(dst + 3 * a + c, r[c] * sib[a], true);
                            warp_atomic_add<DET>(dst + 9 + a, sib[a], true);
                        }
                    }
                }
                node = __any_sync(kFull, open) ? node + 1 : inf.z;
            }
        }
    }
    cnt.flush(counters);
}

inline int blocks(int64_t n, int b) { return int((n + b - 1) / b); }

}  // namespace

void launch_walk_fp64(const TreeDev &t, const PointsDev &p, const VolumeDev &v, const double *nodeMB,
                      const EvalConsts &k, int exact, int nPts, const WalkOut &o, cudaStream_t st) {
    if (v.nVol > 0) k_walk64<<<blocks(v.nVol, 128), 128, 0, st>>>(t, p, v, nodeMB, k, exact, nPts, o);
}

template <bool DET>
void launch_adj64(const TreeDev &t, const PointsDev &p, const VolumeDev &v, const EvalConsts &k, int exact, int nPts,
                  const double *dxv, const double *den, int nSeeds, int64_t seedStride, double *ptAdj,
                  double *nodeAdj, int64_t ptStride, int64_t nodeStride, unsigned long long *counters,
                  cudaStream_t st) {
    const int g = blocks(v.nVol, 128);
    // Seeds are processed in groups of 1, 4 or 16 sharing one walk.
    int s0 = 0;
    while (s0 < nSeeds) {
        int left = nSeeds - s0;
        const double *d = dxv + s0 * seedStride;
        double *pa = ptAdj + s0 * ptStride;
        double *na = nodeAdj + s0 * nodeStride;
        if (left >= 16) {
            k_walk_adj64<16, DET><<<g, 128, 0, st>>>(t, p, v, k, exact, nPts, d, den, seedStride, pa, na, ptStride,
                                                     nodeStride, counters);
            s0 += 16;
        } else if (left >= 4) {
            k_walk_adj64<4, DET><<<g, 128, 0, st>>>(t, p, v, k, exact, nPts, d, den, seedStride, pa, na, ptStride,
                                                    nodeStride, counters);
            s0 += 4;
        } else {
            k_walk_adj64<1, DET><<<g, 128, 0, st>>>(t, p, v, k, exact, nPts, d, den, seedStride, pa, na, ptStride,
                                                    nodeStride, counters);
            s0 += 1;
        }
    }
}

int launch_walk_adjoint_fp64(const TreeDev &t, const PointsDev &p, const VolumeDev &v, const EvalConsts &k, int exact,
                             int nPts, const double *dxv, const double *den, int nSeeds, int64_t seedStride,
                             double *ptAdj, double *nodeAdj, int64_t ptStride, int64_t nodeStride,
                             unsigned long long *counters, cudaStream_t st, int det) {
    if (v.nVol <= 0) return 0;
    // det: order-independent landings (idw_land.cuh)
    if (det)
        launch_adj64<true>(t, p, v, k, exact, nPts, dxv, den, nSeeds, seedStride, ptAdj, nodeAdj, ptStride,
                           nodeStride, counters, st);
    else
        launch_adj64<false>(t, p, v, k, exact, nPts, dxv, den, nSeeds, seedStride, ptAdj, nodeAdj, ptStride,
                            nodeStride, counters, st);
    return 0;
}

IDW_LAND_SETTER(land_set_walk)

}  // namespace idw
