// Exact-mode mixed evaluation (evalMode = exact): every volume node sums
// every surface point, evalNodeExact on the root (src/modules/kd_tree.F90:
// 664-690) driven by warpMesh (src/warp/warpMesh.F90:46-63).
//
// An N-body kernel over the same leaf-by-leaf arithmetic as the mixed walk's
// exact mode: leaves in preorder, per pair the FP32 term of leaf_pair, per
// leaf the gate of leaf_close (double-float re-sum of heavy leaves) and the
// compensated running sums, per mirror finish_mirror.  The sums are therefore
// bitwise those of the walk; what changes is the schedule.  The block stages
// a tile of kTile surface points (contiguous in tree order: the preorder
// leaves tile [0, n)) in shared memory, every thread carries NV volume nodes
// through it, and the control flow is the same for all threads: no tree
// traversal, no divergent lanes, and each staged point feeds 128 NV nodes.
#include "idw_mixed.cuh"

namespace idw {

namespace {

constexpr int kTile = 256;  // surface points per shared-memory pass
constexpr int kThreads = 128;

// Volume nodes carried by each thread: four on large meshes (more reuse of
// each staged point; 168 registers, three blocks per SM), two otherwise.
constexpr int kBlocksPerSmNV4 = 3;

int sm_count() {
    static int cached[16] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    int &n = cached[dev & 15];
    if (n == 0 && cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) n = 1;
    return n;
}

template <int KIND, int NV>
__global__ void __launch_bounds__(kThreads) k_exact_mixed(TreeDevF tf, PointsDevF pf, NodeAggF af, VolumeDev v,
                                                          WalkRecF rec, MixedParams mp, Law32<KIND> law,
                                                          float4 *acc, unsigned long long *counters) {
    const int nPts = tf.nPts;
    __shared__ float4 sDA[kTile], sDL[kTile], sDM[3 * kTile];
    __shared__ float4 sRH[NV][kThreads], sRL[NV][kThreads];  // this mirror's points (hi, lo)
    const int tid = threadIdx.x;
    const int64_t base = int64_t(blockIdx.x) * (kThreads * NV);
    bool valid[NV];
    int64_t g[NV];
    float Ls[NV], LsLo[NV], c1[NV], gv[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        const int64_t gid = base + j * kThreads + tid;
        valid[j] = gid < v.nVol;
        g[j] = valid[j] ? gid : 0;
        const NodeScale ns = node_scale(rec, mp, g[j]);
        Ls[j] = ns.Ls;
        LsLo[j] = ns.LsLo;
        c1[j] = ns.c1;
        gv[j] = ns.gv;
    }
    const float ab = mp.abH, abl = mp.abL;
    MixedCounters cnt;
    for (int kk = 0; kk < mp.nLoop; ++kk) {
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            sRH[j][tid] = rec.hi[kk * v.nVol + g[j]];
            sRL[j][tid] = rec.lo[kk * v.nVol + g[j]];
        }
        float sn[NV][3], cn[NV][3], sd[NV], cd[NV];
        float h[NV][3], l[NV][3], pn[NV][3], pd[NV];
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            sd[j] = cd[j] = 0.f;
#pragma unroll
            for (int a = 0; a < 3; ++a) sn[j][a] = cn[j][a] = h[j][a] = l[j][a] = pn[j][a] = 0.f;
            pd[j] = 0.f;
        }
        int leaf = 0;
        int4 L = tf.leaves[0];  // (l, u, node): the leaf in progress
        for (int p0 = 0; p0 < nPts; p0 += kTile) {
            const int p1 = min(nPts, p0 + kTile);
            __syncthreads();
            for (int q = tid; q < p1 - p0; q += kThreads) {
                sDA[q] = ldgf4(pf.da + p0 + q);
                sDL[q] = ldgf4(pf.dl + p0 + q);
                const float4 *dm = reinterpret_cast<const float4 *>(pf.dm) + 3 * int64_t(p0 + q);
                sDM[3 * q] = ldgf4(dm);
                sDM[3 * q + 1] = ldgf4(dm + 1);
                sDM[3 * q + 2] = ldgf4(dm + 2);
            }
            __syncthreads();
            int p = p0;
            while (p < p1) {
                if (p == L.x) {
                    // leaf start: r - C as hi + lo (exact high parts)
                    const float4 ch = ldgf4(&tf.nodes[L.z].cHi), cl = ldgf4(&tf.nodes[L.z].cLo);
#pragma unroll
                    for (int j = 0; j < NV; ++j) {
                        const float4 rh = sRH[j][tid], rl = sRL[j][tid];
                        two_diff(rh.x, ch.x, h[j][0], l[j][0]);
                        two_diff(rh.y, ch.y, h[j][1], l[j][1]);
                        two_diff(rh.z, ch.z, h[j][2], l[j][2]);
                        l[j][0] += rl.x - cl.x;
                        l[j][1] += rl.y - cl.y;
                        l[j][2] += rl.z - cl.z;
                        pn[j][0] = pn[j][1] = pn[j][2] = pd[j] = 0.f;
                    }
                }
                const int e = min(L.y + 1, p1);
                for (int q = p - p0; q < e - p0; ++q) {
                    const float4 da = sDA[q], dl = sDL[q], m0 = sDM[3 * q], m1 = sDM[3 * q + 1],
                                 m2 = sDM[3 * q + 2];
#pragma unroll
                    for (int j = 0; j < NV; ++j)
                        leaf_pair<KIND>(law, Ls[j], LsLo[j], c1[j], ab, abl, h[j][0], h[j][1], h[j][2], l[j][0],
                                        l[j][1], l[j][2], da, dl, m0, m1, m2, pn[j][0], pn[j][1], pn[j][2], pd[j]);
                }
                p = e;
                if (e == L.y + 1) {
                    // leaf end: gate, compensated sums, heavy leaves in double-float
                    const float dn = __ldg(af.dn + L.z);
                    const unsigned size = unsigned(L.y - L.x + 1);
                    unsigned precisePairs = 0;
#pragma unroll
                    for (int j = 0; j < NV; ++j) {
                        const bool prec = leaf_close<KIND>(pn[j][0], pn[j][1], pn[j][2], pd[j], dn, h[j][0],
                                                           h[j][1], h[j][2], gv[j], sn[j], cn[j], sd[j], cd[j]);
                        if (valid[j]) {
                            cnt.leafPairs += size;
                            cnt.visited++;
                        }
                        if (prec && valid[j]) {
                            const float4 rh = sRH[j][tid], rl = sRL[j][tid];
                            const float rhv[3] = {rh.x, rh.y, rh.z}, rlv[3] = {rl.x, rl.y, rl.z};
                            precise_leaf<KIND>(tf, pf, L.z, L.x, L.y, rhv, rlv, law, Ls[j], LsLo[j], c1[j], mp.abH,
                                               mp.abL, sn[j], cn[j], sd[j], cd[j]);
                            precisePairs += size;
                        }
                    }
                    if (__any_sync(kFull, precisePairs != 0)) warp_count(counters, 6, precisePairs);
                    ++leaf;
                    if (leaf < tf.nLeaves) L = tf.leaves[leaf];
                }
            }
        }
        // the mirror's sums into the running pair (acc, the walk's layout)
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            const float4 rh = sRH[j][tid], rl = sRL[j][tid];
            const float rhv[3] = {rh.x, rh.y, rh.z}, rlv[3] = {rl.x, rl.y, rl.z};
            float4 S4 = make_float4(0.f, 0.f, 0.f, 0.f), C4 = S4;
            if (kk > 0 && valid[j]) {
                S4 = acc[2 * g[j]];
                C4 = acc[2 * g[j] + 1];
            }
            finish_mirror(af, mp, kk, rhv, rlv, sn[j], cn[j], sd[j], cd[j], S4, C4);
            if (valid[j]) {
                acc[2 * g[j]] = S4;
                acc[2 * g[j] + 1] = C4;
            }
        }
    }
    cnt.flush(counters);
}

// Exact-mode reverse product for one seed (evalNodeExact_b on the root,
// kd_tree.F90:942-1031, driven as warpDeriv.F90:71-88): every pair's weight
// as in the forward kernel, times the node's seed numb = dXv / den (reflected
// for the mirror), lands in the point's relative moments (slot 9 + a: w n_a,
// slot 3 a + k: w (r - C)_k n_a, C the leaf centroid), the layout the adjoint
// walk writes.  Each thread sums its NV nodes' products per point; the warp
// reduces them (warp_land_moments) and lands one FP64 atomic per moment.
template <int KIND, int NV>
__global__ void __launch_bounds__(kThreads) k_exact_adjoint(TreeDevF tf, PointsDevF pf, VolumeDev v, WalkRecF rec,
                                                            MixedParams mp, Law32<KIND> law, const double *dxv,
                                                            const double *den, double *ptAdj,
                                                            unsigned long long *counters) {
    const int nPts = tf.nPts;
    __shared__ float4 sDA[kTile], sDL[kTile];
    __shared__ float4 sRH[NV][kThreads], sRL[NV][kThreads];
    const int tid = threadIdx.x;
    const int64_t base = int64_t(blockIdx.x) * (kThreads * NV);
    bool valid[NV];
    int64_t g[NV];
    float Ls[NV], LsLo[NV], c1[NV];
    double q[NV];
    int vi[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        const int64_t gid = base + j * kThreads + tid;
        valid[j] = gid < v.nVol;
        g[j] = valid[j] ? gid : 0;
        vi[j] = v.perm[g[j]];
        const NodeScale ns = node_scale(rec, mp, g[j]);
        Ls[j] = ns.Ls;
        LsLo[j] = ns.LsLo;
        c1[j] = ns.c1;
        // numb = dXv / den with den in the scaled units of the weights
        q[j] = valid[j] ? exp2(-double(ns.s) * mp.bExp) / den[vi[j]] : 0.0;
    }
    const float ab = mp.abH, abl = mp.abL;
    MixedCounters cnt;
    for (int kk = 0; kk < mp.nLoop; ++kk) {
        float nb[NV][3];
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            sRH[j][tid] = rec.hi[kk * v.nVol + g[j]];
            sRL[j][tid] = rec.lo[kk * v.nVol + g[j]];
            const double *dv = dxv + 3 * int64_t(vi[j]);
#pragma unroll
            for (int a = 0; a < 3; ++a) nb[j][a] = valid[j] ? float(dv[a] * q[j]) : 0.f;
            // the transpose of the numerator reflection (getMirrorNumerator_b,
            // src/warp/initializeWarping.F90:603-635)
#pragma unroll
            for (int p = kMaxSym - 1; p >= 0; --p) {
                if (p < mp.nSym && ((kk >> p) & 1)) {
                    const float dp = nb[j][0] * mp.nrm[p][0] + nb[j][1] * mp.nrm[p][1] + nb[j][2] * mp.nrm[p][2];
                    nb[j][0] -= 2.f * dp * mp.nrm[p][0];
                    nb[j][1] -= 2.f * dp * mp.nrm[p][1];
                    nb[j][2] -= 2.f * dp * mp.nrm[p][2];
                }
            }
        }
        float h[NV][3], l[NV][3], R[NV][3];
#pragma unroll
        for (int j = 0; j < NV; ++j)
#pragma unroll
            for (int a = 0; a < 3; ++a) h[j][a] = l[j][a] = R[j][a] = 0.f;
        int leaf = 0;
        int4 L = tf.leaves[0];
        for (int p0 = 0; p0 < nPts; p0 += kTile) {
            const int p1 = min(nPts, p0 + kTile);
            __syncthreads();
            for (int t = tid; t < p1 - p0; t += kThreads) {
                sDA[t] = ldgf4(pf.da + p0 + t);
                sDL[t] = ldgf4(pf.dl + p0 + t);
            }
            __syncthreads();
            int p = p0;
            while (p < p1) {
                if (p == L.x) {
                    const float4 ch = ldgf4(&tf.nodes[L.z].cHi), cl = ldgf4(&tf.nodes[L.z].cLo);
#pragma unroll
                    for (int j = 0; j < NV; ++j) {
                        const float4 rh = sRH[j][tid], rl = sRL[j][tid];
                        two_diff(rh.x, ch.x, h[j][0], l[j][0]);
                        two_diff(rh.y, ch.y, h[j][1], l[j][1]);
                        two_diff(rh.z, ch.z, h[j][2], l[j][2]);
                        l[j][0] += rl.x - cl.x;
                        l[j][1] += rl.y - cl.y;
                        l[j][2] += rl.z - cl.z;
#pragma unroll
                        for (int a = 0; a < 3; ++a) R[j][a] = h[j][a] + l[j][a];
                    }
                }
                const int e = min(L.y + 1, p1);
                for (int t = p - p0; t < e - p0; ++t) {
                    const float4 da = sDA[t], dl = sDL[t];
                    float P[12];
#pragma unroll
                    for (int k = 0; k < 12; ++k) P[k] = 0.f;
#pragma unroll
                    for (int j = 0; j < NV; ++j) {
                        float dx, dy, dz;
                        const float w = leaf_weight<KIND>(law, Ls[j], LsLo[j], c1[j], ab, abl, h[j][0], h[j][1],
                                                          h[j][2], l[j][0], l[j][1], l[j][2], da, dl, dx, dy, dz);
#pragma unroll
                        for (int a = 0; a < 3; ++a) {
                            const float wn = w * nb[j][a];
                            P[a] += wn;
                            P[3 + a] = fmaf(wn, R[j][0], P[3 + a]);
                            P[6 + a] = fmaf(wn, R[j][1], P[6 + a]);
                            P[9 + a] = fmaf(wn, R[j][2], P[9 + a]);
                        }
                    }
                    warp_land_moments(P, ptAdj + 12 * int64_t(p0 + t));
                }
                p = e;
                if (e == L.y + 1) {
#pragma unroll
                    for (int j = 0; j < NV; ++j)
                        if (valid[j]) {
                            cnt.leafPairs += unsigned(L.y - L.x + 1);
                            cnt.visited++;
                        }
                    ++leaf;
                    if (leaf < tf.nLeaves) L = tf.leaves[leaf];
                }
            }
        }
    }
    cnt.flush(counters);
}

inline int blocks_for(int64_t n, int per) { return int((n + per - 1) / per); }

template <int KIND>
void launch_kind(const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af, const VolumeDev &v,
                 const WalkRecF &rec, const MixedParams &mp, const Law32<KIND> &law, float4 *acc,
                 unsigned long long *counters, cudaStream_t st) {
    if (blocks_for(v.nVol, kThreads * 4) >= sm_count() * kBlocksPerSmNV4)
        k_exact_mixed<KIND, 4><<<blocks_for(v.nVol, kThreads * 4), kThreads, 0, st>>>(tf, pf, af, v, rec, mp, law,
                                                                                     acc, counters);
    else
        k_exact_mixed<KIND, 2><<<blocks_for(v.nVol, kThreads * 2), kThreads, 0, st>>>(tf, pf, af, v, rec, mp, law,
                                                                                     acc, counters);
}

}  // namespace

void launch_exact_adjoint(const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v, const WalkRecF &rec,
                          const MixedParams &mp, const WeightLaw &wl, const double *dxv, const double *den,
                          double *ptAdj, unsigned long long *counters, cudaStream_t st) {
    if (v.nVol <= 0 || tf.nPts <= 0 || tf.nLeaves <= 0) return;
    constexpr int NV = 4;
    const int grid = blocks_for(v.nVol, kThreads * NV);
    if (wl.isInt && wl.ia == 3 && wl.ib == 5) {
        k_exact_adjoint<0, NV><<<grid, kThreads, 0, st>>>(tf, pf, v, rec, mp, Law32<0>{3, 5, 3.f, 5.f}, dxv, den,
                                                          ptAdj, counters);
    } else if (wl.isInt) {
        k_exact_adjoint<1, NV><<<grid, kThreads, 0, st>>>(
            tf, pf, v, rec, mp, Law32<1>{wl.ia, wl.ib, float(wl.aExp), float(wl.bExp)}, dxv, den, ptAdj, counters);
    } else {
        k_exact_adjoint<2, NV><<<grid, kThreads, 0, st>>>(
            tf, pf, v, rec, mp, Law32<2>{0, 0, float(wl.aExp), float(wl.bExp)}, dxv, den, ptAdj, counters);
    }
}

bool exact_tiled_fills(int64_t nVol) {
    return blocks_for(nVol, kThreads * 4) >= 2 * sm_count() * kBlocksPerSmNV4;
}

void launch_exact_mixed(const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af, const VolumeDev &v,
                        const WalkRecF &rec, const MixedParams &mp, const WeightLaw &wl, float4 *acc,
                        unsigned long long *counters, cudaStream_t st) {
    if (v.nVol <= 0 || tf.nPts <= 0 || tf.nLeaves <= 0) return;
    if (wl.isInt && wl.ia == 3 && wl.ib == 5) {
        launch_kind<0>(tf, pf, af, v, rec, mp, Law32<0>{3, 5, 3.f, 5.f}, acc, counters, st);
    } else if (wl.isInt) {
        launch_kind<1>(tf, pf, af, v, rec, mp, Law32<1>{wl.ia, wl.ib, float(wl.aExp), float(wl.bExp)}, acc, counters, st);
    } else {
        launch_kind<2>(tf, pf, af, v, rec, mp, Law32<2>{0, 0, float(wl.aExp), float(wl.bExp)}, acc, counters, st);
    }
}

}  // namespace idw
