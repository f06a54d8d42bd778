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
