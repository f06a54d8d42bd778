// Recorded walk decisions and their replay (mixed fast mode).
//
// Every open/approximate decision of the fast walk depends on set-up state
// only: the mirrored initial volume point, the cluster's centroid and radius
// (from Xu0), its error table (the init-time weight law), the denominator
// estimate den0 and errTol (kd_tree.F90:619-662, 882-906).  The surface
// coordinates enter the sums only through the motions (M_i, b_i), never the
// decisions.  So the decisions are taken once - the decision walk of
// idw_mixed.cu, decide32 with the FP64 re-take - and recorded per warp of 32
// Morton-ordered volume nodes and per mirror as the warp's work list: in walk
// order, every tree node where at least one lane approximates a cluster or
// sums a leaf, with the mask of those lanes.  Interior steps where every lane
// opens (or is inside a subtree it already skipped) carry no work and are not
// recorded.
//
// The replay walks a warp's list: the same terms, evaluated by the same
// device functions (cluster_geo, approx_step, leaf_step) in the same order,
// so the sums are bitwise those of the decision walk, without the per-visit
// decision (error-table interpolation, guard bands, FP64 votes) or the
// traversal's dependent loads.
//
// Entry: int2 {node | 0x80000000 for a leaf, lane mask}.  Lists of warp w,
// mirror kk: [offs[w nLoop + kk], offs[w nLoop + kk + 1]).
#include <climits>

#include <cub/cub.cuh>

#include "idw_mixed.cuh"
#include "idwarp_gb300.h"

namespace idw {

namespace {

#ifndef IDW_WALK_MIN_BLOCKS
#define IDW_WALK_MIN_BLOCKS 8
#endif

constexpr int kLeafBit = int(0x80000000u);

// MODE 0: count each warp's entries per mirror into counts; MODE 1: write them
// at offs.  The traversal and decisions are k_walk_mixed's (fast mode).
template <int MODE>
__global__ void __launch_bounds__(128, IDW_WALK_MIN_BLOCKS)
    k_walk_record(TreeDev t, TreeDevF tf, VolumeDev v, WalkRecF rec, MixedParams mp, int64_t nWarps, int64_t *counts,
                  const int64_t *offs, int2 *list, unsigned long long *counters) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t warp = gid >> 5;
    if (warp >= nWarps) return;  // whole warps only
    const int lane = threadIdx.x & 31;
    const bool valid = gid < v.nVol;
    const int64_t g = valid ? gid : 0;
    const float tauf = mp.errTolF * rec.hi[g].w;
    MixedCounters cnt;
    for (int kk = 0; kk < mp.nLoop; ++kk) {
        const float4 rhi = rec.hi[kk * v.nVol + g], rlo = rec.lo[kk * v.nVol + g];
        const float rh[3] = {rhi.x, rhi.y, rhi.z}, rl[3] = {rlo.x, rlo.y, rlo.z};
        int64_t pos = MODE ? offs[warp * mp.nLoop + kk] : 0;
        int node = 0, skip = 0;
        while (node < t.nNodes) {
            const int4 inf = ldgi4(&tf.nodes[node].info);
            const bool active = valid && node >= skip;
            if (inf.w) {
                const unsigned m = __ballot_sync(kFull, active);
                if (m) {
                    if (MODE && lane == 0) list[pos] = make_int2(node | kLeafBit, int(m));
                    ++pos;
                }
                if (active) {
                    cnt.leafPairs += inf.y - inf.x + 1;
                    cnt.visited++;
                }
                node = inf.z;
            } else {
                int dec = 0;
                float rho0, rho1, rho2, d2, rs, wA;
                if (active) {
                    cnt.visited++;
                    dec = decide32(tf, node, rh, rl, tauf, rho0, rho1, rho2, d2, rs, wA);
                }
                dec = resolve64(dec, t, v, g, node, rh, rl, mp.errTol, MODE ? counters : nullptr);
                const unsigned m = __ballot_sync(kFull, dec == 1);
                if (m) {
                    if (MODE && lane == 0) list[pos] = make_int2(node, int(m));
                    ++pos;
                }
                bool open = false;
                if (dec == 1) {
                    skip = inf.z;
                    cnt.approx++;
                } else if (active) {
                    open = true;
                }
                node = __any_sync(kFull, open) ? node + 1 : inf.z;
            }
        }
        if (!MODE && lane == 0) counts[warp * mp.nLoop + kk] = pos;
    }
    if (MODE) cnt.flush(counters);
}

// The forward sums of every volume node from its warp's recorded lists
// (k_walk_mixed's arithmetic and order; fills acc like the walk).
template <int KIND>
__global__ void __launch_bounds__(128, IDW_WALK_MIN_BLOCKS)
    k_walk_replay(TreeDevF tf, PointsDevF pf, NodeAggF af, VolumeDev v, WalkRecF rec, MixedParams mp,
                  Law32<KIND> law, int64_t nWarps, const int64_t *offs, const int2 *list, float4 *acc,
                  unsigned long long *counters) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t warp = gid >> 5;
    if (warp >= nWarps) return;  // whole warps only
    const unsigned lane = threadIdx.x & 31;
    const bool valid = gid < v.nVol;
    const int64_t g = valid ? gid : 0;
    const NodeScale ns = node_scale(rec, mp, g);
    const WalkLane<KIND> wl = {law, ns.Ls, ns.LsLo, ns.c1, mp.abH, mp.abL, ns.gv};
    // running sums over the mirrors, in shared memory between mirror passes
    __shared__ float4 mirS[128], mirC[128];
    mirS[threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    mirC[threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int kk = 0; kk < mp.nLoop; ++kk) {
        const float4 rhi = rec.hi[kk * v.nVol + g], rlo = rec.lo[kk * v.nVol + g];
        const float rh[3] = {rhi.x, rhi.y, rhi.z}, rl[3] = {rlo.x, rlo.y, rlo.z};
        Sums2 rs2 = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        const int64_t e1 = offs[warp * mp.nLoop + kk + 1];
        for (int64_t e = offs[warp * mp.nLoop + kk]; e < e1; ++e) {
            const int2 ent = __ldg(list + e);
            const int node = ent.x & ~kLeafBit;
            const bool mine = (unsigned(ent.y) >> lane) & 1u;
            // the node's replay record: one 128-byte line
            const float4 *rr = af.rr + 8 * int64_t(node);
            if (ent.x < 0) {
                leaf_step<KIND>(mine, tf, pf, node, __float_as_int(__ldg(&rr[1].w)), __float_as_int(__ldg(&rr[2].x)),
                                rr, rr + 1, &rr[0].w, rh, rl, wl, rs2, counters);
            } else {
                const float4 c0 = ldgf4(rr), c1 = ldgf4(rr + 1);
                float rho0, rho1, rho2, d2, rs, wA;
                cluster_geo(c0, c1, rh, rl, rho0, rho1, rho2, d2, rs, wA);
                bool precise = false;
                if (mine) precise = approx_add<KIND>(ldgf4(rr + 2), ldgf4(rr + 3), ldgf4(rr + 4), c0.w, rho0, rho1,
                                                     rho2, rs, wA, wl, rs2);
                approx_vote<KIND>(precise, tf, af, node, rh, rl, wl, rs2, counters);
            }
        }
        float4 S4 = mirS[threadIdx.x], C4 = mirC[threadIdx.x];
        const RunSums fin = to_runsums(rs2);
        finish_mirror(af, mp, kk, rh, rl, fin.sn, fin.cn, fin.sd, fin.cd, S4, C4);
        mirS[threadIdx.x] = S4;
        mirC[threadIdx.x] = C4;
    }
    if (valid) {
        acc[2 * gid] = mirS[threadIdx.x];
        acc[2 * gid + 1] = mirC[threadIdx.x];
    }
}

__global__ void k_add_counters(int n, const unsigned long long *src, unsigned long long *dst) {
    if (int(threadIdx.x) < n) dst[threadIdx.x] += src[threadIdx.x];
}

inline int blocks(int64_t n, int b) { return int((n + b - 1) / b); }

template <int KIND>
void replay_kind(const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af, const VolumeDev &v,
                 const WalkRecF &rec, const MixedParams &mp, const Law32<KIND> &law, const int64_t *offs,
                 const int2 *list, float4 *acc, unsigned long long *counters, cudaStream_t st) {
    const int64_t nWarps = walk_list_warps(v.nVol);
    k_walk_replay<KIND><<<blocks(v.nVol, 128), 128, 0, st>>>(tf, pf, af, v, rec, mp, law, nWarps, offs, list, acc,
                                                             counters);
}

}  // namespace

int64_t walk_list_warps(int64_t nVol) { return (nVol + 31) / 32; }

void launch_add_walk_counters(unsigned long long *dst, const unsigned long long *src, cudaStream_t st) {
    if (dst && src) k_add_counters<<<1, 32, 0, st>>>(4, src, dst);
}

int64_t count_walk_lists(const TreeDev &t, const TreeDevF &tf, const VolumeDev &v, const WalkRecF &rec,
                         const EvalConsts &k, int64_t *offs, cudaStream_t st) {
    const MixedParams mp = make_mixed_params(k);
    const int64_t nWarps = walk_list_warps(v.nVol);
    const int64_t n = nWarps * mp.nLoop;
    if (n <= 0) return 0;
    if (n + 1 > int64_t(INT_MAX)) return -1;
    WalkRecF r0 = rec;
    r0.gden = nullptr;
    int64_t *counts = nullptr;
    void *tmp = nullptr;
    size_t tmpBytes = 0;
    int64_t total = -1;
    bool ok = cudaMalloc(&counts, sizeof(int64_t) * (n + 1)) == cudaSuccess;
    if (ok) ok = cudaMemsetAsync(counts + n, 0, sizeof(int64_t), st) == cudaSuccess;
    if (ok) {
        k_walk_record<0><<<blocks(v.nVol, 128), 128, 0, st>>>(t, tf, v, r0, mp, nWarps, counts, nullptr, nullptr,
                                                              nullptr);
        ok = cudaGetLastError() == cudaSuccess;
    }
    if (ok) ok = cub::DeviceScan::ExclusiveSum(nullptr, tmpBytes, counts, offs, int(n + 1), st) == cudaSuccess;
    if (ok) ok = cudaMalloc(&tmp, tmpBytes) == cudaSuccess;
    if (ok) ok = cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, counts, offs, int(n + 1), st) == cudaSuccess;
    if (ok) ok = cudaMemcpyAsync(&total, offs + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (cudaStreamSynchronize(st) != cudaSuccess) ok = false;
    if (tmp) cudaFree(tmp);
    if (counts) cudaFree(counts);
    return ok ? total : -1;
}

void launch_walk_record(const TreeDev &t, const TreeDevF &tf, const VolumeDev &v, const WalkRecF &rec,
                        const EvalConsts &k, const int64_t *offs, int2 *list, unsigned long long *counters,
                        cudaStream_t st) {
    const MixedParams mp = make_mixed_params(k);
    const int64_t nWarps = walk_list_warps(v.nVol);
    if (nWarps <= 0) return;
    WalkRecF r0 = rec;
    r0.gden = nullptr;
    k_walk_record<1><<<blocks(v.nVol, 128), 128, 0, st>>>(t, tf, v, r0, mp, nWarps, nullptr, offs, list, counters);
}

void launch_walk_replay(const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af, const VolumeDev &v,
                        const WalkRecF &rec, const EvalConsts &k, float4 *acc, unsigned long long *counters,
                        cudaStream_t st) {
    if (v.nVol <= 0) return;
    const MixedParams mp = make_mixed_params(k);
    if (k.law.isInt && k.law.ia == 3 && k.law.ib == 5)
        replay_kind(tf, pf, af, v, rec, mp, Law32<0>{3, 5, 3.f, 5.f}, k.lists.offs, k.lists.list, acc, counters, st);
    else if (k.law.isInt)
        replay_kind(tf, pf, af, v, rec, mp, Law32<1>{k.law.ia, k.law.ib, float(k.law.aExp), float(k.law.bExp)},
                    k.lists.offs, k.lists.list, acc, counters, st);
    else
        replay_kind(tf, pf, af, v, rec, mp, Law32<2>{0, 0, float(k.law.aExp), float(k.law.bExp)}, k.lists.offs,
                    k.lists.list, acc, counters, st);
}

}  // namespace idw
