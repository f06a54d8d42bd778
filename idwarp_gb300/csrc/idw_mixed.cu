// Mixed-precision evaluation of the IDW sums (the product path of warpMesh).
//
// Same warp-cooperative preorder walk as the FP64 form (idw_walk.cu), with the
// per-pair work in FP32:
//   * geometry relative to the visited cluster: r - C is formed from the
//     double-float split of r and of the centroid C, then rounded once to FP32,
//     and leaf points are stored as FP32 offsets from their leaf centroid, so a
//     pair distance never loses digits to the absolute coordinates;
//   * S_i = M_i r + b_i - r is evaluated as D_i (r - Xu0_i) + u_i with
//     D_i = M_i - I and u_i = M_i Xu0_i + b_i - Xu0_i (small quantities);
//   * weights are scaled by sigma^b with sigma = 2^s chosen per volume node
//     from its denominator estimate, so (L/d)^b stays in FP32 range (the ratio
//     num/den is unchanged; powers of two scale exactly);
//   * each leaf's partial sums are added to compensated (two-sum) FP32 running
//     sums; normalisation and the add-back to Xv0 are FP64.
// Open/approximate decisions are taken in FP32 only when they are further
// from the threshold than the FP32 error bound; otherwise they are re-taken
// with the FP64 decision of the FP64 form (decide64), so the mixed walk makes
// exactly the FP64 walk's decisions.
#include "idw_mixed.cuh"
#include "idwarp_gb300.h"

namespace idw {

namespace {

// Resident blocks per SM the register allocation targets (128 threads each).
#ifndef IDW_WALK_MIN_BLOCKS
#define IDW_WALK_MIN_BLOCKS 8
#endif

// STATS: count warp-level lane slots (diagnostics); EXACT: exact mode (every
// leaf, no decisions).  Both are compile-time so that the product walk's loop
// carries neither test.
template <int KIND, int STATS, int EXACT>
__global__ void __launch_bounds__(128, IDW_WALK_MIN_BLOCKS) k_walk_mixed(TreeDev t, TreeDevF tf, PointsDevF pf, NodeAggF af,
                                                    VolumeDev v, WalkRecF rec, MixedParams mp, Law32<KIND> law,
                                                    float4 *acc, unsigned long long *counters) {
    constexpr int exact = EXACT;
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = gid < v.nVol;
    const int64_t g = valid ? gid : 0;
    // per-node scale sigma = 2^s (set-up constant, stored with the record),
    // FP32 decision tolerance and precision gate
    const NodeScale ns = node_scale(rec, mp, g);
    const float Ls = ns.Ls, LsLo = ns.LsLo, c1 = ns.c1, tauf = ns.tauf, gv = ns.gv;
    const float ab = mp.abH, abl = mp.abL;
    // running sums over the mirrors (sum = S + C per component), kept in shared
    // memory between mirror passes to free registers for the walk
    __shared__ float4 mirS[128], mirC[128];
    mirS[threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    mirC[threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    MixedCounters cnt;
    const WalkLane<KIND> wl = {law, Ls, LsLo, c1, ab, abl, gv};
    for (int kk = 0; kk < mp.nLoop; ++kk) {
        const float4 rhi = rec.hi[kk * v.nVol + g], rlo = rec.lo[kk * v.nVol + g];
        const float rh[3] = {rhi.x, rhi.y, rhi.z}, rl[3] = {rlo.x, rlo.y, rlo.z};
        Sums2 rs2 = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        int node = 0, skip = 0;
        while (node < t.nNodes) {
            const int4 inf = ldgi4(&tf.nodes[node].info);
            const bool active = valid && node >= skip;
            if (STATS && __any_sync(kFull, active) && counters && (threadIdx.x & 31) == 0)
                atomicAdd(counters + (inf.w ? 4 : 5), (unsigned long long)(inf.w ? 32 * (inf.y - inf.x + 1) : 32));
            if (inf.w) {
                leaf_step<KIND>(active, tf, pf, node, inf.x, inf.y, &tf.nodes[node].cHi, &tf.nodes[node].cLo,
                                af.dn + node, rh, rl, wl, rs2, counters);
                if (active) {
                    cnt.leafPairs += inf.y - inf.x + 1;
                    cnt.visited++;
                }
                node = inf.z;
            } else {
                int dec = 0;  // 0 open, 1 approximate, 2 undecided in FP32
                float rho0 = 0.f, rho1 = 0.f, rho2 = 0.f, d2 = 0.f, rs = 0.f, wA = 0.f;
                if (active && !exact) {
                    cnt.visited++;
                    dec = decide32(tf, node, rh, rl, tauf, rho0, rho1, rho2, d2, rs, wA);
                }
                dec = resolve64(dec, t, v, g, node, rh, rl, mp.errTol, counters);
                approx_step<KIND>(dec == 1, tf, af, node, rho0, rho1, rho2, rs, wA, rh, rl, wl, rs2, counters);
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
    cnt.flush(counters);
}

// Normalisation and add-back in FP64: Xv = Xv0 + num/den, and the true-unit
// denominator den/sigma^b for the derivative.
__global__ void k_finalize_mixed(VolumeDev v, WalkRecF rec, const float4 *acc, double bExp, int tangent, double *xv,
                                 double *den) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= v.nVol) return;
    const int vi = v.perm[gid];
    const float4 a = acc[2 * gid], c = acc[2 * gid + 1];
    const double N0 = double(a.x) + double(c.x), N1 = double(a.y) + double(c.y), N2 = double(a.z) + double(c.z);
    const double D = double(a.w) + double(c.w);
    const double oden = 1.0 / D;
    if (xv) {
        // tangent mode: the derivative numerator over the (same) denominator
        const double b0 = tangent ? 0.0 : v.xv0[3 * vi + 0], b1 = tangent ? 0.0 : v.xv0[3 * vi + 1],
                     b2 = tangent ? 0.0 : v.xv0[3 * vi + 2];
        xv[3 * vi + 0] = b0 + N0 * oden;
        xv[3 * vi + 1] = b1 + N1 * oden;
        xv[3 * vi + 2] = b2 + N2 * oden;
    }
    if (den) {
        const int s = __float_as_int(rec.lo[gid].w);
        den[vi] = D * exp2(-double(s) * bExp);
    }
}

// Set-up: FP32 walk records of every volume node in Morton order and every
// mirror: the double-float split of the mirrored point, the denominator
// estimate and the node's weight-scale exponent s (sigma = 2^s, sigma^b ~ 1/den0).
__global__ void k_walk_records(VolumeDev v, SymPlanes sym, double bExp, float4 *hi, float4 *lo) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= v.nVol) return;
    const int vi = v.perm[gid];
    const double x0[3] = {v.xv0[3 * vi], v.xv0[3 * vi + 1], v.xv0[3 * vi + 2]};
    const double den0 = v.den0[vi];
    int s = 0;
    if (den0 > 0.0 && den0 < 1e300) s = max(-40, min(40, int(rint(-double(ilogb(den0)) / bExp))));
    const float den0f = float(fmin(den0, 3.0e38));
    for (int kk = 0; kk < sym.nLoop; ++kk) {
        double r[3];
        mirror_point(sym, kk, x0, r);
        float h[3], l[3];
        for (int c = 0; c < 3; ++c) {
            h[c] = float(r[c]);
            l[c] = float(r[c] - double(h[c]));
        }
        hi[kk * v.nVol + gid] = make_float4(h[0], h[1], h[2], den0f);
        lo[kk * v.nVol + gid] = make_float4(l[0], l[1], l[2], __int_as_float(s));
    }
}

__global__ void k_gate_den(int64_t nVol, const float4 *acc, float *gden) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= nVol) return;
    gden[gid] = acc[2 * gid].w + acc[2 * gid + 1].w;
}

inline int blocks(int64_t n, int b) { return int((n + b - 1) / b); }

template <int KIND>
void launch_walk_kind(int g, const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af,
                      const VolumeDev &v, const WalkRecF &rec, const MixedParams &mp, const Law32<KIND> &law,
                      int exact, float4 *acc, unsigned long long *counters, cudaStream_t st) {
    if (mp.slotStats) {
        if (exact)
            k_walk_mixed<KIND, 1, 1><<<g, 128, 0, st>>>(t, tf, pf, af, v, rec, mp, law, acc, counters);
        else
            k_walk_mixed<KIND, 1, 0><<<g, 128, 0, st>>>(t, tf, pf, af, v, rec, mp, law, acc, counters);
    } else {
        if (exact)
            k_walk_mixed<KIND, 0, 1><<<g, 128, 0, st>>>(t, tf, pf, af, v, rec, mp, law, acc, counters);
        else
            k_walk_mixed<KIND, 0, 0><<<g, 128, 0, st>>>(t, tf, pf, af, v, rec, mp, law, acc, counters);
    }
}

}  // namespace

void launch_finalize_mixed(const VolumeDev &v, const WalkRecF &rec, const float4 *acc, double bExp, double *xv,
                           cudaStream_t st, int tangent) {
    if (v.nVol > 0) k_finalize_mixed<<<blocks(v.nVol, 256), 256, 0, st>>>(v, rec, acc, bExp, tangent, xv, nullptr);
}

void launch_gate_den(int64_t nVol, const float4 *acc, float *gden, cudaStream_t st) {
    if (nVol > 0) k_gate_den<<<blocks(nVol, 256), 256, 0, st>>>(nVol, acc, gden);
}

MixedParams make_mixed_params(const EvalConsts &k) {
    MixedParams mp;
    mp.nLoop = k.sym.nLoop;
    mp.nSym = k.sym.n;
    for (int j = 0; j < kMaxSym; ++j)
        for (int c = 0; c < 3; ++c) {
            mp.nrm[j][c] = j < k.sym.n ? float(k.sym.nrm[j][c]) : 0.f;
            mp.nrmLo[j][c] = j < k.sym.n ? float(k.sym.nrm[j][c] - double(mp.nrm[j][c])) : 0.f;
        }
    mp.LdefF = float(k.law.Ldef);
    mp.LdefLo = float(k.law.Ldef - double(mp.LdefF));
    mp.alphaToBexpF = float(k.law.alphaToBexp);
    mp.abH = mp.alphaToBexpF;
    mp.abL = float(k.law.alphaToBexp - double(mp.abH));
    mp.precGate = float(k.precGate);
    mp.errTolF = float(k.errTol);
    mp.errTol = k.errTol;
    mp.intExp = k.law.isInt;
    mp.dExp = k.law.ib - k.law.ia;
    mp.dExpF = float(k.law.bExp - k.law.aExp);
    mp.slotStats = k.slotStats;
    mp.bExp = k.law.bExp;
    mp.bExpF = float(k.law.bExp);
    return mp;
}

void launch_walk_records(const VolumeDev &v, const SymPlanes &sym, double bExp, float4 *hi, float4 *lo,
                         cudaStream_t st) {
    if (v.nVol > 0) k_walk_records<<<blocks(v.nVol, 256), 256, 0, st>>>(v, sym, bExp, hi, lo);
}

void launch_walk_mixed(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af,
                       const VolumeDev &v, const WalkRecF &rec, const EvalConsts &k, int exact, float4 *acc,
                       const WalkOut &o, cudaStream_t st) {
    if (v.nVol <= 0) return;
    const int g = blocks(v.nVol, 128);
    const MixedParams mp = make_mixed_params(k);
    if (exact && tf.nLeaves > 0 && !mp.slotStats && k.exactSchedule != IDW_EXACT_WALK &&
        (k.exactSchedule == IDW_EXACT_TILED || exact_tiled_fills(v.nVol))) {
        // every pair: the tiled kernel, with the walk's arithmetic
        launch_exact_mixed(tf, pf, af, v, rec, mp, k.law, acc, o.counters, st);
    } else if (!exact && k.lists.list && !mp.slotStats) {
        // recorded decisions: the walk's terms without the walk's decisions;
        // the work counters are the recording walk's
        launch_add_walk_counters(o.counters, k.lists.counters, st);
        launch_walk_replay(tf, pf, af, v, rec, k, acc, o.counters, st);
    } else if (k.law.isInt && k.law.ia == 3 && k.law.ib == 5) {
        launch_walk_kind(g, t, tf, pf, af, v, rec, mp, Law32<0>{3, 5, 3.f, 5.f}, exact, acc, o.counters, st);
    } else if (k.law.isInt) {
        launch_walk_kind(g, t, tf, pf, af, v, rec, mp, Law32<1>{k.law.ia, k.law.ib, float(k.law.aExp), float(k.law.bExp)},
                         exact, acc, o.counters, st);
    } else {
        launch_walk_kind(g, t, tf, pf, af, v, rec, mp, Law32<2>{0, 0, float(k.law.aExp), float(k.law.bExp)}, exact,
                         acc, o.counters, st);
    }
    k_finalize_mixed<<<blocks(v.nVol, 256), 256, 0, st>>>(v, rec, acc, k.law.bExp, o.tangent, o.xv,
                                                          o.tangent ? nullptr : o.den);
}

}  // namespace idw
