// Precise form of the mixed reverse walk (warpDeriv), and the walk that gives
// it an accurate denominator.
//   evalNode_b / evalNodeExact_b / evalNodeApprox_b  src/modules/kd_tree.F90:942-1031
//   driven as warpDeriv                              src/warp/warpDeriv.F90:71-88
//
// The FP32 reverse walk (idw_adjoint.cu) forms each weight, each product
// w numb and each lane sum in FP32.  A weight (L/d)^b in FP32 carries a
// relative error of a few 1e-7 (the rounding of d^2 raised to the power
// b/2), so the point adjoints do too, and the rotation adjoint of the nodal
// properties amplifies the moment adjoints' errors at nodes that barely
// rotate.  Here every term is evaluated in double-float (hi + lo FP32 pairs,
// about 44 bits): the weight by precise_weight (the forward walk's
// double-float term), the seeds dXv / den split in two floats from FP64, the
// products v (x) numb by error-free products, and the sums over the lanes of
// a warp by double-float additions; each lane sum lands in the FP64
// accumulators by an FP64 atomic of its two parts.  The decisions are the
// mixed walk's (decide32 + resolve64), so the terms are the reference's.
//
// numb needs den to the same accuracy: the FP32 walk's denominator carries the
// FP32 weights' error.  S = 0 instantiates the same walk as a denominator
// walk (double-float weights, compensated per-lane sums, no seeds); den
// depends on the initial surface and the weight law only, so it is computed
// once per law and kept.
#include "idw_mixed.cuh"
#include "idwarp_gb300.h"

namespace idw {

namespace {

// Shared-memory targets of a batch of cluster terms (batches of more than two
// terms); for two, the kernel keeps them in registers: 16 seeds fill shared
// memory to exactly four blocks per SM, and 8 more bytes per warp make it three.
template <bool SMEM, int KP>
struct PrecTargets {
    int tgt[KP];  // tree nodes of a batch of cluster terms
};
template <int KP>
struct PrecTargets<false, KP> {};

#ifndef IDW_PREC_KP16
#define IDW_PREC_KP16 2
#endif

template <int S>
struct PrecSmem : PrecTargets<(S > 0 && (S <= 4 ? 10 : IDW_PREC_KP16) > 2), (S <= 4 ? 10 : IDW_PREC_KP16)> {
    static constexpr int kC = S > 0 ? 3 * S : 1;
    // leaf points reduced per shared-memory pass: a whole leaf of the default
    // bucket (up to 9 points) in one pass for few seeds; 2 for 16 seeds, whose
    // seed arrays fill shared memory (per warp 20 KB with 8 points: two blocks
    // per SM; 16 KB with 4: three; 14 KB with 2: four; 726, 586 and 527 ms at
    // 8M nodes)
    static constexpr int kP = S == 0 ? 1 : (S <= 4 ? 10 : IDW_PREC_KP16);
    float nh[32][kC], nl[32][kC];      // seeds of every lane (numb, scaled), hi / lo
    float4 vh[kP][32], vl[kP][32];     // per term: w, w (r - C), hi / lo
};

template <int S>
__host__ __device__ constexpr bool prec_smem_targets() {
    return S > 0 && PrecSmem<S>::kP > 2;
}
// 16 seeds at two points per pass: 14 KB per warp, four blocks per SM
static_assert(IDW_PREC_KP16 != 2 || sizeof(PrecSmem<16>) == 2 * 32 * 48 * 4 + 2 * 2 * 32 * 16,
              "the 16-seed shared-memory layout sets the occupancy");

// Terms wait in vh / vl until kP of them (or the end of the mirror pass) and
// are reduced together, one task per (term, seed component), instead of one
// reduction per cluster term and per leaf (whose few points leave task lanes
// idle).  IDW_PREC_CBATCH: 0 none, 1 cluster terms (flushed at each leaf), 2
// every term.
#ifndef IDW_PREC_CBATCH
#define IDW_PREC_CBATCH 2
#endif

// acc += a * b in double-float (error-free product, then two-sum).
__device__ __forceinline__ void df_fma_acc(dfl &acc, dfl a, dfl b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
    float s, t;
    two_sum(acc.h, p, s, t);
    acc.l += t + e;
    acc.h = s;
}

template <bool DET>
__device__ __forceinline__ void land_df(double *d, dfl v) {
    if (v.h != 0.f || v.l != 0.f) land_add<DET>(d, double(v.h) + double(v.l));
}

// Reduction of m terms (vh/vl[0..m)) against the lanes' seeds: one (term,
// seed component) pair per lane task, each summing the 32 lanes in
// double-float; lands w -> slot 9 + a and w (r - C) -> slots 3 a .. 3 a + 2.
// batch: the terms are a batch, targets in sm.tgt (or bt0, bt1 for batches of
// at most two): a point index, or ~node for a cluster term (landed in nodeAdj);
// otherwise points base .. base + m - 1.
template <int S, bool DET>
__device__ __forceinline__ void reduce_tasks_df(PrecSmem<S> &sm, int m, int base, double *adj, int64_t seedStride,
                                                bool batch = false, int bt0 = 0, int bt1 = 0,
                                                double *nodeAdj = nullptr, int64_t nodeStride = 0) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    for (int task = lane; task < 3 * S * m; task += 32) {
        const int p = task / (3 * S), c = task - p * (3 * S);
        dfl a0 = {0.f, 0.f}, a1 = {0.f, 0.f}, a2 = {0.f, 0.f}, a3 = {0.f, 0.f};
        for (int l0 = 0; l0 < 32; ++l0) {
            const int l = (l0 + p) & 31;
            const dfl n = {sm.nh[l][c], sm.nl[l][c]};
            const float4 vh = sm.vh[p][l], vl = sm.vl[p][l];
            df_fma_acc(a0, {vh.x, vl.x}, n);
            df_fma_acc(a1, {vh.y, vl.y}, n);
            df_fma_acc(a2, {vh.z, vl.z}, n);
            df_fma_acc(a3, {vh.w, vl.w}, n);
        }
        const int s = c / 3, a = c - 3 * s;
        int tg = base + p;
        if (batch) {
            if constexpr (prec_smem_targets<S>()) tg = sm.tgt[p];
            else tg = p == 0 ? bt0 : bt1;
        }
        double *d = tg >= 0 ? adj + s * seedStride + 12 * int64_t(tg) : nodeAdj + s * nodeStride + 12 * int64_t(~tg);
        land_df<DET>(d + 9 + a, a0);
        land_df<DET>(d + 3 * a + 0, a1);
        land_df<DET>(d + 3 * a + 1, a2);
        land_df<DET>(d + 3 * a + 2, a3);
    }
    __syncwarp();
}

// One seed, one term: the 12 products v (x) n summed over the warp in
// double-float (two halving exchanges, then three butterflies, as
// warp_land_moments), landed by lanes 0..2 of each lane group.
template <bool DET>
__device__ __forceinline__ void land_one_df(const dfl v[4], const dfl n[3], double *d) {
    const int lane = threadIdx.x & 31;
    dfl P[12];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            P[3 * k + a] = {0.f, 0.f};
            df_fma_acc(P[3 * k + a], v[k], n[a]);
        }
    const bool h16 = lane & 16, h8 = lane & 8;
    dfl Q[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const dfl send = h16 ? P[k] : P[k + 6];
        const dfl keep = h16 ? P[k + 6] : P[k];
        const dfl got = {__shfl_xor_sync(kFull, send.h, 16), __shfl_xor_sync(kFull, send.l, 16)};
        Q[k] = df_add(keep, got);
    }
    dfl R[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const dfl send = h8 ? Q[k] : Q[k + 3];
        const dfl keep = h8 ? Q[k + 3] : Q[k];
        const dfl got = {__shfl_xor_sync(kFull, send.h, 8), __shfl_xor_sync(kFull, send.l, 8)};
        R[k] = df_add(keep, got);
    }
#pragma unroll
    for (int o = 4; o; o >>= 1)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const dfl got = {__shfl_xor_sync(kFull, R[k].h, o), __shfl_xor_sync(kFull, R[k].l, o)};
            R[k] = df_add(R[k], got);
        }
    const int G = lane >> 3, a = lane & 7;
    if (a < 3) land_df<DET>(d + (G == 0 ? 9 + a : 3 * a + G - 1), a == 0 ? R[0] : (a == 1 ? R[1] : R[2]));
}

// (r - C) of a lane as a double-float per axis: exact high-part differences
// plus the low parts of r and C, renormalised (|lo| <= ulp(hi) / 2, which the
// double-float products assume).
__device__ __forceinline__ void rel_df(const float *rh, const float *rl, float4 ch, float4 cl, dfl q[3]) {
    two_diff(rh[0], ch.x, q[0].h, q[0].l);
    two_diff(rh[1], ch.y, q[1].h, q[1].l);
    two_diff(rh[2], ch.z, q[2].h, q[2].l);
    q[0].l += rl[0] - cl.x;
    q[1].l += rl[1] - cl.y;
    q[2].l += rl[2] - cl.z;
#pragma unroll
    for (int k = 0; k < 3; ++k) two_sum(q[k].h, q[k].l, q[k].h, q[k].l);
}

// v = (w, w x) in double-float from the weight (wh, wl) and the offset x.
__device__ __forceinline__ void term_vector(float wh, float wl, const dfl x[3], dfl v[4]) {
    v[0] = df_norm(wh, wl);
#pragma unroll
    for (int k = 0; k < 3; ++k) v[k + 1] = df_mul(v[0], x[k]);
}

// S > 0: S seeds (dxv, common order, stride dxvStride) into ptAdj / nodeAdj.
// S = 0: the denominator walk; denOut receives sum w in true units (common order).
// REPLAY: walk the recorded decisions (idw_replay.cu) instead of deciding.
// DET: order-independent landings (idw_land.cuh).
template <int S, int KIND, int REPLAY, bool DET = false>
__global__ void __launch_bounds__(128) k_adjoint_precise(TreeDev t, TreeDevF tf, PointsDevF pf, VolumeDev v,
                                                         WalkRecF rec, MixedParams mp, Law32<KIND> law, int exact,
                                                         const double *dxv, int64_t dxvStride, const double *den,
                                                         double *ptAdj, int64_t ptStride, double *nodeAdj,
                                                         int64_t nodeStride, double *denOut,
                                                         unsigned long long *counters, WalkLists wlists) {
    extern __shared__ __align__(16) unsigned char smraw[];
    PrecSmem<S> &sm = reinterpret_cast<PrecSmem<S> *>(smraw)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = gid < v.nVol;
    const int64_t g = valid ? gid : 0;
    const int vi = v.perm[g];
    const int s = __float_as_int(rec.lo[g].w);
    const float den0f = rec.hi[g].w;
    const float Ls = mp.LdefF * pow2f(s);
    const float LsLo = mp.LdefLo * pow2f(s);
    const float c1 = mp.intExp ? pow2f(s * mp.dExp) : exp2f(float(s) * mp.dExpF);
    const float tauf = mp.errTolF * den0f;
    // numb = dXv / den with den in the scaled units of the walk's weights
    const double q = (S > 0 && valid) ? exp2(-double(s) * mp.bExp) / den[vi] : 0.0;
    MixedCounters cnt;
    float dsum = 0.f, dcomp = 0.f;  // S = 0: this lane's denominator (all mirrors)
    dfl nl1[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};  // S = 1: this lane's seed
    int npend = 0, pt0 = 0, pt1 = 0;  // terms waiting in sm.vh / vl (warp-uniform)
    auto flush = [&]() {
        if (npend) {
            reduce_tasks_df<(S > 0 ? S : 1), DET>(reinterpret_cast<PrecSmem<(S > 0 ? S : 1)> &>(sm), npend, 0,
                                                  ptAdj, ptStride, true, pt0, pt1, nodeAdj, nodeStride);
            npend = 0;
        }
    };
    // one term into the batch: target = point index, or ~node for a cluster
    auto push = [&](const dfl *vv, int target) {
        constexpr int SS = S > 0 ? S : 1;
        auto &smb = reinterpret_cast<PrecSmem<SS> &>(sm);
        smb.vh[npend][lane] = make_float4(vv[0].h, vv[1].h, vv[2].h, vv[3].h);
        smb.vl[npend][lane] = make_float4(vv[0].l, vv[1].l, vv[2].l, vv[3].l);
        if constexpr (prec_smem_targets<SS>()) {
            if (lane == 0) smb.tgt[npend] = target;
        } else {
            if (npend == 0) pt0 = target;
            else pt1 = target;
        }
        if (++npend == PrecSmem<SS>::kP) flush();
    };
    for (int kk = 0; kk < mp.nLoop; ++kk) {
        const float4 rhi = rec.hi[kk * v.nVol + g], rlo = rec.lo[kk * v.nVol + g];
        const float rh[3] = {rhi.x, rhi.y, rhi.z}, rl[3] = {rlo.x, rlo.y, rlo.z};
        // this mirror's seeds: the transpose of the numerator reflection
        // (getMirrorNumerator_b, src/warp/initializeWarping.F90:603-635), in FP64
        for (int sd = 0; sd < S; ++sd) {
            const double *dv = dxv + sd * dxvStride + 3 * int64_t(vi);
            double n3[3] = {valid ? dv[0] * q : 0.0, valid ? dv[1] * q : 0.0, valid ? dv[2] * q : 0.0};
#pragma unroll
            for (int j = kMaxSym - 1; j >= 0; --j) {
                if (j < mp.nSym && ((kk >> j) & 1)) {
                    const double nr[3] = {double(mp.nrm[j][0]) + double(mp.nrmLo[j][0]),
                                          double(mp.nrm[j][1]) + double(mp.nrmLo[j][1]),
                                          double(mp.nrm[j][2]) + double(mp.nrmLo[j][2])};
                    const double dp = n3[0] * nr[0] + n3[1] * nr[1] + n3[2] * nr[2];
                    n3[0] -= 2.0 * dp * nr[0];
                    n3[1] -= 2.0 * dp * nr[1];
                    n3[2] -= 2.0 * dp * nr[2];
                }
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float h = float(n3[a]);
                sm.nh[lane][3 * sd + a] = h;
                sm.nl[lane][3 * sd + a] = float(n3[a] - double(h));
                if (S == 1) nl1[a] = {h, float(n3[a] - double(h))};
            }
        }
        __syncwarp();
        int node = 0, skip = 0;
        int64_t e = 0, e1 = 0;
        if (REPLAY && (gid >> 5) < (v.nVol + 31) / 32) {
            e = wlists.offs[(gid >> 5) * mp.nLoop + kk];
            e1 = wlists.offs[(gid >> 5) * mp.nLoop + kk + 1];
        }
        while (REPLAY ? e < e1 : node < t.nNodes) {
            bool active;
            if (REPLAY) {
                const int2 ent = __ldg(wlists.list + e);
                ++e;
                node = ent.x & 0x7fffffff;
                active = (unsigned(ent.y) >> lane) & 1u;
            } else {
                active = valid && node >= skip;
            }
            const int4 inf = ldgi4(&tf.nodes[node].info);
            if (inf.w) {
                if constexpr (S > 0 && IDW_PREC_CBATCH == 1) flush();  // the leaf reuses vh / vl
                const float4 ch = ldgf4(&tf.nodes[node].cHi), cl = ldgf4(&tf.nodes[node].cLo);
                dfl R[3];
                rel_df(rh, rl, ch, cl, R);
                if (active) {
                    cnt.leafPairs += inf.y - inf.x + 1;
                    cnt.visited++;
                }
                if constexpr (S > 0 && IDW_PREC_CBATCH >= 2) {
                    // every point into the batch
                    for (int i = inf.x; i <= inf.y; ++i) {
                        float wh = 0.f, wl = 0.f;
                        dfl xr[3];
                        if (active) {
                            const float4 da = ldgf4(pf.da + i), dl = ldgf4(pf.dl + i);
                            dfl x[3];
                            two_diff(R[0].h, da.x, x[0].h, x[0].l);
                            two_diff(R[1].h, da.y, x[1].h, x[1].l);
                            two_diff(R[2].h, da.z, x[2].h, x[2].l);
                            x[0].l += R[0].l - dl.x;
                            x[1].l += R[1].l - dl.y;
                            x[2].l += R[2].l - dl.z;
                            precise_weight<KIND>(x, 1e-15f, da.w, dl.w, law, Ls, LsLo, c1, mp.abH, mp.abL, xr, wh, wl);
                        }
                        dfl vv[4];
                        term_vector(wh, wl, R, vv);  // moments relative to the leaf centroid
                        push(vv, i);
                    }
                } else {
                    for (int i0 = inf.x; i0 <= inf.y; i0 += PrecSmem<S>::kP) {
                        const int m = min(PrecSmem<S>::kP, inf.y - i0 + 1);
                        for (int p = 0; p < m; ++p) {
                            const int i = i0 + p;
                            float wh = 0.f, wl = 0.f;
                            dfl xr[3];
                            if (active) {
                                // r - Xu0_i = (r - C) - (Xu0_i - C), offsets from the leaf centroid
                                const float4 da = ldgf4(pf.da + i), dl = ldgf4(pf.dl + i);
                                dfl x[3];
                                two_diff(R[0].h, da.x, x[0].h, x[0].l);
                                two_diff(R[1].h, da.y, x[1].h, x[1].l);
                                two_diff(R[2].h, da.z, x[2].h, x[2].l);
                                x[0].l += R[0].l - dl.x;
                                x[1].l += R[1].l - dl.y;
                                x[2].l += R[2].l - dl.z;
                                precise_weight<KIND>(x, 1e-15f, da.w, dl.w, law, Ls, LsLo, c1, mp.abH, mp.abL, xr, wh, wl);
                            }
                            if constexpr (S == 0) {
                                comp_add_df(dsum, dcomp, wh, wl);
                            } else {
                                // moments relative to the leaf centroid
                                dfl vv[4];
                                term_vector(wh, wl, R, vv);
                                sm.vh[p][lane] = make_float4(vv[0].h, vv[1].h, vv[2].h, vv[3].h);
                                sm.vl[p][lane] = make_float4(vv[0].l, vv[1].l, vv[2].l, vv[3].l);
                            }
                        }
                        if constexpr (S > 0) reduce_tasks_df<S, DET>(sm, m, i0, ptAdj, ptStride);
                    }
                }
                if (!REPLAY) node = inf.z;
            } else {
                bool open = false;
                int dec = 0;
                float rho0 = 0.f, rho1 = 0.f, rho2 = 0.f, d2 = 0.f, rs = 0.f, wA = 0.f;
                if (REPLAY) {
                    dec = active ? 1 : 0;
                } else {
                    if (active && !exact) {
                        cnt.visited++;
                        dec = decide32(tf, node, rh, rl, tauf, rho0, rho1, rho2, d2, rs, wA);
                    }
                    dec = resolve64(dec, t, v, g, node, rh, rl, mp.errTol, counters);
                }
                if (__any_sync(kFull, dec == 1)) {
                    float wh = 0.f, wl = 0.f;
                    dfl x[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
                    if (dec == 1) {
                        const float4 ch = ldgf4(&tf.nodes[node].cHi), cl = ldgf4(&tf.nodes[node].cLo);
                        dfl xin[3];
                        rel_df(rh, rl, ch, cl, xin);
                        precise_weight<KIND>(xin, 0.f, cl.w, __ldg(&tf.nodes[node].aLo), law, Ls, LsLo, c1, mp.abH,
                                             mp.abL, x, wh, wl);
                        skip = inf.z;
                        cnt.approx++;
                    }
                    if constexpr (S == 0) {
                        comp_add_df(dsum, dcomp, wh, wl);
                    } else {
                        dfl vv[4];
                        term_vector(wh, wl, x, vv);
                        if constexpr (IDW_PREC_CBATCH) {
                            push(vv, ~node);
                        } else if constexpr (S == 1) {
                            land_one_df<DET>(vv, nl1, nodeAdj + 12 * int64_t(node));
                        } else {
                            sm.vh[0][lane] = make_float4(vv[0].h, vv[1].h, vv[2].h, vv[3].h);
                            sm.vl[0][lane] = make_float4(vv[0].l, vv[1].l, vv[2].l, vv[3].l);
                            reduce_tasks_df<S, DET>(sm, 1, node, nodeAdj, nodeStride);
                        }
                    }
                }
                if (!REPLAY) {
                    if (dec != 1 && active) open = true;
                    node = __any_sync(kFull, open) ? node + 1 : inf.z;
                }
            }
        }
        if constexpr (S > 0 && IDW_PREC_CBATCH) flush();  // before the next pass's seeds
        __syncwarp();
    }
    if (S == 0 && valid) denOut[vi] = (double(dsum) + double(dcomp)) * exp2(-double(s) * mp.bExp);
    if (!REPLAY) cnt.flush(counters);
}

template <int S, int KIND>
void launch_prec(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v, const WalkRecF &rec,
                 const MixedParams &mp, const Law32<KIND> &law, int exact, const double *dxv, int64_t dxvStride,
                 const double *den, double *ptAdj, int64_t ptStride, double *nodeAdj, int64_t nodeStride,
                 double *denOut, unsigned long long *counters, const WalkLists &wl, cudaStream_t st, int det) {
    const size_t smem = 4 * sizeof(PrecSmem<S>);
    const int g = int((v.nVol + 127) / 128);
    if constexpr (S > 0) {
        if (det) {  // order-independent landings: the deciding walk
            cudaFuncSetAttribute(k_adjoint_precise<S, KIND, 0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(smem));
            k_adjoint_precise<S, KIND, 0, true><<<g, 128, smem, st>>>(t, tf, pf, v, rec, mp, law, exact, dxv,
                                                                      dxvStride, den, ptAdj, ptStride, nodeAdj,
                                                                      nodeStride, denOut, counters, wl);
            return;
        }
    }
    // sixteen seeds keep deciding as they go: at four blocks per SM (shared
    // memory) the replay's schedule measured slower (8M-node wing: 622 against
    // 586 ms with 4 points per pass); fewer seeds replay (one seed 73 against
    // 86 ms)
    if (wl.list && !exact && S < 16) {
        launch_add_walk_counters(counters, wl.counters, st);
        cudaFuncSetAttribute(k_adjoint_precise<S, KIND, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        k_adjoint_precise<S, KIND, 1><<<g, 128, smem, st>>>(t, tf, pf, v, rec, mp, law, exact, dxv, dxvStride, den,
                                                            ptAdj, ptStride, nodeAdj, nodeStride, denOut, counters,
                                                            wl);
    } else {
        cudaFuncSetAttribute(k_adjoint_precise<S, KIND, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        k_adjoint_precise<S, KIND, 0><<<g, 128, smem, st>>>(t, tf, pf, v, rec, mp, law, exact, dxv, dxvStride, den,
                                                            ptAdj, ptStride, nodeAdj, nodeStride, denOut, counters,
                                                            wl);
    }
}

template <int S>
void launch_prec_law(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v,
                     const WalkRecF &rec, const MixedParams &mp, const WeightLaw &wl, int exact, const double *dxv,
                     int64_t dxvStride, const double *den, double *ptAdj, int64_t ptStride, double *nodeAdj,
                     int64_t nodeStride, double *denOut, unsigned long long *counters, const WalkLists &lists,
                     cudaStream_t st, int det) {
    if (wl.isInt && wl.ia == 3 && wl.ib == 5)
        launch_prec<S, 0>(t, tf, pf, v, rec, mp, Law32<0>{3, 5, 3.f, 5.f}, exact, dxv, dxvStride, den, ptAdj,
                          ptStride, nodeAdj, nodeStride, denOut, counters, lists, st, det);
    else
        launch_prec<S, 1>(t, tf, pf, v, rec, mp, Law32<1>{wl.ia, wl.ib, float(wl.aExp), float(wl.bExp)}, exact, dxv,
                          dxvStride, den, ptAdj, ptStride, nodeAdj, nodeStride, denOut, counters, lists, st, det);
}

}  // namespace

bool precise_adjoint_supported(const WeightLaw &wl) { return wl.isInt != 0; }

void launch_precise_denominator(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v,
                                const WalkRecF &rec, const EvalConsts &k, int exact, double *denOut,
                                cudaStream_t st) {
    if (v.nVol <= 0) return;
    const MixedParams mp = make_mixed_params(k);
    launch_prec_law<0>(t, tf, pf, v, rec, mp, k.law, exact, nullptr, 0, nullptr, nullptr, 0, nullptr, 0, denOut,
                       nullptr, k.lists, st, 0);
}

int launch_adjoint_precise(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v,
                           const WalkRecF &rec, const EvalConsts &k, int exact, const double *dxv, int nSeeds,
                           int64_t dxvStride, const double *den, double *ptAcc, double *nodeAcc, int nPts,
                           unsigned long long *counters, cudaStream_t st, int det) {
    if (nSeeds <= 0 || v.nVol <= 0) return 0;
    const MixedParams mp = make_mixed_params(k);
    const int64_t ptStride = 12 * int64_t(nPts), nodeStride = 12 * int64_t(t.nNodes);
    int s0 = 0;
    while (s0 < nSeeds) {
        const int left = nSeeds - s0;
        const double *d = dxv + s0 * dxvStride;
        double *pa = ptAcc + s0 * ptStride, *na = nodeAcc + s0 * nodeStride;
        if (left >= 16) {
            launch_prec_law<16>(t, tf, pf, v, rec, mp, k.law, exact, d, dxvStride, den, pa, ptStride, na, nodeStride,
                                nullptr, counters, k.lists, st, det);
            s0 += 16;
        } else if (left >= 4) {
            launch_prec_law<4>(t, tf, pf, v, rec, mp, k.law, exact, d, dxvStride, den, pa, ptStride, na, nodeStride,
                               nullptr, counters, k.lists, st, det);
            s0 += 4;
        } else {
            launch_prec_law<1>(t, tf, pf, v, rec, mp, k.law, exact, d, dxvStride, den, pa, ptStride, na, nodeStride,
                               nullptr, counters, k.lists, st, det);
            s0 += 1;
        }
    }
    return 0;
}

IDW_LAND_SETTER(land_set_precise)

}  // namespace idw
