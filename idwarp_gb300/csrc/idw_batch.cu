// Mixed-precision walk over NB surfaces at once (several perturbations of the
// same surface, i.e. the same Xu0 and tree): the weights depend on Xu0 and the
// volume node only (src/modules/kd_tree.F90:677-688, 705-711), so the walk,
// its decisions and every weight are computed once and shared, and only the
// motions S_b = M_b r + b_b - r differ per surface.  Each surface's result
// equals that of the single-surface walk (idw_mixed.cu) up to rounding.
//
// The surfaces' point and cluster arrays are point-major (all surfaces of a
// point, or of a cluster, in adjacent 48-byte rows), so a point's motions for
// every surface come from one or two cache lines.
//
// Per lane: the denominator pair in registers; per surface the running
// numerator pairs in shared memory.  Terms are summed in FP32 partials of at
// most a leaf, or at most kFlush cluster terms, which are then added to the
// compensated pairs (so a partial never spans more than a few terms).
#include "idw_mixed.cuh"

namespace idw {

namespace {

constexpr int kFlush = 4;  // cluster terms per FP32 partial

// Resident blocks per SM the register allocation targets (128 threads each).
#ifndef IDW_BATCH_MIN_BLOCKS
#define IDW_BATCH_MIN_BLOCKS 6
#endif

template <int NB>
struct BatchSmem {
    float sn[NB][3][128], cn[NB][3][128];  // this mirror's numerator pairs
    float4 mirS[NB][128], mirC[NB][128];   // over the mirrors: (num, den) pairs
};

template <int NB>
__device__ __forceinline__ void flush_partials(BatchSmem<NB> &sm, float (&pn)[NB][3]) {
    const int tid = threadIdx.x;
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float s = sm.sn[b][a][tid], c = sm.cn[b][a][tid];
            kahan_add(s, c, pn[b][a]);
            sm.sn[b][a][tid] = s;
            sm.cn[b][a][tid] = c;
            pn[b][a] = 0.f;
        }
}

// REPLAY: walk the recorded decisions (idw_replay.cu) instead of deciding;
// the terms, their order and their arithmetic are the deciding walk's.
template <int KIND, int NB, int REPLAY>
__global__ void __launch_bounds__(128, IDW_BATCH_MIN_BLOCKS)
    k_walk_mixed_batch(TreeDev t, TreeDevF tf, PointsDevF pf, NodeAggF af, VolumeDev v, WalkRecF rec, MixedParams mp,
                       Law32<KIND> law, int exact, float4 *acc, int64_t accStrideB, unsigned long long *counters,
                       WalkLists wlists) {
    extern __shared__ __align__(16) unsigned char smraw[];
    BatchSmem<NB> &sm = *reinterpret_cast<BatchSmem<NB> *>(smraw);
    const int tid = threadIdx.x;
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + tid;
    const bool valid = gid < v.nVol;
    const int64_t g = valid ? gid : 0;
    const float4 r0lo = rec.lo[g];
    const int s = __float_as_int(r0lo.w);
    const float den0f = rec.hi[g].w;
    const float Ls = mp.LdefF * pow2f(s);
    const float LsLo = mp.LdefLo * pow2f(s);
    const float c1 = mp.intExp ? pow2f(s * mp.dExp) : exp2f(float(s) * mp.dExpF);
    const float ab = mp.abH, abl = mp.abL;
    const float tauf = mp.errTolF * den0f;
    float gv;
    if (rec.gden) {
        gv = mp.precGate * rec.gden[g];
    } else {
        const float gexp = float(s) * mp.bExpF;
        const float gexpi = floorf(gexp);
        gv = mp.precGate * ldexpf(den0f, int(gexpi)) * exp2f(gexp - gexpi);
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        sm.mirS[b][tid] = make_float4(0.f, 0.f, 0.f, 0.f);
        sm.mirC[b][tid] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    MixedCounters cnt;
    for (int kk = 0; kk < mp.nLoop; ++kk) {
        const float4 rhi = rec.hi[kk * v.nVol + g], rlo = rec.lo[kk * v.nVol + g];
        const float rh[3] = {rhi.x, rhi.y, rhi.z}, rl[3] = {rlo.x, rlo.y, rlo.z};
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int a = 0; a < 3; ++a) sm.sn[b][a][tid] = sm.cn[b][a][tid] = 0.f;
        float sd = 0.f, cd = 0.f;
        float pn[NB][3];
#pragma unroll
        for (int b = 0; b < NB; ++b) pn[b][0] = pn[b][1] = pn[b][2] = 0.f;
        float pdc = 0.f;  // cluster partial of the denominator
        int nPart = 0;    // cluster terms in the partials
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
                active = (unsigned(ent.y) >> (tid & 31)) & 1u;
            } else {
                active = valid && node >= skip;
            }
            const int4 inf = ldgi4(&tf.nodes[node].info);
            if (inf.w) {
                bool leafPrecise = false;
                if (active) {
                    // close the cluster partial before the leaf's own
                    if (nPart) {
                        flush_partials<NB>(sm, pn);
                        kahan_add(sd, cd, pdc);
                        pdc = 0.f;
                        nPart = 0;
                    }
                    const float4 ch = ldgf4(&tf.nodes[node].cHi), cl = ldgf4(&tf.nodes[node].cLo);
                    float h0, h1, h2, l0, l1, l2;
                    two_diff(rh[0], ch.x, h0, l0);
                    two_diff(rh[1], ch.y, h1, l1);
                    two_diff(rh[2], ch.z, h2, l2);
                    l0 += rl[0] - cl.x;
                    l1 += rl[1] - cl.y;
                    l2 += rl[2] - cl.z;
                    float pd = 0.f;
                    for (int i = inf.x; i <= inf.y; ++i) {
                        const float4 da = ldgf4(pf.da + i), dl = ldgf4(pf.dl + i);
                        const float dx = (h0 - da.x) + (l0 - dl.x);
                        const float dy = (h1 - da.y) + (l1 - dl.y);
                        const float dz = (h2 - da.z) + (l2 - dl.z);
                        const float d2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, 1e-15f)));
                        const float r1 = rsqrt_normal(d2);
                        const float tt = fmaf(Ls, r1, LsLo * r1);
                        const float w = da.w * law.eval(tt, c1, ab, abl);
#pragma unroll
                        for (int b = 0; b < NB; ++b) {
                            const float4 *dm = reinterpret_cast<const float4 *>(pf.dm + 12 * (kBatchMax * int64_t(i) + b));
                            const float4 m0 = ldgf4(dm), m1 = ldgf4(dm + 1), m2 = ldgf4(dm + 2);
                            pn[b][0] = fmaf(w, fmaf(m0.x, dx, fmaf(m0.y, dy, fmaf(m0.z, dz, m2.y))), pn[b][0]);
                            pn[b][1] = fmaf(w, fmaf(m0.w, dx, fmaf(m1.x, dy, fmaf(m1.y, dz, m2.z))), pn[b][1]);
                            pn[b][2] = fmaf(w, fmaf(m1.z, dx, fmaf(m1.w, dy, fmaf(m2.x, dz, m2.w))), pn[b][2]);
                        }
                        pd += w;
                    }
                    // the same gate as the single-surface walk, on the largest surface
                    const float hsum = fabsf(h0) + fabsf(h1) + fabsf(h2);
                    float lmag = 0.f;
#pragma unroll
                    for (int b = 0; b < NB; ++b)
                        lmag = fmaxf(lmag, fabsf(pn[b][0]) + fabsf(pn[b][1]) + fabsf(pn[b][2]) +
                                               pd * __ldg(af.dn + kBatchMax * int64_t(node) + b) * hsum);
                    leafPrecise = KIND != 2 && lmag > gv;
                    if (!leafPrecise) {
                        flush_partials<NB>(sm, pn);
                        kahan_add(sd, cd, pd);
                    } else {
#pragma unroll
                        for (int b = 0; b < NB; ++b) pn[b][0] = pn[b][1] = pn[b][2] = 0.f;
                    }
                    cnt.leafPairs += inf.y - inf.x + 1;
                    cnt.visited++;
                }
                if (__any_sync(kFull, leafPrecise)) {
                    if (leafPrecise) {
                        const float4 ch = ldgf4(&tf.nodes[node].cHi), cl = ldgf4(&tf.nodes[node].cLo);
                        dfl q0, q1, q2;
                        two_diff(rh[0], ch.x, q0.h, q0.l);
                        two_diff(rh[1], ch.y, q1.h, q1.l);
                        two_diff(rh[2], ch.z, q2.h, q2.l);
                        q0.l += rl[0] - cl.x;
                        q1.l += rl[1] - cl.y;
                        q2.l += rl[2] - cl.z;
                        for (int i = inf.x; i <= inf.y; ++i) {
                            const float4 da = ldgf4(pf.da + i), dl = ldgf4(pf.dl + i);
                            dfl xi[3];
                            two_diff(q0.h, da.x, xi[0].h, xi[0].l);
                            two_diff(q1.h, da.y, xi[1].h, xi[1].l);
                            two_diff(q2.h, da.z, xi[2].h, xi[2].l);
                            xi[0].l += q0.l - dl.x;
                            xi[1].l += q1.l - dl.y;
                            xi[2].l += q2.l - dl.z;
                            dfl x[3];
                            float wh, wl;
                            precise_weight<KIND>(xi, 1e-15f, da.w, dl.w, law, Ls, LsLo, c1, mp.abH, mp.abL, x, wh, wl);
#pragma unroll
                            for (int b = 0; b < NB; ++b) {
                                float s3[3] = {sm.sn[b][0][tid], sm.sn[b][1][tid], sm.sn[b][2][tid]};
                                float c3[3] = {sm.cn[b][0][tid], sm.cn[b][1][tid], sm.cn[b][2][tid]};
                                precise_motion(x, wh, wl, pf.dm + 12 * (kBatchMax * int64_t(i) + b),
                                               pf.dml + 12 * (kBatchMax * int64_t(i) + b), s3, c3);
#pragma unroll
                                for (int a = 0; a < 3; ++a) {
                                    sm.sn[b][a][tid] = s3[a];
                                    sm.cn[b][a][tid] = c3[a];
                                }
                            }
                            comp_add_df(sd, cd, wh, wl);
                        }
                    }
                    warp_count(counters, 6, leafPrecise ? unsigned(inf.y - inf.x + 1) : 0u);
                }
                if (!REPLAY) node = inf.z;
            } else {
                bool open = false;
                int dec = 0;
                float rho0 = 0.f, rho1 = 0.f, rho2 = 0.f, d2 = 0.f, rs = 0.f, wA = 0.f;
                if (REPLAY) {
                    if (active) {
                        cluster_geo(ldgf4(&tf.nodes[node].cHi), ldgf4(&tf.nodes[node].cLo), rh, rl, rho0, rho1, rho2,
                                    d2, rs, wA);
                        dec = 1;
                    }
                } else {
                    if (active && !exact) {
                        cnt.visited++;
                        dec = decide32(tf, node, rh, rl, tauf, rho0, rho1, rho2, d2, rs, wA);
                    }
                    dec = resolve64(dec, t, v, g, node, rh, rl, mp.errTol, counters);
                }
                bool precise = false;
                if (dec == 1) {
                    const float tt = fmaf(Ls, rs, LsLo * rs);
                    const float w = wA * law.eval(tt, c1, ab, abl);
                    const float rsum = fabsf(rho0) + fabsf(rho1) + fabsf(rho2);
                    float S[NB][3];
                    float mag = 0.f;
#pragma unroll
                    for (int b = 0; b < NB; ++b) {
                        const float4 *dc = reinterpret_cast<const float4 *>(af.dc + 12 * (kBatchMax * int64_t(node) + b));
                        const float4 m0 = ldgf4(dc), m1 = ldgf4(dc + 1), m2 = ldgf4(dc + 2);
                        S[b][0] = fmaf(m0.x, rho0, fmaf(m0.y, rho1, fmaf(m0.z, rho2, m2.y)));
                        S[b][1] = fmaf(m0.w, rho0, fmaf(m1.x, rho1, fmaf(m1.y, rho2, m2.z)));
                        S[b][2] = fmaf(m1.z, rho0, fmaf(m1.w, rho1, fmaf(m2.x, rho2, m2.w)));
                        mag = fmaxf(mag, fabsf(S[b][0]) + fabsf(S[b][1]) + fabsf(S[b][2]) +
                                             __ldg(af.dn + kBatchMax * int64_t(node) + b) * rsum);
                    }
                    precise = KIND != 2 && w * mag > gv;
                    if (!precise) {
#pragma unroll
                        for (int b = 0; b < NB; ++b) {
                            pn[b][0] = fmaf(w, S[b][0], pn[b][0]);
                            pn[b][1] = fmaf(w, S[b][1], pn[b][1]);
                            pn[b][2] = fmaf(w, S[b][2], pn[b][2]);
                        }
                        pdc += w;
                        if (++nPart == kFlush) {
                            flush_partials<NB>(sm, pn);
                            kahan_add(sd, cd, pdc);
                            pdc = 0.f;
                            nPart = 0;
                        }
                    }
                    skip = inf.z;
                    cnt.approx++;
                } else if (active) {
                    open = true;
                }
                if (__any_sync(kFull, precise)) {
                    if (precise) {
                        const float4 ch = ldgf4(&tf.nodes[node].cHi), cl = ldgf4(&tf.nodes[node].cLo);
                        dfl q[3];
                        two_diff(rh[0], ch.x, q[0].h, q[0].l);
                        two_diff(rh[1], ch.y, q[1].h, q[1].l);
                        two_diff(rh[2], ch.z, q[2].h, q[2].l);
                        q[0].l += rl[0] - cl.x;
                        q[1].l += rl[1] - cl.y;
                        q[2].l += rl[2] - cl.z;
                        dfl x[3];
                        float wh, wl;
                        precise_weight<KIND>(q, 0.f, cl.w, __ldg(&tf.nodes[node].aLo), law, Ls, LsLo, c1, mp.abH,
                                             mp.abL, x, wh, wl);
#pragma unroll
                        for (int b = 0; b < NB; ++b) {
                            float s3[3] = {sm.sn[b][0][tid], sm.sn[b][1][tid], sm.sn[b][2][tid]};
                            float c3[3] = {sm.cn[b][0][tid], sm.cn[b][1][tid], sm.cn[b][2][tid]};
                            precise_motion(x, wh, wl, af.dc + 12 * (kBatchMax * int64_t(node) + b),
                                           af.dcl + 12 * (kBatchMax * int64_t(node) + b), s3, c3);
#pragma unroll
                            for (int a = 0; a < 3; ++a) {
                                sm.sn[b][a][tid] = s3[a];
                                sm.cn[b][a][tid] = c3[a];
                            }
                        }
                        comp_add_df(sd, cd, wh, wl);
                    }
                    warp_count(counters, 6, precise ? 1u : 0u);
                }
                if (!REPLAY) node = __any_sync(kFull, open) ? node + 1 : inf.z;
            }
        }
        if (nPart) {
            flush_partials<NB>(sm, pn);
            kahan_add(sd, cd, pdc);
        }
        // per surface: add its reference motion back, reflect, accumulate over
        // the mirrors (as the single-surface walk)
        const dfl den = df_norm(sd, cd);
#pragma unroll 1
        for (int b = 0; b < NB; ++b) {
            const float *ref = af.ref + 24 * b;
            dfl num[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                dfl sr = {__ldg(ref + 9 + a), __ldg(ref + 21 + a)};
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    sr = df_add(sr, df_mul({__ldg(ref + 3 * a + k), __ldg(ref + 12 + 3 * a + k)}, {rh[k], rl[k]}));
                num[a] = df_add(df_norm(sm.sn[b][a][tid], sm.cn[b][a][tid]), df_mul(den, sr));
            }
#pragma unroll
            for (int j = 0; j < kMaxSym; ++j) {
                if (j < mp.nSym && ((kk >> j) & 1)) {
                    const dfl n0 = {mp.nrm[j][0], mp.nrmLo[j][0]}, n1 = {mp.nrm[j][1], mp.nrmLo[j][1]},
                              n2 = {mp.nrm[j][2], mp.nrmLo[j][2]};
                    dfl dp = df_add(df_add(df_mul(num[0], n0), df_mul(num[1], n1)), df_mul(num[2], n2));
                    dp = {-2.0f * dp.h, -2.0f * dp.l};
                    num[0] = df_add(num[0], df_mul(dp, n0));
                    num[1] = df_add(num[1], df_mul(dp, n1));
                    num[2] = df_add(num[2], df_mul(dp, n2));
                }
            }
            float4 S4 = sm.mirS[b][tid], C4 = sm.mirC[b][tid];
            kahan_add_df(S4.x, C4.x, num[0]);
            kahan_add_df(S4.y, C4.y, num[1]);
            kahan_add_df(S4.z, C4.z, num[2]);
            kahan_add_df(S4.w, C4.w, den);
            sm.mirS[b][tid] = S4;
            sm.mirC[b][tid] = C4;
        }
    }
    if (valid) {
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            acc[b * accStrideB + 2 * gid] = sm.mirS[b][tid];
            acc[b * accStrideB + 2 * gid + 1] = sm.mirC[b][tid];
        }
    }
    if (!REPLAY) cnt.flush(counters);
}

template <int KIND, int NB>
void launch_batch_nb(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af,
                     const VolumeDev &v, const WalkRecF &rec, const MixedParams &mp, const Law32<KIND> &law, int exact,
                     float4 *acc, int64_t accStrideB, unsigned long long *counters, const WalkLists &wl,
                     cudaStream_t st) {
    const size_t smem = sizeof(BatchSmem<NB>);
    const int g = int((v.nVol + 127) / 128);
    if (wl.list && !exact) {
        cudaFuncSetAttribute(k_walk_mixed_batch<KIND, NB, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        k_walk_mixed_batch<KIND, NB, 1><<<g, 128, smem, st>>>(t, tf, pf, af, v, rec, mp, law, exact, acc, accStrideB,
                                                              counters, wl);
    } else {
        cudaFuncSetAttribute(k_walk_mixed_batch<KIND, NB, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        k_walk_mixed_batch<KIND, NB, 0><<<g, 128, smem, st>>>(t, tf, pf, af, v, rec, mp, law, exact, acc, accStrideB,
                                                              counters, wl);
    }
}

template <int KIND>
void launch_batch_kind(int nb, const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af,
                       const VolumeDev &v, const WalkRecF &rec, const MixedParams &mp, const Law32<KIND> &law,
                       int exact, float4 *acc, int64_t accStrideB, unsigned long long *counters, const WalkLists &wl,
                       cudaStream_t st) {
    switch (nb) {
        case 1:
            launch_batch_nb<KIND, 1>(t, tf, pf, af, v, rec, mp, law, exact, acc, accStrideB, counters, wl, st);
            break;
        case 2:
            launch_batch_nb<KIND, 2>(t, tf, pf, af, v, rec, mp, law, exact, acc, accStrideB, counters, wl, st);
            break;
        case 3:
            launch_batch_nb<KIND, 3>(t, tf, pf, af, v, rec, mp, law, exact, acc, accStrideB, counters, wl, st);
            break;
        case 4:
            launch_batch_nb<KIND, 4>(t, tf, pf, af, v, rec, mp, law, exact, acc, accStrideB, counters, wl, st);
            break;
        default:
            launch_batch_nb<KIND, kBatchMax>(t, tf, pf, af, v, rec, mp, law, exact, acc, accStrideB, counters, wl, st);
            break;
    }
}

}  // namespace

void launch_walk_mixed_batch(int nb, const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af,
                             const VolumeDev &v, const WalkRecF &rec, const EvalConsts &k, int exact, float4 *acc,
                             int64_t accStrideB, unsigned long long *counters, cudaStream_t st) {
    if (v.nVol <= 0 || nb <= 0) return;
    const MixedParams mp = make_mixed_params(k);
    if (k.law.isInt && k.law.ia == 3 && k.law.ib == 5) {
        Law32<0> law{3, 5, 3.f, 5.f};
        launch_batch_kind<0>(nb, t, tf, pf, af, v, rec, mp, law, exact, acc, accStrideB, counters, k.lists, st);
    } else if (k.law.isInt) {
        Law32<1> law{k.law.ia, k.law.ib, float(k.law.aExp), float(k.law.bExp)};
        launch_batch_kind<1>(nb, t, tf, pf, af, v, rec, mp, law, exact, acc, accStrideB, counters, k.lists, st);
    } else {
        Law32<2> law{0, 0, float(k.law.aExp), float(k.law.bExp)};
        launch_batch_kind<2>(nb, t, tf, pf, af, v, rec, mp, law, exact, acc, accStrideB, counters, k.lists, st);
    }
}

}  // namespace idw
