// Mixed-precision reverse walk of warpDeriv for S seeds at once.
//   evalNode_b / evalNodeExact_b / evalNodeApprox_b  src/modules/kd_tree.F90:942-1031
//   driven as warpDeriv                              src/warp/warpDeriv.F90:71-88
//   setData_b                                        src/modules/kd_tree.F90:1033-1051
//
// Same warp-cooperative walk and the same guarded decisions as the forward
// mixed walk (decide32 + resolve64), so every lane visits exactly the terms
// the forward pass used.  A term (surface point i of a leaf, or an
// approximated cluster q) receives from lane l the contribution
//     sib = w_l * numb_l (3 per seed),   (r_l - C) (x) sib  (9 per seed),
// with C the leaf centroid (points) or the cluster centroid (clusters): the
// moments are kept relative to C so that nothing of size |r| is accumulated
// and later cancelled.  Writing v_l = w_l (1, r_l - C), the warp's sum over
// lanes is the small product  V (4 x 32) . N (32 x 3S)  with N the lanes'
// seeds, which the warp forms from shared memory; one FP64 atomic per result
// lands it in the per-point / per-cluster accumulators.
#include "idw_mixed.cuh"
#include "idwarp_gb300.h"

namespace idw {

namespace {

// Leaf points reduced per shared-memory pass: ten for the small-S forms (a
// 9-point leaf of the default bucket in one pass), eight for the blocked one.
template <int S>
struct AdjSmem {
    static constexpr int kChunk = S <= 4 ? 10 : 8;
    float nb[32][3 * S];       // seeds of every lane (numerator adjoints, scaled)
    // per point: w, w (r - C); for 8 seeds the rows are padded so that lane
    // groups reading different points hit different banks
    static constexpr int kRow = S == 8 ? 33 : 32;
    float4 vb[kChunk][kRow];
    int tgt[S <= 4 ? kChunk : 1];  // few seeds: targets of a batch of terms
};

// Few seeds (S <= 4): a warp's terms, leaf points and approximated clusters
// alike, wait in vb until kChunk of them (or the end of the mirror pass) and
// reduce together, one lane task per (term, seed component), instead of one
// reduction per leaf (about 5.5 points: half the task lanes idle) and one
// warp butterfly per cluster term.
#ifndef IDW_ADJ_BATCH
#define IDW_ADJ_BATCH 1
#endif

// Lands the four moment sums of term `target`, seed component c (seed s, axis
// a): w -> B (slot 9 + a), w (r - C) -> row a of P (slots 3a .. 3a + 2).
template <bool DET>
__device__ __forceinline__ void land_moments(double *adj, int64_t seedStride, int c, int64_t target, float w,
                                             float m0, float m1, float m2) {
    if (w == 0.f && m0 == 0.f && m1 == 0.f && m2 == 0.f) return;
    const int s = c / 3, a = c - 3 * s;
    double *d = adj + s * seedStride + 12 * target;
    land_add<DET>(d + 9 + a, double(w));
    land_add<DET>(d + 3 * a + 0, double(m0));
    land_add<DET>(d + 3 * a + 1, double(m1));
    land_add<DET>(d + 3 * a + 2, double(m2));
}

// Warp reduction of m point contributions (vb[0..m)) against the lanes'
// seeds, blocked for many seeds: lane c owns seed component c and all m terms.
template <int S, bool DET>
__device__ __forceinline__ void reduce_terms(AdjSmem<S> &sm, int m, const int *targets, double *adj,
                                             int64_t seedStride) {
    constexpr int kChunk = AdjSmem<S>::kChunk;
    const int lane = threadIdx.x & 31;
    __syncwarp();
    for (int c = lane; c < 3 * S; c += 32) {
        const int s = c / 3, a = c - 3 * s;
        float acc[kChunk][4];
#pragma unroll
        for (int p = 0; p < kChunk; ++p) acc[p][0] = acc[p][1] = acc[p][2] = acc[p][3] = 0.f;
        for (int l = 0; l < 32; ++l) {
            const float nbv = sm.nb[l][c];
#pragma unroll
            for (int p = 0; p < kChunk; ++p) {
                if (p < m) {
                    const float4 v = sm.vb[p][l];
                    acc[p][0] = fmaf(v.x, nbv, acc[p][0]);
                    acc[p][1] = fmaf(v.y, nbv, acc[p][1]);
                    acc[p][2] = fmaf(v.z, nbv, acc[p][2]);
                    acc[p][3] = fmaf(v.w, nbv, acc[p][3]);
                }
            }
        }
#pragma unroll
        for (int p = 0; p < kChunk; ++p) {
            if (p < m && (acc[p][0] != 0.f || acc[p][1] != 0.f || acc[p][2] != 0.f || acc[p][3] != 0.f)) {
                double *d = adj + s * seedStride + 12 * int64_t(targets[p]);
                land_add<DET>(d + 9 + a, double(acc[p][0]));
                land_add<DET>(d + 3 * a + 0, double(acc[p][1]));
                land_add<DET>(d + 3 * a + 1, double(acc[p][2]));
                land_add<DET>(d + 3 * a + 2, double(acc[p][3]));
            }
        }
    }
    __syncwarp();
}

// Leaf chunks for 8 seeds: lane group g = lane / S (32 / S groups) takes
// every (32/S)-th point of the chunk, lane s = lane % S all three axes of seed
// s, so all 32 lanes work where the blocked form keeps 24 (13% faster at 8M
// nodes; for 16 seeds the blocked form measured faster and stays).
template <int S, bool DET>
__device__ __forceinline__ void reduce_groups(AdjSmem<S> &sm, int m, int base, double *adj, int64_t seedStride) {
    constexpr int G = 32 / S;
    constexpr int P = (AdjSmem<S>::kChunk + G - 1) / G;
    const int lane = threadIdx.x & 31;
    const int s = lane % S, g = lane / S;
    __syncwarp();
    float acc[P][3][4];
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
        for (int a = 0; a < 3; ++a) acc[q][a][0] = acc[q][a][1] = acc[q][a][2] = acc[q][a][3] = 0.f;
    for (int l = 0; l < 32; ++l) {
        const float n[3] = {sm.nb[l][3 * s], sm.nb[l][3 * s + 1], sm.nb[l][3 * s + 2]};
#pragma unroll
        for (int q = 0; q < P; ++q) {
            if (g + G * q < m) {
                const float4 v = sm.vb[g + G * q][l];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    acc[q][a][0] = fmaf(v.x, n[a], acc[q][a][0]);
                    acc[q][a][1] = fmaf(v.y, n[a], acc[q][a][1]);
                    acc[q][a][2] = fmaf(v.z, n[a], acc[q][a][2]);
                    acc[q][a][3] = fmaf(v.w, n[a], acc[q][a][3]);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < P; ++q)
        if (g + G * q < m)
#pragma unroll
            for (int a = 0; a < 3; ++a)
                land_moments<DET>(adj, seedStride, 3 * s + a, base + g + G * q, acc[q][a][0], acc[q][a][1], acc[q][a][2],
                             acc[q][a][3]);
    __syncwarp();
}

// The same reduction for few seeds: one (term, seed component) pair per lane
// task, so that 3 S m tasks keep the warp busy where 3 S lanes alone would
// not.  Each task walks the lanes starting at its term index, which spreads
// the tasks of different terms over the shared-memory banks.
// batch: targets in sm.tgt, a point index or ~node for a cluster term (landed
// in nodeAdj); otherwise points base .. base + m - 1.
template <int S, bool DET>
__device__ __forceinline__ void reduce_tasks(AdjSmem<S> &sm, int m, int base, double *adj, int64_t seedStride,
                                             bool batch = false, double *nodeAdj = nullptr, int64_t nodeStride = 0) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    for (int task = lane; task < 3 * S * m; task += 32) {
        const int p = task / (3 * S), c = task - p * (3 * S);
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll 8
        for (int l0 = 0; l0 < 32; ++l0) {
            const int l = (l0 + p) & 31;
            const float nbv = sm.nb[l][c];
            const float4 v = sm.vb[p][l];
            a0 = fmaf(v.x, nbv, a0);
            a1 = fmaf(v.y, nbv, a1);
            a2 = fmaf(v.z, nbv, a2);
            a3 = fmaf(v.w, nbv, a3);
        }
        if (batch) {
            const int tg = sm.tgt[p];
            if (tg >= 0) land_moments<DET>(adj, seedStride, c, tg, a0, a1, a2, a3);
            else land_moments<DET>(nodeAdj, nodeStride, c, ~tg, a0, a1, a2, a3);
        } else {
            land_moments<DET>(adj, seedStride, c, base + p, a0, a1, a2, a3);
        }
    }
    __syncwarp();
}

// One seed, one term: the 12 products v (x) n of every lane summed over the
// warp (warp_land_moments).  Called by all 32 lanes.
template <bool DET>
__device__ __forceinline__ void reduce_one_s1(const float4 v, const float n[3], double *d) {
    const float vc[4] = {v.x, v.y, v.z, v.w};
    float P[12];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int a = 0; a < 3; ++a) P[3 * k + a] = vc[k] * n[a];
    warp_land_moments<DET>(P, d);
}

// REPLAY: walk the recorded decisions (idw_replay.cu) instead of deciding.
// DET: order-independent landings (idw_land.cuh).
template <int S, int KIND, int REPLAY, bool DET = false>
__global__ void __launch_bounds__(128) k_adjoint_mixed(TreeDev t, TreeDevF tf, PointsDevF pf, VolumeDev v,
                                                       WalkRecF rec, MixedParams mp, Law32<KIND> law, int exact,
                                                       const double *dxv, int64_t dxvStride, const double *den,
                                                       double *ptAdj, int64_t ptStride, double *nodeAdj,
                                                       int64_t nodeStride, unsigned long long *counters,
                                                       WalkLists wlists) {
    extern __shared__ __align__(16) unsigned char smraw[];
    AdjSmem<S> &sm = reinterpret_cast<AdjSmem<S> *>(smraw)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = gid < v.nVol;
    const int64_t g = valid ? gid : 0;
    const int vi = v.perm[g];
    const float4 r0lo = rec.lo[g];
    const int s = __float_as_int(r0lo.w);
    const float den0f = rec.hi[g].w;
    const float Ls = mp.LdefF * pow2f(s);
    const float LsLo = mp.LdefLo * pow2f(s);
    const float c1 = mp.intExp ? pow2f(s * mp.dExp) : exp2f(float(s) * mp.dExpF);
    const float ab = mp.abH, abl = mp.abL;
    const float tauf = mp.errTolF * den0f;
    // numb = dXv / den with den in the scaled units of the walk's weights
    const double q = valid ? exp2(-double(s) * mp.bExp) / den[vi] : 0.0;
    MixedCounters cnt;
    constexpr int kChunk = AdjSmem<S>::kChunk;
    // term indices of the blocked reduction; passed as an array rather than
    // a chunk base, which keeps the 16-seed kernel's register allocation that
    // measured 6% faster at 8M nodes (161.5 vs 171.9 ms)
    int targets[S >= 8 ? kChunk : 1];
    float nl[3] = {0.f, 0.f, 0.f};  // one seed: this lane's, kept in registers
    constexpr bool kBatch = IDW_ADJ_BATCH && S <= 4;
    int npend = 0;  // few seeds: terms waiting in sm.vb (warp-uniform)
    auto flush = [&]() {
        if (npend) {
            reduce_tasks<S, DET>(sm, npend, 0, ptAdj, ptStride, true, nodeAdj, nodeStride);
            npend = 0;
        }
    };
    // one term into the batch: target = point index, or ~node for a cluster
    auto push = [&](const float4 vv, int target) {
        sm.vb[npend][lane] = vv;
        if (lane == 0) sm.tgt[npend] = target;
        if (++npend == kChunk) flush();
    };
    for (int kk = 0; kk < mp.nLoop; ++kk) {
        const float4 rhi = rec.hi[kk * v.nVol + g], rlo = rec.lo[kk * v.nVol + g];
        const float rh[3] = {rhi.x, rhi.y, rhi.z}, rl[3] = {rlo.x, rlo.y, rlo.z};
        // this mirror's seeds: the transpose of the numerator reflection
        // (getMirrorNumerator_b, src/warp/initializeWarping.F90:603-635)
        for (int sd = 0; sd < S; ++sd) {
            const double *dv = dxv + sd * dxvStride + 3 * int64_t(vi);
            float n3[3] = {valid ? float(dv[0] * q) : 0.f, valid ? float(dv[1] * q) : 0.f,
                           valid ? float(dv[2] * q) : 0.f};
#pragma unroll
            for (int j = kMaxSym - 1; j >= 0; --j) {
                if (j < mp.nSym && ((kk >> j) & 1)) {
                    const float dp = n3[0] * mp.nrm[j][0] + n3[1] * mp.nrm[j][1] + n3[2] * mp.nrm[j][2];
                    n3[0] -= 2.f * dp * mp.nrm[j][0];
                    n3[1] -= 2.f * dp * mp.nrm[j][1];
                    n3[2] -= 2.f * dp * mp.nrm[j][2];
                }
            }
            sm.nb[lane][3 * sd] = n3[0];
            sm.nb[lane][3 * sd + 1] = n3[1];
            sm.nb[lane][3 * sd + 2] = n3[2];
            if (S == 1) {
                nl[0] = n3[0];
                nl[1] = n3[1];
                nl[2] = n3[2];
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
                if (__any_sync(kFull, active)) {
                    float h0 = 0.f, h1 = 0.f, h2 = 0.f, l0 = 0.f, l1 = 0.f, l2 = 0.f;
                    if (active) {
                        const float4 ch = ldgf4(&tf.nodes[node].cHi), cl = ldgf4(&tf.nodes[node].cLo);
                        two_diff(rh[0], ch.x, h0, l0);
                        two_diff(rh[1], ch.y, h1, l1);
                        two_diff(rh[2], ch.z, h2, l2);
                        l0 += rl[0] - cl.x;
                        l1 += rl[1] - cl.y;
                        l2 += rl[2] - cl.z;
                        cnt.leafPairs += inf.y - inf.x + 1;
                        cnt.visited++;
                    }
                    const float R0 = h0 + l0, R1 = h1 + l1, R2 = h2 + l2;
                    if constexpr (kBatch) {
                        for (int i = inf.x; i <= inf.y; ++i) {
                            float w = 0.f;
                            if (active) {
                                float dx, dy, dz;
                                w = leaf_weight<KIND>(law, Ls, LsLo, c1, ab, abl, h0, h1, h2, l0, l1, l2,
                                                      ldgf4(pf.da + i), ldgf4(pf.dl + i), dx, dy, dz);
                            }
                            push(make_float4(w, w * R0, w * R1, w * R2), i);
                        }
                    }
                    for (int i0 = inf.x; !kBatch && i0 <= inf.y; i0 += kChunk) {
                        const int m = min(kChunk, inf.y - i0 + 1);
                        for (int p = 0; p < m; ++p) {
                            const int i = i0 + p;
                            if (S >= 16) targets[p] = i;
                            float w = 0.f;
                            if (active) {
                                float dx, dy, dz;
                                w = leaf_weight<KIND>(law, Ls, LsLo, c1, ab, abl, h0, h1, h2, l0, l1, l2,
                                                      ldgf4(pf.da + i), ldgf4(pf.dl + i), dx, dy, dz);
                            }
                            sm.vb[p][lane] = make_float4(w, w * R0, w * R1, w * R2);
                        }
                        if constexpr (S <= 4)
                            reduce_tasks<S, DET>(sm, m, i0, ptAdj, ptStride);
                        else if constexpr (S == 8)
                            reduce_groups<S, DET>(sm, m, i0, ptAdj, ptStride);
                        else
                            reduce_terms<S, DET>(sm, m, targets, ptAdj, ptStride);
                    }
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
                if (__any_sync(kFull, dec == 1)) {
                    float w = 0.f;
                    if (dec == 1) {
                        w = wA * law.eval(fmaf(Ls, rs, LsLo * rs), c1, ab, abl);
                        skip = inf.z;
                        cnt.approx++;
                    }
                    const float4 vv = make_float4(w, w * rho0, w * rho1, w * rho2);
                    if constexpr (kBatch) {
                        push(vv, ~node);
                    } else if constexpr (S == 1) {
                        reduce_one_s1<DET>(vv, nl, nodeAdj + 12 * int64_t(node));
                    } else {
                        sm.vb[0][lane] = vv;
                        if constexpr (S <= 4) {
                            reduce_tasks<S, DET>(sm, 1, node, nodeAdj, nodeStride);
                        } else {
                            targets[0] = node;
                            reduce_terms<S, DET>(sm, 1, targets, nodeAdj, nodeStride);
                        }
                    }
                }
                if (!REPLAY) {
                    if (dec != 1 && active) open = true;
                    node = __any_sync(kFull, open) ? node + 1 : inf.z;
                }
            }
        }
        if constexpr (kBatch) flush();  // before the next pass's seeds
        __syncwarp();
    }
    if (!REPLAY) cnt.flush(counters);
}

// Combine the point and cluster moments into the relative adjoints the
// reverse nodal-property step consumes (setData_b, kd_tree.F90:1033-1051):
//   Bib_i = B_i + sum_q Bq/n_q
//   Mrel_i = P_i - (Xu0_i - C_L) (x) B_i + sum_q (Pq + (C_q - Xu0_i) (x) Bq)/n_q
// where q runs over the interior ancestors of point i.  FP64, one thread per
// (point, seed).
__global__ void k_adjoint_combine(TreeDev t, const dbl4 *ptXA, int nPts, int nSeeds, const double *ptAcc,
                                  int64_t ptStride, const double *nodeAcc, int64_t nodeStride, double *out) {
    const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (tid >= int64_t(nPts) * nSeeds) return;
    const int sd = int(tid / nPts), i = int(tid - int64_t(sd) * nPts);
    const dbl4 x = ptXA[i];
    const double X[3] = {x.x, x.y, x.z};
    double B[3] = {0, 0, 0}, M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int q = 0;
    while (q < t.nNodes) {
        const int4 inf = t.info[q];
        if (inf.w) break;
        const double on = 1.0 / double(inf.y - inf.x + 1);
        const double *a = nodeAcc + sd * nodeStride + 12 * int64_t(q);
        const dbl4 g = t.geom[q];
        const double dc[3] = {g.x - X[0], g.y - X[1], g.z - X[2]};
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            B[r] += a[9 + r] * on;
#pragma unroll
            for (int k = 0; k < 3; ++k) M[3 * r + k] += (a[3 * r + k] + dc[k] * a[9 + r]) * on;
        }
        const int4 li = t.info[q + 1];
        q = (i <= li.y) ? q + 1 : li.z;
    }
    // q is now the leaf of point i
    const dbl4 g = t.geom[q];
    const double dl[3] = {X[0] - g.x, X[1] - g.y, X[2] - g.z};
    const double *p = ptAcc + sd * ptStride + 12 * int64_t(i);
    double *o = out + sd * ptStride + 12 * int64_t(i);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        o[9 + r] = p[9 + r] + B[r];
#pragma unroll
        for (int k = 0; k < 3; ++k) o[3 * r + k] = p[3 * r + k] - dl[k] * p[9 + r] + M[3 * r + k];
    }
}

template <int S, int KIND>
void launch_adj(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v, const WalkRecF &rec,
                const MixedParams &mp, const Law32<KIND> &law, int exact, const double *dxv, int64_t dxvStride,
                const double *den, double *ptAdj, int64_t ptStride, double *nodeAdj, int64_t nodeStride,
                unsigned long long *counters, const WalkLists &wl, cudaStream_t st, int det) {
    const size_t smem = 4 * sizeof(AdjSmem<S>);
    const int g = int((v.nVol + 127) / 128);
    if (det) {  // order-independent landings: the deciding walk
        cudaFuncSetAttribute(k_adjoint_mixed<S, KIND, 0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem));
        k_adjoint_mixed<S, KIND, 0, true><<<g, 128, smem, st>>>(t, tf, pf, v, rec, mp, law, exact, dxv, dxvStride,
                                                                den, ptAdj, ptStride, nodeAdj, nodeStride, counters, wl);
    } else if (wl.list && !exact) {
        launch_add_walk_counters(counters, wl.counters, st);
        cudaFuncSetAttribute(k_adjoint_mixed<S, KIND, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        k_adjoint_mixed<S, KIND, 1><<<g, 128, smem, st>>>(t, tf, pf, v, rec, mp, law, exact, dxv, dxvStride, den,
                                                          ptAdj, ptStride, nodeAdj, nodeStride, counters, wl);
    } else {
        cudaFuncSetAttribute(k_adjoint_mixed<S, KIND, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        k_adjoint_mixed<S, KIND, 0><<<g, 128, smem, st>>>(t, tf, pf, v, rec, mp, law, exact, dxv, dxvStride, den,
                                                          ptAdj, ptStride, nodeAdj, nodeStride, counters, wl);
    }
}

template <int S>
void launch_adj_law(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v,
                    const WalkRecF &rec, const MixedParams &mp, const WeightLaw &wl, int exact, const double *dxv,
                    int64_t dxvStride, const double *den, double *ptAdj, int64_t ptStride, double *nodeAdj,
                    int64_t nodeStride, unsigned long long *counters, const WalkLists &lists, cudaStream_t st,
                    int det) {
    if (wl.isInt && wl.ia == 3 && wl.ib == 5) {
        launch_adj<S, 0>(t, tf, pf, v, rec, mp, Law32<0>{3, 5, 3.f, 5.f}, exact, dxv, dxvStride, den, ptAdj, ptStride,
                         nodeAdj, nodeStride, counters, lists, st, det);
    } else if (wl.isInt) {
        launch_adj<S, 1>(t, tf, pf, v, rec, mp, Law32<1>{wl.ia, wl.ib, float(wl.aExp), float(wl.bExp)}, exact, dxv,
                         dxvStride, den, ptAdj, ptStride, nodeAdj, nodeStride, counters, lists, st, det);
    } else {
        launch_adj<S, 2>(t, tf, pf, v, rec, mp, Law32<2>{0, 0, float(wl.aExp), float(wl.bExp)}, exact, dxv,
                         dxvStride, den, ptAdj, ptStride, nodeAdj, nodeStride, counters, lists, st, det);
    }
}

}  // namespace

void launch_adjoint_combine(const TreeDev &t, const dbl4 *ptXA, int nPts, int nSeeds, const double *ptAcc,
                            const double *nodeAcc, double *ptAdj, cudaStream_t st) {
    const int64_t total = int64_t(nPts) * nSeeds;
    if (total <= 0) return;
    k_adjoint_combine<<<int((total + 127) / 128), 128, 0, st>>>(t, ptXA, nPts, nSeeds, ptAcc, 12 * int64_t(nPts),
                                                                nodeAcc, 12 * int64_t(t.nNodes), ptAdj);
}

int launch_adjoint_mixed(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v,
                         const WalkRecF &rec, const EvalConsts &k, int exact, const double *dxv, int nSeeds,
                         int64_t dxvStride, const double *den, double *ptAcc, double *nodeAcc, double *ptAdj,
                         const dbl4 *ptXA, int nPts, unsigned long long *counters, cudaStream_t st, int maxGroup,
                         int combine, int det) {
    if (nSeeds <= 0) return 0;
    const MixedParams mp = make_mixed_params(k);
    const int64_t ptStride = 12 * int64_t(nPts), nodeStride = 12 * int64_t(t.nNodes);
    // no volume nodes: no walk, the combination below writes zero adjoints
    int s0 = v.nVol > 0 ? 0 : nSeeds;
    // exact mode on a mesh that fills the GPU: seeds that would walk alone go
    // through the tiled kernel (2.6x the one-seed walk on the 2M-node wing);
    // groups of 4, 8 or 16 keep the shared walk (16 seeds: 4.7 s against 16
    // tiled passes, 5.8 s)
    const bool tiledOne = exact && tf.nLeaves > 0 && k.exactSchedule != IDW_EXACT_WALK &&
                          (k.exactSchedule == IDW_EXACT_TILED || exact_tiled_fills(v.nVol));
    while (s0 < nSeeds) {
        const int left = nSeeds - s0;
        const double *d = dxv + s0 * dxvStride;
        double *pa = ptAcc + s0 * ptStride, *na = nodeAcc + s0 * nodeStride;
        // seeds in groups of 16, 8, 4 or 1 sharing one walk, none above maxGroup
        if (left >= 16 && maxGroup >= 16) {
            launch_adj_law<16>(t, tf, pf, v, rec, mp, k.law, exact, d, dxvStride, den, pa, ptStride, na, nodeStride,
                               counters, k.lists, st, det);
            s0 += 16;
        } else if (left >= 8 && maxGroup >= 8) {
            launch_adj_law<8>(t, tf, pf, v, rec, mp, k.law, exact, d, dxvStride, den, pa, ptStride, na, nodeStride,
                              counters, k.lists, st, det);
            s0 += 8;
        } else if (left >= 4 && maxGroup >= 4) {
            launch_adj_law<4>(t, tf, pf, v, rec, mp, k.law, exact, d, dxvStride, den, pa, ptStride, na, nodeStride,
                              counters, k.lists, st, det);
            s0 += 4;
        } else if (tiledOne) {
            launch_exact_adjoint(tf, pf, v, rec, mp, k.law, d, den, pa, counters, st, det);
            s0 += 1;
        } else {
            launch_adj_law<1>(t, tf, pf, v, rec, mp, k.law, exact, d, dxvStride, den, pa, ptStride, na, nodeStride,
                              counters, k.lists, st, det);
            s0 += 1;
        }
    }
    if (!combine) return 0;
    const int64_t total = int64_t(nPts) * nSeeds;
    k_adjoint_combine<<<int((total + 127) / 128), 128, 0, st>>>(t, ptXA, nPts, nSeeds, ptAcc, ptStride, nodeAcc,
                                                                nodeStride, ptAdj);
    return 0;
}

IDW_LAND_SETTER(land_set_adjoint)

}  // namespace idw
