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

// k_exact_mixed for the default exponents (3, 5) with the volume nodes of a
// thread taken two at a time in packed FP32 pairs (f32x2): each node's
// arithmetic is leaf_pair's, rounding for rounding, so the sums stay bitwise
// the walk's, while one instruction serves two nodes.  The staged points are
// kept duplicated ((x, x, y, y) per float4), so every point operand of a pair
// instruction comes straight from shared memory.
constexpr int kTile2 = 128;  // surface points per shared-memory pass (static shared memory)

template <int NV>
__global__ void __launch_bounds__(kThreads) k_exact_mixed2(TreeDevF tf, PointsDevF pf, NodeAggF af, VolumeDev v,
                                                           WalkRecF rec, MixedParams mp, Law32<0> law, float4 *acc,
                                                           unsigned long long *counters) {
    constexpr int NP = NV / 2;  // node pairs per thread
    const int nPts = tf.nPts;
    // per point: (dx, dx, dy, dy), (dz, dz, A, A), (lx, lx, ly, ly), (lz, lz, 0, 0), then D', u' in pairs
    __shared__ float4 sP[10 * kTile2];
    __shared__ float4 sRH[NV][kThreads], sRL[NV][kThreads];
    const int tid = threadIdx.x;
    const int64_t base = int64_t(blockIdx.x) * (kThreads * NV);
    bool valid[NV];
    int64_t g[NV];
    float2 LS[NP], LSLO[NP], C1[NP];
    float gv[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        const int64_t gid = base + j * kThreads + tid;
        valid[j] = gid < v.nVol;
        g[j] = valid[j] ? gid : 0;
        const NodeScale ns = node_scale(rec, mp, g[j]);
        if (j & 1) {
            LS[j >> 1].y = ns.Ls;
            LSLO[j >> 1].y = ns.LsLo;
            C1[j >> 1].y = ns.c1;
        } else {
            LS[j >> 1].x = ns.Ls;
            LSLO[j >> 1].x = ns.LsLo;
            C1[j >> 1].x = ns.c1;
        }
        gv[j] = ns.gv;
    }
    const float2 AB = dup2(mp.abH), ABL = dup2(mp.abL), EPS = dup2(1e-15f);
    MixedCounters cnt;
    for (int kk = 0; kk < mp.nLoop; ++kk) {
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            sRH[j][tid] = rec.hi[kk * v.nVol + g[j]];
            sRL[j][tid] = rec.lo[kk * v.nVol + g[j]];
        }
        // running compensated sums (numerator 3, denominator) of the node pairs
        float2 SN[NP][3], CN[NP][3], SD[NP], CD[NP];
        float2 H[NP][3], Lw[NP][3], PN[NP][3], PD[NP];
#pragma unroll
        for (int jj = 0; jj < NP; ++jj) {
#pragma unroll
            for (int a = 0; a < 3; ++a)
                SN[jj][a] = CN[jj][a] = H[jj][a] = Lw[jj][a] = PN[jj][a] = make_float2(0.f, 0.f);
            SD[jj] = CD[jj] = PD[jj] = make_float2(0.f, 0.f);
        }
        int leaf = 0;
        int4 L = tf.leaves[0];  // (l, u, node): the leaf in progress
        for (int p0 = 0; p0 < nPts; p0 += kTile2) {
            const int p1 = min(nPts, p0 + kTile2);
            __syncthreads();
            for (int q = tid; q < p1 - p0; q += kThreads) {
                const float4 da = ldgf4(pf.da + p0 + q), dl = ldgf4(pf.dl + p0 + q);
                const float4 *dmp = reinterpret_cast<const float4 *>(pf.dm) + 3 * int64_t(p0 + q);
                const float4 m0 = ldgf4(dmp), m1 = ldgf4(dmp + 1), m2 = ldgf4(dmp + 2);
                float4 *o = sP + 10 * q;
                o[0] = make_float4(da.x, da.x, da.y, da.y);
                o[1] = make_float4(da.z, da.z, da.w, da.w);
                o[2] = make_float4(dl.x, dl.x, dl.y, dl.y);
                o[3] = make_float4(dl.z, dl.z, 0.f, 0.f);
                o[4] = make_float4(m0.x, m0.x, m0.y, m0.y);
                o[5] = make_float4(m0.z, m0.z, m0.w, m0.w);
                o[6] = make_float4(m1.x, m1.x, m1.y, m1.y);
                o[7] = make_float4(m1.z, m1.z, m1.w, m1.w);
                o[8] = make_float4(m2.x, m2.x, m2.y, m2.y);
                o[9] = make_float4(m2.z, m2.z, m2.w, m2.w);
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
                        float hh[3], ll[3];
                        two_diff(rh.x, ch.x, hh[0], ll[0]);
                        two_diff(rh.y, ch.y, hh[1], ll[1]);
                        two_diff(rh.z, ch.z, hh[2], ll[2]);
                        ll[0] += rl.x - cl.x;
                        ll[1] += rl.y - cl.y;
                        ll[2] += rl.z - cl.z;
#pragma unroll
                        for (int a = 0; a < 3; ++a) {
                            if (j & 1) {
                                H[j >> 1][a].y = hh[a];
                                Lw[j >> 1][a].y = ll[a];
                            } else {
                                H[j >> 1][a].x = hh[a];
                                Lw[j >> 1][a].x = ll[a];
                            }
                        }
                    }
#pragma unroll
                    for (int jj = 0; jj < NP; ++jj) {
                        PN[jj][0] = PN[jj][1] = PN[jj][2] = PD[jj] = make_float2(0.f, 0.f);
                    }
                }
                const int e = min(L.y + 1, p1);
                for (int q = p - p0; q < e - p0; ++q) {
                    const float4 *o = sP + 10 * q;
                    const float4 a0 = o[0], a1 = o[1], l0 = o[2], l1 = o[3];
                    const float4 d0 = o[4], d1 = o[5], d2 = o[6], d3 = o[7], d4 = o[8], d5 = o[9];
#pragma unroll
                    for (int jj = 0; jj < NP; ++jj) {
                        // leaf_pair for two nodes
                        const float2 dx = add2(sub2(H[jj][0], lo2(a0)), sub2(Lw[jj][0], lo2(l0)));
                        const float2 dy = add2(sub2(H[jj][1], hi2(a0)), sub2(Lw[jj][1], hi2(l0)));
                        const float2 dz = add2(sub2(H[jj][2], lo2(a1)), sub2(Lw[jj][2], lo2(l1)));
                        const float2 q2 = fma2(dx, dx, fma2(dy, dy, fma2(dz, dz, EPS)));
                        const float2 r1 = make_float2(rsqrt_normal(q2.x), rsqrt_normal(q2.y));
                        const float2 tt = fma2(LS[jj], r1, mul2(LSLO[jj], r1));
                        const float2 t2 = mul2(tt, tt);
                        const float2 t3 = mul2(t2, tt);
                        const float2 t5 = mul2(t3, t2);
                        const float2 lw = fma2(C1[jj], t3, fma2(AB, t5, mul2(ABL, t5)));
                        const float2 w = mul2(hi2(a1), lw);
                        const float2 S0 = fma2(lo2(d0), dx, fma2(hi2(d0), dy, fma2(lo2(d1), dz, hi2(d4))));
                        const float2 S1 = fma2(hi2(d1), dx, fma2(lo2(d2), dy, fma2(hi2(d2), dz, lo2(d5))));
                        const float2 S2 = fma2(lo2(d3), dx, fma2(hi2(d3), dy, fma2(lo2(d4), dz, hi2(d5))));
                        PN[jj][0] = fma2(w, S0, PN[jj][0]);
                        PN[jj][1] = fma2(w, S1, PN[jj][1]);
                        PN[jj][2] = fma2(w, S2, PN[jj][2]);
                        PD[jj] = add2(PD[jj], w);
                    }
                }
                p = e;
                if (e == L.y + 1) {
                    // leaf end: gate, compensated sums, heavy leaves in double-float
                    const float dn = __ldg(af.dn + L.z);
                    const unsigned size = unsigned(L.y - L.x + 1);
                    unsigned precisePairs = 0;
#pragma unroll
                    for (int jj = 0; jj < NP; ++jj) {
                        // leaf_close for the pair: the gate per node, the
                        // compensated adds packed (bitwise kahan_add per node)
                        const bool pa = leaf_gate_mag(PN[jj][0].x, PN[jj][1].x, PN[jj][2].x, PD[jj].x, dn,
                                                      H[jj][0].x, H[jj][1].x, H[jj][2].x) > gv[2 * jj];
                        const bool pb = leaf_gate_mag(PN[jj][0].y, PN[jj][1].y, PN[jj][2].y, PD[jj].y, dn,
                                                      H[jj][0].y, H[jj][1].y, H[jj][2].y) > gv[2 * jj + 1];
                        if (!pa && !pb) {
#pragma unroll
                            for (int a = 0; a < 3; ++a) kahan_add2(SN[jj][a], CN[jj][a], PN[jj][a]);
                            kahan_add2(SD[jj], CD[jj], PD[jj]);
                        } else {
#pragma unroll
                            for (int a = 0; a < 3; ++a) {
                                if (!pa) kahan_add(SN[jj][a].x, CN[jj][a].x, PN[jj][a].x);
                                if (!pb) kahan_add(SN[jj][a].y, CN[jj][a].y, PN[jj][a].y);
                            }
                            if (!pa) kahan_add(SD[jj].x, CD[jj].x, PD[jj].x);
                            if (!pb) kahan_add(SD[jj].y, CD[jj].y, PD[jj].y);
                        }
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int j = 2 * jj + h;
                            if (valid[j]) {
                                cnt.leafPairs += size;
                                cnt.visited++;
                            }
                            if ((h ? pb : pa) && valid[j]) {
                                const float4 rh = sRH[j][tid], rl = sRL[j][tid];
                                const float rhv[3] = {rh.x, rh.y, rh.z}, rlv[3] = {rl.x, rl.y, rl.z};
                                float sn[3], cn[3], sd, cd;
#pragma unroll
                                for (int a = 0; a < 3; ++a) {
                                    sn[a] = h ? SN[jj][a].y : SN[jj][a].x;
                                    cn[a] = h ? CN[jj][a].y : CN[jj][a].x;
                                }
                                sd = h ? SD[jj].y : SD[jj].x;
                                cd = h ? CD[jj].y : CD[jj].x;
                                precise_leaf<0>(tf, pf, L.z, L.x, L.y, rhv, rlv, law, h ? LS[jj].y : LS[jj].x,
                                                h ? LSLO[jj].y : LSLO[jj].x, h ? C1[jj].y : C1[jj].x, mp.abH,
                                                mp.abL, sn, cn, sd, cd);
#pragma unroll
                                for (int a = 0; a < 3; ++a) {
                                    if (h) {
                                        SN[jj][a].y = sn[a];
                                        CN[jj][a].y = cn[a];
                                    } else {
                                        SN[jj][a].x = sn[a];
                                        CN[jj][a].x = cn[a];
                                    }
                                }
                                if (h) {
                                    SD[jj].y = sd;
                                    CD[jj].y = cd;
                                } else {
                                    SD[jj].x = sd;
                                    CD[jj].x = cd;
                                }
                                precisePairs += size;
                            }
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
            const int jj = j >> 1;
            const bool odd = j & 1;
            const float snj[3] = {odd ? SN[jj][0].y : SN[jj][0].x, odd ? SN[jj][1].y : SN[jj][1].x,
                                  odd ? SN[jj][2].y : SN[jj][2].x};
            const float cnj[3] = {odd ? CN[jj][0].y : CN[jj][0].x, odd ? CN[jj][1].y : CN[jj][1].x,
                                  odd ? CN[jj][2].y : CN[jj][2].x};
            finish_mirror(af, mp, kk, rhv, rlv, snj, cnj, odd ? SD[jj].y : SD[jj].x, odd ? CD[jj].y : CD[jj].x, S4,
                          C4);
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
template <int KIND, int NV, bool DET = false>
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
                    warp_land_moments<DET>(P, ptAdj + 12 * int64_t(p0 + t));
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
    if constexpr (KIND == 0) {
        if (blocks_for(v.nVol, kThreads * 4) >= sm_count() * kBlocksPerSmNV4)
            k_exact_mixed2<4><<<blocks_for(v.nVol, kThreads * 4), kThreads, 0, st>>>(tf, pf, af, v, rec, mp, law, acc,
                                                                                    counters);
        else
            k_exact_mixed2<2><<<blocks_for(v.nVol, kThreads * 2), kThreads, 0, st>>>(tf, pf, af, v, rec, mp, law, acc,
                                                                                    counters);
        return;
    }
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
                          double *ptAdj, unsigned long long *counters, cudaStream_t st, int det) {
    if (v.nVol <= 0 || tf.nPts <= 0 || tf.nLeaves <= 0) return;
    constexpr int NV = 4;
    const int grid = blocks_for(v.nVol, kThreads * NV);
    if (det) {  // order-independent landings (idw_land.cuh)
        if (wl.isInt && wl.ia == 3 && wl.ib == 5)
            k_exact_adjoint<0, NV, true><<<grid, kThreads, 0, st>>>(tf, pf, v, rec, mp, Law32<0>{3, 5, 3.f, 5.f}, dxv,
                                                                    den, ptAdj, counters);
        else if (wl.isInt)
            k_exact_adjoint<1, NV, true><<<grid, kThreads, 0, st>>>(
                tf, pf, v, rec, mp, Law32<1>{wl.ia, wl.ib, float(wl.aExp), float(wl.bExp)}, dxv, den, ptAdj, counters);
        else
            k_exact_adjoint<2, NV, true><<<grid, kThreads, 0, st>>>(
                tf, pf, v, rec, mp, Law32<2>{0, 0, float(wl.aExp), float(wl.bExp)}, dxv, den, ptAdj, counters);
    } else if (wl.isInt && wl.ia == 3 && wl.ib == 5) {
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

IDW_LAND_SETTER(land_set_exact)

}  // namespace idw
