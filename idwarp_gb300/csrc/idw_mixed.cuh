// Shared device code of the mixed-precision walks (forward and adjoint):
// FP32 weight law, error-table lookup, compensated sums, double-float
// arithmetic and the guarded open/approximate decision.
#pragma once
#include "idw_common.cuh"
#include "idw_kernels.h"
#include "idw_land.cuh"

namespace idw {

// Per-lane work counters of the frequent events (32-bit per lane; summed in
// 64 bits per warp at the end).  Slots: dst[0] leaf pairs, dst[1] cluster
// approximations, dst[2] visited nodes; the rare events (FP64 decision
// fallbacks dst[3], diagnostic slot counts dst[4..5], double-float terms
// dst[6]) go straight to memory with warp_count, which keeps them out of the
// walk's registers.
struct MixedCounters {
    unsigned leafPairs = 0, approx = 0, visited = 0;
    __device__ void flush(unsigned long long *dst) {
        if (!dst) return;
        const unsigned long long v[3] = {leafPairs, approx, visited};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const unsigned long long s = warp_sum(v[k]);
            if ((threadIdx.x & 31) == 0 && s) atomicAdd(dst + k, s);
        }
    }
};

// Warp-wide count into dst[k]; every lane of a converged warp must call it.
__device__ __forceinline__ void warp_count(unsigned long long *dst, int k, unsigned v) {
    const unsigned s = __reduce_add_sync(kFull, v);
    if (dst && s && (threadIdx.x & 31) == 0) atomicAdd(dst + k, (unsigned long long)s);
}

// Law kinds: 0 = exponents (3,5); 1 = other integer exponents; 2 = real.
template <int KIND>
struct Law32 {
    int ia, ib;
    float fa, fb;
    // c1 t^a + (ab + abl) t^b; ab + abl is alpha^b split in two floats so the
    // FP32 terms carry the same alpha^b as the double-float terms.
    __device__ __forceinline__ float eval(float t, float c1, float ab, float abl) const {
        if (KIND == 0) {
            float t2 = t * t;
            float t3 = t2 * t;
            float t5 = t3 * t2;
            return fmaf(c1, t3, fmaf(ab, t5, abl * t5));
        } else if (KIND == 1) {
            float ta = ipowf(t, ia);
            float tb = ta * ipowf(t, ib - ia);
            return fmaf(c1, ta, fmaf(ab, tb, abl * tb));
        } else {
            return c1 * powf(t, fa) + ab * powf(t, fb);
        }
    }
};

// Compensated summation (Neumaier / Ogita-Rump-Oishi Sum2): the sum is s + c,
// with every rounding error of the running sum captured exactly by two-sum
// and collected in c, so the pair is accurate to ~u^2 relative.
__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
    const float t = s + x;
    const float bp = t - s;
    c += (s - (t - bp)) + (x - bp);
    s = t;
}

// Packed FP32 pairs (the f32x2 instructions of sm_100 and later): each half
// is rounded exactly as the scalar operation, so a packed sequence gives the
// scalar results bit for bit with one instruction issued for two.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;"
        : "=l"(d)
        : "l"(*reinterpret_cast<const unsigned long long *>(&a)), "l"(*reinterpret_cast<const unsigned long long *>(&b)));
    return *reinterpret_cast<const float2 *>(&d);
}

// kahan_add on two independent pairs at once (bitwise two kahan_add calls).
__device__ __forceinline__ void kahan_add2(float2 &s, float2 &c, float2 x) {
    const float2 t = add2(s, x);
    const float2 bp = sub2(t, s);
    c = add2(c, add2(sub2(s, sub2(t, bp)), sub2(x, bp)));
    s = t;
}

// Running sums of one mirror pass in the forward walks: numerator and
// denominator, each a compensated pair (sum = s + c), packed as (num0, num1)
// and (num2, den) for kahan_add2.
struct Sums2 {
    float2 s01, s2d, c01, c2d;
};

__device__ __forceinline__ float4 ldgf4(const float4 *p) { return __ldg(p); }
__device__ __forceinline__ int4 ldgi4(const int4 *p) { return __ldg(p); }

// 1/sqrt(x) for an x that is normal or zero: the flush-to-zero form of the
// approximate reciprocal square root gives the value rsqrtf gives, without
// rsqrtf's handling of subnormal inputs.
__device__ __forceinline__ float rsqrt_normal(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// FP32 error-table interpolation with a bound on its deviation from the FP64
// value (see the file comment).  dOvrR >= 2 here.  The bracket index follows
// the radii 2,3,4,5,7.5,10,20,40,...,640: unit steps below 5, then 7.5 and 10,
// then doublings from 20.  Returns err, sets bnd.
__device__ __forceinline__ float get_error32(const float *e, float dOvrR, float &bnd) {
    // Bracket [r0, r1) and 1/(r1 - r0) by selects, so lanes in different
    // brackets do not diverge; the values equal the reference's bracket and
    // the correctly rounded reciprocal (1, 0.4, 0.4, 0.1, 0.05 * 2^-m).
    const float d = dOvrR;
    const float fl = floorf(d);
    // 20 * 2^m <= d < 20 * 2^(m+1) for d in [20, 640), m = 0..4
    const int m = min(4, max(0, ((__float_as_int(d * 0.05f) >> 23) & 0xff) - 127));
    const float p2 = __int_as_float((127 + m) << 23), ip2 = __int_as_float((127 - m) << 23);
    const bool a = d < 5.0f, b = d < 7.5f, c = d < 10.0f, t = d < 20.0f, far = d >= 640.0f;
    int i = a ? int(fl) - 2 : (b ? 3 : (c ? 4 : (t ? 5 : 6 + m)));
    const float r0 = a ? fl : (b ? 5.0f : (c ? 7.5f : (t ? 10.0f : 20.0f * p2)));
    const float orst = a ? 1.0f : (c ? 0.4f : (t ? 0.1f : 0.05f * ip2));
    i = far ? kNerr - 2 : i;
    const float e0 = __ldg(e + i), e1 = __ldg(e + i + 1);
    const float fact = (d - r0) * orst;
    bnd = far ? 2e-6f * fabsf(e1) : 2e-6f * (d * orst * fabsf(e1 - e0) + fabsf(e0) + fabsf(e1));
    return far ? e1 : (1.0f - fact) * e0 + fact * e1;
}

// Exact difference a - b as (hi, lo) (Knuth two-sum).
__device__ __forceinline__ void two_diff(float a, float b, float &hi, float &lo) {
    hi = a - b;
    const float bb = hi - a;
    lo = (a - (hi - bb)) - (b + bb);
}

// ---- double-float (hi + lo) arithmetic for the precision-critical far-field
// cluster terms (Dekker/Knuth error-free transformations with FMA) ----
struct dfl {
    float h, l;
};
__device__ __forceinline__ dfl df_norm(float h, float l) {
    const float s = h + l;
    return {s, l - (s - h)};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    float s, e;
    s = a.h + b.h;
    const float bb = s - a.h;
    e = (a.h - (s - bb)) + (b.h - bb);
    e += a.l + b.l;
    return df_norm(s, e);
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return df_norm(p, e);
}
// 1/sqrt(q) with one Newton step carried in double-float.
__device__ __forceinline__ dfl df_rsqrt(dfl q) {
    const float y0 = rsqrtf(q.h);
    const float t = y0 * y0;
    const float te = fmaf(y0, y0, -t);  // y0^2 = t + te exactly
    const float p = q.h * t;
    float e = fmaf(q.h, t, -p);
    e = fmaf(q.h, te, e);
    e = fmaf(q.l, t, e);
    const float r = (1.0f - p) - e;  // 1 - q y0^2 (1 - p is exact near 1)
    return df_norm(y0, 0.5f * y0 * r);
}
template <int KIND>
__device__ __forceinline__ dfl df_pow_int(dfl t, int n) {
    if (KIND == 0 && n == 3) return df_mul(df_mul(t, t), t);
    dfl r = {1.0f, 0.0f}, b = t;
    while (n > 0) {
        if (n & 1) r = df_mul(r, b);
        n >>= 1;
        if (n) b = df_mul(b, b);
    }
    return r;
}
// Compensated accumulation of a double-float term into a pair (s + c).
__device__ __forceinline__ void kahan_add_df(float &s, float &c, dfl x) {
    kahan_add(s, c, x.h);
    kahan_add(s, c, x.l);
}

// Knuth two-sum: a + b = s + e exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

// Accumulate a double-float value (h + l) into the compensated pair (s + c).
__device__ __forceinline__ void comp_add_df(float &s, float &c, float h, float l) {
    float e;
    two_sum(s, h, s, e);
    c += e + l;
}

// One term of the IDW sums in double-float, for terms whose FP32 rounding
// would show in Xv: x (hi + lo) is the volume point relative to the term's
// reference point (a surface point, or a cluster centroid), eps the distance
// softening (1e-15 for surface points, 0 for clusters), A (hi + lo) the area,
// and S = D x + c with D (9) and c (3) from the hi/lo arrays dh, dl.
// precise_weight returns the renormalised x and the weight w (hi + lo),
// specialised to the default exponents (3, 5), other exponents through the
// generic double-float routines; precise_motion adds w S to a compensated
// pair; precise_term is both, and adds w to the denominator pair.
template <int KIND>
__device__ __forceinline__ void precise_weight(const dfl xin[3], float eps, float Ah, float Al, const Law32<KIND> &law,
                                               float Ls, float LsLo, float c1, float abH, float abL, dfl x[3],
                                               float &wh, float &wl) {
    // x arrives as an exact difference plus a correction that can be as
    // large as the difference itself (a volume node on a surface node:
    // hi = -lo); renormalise so that |lo| <= ulp(hi) / 2, which the
    // products below assume (they drop lo * lo)
#pragma unroll
    for (int k = 0; k < 3; ++k) two_sum(xin[k].h, xin[k].l, x[k].h, x[k].l);
    if (KIND == 0) {
        // d^2 = |x|^2 + eps
        const float p0 = x[0].h * x[0].h, p1 = x[1].h * x[1].h, p2 = x[2].h * x[2].h;
        const float e0 = fmaf(x[0].h, x[0].h, -p0), e1 = fmaf(x[1].h, x[1].h, -p1), e2 = fmaf(x[2].h, x[2].h, -p2);
        float s1, f1, s2, f2;
        two_sum(p0, p1, s1, f1);
        two_sum(s1, p2, s2, f2);
        // the softening eps can be as large as |x|^2 (a volume node on a
        // surface node): add it with an exact two-sum, collect every rounding
        // error in the low part, then renormalise so that |dl| is below half
        // an ulp of dh, which the Newton residual below relies on
        float s3, f3;
        two_sum(s2, eps, s3, f3);
        const float lo0 = ((e0 + e1) + (e2 + f1)) + (f2 + f3) +
                          2.f * fmaf(x[0].h, x[0].l, fmaf(x[1].h, x[1].l, x[2].h * x[2].l));
        float dh2, dl2;
        two_sum(s3, lo0, dh2, dl2);
        // y = 1/sqrt(d^2): FP32 seed, one Newton step carried in double-float
        const float y0 = rsqrtf(dh2);
        const float t = y0 * y0, te = fmaf(y0, y0, -t);
        const float p = dh2 * t;
        float e = fmaf(dh2, t, -p);
        e = fmaf(dh2, te, e);
        e = fmaf(dl2, t, e);
        const float y1 = 0.5f * y0 * ((1.0f - p) - e);
        // t = L y and its powers (unnormalised double-float products)
        const float th = Ls * y0;
        float tl = fmaf(Ls, y0, -th);
        tl = fmaf(Ls, y1, fmaf(LsLo, y0, tl));
        const float t2h = th * th;
        const float t2l = fmaf(2.f * th, tl, fmaf(th, th, -t2h));
        const float t3h = t2h * th;
        const float t3l = fmaf(t2l, th, fmaf(t2h, tl, fmaf(t2h, th, -t3h)));
        const float t5h = t3h * t2h;
        const float t5l = fmaf(t3l, t2h, fmaf(t3h, t2l, fmaf(t3h, t2h, -t5h)));
        // law = c1 t^3 + alpha^b t^5, then w = A law
        const float bh = abH * t5h;
        const float bl = fmaf(abL, t5h, fmaf(abH, t5l, fmaf(abH, t5h, -bh)));
        float lh, ll;
        two_sum(c1 * t3h, bh, lh, ll);
        ll += fmaf(c1, t3l, bl);
        wh = Ah * lh;
        wl = fmaf(Al, lh, fmaf(Ah, ll, fmaf(Ah, lh, -wh)));
    } else {
        dfl d2 = df_add(df_add(df_add(df_mul(x[0], x[0]), df_mul(x[1], x[1])), df_mul(x[2], x[2])), {eps, 0.f});
        const dfl tt = df_mul({Ls, LsLo}, df_rsqrt(d2));
        const dfl ta = df_pow_int<KIND>(tt, law.ia);
        const dfl tb = df_mul(ta, df_pow_int<KIND>(tt, law.ib - law.ia));
        const dfl lawv = df_add({c1 * ta.h, c1 * ta.l}, df_mul(tb, {abH, abL}));
        const dfl w = df_mul(lawv, {Ah, Al});
        wh = w.h;
        wl = w.l;
    }
}

__device__ __forceinline__ void precise_motion(const dfl x[3], float wh, float wl, const float *dh, const float *dl,
                                               float *sn, float *cn) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // S_a = c_a + sum_k D_ak x_k, each product split exactly, sums by two-sum
        float Sh = __ldg(dh + 9 + a), Sl = __ldg(dl + 9 + a);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float Dh = __ldg(dh + 3 * a + k), Dl = __ldg(dl + 3 * a + k);
            const float ph = Dh * x[k].h;
            const float pl = fmaf(Dl, x[k].h, fmaf(Dh, x[k].l, fmaf(Dh, x[k].h, -ph)));
            float er;
            two_sum(Sh, ph, Sh, er);
            Sl += er + pl;
        }
        // w S (double-float product) into the running pair
        const float qh = wh * Sh;
        const float ql = fmaf(wl, Sh, fmaf(wh, Sl, fmaf(wh, Sh, -qh)));
        comp_add_df(sn[a], cn[a], qh, ql);
    }
}


template <int KIND>
__device__ __forceinline__ void precise_term(const dfl xin[3], float eps, float Ah, float Al, const float *dh,
                                             const float *dl, const Law32<KIND> &law, float Ls, float LsLo, float c1,
                                             float abH, float abL, float *sn, float *cn, float &sd, float &cd) {
    dfl x[3];
    float wh, wl;
    precise_weight<KIND>(xin, eps, Ah, Al, law, Ls, LsLo, c1, abH, abL, x, wh, wl);
    precise_motion(x, wh, wl, dh, dl, sn, cn);
    comp_add_df(sd, cd, wh, wl);
}

// Interior-node decision of the mixed walks from the FP32 records.  Returns 0
// (open), 1 (approximate) or 2 (too close to a threshold for FP32: the caller
// re-takes it with decide64).  Also returns r - C (FP32), |r - C|^2, its
// reciprocal square root and the node area, which the approximation needs.
// The geometry of a cluster term from the split point (rh + rl) and the split
// centroid (ch + cl; cl.w is the node area): r - C in FP32, |r - C|^2 and its
// reciprocal square root.  Shared by the decision and by every walk that
// evaluates the term, so a replayed term is bitwise the walked one.
__device__ __forceinline__ void cluster_geo(const float4 ch, const float4 cl, const float *rh, const float *rl,
                                            float &rho0, float &rho1, float &rho2, float &d2, float &rs, float &wA) {
    wA = cl.w;
    rho0 = (rh[0] - ch.x) + (rl[0] - cl.x);
    rho1 = (rh[1] - ch.y) + (rl[1] - cl.y);
    rho2 = (rh[2] - ch.z) + (rl[2] - cl.z);
    d2 = fmaf(rho0, rho0, fmaf(rho1, rho1, rho2 * rho2));
    // d2 is zero (a node on the centroid: dOvrR is NaN, the decision goes to
    // FP64) or far above the subnormal range (the components are differences
    // of hi/lo splits, resolved to ~1e-15), so the flush-to-zero form serves
    rs = rsqrt_normal(d2);
}

__device__ __forceinline__ int decide32(const TreeDevF &tf, int node, const float *rh, const float *rl, float tauf,
                                        float &rho0, float &rho1, float &rho2, float &d2, float &rs, float &wA) {
    const float4 ch = ldgf4(&tf.nodes[node].cHi), cl = ldgf4(&tf.nodes[node].cLo);
    cluster_geo(ch, cl, rh, rl, rho0, rho1, rho2, d2, rs, wA);
    const float dOvrR = d2 * rs * ch.w;
    if (dOvrR < 2.0f * (1.0f - 4e-6f)) return 0;
    if (dOvrR <= 2.0f * (1.0f + 4e-6f)) return 2;
    float bnd;
    const float err = get_error32(tf.nodes[node].err, dOvrR, bnd);
    bnd += 1e-6f * tauf;
    return (err + bnd < tauf) ? 1 : ((err - bnd > tauf) ? 0 : 2);
}

// The FP64 decision of one lane, out of line: it is rare (about one visit in
// 1e5), and keeping its FP64 code out of the walks' loops keeps their
// register allocation to the FP32 path.
static __device__ __noinline__ int decide64_lane(const dbl4 *geom, const double *err, const int *perm, const double *den0,
                                          int64_t g, int node, float rh0, float rh1, float rh2, float rl0,
                                          float rl1, float rl2, double errTol) {
    const int vi = perm[g];
    const double r[3] = {double(rh0) + double(rl0), double(rh1) + double(rl1), double(rh2) + double(rl2)};
    double dist64;
    return decide64(geom[node], err + kNerr * node, r, errTol * den0[vi], dist64);
}

// Re-take undecided decisions with the FP64 rule (all lanes of the warp call
// this; the FP64 work runs only when some lane needs it).
__device__ __forceinline__ int resolve64(int dec, const TreeDev &t, const VolumeDev &v, int64_t g, int node,
                                         const float *rh, const float *rl, double errTol,
                                         unsigned long long *counters) {
    if (__any_sync(kFull, dec == 2)) {
        const bool redo = dec == 2;
        if (redo) dec = decide64_lane(t.geom, t.err, v.perm, v.den0, g, node, rh[0], rh[1], rh[2], rl[0], rl[1], rl[2],
                                      errTol);
        warp_count(counters, 3, redo ? 1u : 0u);
    }
    return dec;
}

// The warp's sum of the 12 moment products P[3 k + a] (k = 0: w, k = 1..3:
// w (r - C)_k; a the seed axis) of every lane, landed in one term's adjoint
// accumulator d (slots 9 + a for w, 3 a + k - 1 for the moments).  Two
// halving exchanges (xor 16, 8) leave lane group G = lane >> 3 with the 3
// products of moment G; three butterflies (xor 4, 2, 1) complete the sums;
// lanes 0..2 of each group land them.  Called by all 32 lanes.
template <bool DET>
__device__ __forceinline__ void warp_land_moments(const float *P, double *d) {
    const int lane = threadIdx.x & 31;
    const bool h16 = lane & 16, h8 = lane & 8;
    float Q[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float send = h16 ? P[k] : P[k + 6];
        Q[k] = (h16 ? P[k + 6] : P[k]) + __shfl_xor_sync(kFull, send, 16);
    }
    float R[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float send = h8 ? Q[k] : Q[k + 3];
        R[k] = (h8 ? Q[k + 3] : Q[k]) + __shfl_xor_sync(kFull, send, 8);
    }
#pragma unroll
    for (int o = 4; o; o >>= 1)
#pragma unroll
        for (int k = 0; k < 3; ++k) R[k] += __shfl_xor_sync(kFull, R[k], o);
    const int G = lane >> 3, a = lane & 7;
    if (a < 3) {
        const float val = a == 0 ? R[0] : (a == 1 ? R[1] : R[2]);
        if (val != 0.f) land_add<DET>(d + (G == 0 ? 9 + a : 3 * a + G - 1), double(val));
    }
}

// Power of two 2^e as a float (|e| <= 126).
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + max(-126, min(127, e))) << 23); }

// Per-volume-node constants of the mixed evaluation, from its walk record:
// sigma = 2^s scales the weights (Ls = Ldef sigma split in two floats, c1 =
// sigma^(b-a)), tauf = errTol den0 (FP32 decisions), and the precision gate
// gv: a term whose FP32 rounding, w (|S'| + |D'| |r - X|) u, could exceed
// mixedGate * Ldef * u of the final denominator is summed in double-float.
// The final (scaled) denominator is the walk's own from an earlier pass (it
// depends on Xu0 and the weight law only), else the estimate den0 sigma^b
// (which overestimates it on the wall, where den0's softening 1e-16 is below
// the walk's 1e-15).
struct NodeScale {
    float Ls, LsLo, c1, tauf, gv;
    int s;
};
__device__ __forceinline__ NodeScale node_scale(const WalkRecF &rec, const MixedParams &mp, int64_t g) {
    NodeScale n;
    const float4 r0lo = rec.lo[g];
    n.s = __float_as_int(r0lo.w);
    const float den0f = rec.hi[g].w;
    n.Ls = mp.LdefF * pow2f(n.s);
    n.LsLo = mp.LdefLo * pow2f(n.s);
    n.c1 = mp.intExp ? pow2f(n.s * mp.dExp) : exp2f(float(n.s) * mp.dExpF);
    n.tauf = mp.errTolF * den0f;
    if (rec.gden) {
        n.gv = mp.precGate * rec.gden[g];
    } else {
        const float gexp = float(n.s) * mp.bExpF;
        const float gexpi = floorf(gexp);
        n.gv = mp.precGate * ldexpf(den0f, int(gexpi)) * exp2f(gexp - gexpi);
    }
    return n;
}


// One leaf pair in FP32 (evalNodeExact's term, kd_tree.F90:664-690): h + l
// is r - C (leaf centroid), da + dl the point's offset from C and its area,
// m0..m2 the point's D' (row-major, 9) and u' (3); accumulates w S and w.
// The weight of one leaf pair (and the pair's offset dx, dy, dz).
template <int KIND>
__device__ __forceinline__ float leaf_weight(const Law32<KIND> &law, float Ls, float LsLo, float c1, float ab,
                                             float abl, float h0, float h1, float h2, float l0, float l1, float l2,
                                             const float4 da, const float4 dl, float &dx, float &dy, float &dz) {
    dx = (h0 - da.x) + (l0 - dl.x);
    dy = (h1 - da.y) + (l1 - dl.y);
    dz = (h2 - da.z) + (l2 - dl.z);
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, 1e-15f)));
    const float r1 = rsqrt_normal(d2);
    const float tt = fmaf(Ls, r1, LsLo * r1);
    return da.w * law.eval(tt, c1, ab, abl);
}

template <int KIND>
__device__ __forceinline__ void leaf_pair(const Law32<KIND> &law, float Ls, float LsLo, float c1, float ab,
                                          float abl, float h0, float h1, float h2, float l0, float l1, float l2,
                                          const float4 da, const float4 dl, const float4 m0, const float4 m1,
                                          const float4 m2, float &pn0, float &pn1, float &pn2, float &pd) {
    float dx, dy, dz;
    const float w = leaf_weight<KIND>(law, Ls, LsLo, c1, ab, abl, h0, h1, h2, l0, l1, l2, da, dl, dx, dy, dz);
    // S = D dx + u ; D row-major in m0.xyzw m1.xyzw m2.x, u in m2.yzw
    const float S0 = fmaf(m0.x, dx, fmaf(m0.y, dy, fmaf(m0.z, dz, m2.y)));
    const float S1 = fmaf(m0.w, dx, fmaf(m1.x, dy, fmaf(m1.y, dz, m2.z)));
    const float S2 = fmaf(m1.z, dx, fmaf(m1.w, dy, fmaf(m2.x, dz, m2.w)));
    pn0 = fmaf(w, S0, pn0);
    pn1 = fmaf(w, S1, pn1);
    pn2 = fmaf(w, S2, pn2);
    pd += w;
}

// The leaf gate's measure: the leaf's FP32 partial sums bound the rounding
// of its terms, pd |D'| |r - C| that of the lever arm (all forms share it,
// so their gates decide alike).
__device__ __forceinline__ float leaf_gate_mag(float pn0, float pn1, float pn2, float pd, float dn, float h0,
                                               float h1, float h2) {
    return fabsf(pn0) + fabsf(pn1) + fabsf(pn2) + pd * dn * (fabsf(h0) + fabsf(h1) + fabsf(h2));
}

// End of a leaf: its partial sums go into the compensated running sums,
// unless the leaf carries a large weight at a long lever arm (the cluster
// terms' gate, with dn the leaf's bound on |D'|); returns true for such a
// leaf, which the caller re-sums in double-float (precise_leaf).
template <int KIND>
__device__ __forceinline__ bool leaf_close(float pn0, float pn1, float pn2, float pd, float dn, float h0, float h1,
                                           float h2, float gv, float *sn, float *cn, float &sd, float &cd) {
    const bool precise = KIND != 2 && leaf_gate_mag(pn0, pn1, pn2, pd, dn, h0, h1, h2) > gv;
    if (!precise) {
        kahan_add(sn[0], cn[0], pn0);
        kahan_add(sn[1], cn[1], pn1);
        kahan_add(sn[2], cn[2], pn2);
        kahan_add(sd, cd, pd);
    }
    return precise;
}

// leaf_close on the packed running sums (the same gate, bitwise the same sums).
template <int KIND>
__device__ __forceinline__ bool leaf_close2(float pn0, float pn1, float pn2, float pd, float dn, float h0, float h1,
                                            float h2, float gv, Sums2 &r) {
    const bool precise = KIND != 2 && leaf_gate_mag(pn0, pn1, pn2, pd, dn, h0, h1, h2) > gv;
    if (!precise) {
        kahan_add2(r.s01, r.c01, make_float2(pn0, pn1));
        kahan_add2(r.s2d, r.c2d, make_float2(pn2, pd));
    }
    return precise;
}

// A leaf's terms (points lo..hi) re-summed in double-float.
template <int KIND>
__device__ __forceinline__ void precise_leaf(const TreeDevF &tf, const PointsDevF &pf, int node, int lo, int hi,
                                             const float *rh, const float *rl, const Law32<KIND> &law, float Ls,
                                             float LsLo, float c1, float abH, float abL, float *sn, float *cn,
                                             float &sd, float &cd) {
    const float4 ch = ldgf4(&tf.nodes[node].cHi), cl = ldgf4(&tf.nodes[node].cLo);
    dfl q0, q1, q2;
    two_diff(rh[0], ch.x, q0.h, q0.l);
    two_diff(rh[1], ch.y, q1.h, q1.l);
    two_diff(rh[2], ch.z, q2.h, q2.l);
    q0.l += rl[0] - cl.x;
    q1.l += rl[1] - cl.y;
    q2.l += rl[2] - cl.z;
    for (int i = lo; i <= hi; ++i) {
        const float4 da = ldgf4(pf.da + i), dl = ldgf4(pf.dl + i);
        dfl x[3];
        two_diff(q0.h, da.x, x[0].h, x[0].l);
        two_diff(q1.h, da.y, x[1].h, x[1].l);
        two_diff(q2.h, da.z, x[2].h, x[2].l);
        x[0].l += q0.l - dl.x;
        x[1].l += q1.l - dl.y;
        x[2].l += q2.l - dl.z;
        precise_term<KIND>(x, 1e-15f, da.w, dl.w, pf.dm + 12 * i, pf.dml + 12 * i, law, Ls, LsLo, c1, abH, abL, sn,
                           cn, sd, cd);
    }
}

// Running sums of one mirror pass (num 3 + den, each a compensated pair),
// passed by value to the out-of-line double-float paths below so that the
// walks keep them in registers.
struct RunSums {
    float sn[3], cn[3], sd, cd;
};
__device__ __forceinline__ RunSums to_runsums(const Sums2 &r) {
    return {{r.s01.x, r.s01.y, r.s2d.x}, {r.c01.x, r.c01.y, r.c2d.x}, r.s2d.y, r.c2d.y};
}
__device__ __forceinline__ Sums2 from_runsums(const RunSums &a) {
    return {make_float2(a.sn[0], a.sn[1]), make_float2(a.sn[2], a.sd), make_float2(a.cn[0], a.cn[1]),
            make_float2(a.cn[2], a.cd)};
}

// A cluster term in double-float (the walk's precision gate sent it here):
// h + l is the split volume point, ch/cl the split centroid (cl.w = area hi),
// aLo the area's low part, dc/dcl the cluster's D', c' hi/lo.  Out of line,
// like precise_leaf: rare, and register-heavy.
template <int KIND>
__device__ __noinline__ RunSums precise_cluster(RunSums a, float rh0, float rh1, float rh2, float rl0, float rl1,
                                                float rl2, float4 ch, float4 cl, float aLo, const float *dc,
                                                const float *dcl, Law32<KIND> law, float Ls, float LsLo, float c1,
                                                float abH, float abL) {
    dfl q[3];
    two_diff(rh0, ch.x, q[0].h, q[0].l);
    two_diff(rh1, ch.y, q[1].h, q[1].l);
    two_diff(rh2, ch.z, q[2].h, q[2].l);
    q[0].l += rl0 - cl.x;
    q[1].l += rl1 - cl.y;
    q[2].l += rl2 - cl.z;
    precise_term<KIND>(q, 0.f, cl.w, aLo, dc, dcl, law, Ls, LsLo, c1, abH, abL, a.sn, a.cn, a.sd, a.cd);
    return a;
}

// precise_leaf out of line, on the running sums by value.
template <int KIND>
__device__ __noinline__ RunSums precise_leaf_ool(RunSums a, const TreeDevF tf, const PointsDevF pf, int node, int lo,
                                                 int hi, float rh0, float rh1, float rh2, float rl0, float rl1,
                                                 float rl2, Law32<KIND> law, float Ls, float LsLo, float c1, float abH,
                                                 float abL) {
    const float rh[3] = {rh0, rh1, rh2}, rl[3] = {rl0, rl1, rl2};
    precise_leaf<KIND>(tf, pf, node, lo, hi, rh, rl, law, Ls, LsLo, c1, abH, abL, a.sn, a.cn, a.sd, a.cd);
    return a;
}

// ---- the two kinds of walk step, shared by the decision walk (idw_mixed.cu)
// and the replay of recorded decisions (idw_replay.cu), so both sum the same
// terms with the same arithmetic in the same order ----

// Per-lane constants of a forward mixed walk.
template <int KIND>
struct WalkLane {
    Law32<KIND> law;
    float Ls, LsLo, c1, ab, abl, gv;
};

// A leaf summed by the lanes with `mine` set: pair terms relative to the leaf
// centroid (split in *chp + *clp; .w unused), partial sums into the running
// pairs, and heavy leaves (the gate of leaf_close with the leaf's |D'| bound
// *dnp) re-summed in double-float.  Called by all 32 lanes; the record
// pointers let the deciding walk and the replay read their own layouts.
template <int KIND>
__device__ __forceinline__ void leaf_step(bool mine, const TreeDevF &tf, const PointsDevF &pf, int node, int lo,
                                          int hi, const float4 *chp, const float4 *clp, const float *dnp,
                                          const float *rh, const float *rl, const WalkLane<KIND> &wl, Sums2 &r,
                                          unsigned long long *counters) {
    bool leafPrecise = false;
    if (mine) {
        const float4 ch = ldgf4(chp), cl = ldgf4(clp);
        // r - C as hi + lo: exact high parts, so a volume node on a surface
        // node resolves d^2 = eps (1e-15) to full precision
        float h0, h1, h2, l0, l1, l2;
        two_diff(rh[0], ch.x, h0, l0);
        two_diff(rh[1], ch.y, h1, l1);
        two_diff(rh[2], ch.z, h2, l2);
        l0 += rl[0] - cl.x;
        l1 += rl[1] - cl.y;
        l2 += rl[2] - cl.z;
        float pn0 = 0.f, pn1 = 0.f, pn2 = 0.f, pd = 0.f;
        for (int i = lo; i <= hi; ++i) {
            const float4 *dm = reinterpret_cast<const float4 *>(pf.dm + 12 * i);
            leaf_pair<KIND>(wl.law, wl.Ls, wl.LsLo, wl.c1, wl.ab, wl.abl, h0, h1, h2, l0, l1, l2, ldgf4(pf.da + i),
                            ldgf4(pf.dl + i), ldgf4(dm), ldgf4(dm + 1), ldgf4(dm + 2), pn0, pn1, pn2, pd);
        }
        // a leaf carrying a large weight at a long lever arm is re-summed in
        // double-float (same gate as cluster terms)
        leafPrecise = leaf_close2<KIND>(pn0, pn1, pn2, pd, __ldg(dnp), h0, h1, h2, wl.gv, r);
    }
    if (__any_sync(kFull, leafPrecise)) {
        if (leafPrecise)
            r = from_runsums(precise_leaf_ool<KIND>(to_runsums(r), tf, pf, node, lo, hi, rh[0], rh[1], rh[2], rl[0],
                                                    rl[1], rl[2], wl.law, wl.Ls, wl.LsLo, wl.c1, wl.ab, wl.abl));
        warp_count(counters, 6, leafPrecise ? unsigned(hi - lo + 1) : 0u);
    }
}

// One cluster term from its geometry (cluster_geo) and the cluster's D', c'
// (m0..m2, 12 floats) and |D'| bound dn: w = A law(L/d), S = D' (r - C) + c',
// added to the running pairs unless the term carries a large weight at a long
// lever arm (then returns true: the caller re-evaluates it in double-float).
template <int KIND>
__device__ __forceinline__ bool approx_add(const float4 m0, const float4 m1, const float4 m2, float dn, float rho0,
                                           float rho1, float rho2, float rs, float wA, const WalkLane<KIND> &wl,
                                           Sums2 &r) {
    const float tt = fmaf(wl.Ls, rs, wl.LsLo * rs);
    const float w = wA * wl.law.eval(tt, wl.c1, wl.ab, wl.abl);
    const float S0 = fmaf(m0.x, rho0, fmaf(m0.y, rho1, fmaf(m0.z, rho2, m2.y)));
    const float S1 = fmaf(m0.w, rho0, fmaf(m1.x, rho1, fmaf(m1.y, rho2, m2.z)));
    const float S2 = fmaf(m1.z, rho0, fmaf(m1.w, rho1, fmaf(m2.x, rho2, m2.w)));
    const float mag = fabsf(S0) + fabsf(S1) + fabsf(S2) + dn * (fabsf(rho0) + fabsf(rho1) + fabsf(rho2));
    const bool precise = KIND != 2 && w * mag > wl.gv;
    if (!precise) {
        const float2 ww = make_float2(w, w);
        kahan_add2(r.s01, r.c01, mul2(make_float2(S0, S1), ww));
        kahan_add2(r.s2d, r.c2d, mul2(make_float2(S2, 1.0f), ww));
    }
    return precise;
}

// The double-float re-evaluation of the cluster terms approx_add declined.
// Called by all 32 lanes.
template <int KIND>
__device__ __forceinline__ void approx_vote(bool precise, const TreeDevF &tf, const NodeAggF &af, int node,
                                            const float *rh, const float *rl, const WalkLane<KIND> &wl, Sums2 &r,
                                            unsigned long long *counters) {
    if (__any_sync(kFull, precise)) {
        if (precise)
            r = from_runsums(precise_cluster<KIND>(to_runsums(r), rh[0], rh[1], rh[2], rl[0], rl[1], rl[2],
                                                   ldgf4(&tf.nodes[node].cHi), ldgf4(&tf.nodes[node].cLo),
                                                   __ldg(&tf.nodes[node].aLo), af.dc + 12 * node, af.dcl + 12 * node,
                                                   wl.law, wl.Ls, wl.LsLo, wl.c1, wl.ab, wl.abl));
        warp_count(counters, 6, precise ? 1u : 0u);
    }
}

// A cluster approximated by the lanes with `mine` set (the deciding walk:
// the cluster's motion is loaded where a lane approximates).  The arithmetic
// is approx_add's, written out here: inlined through approx_add the deciding
// walk's register allocation spilled five times more.  Called by all 32
// lanes.
template <int KIND>
__device__ __forceinline__ void approx_step(bool mine, const TreeDevF &tf, const NodeAggF &af, int node, float rho0,
                                            float rho1, float rho2, float rs, float wA, const float *rh,
                                            const float *rl, const WalkLane<KIND> &wl, Sums2 &r,
                                            unsigned long long *counters) {
    bool precise = false;
    if (mine) {
        const float tt = fmaf(wl.Ls, rs, wl.LsLo * rs);
        const float w = wA * wl.law.eval(tt, wl.c1, wl.ab, wl.abl);
        const float4 *dc = reinterpret_cast<const float4 *>(af.dc + 12 * node);
        const float4 m0 = ldgf4(dc), m1 = ldgf4(dc + 1), m2 = ldgf4(dc + 2);
        const float S0 = fmaf(m0.x, rho0, fmaf(m0.y, rho1, fmaf(m0.z, rho2, m2.y)));
        const float S1 = fmaf(m0.w, rho0, fmaf(m1.x, rho1, fmaf(m1.y, rho2, m2.z)));
        const float S2 = fmaf(m1.z, rho0, fmaf(m1.w, rho1, fmaf(m2.x, rho2, m2.w)));
        const float mag = fabsf(S0) + fabsf(S1) + fabsf(S2) +
                          __ldg(af.dn + node) * (fabsf(rho0) + fabsf(rho1) + fabsf(rho2));
        precise = KIND != 2 && w * mag > wl.gv;
        if (!precise) {
            const float2 ww = make_float2(w, w);
            kahan_add2(r.s01, r.c01, mul2(make_float2(S0, S1), ww));
            kahan_add2(r.s2d, r.c2d, mul2(make_float2(S2, 1.0f), ww));
        }
    }
    approx_vote<KIND>(precise, tf, af, node, rh, rl, wl, r, counters);
}

// End of one mirror pass: add the reference motion back, num += den (Dref r +
// bref) with r the mirror's point, reflect the numerator back (vector
// reflection) and add (num, den) into the running pair S4 + C4, all in
// double-float so no digits are lost between mirrors.  S4, C4 are overwritten
// when there is a single pass.
__device__ __forceinline__ void finish_mirror(const NodeAggF &af, const MixedParams &mp, int kk, const float *rh,
                                              const float *rl, const float *sn, const float *cn, float sd, float cd,
                                              float4 &S4, float4 &C4) {
    const dfl den = df_norm(sd, cd);
    dfl num[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        dfl sr = {__ldg(af.ref + 9 + a), __ldg(af.ref + 21 + a)};
#pragma unroll
        for (int k = 0; k < 3; ++k)
            sr = df_add(sr, df_mul({__ldg(af.ref + 3 * a + k), __ldg(af.ref + 12 + 3 * a + k)}, {rh[k], rl[k]}));
        num[a] = df_add(df_norm(sn[a], cn[a]), df_mul(den, sr));
    }
    if (mp.nLoop == 1) {
        S4 = make_float4(num[0].h, num[1].h, num[2].h, den.h);
        C4 = make_float4(num[0].l, num[1].l, num[2].l, den.l);
        return;
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
    kahan_add_df(S4.x, C4.x, num[0]);
    kahan_add_df(S4.y, C4.y, num[1]);
    kahan_add_df(S4.z, C4.z, num[2]);
    kahan_add_df(S4.w, C4.w, den);
}

}  // namespace idw
