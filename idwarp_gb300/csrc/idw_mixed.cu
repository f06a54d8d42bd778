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
//   * each leaf's partial sums are added to Kahan-compensated FP32 running
//     sums; normalisation, mirror reflection and the add-back to Xv0 are FP64.
// Open/approximate decisions are taken in FP32 only when they are further
// from the threshold than the FP32 error bound; otherwise they are re-taken
// with the FP64 decision of the FP64 form (decide64), so the mixed walk makes
// exactly the FP64 walk's decisions.
#include "idw_common.cuh"
#include "idw_kernels.h"

namespace idw {

namespace {

struct MixedCounters {
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

// Law kinds: 0 = exponents (3,5); 1 = other integer exponents; 2 = real.
template <int KIND>
struct Law32 {
    int ia, ib;
    float fa, fb;
    __device__ __forceinline__ float eval(float t, float c1, float ab) const {
        if (KIND == 0) {
            float t2 = t * t;
            float t3 = t2 * t;
            float t5 = t3 * t2;
            return c1 * t3 + ab * t5;
        } else if (KIND == 1) {
            float ta = ipowf(t, ia);
            float tb = ta * ipowf(t, ib - ia);
            return c1 * ta + ab * tb;
        } else {
            return c1 * powf(t, fa) + ab * powf(t, fb);
        }
    }
};

__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

__device__ __forceinline__ float4 ldgf4(const float4 *p) { return __ldg(p); }

// FP32 error-table interpolation with a bound on its deviation from the FP64
// value (see the file comment).  Returns err, sets bnd.
__device__ __forceinline__ float get_error32(const float *e, float dOvrR, float &bnd) {
    const float rs[kNerr] = {2.f, 3.f, 4.f, 5.f, 7.5f, 10.f, 20.f, 40.f, 80.f, 160.f, 320.f, 640.f};
#pragma unroll
    for (int i = 0; i < kNerr - 1; ++i) {
        if (dOvrR < rs[i + 1]) {
            float orst = 1.0f / (rs[i + 1] - rs[i]);
            float e0 = __ldg(e + i), e1 = __ldg(e + i + 1);
            float fact = (dOvrR - rs[i]) * orst;
            bnd = 2e-6f * (dOvrR * orst * fabsf(e1 - e0) + fabsf(e0) + fabsf(e1));
            return (1.0f - fact) * e0 + fact * e1;
        }
    }
    float e11 = __ldg(e + kNerr - 1);
    bnd = 2e-6f * fabsf(e11);
    return e11;
}

template <int KIND>
__global__ void __launch_bounds__(128) k_walk_mixed(TreeDev t, TreeDevF tf, PointsDevF pf, NodeAggF af,
                                                    VolumeDev v, EvalConsts k, Law32<KIND> law, int exact,
                                                    WalkOut o) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = gid < v.nVol;
    const int vi = valid ? v.perm[gid] : 0;
    const double x0[3] = {v.xv0[3 * vi], v.xv0[3 * vi + 1], v.xv0[3 * vi + 2]};
    const double den0 = v.den0[vi];
    const double tolDen = k.errTol * den0;
    // per-node power-of-two scale: sigma^b ~ 1/den0
    int s = 0;
    if (den0 > 0.0 && den0 < 1e300) {
        int e = ilogb(den0);
        double sb = -double(e) / k.law.bExp;
        s = max(-40, min(40, int(rint(sb))));
    }
    const float Ls = float(ldexp(k.law.Ldef, s));
    const float c1 = float(exp2(double(s) * (k.law.bExp - k.law.aExp)));
    const float ab = float(k.law.alphaToBexp);
    const float tauf = float(fmin(tolDen, 3.0e38));
    double numer[3] = {0, 0, 0}, denom = 0.0;
    MixedCounters cnt;
    for (int kk = 0; kk < k.sym.nLoop; ++kk) {
        double r[3];
        mirror_point(k.sym, kk, x0, r);
        float rh[3], rl[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            rh[c] = float(r[c]);
            rl[c] = float(r[c] - double(rh[c]));
        }
        float sn[3] = {0, 0, 0}, cn[3] = {0, 0, 0}, sd = 0.f, cd = 0.f;
        int node = 0, skip = 0;
        while (node < t.nNodes) {
            const int4 inf = t.info[node];
            const bool active = valid && node >= skip;
            if (inf.w) {
                if (active) {
                    const float4 ch = ldgf4(tf.cHi + node), cl = ldgf4(tf.cLo + node);
                    const float rho0 = (rh[0] - ch.x) + (rl[0] - cl.x);
                    const float rho1 = (rh[1] - ch.y) + (rl[1] - cl.y);
                    const float rho2 = (rh[2] - ch.z) + (rl[2] - cl.z);
                    float pn0 = 0.f, pn1 = 0.f, pn2 = 0.f, pd = 0.f;
                    for (int i = inf.x; i <= inf.y; ++i) {
                        const float4 da = ldgf4(pf.da + i);
                        const float4 *dm = reinterpret_cast<const float4 *>(pf.dm + 12 * i);
                        const float4 m0 = ldgf4(dm), m1 = ldgf4(dm + 1), m2 = ldgf4(dm + 2);
                        const float dx = rho0 - da.x, dy = rho1 - da.y, dz = rho2 - da.z;
                        const float d2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, 1e-15f)));
                        const float tt = Ls * rsqrtf(d2);
                        const float w = da.w * law.eval(tt, c1, ab);
                        // S = D dx + u ; D row-major in m0.xyzw m1.xyzw m2.x, u in m2.yzw
                        const float S0 = fmaf(m0.x, dx, fmaf(m0.y, dy, fmaf(m0.z, dz, m2.y)));
                        const float S1 = fmaf(m0.w, dx, fmaf(m1.x, dy, fmaf(m1.y, dz, m2.z)));
                        const float S2 = fmaf(m1.z, dx, fmaf(m1.w, dy, fmaf(m2.x, dz, m2.w)));
                        pn0 = fmaf(w, S0, pn0);
                        pn1 = fmaf(w, S1, pn1);
                        pn2 = fmaf(w, S2, pn2);
                        pd += w;
                    }
                    kahan_add(sn[0], cn[0], pn0);
                    kahan_add(sn[1], cn[1], pn1);
                    kahan_add(sn[2], cn[2], pn2);
                    kahan_add(sd, cd, pd);
                    cnt.leafPairs += inf.y - inf.x + 1;
                    cnt.visited++;
                }
                node = inf.z;
            } else {
                bool open = false;
                if (active) {
                    if (exact) {
                        open = true;
                    } else {
                        cnt.visited++;
                        const float4 ch = ldgf4(tf.cHi + node), cl = ldgf4(tf.cLo + node);
                        const float rho0 = (rh[0] - ch.x) + (rl[0] - cl.x);
                        const float rho1 = (rh[1] - ch.y) + (rl[1] - cl.y);
                        const float rho2 = (rh[2] - ch.z) + (rl[2] - cl.z);
                        const float d2 = fmaf(rho0, rho0, fmaf(rho1, rho1, rho2 * rho2));
                        const float dist = sqrtf(d2);
                        const float dOvrR = dist * ch.w;
                        int dec;  // 0 open, 1 approximate, 2 undecided in FP32
                        if (dOvrR < 2.0f * (1.0f - 4e-6f)) {
                            dec = 0;
                        } else if (dOvrR <= 2.0f * (1.0f + 4e-6f)) {
                            dec = 2;
                        } else {
                            float bnd;
                            float err = get_error32(tf.err + kNerr * node, dOvrR, bnd);
                            bnd += 1e-6f * tauf;
                            if (err + bnd < tauf)
                                dec = 1;
                            else if (err - bnd > tauf)
                                dec = 0;
                            else
                                dec = 2;
                        }
                        if (dec == 2) {
                            double dist64;
                            dec = decide64(t.geom[node], t.err + kNerr * node, r, tolDen, dist64);
                            cnt.fallback++;
                        }
                        if (dec == 1) {
                            const float tt = Ls * rsqrtf(d2);
                            const float w = cl.w * law.eval(tt, c1, ab);
                            const float4 *dc = reinterpret_cast<const float4 *>(af.dc + 12 * node);
                            const float4 m0 = ldgf4(dc), m1 = ldgf4(dc + 1), m2 = ldgf4(dc + 2);
                            const float S0 = fmaf(m0.x, rho0, fmaf(m0.y, rho1, fmaf(m0.z, rho2, m2.y)));
                            const float S1 = fmaf(m0.w, rho0, fmaf(m1.x, rho1, fmaf(m1.y, rho2, m2.z)));
                            const float S2 = fmaf(m1.z, rho0, fmaf(m1.w, rho1, fmaf(m2.x, rho2, m2.w)));
                            kahan_add(sn[0], cn[0], w * S0);
                            kahan_add(sn[1], cn[1], w * S1);
                            kahan_add(sn[2], cn[2], w * S2);
                            kahan_add(sd, cd, w);
                            skip = inf.z;
                            cnt.approx++;
                        } else {
                            open = true;
                        }
                    }
                }
                node = __any_sync(kFull, open) ? node + 1 : inf.z;
            }
        }
        double num[3] = {double(sn[0]) - double(cn[0]), double(sn[1]) - double(cn[1]), double(sn[2]) - double(cn[2])};
        mirror_vector(k.sym, kk, num);
        numer[0] += num[0];
        numer[1] += num[1];
        numer[2] += num[2];
        denom += double(sd) - double(cd);
    }
    if (valid) {
        double oden = 1.0 / denom;
        if (o.xv) {
            o.xv[3 * vi + 0] = x0[0] + numer[0] * oden;
            o.xv[3 * vi + 1] = x0[1] + numer[1] * oden;
            o.xv[3 * vi + 2] = x0[2] + numer[2] * oden;
        }
        // true-unit denominator: divide out sigma^b
        if (o.den) o.den[vi] = denom * exp2(-double(s) * k.law.bExp);
    }
    cnt.flush(o.counters);
}

inline int blocks(int64_t n, int b) { return int((n + b - 1) / b); }

}  // namespace

void launch_walk_mixed(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af,
                       const VolumeDev &v, const EvalConsts &k, int exact, const WalkOut &o, cudaStream_t st) {
    if (v.nVol <= 0) return;
    const int g = blocks(v.nVol, 128);
    if (k.law.isInt && k.law.ia == 3 && k.law.ib == 5) {
        Law32<0> law{3, 5, 3.f, 5.f};
        k_walk_mixed<0><<<g, 128, 0, st>>>(t, tf, pf, af, v, k, law, exact, o);
    } else if (k.law.isInt) {
        Law32<1> law{k.law.ia, k.law.ib, float(k.law.aExp), float(k.law.bExp)};
        k_walk_mixed<1><<<g, 128, 0, st>>>(t, tf, pf, af, v, k, law, exact, o);
    } else {
        Law32<2> law{0, 0, float(k.law.aExp), float(k.law.bExp)};
        k_walk_mixed<2><<<g, 128, 0, st>>>(t, tf, pf, af, v, k, law, exact, o);
    }
}

}  // namespace idw
