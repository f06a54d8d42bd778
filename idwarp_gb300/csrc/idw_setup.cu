// Set-up kernels: error tables, denominator estimate, Morton ordering of the
// volume nodes and the FP32 companion arrays of the mixed-precision path.
//   computeErrors  src/modules/kd_tree.F90:832-880 (+ getSpherePts, src/utils/getSpherePts.F90)
//   getWiEstimate  src/modules/kd_tree.F90:751-787, driven by src/warp/initializeWarping.F90:241-247
//   restart check  src/warp/initializeWarping.F90:190-209 (every stride-th node re-estimated)
//   dryRun         src/modules/kd_tree.F90:789-830, driven by src/warp/initializeWarping.F90:258-266
#include <cub/cub.cuh>

#include <climits>
#include <cmath>
#include <vector>

#include "idw_common.cuh"
#include "idw_kernels.h"

namespace idw {

namespace {

// Dodecahedron vertices before scaling (src/utils/getSpherePts.F90:16-39);
// phi = 2.1180339887498949 as in src/modules/constants.F90:32.
__device__ __forceinline__ void sphere_vertex(int ii, double *v) {
    const double p = 2.1180339887498949, ip = 1.0 / 2.1180339887498949;
    const double o = 1.0;
    switch (ii) {
        case 0: v[0] = -o; v[1] = -o; v[2] = -o; break;
        case 1: v[0] = o; v[1] = -o; v[2] = -o; break;
        case 2: v[0] = -o; v[1] = o; v[2] = -o; break;
        case 3: v[0] = o; v[1] = o; v[2] = -o; break;
        case 4: v[0] = -o; v[1] = -o; v[2] = o; break;
        case 5: v[0] = o; v[1] = -o; v[2] = o; break;
        case 6: v[0] = -o; v[1] = o; v[2] = o; break;
        case 7: v[0] = o; v[1] = o; v[2] = o; break;
        case 8: v[0] = 0; v[1] = -ip; v[2] = -p; break;
        case 9: v[0] = 0; v[1] = ip; v[2] = -p; break;
        case 10: v[0] = 0; v[1] = -ip; v[2] = p; break;
        case 11: v[0] = 0; v[1] = ip; v[2] = p; break;
        case 12: v[0] = -ip; v[1] = -p; v[2] = 0; break;
        case 13: v[0] = ip; v[1] = -p; v[2] = 0; break;
        case 14: v[0] = -ip; v[1] = p; v[2] = 0; break;
        case 15: v[0] = ip; v[1] = p; v[2] = 0; break;
        case 16: v[0] = -p; v[1] = 0; v[2] = -ip; break;
        case 17: v[0] = -p; v[1] = 0; v[2] = ip; break;
        case 18: v[0] = p; v[1] = 0; v[2] = -ip; break;
        default: v[0] = p; v[1] = 0; v[2] = ip; break;
    }
}

__device__ __forceinline__ void sphere_point(const dbl4 &g, int t, double *pt) {
    // t = 20*j + ii: radius (1/oradius)*rstar(j), vertex ii
    int j = t / 20, ii = t - 20 * j;
    double v[3];
    sphere_vertex(ii, v);
    double radius = (1.0 / g.w) * c_rstar[j];
    double s = radius / sqrt(3.0);
    pt[0] = v[0] * s + g.x;
    pt[1] = v[1] * s + g.y;
    pt[2] = v[2] * s + g.z;
}

struct ErrItem {
    int node, i0, i1, pad;
};

constexpr int kErrChunk = 512;

// Partial exact sums over one chunk of one node's members for its 240 probe
// points.
__global__ void k_err_partial(TreeDev t, const dbl4 *ptXA, WeightLaw law, const ErrItem *items, double *part) {
    const ErrItem it = items[blockIdx.x];
    const dbl4 g = t.geom[it.node];
    __shared__ dbl4 sx[256];
    const int tid = threadIdx.x;
    double pt[3] = {0, 0, 0};
    if (tid < 240) sphere_point(g, tid, pt);
    double acc = 0.0;
    for (int base = it.i0; base < it.i1; base += 256) {
        int m = min(256, it.i1 - base);
        __syncthreads();
        if (tid < m) sx[tid] = ptXA[base + tid];
        __syncthreads();
        if (tid < 240) {
            for (int k = 0; k < m; ++k) {
                dbl4 x = sx[k];
                double r0 = pt[0] - x.x, r1 = pt[1] - x.y, r2 = pt[2] - x.z;
                double dist = sqrt(r0 * r0 + r1 * r1 + r2 * r2);
                acc += x.w * law64(law, law.Ldef / dist);
            }
        }
    }
    if (tid < 240) part[(int64_t)blockIdx.x * 240 + tid] = acc;
}

__global__ void k_err_final(TreeDev t, WeightLaw law, const int *nodeItem0, const int *interior, const double *part,
                            double *err) {
    const int q = interior[blockIdx.x];
    const int tid = threadIdx.x;
    __shared__ double sq[240];
    if (tid < 240) {
        int a = nodeItem0[blockIdx.x], b = nodeItem0[blockIdx.x + 1];
        double dExact = 0.0;
        for (int k = a; k < b; ++k) dExact += part[(int64_t)k * 240 + tid];
        const dbl4 g = t.geom[q];
        double pt[3];
        sphere_point(g, tid, pt);
        double r0 = pt[0] - g.x, r1 = pt[1] - g.y, r2 = pt[2] - g.z;
        double dist = sqrt(r0 * r0 + r1 * r1 + r2 * r2);
        double dApprox = t.ai[q] * law64(law, law.Ldef / dist);
        double d = dExact - dApprox;
        sq[tid] = d * d;
    }
    __syncthreads();
    if (tid < kNerr) {
        double s = 0.0;
        for (int ii = 0; ii < 20; ++ii) s += sq[20 * tid + ii];
        err[(int64_t)kNerr * q + tid] = sqrt(s / 20);
    }
}

// Denominator estimate: warp-cooperative walk with the 5-radius far-field
// rule; every lane follows exactly its own recursion of getWiEstimate.
// stride 0: every node in Morton order, out[common index]; stride > 0: the
// common-order nodes 0, stride, 2 stride, ... (nOut of them), out[k].
//
// The far-field test dist * oradius > 5 is first taken in FP32 from the split
// centroid of the node records (rf): the volume point split in two floats, r
// - C formed from the splits, |r - C|^2 + 1e-16 and its square root; it
// stands when it is further than 4e-6 (relative) from 5, which bounds its
// FP32 rounding (a few 1e-7) once |r - C|^2 >= 1e-12 (the splits' own
// representation error, ~1e-13 absolute, is then below 1e-7 relative).
// Otherwise, and for every approximated cluster's term, the test and the
// distance are FP64, so decisions and terms are the FP64 walk's.
__global__ void k_den0(TreeDev t, const NodeRecF *rf, const dbl4 *ptXA, VolumeDev v, WeightLaw law, SymPlanes sym,
                       int64_t stride, int64_t nOut, double *out) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = gid < nOut;
    const int vi = !valid ? 0 : (stride > 0 ? int(gid * stride) : v.perm[gid]);
    double x0[3] = {v.xv0[3 * vi], v.xv0[3 * vi + 1], v.xv0[3 * vi + 2]};
    double acc = 0.0;
    for (int kk = 0; kk < sym.nLoop; ++kk) {
        double r[3];
        mirror_point(sym, kk, x0, r);
        float rh[3], rl[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            rh[c] = float(r[c]);
            rl[c] = float(r[c] - double(rh[c]));
        }
        int node = 0, skip = 0;
        while (node < t.nNodes) {
            const int4 inf = t.info[node];
            const bool active = valid && node >= skip;
            if (inf.w) {
                if (active) {
                    for (int i = inf.x; i <= inf.y; ++i) {
                        dbl4 x = ptXA[i];
                        double r0 = r[0] - x.x, r1 = r[1] - x.y, r2 = r[2] - x.z;
                        double LoD = law.Ldef / sqrt(r0 * r0 + r1 * r1 + r2 * r2 + 1e-16);
                        acc += x.w * law64(law, LoD);
                    }
                }
                node = inf.z;
            } else {
                bool open = false;
                if (active) {
                    // 0 open, 1 far field, 2 undecided in FP32
                    int dec = 2;
                    const float4 ch = __ldg(&rf[node].cHi), cl = __ldg(&rf[node].cLo);
                    const float f0 = (rh[0] - ch.x) + (rl[0] - cl.x), f1 = (rh[1] - ch.y) + (rl[1] - cl.y),
                                f2 = (rh[2] - ch.z) + (rl[2] - cl.z);
                    const float d2f = fmaf(f0, f0, fmaf(f1, f1, fmaf(f2, f2, 1e-16f)));
                    if (d2f >= 1e-12f) {
                        const float xf = sqrtf(d2f) * ch.w;
                        dec = xf > 5.0f * (1.0f + 4e-6f) ? 1 : (xf < 5.0f * (1.0f - 4e-6f) ? 0 : 2);
                    }
                    if (dec != 0) {
                        const dbl4 g = t.geom[node];
                        double r0 = r[0] - g.x, r1 = r[1] - g.y, r2 = r[2] - g.z;
                        double dist = sqrt(r0 * r0 + r1 * r1 + r2 * r2 + 1e-16);
                        if (dec == 1 || dist * g.w > 5.0) {
                            acc += t.ai[node] * law64(law, law.Ldef / dist);
                            skip = inf.z;
                        } else {
                            open = true;
                        }
                    } else {
                        open = true;
                    }
                }
                node = __any_sync(kFull, open) ? node + 1 : inf.z;
            }
        }
    }
    if (valid) out[stride > 0 ? gid : int64_t(vi)] = acc;
}

// Load-balancing cost of every volume node: per mirror, leaves cost their
// point count, every interior visit 0.5 and an accepted approximation 1.1
// more; the sum over mirrors of cost / nPts.  Decisions as dryRun takes them:
// dist with the 1e-16 softening and errTol * den0 as the tolerance.
__global__ void k_dry_run(TreeDev t, VolumeDev v, SymPlanes sym, double errTol, double nPts, double *costs) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = gid < v.nVol;
    const int vi = valid ? v.perm[gid] : 0;
    const double x0[3] = {v.xv0[3 * vi], v.xv0[3 * vi + 1], v.xv0[3 * vi + 2]};
    const double tolDen = errTol * v.den0[vi];
    double acc = 0.0;
    for (int kk = 0; kk < sym.nLoop; ++kk) {
        double r[3];
        mirror_point(sym, kk, x0, r);
        double cst = 0.0;
        int node = 0, skip = 0;
        while (node < t.nNodes) {
            const int4 inf = t.info[node];
            const bool active = valid && node >= skip;
            if (inf.w) {
                if (active) cst += double(inf.y - inf.x + 1);
                node = inf.z;
            } else {
                bool open = false;
                if (active) {
                    const dbl4 g = t.geom[node];
                    const double r0 = r[0] - g.x, r1 = r[1] - g.y, r2 = r[2] - g.z;
                    const double dist = sqrt(r0 * r0 + r1 * r1 + r2 * r2 + 1e-16);
                    cst += 0.5;
                    if (dist * g.w < 2.0) {
                        open = true;
                    } else if (get_error64(t.err + kNerr * node, dist * g.w) < tolDen) {
                        cst += 1.1;
                        skip = inf.z;
                    } else {
                        open = true;
                    }
                }
                node = __any_sync(kFull, open) ? node + 1 : inf.z;
            }
        }
        acc += cst / nPts;
    }
    if (valid) costs[vi] = acc;
}

// Per-block bounding box and count of non-finite values of n points (3
// doubles each), for the Morton codes: out[7 b .. 7 b + 2] minima, [+3 .. +5]
// maxima, [+6] the count.  Minima and maxima are exact, so the box equals a
// sequential scan's.
__global__ void k_bbox(int64_t n, const double *x, double *out) {
    __shared__ double s[7][256];
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY}, bad = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        for (int k = 0; k < 3; ++k) {
            const double v = x[3 * i + k];
            if (!isfinite(v)) {
                bad += 1.0;
            } else {
                lo[k] = fmin(lo[k], v);
                hi[k] = fmax(hi[k], v);
            }
        }
    const int t = threadIdx.x;
    for (int k = 0; k < 3; ++k) {
        s[k][t] = lo[k];
        s[3 + k][t] = hi[k];
    }
    s[6][t] = bad;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (t < w) {
            for (int k = 0; k < 3; ++k) {
                s[k][t] = fmin(s[k][t], s[k][t + w]);
                s[3 + k][t] = fmax(s[3 + k][t], s[3 + k][t + w]);
            }
            s[6][t] += s[6][t + w];
        }
        __syncthreads();
    }
    if (t < 7) out[7 * int64_t(blockIdx.x) + t] = s[t][0];
}

__device__ __forceinline__ unsigned long long spread21(unsigned long long x) {
    x &= 0x1fffffull;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(int64_t n, const double *xv0, double lo0, double lo1, double lo2, double s0, double s1,
                         double s2, unsigned long long *codes, int *idx) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double f[3] = {(xv0[3 * i] - lo0) * s0, (xv0[3 * i + 1] - lo1) * s1, (xv0[3 * i + 2] - lo2) * s2};
    unsigned long long q[3];
    for (int k = 0; k < 3; ++k) {
        double c = fmin(fmax(f[k], 0.0), 2097151.0);
        q[k] = (unsigned long long)c;
    }
    codes[i] = spread21(q[0]) | (spread21(q[1]) << 1) | (spread21(q[2]) << 2);
    idx[i] = int(i);
}

// Reference motion of the mixed walk: Dref = Mbar - I and bref = bbar of the
// root cluster (the mean over all surface points), or zero when the root is a
// leaf.  The walk sums S - Sref(r) in FP32, where Sref(r) = Dref r + bref, and
// adds den * Sref(r) back in double-float: the weighted mean is unchanged,
// while the FP32 rounding scales with how far each term's motion departs from
// the mean motion (a rigid rotation of the whole surface leaves nothing).
__device__ __forceinline__ void ref_motion(const TreeDev &t, const double *nodeMB, double Dr[9], double br[3]) {
    const bool leafRoot = t.info[0].w != 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int k = 0; k < 3; ++k) Dr[3 * a + k] = leafRoot ? 0.0 : nodeMB[3 * a + k] - (a == k ? 1.0 : 0.0);
        br[a] = leafRoot ? 0.0 : nodeMB[9 + a];
    }
}

__device__ __forceinline__ void split_store(double v, float *hi, float *lo) {
    *hi = float(v);
    *lo = float(v - double(float(v)));
}

// Per point: D' = M - I - Dref and u' = S'(Xu0) = (M - I) Xu0 + b - Dref Xu0 - bref,
// FP32 high and low parts.
__global__ void k_mixed_nodal(int n, TreeDev t, const double *nodeMB, const dbl4 *ptXA, const double *ptMB,
                              float *ptDM, float *ptDMl, int pStride) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double Dr[9], br[3];
    ref_motion(t, nodeMB, Dr, br);
    const double *m = ptMB + 12 * i;
    dbl4 x = ptXA[i];
    float *o = ptDM + int64_t(pStride) * i;
    float *ol = ptDMl + int64_t(pStride) * i;
    double X[3] = {x.x, x.y, x.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double Mx = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double d = m[3 * a + k] - (a == k ? 1.0 : 0.0) - Dr[3 * a + k];
            split_store(d, o + 3 * a + k, ol + 3 * a + k);
            Mx += d * X[k];
        }
        split_store(Mx + (m[9 + a] - br[a]), o + 9 + a, ol + 9 + a);
    }
}

// Per node: cluster D' = Mbar - I - Dref and c' = S'(C) = (Mbar - I) C + bbar -
// Dref C - bref as FP32 high and low parts (interior nodes), and for every node
// a bound on |D'| (the largest absolute row sum of the cluster's D', or of the
// members' D' for a leaf) that sizes the FP32 rounding of D' (r - C) in the
// walk's precision gate.  Thread 0 also stores the reference motion (Dref 9,
// bref 3; high parts then low parts) that the walk adds back.
__global__ void k_mixed_nodes(TreeDev t, const double *nodeMB, const double *ptMB, float *nodeDC, float *nodeDCl,
                              float *nodeDn, float *refDB, int nStride, int dnStride) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= t.nNodes) return;
    double Dr[9], br[3];
    ref_motion(t, nodeMB, Dr, br);
    if (q == 0) {
        for (int j = 0; j < 9; ++j) split_store(Dr[j], refDB + j, refDB + 12 + j);
        for (int a = 0; a < 3; ++a) split_store(br[a], refDB + 9 + a, refDB + 21 + a);
    }
    const int4 inf = t.info[q];
    if (inf.w) {
        double dn = 0.0;
        for (int i = inf.x; i <= inf.y; ++i) {
            const double *m = ptMB + 12 * i;
            for (int a = 0; a < 3; ++a) {
                double rs = 0.0;
                for (int k = 0; k < 3; ++k) rs += fabs(m[3 * a + k] - (a == k ? 1.0 : 0.0) - Dr[3 * a + k]);
                dn = fmax(dn, rs);
            }
        }
        nodeDn[int64_t(dnStride) * q] = float(dn);
        return;
    }
    const double *m = nodeMB + 12 * q;
    dbl4 g = t.geom[q];
    double X[3] = {g.x, g.y, g.z};
    float *o = nodeDC + int64_t(nStride) * q;
    float *ol = nodeDCl + int64_t(nStride) * q;
    double dn = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double Mx = 0.0, rowsum = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double d = m[3 * a + k] - (a == k ? 1.0 : 0.0) - Dr[3 * a + k];
            split_store(d, o + 3 * a + k, ol + 3 * a + k);
            Mx += d * X[k];
            rowsum += fabs(d);
        }
        dn = fmax(dn, rowsum);
        split_store(Mx + (m[9 + a] - br[a]), o + 9 + a, ol + 9 + a);
    }
    nodeDn[int64_t(dnStride) * q] = float(dn);
}


inline int blocks(int64_t n, int b) { return int((n + b - 1) / b); }

}  // namespace


int launch_compute_errors(const TreeDev &t, const dbl4 *ptXA, const WeightLaw &law, double *err, cudaStream_t st) {
    // Build the (node, chunk) work list on the host.
    std::vector<int4> info(t.nNodes);
    if (cudaMemcpyAsync(info.data(), t.info, sizeof(int4) * t.nNodes, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return -1;
    std::vector<ErrItem> items;
    std::vector<int> item0, interior;
    for (int q = 0; q < t.nNodes; ++q) {
        if (info[q].w) continue;
        interior.push_back(q);
        item0.push_back(int(items.size()));
        for (int a = info[q].x; a <= info[q].y; a += kErrChunk) items.push_back({q, a, min(a + kErrChunk, info[q].y + 1), 0});
    }
    item0.push_back(int(items.size()));
    if (cudaMemsetAsync(err, 0, sizeof(double) * kNerr * t.nNodes, st) != cudaSuccess) return -1;
    if (interior.empty()) return 0;
    ErrItem *dItems = nullptr;
    int *dItem0 = nullptr, *dInterior = nullptr;
    double *dPart = nullptr;
    // every allocation checked before any copy or launch uses it
    int rc = 0;
    if (cudaMalloc(&dItems, sizeof(ErrItem) * items.size()) != cudaSuccess ||
        cudaMalloc(&dItem0, sizeof(int) * item0.size()) != cudaSuccess ||
        cudaMalloc(&dInterior, sizeof(int) * interior.size()) != cudaSuccess ||
        cudaMalloc(&dPart, sizeof(double) * 240 * items.size()) != cudaSuccess) {
        rc = -2;
    } else if (cudaMemcpyAsync(dItems, items.data(), sizeof(ErrItem) * items.size(), cudaMemcpyHostToDevice, st) !=
                   cudaSuccess ||
               cudaMemcpyAsync(dItem0, item0.data(), sizeof(int) * item0.size(), cudaMemcpyHostToDevice, st) !=
                   cudaSuccess ||
               cudaMemcpyAsync(dInterior, interior.data(), sizeof(int) * interior.size(), cudaMemcpyHostToDevice,
                               st) != cudaSuccess) {
        rc = -1;
    } else {
        k_err_partial<<<int(items.size()), 256, 0, st>>>(t, ptXA, law, dItems, dPart);
        k_err_final<<<int(interior.size()), 256, 0, st>>>(t, law, dItem0, dInterior, dPart, err);
        if (cudaGetLastError() != cudaSuccess) rc = -1;
    }
    // the scratch is freed only once the kernels that read it are done
    if (cudaStreamSynchronize(st) != cudaSuccess) rc = -1;
    if (dItems) cudaFree(dItems);
    if (dItem0) cudaFree(dItem0);
    if (dInterior) cudaFree(dInterior);
    if (dPart) cudaFree(dPart);
    return rc;
}

void launch_denominator0(const TreeDev &t, const NodeRecF *rf, const dbl4 *ptXA, const VolumeDev &v,
                         const WeightLaw &law, const SymPlanes &sym, double *den0, cudaStream_t st) {
    if (v.nVol > 0) k_den0<<<blocks(v.nVol, 128), 128, 0, st>>>(t, rf, ptXA, v, law, sym, 0, v.nVol, den0);
}

int64_t launch_denominator0_strided(const TreeDev &t, const NodeRecF *rf, const dbl4 *ptXA, const VolumeDev &v,
                                    const WeightLaw &law, const SymPlanes &sym, int64_t stride, double *out,
                                    cudaStream_t st) {
    const int64_t n = stride > 0 ? (v.nVol + stride - 1) / stride : 0;
    if (n > 0) k_den0<<<blocks(n, 128), 128, 0, st>>>(t, rf, ptXA, v, law, sym, stride, n, out);
    return n;
}

void launch_dry_run(const TreeDev &t, const VolumeDev &v, const SymPlanes &sym, double errTol, int nPts,
                    double *costs, cudaStream_t st) {
    if (v.nVol > 0 && nPts > 0) k_dry_run<<<blocks(v.nVol, 128), 128, 0, st>>>(t, v, sym, errTol, double(nPts), costs);
}

int volume_bbox(int64_t n, const double *x, double *lo, double *hi, int64_t *nonFinite, cudaStream_t st) {
    const int nb = int(std::min<int64_t>(1024, std::max<int64_t>(1, (n + 255) / 256)));
    double *dOut = nullptr;
    if (cudaMalloc(&dOut, sizeof(double) * 7 * nb) != cudaSuccess) return -1;
    k_bbox<<<nb, 256, 0, st>>>(n, x, dOut);
    std::vector<double> h(7 * size_t(nb));
    cudaError_t e = cudaMemcpyAsync(h.data(), dOut, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dOut);
    if (e != cudaSuccess) return -1;
    double bad = 0.0;
    for (int k = 0; k < 3; ++k) {
        lo[k] = INFINITY;
        hi[k] = -INFINITY;
    }
    for (int b = 0; b < nb; ++b) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::fmin(lo[k], h[7 * b + k]);
            hi[k] = std::fmax(hi[k], h[7 * b + 3 + k]);
        }
        bad += h[7 * b + 6];
    }
    *nonFinite = int64_t(bad);
    return 0;
}

void launch_morton_codes(int64_t nVol, const double *xv0, const double *lo, const double *hi,
                         unsigned long long *codes, int *idx, cudaStream_t st) {
    double s[3];
    for (int k = 0; k < 3; ++k) s[k] = (hi[k] > lo[k]) ? 2097151.0 / (hi[k] - lo[k]) : 0.0;
    if (nVol > 0)
        k_morton<<<blocks(nVol, 256), 256, 0, st>>>(nVol, xv0, lo[0], lo[1], lo[2], s[0], s[1], s[2], codes, idx);
}


void launch_mixed_nodal(int n, const TreeDev &t, const double *nodeMB, const dbl4 *ptXA, const double *ptMB,
                        float *ptDM, float *ptDMl, cudaStream_t st, int pStride) {
    if (n > 0 && t.nNodes > 0)
        k_mixed_nodal<<<blocks(n, 256), 256, 0, st>>>(n, t, nodeMB, ptXA, ptMB, ptDM, ptDMl, pStride);
}

__global__ void k_replay_records(int nNodes, const float *nodeDC, const float *nodeDn, float4 *rr) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nNodes) return;
    float4 *r = rr + 8 * int64_t(q);
    r[0].w = nodeDn[q];
    const float4 *dc = reinterpret_cast<const float4 *>(nodeDC + 12 * int64_t(q));
    // leaves (flag in r[5].x) keep their point range in r[1].w and r[2].x
    if (__float_as_int(r[5].x) != 0) return;
    r[2] = dc[0];
    r[3] = dc[1];
    r[4] = dc[2];
}

void launch_replay_records(int nNodes, const float *nodeDC, const float *nodeDn, float4 *rr, cudaStream_t st) {
    if (nNodes > 0 && rr) k_replay_records<<<blocks(nNodes, 256), 256, 0, st>>>(nNodes, nodeDC, nodeDn, rr);
}

void launch_mixed_nodes(const TreeDev &t, const double *nodeMB, const double *ptMB, float *nodeDC, float *nodeDCl,
                        float *nodeDn, float *refDB, cudaStream_t st, int nStride, int dnStride) {
    if (t.nNodes > 0)
        k_mixed_nodes<<<blocks(t.nNodes, 256), 256, 0, st>>>(t, nodeMB, ptMB, nodeDC, nodeDCl, nodeDn, refDB, nStride,
                                                              dnStride);
}

// Sort volume nodes by Morton code (set-up).  perm[k] = common index of the
// k-th node in Morton order.
int sort_morton(int64_t nVol, unsigned long long *codes, int *idx, unsigned long long *codesAlt, int *perm,
                cudaStream_t st) {
    // cub takes the item count as int
    if (nVol > INT_MAX) return -1;
    size_t tmp = 0;
    if (cub::DeviceRadixSort::SortPairs(nullptr, tmp, codes, codesAlt, idx, perm, int(nVol), 0, 63, st) !=
        cudaSuccess)
        return -1;
    void *dTmp = nullptr;
    if (cudaMalloc(&dTmp, tmp) != cudaSuccess) return -1;
    int rc = 0;
    if (cub::DeviceRadixSort::SortPairs(dTmp, tmp, codes, codesAlt, idx, perm, int(nVol), 0, 63, st) != cudaSuccess)
        rc = -1;
    if (cudaStreamSynchronize(st) != cudaSuccess) rc = -1;
    cudaFree(dTmp);
    return rc;
}

}  // namespace idw
