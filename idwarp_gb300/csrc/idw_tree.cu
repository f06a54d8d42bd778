// Device-built surface tree (option treeBuild IDW_TREE_MORTON).
//
// The reference builds a kd tree on the host (build_tree,
// src/modules/kd_tree.F90:123-300: median split on the axis of largest
// spread).  This build replaces it when asked, on the GPU:
//   1. the unique surface points get 63-bit Morton codes, 21 bits per axis
//      over their bounding cube (x in the highest bit of each triple);
//   2. a stable radix sort orders them by code (ties keep the point order);
//   3. one thread per interior node builds the binary radix tree of the
//      sorted keys (code, point index) as published by T. Karras,
//      "Maximizing parallelism in the construction of BVHs, octrees, and k-d
//      trees", HPG 2012: the node's direction and range from the common-prefix
//      lengths with its neighbours, its split by binary search;
//   4. the tree is cut where a node holds at most bucketSize+1 points (the kd
//      tree's leaf rule u - l <= bucketSize); the nodes kept are numbered in
//      preorder by sorting their point ranges on (first ascending, last
//      descending), and a node's escape index is the first kept range that
//      starts after its own (one binary search);
//   5. aggregates as setCenters (kd_tree.F90:558-593): unweighted centroid and
//      1/max distance.  The centroid sums are formed bottom-up (a leaf's
//      points in order, an interior node's as left + right), so they are
//      deterministic; the radius is a maximum, whatever the order.
// The result has the layout of the host kd build (preorder, point ranges,
// escape indices, leaf flags, depth, centroid, 1/radius), so the rest of the
// set-up and every walk take it unchanged.  Its clusters differ from the kd
// tree's, so fast-mode results differ within what errTol allows; exact mode
// is the same sum in another order.
#include <cub/cub.cuh>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "idw_host.hpp"
#include "idw_kernels.h"

namespace idw {

namespace {

constexpr int kMortonBits = 21;
constexpr double kMortonCells = 2097152.0;  // 2^21
constexpr unsigned kMortonMax = 2097151u;
constexpr int kMaxTreeDepth = 128;

inline int grid_of(int64_t n, int b) { return int((n + b - 1) / b); }

constexpr int kBoxBlocks = 64;  // partial bounding boxes
constexpr int kRadChunk = 256;  // points per warp task of the radius pass

// Partial bounding boxes: block b writes (lo x, y, z, hi x, y, z) of its
// grid-stride share of the points to part[6 b ...].
__global__ void k_tree_box(const double *pts, int n, double *part) {
    __shared__ double sLo[3][32], sHi[3][32];
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        for (int c = 0; c < 3; ++c) {
            const double x = pts[3 * i + c];
            lo[c] = fmin(lo[c], x);
            hi[c] = fmax(hi[c], x);
        }
    for (int c = 0; c < 3; ++c)
        for (int o = 16; o > 0; o >>= 1) {
            lo[c] = fmin(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
            hi[c] = fmax(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
        }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (lane == 0)
        for (int c = 0; c < 3; ++c) {
            sLo[c][w] = lo[c];
            sHi[c][w] = hi[c];
        }
    __syncthreads();
    if (w == 0) {
        for (int c = 0; c < 3; ++c) {
            lo[c] = lane < nw ? sLo[c][lane] : INFINITY;
            hi[c] = lane < nw ? sHi[c][lane] : -INFINITY;
            for (int o = 16; o > 0; o >>= 1) {
                lo[c] = fmin(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
                hi[c] = fmax(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
            }
        }
        if (lane == 0)
            for (int c = 0; c < 3; ++c) {
                part[6 * blockIdx.x + c] = lo[c];
                part[6 * blockIdx.x + 3 + c] = hi[c];
            }
    }
}

// The box of the partial boxes (one warp; minimum and maximum are exact in
// any order).
__global__ void k_tree_box_final(const double *part, int nPart, double *box) {
    const int lane = threadIdx.x;
    for (int c = 0; c < 6; ++c) {
        const bool isLo = c < 3;
        double v = isLo ? INFINITY : -INFINITY;
        for (int b = lane; b < nPart; b += 32) v = isLo ? fmin(v, part[6 * b + c]) : fmax(v, part[6 * b + c]);
        for (int o = 16; o > 0; o >>= 1) {
            const double w = __shfl_xor_sync(0xffffffffu, v, o);
            v = isLo ? fmin(v, w) : fmax(v, w);
        }
        if (lane == 0) box[c] = v;
    }
}

// Morton code of every point: cell index floor((x - lo) * 2^21 / extent) on
// each axis (extent = the box's largest side, clamped to 2^21 - 1), bits
// interleaved x, y, z from the most significant end.  Products and
// differences are single IEEE roundings (no contraction), as in the oracle.
__global__ void k_tree_codes(const double *pts, int n, const double *box, unsigned long long *codes, int *idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ext = fmax(fmax(__dsub_rn(box[3], box[0]), __dsub_rn(box[4], box[1])), __dsub_rn(box[5], box[2]));
    const double inv = ext > 0.0 ? kMortonCells / ext : 0.0;
    unsigned q[3];
    for (int c = 0; c < 3; ++c) {
        const double f = floor(__dmul_rn(__dsub_rn(pts[3 * int64_t(i) + c], box[c]), inv));
        q[c] = f >= double(kMortonMax) ? kMortonMax : unsigned(f);
    }
    unsigned long long code = 0;
    for (int b = 0; b < kMortonBits; ++b)
        for (int c = 0; c < 3; ++c) code |= (unsigned long long)((q[c] >> b) & 1u) << (3 * b + 2 - c);
    codes[i] = code;
    idx[i] = i;
}

// Length of the common prefix of the keys (code, index) at sorted positions
// i and j; -1 outside [0, n).  Codes use 63 bits, so equal codes give 64 +
// the common prefix of the 32-bit indexes.
__device__ __forceinline__ int key_prefix(const unsigned long long *k, int n, int i, long long j) {
    if (j < 0 || j >= n) return -1;
    const unsigned long long a = k[i], b = k[j];
    return a != b ? __clzll(a ^ b) : 64 + __clz(i ^ int(j));
}

// Interior node i of the radix tree over n sorted keys (Karras 2012,
// section 4): its point range and its two children.  Radix ids: interior i
// -> i, leaf (point) j -> n - 1 + j; the root is interior 0.
__global__ void k_tree_radix(const unsigned long long *k, int n, int2 *range, int *parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = key_prefix(k, n, i, i + 1) > key_prefix(k, n, i, i - 1) ? 1 : -1;
    const int dmin = key_prefix(k, n, i, i - d);
    long long lmax = 2;
    while (key_prefix(k, n, i, i + lmax * d) > dmin) lmax *= 2;
    long long len = 0;
    for (long long t = lmax / 2; t >= 1; t /= 2)
        if (key_prefix(k, n, i, i + (len + t) * d) > dmin) len += t;
    const long long j = i + len * d;
    const int dnode = key_prefix(k, n, i, j);
    long long s = 0;
    for (long long div = 2;; div *= 2) {
        const long long t = (len + div - 1) / div;
        if (key_prefix(k, n, i, i + (s + t) * d) > dnode) s += t;
        if (t <= 1) break;
    }
    const int gamma = int(i + s * d + (d < 0 ? -1 : 0));
    const int lo = int(min((long long)i, j)), hi = int(max((long long)i, j));
    const int left = lo == gamma ? n - 1 + gamma : gamma;
    const int right = hi == gamma + 1 ? n - 1 + gamma + 1 : gamma + 1;
    range[i] = make_int2(lo, hi);
    parent[left] = i;
    parent[right] = i;
}

__device__ __forceinline__ int2 radix_range(const int2 *range, int n, int r) {
    return r < n - 1 ? range[r] : make_int2(r - (n - 1), r - (n - 1));
}

// A radix node is kept when it is the root or its parent holds more than
// bucket+1 points; its sort key orders the kept nodes in preorder.
__global__ void k_tree_keep(const int2 *range, const int *parent, int n, int bucket, unsigned long long *key,
                            int *rid, unsigned *count) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= 2 * n - 1) return;
    const int2 g = radix_range(range, n, r);
    const int p = parent[r];
    bool keep = p < 0;
    if (!keep) {
        const int2 pg = range[p];
        keep = pg.y - pg.x > bucket;
    }
    key[r] = keep ? ((unsigned long long)unsigned(g.x) << 32) | (unsigned long long)(0xffffffffu - unsigned(g.y))
                  : ~0ull;
    rid[r] = r;
    if (keep) atomicAdd(count, 1u);
}

// Kept node k (preorder): range, escape, leaf flag, depth; pre[radix id] = k;
// chunks[k] = radius-pass tasks of the node (0 past the nn kept nodes).
__global__ void k_tree_nodes(const unsigned long long *key, const int *rid, const unsigned *count, int nr,
                             int bucket, const int *parent, int4 *info, int *depth, int *pre, int *chunks) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nr) return;
    const int nn = int(*count);
    if (k >= nn) {
        chunks[k] = 0;
        return;
    }
    const unsigned long long kk = key[k];
    const int l = int(kk >> 32), u = int(0xffffffffu - unsigned(kk & 0xffffffffull));
    const unsigned long long target = (unsigned long long)unsigned(u + 1) << 32;
    int a = k + 1, b = nn;  // first key >= target in [k+1, nn)
    while (a < b) {
        const int m = (a + b) >> 1;
        if (key[m] < target) a = m + 1;
        else b = m;
    }
    info[k] = make_int4(l, u, a, u - l <= bucket ? 1 : 0);
    int dep = 1;  // a radix tree over 95-bit keys is at most 96 levels deep
    for (int p = parent[rid[k]]; p >= 0 && dep < kMaxTreeDepth; p = parent[p]) ++dep;
    depth[k] = dep;
    pre[rid[k]] = k;
    chunks[k] = (u - l + kRadChunk) / kRadChunk;
}

// Tree-order points: tp[i] = pts[perm[i]].
__global__ void k_tree_gather(const double *pts, const int *perm, int n, double *tp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = perm[i];
    for (int c = 0; c < 3; ++c) tp[3 * int64_t(i) + c] = pts[3 * int64_t(s) + c];
}

// Centroid sums bottom-up: each leaf sums its points in order, then climbs;
// at each interior node the second child to arrive forms left + right (always
// in that order) and goes on.  X = sum / count.
__global__ void k_tree_sums(const int4 *info, const int *rid, const int *parent, const int *pre,
                            const unsigned *count, int nr, const double *tp, double *sum, unsigned *arrived,
                            double *X) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nr || k >= int(*count)) return;
    const int4 g = info[k];
    if (!g.w) return;
    double s[3] = {0.0, 0.0, 0.0};
    for (int i = g.x; i <= g.y; ++i)
        for (int c = 0; c < 3; ++c) s[c] = __dadd_rn(s[c], tp[3 * int64_t(i) + c]);
    int cur = k;
    for (int level = 0; level < kMaxTreeDepth; ++level) {
        const int4 gc = info[cur];
        const double cnt = double(gc.y - gc.x + 1);
        for (int c = 0; c < 3; ++c) {
            sum[3 * int64_t(cur) + c] = s[c];
            X[3 * int64_t(cur) + c] = s[c] / cnt;
        }
        const int pr = parent[rid[cur]];
        if (pr < 0) return;
        const int p = pre[pr];
        __threadfence();
        if (atomicAdd(&arrived[p], 1u) == 0u) return;  // the sibling finishes this node
        __threadfence();
        const int left = p + 1, right = info[left].z;
        for (int c = 0; c < 3; ++c)
            s[c] = __dadd_rn(__ldcg(&sum[3 * int64_t(left) + c]), __ldcg(&sum[3 * int64_t(right) + c]));
        cur = p;
    }
}

// Largest |x - X| over each node's points: one warp per task of up to
// kRadChunk points of one node (tasks numbered through the inclusive sums of
// the chunk counts), folded into the node's maximum with an integer atomic
// on the bits (non-negative doubles order as their bit patterns).
__global__ void k_tree_radius(const int4 *info, const unsigned *count, const int *incl, int nr, const double *tp,
                              const double *X, unsigned long long *radBits) {
    const int nn = int(*count);
    const int total = incl[nr - 1];
    const int lane = threadIdx.x & 31;
    const int nw = int((int64_t(gridDim.x) * blockDim.x) >> 5);
    for (int c = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5); c < total; c += nw) {
        int a = 0, b = nn - 1;  // first node k with incl[k] > c
        while (a < b) {
            const int m = (a + b) >> 1;
            if (incl[m] > c) b = m;
            else a = m + 1;
        }
        const int4 g = info[a];
        const int first = incl[a] - (g.y - g.x + kRadChunk) / kRadChunk;
        const int i0 = g.x + (c - first) * kRadChunk, i1 = min(g.y, i0 + kRadChunk - 1);
        const double cx = X[3 * int64_t(a)], cy = X[3 * int64_t(a) + 1], cz = X[3 * int64_t(a) + 2];
        double r = 0.0;
        for (int i = i0 + lane; i <= i1; i += 32) {
            const double dx = __dsub_rn(tp[3 * int64_t(i)], cx), dy = __dsub_rn(tp[3 * int64_t(i) + 1], cy),
                         dz = __dsub_rn(tp[3 * int64_t(i) + 2], cz);
            r = fmax(r, __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz))));
        }
        for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
        if (lane == 0) atomicMax(&radBits[a], (unsigned long long)__double_as_longlong(r));
    }
}

__global__ void k_tree_oradius(const unsigned long long *radBits, const unsigned *count, int nr, double *oradius) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nr || k >= int(*count)) return;
    oradius[k] = 1.0 / __longlong_as_double((long long)radBits[k]);
}

// Sub-buffers of one device allocation, each 256-byte aligned.
struct Arena {
    size_t off = 0;
    template <class T>
    size_t take(size_t count) {
        const size_t at = off;
        off += (std::max<size_t>(count, 1) * sizeof(T) + 255) & ~size_t(255);
        return at;
    }
};

}  // namespace

int build_morton_tree(const double *pts, int n, int bucket, FlatTree &t, cudaStream_t st) {
    t = FlatTree();
    t.n = n;
    t.bucket = bucket;
    if (n <= 0) return 0;
    if (n > (INT_MAX - 1) / 2) return -3;  // radix node ids are int
    const int nr = 2 * n - 1;  // radix nodes; at most nr are kept
    // cub scratch: the larger of the two sorts and the scan
    size_t tmpA = 0, tmpB = 0, tmpC = 0;
    if (cub::DeviceRadixSort::SortPairs(nullptr, tmpA, (unsigned long long *)nullptr, (unsigned long long *)nullptr,
                                        (int *)nullptr, (int *)nullptr, n, 0, 63, st) != cudaSuccess ||
        cub::DeviceRadixSort::SortPairs(nullptr, tmpB, (unsigned long long *)nullptr, (unsigned long long *)nullptr,
                                        (int *)nullptr, (int *)nullptr, nr, 0, 64, st) != cudaSuccess ||
        cub::DeviceScan::InclusiveSum(nullptr, tmpC, (int *)nullptr, (int *)nullptr, nr, st) != cudaSuccess)
        return -1;
    const size_t tmp = std::max(std::max(tmpA, tmpB), tmpC);
    Arena ar;
    const size_t oPts = ar.take<double>(3 * size_t(n)), oPart = ar.take<double>(6 * kBoxBlocks),
                 oBox = ar.take<double>(6), oTp = ar.take<double>(3 * size_t(n)),
                 oCodes = ar.take<unsigned long long>(n), oCodesS = ar.take<unsigned long long>(n),
                 oIdx = ar.take<int>(n), oPerm = ar.take<int>(n), oParent = ar.take<int>(nr),
                 oRange = ar.take<int2>(n - 1), oKey = ar.take<unsigned long long>(nr),
                 oKeyS = ar.take<unsigned long long>(nr), oRid = ar.take<int>(nr), oRidS = ar.take<int>(nr),
                 oPre = ar.take<int>(nr), oCount = ar.take<unsigned>(1), oInfo = ar.take<int4>(nr),
                 oDepth = ar.take<int>(nr), oSum = ar.take<double>(3 * size_t(nr)), oX = ar.take<double>(3 * size_t(nr)),
                 oOr = ar.take<double>(nr), oRad = ar.take<unsigned long long>(nr), oArr = ar.take<unsigned>(nr),
                 oChunks = ar.take<int>(nr), oIncl = ar.take<int>(nr), oTmp = ar.take<char>(tmp);
    char *base = nullptr;
    if (cudaMalloc(&base, ar.off) != cudaSuccess) return -2;
    auto at = [&](size_t o) { return static_cast<void *>(base + o); };
    double *dPts = (double *)at(oPts), *dPart = (double *)at(oPart), *dBox = (double *)at(oBox),
           *dTp = (double *)at(oTp), *dSum = (double *)at(oSum), *dX = (double *)at(oX), *dOr = (double *)at(oOr);
    unsigned long long *dCodes = (unsigned long long *)at(oCodes), *dCodesS = (unsigned long long *)at(oCodesS),
                       *dKey = (unsigned long long *)at(oKey), *dKeyS = (unsigned long long *)at(oKeyS),
                       *dRad = (unsigned long long *)at(oRad);
    int *dIdx = (int *)at(oIdx), *dPerm = (int *)at(oPerm), *dParent = (int *)at(oParent), *dRid = (int *)at(oRid),
        *dRidS = (int *)at(oRidS), *dPre = (int *)at(oPre), *dDepth = (int *)at(oDepth), *dChunks = (int *)at(oChunks),
        *dIncl = (int *)at(oIncl);
    int2 *dRange = (int2 *)at(oRange);
    int4 *dInfo = (int4 *)at(oInfo);
    unsigned *dCount = (unsigned *)at(oCount), *dArr = (unsigned *)at(oArr);
    void *dTmp = at(oTmp);
    int sms = 0, dev = 0;
    int rc = 0;
    size_t tb = tmp;
    const int boxBlocks = std::min(kBoxBlocks, grid_of(n, 1024));
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaMemcpyAsync(dPts, pts, 3 * sizeof(double) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(dParent, 0xff, sizeof(int) * nr, st) != cudaSuccess ||
        cudaMemsetAsync(dCount, 0, sizeof(unsigned), st) != cudaSuccess ||
        cudaMemsetAsync(dArr, 0, sizeof(unsigned) * nr, st) != cudaSuccess ||
        cudaMemsetAsync(dRad, 0, sizeof(unsigned long long) * nr, st) != cudaSuccess) {
        rc = -1;
    } else {
        k_tree_box<<<boxBlocks, 1024, 0, st>>>(dPts, n, dPart);
        k_tree_box_final<<<1, 32, 0, st>>>(dPart, boxBlocks, dBox);
        k_tree_codes<<<grid_of(n, 256), 256, 0, st>>>(dPts, n, dBox, dCodes, dIdx);
        if (cub::DeviceRadixSort::SortPairs(dTmp, tb, dCodes, dCodesS, dIdx, dPerm, n, 0, 63, st) != cudaSuccess)
            rc = -1;
    }
    if (rc == 0) {
        if (n > 1) k_tree_radix<<<grid_of(n - 1, 256), 256, 0, st>>>(dCodesS, n, dRange, dParent);
        k_tree_keep<<<grid_of(nr, 256), 256, 0, st>>>(dRange, dParent, n, bucket, dKey, dRid, dCount);
        tb = tmp;
        if (cub::DeviceRadixSort::SortPairs(dTmp, tb, dKey, dKeyS, dRid, dRidS, nr, 0, 64, st) != cudaSuccess)
            rc = -1;
    }
    if (rc == 0) {
        k_tree_nodes<<<grid_of(nr, 256), 256, 0, st>>>(dKeyS, dRidS, dCount, nr, bucket, dParent, dInfo, dDepth, dPre,
                                                       dChunks);
        k_tree_gather<<<grid_of(n, 256), 256, 0, st>>>(dPts, dPerm, n, dTp);
        k_tree_sums<<<grid_of(nr, 128), 128, 0, st>>>(dInfo, dRidS, dParent, dPre, dCount, nr, dTp, dSum, dArr, dX);
        tb = tmp;
        if (cub::DeviceScan::InclusiveSum(dTmp, tb, dChunks, dIncl, nr, st) != cudaSuccess) rc = -1;
    }
    if (rc == 0) {
        k_tree_radius<<<8 * std::max(sms, 1), 256, 0, st>>>(dInfo, dCount, dIncl, nr, dTp, dX, dRad);
        k_tree_oradius<<<grid_of(nr, 256), 256, 0, st>>>(dRad, dCount, nr, dOr);
        if (cudaGetLastError() != cudaSuccess) rc = -1;
    }
    unsigned nnU = 0;
    if (rc == 0 && (cudaMemcpyAsync(&nnU, dCount, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                    cudaStreamSynchronize(st) != cudaSuccess || nnU < 1 || nnU > unsigned(nr)))
        rc = -1;
    const int nn = int(nnU);
    std::vector<int4> info;
    if (rc == 0) {
        info.resize(nn);
        t.perm.resize(n);
        t.depth.resize(nn);
        t.X.resize(3 * size_t(nn));
        t.oradius.resize(nn);
        if (cudaMemcpyAsync(t.perm.data(), dPerm, sizeof(int) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(info.data(), dInfo, sizeof(int4) * nn, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(t.depth.data(), dDepth, sizeof(int) * nn, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(t.X.data(), dX, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(t.oradius.data(), dOr, sizeof(double) * nn, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            rc = -1;
    }
    cudaFree(base);
    if (rc != 0) return rc;
    t.l.resize(nn);
    t.u.resize(nn);
    t.escape.resize(nn);
    t.leaf.resize(nn);
    t.maxDepth = 1;
    for (int k = 0; k < nn; ++k) {
        t.l[k] = info[k].x;
        t.u[k] = info[k].y;
        t.escape[k] = info[k].z;
        t.leaf[k] = info[k].w;
        t.maxDepth = std::max(t.maxDepth, t.depth[k]);
    }
    return 0;
}

}  // namespace idw
