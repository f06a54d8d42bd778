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

template <class T>
struct TreeBuf {
    T *p = nullptr;
    TreeBuf() = default;
    TreeBuf(const TreeBuf &) = delete;
    TreeBuf &operator=(const TreeBuf &) = delete;
    ~TreeBuf() {
        if (p) cudaFree(p);
    }
    bool alloc(size_t count) {
        return cudaMalloc(reinterpret_cast<void **>(&p), std::max<size_t>(count, 1) * sizeof(T)) == cudaSuccess;
    }
};

inline int grid_of(int64_t n, int b) { return int((n + b - 1) / b); }

// Bounding box of the points (one block): box = (lo x, y, z, hi x, y, z).
__global__ void k_tree_box(const double *pts, int n, double *box) {
    __shared__ double sLo[3][32], sHi[3][32];
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        for (int c = 0; c < 3; ++c) {
            const double x = pts[3 * int64_t(i) + c];
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
                box[c] = lo[c];
                box[3 + c] = hi[c];
            }
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

// Kept node k (preorder): range, escape, leaf flag, depth; pre[radix id] = k.
__global__ void k_tree_nodes(const unsigned long long *key, const int *rid, int nn, int bucket, const int *parent,
                             int4 *info, int *depth, int *pre) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nn) return;
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
__global__ void k_tree_sums(const int4 *info, const int *rid, const int *parent, const int *pre, int nn,
                            const double *tp, double *sum, unsigned *arrived, double *X) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nn) return;
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

// 1/max |x - X| over each node's points, one warp per node.
__global__ void k_tree_radius(const int4 *info, int nn, const double *tp, const double *X, double *oradius) {
    const int64_t w = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nn) return;
    const int4 g = info[w];
    const double cx = X[3 * w], cy = X[3 * w + 1], cz = X[3 * w + 2];
    double r = 0.0;
    for (int i = g.x + lane; i <= g.y; i += 32) {
        const double dx = __dsub_rn(tp[3 * int64_t(i)], cx), dy = __dsub_rn(tp[3 * int64_t(i) + 1], cy),
                     dz = __dsub_rn(tp[3 * int64_t(i) + 2], cz);
        const double d = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
        r = fmax(r, d);
    }
    for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
    if (lane == 0) oradius[w] = 1.0 / r;
}

}  // namespace

int build_morton_tree(const double *pts, int n, int bucket, FlatTree &t, cudaStream_t st) {
    t = FlatTree();
    t.n = n;
    t.bucket = bucket;
    if (n <= 0) return 0;
    if (n > (INT_MAX - 1) / 2) return -1;
    const int nr = 2 * n - 1;  // radix nodes
    TreeBuf<double> dPts, dBox, dTp, dSum, dX, dOr;
    TreeBuf<unsigned long long> dCodes, dCodesS, dKey, dKeyS;
    TreeBuf<int> dIdx, dPerm, dParent, dRid, dRidS, dPre, dDepth;
    TreeBuf<int2> dRange;
    TreeBuf<int4> dInfo;
    TreeBuf<unsigned> dCount, dArrived;
    TreeBuf<char> dTmp;
    if (!dPts.alloc(3 * size_t(n)) || !dBox.alloc(6) || !dTp.alloc(3 * size_t(n)) || !dCodes.alloc(n) ||
        !dCodesS.alloc(n) || !dIdx.alloc(n) || !dPerm.alloc(n) || !dParent.alloc(nr) || !dRange.alloc(n - 1) ||
        !dKey.alloc(nr) || !dKeyS.alloc(nr) || !dRid.alloc(nr) || !dRidS.alloc(nr) || !dPre.alloc(nr) ||
        !dCount.alloc(1))
        return -2;
    // cub scratch: the larger of the two sorts
    size_t tmpA = 0, tmpB = 0;
    if (cub::DeviceRadixSort::SortPairs(nullptr, tmpA, dCodes.p, dCodesS.p, dIdx.p, dPerm.p, n, 0, 63, st) !=
            cudaSuccess ||
        cub::DeviceRadixSort::SortPairs(nullptr, tmpB, dKey.p, dKeyS.p, dRid.p, dRidS.p, nr, 0, 64, st) !=
            cudaSuccess)
        return -1;
    size_t tmp = std::max(tmpA, tmpB);
    if (!dTmp.alloc(tmp)) return -2;
    if (cudaMemcpyAsync(dPts.p, pts, 3 * sizeof(double) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(dParent.p, 0xff, sizeof(int) * nr, st) != cudaSuccess ||
        cudaMemsetAsync(dCount.p, 0, sizeof(unsigned), st) != cudaSuccess)
        return -1;
    k_tree_box<<<1, 1024, 0, st>>>(dPts.p, n, dBox.p);
    k_tree_codes<<<grid_of(n, 256), 256, 0, st>>>(dPts.p, n, dBox.p, dCodes.p, dIdx.p);
    if (cub::DeviceRadixSort::SortPairs(dTmp.p, tmp, dCodes.p, dCodesS.p, dIdx.p, dPerm.p, n, 0, 63, st) !=
        cudaSuccess)
        return -1;
    if (n > 1) k_tree_radix<<<grid_of(n - 1, 256), 256, 0, st>>>(dCodesS.p, n, dRange.p, dParent.p);
    k_tree_keep<<<grid_of(nr, 256), 256, 0, st>>>(dRange.p, dParent.p, n, bucket, dKey.p, dRid.p, dCount.p);
    tmp = std::max(tmpA, tmpB);
    if (cub::DeviceRadixSort::SortPairs(dTmp.p, tmp, dKey.p, dKeyS.p, dRid.p, dRidS.p, nr, 0, 64, st) !=
        cudaSuccess)
        return -1;
    unsigned nnU = 0;
    if (cudaMemcpyAsync(&nnU, dCount.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return -1;
    const int nn = int(nnU);
    if (nn < 1 || nn > nr) return -1;
    if (!dInfo.alloc(nn) || !dDepth.alloc(nn) || !dSum.alloc(3 * size_t(nn)) || !dX.alloc(3 * size_t(nn)) ||
        !dOr.alloc(nn) || !dArrived.alloc(nn))
        return -2;
    if (cudaMemsetAsync(dArrived.p, 0, sizeof(unsigned) * nn, st) != cudaSuccess) return -1;
    k_tree_nodes<<<grid_of(nn, 256), 256, 0, st>>>(dKeyS.p, dRidS.p, nn, bucket, dParent.p, dInfo.p, dDepth.p,
                                                   dPre.p);
    k_tree_gather<<<grid_of(n, 256), 256, 0, st>>>(dPts.p, dPerm.p, n, dTp.p);
    k_tree_sums<<<grid_of(nn, 128), 128, 0, st>>>(dInfo.p, dRidS.p, dParent.p, dPre.p, nn, dTp.p, dSum.p,
                                                  dArrived.p, dX.p);
    k_tree_radius<<<grid_of(32 * int64_t(nn), 256), 256, 0, st>>>(dInfo.p, nn, dTp.p, dX.p, dOr.p);
    if (cudaGetLastError() != cudaSuccess) return -1;
    std::vector<int4> info(nn);
    t.perm.resize(n);
    t.depth.resize(nn);
    t.X.resize(3 * size_t(nn));
    t.oradius.resize(nn);
    if (cudaMemcpyAsync(t.perm.data(), dPerm.p, sizeof(int) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(info.data(), dInfo.p, sizeof(int4) * nn, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(t.depth.data(), dDepth.p, sizeof(int) * nn, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(t.X.data(), dX.p, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(t.oradius.data(), dOr.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return -1;
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
