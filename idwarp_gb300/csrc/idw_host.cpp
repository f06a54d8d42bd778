#include "idw_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include <thread>
#include <map>

namespace idw {

namespace {

struct CellKey {
    int64_t x, y, z;
    bool operator==(const CellKey &o) const { return x == o.x && y == o.y && z == o.z; }
};
struct CellHash {
    size_t operator()(const CellKey &k) const {
        uint64_t h = uint64_t(k.x) * 0x9E3779B97F4A7C15ull;
        h ^= uint64_t(k.y) * 0xC2B2AE3D27D4EB4Full + (h << 6) + (h >> 2);
        h ^= uint64_t(k.z) * 0x165667B19E3779F9ull + (h << 6) + (h >> 2);
        return size_t(h);
    }
};

}  // namespace

int point_reduce(const double *pts, int n, double tol, double *uniquePts, int32_t *link) {
    if (n <= 0) return 0;
    // Spatial hash with cells no smaller than tol, so every partner of a point
    // lies in the 27 cells around it.  Buckets are linked lists of point
    // indices in flat arrays (head per bucket, next per point); a bucket that
    // other cells share only adds candidates, which the distance test rejects
    // (points two cells apart are more than tol apart).
    double lo[3] = {pts[0], pts[1], pts[2]}, hi[3] = {pts[0], pts[1], pts[2]};
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], pts[3 * i + k]);
            hi[k] = std::max(hi[k], pts[3 * i + k]);
        }
    double ext = std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2], 1e-300});
    double h = std::max(tol, ext * std::ldexp(1.0, -40));
    std::vector<int64_t> cell(3 * size_t(n));
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) cell[3 * size_t(i) + k] = int64_t(std::floor((pts[3 * i + k] - lo[k]) / h));
    size_t nb = 1;
    while (nb < 2 * size_t(n)) nb <<= 1;
    const CellHash hash;
    auto bucket = [&](int64_t x, int64_t y, int64_t z) { return hash(CellKey{x, y, z}) & (nb - 1); };
    std::vector<int32_t> head(nb, -1), next(n);
    for (int i = 0; i < n; ++i) {
        const size_t b = bucket(cell[3 * size_t(i)], cell[3 * size_t(i) + 1], cell[3 * size_t(i) + 2]);
        next[i] = head[b];
        head[b] = i;
    }
    const double tol2 = tol * tol;
    std::memset(link, 0, sizeof(int32_t) * n);
    int nUnique = 0;
    for (int i = 0; i < n; ++i) {
        if (link[i] != 0) continue;
        const double *p = pts + 3 * i;
        ++nUnique;
        std::memcpy(uniquePts + 3 * (nUnique - 1), p, 3 * sizeof(double));
        const int64_t *c = cell.data() + 3 * size_t(i);
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz)
                    for (int32_t j = head[bucket(c[0] + dx, c[1] + dy, c[2] + dz)]; j >= 0; j = next[j]) {
                        const double *q = pts + 3 * j;
                        double ax = q[0] - p[0], ay = q[1] - p[1], az = q[2] - p[2];
                        if (ax * ax + ay * ay + az * az <= tol2) link[j] = nUnique;
                    }
    }
    return nUnique;
}

namespace {

// Spread of axis c over ranks [l,u] of perm, sampling ranks l..min(u,l+200)
// pairwise as the reference does (kd_tree.F90:257-298).
double sampled_spread(const double *p, const int32_t *perm, int c, int l, int u) {
    double smin = p[3 * perm[l] + c], smax = smin;
    int last = std::min(u, l + 200);
    int i = l + 2;
    for (; i <= last; i += 2) {
        double a = p[3 * perm[i - 1] + c], b = p[3 * perm[i] + c];
        if (a > b) std::swap(a, b);
        smin = std::min(smin, a);
        smax = std::max(smax, b);
    }
    if (i == last + 1) {
        double z = p[3 * perm[last] + c];
        smin = std::min(smin, z);
        smax = std::max(smax, z);
    }
    return smax - smin;
}

// Partial selection of rank k in [lo, hi] on axis c with the first element of
// the current window as pivot (kd_tree.F90:199-231).
void select_rank(const double *p, int32_t *perm, int c, int k, int lo, int hi) {
    while (lo < hi) {
        const double pivot = p[3 * perm[lo] + c];
        int m = lo;
        for (int i = lo + 1; i <= hi; ++i)
            if (p[3 * perm[i] + c] < pivot) std::swap(perm[++m], perm[i]);
        std::swap(perm[lo], perm[m]);
        if (m <= k) lo = m + 1;
        if (m >= k) hi = m - 1;
    }
}

}  // namespace

namespace {

// Nodes of the subtree over m points: the split index (l+u)/2 gives the left
// child (m-1)/2 + 1 points, so the count depends on m only.
int subtree_nodes(int m, int bucket, std::map<int, int> &memo) {
    if (m - 1 <= bucket) return 1;
    auto it = memo.find(m);
    if (it != memo.end()) return it->second;
    const int left = (m - 1) / 2 + 1;
    const int v = 1 + subtree_nodes(left, bucket, memo) + subtree_nodes(m - left, bucket, memo);
    memo[m] = v;
    return v;
}

struct KdBuild {
    const double *pts;
    int bucket;
    FlatTree &t;
    const std::map<int, int> &nodes;  // subtree node counts, filled before the build
    int count(int m) const { return m - 1 <= bucket ? 1 : nodes.at(m); }

    // Node id over ranks [l, u]; its subtree takes preorder ids
    // [id, id + count(u - l + 1)), left child id + 1, right child after the
    // left subtree.  The two halves of the top `spawn` levels are built on
    // two threads: they touch disjoint ranks and ids.
    void build(int l, int u, int depth, int id, int spawn, int &maxDepth) {
        t.l[id] = l;
        t.u[id] = u;
        t.depth[id] = depth;
        t.escape[id] = id + count(u - l + 1);
        maxDepth = std::max(maxDepth, depth);
        if (u - l <= bucket) {
            t.leaf[id] = 1;
            return;
        }
        t.leaf[id] = 0;
        int best = 0;
        double bsp = -1.0;
        for (int c = 0; c < 3; ++c) {
            double sp = sampled_spread(pts, t.perm.data(), c, l, u);
            if (sp > bsp) {
                best = c;
                bsp = sp;
            }
        }
        const int m = (l + u) / 2;
        select_rank(pts, t.perm.data(), best, m, l, u);
        const int leftId = id + 1, rightId = id + 1 + count(m - l + 1);
        if (spawn > 0) {
            int rightDepth = 0;
            std::thread right([&] { build(m + 1, u, depth + 1, rightId, spawn - 1, rightDepth); });
            build(l, m, depth + 1, leftId, spawn - 1, maxDepth);
            right.join();
            maxDepth = std::max(maxDepth, rightDepth);
        } else {
            build(l, m, depth + 1, leftId, 0, maxDepth);
            build(m + 1, u, depth + 1, rightId, 0, maxDepth);
        }
    }
};

}  // namespace

void build_kdtree(const double *pts, int n, int bucket, FlatTree &t) {
    t = FlatTree();
    t.n = n;
    t.bucket = bucket;
    if (n <= 0) return;
    t.perm.resize(n);
    for (int i = 0; i < n; ++i) t.perm[i] = i;
    std::map<int, int> memo;
    const int nn = subtree_nodes(n, bucket, memo);
    t.l.assign(nn, 0);
    t.u.assign(nn, 0);
    t.depth.assign(nn, 0);
    t.escape.assign(nn, 0);
    t.leaf.assign(nn, 0);
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int spawn = 0;  // 2^spawn threads in the top levels
    while ((2u << spawn) <= std::min(hw, 16u) && spawn < 4) ++spawn;
    KdBuild kb{pts, bucket, t, memo};
    int maxDepth = 1;
    kb.build(0, n - 1, 1, 0, n > 4096 ? spawn : 0, maxDepth);
    t.maxDepth = maxDepth;
    // setCenters: unweighted centroid of the range, 1/max distance (one
    // node's work is independent of every other's)
    t.X.assign(3 * size_t(nn), 0.0);
    t.oradius.assign(nn, 0.0);
    auto centres = [&](int k0, int k1) {
        for (int k = k0; k < k1; ++k) {
            double s[3] = {0, 0, 0};
            for (int i = t.l[k]; i <= t.u[k]; ++i)
                for (int c = 0; c < 3; ++c) s[c] += pts[3 * t.perm[i] + c];
            const int cnt = t.u[k] - t.l[k] + 1;
            for (int c = 0; c < 3; ++c) s[c] = s[c] / cnt;
            double radius = 0;
            for (int i = t.l[k]; i <= t.u[k]; ++i) {
                double dx = pts[3 * t.perm[i]] - s[0], dy = pts[3 * t.perm[i] + 1] - s[1],
                       dz = pts[3 * t.perm[i] + 2] - s[2];
                radius = std::max(radius, std::sqrt(dx * dx + dy * dy + dz * dz));
            }
            for (int c = 0; c < 3; ++c) t.X[3 * k + c] = s[c];
            t.oradius[k] = 1.0 / radius;
        }
    };
    const int nt = (n > 4096) ? int(std::min(hw, 16u)) : 1;
    std::vector<std::thread> pool;
    for (int q = 1; q < nt; ++q) pool.emplace_back(centres, int(int64_t(nn) * q / nt), int(int64_t(nn) * (q + 1) / nt));
    centres(0, int(int64_t(nn) / nt));
    for (auto &th : pool) th.join();
}

}  // namespace idw
