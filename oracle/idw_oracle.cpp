// ============================================================================
// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement, in FP64 (and std::complex<double> for complex-step
// derivatives), of IDWarp's inverse-distance-weighted volume-mesh warping path
// (mdolab/idwarp v2.6.2).  It exists to CHECK the GPU library: only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.  The
// product (idwarp_gb300/) never links, imports or calls anything here.
//
// Every routine below restates one routine of the reference, cited by
// file:line.  The reference itself is Fortran 90 + PETSc/MPI and cannot be
// compiled in this container (no Fortran compiler, no PETSc/MPI), so parity of
// this restatement with the reference is pinned by the reference's own
// derivative identities (dot-product, central FD, complex step) and analytic
// invariants, not by running the reference.  The reference's regression sums
// (tests/ref/*.ref) need CGNS meshes that are downloaded at test time and are
// not available here.
//
// Conventions: all index arrays are 0-based here (the reference is 1-based);
// xyz are interleaved (N,3) C-order == Fortran (3,N).  Mi is stored row-major,
// Mi[3*a+b] == Fortran Mi(a+1,b+1).
// ============================================================================
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

typedef std::complex<double> cplx;

static inline double re(double x) { return x; }
static inline double re(const cplx &x) { return x.real(); }

// src/modules/constants.F90:31-33 (compiled with -fdefault-real-8, so the
// literals are double precision).
static const double kPi = 3.1415926535897931;
static const double kPhi = 2.1180339887498949;
static const double kEps = 1e-15;
// src/modules/kd_tree.F90:34-35
static const double kRstar[12] = {2.0, 3.0, 4.0, 5.0, 7.5, 10.0, 20.0, 40.0, 80.0, 160.0, 320.0, 640.0};
static const int kNerr = 12;

struct Opts {
    double aExp, bExp, LdefFact, alpha, errTol, cornerAngle;
    int evalMode;  // 0 exact, 1 fast (src/modules/gridInput.f90:16-17)
    int useRotations, zeroCornerRotations, bucketSize;
    int treeBuild;  // 0: the reference's kd tree; 1: the library's Morton tree (no reference counterpart)
};

// src/modules/kd_tree.F90:63-79 (tree_node)
struct Node {
    int dnum;      // 0 = leaf, otherwise the split axis 1..3
    int l, u, n;   // 0-based inclusive range into tree order
    int left, right;
    double X[3];
    double oradius;
    double Ai;
    double err[kNerr];
    int lvl;
};

struct Tree {
    int n = 0;
    std::vector<int> indexes;   // tree order -> unique (lexsorted) index
    std::vector<Node> nodes;
    int root = -1;
    int maxDepth = 1;
    std::vector<double> theData;  // unique points (3,n) in input order
    std::vector<double> Xu0;      // (3,n) tree order
    std::vector<double> Ai, normals0;
    std::vector<char> isCorner;
    std::vector<int> XuInd;       // tree index -> first caller point index
    std::vector<int> facePtr;     // nFace+1
    std::vector<int> faceConn;    // tree-order indices
    std::vector<int> n2ePtr, n2e; // node -> faces, in the reference's order
    double Ldef0 = 0, Ldef = 0, alphaToBexp = 0, aExp = 3, bExp = 5, errTol = 0;
    double orstar[kNerr - 1];
};

struct Stats {
    long long leafPairs = 0, approx = 0, visited = 0;
};

struct Ctx {
    Opts o;
    Tree tp;
    int nSym = 0, nLoop = 1;
    std::vector<double> symPts, symNormals;
    long long nVol = 0;
    std::vector<double> Xv0, Xv, den0, numer, denom;
    int nPts = 0;
    std::vector<double> Xs;  // current surface (3,nPts), caller order
    bool haveTree = false, haveDenom = false;
    Stats st;
};

// ---------------------------------------------------------------------------
// pointReduce: src/utils/pointReduce.F90:1-83.  Points within tol (squared
// distance <= tol^2, kdtree2_r_nearest semantics, src/modules/kd_tree2.f90:1537)
// of the first not-yet-linked point i form a new unique point whose
// coordinates are pts(:,i); every point found is (re)linked to it.
// link is 1-based as in the reference.
// ---------------------------------------------------------------------------
static int point_reduce(const double *pts, int N, double tol, double *uniquePts, int *link) {
    if (N == 0) return 0;
    std::vector<int> order(N);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        if (pts[3 * a] != pts[3 * b]) return pts[3 * a] < pts[3 * b];
        return a < b;
    });
    std::vector<double> xs(N);
    for (int k = 0; k < N; ++k) xs[k] = pts[3 * order[k]];
    const double tol2 = tol * tol;
    for (int i = 0; i < N; ++i) link[i] = 0;
    int nUnique = 0;
    for (int i = 0; i < N; ++i) {
        if (link[i] != 0) continue;
        const double *p = pts + 3 * i;
        ++nUnique;
        uniquePts[3 * (nUnique - 1) + 0] = p[0];
        uniquePts[3 * (nUnique - 1) + 1] = p[1];
        uniquePts[3 * (nUnique - 1) + 2] = p[2];
        // candidates with |x - p.x| <= tol
        int lo = int(std::lower_bound(xs.begin(), xs.end(), p[0] - tol) - xs.begin());
        for (int k = lo; k < N && xs[k] <= p[0] + tol; ++k) {
            const double *q = pts + 3 * order[k];
            double dx = q[0] - p[0], dy = q[1] - p[1], dz = q[2] - p[2];
            double sd = dx * dx + dy * dy + dz * dz;
            if (sd <= tol2) link[order[k]] = nUnique;
        }
    }
    return nUnique;
}

// ---------------------------------------------------------------------------
// build_tree & helpers: src/modules/kd_tree.F90:123-300.
// ---------------------------------------------------------------------------
static double spread_in_coordinate(const Tree &tp, int c, int l, int u) {
    // kd_tree.F90:257-298.  0-based l,u; the pair loop starts at l+1.
    const double *v = tp.theData.data();
    const int *ind = tp.indexes.data();
    double smin = v[3 * ind[l] + c], smax = smin;
    int ulocal = std::min(u, l + 200);
    int i;
    for (i = l + 2; i <= ulocal; i += 2) {
        double lmin = v[3 * ind[i - 1] + c], lmax = v[3 * ind[i] + c];
        if (lmin > lmax) std::swap(lmin, lmax);
        if (smin > lmin) smin = lmin;
        if (smax < lmax) smax = lmax;
    }
    if (i == ulocal + 1) {
        double last = v[3 * ind[ulocal] + c];
        if (smin > last) smin = last;
        if (smax < last) smax = last;
    }
    return smax - smin;
}

static int most_spread_coordinate(const Tree &tp, int l, int u) {
    // kd_tree.F90:233-255; returns 1-based axis
    int res = 0;
    double bsp = -1.0;
    for (int i = 1; i <= 3; ++i) {
        double sp = spread_in_coordinate(tp, i - 1, l, u);
        if (sp > bsp) {
            res = i;
            bsp = sp;
        }
    }
    return res;
}

static void select_on_coordinate(const double *v, int *ind, int c, int k, int li, int ui) {
    // kd_tree.F90:199-231 (c 0-based axis, indices 0-based)
    int l = li, u = ui;
    while (l < u) {
        int t = ind[l];
        int m = l;
        for (int i = l + 1; i <= u; ++i) {
            if (v[3 * ind[i] + c] < v[3 * t + c]) {
                ++m;
                std::swap(ind[m], ind[i]);
            }
        }
        std::swap(ind[l], ind[m]);
        if (m <= k) l = m + 1;
        if (m >= k) u = m - 1;
    }
}

static int build_range(Tree &tp, int l, int u, int bucket) {
    // kd_tree.F90:138-183
    int id = int(tp.nodes.size());
    tp.nodes.push_back(Node());
    Node nd;
    std::memset(&nd, 0, sizeof(nd));
    nd.l = l;
    nd.u = u;
    nd.n = u - l + 1;
    nd.left = nd.right = -1;
    if ((u - l) <= bucket) {
        nd.dnum = 0;
        tp.nodes[id] = nd;
    } else {
        int c = most_spread_coordinate(tp, l, u);
        int m = (l + u) / 2;
        select_on_coordinate(tp.theData.data(), tp.indexes.data(), c - 1, m, l, u);
        nd.dnum = c;
        tp.nodes[id] = nd;
        int left = build_range(tp, l, m, bucket);
        int right = build_range(tp, m + 1, u, bucket);
        tp.nodes[id].left = left;
        tp.nodes[id].right = right;
    }
    return id;
}

// ---------------------------------------------------------------------------
// Morton tree: the library's treeBuild "morton" option, which has no
// counterpart in the reference.  Restated here from its definition, top-down,
// to check the device build (which forms the same tree bottom-up in parallel):
// points ordered by 63-bit Morton code (21 bits per axis over the bounding
// cube, x in the highest bit of each triple; ties keep the point order); the
// binary radix tree of the keys (code, index), whose node over [l, u] splits
// after the last key sharing more than the common prefix of keys l and u;
// leaves where u - l <= bucketSize; centroid sums bottom-up (a leaf's points
// in order, an interior node's as left + right); radius as setCenters.
// ---------------------------------------------------------------------------
static void morton_order(const double *pts, int n, std::vector<unsigned long long> &codes, std::vector<int> &order) {
    double lo[3], hi[3];
    for (int c = 0; c < 3; ++c) lo[c] = hi[c] = pts[c];
    for (int i = 1; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            lo[c] = std::min(lo[c], pts[3 * i + c]);
            hi[c] = std::max(hi[c], pts[3 * i + c]);
        }
    const double ext = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    const double inv = ext > 0.0 ? 2097152.0 / ext : 0.0;
    std::vector<unsigned long long> code(n);
    for (int i = 0; i < n; ++i) {
        unsigned q[3];
        for (int c = 0; c < 3; ++c) {
            const double f = std::floor((pts[3 * i + c] - lo[c]) * inv);
            q[c] = f >= 2097151.0 ? 2097151u : unsigned(f);
        }
        unsigned long long k = 0;
        for (int b = 0; b < 21; ++b)
            for (int c = 0; c < 3; ++c) k |= (unsigned long long)((q[c] >> b) & 1u) << (3 * b + 2 - c);
        code[i] = k;
    }
    order.resize(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return code[a] < code[b]; });
    codes.resize(n);
    for (int i = 0; i < n; ++i) codes[i] = code[order[i]];
}

// common prefix of the keys (code, position) at sorted positions i != j
static int morton_prefix(const std::vector<unsigned long long> &k, int i, int j) {
    if (k[i] != k[j]) return __builtin_clzll(k[i] ^ k[j]);
    return 64 + __builtin_clz(unsigned(i ^ j));
}

static int build_morton_range(Tree &tp, const std::vector<unsigned long long> &k, int l, int u, int bucket) {
    int id = int(tp.nodes.size());
    tp.nodes.push_back(Node());
    Node nd;
    std::memset(&nd, 0, sizeof(nd));
    nd.l = l;
    nd.u = u;
    nd.n = u - l + 1;
    nd.left = nd.right = -1;
    if ((u - l) <= bucket) {
        nd.dnum = 0;
        tp.nodes[id] = nd;
        return id;
    }
    const int dnode = morton_prefix(k, l, u);
    // last m in [l, u-1] with prefix(l, m) > dnode (prefix(l, .) does not grow along the keys)
    int a = l, b = u - 1;
    while (a < b) {
        const int m = (a + b + 1) / 2;
        if (morton_prefix(k, l, m) > dnode) a = m;
        else b = m - 1;
    }
    const int m = a;
    // split axis of the first differing bit (1..3), 1 when only the positions differ
    nd.dnum = dnode < 64 ? 1 + (2 - (63 - dnode) % 3) : 1;
    tp.nodes[id] = nd;
    int left = build_morton_range(tp, k, l, m, bucket);
    int right = build_morton_range(tp, k, m + 1, u, bucket);
    tp.nodes[id].left = left;
    tp.nodes[id].right = right;
    return id;
}

static void morton_sums(Tree &tp, int np, double *s) {
    Node &nd = tp.nodes[np];
    if (nd.dnum == 0) {
        s[0] = s[1] = s[2] = 0.0;
        for (int i = nd.l; i <= nd.u; ++i)
            for (int c = 0; c < 3; ++c) s[c] += tp.theData[3 * tp.indexes[i] + c];
    } else {
        double sl[3], sr[3];
        morton_sums(tp, nd.left, sl);
        morton_sums(tp, nd.right, sr);
        for (int c = 0; c < 3; ++c) s[c] = sl[c] + sr[c];
    }
    Node &me = tp.nodes[np];
    double radius = 0;
    for (int c = 0; c < 3; ++c) me.X[c] = s[c] / me.n;
    for (int i = me.l; i <= me.u; ++i) {
        double dx[3];
        for (int c = 0; c < 3; ++c) dx[c] = tp.theData[3 * tp.indexes[i] + c] - me.X[c];
        double dist = std::sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
        if (dist > radius) radius = dist;
    }
    me.oradius = 1.0 / radius;
}

static void label_nodes(Tree &tp, int np, int level) {
    // kd_tree.F90:502-534
    tp.nodes[np].lvl = level;
    tp.maxDepth = std::max(tp.maxDepth, level);
    if (tp.nodes[np].dnum != 0) {
        label_nodes(tp, tp.nodes[np].left, level + 1);
        label_nodes(tp, tp.nodes[np].right, level + 1);
    }
}

static void set_centers(Tree &tp, int np) {
    // kd_tree.F90:558-593: unweighted centroid, oradius = 1/max|x-X|
    Node &nd = tp.nodes[np];
    double X[3] = {0, 0, 0};
    for (int i = nd.l; i <= nd.u; ++i)
        for (int k = 0; k < 3; ++k) X[k] += tp.theData[3 * tp.indexes[i] + k];
    for (int k = 0; k < 3; ++k) X[k] = X[k] / nd.n;
    double radius = 0;
    for (int i = nd.l; i <= nd.u; ++i) {
        double dx[3];
        for (int k = 0; k < 3; ++k) dx[k] = tp.theData[3 * tp.indexes[i] + k] - X[k];
        double dist = std::sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
        if (dist > radius) radius = dist;
        nd.oradius = 1.0 / radius;
    }
    for (int k = 0; k < 3; ++k) nd.X[k] = X[k];
    if (nd.dnum != 0) {
        int lft = nd.left, rgt = nd.right;
        set_centers(tp, lft);
        set_centers(tp, rgt);
    }
}

static void set_ai(Tree &tp, int np) {
    // kd_tree.F90:536-556
    Node &nd = tp.nodes[np];
    if (nd.dnum == 0) {
        double a = 0;
        for (int i = nd.l; i <= nd.u; ++i) a = a + tp.Ai[i];
        nd.Ai = a;
    } else {
        set_ai(tp, nd.left);
        set_ai(tp, nd.right);
        tp.nodes[np].Ai = tp.nodes[tp.nodes[np].left].Ai + tp.nodes[tp.nodes[np].right].Ai;
    }
}

// ---------------------------------------------------------------------------
// Geometry: src/utils/vectorUtils.f90:7-103, src/warp/getElementProps.F90:1-46,
// src/utils/getSpherePts.F90:1-71
// ---------------------------------------------------------------------------
template <class A, class B, class C>
static inline void cross3(const A *v1, const B *v2, C *c) {
    c[0] = (v1[1] * v2[2] - v1[2] * v2[1]);
    c[1] = (v1[2] * v2[0] - v1[0] * v2[2]);
    c[2] = (v1[0] * v2[1] - v1[1] * v2[0]);
}

template <class T>
static inline T get_mag(const T *v) {
    return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + 1e-30);
}

template <class T>
static void get_element_props(const T *points, int nPts, T &area, T *normal) {
    T center[3] = {T(0), T(0), T(0)};
    for (int i = 0; i < nPts; ++i)
        for (int k = 0; k < 3; ++k) center[k] = center[k] + points[3 * i + k];
    for (int k = 0; k < 3; ++k) center[k] = center[k] / double(nPts);
    std::vector<T> rv(3 * nPts);
    for (int i = 0; i < nPts; ++i)
        for (int k = 0; k < 3; ++k) rv[3 * i + k] = points[3 * i + k] - center[k];
    normal[0] = normal[1] = normal[2] = T(0);
    area = T(0);
    for (int i = 0; i < nPts; ++i) {
        T c[3];
        int j = (i < nPts - 1) ? i + 1 : 0;
        cross3(&rv[3 * i], &rv[3 * j], c);
        T cn = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + 1e-15);
        area = area + 0.5 * cn;
        for (int k = 0; k < 3; ++k) normal[k] = normal[k] + c[k] / cn;
    }
    T nm = std::sqrt(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]);
    for (int k = 0; k < 3; ++k) normal[k] = normal[k] / nm;
}

// Reverse of get_element_props: given areab and normalb accumulate pointsb.
// Hand-derived adjoint of the routine above; it reproduces the semantics of
// src/adjoint/outputReverse/getElementProps_b.f90:7-115 (including the
// zero-guard on |normal|^2 == 0).
static void get_element_props_b(const double *points, int nPts, double areab, const double *normalb,
                                double *pointsb) {
    double center[3] = {0, 0, 0};
    for (int i = 0; i < nPts; ++i)
        for (int k = 0; k < 3; ++k) center[k] += points[3 * i + k];
    for (int k = 0; k < 3; ++k) center[k] = center[k] / double(nPts);
    std::vector<double> rv(3 * nPts), rvb(3 * nPts, 0.0), cr(3 * nPts), cn(nPts);
    for (int i = 0; i < nPts; ++i)
        for (int k = 0; k < 3; ++k) rv[3 * i + k] = points[3 * i + k] - center[k];
    double nsum[3] = {0, 0, 0};
    for (int i = 0; i < nPts; ++i) {
        int j = (i < nPts - 1) ? i + 1 : 0;
        cross3(&rv[3 * i], &rv[3 * j], &cr[3 * i]);
        const double *c = &cr[3 * i];
        cn[i] = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + 1e-15);
        for (int k = 0; k < 3; ++k) nsum[k] += c[k] / cn[i];
    }
    // normal = nsum / |nsum|
    double t = nsum[0] * nsum[0] + nsum[1] * nsum[1] + nsum[2] * nsum[2];
    double t0 = std::sqrt(t);
    double nsumb[3];
    double dotb = nsum[0] * normalb[0] + nsum[1] * normalb[1] + nsum[2] * normalb[2];
    double tempb = (t == 0.0) ? 0.0 : -(dotb / (2.0 * t0 * t0 * t0));
    for (int k = 0; k < 3; ++k) nsumb[k] = normalb[k] / t0 + 2 * nsum[k] * tempb;
    for (int i = nPts - 1; i >= 0; --i) {
        const double *c = &cr[3 * i];
        double crb[3];
        for (int k = 0; k < 3; ++k) crb[k] = nsumb[k] / cn[i];
        double cnb = 0.5 * areab - (c[0] * nsumb[0] + c[1] * nsumb[1] + c[2] * nsumb[2]) / (cn[i] * cn[i]);
        double tb = cnb / (2.0 * cn[i]);
        for (int k = 0; k < 3; ++k) crb[k] += 2 * c[k] * tb;
        int j = (i < nPts - 1) ? i + 1 : 0;
        // c = a x b; ab += b x crb, bb += crb x a
        double tmp[3];
        cross3(&rv[3 * j], crb, tmp);
        for (int k = 0; k < 3; ++k) rvb[3 * i + k] += tmp[k];
        cross3(crb, &rv[3 * i], tmp);
        for (int k = 0; k < 3; ++k) rvb[3 * j + k] += tmp[k];
    }
    double centerb[3] = {0, 0, 0};
    for (int i = 0; i < nPts; ++i)
        for (int k = 0; k < 3; ++k) {
            pointsb[3 * i + k] += rvb[3 * i + k];
            centerb[k] -= rvb[3 * i + k];
        }
    for (int k = 0; k < 3; ++k) centerb[k] = centerb[k] / double(nPts);
    for (int i = 0; i < nPts; ++i)
        for (int k = 0; k < 3; ++k) pointsb[3 * i + k] += centerb[k];
}

// src/utils/vectorUtils.f90:31-103 (v1 = normals0 is real and fixed).
template <class T>
static void get_rotation_matrix(const double *v1, const T *v2, T *Mi) {
    const double tol = 1.4901161193847656e-08;
    double magV1 = get_mag(v1);
    T magV2 = get_mag(v2);
    T axis[3];
    cross3(v1, v2, axis);
    T axisMag = get_mag(axis);
    T angle;
    if (re(axisMag) < tol) {
        angle = T(0);
        axis[0] = T(1);
        axis[1] = T(0);
        axis[2] = T(0);
    } else {
        for (int k = 0; k < 3; ++k) axis[k] = axis[k] / axisMag;
        double vv1[3];
        T vv2[3];
        for (int k = 0; k < 3; ++k) {
            vv1[k] = v1[k] / magV1;
            vv2[k] = v2[k] / magV2;
        }
        T d = vv1[0] * vv2[0] + vv1[1] * vv2[1] + vv1[2] * vv2[2];
        T arg = (1.0 > re(d)) ? d : T(1.0);
        angle = std::acos(arg);
    }
    T A[9] = {T(0), -axis[2], axis[1], axis[2], T(0), -axis[0], -axis[1], axis[0], T(0)};
    T C[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C[3 * i + j] = A[3 * i + 0] * A[0 + j] + A[3 * i + 1] * A[3 + j] + A[3 * i + 2] * A[6 + j];
    T s = std::sin(angle), omc = 1.0 - std::cos(angle);
    for (int i = 0; i < 9; ++i) Mi[i] = T((i % 4 == 0) ? 1.0 : 0.0) + s * A[i] + omc * C[i];
}

// Reverse of get_rotation_matrix w.r.t. v2, given Mib.  Hand-derived adjoint
// reproducing src/adjoint/outputReverse/vectorUtils_b.f90:7-154: a zero
// derivative when axisMag < tol, and when the acos argument was clamped to 1.
static void get_rotation_matrix_b(const double *v1, const double *v2, const double *Mib, double *v2b) {
    const double tol = 1.4901161193847656e-08;
    double magV1 = get_mag(v1);
    double magV2 = get_mag(v2);
    double axis0[3];
    cross3(v1, v2, axis0);
    double axisMag = get_mag(axis0);
    if (axisMag < tol) return;
    double axis[3], vv1[3], vv2[3];
    for (int k = 0; k < 3; ++k) {
        axis[k] = axis0[k] / axisMag;
        vv1[k] = v1[k] / magV1;
        vv2[k] = v2[k] / magV2;
    }
    double d = vv1[0] * vv2[0] + vv1[1] * vv2[1] + vv1[2] * vv2[2];
    bool clamped = !(1.0 > d);
    double arg = clamped ? 1.0 : d;
    double angle = std::acos(arg);
    double A[9] = {0, -axis[2], axis[1], axis[2], 0, -axis[0], -axis[1], axis[0], 0};
    double C[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C[3 * i + j] = A[3 * i + 0] * A[0 + j] + A[3 * i + 1] * A[3 + j] + A[3 * i + 2] * A[6 + j];
    double s = std::sin(angle), c = std::cos(angle);
    double angleb = 0;
    for (int i = 0; i < 9; ++i) angleb += c * A[i] * Mib[i] + s * C[i] * Mib[i];
    double Ab[9], Cb[9];
    for (int i = 0; i < 9; ++i) {
        Ab[i] = s * Mib[i];
        Cb[i] = (1.0 - c) * Mib[i];
    }
    // C = A A  ->  Ab += Cb A^T + A^T Cb
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0;
            for (int k = 0; k < 3; ++k) acc += Cb[3 * i + k] * A[3 * j + k] + A[3 * k + i] * Cb[3 * k + j];
            Ab[3 * i + j] += acc;
        }
    double axisb[3];
    axisb[0] = Ab[3 * 2 + 1] - Ab[3 * 1 + 2];
    axisb[1] = Ab[3 * 0 + 2] - Ab[3 * 2 + 0];
    axisb[2] = Ab[3 * 1 + 0] - Ab[3 * 0 + 1];
    double argb = (arg == 1.0 || arg == -1.0) ? 0.0 : -(angleb / std::sqrt(1.0 - arg * arg));
    double vv2b[3] = {0, 0, 0};
    if (!clamped)
        for (int k = 0; k < 3; ++k) vv2b[k] = vv1[k] * argb;
    double magV2b = 0;
    for (int k = 0; k < 3; ++k) {
        v2b[k] += vv2b[k] / magV2;
        magV2b -= v2[k] * vv2b[k];
    }
    magV2b = magV2b / (magV2 * magV2);
    double axisMagb = -(axis0[0] * axisb[0] + axis0[1] * axisb[1] + axis0[2] * axisb[2]) / (axisMag * axisMag);
    double axis0b[3];
    for (int k = 0; k < 3; ++k) axis0b[k] = axisb[k] / axisMag + axis0[k] * axisMagb / axisMag;
    double tmp[3];
    cross3(axis0b, v1, tmp);  // axis0 = v1 x v2 -> v2b += axis0b x v1
    for (int k = 0; k < 3; ++k) v2b[k] += tmp[k] + v2[k] * magV2b / magV2;
}

static void get_sphere_pts(const double *x0, double radius, double *vpts /*3*20*/) {
    // src/utils/getSpherePts.F90:16-52
    const double o = 1.0, z = 0.0, p = kPhi, ip = 1.0 / kPhi;
    const double nom[20][3] = {{-o, -o, -o}, {o, -o, -o}, {-o, o, -o}, {o, o, -o}, {-o, -o, o},
                               {o, -o, o},   {-o, o, o},  {o, o, o},   {z, -ip, -p}, {z, ip, -p},
                               {z, -ip, p},  {z, ip, p},  {-ip, -p, z}, {ip, -p, z}, {-ip, p, z},
                               {ip, p, z},   {-p, z, -ip}, {-p, z, ip}, {p, z, -ip}, {p, z, ip}};
    for (int i = 0; i < 20; ++i)
        for (int k = 0; k < 3; ++k) vpts[3 * i + k] = nom[i][k] * radius / std::sqrt(3.0) + x0[k];
}

// ---------------------------------------------------------------------------
// Nodal properties: src/modules/kd_tree.F90:1580-1664 and 1666-1715.
// ---------------------------------------------------------------------------
template <class T>
struct Nodal {
    std::vector<T> Xu, normals, Mi, Bi;
};

template <class T>
static void compute_nodal_properties(Ctx &c, const T *Xs, bool initialPoint, Nodal<T> &nd) {
    Tree &tp = c.tp;
    const int n = tp.n;
    nd.Xu.assign(3 * n, T(0));
    nd.normals.assign(3 * n, T(0));
    nd.Mi.assign(9 * n, T(0));
    nd.Bi.assign(3 * n, T(0));
    for (int i = 0; i < n; ++i) {
        int j = tp.XuInd[i];
        for (int k = 0; k < 3; ++k) nd.Xu[3 * i + k] = Xs[3 * j + k];
    }
    std::vector<T> pts;
    for (int i = 0; i < n; ++i) {
        T sumArea = T(0);
        T sumNormal[3] = {T(0), T(0), T(0)};
        for (int e = tp.n2ePtr[i]; e < tp.n2ePtr[i + 1]; ++e) {
            int f = tp.n2e[e];
            int nPts = tp.facePtr[f + 1] - tp.facePtr[f];
            pts.resize(3 * nPts);
            for (int kk = 0; kk < nPts; ++kk) {
                int p = tp.faceConn[tp.facePtr[f] + kk];
                for (int k = 0; k < 3; ++k) pts[3 * kk + k] = nd.Xu[3 * p + k];
            }
            T area, fn[3];
            get_element_props(pts.data(), nPts, area, fn);
            T dA = area / double(nPts);
            sumArea = sumArea + dA;
            for (int k = 0; k < 3; ++k) sumNormal[k] = sumNormal[k] + dA * fn[k];
        }
        for (int k = 0; k < 3; ++k) nd.normals[3 * i + k] = sumNormal[k] / sumArea;
        if (initialPoint) {
            for (int k = 0; k < 3; ++k) tp.normals0[3 * i + k] = re(nd.normals[3 * i + k]);
            tp.Ai[i] = re(sumArea);
        } else {
            T *M = &nd.Mi[9 * i];
            if (c.o.useRotations && !tp.isCorner[i]) {
                get_rotation_matrix(&tp.normals0[3 * i], &nd.normals[3 * i], M);
            } else {
                for (int q = 0; q < 9; ++q) M[q] = T((q % 4 == 0) ? 1.0 : 0.0);
            }
            const double *x0 = &tp.Xu0[3 * i];
            for (int a = 0; a < 3; ++a)
                nd.Bi[3 * i + a] = nd.Xu[3 * i + a] - (M[3 * a + 0] * x0[0] + M[3 * a + 1] * x0[1] + M[3 * a + 2] * x0[2]);
        }
    }
    for (int i = 0; i < n; ++i) {
        if (tp.Ai[i] == 0.0) {
            for (int k = 0; k < 3; ++k) {
                nd.normals[3 * i + k] = T(0);
                nd.Bi[3 * i + k] = T(0);
            }
            for (int q = 0; q < 9; ++q) nd.Mi[9 * i + q] = T((q % 4 == 0) ? 1.0 : 0.0);
        }
    }
}

static void determine_corners(Ctx &c, const std::vector<double> &Xu) {
    Tree &tp = c.tp;
    double threshold = std::cos(c.o.cornerAngle * kPi / 180.0);
    tp.isCorner.assign(tp.n, 0);
    if (!c.o.zeroCornerRotations) return;
    std::vector<double> pts;
    for (int i = 0; i < tp.n; ++i) {
        for (int e = tp.n2ePtr[i]; e < tp.n2ePtr[i + 1]; ++e) {
            int f = tp.n2e[e];
            int nPts = tp.facePtr[f + 1] - tp.facePtr[f];
            pts.resize(3 * nPts);
            for (int kk = 0; kk < nPts; ++kk) {
                int p = tp.faceConn[tp.facePtr[f] + kk];
                for (int k = 0; k < 3; ++k) pts[3 * kk + k] = Xu[3 * p + k];
            }
            double area, fn[3];
            get_element_props(pts.data(), nPts, area, fn);
            const double *n0 = &tp.normals0[3 * i];
            double dp = fn[0] * n0[0] + fn[1] * n0[1] + fn[2] * n0[2];
            if (std::fabs(dp) < threshold) tp.isCorner[i] = 1;
        }
    }
}

// Reverse nodal properties: src/modules/kd_tree.F90:1057-1162.  Bib/Mib hold
// the per-point adjoints; the result is ADDED into xsb (caller order) at the
// FIRST caller occurrence of each unique point only (kd_tree.F90:1155-1159).
static void compute_nodal_properties_b(Ctx &c, const Nodal<double> &nd, std::vector<double> &Bib,
                                       std::vector<double> &Mib, double *xsb) {
    Tree &tp = c.tp;
    const int n = tp.n;
    std::vector<double> Xub(3 * n, 0.0);
    std::vector<double> pts, ptsb;
    for (int i = 0; i < n; ++i) {
        // forward recompute of the face sums for node i (from the Xu's)
        double sumArea = 0, sumNormal[3] = {0, 0, 0};
        int e0 = tp.n2ePtr[i], e1 = tp.n2ePtr[i + 1];
        std::vector<double> fnAll(3 * (e1 - e0)), dAAll(e1 - e0);
        for (int e = e0; e < e1; ++e) {
            int f = tp.n2e[e];
            int nPts = tp.facePtr[f + 1] - tp.facePtr[f];
            pts.resize(3 * nPts);
            for (int kk = 0; kk < nPts; ++kk) {
                int p = tp.faceConn[tp.facePtr[f] + kk];
                for (int k = 0; k < 3; ++k) pts[3 * kk + k] = nd.Xu[3 * p + k];
            }
            double area, fn[3];
            get_element_props(pts.data(), nPts, area, fn);
            double dA = area / double(nPts);
            sumArea = sumArea + dA;
            for (int k = 0; k < 3; ++k) sumNormal[k] = sumNormal[k] + dA * fn[k];
            for (int k = 0; k < 3; ++k) fnAll[3 * (e - e0) + k] = fn[k];
            dAAll[e - e0] = dA;
        }
        double normals[3];
        for (int k = 0; k < 3; ++k) normals[k] = sumNormal[k] / sumArea;
        double normalsb[3] = {0, 0, 0};
        double *bib = &Bib[3 * i];
        double *mib = &Mib[9 * i];
        for (int a = 0; a < 3; ++a) {
            Xub[3 * i + a] += bib[a];
            for (int k = 0; k < 3; ++k) mib[3 * a + k] -= tp.Xu0[3 * i + k] * bib[a];
        }
        if (c.o.useRotations && !tp.isCorner[i]) get_rotation_matrix_b(&tp.normals0[3 * i], normals, mib, normalsb);
        double sumNormalb[3];
        for (int k = 0; k < 3; ++k) sumNormalb[k] = normalsb[k] / sumArea;
        double sumAreab = -(sumNormal[0] * normalsb[0] + sumNormal[1] * normalsb[1] + sumNormal[2] * normalsb[2]) /
                          sumArea / sumArea;
        for (int e = e1 - 1; e >= e0; --e) {
            int f = tp.n2e[e];
            int nPts = tp.facePtr[f + 1] - tp.facePtr[f];
            const double *fn = &fnAll[3 * (e - e0)];
            double dA = dAAll[e - e0];
            double dAb = sumAreab + fn[0] * sumNormalb[0] + fn[1] * sumNormalb[1] + fn[2] * sumNormalb[2];
            double fnb[3];
            for (int k = 0; k < 3; ++k) fnb[k] = dA * sumNormalb[k];
            double areab = dAb / double(nPts);
            pts.resize(3 * nPts);
            ptsb.assign(3 * nPts, 0.0);
            for (int kk = 0; kk < nPts; ++kk) {
                int p = tp.faceConn[tp.facePtr[f] + kk];
                for (int k = 0; k < 3; ++k) pts[3 * kk + k] = nd.Xu[3 * p + k];
            }
            get_element_props_b(pts.data(), nPts, areab, fnb, ptsb.data());
            for (int kk = nPts - 1; kk >= 0; --kk) {
                int p = tp.faceConn[tp.facePtr[f] + kk];
                for (int k = 0; k < 3; ++k) Xub[3 * p + k] += ptsb[3 * kk + k];
            }
        }
    }
    for (int i = 0; i < n; ++i) {
        int j = tp.XuInd[i];
        for (int k = 0; k < 3; ++k) xsb[3 * j + k] += Xub[3 * i + k];
    }
}

// ---------------------------------------------------------------------------
// Tree aggregates, error tables and evaluation: kd_tree.F90:595-1051.
// ---------------------------------------------------------------------------
template <class T>
struct NodeAgg {
    std::vector<T> Mi, Bi;  // per tree node (9 / 3)
};

template <class T>
static void set_data(const Tree &tp, const Nodal<T> &nd, NodeAgg<T> &ag) {
    // kd_tree.F90:595-617: UNWEIGHTED means over [l,u] for interior nodes
    ag.Mi.assign(9 * tp.nodes.size(), T(0));
    ag.Bi.assign(3 * tp.nodes.size(), T(0));
    for (size_t q = 0; q < tp.nodes.size(); ++q) {
        const Node &np = tp.nodes[q];
        if (np.dnum == 0) continue;
        T B[3] = {T(0), T(0), T(0)};
        T M[9];
        for (int s = 0; s < 9; ++s) M[s] = T(0);
        for (int i = np.l; i <= np.u; ++i) {
            for (int k = 0; k < 3; ++k) B[k] = B[k] + nd.Bi[3 * i + k];
            for (int s = 0; s < 9; ++s) M[s] = M[s] + nd.Mi[9 * i + s];
        }
        for (int k = 0; k < 3; ++k) ag.Bi[3 * q + k] = B[k] / double(np.n);
        for (int s = 0; s < 9; ++s) ag.Mi[9 * q + s] = M[s] / double(np.n);
    }
}

static inline double weight(const Tree &tp, double A, double LdefoDist) {
    return A * (std::pow(LdefoDist, tp.aExp) + tp.alphaToBexp * std::pow(LdefoDist, tp.bExp));
}

static double get_error(const Tree &tp, const Node &np, double dist) {
    // kd_tree.F90:882-906
    double dOvrR = dist * np.oradius;
    double err = np.err[kNerr - 1];
    for (int i = 0; i < 11; ++i) {
        if (dOvrR < kRstar[i + 1]) {
            double fact = (dOvrR - kRstar[i]) * tp.orstar[i];
            err = (1.0 - fact) * np.err[i] + fact * np.err[i + 1];
            break;
        }
    }
    return err;
}

template <class T>
static void eval_node_exact(const Tree &tp, const Nodal<T> &nd, const Node &np, const double *r, T *num, T &den,
                            Stats &st) {
    // kd_tree.F90:664-690
    for (int i = np.l; i <= np.u; ++i) {
        double rr0 = r[0] - tp.Xu0[3 * i], rr1 = r[1] - tp.Xu0[3 * i + 1], rr2 = r[2] - tp.Xu0[3 * i + 2];
        double LdefoDist = tp.Ldef / std::sqrt(rr0 * rr0 + rr1 * rr1 + rr2 * rr2 + kEps);
        double Wi = weight(tp, tp.Ai[i], LdefoDist);
        const T *M = &nd.Mi[9 * i];
        const T *B = &nd.Bi[3 * i];
        for (int a = 0; a < 3; ++a) {
            T Si = M[3 * a + 0] * r[0] + M[3 * a + 1] * r[1] + M[3 * a + 2] * r[2] + B[a] - r[a];
            num[a] = num[a] + Wi * Si;
        }
        den = den + Wi;
    }
    st.leafPairs += np.n;
}

template <class T>
static void eval_node_approx(const Tree &tp, const NodeAgg<T> &ag, int q, const double *r, T *num, T &den,
                             double dist) {
    // kd_tree.F90:692-713
    const Node &np = tp.nodes[q];
    double LdefoDist = tp.Ldef / dist;
    double Wi = weight(tp, np.Ai, LdefoDist);
    const T *M = &ag.Mi[9 * q];
    const T *B = &ag.Bi[3 * q];
    for (int a = 0; a < 3; ++a) {
        T Si = M[3 * a + 0] * r[0] + M[3 * a + 1] * r[1] + M[3 * a + 2] * r[2] + B[a] - r[a];
        num[a] = num[a] + Wi * Si;
    }
    den = den + Wi;
}

template <class T>
static void eval_node(const Tree &tp, const Nodal<T> &nd, const NodeAgg<T> &ag, int q, const double *r, T *num,
                      T &den, double approxDen, Stats &st) {
    // kd_tree.F90:619-662
    const Node &np = tp.nodes[q];
    st.visited++;
    if (np.dnum == 0) {
        eval_node_exact(tp, nd, np, r, num, den, st);
    } else {
        double dist = std::sqrt((r[0] - np.X[0]) * (r[0] - np.X[0]) + (r[1] - np.X[1]) * (r[1] - np.X[1]) +
                                (r[2] - np.X[2]) * (r[2] - np.X[2]));
        if (dist * np.oradius < 2.0) {
            eval_node(tp, nd, ag, np.left, r, num, den, approxDen, st);
            eval_node(tp, nd, ag, np.right, r, num, den, approxDen, st);
        } else {
            double err = get_error(tp, np, dist);
            if (err < tp.errTol * approxDen) {
                eval_node_approx(tp, ag, q, r, num, den, dist);
                st.approx++;
            } else {
                eval_node(tp, nd, ag, np.left, r, num, den, approxDen, st);
                eval_node(tp, nd, ag, np.right, r, num, den, approxDen, st);
            }
        }
    }
}

static void get_wi_estimate(const Tree &tp, int q, const double *r, double &den) {
    // kd_tree.F90:751-787
    const Node &np = tp.nodes[q];
    if (np.dnum == 0) {
        for (int i = np.l; i <= np.u; ++i) {
            double rr0 = r[0] - tp.Xu0[3 * i], rr1 = r[1] - tp.Xu0[3 * i + 1], rr2 = r[2] - tp.Xu0[3 * i + 2];
            double LdefoDist = tp.Ldef / std::sqrt(rr0 * rr0 + rr1 * rr1 + rr2 * rr2 + 1e-16);
            den = den + weight(tp, tp.Ai[i], LdefoDist);
        }
    } else {
        double rr0 = r[0] - np.X[0], rr1 = r[1] - np.X[1], rr2 = r[2] - np.X[2];
        double dist = std::sqrt(rr0 * rr0 + rr1 * rr1 + rr2 * rr2 + 1e-16);
        if (dist * np.oradius > 5.0) {
            double LdefoDist = tp.Ldef / dist;
            den = den + weight(tp, np.Ai, LdefoDist);
        } else {
            get_wi_estimate(tp, np.left, r, den);
            get_wi_estimate(tp, np.right, r, den);
        }
    }
}

static void dry_run(const Tree &tp, int q, const double *r, double approxDen, double &cst) {
    // kd_tree.F90:789-830 (load-balancing cost model)
    const Node &np = tp.nodes[q];
    if (np.dnum == 0) {
        cst = cst + double(np.n);
    } else {
        double rr0 = r[0] - np.X[0], rr1 = r[1] - np.X[1], rr2 = r[2] - np.X[2];
        double dist = std::sqrt(rr0 * rr0 + rr1 * rr1 + rr2 * rr2 + 1e-16);
        cst = cst + 0.5;
        if (dist * np.oradius < 2.0) {
            dry_run(tp, np.left, r, approxDen, cst);
            dry_run(tp, np.right, r, approxDen, cst);
        } else {
            double err = get_error(tp, np, dist);
            if (err < tp.errTol * approxDen) {
                cst = cst + 1.1;
            } else {
                dry_run(tp, np.left, r, approxDen, cst);
                dry_run(tp, np.right, r, approxDen, cst);
            }
        }
    }
}

static void compute_errors(Tree &tp) {
    // kd_tree.F90:832-880
#pragma omp parallel for schedule(dynamic, 4)
    for (long q = 0; q < (long)tp.nodes.size(); ++q) {
        Node &np = tp.nodes[q];
        if (np.dnum == 0) continue;
        for (int j = 0; j < kNerr; ++j) {
            double vpts[60];
            get_sphere_pts(np.X, 1.0 / np.oradius * kRstar[j], vpts);
            double e = 0;
            for (int ii = 0; ii < 20; ++ii) {
                double dExact = 0, dApprox = 0;
                for (int i = np.l; i <= np.u; ++i) {
                    double rr0 = vpts[3 * ii] - tp.Xu0[3 * i], rr1 = vpts[3 * ii + 1] - tp.Xu0[3 * i + 1],
                           rr2 = vpts[3 * ii + 2] - tp.Xu0[3 * i + 2];
                    double dist = std::sqrt(rr0 * rr0 + rr1 * rr1 + rr2 * rr2);
                    dExact = dExact + weight(tp, tp.Ai[i], tp.Ldef / dist);
                }
                double rr0 = vpts[3 * ii] - np.X[0], rr1 = vpts[3 * ii + 1] - np.X[1], rr2 = vpts[3 * ii + 2] - np.X[2];
                double dist = std::sqrt(rr0 * rr0 + rr1 * rr1 + rr2 * rr2);
                dApprox = dApprox + weight(tp, np.Ai, tp.Ldef / dist);
                e = e + (dExact - dApprox) * (dExact - dApprox);
            }
            np.err[j] = std::sqrt(e / 20);
        }
    }
}

// ---- reverse walk: kd_tree.F90:942-1051 ----
struct Adj {
    std::vector<double> Bib, Mib;    // per point (3 / 9)
    std::vector<double> nBib, nMib;  // per tree node (3 / 9)
    void init(size_t n, size_t nn) {
        Bib.assign(3 * n, 0.0);
        Mib.assign(9 * n, 0.0);
        nBib.assign(3 * nn, 0.0);
        nMib.assign(9 * nn, 0.0);
    }
};

static void eval_node_exact_b(const Tree &tp, const Node &np, const double *r, const double *numb, Adj &ad) {
    for (int i = np.l; i <= np.u; ++i) {
        double rr0 = r[0] - tp.Xu0[3 * i], rr1 = r[1] - tp.Xu0[3 * i + 1], rr2 = r[2] - tp.Xu0[3 * i + 2];
        double dist = std::sqrt(rr0 * rr0 + rr1 * rr1 + rr2 * rr2 + kEps);
        double Wi = weight(tp, tp.Ai[i], tp.Ldef / dist);
        double sib[3] = {Wi * numb[0], Wi * numb[1], Wi * numb[2]};
        for (int a = 0; a < 3; ++a) {
            for (int k = 0; k < 3; ++k) ad.Mib[9 * i + 3 * a + k] += r[k] * sib[a];
            ad.Bib[3 * i + a] += sib[a];
        }
    }
}

static void eval_node_approx_b(const Tree &tp, int q, const double *numb, const double *r, double dist, Adj &ad) {
    const Node &np = tp.nodes[q];
    double Wi = weight(tp, np.Ai, tp.Ldef / dist);
    double sib[3] = {Wi * numb[0], Wi * numb[1], Wi * numb[2]};
    for (int a = 0; a < 3; ++a) {
        for (int k = 0; k < 3; ++k) ad.nMib[9 * q + 3 * a + k] += r[k] * sib[a];
        ad.nBib[3 * q + a] += sib[a];
    }
}

static void eval_node_b(const Tree &tp, int q, const double *r, const double *numb, double approxDen, Adj &ad) {
    const Node &np = tp.nodes[q];
    if (np.dnum == 0) {
        eval_node_exact_b(tp, np, r, numb, ad);
    } else {
        double rr0 = r[0] - np.X[0], rr1 = r[1] - np.X[1], rr2 = r[2] - np.X[2];
        double dist = std::sqrt(rr0 * rr0 + rr1 * rr1 + rr2 * rr2);
        if (dist * np.oradius < 2.0) {
            eval_node_b(tp, np.left, r, numb, approxDen, ad);
            eval_node_b(tp, np.right, r, numb, approxDen, ad);
        } else {
            double err = get_error(tp, np, dist);
            if (err < tp.errTol * approxDen) {
                eval_node_approx_b(tp, q, numb, r, dist, ad);
            } else {
                eval_node_b(tp, np.left, r, numb, approxDen, ad);
                eval_node_b(tp, np.right, r, numb, approxDen, ad);
            }
        }
    }
}

static void set_data_b(const Tree &tp, Adj &ad) {
    // kd_tree.F90:1033-1051
    for (size_t q = 0; q < tp.nodes.size(); ++q) {
        const Node &np = tp.nodes[q];
        if (np.dnum == 0) continue;
        double ovrN = 1.0 / np.n;
        for (int i = np.l; i <= np.u; ++i) {
            for (int k = 0; k < 3; ++k) ad.Bib[3 * i + k] += ad.nBib[3 * q + k] * ovrN;
            for (int s = 0; s < 9; ++s) ad.Mib[9 * i + s] += ad.nMib[9 * q + s] * ovrN;
        }
    }
}

// ---- symmetry mirrors: src/warp/initializeWarping.F90:533-659 ----
static void get_mirror_pt(const Ctx &c, const double *pt, double *r, int kk) {
    // kk is 1-based as in the reference
    r[0] = pt[0];
    r[1] = pt[1];
    r[2] = pt[2];
    for (int j = 1; j <= c.nSym; ++j) {
        if (((kk - 1) % (1 << j)) >= (1 << (j - 1))) {
            const double *p = &c.symPts[3 * (j - 1)];
            const double *n = &c.symNormals[3 * (j - 1)];
            double d[3] = {r[0] - p[0], r[1] - p[1], r[2] - p[2]};
            double dp = d[0] * n[0] + d[1] * n[1] + d[2] * n[2];
            for (int k = 0; k < 3; ++k) r[k] = r[k] - 2 * n[k] * dp;
        }
    }
}

template <class T>
static void get_mirror_numerator(const Ctx &c, T *num, int kk) {
    for (int j = 1; j <= c.nSym; ++j) {
        if (((kk - 1) % (1 << j)) >= (1 << (j - 1))) {
            const double *n = &c.symNormals[3 * (j - 1)];
            T dp = num[0] * n[0] + num[1] * n[1] + num[2] * n[2];
            for (int k = 0; k < 3; ++k) num[k] = num[k] - 2.0 * dp * n[k];
        }
    }
}

static void get_mirror_numerator_b(const Ctx &c, double *numb, int kk) {
    for (int j = c.nSym; j >= 1; --j) {
        if (((kk - 1) % (1 << j)) >= (1 << (j - 1))) {
            const double *n = &c.symNormals[3 * (j - 1)];
            double dpb = -(n[0] * 2.0 * numb[0] + n[1] * 2.0 * numb[1] + n[2] * 2.0 * numb[2]);
            for (int k = 0; k < 3; ++k) numb[k] = numb[k] + n[k] * dpb;
        }
    }
}

// ---------------------------------------------------------------------------
// myCreateTree: kd_tree.F90:1365-1545, plus the denominator estimate of
// src/warp/initializeWarping.F90:235-247.
// ---------------------------------------------------------------------------
static int create_tree(Ctx &c, const double *uniquePts, int nUnique, const int *link, int nLink,
                       const int *faceSizes, int nFaces, const int *conn, int nConn) {
    Tree &tp = c.tp;
    tp = Tree();
    tp.facePtr.assign(nFaces + 1, 0);
    for (int i = 0; i < nFaces; ++i) tp.facePtr[i + 1] = tp.facePtr[i] + faceSizes[i];
    if (tp.facePtr[nFaces] != nConn) return -3;
    tp.n = nUnique;
    if (nUnique < 1) return -3;
    tp.theData.assign(uniquePts, uniquePts + 3 * nUnique);
    tp.indexes.resize(nUnique);
    std::iota(tp.indexes.begin(), tp.indexes.end(), 0);
    tp.nodes.reserve(2 * nUnique);
    if (c.o.treeBuild == 1) {
        std::vector<unsigned long long> codes;
        morton_order(uniquePts, nUnique, codes, tp.indexes);
        tp.root = build_morton_range(tp, codes, 0, nUnique - 1, c.o.bucketSize);
        tp.maxDepth = 1;
        label_nodes(tp, tp.root, 1);
        double s[3];
        morton_sums(tp, tp.root, s);
    } else {
        tp.root = build_range(tp, 0, nUnique - 1, c.o.bucketSize);
        tp.maxDepth = 1;
        label_nodes(tp, tp.root, 1);
        set_centers(tp, tp.root);
    }
    tp.Xu0.resize(3 * nUnique);
    for (int i = 0; i < nUnique; ++i)
        for (int k = 0; k < 3; ++k) tp.Xu0[3 * i + k] = uniquePts[3 * tp.indexes[i] + k];
    std::vector<int> invIndices(nUnique);
    for (int i = 0; i < nUnique; ++i) invIndices[tp.indexes[i]] = i;
    tp.faceConn.resize(nConn);
    for (int i = 0; i < nConn; ++i) {
        if (conn[i] < 0 || conn[i] >= nLink) return -3;
        tp.faceConn[i] = invIndices[link[conn[i]] - 1];
    }
    // node -> faces, one entry per occurrence, faces in increasing order
    std::vector<int> cnt(nUnique, 0);
    for (int f = 0; f < nFaces; ++f)
        for (int j = tp.facePtr[f]; j < tp.facePtr[f + 1]; ++j) cnt[tp.faceConn[j]]++;
    tp.n2ePtr.assign(nUnique + 1, 0);
    for (int i = 0; i < nUnique; ++i) tp.n2ePtr[i + 1] = tp.n2ePtr[i] + cnt[i];
    tp.n2e.assign(tp.n2ePtr[nUnique], 0);
    std::vector<int> fill(tp.n2ePtr.begin(), tp.n2ePtr.end() - 1);
    for (int f = 0; f < nFaces; ++f)
        for (int j = tp.facePtr[f]; j < tp.facePtr[f + 1]; ++j) tp.n2e[fill[tp.faceConn[j]]++] = f;
    tp.XuInd.assign(nUnique, -1);
    for (int i = 0; i < nLink; ++i) {
        int t = invIndices[link[i] - 1];
        if (tp.XuInd[t] < 0) tp.XuInd[t] = i;
    }
    double Xcen[3] = {0, 0, 0};
    for (int i = 0; i < nUnique; ++i)
        for (int k = 0; k < 3; ++k) Xcen[k] += tp.Xu0[3 * i + k];
    for (int k = 0; k < 3; ++k) Xcen[k] = Xcen[k] / nUnique;
    tp.Ldef0 = 0;
    for (int i = 0; i < nUnique; ++i) {
        double dx[3];
        for (int k = 0; k < 3; ++k) dx[k] = tp.theData[3 * i + k] - Xcen[k];
        tp.Ldef0 = std::max(tp.Ldef0, std::sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]));
    }
    tp.Ai.assign(nUnique, 0.0);
    tp.normals0.assign(3 * nUnique, 0.0);
    tp.isCorner.assign(nUnique, 0);
    // initNodalProperties (kd_tree.F90:1547-1578): normals0, Ai, corners.
    Nodal<double> nd;
    compute_nodal_properties(c, c.Xs.data(), true, nd);
    determine_corners(c, nd.Xu);
    set_ai(tp, tp.root);
    tp.Ldef = tp.Ldef0 * c.o.LdefFact;
    tp.alphaToBexp = std::pow(c.o.alpha, c.o.bExp);
    tp.aExp = c.o.aExp;
    tp.bExp = c.o.bExp;
    tp.errTol = c.o.errTol;
    for (int i = 0; i < kNerr - 1; ++i) tp.orstar[i] = 1.0 / (kRstar[i + 1] - kRstar[i]);
    compute_errors(tp);
    return 0;
}

}  // namespace orc

using namespace orc;

extern "C" {

static void unpack_opts(const double *v, Opts &o) {
    o.aExp = v[0];
    o.bExp = v[1];
    o.LdefFact = v[2];
    o.alpha = v[3];
    o.errTol = v[4];
    o.evalMode = int(v[5]);
    o.useRotations = int(v[6]);
    o.zeroCornerRotations = int(v[7]);
    o.cornerAngle = v[8];
    o.bucketSize = int(v[9]);
    o.treeBuild = int(v[10]);
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void *orc_new(const double *opts) {
    Ctx *c = new Ctx();
    unpack_opts(opts, c->o);
    return c;
}

void orc_free(void *h) { delete (Ctx *)h; }

// _setMeshOptions (idwarp/UnstructuredMesh.py:1051-1069)
int orc_set_options(void *h, const double *opts) {
    unpack_opts(opts, ((Ctx *)h)->o);
    return 0;
}

// setSymmetryPlanes (src/warp/initializeWarping.F90:511-531)
int orc_set_symmetry(void *h, const double *pts, const double *normals, int n) {
    Ctx *c = (Ctx *)h;
    if (n < 0 || n > 6) return -2;
    c->nSym = n;
    c->nLoop = 1 << n;
    c->symPts.assign(pts, pts + 3 * n);
    c->symNormals.assign(normals, normals + 3 * n);
    return 0;
}

// createCommonGrid (src/IO/createGrid.F90)
int orc_set_volume(void *h, const double *xv0, long long nVol) {
    Ctx *c = (Ctx *)h;
    c->nVol = nVol;
    c->Xv0.assign(xv0, xv0 + 3 * nVol);
    c->Xv = c->Xv0;
    return 0;
}

int orc_point_reduce(const double *pts, int n, double tol, double *uniquePts, int *link) {
    return point_reduce(pts, n, tol, uniquePts, link);
}

// USMesh.setSurfaceDefinition (idwarp/UnstructuredMesh.py:196-262) followed by
// initializeWarping (src/warp/initializeWarping.F90:1-247, one process).
int orc_set_surface_definition(void *h, const double *pts, int nPts, const int *conn, int nConn,
                               const int *faceSizes, int nFaces) {
    Ctx *c = (Ctx *)h;
    c->nPts = nPts;
    c->Xs.assign(pts, pts + 3 * nPts);
    std::vector<double> uniq(3 * (size_t)std::max(nPts, 1));
    std::vector<int> link(std::max(nPts, 1));
    int nUnique = point_reduce(pts, nPts, 1e-12, uniq.data(), link.data());
    // np.lexsort(uniquePts.T): z primary, then y, then x; stable
    std::vector<int> ind(nUnique);
    std::iota(ind.begin(), ind.end(), 0);
    std::stable_sort(ind.begin(), ind.end(), [&](int a, int b) {
        const double *pa = &uniq[3 * a], *pb = &uniq[3 * b];
        if (pa[2] != pb[2]) return pa[2] < pb[2];
        if (pa[1] != pb[1]) return pa[1] < pb[1];
        return pa[0] < pb[0];
    });
    std::vector<double> sorted(3 * (size_t)nUnique);
    for (int i = 0; i < nUnique; ++i)
        for (int k = 0; k < 3; ++k) sorted[3 * i + k] = uniq[3 * ind[i] + k];
    std::vector<int> inv(nUnique);
    for (int i = 0; i < nUnique; ++i) inv[ind[i]] = i;
    for (int i = 0; i < nPts; ++i) link[i] = inv[link[i] - 1] + 1;
    int rc = create_tree(*c, sorted.data(), nUnique, link.data(), nPts, faceSizes, nFaces, conn, nConn);
    if (rc) return rc;
    c->haveTree = true;
    // denominator0 (initializeWarping.F90:241-247)
    c->den0.assign(c->nVol, 0.0);
    Tree &tp = c->tp;
#pragma omp parallel for schedule(dynamic, 256)
    for (long long j = 0; j < c->nVol; ++j) {
        double acc = 0;
        for (int kk = 1; kk <= c->nLoop; ++kk) {
            double r[3];
            get_mirror_pt(*c, &c->Xv0[3 * j], r, kk);
            get_wi_estimate(tp, tp.root, r, acc);
        }
        c->den0[j] = acc;
    }
    c->numer.assign(3 * c->nVol, 0.0);
    c->denom.assign(c->nVol, 0.0);
    c->haveDenom = false;
    return 0;
}

// setSurfaceCoordinates (src/warp/setSurfaceCoordinates.F90:1-28)
int orc_set_surface_coords(void *h, const double *xs) {
    Ctx *c = (Ctx *)h;
    c->Xs.assign(xs, xs + 3 * c->nPts);
    return 0;
}

}  // extern "C"

// warpMesh (src/warp/warpMesh.F90:1-82), templated so the same code runs in
// complex arithmetic for complex-step derivatives.
template <class T>
static int warp_impl(Ctx *c, const T *Xs, T *XvOut, double *denOut, long long j0, long long j1) {
    Tree &tp = c->tp;
    Nodal<T> nd;
    compute_nodal_properties(*c, Xs, false, nd);
    tp.Ldef = tp.Ldef0 * c->o.LdefFact;
    tp.alphaToBexp = std::pow(c->o.alpha, c->o.bExp);
    tp.errTol = c->o.errTol;
    NodeAgg<T> ag;
    set_data(tp, nd, ag);
    long long lp = 0, ap = 0, vi = 0;
#pragma omp parallel reduction(+ : lp, ap, vi)
    {
        Stats st;
#pragma omp for schedule(dynamic, 64)
        for (long long j = j0; j < j1; ++j) {
            T numer[3] = {T(0), T(0), T(0)};
            T denom = T(0);
            for (int kk = 1; kk <= c->nLoop; ++kk) {
                double r[3];
                get_mirror_pt(*c, &c->Xv0[3 * j], r, kk);
                T num[3] = {T(0), T(0), T(0)};
                T den = T(0);
                if (c->o.evalMode == 0) {
                    eval_node_exact(tp, nd, tp.nodes[tp.root], r, num, den, st);
                    st.visited++;
                } else {
                    eval_node(tp, nd, ag, tp.root, r, num, den, c->den0[j], st);
                }
                get_mirror_numerator(*c, num, kk);
                for (int k = 0; k < 3; ++k) numer[k] = numer[k] + num[k];
                denom = denom + den;
            }
            T oden = 1.0 / denom;
            for (int k = 0; k < 3; ++k) XvOut[3 * j + k] = c->Xv0[3 * j + k] + numer[k] * oden;
            if (denOut) denOut[j] = re(denom);
        }
        lp += st.leafPairs;
        ap += st.approx;
        vi += st.visited;
    }
    c->st.leafPairs = lp;
    c->st.approx = ap;
    c->st.visited = vi;
    return 0;
}

extern "C" {

int orc_warp(void *h, double *xvOut) {
    Ctx *c = (Ctx *)h;
    if (!c->haveTree) return -4;
    int rc = warp_impl<double>(c, c->Xs.data(), c->Xv.data(), c->denom.data(), 0, c->nVol);
    c->haveDenom = true;
    if (xvOut) std::memcpy(xvOut, c->Xv.data(), sizeof(double) * 3 * c->nVol);
    return rc;
}

// Warp only the volume nodes [j0, j1) (bounded CPU-baseline samples).  Does
// not change the stored state other than Xv rows j0..j1.
int orc_warp_range(void *h, long long j0, long long j1) {
    Ctx *c = (Ctx *)h;
    if (!c->haveTree) return -4;
    return warp_impl<double>(c, c->Xs.data(), c->Xv.data(), nullptr, j0, j1);
}

int orc_warp_complex(void *h, const double *xsRe, const double *xsIm, double *xvRe, double *xvIm) {
    Ctx *c = (Ctx *)h;
    if (!c->haveTree) return -4;
    std::vector<cplx> xs(3 * c->nPts), xv(3 * c->nVol);
    for (int i = 0; i < 3 * c->nPts; ++i) xs[i] = cplx(xsRe[i], xsIm[i]);
    int rc = warp_impl<cplx>(c, xs.data(), xv.data(), nullptr, 0, c->nVol);
    for (long long i = 0; i < 3 * c->nVol; ++i) {
        xvRe[i] = xv[i].real();
        xvIm[i] = xv[i].imag();
    }
    return rc;
}

}  // extern "C"

// warpDeriv (src/warp/warpDeriv.F90:1-131): dXs = (dXv/dXs)^T dXv, using the
// denominator of the last orc_warp call.
static int warp_deriv_impl(Ctx *c, const double *dXv, double *dXs, long long j0, long long j1) {
    Tree &tp = c->tp;
    Nodal<double> nd;
    compute_nodal_properties(*c, c->Xs.data(), false, nd);
    tp.Ldef = tp.Ldef0 * c->o.LdefFact;
    tp.alphaToBexp = std::pow(c->o.alpha, c->o.bExp);
    tp.errTol = c->o.errTol;
    int nth = 1;
#ifdef _OPENMP
    nth = omp_get_max_threads();
#endif
    std::vector<Adj> ads(nth);
#pragma omp parallel
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        Adj &ad = ads[t];
        ad.init(tp.n, tp.nodes.size());
#pragma omp for schedule(dynamic, 64)
        for (long long j = j0; j < j1; ++j) {
            for (int kk = 1; kk <= c->nLoop; ++kk) {
                double r[3];
                get_mirror_pt(*c, &c->Xv0[3 * j], r, kk);
                double oden = 1.0 / c->denom[j];
                double numb[3] = {dXv[3 * j] * oden, dXv[3 * j + 1] * oden, dXv[3 * j + 2] * oden};
                get_mirror_numerator_b(*c, numb, kk);
                if (c->o.evalMode == 0)
                    eval_node_exact_b(tp, tp.nodes[tp.root], r, numb, ad);
                else
                    eval_node_b(tp, tp.root, r, numb, c->den0[j], ad);
            }
        }
    }
    Adj &ad = ads[0];
    for (int t = 1; t < nth; ++t) {
        for (size_t i = 0; i < ad.Bib.size(); ++i) ad.Bib[i] += ads[t].Bib[i];
        for (size_t i = 0; i < ad.Mib.size(); ++i) ad.Mib[i] += ads[t].Mib[i];
        for (size_t i = 0; i < ad.nBib.size(); ++i) ad.nBib[i] += ads[t].nBib[i];
        for (size_t i = 0; i < ad.nMib.size(); ++i) ad.nMib[i] += ads[t].nMib[i];
    }
    set_data_b(tp, ad);
    std::fill(dXs, dXs + 3 * c->nPts, 0.0);
    compute_nodal_properties_b(*c, nd, ad.Bib, ad.Mib, dXs);
    return 0;
}

extern "C" {

int orc_warp_deriv(void *h, const double *dXv, double *dXs) {
    Ctx *c = (Ctx *)h;
    if (!c->haveTree) return -4;
    if (!c->haveDenom) return -5;
    return warp_deriv_impl(c, dXv, dXs, 0, c->nVol);
}

int orc_warp_deriv_range(void *h, const double *dXv, double *dXs, long long j0, long long j1) {
    Ctx *c = (Ctx *)h;
    if (!c->haveTree) return -4;
    if (!c->haveDenom) return -5;
    return warp_deriv_impl(c, dXv, dXs, j0, j1);
}

// warpDerivFwd (src/warp/warpDerivFwd.F90:1-111): dXv = (dXv/dXs) dXs.  The
// oracle obtains the tangent by complex step through the templated forward
// code (same piecewise semantics as src/adjoint/outputForward/*.f90), scaled
// by the denominator of the last orc_warp call as warpDerivFwd.F90:101-106.
int orc_warp_deriv_fwd(void *h, const double *dXs, double *dXv) {
    Ctx *c = (Ctx *)h;
    if (!c->haveTree) return -4;
    if (!c->haveDenom) return -5;
    const double hstep = 1e-40;
    std::vector<double> im(3 * c->nPts), xr(3 * c->nVol), xi(3 * c->nVol);
    for (int i = 0; i < 3 * c->nPts; ++i) im[i] = hstep * dXs[i];
    orc_warp_complex(h, c->Xs.data(), im.data(), xr.data(), xi.data());
    // Xv = Xv0 + num/den(current) -> imag(Xv)/h = numd / den(current); the
    // reference divides by the stored denominator, identical here because
    // the current and stored denominators come from the same surface.
    for (long long i = 0; i < 3 * c->nVol; ++i) dXv[i] = xi[i] / hstep;
    return 0;
}

// ---- accessors used by the tests ----
int orc_sizes(void *h, long long *out) {
    Ctx *c = (Ctx *)h;
    out[0] = c->tp.n;
    out[1] = (long long)c->tp.nodes.size();
    out[2] = c->tp.maxDepth;
    out[3] = c->nVol;
    out[4] = c->nPts;
    out[5] = c->nLoop;
    out[6] = (long long)c->tp.facePtr.size() - 1;
    return 0;
}

double orc_ldef0(void *h) { return ((Ctx *)h)->tp.Ldef0; }

// Tree nodes in preorder (root first, left subtree, right subtree).
int orc_get_tree(void *h, int *lu /*4 per node: l,u,dnum,escape*/, double *geom /*4: X,oradius*/, double *ai,
                 double *err /*12*/) {
    Ctx *c = (Ctx *)h;
    Tree &tp = c->tp;
    // preorder numbering
    std::vector<int> order;
    std::vector<int> stack{tp.root};
    while (!stack.empty()) {
        int q = stack.back();
        stack.pop_back();
        order.push_back(q);
        if (tp.nodes[q].dnum != 0) {
            stack.push_back(tp.nodes[q].right);
            stack.push_back(tp.nodes[q].left);
        }
    }
    std::vector<int> pre(tp.nodes.size());
    for (size_t i = 0; i < order.size(); ++i) pre[order[i]] = int(i);
    // escape index = preorder index after the subtree
    std::vector<int> subtreeSize(tp.nodes.size(), 1);
    for (int i = int(order.size()) - 1; i >= 0; --i) {
        const Node &nd = tp.nodes[order[i]];
        if (nd.dnum != 0) subtreeSize[order[i]] = 1 + subtreeSize[nd.left] + subtreeSize[nd.right];
    }
    for (size_t i = 0; i < order.size(); ++i) {
        const Node &nd = tp.nodes[order[i]];
        lu[4 * i + 0] = nd.l;
        lu[4 * i + 1] = nd.u;
        lu[4 * i + 2] = nd.dnum;
        lu[4 * i + 3] = int(i) + subtreeSize[order[i]];
        for (int k = 0; k < 3; ++k) geom[4 * i + k] = nd.X[k];
        geom[4 * i + 3] = nd.oradius;
        ai[i] = nd.Ai;
        for (int e = 0; e < kNerr; ++e) err[kNerr * i + e] = nd.err[e];
    }
    return 0;
}

int orc_get_surface(void *h, double *xu0, double *ai, double *normals0, int *isCorner, int *xuInd) {
    Ctx *c = (Ctx *)h;
    Tree &tp = c->tp;
    for (int i = 0; i < tp.n; ++i) {
        for (int k = 0; k < 3; ++k) {
            xu0[3 * i + k] = tp.Xu0[3 * i + k];
            normals0[3 * i + k] = tp.normals0[3 * i + k];
        }
        ai[i] = tp.Ai[i];
        isCorner[i] = tp.isCorner[i];
        xuInd[i] = tp.XuInd[i];
    }
    return 0;
}

int orc_get_den0(void *h, double *den0) {
    Ctx *c = (Ctx *)h;
    std::memcpy(den0, c->den0.data(), sizeof(double) * c->nVol);
    return 0;
}

int orc_get_denom(void *h, double *den) {
    Ctx *c = (Ctx *)h;
    std::memcpy(den, c->denom.data(), sizeof(double) * c->nVol);
    return 0;
}

int orc_get_nodal(void *h, double *Mi, double *Bi) {
    Ctx *c = (Ctx *)h;
    Nodal<double> nd;
    compute_nodal_properties(*c, c->Xs.data(), false, nd);
    std::memcpy(Mi, nd.Mi.data(), sizeof(double) * 9 * c->tp.n);
    std::memcpy(Bi, nd.Bi.data(), sizeof(double) * 3 * c->tp.n);
    return 0;
}

int orc_stats(void *h, long long *out) {
    Ctx *c = (Ctx *)h;
    out[0] = c->st.leafPairs;
    out[1] = c->st.approx;
    out[2] = c->st.visited;
    return 0;
}

// dryRun cost of every volume node (kd_tree.F90:789-830 as driven by
// initializeWarping.F90:258-266), cost/n per node.
int orc_dry_run(void *h, double *costs) {
    Ctx *c = (Ctx *)h;
    Tree &tp = c->tp;
    for (long long j = 0; j < c->nVol; ++j) {
        double acc = 0;
        for (int kk = 1; kk <= c->nLoop; ++kk) {
            double r[3], cst = 0;
            get_mirror_pt(*c, &c->Xv0[3 * j], r, kk);
            dry_run(tp, tp.root, r, c->den0[j], cst);
            acc += cst / tp.n;
        }
        costs[j] = acc;
    }
    return 0;
}

}  // extern "C"
