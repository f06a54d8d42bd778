// C ABI of the GB300 IDW warping library (declared in include/idwarp_gb300.h).
// One context per mesh instance owns all device state of that mesh.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "idwarp_gb300.h"
#include "idw_host.hpp"
#include "idw_cplx.cuh"
#include "idw_kernels.h"
#include "idw_land.cuh"

using namespace idw;

namespace {

template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count) {
        if (p && count <= n) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&p), std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
};

struct Ctx {
    int device = 0;
    idw_options opt{};      // options now in force
    idw_options optInit{};  // options at the last initialize (tree/error-table constants)
    cudaStream_t stream = nullptr;
    std::string err;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // volume
    int64_t nVol = 0;
    bool haveVolume = false;
    DevBuf<double> xv0, xv, den0, den;
    DevBuf<int> perm;
    // symmetry
    SymPlanes sym{};
    // surface
    int nPts = 0, nUnique = 0, nFaces = 0;
    DevBuf<double> xs, xu, normals0, ptMB, tmpAi;
    DevBuf<dbl4> ptXA;
    DevBuf<int> xuInd, facePtr, faceConn, n2ePtr, n2e, isCorner;
    DevBuf<double> faceScratch;  // per face: area, normal and their adjoints (nodal kernels)
    // tree
    int nNodes = 0, maxDepth = 0;
    double Ldef0 = 0.0;
    DevBuf<int4> info;
    DevBuf<dbl4> geom;
    DevBuf<double> nodeErr, nodeAi, nodeMB, nodeSum;
    DevBuf<int> parent;
    DevBuf<unsigned> nodeFlags;
    bool haveTree = false, haveWarp = false, nodalValid = false;
    bool den0Valid = false;  // denominator estimate and walk records (computed at the first walk, or loaded)
    // FP32 companion arrays of the mixed-precision walk
    DevBuf<NodeRecF> nodeRec;
    DevBuf<int4> leafList;  // leaves in preorder (exact-mode kernel)
    int nLeaves = 0;
    DevBuf<float4> ptDA, ptDL;
    DevBuf<float4> recHi, recLo, acc;  // per-volume-node walk records and accumulators
    DevBuf<float> gden;                // per node: scaled denominator of a mixed walk (precision gate)
    // per-surface state of the batched mixed walk (grown on demand)
    int batchCap = 0;
    DevBuf<double> bXs, bXu, bPtMB, bNodeMB;
    DevBuf<float> bPtDM, bPtDMl, bNodeDC, bNodeDCl, bNodeDn, bRef;
    DevBuf<float4> bAcc;
    // tuned launch shapes (idw_autotune)
    int batchGroup = kBatchMax;  // surfaces per batched walk
    int adjMaxGroup = 16;        // seeds per adjoint walk
    // warpDeriv accumulators (grown on demand)
    int adjSeeds = 0;
    DevBuf<double> adjPt, adjNode, adjRel;
    // order-independent landings (option deterministic): per accumulator
    // element an exponent and a 192-bit fixed-point sum
    DevBuf<int> landExpo;
    DevBuf<unsigned long long> landFix;
    bool gdenValid = false;
    double gdenLdefFact = 0.0, gdenAlpha = 0.0;
    int gdenMode = -1;
    // the precise adjoint's denominator (double-float weights), per law and mode
    DevBuf<double> denP;
    bool denPValid = false;
    double denPLdefFact = 0.0, denPAlpha = 0.0;
    int denPMode = -1;
    DevBuf<float> ptDM, ptDMl, nodeDC, nodeDCl, nodeDn, refDB;
    DevBuf<float4> replayRec;  // NodeAggF::rr: 8 float4 per tree node
    // recorded decisions of the fast walk (idw_replay.cu), valid for the
    // current den0 and listErrTol; listState 1 = recorded, -1 = too large
    // (the walks decide as they go), 0 = not yet recorded
    DevBuf<int64_t> walkOffs;
    DevBuf<int2> walkList;
    DevBuf<unsigned long long> walkCnt;
    int listState = 0;
    double listErrTol = 0.0;
    int64_t listEntries = 0;
    // adjoint
    DevBuf<double> ptAdj, nodeAdj, xub, dxs;
    bool haveDxs = false;
    // complex step: interleaved complex surface coordinates, the imaginary
    // parts of the nodal properties and of the warped grid
    DevBuf<double> xsC, ptMBim, nodeMBim, xvIm;
    DevBuf<cplx> xuC;
    bool haveCs = false;
    // solver ordering
    DevBuf<int> solverInd;
    int64_t nSolver = -1;
    // asynchronous reads of the warped grid (idw_get_volume_coordinates_async):
    // a copy stream, the grid's second buffer, and per buffer the event that
    // ends its last read (a warp writes the other buffer while a read of the
    // current one may still run)
    cudaStream_t copyStream = nullptr;
    cudaEvent_t evReady = nullptr;
    DevBuf<double> xvAlt;
    struct PendingRead {
        const double *p = nullptr;
        cudaEvent_t ev = nullptr;
        bool on = false;
    } rd[2];
    // misc
    DevBuf<unsigned long long> counters;
    bool eventsRecorded = false;
    idw_stats stats{};
};

int fail(Ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return fail(c, IDW_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define CKA(call)                                                                                         \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return fail(c, IDW_ERR_NOMEM, "allocation failed: %s", cudaGetErrorString(e_)); \
    } while (0)

int check_launch(Ctx *c, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, IDW_ERR_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
    return IDW_OK;
}

// Copy n doubles from a host or device pointer into device buffer dst.
int copy_in(Ctx *c, double *dst, const double *src, size_t n, int where) {
    if (n == 0) return IDW_OK;
    if (!src) return fail(c, IDW_ERR_ARG, "null input pointer");
    CK(cudaMemcpyAsync(dst, src, n * sizeof(double), where == IDW_DEVICE ? cudaMemcpyDeviceToDevice
                                                                           : cudaMemcpyHostToDevice,
                       c->stream));
    return IDW_OK;
}

int copy_out(Ctx *c, double *dst, const double *src, size_t n, int where) {
    if (n == 0) return IDW_OK;
    if (!dst) return fail(c, IDW_ERR_ARG, "null output pointer");
    CK(cudaMemcpyAsync(dst, src, n * sizeof(double), where == IDW_DEVICE ? cudaMemcpyDeviceToDevice
                                                                           : cudaMemcpyDeviceToHost,
                       c->stream));
    if (where != IDW_DEVICE) CK(cudaStreamSynchronize(c->stream));
    return IDW_OK;
}

WeightLaw make_law(const Ctx *c) {
    WeightLaw w{};
    // exponents are fixed at tree creation (kd_tree.F90:1529-1530); Ldef and
    // alpha^bExp are refreshed from the current options on every warp
    // (warpMesh.F90:39-40), using the current bExp for alpha^bExp.
    w.aExp = c->optInit.aExp;
    w.bExp = c->optInit.bExp;
    w.Ldef = c->Ldef0 * c->opt.LdefFact;
    w.alphaToBexp = std::pow(c->opt.alpha, c->opt.bExp);
    double ra = std::nearbyint(w.aExp), rb = std::nearbyint(w.bExp);
    w.isInt = (ra == w.aExp && rb == w.bExp && ra >= 0 && rb >= ra && rb <= 64);
    w.ia = int(ra);
    w.ib = int(rb);
    return w;
}

WeightLaw make_init_law(const Ctx *c) {
    WeightLaw w = make_law(c);
    w.Ldef = c->Ldef0 * c->optInit.LdefFact;
    w.alphaToBexp = std::pow(c->optInit.alpha, c->optInit.bExp);
    return w;
}

struct DevView {
    double *p;
};

TreeDev tree_dev(Ctx *c) {
    TreeDev t;
    t.nNodes = c->nNodes;
    t.info = c->info.p;
    t.geom = c->geom.p;
    t.err = c->nodeErr.p;
    t.ai = c->nodeAi.p;
    t.parent = c->parent.p;
    return t;
}

SetDataScratch setdata_scratch(Ctx *c) {
    SetDataScratch sc;
    sc.sum = c->nodeSum.p;
    sc.flags = c->nodeFlags.p;
    return sc;
}

SurfaceDev surf_dev(Ctx *c) {
    SurfaceDev s;
    s.n = c->nUnique;
    s.facePtr = c->facePtr.p;
    s.faceConn = c->faceConn.p;
    s.n2ePtr = c->n2ePtr.p;
    s.n2e = c->n2e.p;
    s.nFaces = c->nFaces;
    s.faceScratch = c->faceScratch.p;
    return s;
}

TreeDevF tree_devf(Ctx *c) {
    TreeDevF tf;
    tf.nodes = c->nodeRec.p;
    tf.leaves = c->leafList.p;
    tf.nLeaves = c->nLeaves;
    tf.nPts = c->nUnique;
    return tf;
}

VolumeDev vol_dev(Ctx *c) {
    VolumeDev v;
    v.nVol = c->nVol;
    v.perm = c->perm.p;
    v.xv0 = c->xv0.p;
    v.den0 = c->den0.p;
    return v;
}

int validate_options(Ctx *c, const idw_options *o) {
    if (!o) return fail(c, IDW_ERR_ARG, "null options");
    if (o->evalMode != IDW_EVAL_EXACT && o->evalMode != IDW_EVAL_FAST)
        return fail(c, IDW_ERR_ARG, "evalMode must be IDW_EVAL_EXACT or IDW_EVAL_FAST");
    if (o->precision != IDW_PREC_FP64 && o->precision != IDW_PREC_MIXED)
        return fail(c, IDW_ERR_ARG, "precision must be IDW_PREC_FP64 or IDW_PREC_MIXED");
    if (o->bucketSize < 1) return fail(c, IDW_ERR_ARG, "bucketSize must be >= 1");
    if (!(o->LdefFact > 0.0)) return fail(c, IDW_ERR_ARG, "LdefFact must be > 0");
    if (!(o->mixedGate >= 0.0)) return fail(c, IDW_ERR_ARG, "mixedGate must be >= 0");
    if (o->exactSchedule < IDW_EXACT_AUTO || o->exactSchedule > IDW_EXACT_WALK)
        return fail(c, IDW_ERR_ARG, "exactSchedule must be IDW_EXACT_AUTO, IDW_EXACT_TILED or IDW_EXACT_WALK");
    if (o->adjointPrecision != IDW_ADJ_PRECISE && o->adjointPrecision != IDW_ADJ_FAST)
        return fail(c, IDW_ERR_ARG, "adjointPrecision must be IDW_ADJ_PRECISE or IDW_ADJ_FAST");
    if (o->walkLists != IDW_WALK_LISTS_AUTO && o->walkLists != IDW_WALK_LISTS_OFF)
        return fail(c, IDW_ERR_ARG, "walkLists must be IDW_WALK_LISTS_AUTO or IDW_WALK_LISTS_OFF");
    if (o->treeBuild != IDW_TREE_KD && o->treeBuild != IDW_TREE_MORTON)
        return fail(c, IDW_ERR_ARG, "treeBuild must be IDW_TREE_KD or IDW_TREE_MORTON");
    if (o->deterministic != 0 && o->deterministic != 1) return fail(c, IDW_ERR_ARG, "deterministic must be 0 or 1");
    return IDW_OK;
}

// Per-warp nodal properties and cluster aggregates of the current surface.
int refresh_nodal(Ctx *c) {
    SurfaceDev s = surf_dev(c);
    launch_gather_xu(c->nUnique, c->xuInd.p, c->xs.p, c->xu.p, c->stream);
    launch_nodal(s, c->xu.p, c->ptXA.p, c->normals0.p, c->tmpAi.p, c->isCorner.p, c->opt.useRotations, c->ptMB.p,
                 c->stream);
    launch_set_data(tree_dev(c), c->ptMB.p, c->nodeMB.p, setdata_scratch(c), c->stream);
    if (c->opt.precision == IDW_PREC_MIXED) {
        launch_mixed_nodal(c->nUnique, tree_dev(c), c->nodeMB.p, c->ptXA.p, c->ptMB.p, c->ptDM.p, c->ptDMl.p,
                           c->stream);
        launch_mixed_nodes(tree_dev(c), c->nodeMB.p, c->ptMB.p, c->nodeDC.p, c->nodeDCl.p, c->nodeDn.p, c->refDB.p,
                           c->stream);
        launch_replay_records(c->nNodes, c->nodeDC.p, c->nodeDn.p, c->replayRec.p, c->stream);
    }
    c->nodalValid = true;
    return check_launch(c, "nodal properties");
}

// Walk records of every volume node from the denominator estimate in den0.
int finish_den0(Ctx *c) {
    launch_walk_records(vol_dev(c), c->sym, c->optInit.bExp, c->recHi.p, c->recLo.p, c->stream);
    int e = check_launch(c, "walk records");
    if (e) return e;
    c->gdenValid = false;
    c->denPValid = false;
    c->listState = 0;
    c->den0Valid = true;
    return IDW_OK;
}

// The denominator estimate over the mirrors (initializeWarping.F90:241-247),
// unless it was computed or loaded since the last initialize.
int ensure_den0(Ctx *c) {
    if (c->den0Valid) return IDW_OK;
    CK(cudaSetDevice(c->device));
    launch_denominator0(tree_dev(c), c->nodeRec.p, c->ptXA.p, vol_dev(c), make_init_law(c), c->sym, c->den0.p, c->stream);
    int e = check_launch(c, "denominator0");
    if (e) return e;
    return finish_den0(c);
}

bool all_finite(const double *v, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

}  // namespace

extern "C" {

void idw_default_options(idw_options *o) {
    std::memset(o, 0, sizeof(*o));
    o->aExp = 3.0;
    o->bExp = 5.0;
    o->LdefFact = 1.0;
    o->alpha = 0.25;
    o->errTol = 0.0005;
    o->symmTol = 1e-6;
    o->cornerAngle = 30.0;
    o->evalMode = IDW_EVAL_FAST;
    o->useRotations = 1;
    o->zeroCornerRotations = 1;
    o->bucketSize = 8;
    o->precision = IDW_PREC_MIXED;
    o->diagnostics = 0;
    o->mixedGate = 2e-3;
    o->adjointPrecision = IDW_ADJ_PRECISE;
    o->walkLists = IDW_WALK_LISTS_AUTO;
    o->treeBuild = IDW_TREE_KD;
}

int idw_create(const idw_options *opts, void **ctx_out) {
    if (!ctx_out) return IDW_ERR_ARG;
    *ctx_out = nullptr;
    Ctx *c = new Ctx();
    idw_default_options(&c->opt);
    if (opts) {
        int rc = validate_options(c, opts);
        if (rc) {
            delete c;
            return rc;
        }
        c->opt = *opts;
    }
    c->optInit = c->opt;
    if (cudaGetDevice(&c->device) != cudaSuccess) {
        delete c;
        return IDW_ERR_CUDA;
    }
    if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
        delete c;
        return IDW_ERR_CUDA;
    }
    c->sym.n = 0;
    c->sym.nLoop = 1;
    if (c->counters.alloc(8) != cudaSuccess) {
        delete c;
        return IDW_ERR_NOMEM;
    }
    *ctx_out = c;
    return IDW_OK;
}

int idw_destroy(void *ctx) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->copyStream) {
        cudaStreamSynchronize(c->copyStream);
        cudaStreamDestroy(c->copyStream);
    }
    if (c->evReady) cudaEventDestroy(c->evReady);
    for (auto &r : c->rd)
        if (r.ev) cudaEventDestroy(r.ev);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    delete c;
    return IDW_OK;
}

int idw_last_error(void *ctx, char *buf, int len) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c || !buf || len <= 0) return IDW_ERR_ARG;
    std::snprintf(buf, size_t(len), "%s", c->err.c_str());
    return IDW_OK;
}

int idw_set_stream(void *ctx, void *stream) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    c->stream = static_cast<cudaStream_t>(stream);
    return IDW_OK;
}

int idw_synchronize(void *ctx) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    CK(cudaStreamSynchronize(c->stream));
    if (c->copyStream) CK(cudaStreamSynchronize(c->copyStream));
    return IDW_OK;
}

int idw_set_options(void *ctx, const idw_options *opts) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    int rc = validate_options(c, opts);
    if (rc) return rc;
    if (opts->useRotations != c->opt.useRotations || opts->precision != c->opt.precision) c->nodalValid = false;
    c->opt = *opts;
    return IDW_OK;
}

int idw_create_common_grid(void *ctx, const double *volnodes, int64_t nvol, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (nvol < 0 || nvol > (int64_t(1) << 31) - 1) return fail(c, IDW_ERR_ARG, "nvol out of range: %lld", (long long)nvol);
    CK(cudaSetDevice(c->device));
    // a new grid: asynchronous reads of the old one end first
    if (c->copyStream) CK(cudaStreamSynchronize(c->copyStream));
    for (auto &r : c->rd) {
        r.on = false;
        r.p = nullptr;
    }
    c->xvAlt.release();
    c->nVol = nvol;
    CKA(c->xv0.alloc(3 * nvol));
    CKA(c->xv.alloc(3 * nvol));
    CKA(c->den0.alloc(nvol));
    CKA(c->den.alloc(nvol));
    CKA(c->perm.alloc(nvol));
    int rc = copy_in(c, c->xv0.p, volnodes, 3 * size_t(nvol), where);
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->xv.p, c->xv0.p, 3 * nvol * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    // bounding box and finiteness on the device (set-up only)
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (nvol > 0) {
        int64_t nonFinite = 0;
        if (volume_bbox(nvol, c->xv0.p, lo, hi, &nonFinite, c->stream))
            return fail(c, IDW_ERR_CUDA, "volume bounding box failed");
        if (nonFinite) return fail(c, IDW_ERR_NONFINITE, "non-finite volume coordinates");
        DevBuf<unsigned long long> codes, codesAlt;
        DevBuf<int> idx;
        CKA(codes.alloc(nvol));
        CKA(codesAlt.alloc(nvol));
        CKA(idx.alloc(nvol));
        launch_morton_codes(nvol, c->xv0.p, lo, hi, codes.p, idx.p, c->stream);
        if (sort_morton(nvol, codes.p, idx.p, codesAlt.p, c->perm.p, c->stream))
            return fail(c, IDW_ERR_NOMEM, "Morton sort failed");
        int e = check_launch(c, "morton");
        if (e) return e;
    }
    c->haveVolume = true;
    // a new volume needs a new initialize (records and estimates are per node)
    c->haveTree = false;
    c->listState = 0;
    c->den0Valid = false;
    c->haveWarp = false;
    c->haveDxs = false;
    c->stats.nVol = nvol;
    return IDW_OK;
}

int idw_set_symmetry_planes(void *ctx, const double *pts, const double *normals, int32_t n) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (n < 0 || n > kMaxSym) return fail(c, IDW_ERR_LIMIT, "at most %d symmetry planes are supported", kMaxSym);
    if (n > 0 && (!pts || !normals)) return fail(c, IDW_ERR_ARG, "null symmetry arrays");
    c->sym.n = n;
    c->sym.nLoop = 1 << n;
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < 3; ++k) {
            c->sym.p[j][k] = pts[3 * j + k];
            c->sym.nrm[j][k] = normals[3 * j + k];
        }
    c->stats.nLoop = c->sym.nLoop;
    return IDW_OK;
}

int idw_point_reduce(const double *pts, int32_t n, double tol, double *uniquepts, int32_t *link, int32_t *nunique) {
    if (n < 0 || !nunique || (n > 0 && (!pts || !uniquepts || !link))) return IDW_ERR_ARG;
    *nunique = point_reduce(pts, n, tol, uniquepts, link);
    return IDW_OK;
}

int idw_initialize_warping(void *ctx, const double *pts, int32_t npts, const double *uniquepts, int32_t nunique,
                           const int32_t *link, const int32_t *faceSizes, int32_t nfaces, const int32_t *faceConn,
                           int32_t nconn) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    CK(cudaSetDevice(c->device));
    if (!c->haveVolume) return fail(c, IDW_ERR_STATE, "the volume grid must be set before the surface definition");
    if (nunique < 1 || npts < 1) return fail(c, IDW_ERR_ARG, "empty surface (npts=%d, nunique=%d)", npts, nunique);
    if (!pts || !uniquepts || !link || !faceSizes || !faceConn) return fail(c, IDW_ERR_ARG, "null surface array");
    if (!all_finite(pts, 3 * size_t(npts)) || !all_finite(uniquepts, 3 * size_t(nunique)))
        return fail(c, IDW_ERR_NONFINITE, "non-finite surface coordinates");
    std::vector<int> fptr(nfaces + 1, 0);
    for (int f = 0; f < nfaces; ++f) {
        if (faceSizes[f] < 1 || faceSizes[f] > kMaxFacePts)
            return fail(c, IDW_ERR_LIMIT, "face %d has %d points (supported: 1..%d)", f, faceSizes[f], kMaxFacePts);
        fptr[f + 1] = fptr[f] + faceSizes[f];
    }
    if (fptr[nfaces] != nconn) return fail(c, IDW_ERR_ARG, "sum(faceSizes)=%d != len(conn)=%d", fptr[nfaces], nconn);
    for (int i = 0; i < npts; ++i)
        if (link[i] < 1 || link[i] > nunique) return fail(c, IDW_ERR_ARG, "link[%d]=%d out of range", i, link[i]);
    for (int i = 0; i < nconn; ++i)
        if (faceConn[i] < 0 || faceConn[i] >= npts) return fail(c, IDW_ERR_ARG, "conn[%d]=%d out of range", i, faceConn[i]);
    c->optInit = c->opt;
    c->haveTree = c->haveWarp = c->haveDxs = c->nodalValid = false;

    FlatTree t;
    const auto tTree = std::chrono::steady_clock::now();
    if (c->opt.treeBuild == IDW_TREE_MORTON) {
        const int rc = build_morton_tree(uniquepts, nunique, c->opt.bucketSize, t, c->stream);
        if (rc == -2) return fail(c, IDW_ERR_NOMEM, "out of device memory in the surface tree build");
        if (rc == -3) return fail(c, IDW_ERR_LIMIT, "the Morton tree takes at most 2^30 unique surface points");
        if (rc != 0) return fail(c, IDW_ERR_CUDA, "surface tree build: %s", cudaGetErrorString(cudaGetLastError()));
    } else {
        build_kdtree(uniquepts, nunique, c->opt.bucketSize, t);
    }
    const double treeMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tTree).count();
    const int n = nunique, nn = t.nodes();
    std::vector<int> inv(n);
    for (int i = 0; i < n; ++i) inv[t.perm[i]] = i;
    std::vector<dbl4> xa(n);
    for (int i = 0; i < n; ++i) {
        const double *q = uniquepts + 3 * t.perm[i];
        xa[i] = mk_dbl4(q[0], q[1], q[2], 0.0);
    }
    std::vector<int> tconn(nconn);
    for (int i = 0; i < nconn; ++i) tconn[i] = inv[link[faceConn[i]] - 1];
    std::vector<int> cnt(n + 1, 0);
    for (int i = 0; i < nconn; ++i) cnt[tconn[i] + 1]++;
    for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    std::vector<int> n2e(nconn), fill(cnt.begin(), cnt.end() - 1);
    for (int f = 0; f < nfaces; ++f)
        for (int j = fptr[f]; j < fptr[f + 1]; ++j) n2e[fill[tconn[j]]++] = f;
    std::vector<int> xuInd(n, -1);
    for (int i = 0; i < npts; ++i) {
        int q = inv[link[i] - 1];
        if (xuInd[q] < 0) xuInd[q] = i;
    }
    // Ldef0: largest distance from the centroid (kd_tree.F90:1500-1512)
    double cen[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i) {
        cen[0] += xa[i].x;
        cen[1] += xa[i].y;
        cen[2] += xa[i].z;
    }
    for (int k = 0; k < 3; ++k) cen[k] = cen[k] / n;
    double L0 = 0.0;
    for (int i = 0; i < n; ++i) {
        const double *q = uniquepts + 3 * i;
        double dx = q[0] - cen[0], dy = q[1] - cen[1], dz = q[2] - cen[2];
        L0 = std::max(L0, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    c->Ldef0 = L0;
    c->nPts = npts;
    c->nUnique = n;
    c->nFaces = nfaces;
    c->nNodes = nn;
    c->maxDepth = t.maxDepth;
    // device arrays
    CKA(c->xs.alloc(3 * size_t(npts)));
    CKA(c->dxs.alloc(3 * size_t(npts)));
    CKA(c->xu.alloc(3 * size_t(n)));
    CKA(c->xub.alloc(3 * size_t(n)));
    CKA(c->normals0.alloc(3 * size_t(n)));
    CKA(c->tmpAi.alloc(n));
    CKA(c->ptMB.alloc(12 * size_t(n)));
    CKA(c->ptAdj.alloc(12 * size_t(n)));
    CKA(c->ptXA.alloc(n));
    CKA(c->xuInd.alloc(n));
    CKA(c->isCorner.alloc(n));
    CKA(c->facePtr.alloc(nfaces + 1));
    CKA(c->faceScratch.alloc(8 * size_t(std::max(nfaces, 1))));
    CKA(c->faceConn.alloc(std::max(nconn, 1)));
    CKA(c->n2ePtr.alloc(n + 1));
    CKA(c->n2e.alloc(std::max(nconn, 1)));
    CKA(c->info.alloc(nn));
    CKA(c->geom.alloc(nn));
    CKA(c->nodeErr.alloc(kNerr * size_t(nn)));
    CKA(c->nodeAi.alloc(nn));
    CKA(c->nodeMB.alloc(12 * size_t(nn)));
    CKA(c->nodeSum.alloc(12 * size_t(nn)));
    CKA(c->nodeFlags.alloc(size_t(nn)));
    CKA(c->parent.alloc(size_t(nn)));
    CKA(c->nodeAdj.alloc(12 * size_t(nn)));
    CKA(c->nodeRec.alloc(nn));
    CKA(c->nodeDC.alloc(12 * size_t(nn)));
    CKA(c->nodeDCl.alloc(12 * size_t(nn)));
    CKA(c->nodeDn.alloc(nn));
    CKA(c->refDB.alloc(24));
    CKA(c->ptDA.alloc(n));
    CKA(c->ptDL.alloc(n));
    CKA(c->ptDM.alloc(12 * size_t(n)));
    CKA(c->ptDMl.alloc(12 * size_t(n)));
    cudaStream_t st = c->stream;
    CK(cudaMemcpyAsync(c->xs.p, pts, 3 * sizeof(double) * npts, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->xuInd.p, xuInd.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->facePtr.p, fptr.data(), sizeof(int) * (nfaces + 1), cudaMemcpyHostToDevice, st));
    if (nconn > 0) {
        CK(cudaMemcpyAsync(c->faceConn.p, tconn.data(), sizeof(int) * nconn, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(c->n2e.p, n2e.data(), sizeof(int) * nconn, cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemcpyAsync(c->n2ePtr.p, cnt.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st));
    std::vector<int4> info(nn);
    std::vector<dbl4> geom(nn);
    for (int k = 0; k < nn; ++k) {
        info[k] = make_int4(t.l[k], t.u[k], t.escape[k], t.leaf[k]);
        geom[k] = mk_dbl4(t.X[3 * k], t.X[3 * k + 1], t.X[3 * k + 2], t.oradius[k]);
    }
    CK(cudaMemcpyAsync(c->info.p, info.data(), sizeof(int4) * nn, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->geom.p, geom.data(), sizeof(dbl4) * nn, cudaMemcpyHostToDevice, st));
    std::vector<int4> leaves;
    for (int k = 0; k < nn; ++k)
        if (t.leaf[k]) leaves.push_back(make_int4(t.l[k], t.u[k], k, 0));
    c->nLeaves = int(leaves.size());
    CKA(c->leafList.alloc(leaves.size()));
    if (!leaves.empty())
        CK(cudaMemcpyAsync(c->leafList.p, leaves.data(), sizeof(int4) * leaves.size(), cudaMemcpyHostToDevice, st));
    launch_tree_parents(tree_dev(c), c->parent.p, st);
    // initial nodal properties: normals0, Ai, corners (kd_tree.F90:1547-1578)
    SurfaceDev s = surf_dev(c);
    launch_gather_xu(n, c->xuInd.p, c->xs.p, c->xu.p, st);
    launch_nodal_init(s, c->xu.p, c->normals0.p, c->tmpAi.p, st);
    double thr = std::cos(c->opt.cornerAngle * 3.1415926535897931 / 180.0);
    launch_corners(s, c->xu.p, c->normals0.p, thr, c->opt.zeroCornerRotations, c->isCorner.p, st);
    int e = check_launch(c, "nodal init");
    if (e) return e;
    std::vector<double> ai(n), nodeAi(nn, 0.0);
    CK(cudaMemcpyAsync(ai.data(), c->tmpAi.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    // setAi: leaf sums in range order, interior = left + right (kd_tree.F90:536-556)
    for (int k = nn - 1; k >= 0; --k) {
        if (t.leaf[k]) {
            double a = 0.0;
            for (int i = t.l[k]; i <= t.u[k]; ++i) a = a + ai[i];
            nodeAi[k] = a;
        } else {
            nodeAi[k] = nodeAi[k + 1] + nodeAi[t.escape[k + 1]];
        }
    }
    for (int i = 0; i < n; ++i) xa[i].w = ai[i];
    CK(cudaMemcpyAsync(c->ptXA.p, xa.data(), sizeof(dbl4) * n, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->nodeAi.p, nodeAi.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, st));
    // error tables (kd_tree.F90:1528-1544) with the creation-time law
    WeightLaw law0 = make_init_law(c);
    {
        const int rc = launch_compute_errors(tree_dev(c), c->ptXA.p, law0, c->nodeErr.p, st);
        if (rc == -2) return fail(c, IDW_ERR_NOMEM, "computeErrors: scratch allocation failed");
        if (rc) return fail(c, IDW_ERR_CUDA, "computeErrors: %s", cudaGetErrorString(cudaGetLastError()));
    }
    e = check_launch(c, "computeErrors");
    if (e) return e;
    // FP32 companions: node records (split centroid, radius, area, error
    // table) and leaf-relative point offsets
    {
        std::vector<double> errH(kNerr * size_t(nn));
        CK(cudaMemcpyAsync(errH.data(), c->nodeErr.p, sizeof(double) * kNerr * nn, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        std::vector<NodeRecF> recs(nn);
        std::vector<float4> da(n), dl(n);
        for (int k = 0; k < nn; ++k) {
            NodeRecF &r = recs[k];
            std::memset(&r, 0, sizeof(r));
            r.info = info[k];
            float h[3], l[3];
            for (int q = 0; q < 3; ++q) {
                h[q] = float(t.X[3 * k + q]);
                l[q] = float(t.X[3 * k + q] - double(h[q]));
            }
            r.cHi = make_float4(h[0], h[1], h[2], float(t.oradius[k]));
            r.cLo = make_float4(l[0], l[1], l[2], float(nodeAi[k]));
            r.aLo = float(nodeAi[k] - double(float(nodeAi[k])));
            for (int e2 = 0; e2 < kNerr; ++e2) r.err[e2] = float(errH[kNerr * size_t(k) + e2]);
            if (t.leaf[k]) {
                for (int i = t.l[k]; i <= t.u[k]; ++i) {
                    const double d[3] = {xa[i].x - t.X[3 * k], xa[i].y - t.X[3 * k + 1], xa[i].z - t.X[3 * k + 2]};
                    float dh[3], dlo[3];
                    for (int q = 0; q < 3; ++q) {
                        dh[q] = float(d[q]);
                        dlo[q] = float(d[q] - double(dh[q]));
                    }
                    da[i] = make_float4(dh[0], dh[1], dh[2], float(ai[i]));
                    dl[i] = make_float4(dlo[0], dlo[1], dlo[2], float(ai[i] - double(float(ai[i]))));
                }
            }
        }
        CK(cudaMemcpyAsync(c->nodeRec.p, recs.data(), sizeof(NodeRecF) * nn, cudaMemcpyHostToDevice, st));
        // static fields of the replay records; dn and dc follow per surface
        {
            std::vector<float4> rr(8 * size_t(nn), make_float4(0.f, 0.f, 0.f, 0.f));
            const auto bits = [](int v) {
                float f;
                std::memcpy(&f, &v, sizeof(f));
                return f;
            };
            for (int k = 0; k < nn; ++k) {
                float4 *r = rr.data() + 8 * size_t(k);
                r[0] = make_float4(recs[k].cHi.x, recs[k].cHi.y, recs[k].cHi.z, 0.f);
                r[1] = recs[k].cLo;
                if (t.leaf[k]) {
                    r[1].w = bits(t.l[k]);
                    r[2].x = bits(t.u[k]);
                    r[5].x = bits(1);
                }
            }
            CKA(c->replayRec.alloc(rr.size()));
            CK(cudaMemcpyAsync(c->replayRec.p, rr.data(), sizeof(float4) * rr.size(), cudaMemcpyHostToDevice, st));
        }
        CK(cudaMemcpyAsync(c->ptDA.p, da.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(c->ptDL.p, dl.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
    }
    // the denominator estimate and the walk records follow at the first walk
    // (ensure_den0), or come from idw_compute_denominator0 / idw_set_denominator0
    CKA(c->recHi.alloc(size_t(c->sym.nLoop) * c->nVol));
    CKA(c->recLo.alloc(size_t(c->sym.nLoop) * c->nVol));
    CKA(c->acc.alloc(2 * size_t(c->nVol)));
    CKA(c->gden.alloc(size_t(c->nVol)));
    c->gdenValid = false;
    c->denPValid = false;
    c->listState = 0;
    c->den0Valid = false;
    CK(cudaStreamSynchronize(st));
    c->haveTree = true;
    c->stats.nUnique = n;
    c->stats.nTreeNodes = nn;
    c->stats.maxDepth = t.maxDepth;
    c->stats.treeBuildMs = treeMs;
    c->stats.nSurfPts = npts;
    c->stats.nLoop = c->sym.nLoop;
    c->stats.Ldef0 = L0;
    return IDW_OK;
}

int idw_set_surface_coordinates(void *ctx, const double *coords, int64_t cdof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (cdof != 3 * int64_t(c->nPts))
        return fail(c, IDW_ERR_ARG, "incorrect length of coordinates: expected %lld, received %lld",
                    (long long)(3 * int64_t(c->nPts)), (long long)cdof);
    CK(cudaSetDevice(c->device));
    if (where != IDW_DEVICE && !all_finite(coords, size_t(cdof)))
        return fail(c, IDW_ERR_NONFINITE, "non-finite surface coordinates");
    int rc = copy_in(c, c->xs.p, coords, size_t(cdof), where);
    if (rc) return rc;
    if (where != IDW_DEVICE) CK(cudaStreamSynchronize(c->stream));
    c->nodalValid = false;
    c->haveCs = false;
    return IDW_OK;
}

int idw_get_surface_coordinates(void *ctx, double *coords, int64_t cdof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (cdof != 3 * int64_t(c->nPts)) return fail(c, IDW_ERR_ARG, "cdof mismatch");
    CK(cudaSetDevice(c->device));
    return copy_out(c, coords, c->xs.p, size_t(cdof), where);
}

// Threshold of the mixed walk's double-float terms: mixedGate * Ldef0 (the
// motions are lengths: Ldef0, not the weight law's LdefFact-scaled L),
// tightened beyond one symmetry plane, where every node sums nLoop mirror walks
// of FP32 terms.
static double mixed_gate(const Ctx *c) {
    return c->opt.mixedGate * c->Ldef0 * std::min(1.0, 2.0 / double(std::max(1, c->sym.nLoop)));
}

// The fast walk's decisions depend on set-up state and errTol only: record
// them once (count pass, offsets, record pass) and hand them to every later
// mixed walk in k.lists.  The lists take up to half of the free device memory;
// beyond that the walks keep deciding as they go.  Returns a status; k.lists
// stays null when the lists are off or do not fit.
static int ensure_walk_lists(Ctx *c, const TreeDevF &tf, const WalkRecF &rec, EvalConsts &k) {
    k.lists = WalkLists{};
    if (c->opt.precision != IDW_PREC_MIXED || c->opt.evalMode != IDW_EVAL_FAST ||
        c->opt.walkLists == IDW_WALK_LISTS_OFF || c->nVol <= 0 || k.slotStats)
        return IDW_OK;
    if (c->listState != 0 && c->listErrTol != c->opt.errTol) c->listState = 0;
    if (c->listState == 0) {
        c->walkList.release();
        const int64_t nOff = walk_list_warps(c->nVol) * c->sym.nLoop + 1;
        CKA(c->walkOffs.alloc(size_t(nOff)));
        CKA(c->walkCnt.alloc(8));
        const int64_t total = count_walk_lists(tree_dev(c), tf, vol_dev(c), rec, k, c->walkOffs.p, c->stream);
        if (total < 0) return fail(c, IDW_ERR_CUDA, "walk lists: count pass failed");
        size_t freeB = 0, totalB = 0;
        CK(cudaMemGetInfo(&freeB, &totalB));
        c->listErrTol = c->opt.errTol;
        c->listEntries = total;
        if (double(total) * sizeof(int2) > 0.5 * double(freeB)) {
            c->listState = -1;
            return IDW_OK;
        }
        CKA(c->walkList.alloc(size_t(std::max<int64_t>(total, 1))));
        CK(cudaMemsetAsync(c->walkCnt.p, 0, 8 * sizeof(unsigned long long), c->stream));
        launch_walk_record(tree_dev(c), tf, vol_dev(c), rec, k, c->walkOffs.p, c->walkList.p, c->walkCnt.p,
                           c->stream);
        int rc = check_launch(c, "walk lists");
        if (rc) return rc;
        c->listState = 1;
    }
    if (c->listState == 1) {
        k.lists.offs = c->walkOffs.p;
        k.lists.list = c->walkList.p;
        k.lists.counters = c->walkCnt.p;
    }
    return IDW_OK;
}

// The mixed walk's precision gate wants each node's final denominator, which
// depends on Xu0 and the weight law only (not on the surface coordinates):
// one walk that keeps only the denominators, run once per law.
static int ensure_gate_den(Ctx *c, const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af, const WalkRecF &rec,
                           const EvalConsts &k, int exact) {
    if (c->gdenValid && c->gdenLdefFact == c->opt.LdefFact && c->gdenAlpha == c->opt.alpha &&
        c->gdenMode == c->opt.evalMode)
        return IDW_OK;
    WalkOut none;
    EvalConsts k0 = k;
    k0.precGate = 3.0e38;  // FP32 terms only: a gate needs no more
    launch_walk_mixed(tree_dev(c), tf, pf, af, vol_dev(c), rec, k0, exact, c->acc.p, none, c->stream);
    launch_gate_den(c->nVol, c->acc.p, c->gden.p, c->stream);
    int rc = check_launch(c, "gate denominators");
    if (rc) return rc;
    CK(cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream));
    c->gdenValid = true;
    c->gdenLdefFact = c->opt.LdefFact;
    c->gdenAlpha = c->opt.alpha;
    c->gdenMode = c->opt.evalMode;
    return IDW_OK;
}

// Before the warped grid is overwritten: if an asynchronous read of the
// current grid may still run, the next grid goes to the other buffer; an
// older read of that buffer (one warp back) is waited for on the stream.
static int prepare_xv_write(Ctx *c) {
    for (auto &r : c->rd) {
        if (r.on && r.p == c->xv.p) {
            CKA(c->xvAlt.alloc(c->xv.n));
            std::swap(c->xv.p, c->xvAlt.p);
            std::swap(c->xv.n, c->xvAlt.n);
            break;
        }
    }
    for (auto &r : c->rd) {
        if (r.on && r.p == c->xv.p) {
            CK(cudaStreamWaitEvent(c->stream, r.ev, 0));
            r.on = false;
        }
    }
    return IDW_OK;
}

static int run_warp(Ctx *c, double *xvOut, double *denOut) {
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (int e0 = ensure_den0(c)) return e0;
    int rc = refresh_nodal(c);
    if (rc) return rc;
    EvalConsts k;
    k.law = make_law(c);
    k.errTol = c->opt.errTol;
    k.sym = c->sym;
    k.slotStats = c->opt.diagnostics & 1;
    k.exactSchedule = c->opt.exactSchedule;
    // terms whose weight x (motion + lever arm) exceeds mixedGate*Ldef*den0 are summed in double-float
    k.precGate = mixed_gate(c);
    PointsDev p;
    p.xa = c->ptXA.p;
    p.mb = c->ptMB.p;
    WalkOut o;
    o.xv = xvOut;
    o.den = denOut;
    o.counters = c->counters.p;
    CK(cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream));
    CK(cudaEventRecord(c->ev0, c->stream));
    const int exact = c->opt.evalMode == IDW_EVAL_EXACT;
    if (c->opt.precision == IDW_PREC_MIXED) {
        const TreeDevF tf = tree_devf(c);
        PointsDevF pf;
        pf.da = c->ptDA.p;
        pf.dl = c->ptDL.p;
        pf.dm = c->ptDM.p;
        pf.dml = c->ptDMl.p;
        NodeAggF af;
        af.dc = c->nodeDC.p;
        af.dcl = c->nodeDCl.p;
        af.dn = c->nodeDn.p;
        af.ref = c->refDB.p;
        af.rr = c->replayRec.p;
        WalkRecF rec;
        rec.hi = c->recHi.p;
        rec.lo = c->recLo.p;
        int rc2 = ensure_walk_lists(c, tf, rec, k);
        if (rc2) return rc2;
        rc2 = ensure_gate_den(c, tf, pf, af, rec, k, exact);
        if (rc2) return rc2;
        rec.gden = c->gden.p;
        CK(cudaEventRecord(c->ev0, c->stream));
        launch_walk_mixed(tree_dev(c), tf, pf, af, vol_dev(c), rec, k, exact, c->acc.p, o, c->stream);
    } else {
        launch_walk_fp64(tree_dev(c), p, vol_dev(c), c->nodeMB.p, k, exact, c->nUnique, o, c->stream);
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    c->eventsRecorded = true;
    return check_launch(c, "warp");
}

static int read_counters(Ctx *c) {
    unsigned long long h[8];
    CK(cudaMemcpyAsync(h, c->counters.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->stats.warpLeafSlots = int64_t(h[4]);
    c->stats.warpNodeSlots = int64_t(h[5]);
    c->stats.leafPairs = int64_t(h[0]);
    c->stats.approx = int64_t(h[1]);
    c->stats.visited = int64_t(h[2]);
    c->stats.fp64Fallback = int64_t(h[3]);
    c->stats.preciseTerms = int64_t(h[6]);
    c->stats.walkListEntries = c->listState == 1 ? c->listEntries : (c->listState == -1 ? -1 : 0);
    if (c->eventsRecorded) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) c->stats.lastKernelMs = ms;
        (void)cudaGetLastError();
    }
    return IDW_OK;
}

int idw_warp_mesh(void *ctx) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    CK(cudaSetDevice(c->device));
    int rc = prepare_xv_write(c);
    if (rc) return rc;
    rc = run_warp(c, c->xv.p, c->den.p);
    if (rc) return rc;
    c->haveWarp = true;
    return IDW_OK;
}

int idw_set_surface_coordinates_cs(void *ctx, const double *coords, int64_t cdof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (cdof != 3 * int64_t(c->nPts))
        return fail(c, IDW_ERR_ARG, "incorrect length of coordinates: expected %lld, received %lld",
                    (long long)(3 * int64_t(c->nPts)), (long long)cdof);
    CK(cudaSetDevice(c->device));
    if (where != IDW_DEVICE && !all_finite(coords, 2 * size_t(cdof)))
        return fail(c, IDW_ERR_NONFINITE, "non-finite surface coordinates");
    CKA(c->xsC.alloc(2 * size_t(cdof)));
    int rc = copy_in(c, c->xsC.p, coords, 2 * size_t(cdof), where);
    if (rc) return rc;
    DevBuf<double> im;
    CKA(im.alloc(size_t(cdof)));
    launch_split(cdof, c->xsC.p, c->xs.p, im.p, c->stream);
    rc = check_launch(c, "complex coordinates");
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    c->nodalValid = false;
    c->haveCs = true;
    return IDW_OK;
}

int idw_warp_mesh_cs(void *ctx) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (c->opt.precision != IDW_PREC_FP64) return fail(c, IDW_ERR_STATE, "the complex step runs in FP64 precision");
    if (!c->haveCs) return fail(c, IDW_ERR_STATE, "complex surface coordinates must be set first");
    CK(cudaSetDevice(c->device));
    int rc = prepare_xv_write(c);
    if (rc) return rc;
    // real part: the ordinary warp of the real coordinates (also sets den)
    rc = run_warp(c, c->xv.p, c->den.p);
    if (rc) return rc;
    c->haveWarp = true;
    // imaginary part: complex nodal properties, their cluster means, and
    // the FP64 walk in tangent mode over (Im M, Im b) divided by the real
    // denominator
    const int n = c->nUnique;
    CKA(c->xuC.alloc(3 * size_t(n)));
    CKA(c->ptMBim.alloc(12 * size_t(n)));
    CKA(c->nodeMBim.alloc(12 * size_t(c->nNodes)));
    CKA(c->xvIm.alloc(3 * size_t(c->nVol)));
    launch_nodal_cs(surf_dev(c), c->xuInd.p, c->xsC.p, c->xuC.p, c->ptXA.p, c->normals0.p, c->tmpAi.p,
                    c->isCorner.p, c->opt.useRotations, c->ptMBim.p, c->stream);
    launch_set_data(tree_dev(c), c->ptMBim.p, c->nodeMBim.p, setdata_scratch(c), c->stream);
    rc = check_launch(c, "complex nodal properties");
    if (rc) return rc;
    EvalConsts k;
    k.law = make_law(c);
    k.errTol = c->opt.errTol;
    k.sym = c->sym;
    k.slotStats = 0;
    k.exactSchedule = c->opt.exactSchedule;
    k.precGate = 0.0;
    PointsDev p;
    p.xa = c->ptXA.p;
    p.mb = c->ptMBim.p;
    WalkOut o;
    o.xv = c->xvIm.p;
    o.counters = nullptr;
    o.tangent = 1;
    o.denIn = c->den.p;
    launch_walk_fp64(tree_dev(c), p, vol_dev(c), c->nodeMBim.p, k, c->opt.evalMode == IDW_EVAL_EXACT, n, o,
                     c->stream);
    rc = check_launch(c, "complex walk");
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return IDW_OK;
}

int idw_get_volume_coordinates_cs(void *ctx, double *out, int64_t ndof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (ndof != 3 * c->nVol)
        return fail(c, IDW_ERR_ARG, "ndof mismatch: %lld vs %lld", (long long)ndof, (long long)(3 * c->nVol));
    if (!c->haveCs || !c->xvIm.p) return fail(c, IDW_ERR_STATE, "no complex warp has been run");
    CK(cudaSetDevice(c->device));
    DevBuf<double> tmp;
    double *dst = out;
    if (where != IDW_DEVICE) {
        CKA(tmp.alloc(2 * size_t(ndof)));
        dst = tmp.p;
    }
    launch_interleave(ndof, c->xv.p, c->xvIm.p, dst, c->stream);
    int rc = check_launch(c, "complex grid");
    if (rc) return rc;
    if (where != IDW_DEVICE) return copy_out(c, out, tmp.p, 2 * size_t(ndof), IDW_HOST);
    CK(cudaStreamSynchronize(c->stream));
    return IDW_OK;
}

}  // extern "C"

// Up to kBatchWalk surfaces share one mixed walk (idw_batch.cu): per surface
// the nodal properties, cluster means and FP32 motion arrays, then one walk
// and a finalisation per surface.  coords/out are device pointers.
static constexpr int kBatchWalk = kBatchMax;

// tangent = 1: coordsDev holds surface tangents dXs; the walk then uses the
// tangent nodal properties (Md + I, bd) at the current surface and writes
// dXv = num / den (warpDerivFwd for nb directions), gated by tangentGate.
static int run_warp_batch_mixed(Ctx *c, const double *coordsDev, int nb, double *outDev, int tangent = 0,
                                double tangentGate = 0.0) {
    const int n = c->nUnique, nn = c->nNodes;
    const size_t sdof = 3 * size_t(c->nPts), vdof = 3 * size_t(c->nVol);
    if (c->batchCap < nb) {
        const size_t B = kBatchWalk;
        CKA(c->bXu.alloc(B * 3 * n));
        CKA(c->bPtMB.alloc(B * 12 * n));
        CKA(c->bNodeMB.alloc(B * 12 * size_t(nn)));
        CKA(c->bPtDM.alloc(B * 12 * n));
        CKA(c->bPtDMl.alloc(B * 12 * n));
        CKA(c->bNodeDC.alloc(B * 12 * size_t(nn)));
        CKA(c->bNodeDCl.alloc(B * 12 * size_t(nn)));
        CKA(c->bNodeDn.alloc(B * size_t(nn)));
        CKA(c->bRef.alloc(B * 24));
        CKA(c->bAcc.alloc(B * 2 * size_t(c->nVol)));
        c->batchCap = kBatchWalk;
    }
    SurfaceDev s = surf_dev(c);
    const int exact = c->opt.evalMode == IDW_EVAL_EXACT;
    // exact mode on a mesh that fills the GPU runs the tiled kernel once per
    // surface (no decisions to share), on surface-major arrays; the batched
    // walk reads point-major ones
    const bool tiledExact = exact && c->nLeaves > 0 && c->opt.exactSchedule != IDW_EXACT_WALK &&
                            (c->opt.exactSchedule == IDW_EXACT_TILED || exact_tiled_fills(c->nVol));
    if (tangent) launch_gather_xu(n, c->xuInd.p, c->xs.p, c->xu.p, c->stream);
    for (int b = 0; b < nb; ++b) {
        double *xu = c->bXu.p + size_t(b) * 3 * n, *mb = c->bPtMB.p + size_t(b) * 12 * n;
        double *nmb = c->bNodeMB.p + size_t(b) * 12 * nn;
        launch_gather_xu(n, c->xuInd.p, coordsDev + size_t(b) * sdof, xu, c->stream);
        if (tangent)
            launch_nodal_d(s, c->xu.p, xu, c->ptXA.p, c->normals0.p, c->tmpAi.p, c->isCorner.p, c->opt.useRotations, 1,
                           mb, c->stream);
        else
            launch_nodal(s, xu, c->ptXA.p, c->normals0.p, c->tmpAi.p, c->isCorner.p, c->opt.useRotations, mb,
                         c->stream);
        launch_set_data(tree_dev(c), mb, nmb, setdata_scratch(c), c->stream);
        if (tiledExact) {
            launch_mixed_nodal(n, tree_dev(c), nmb, c->ptXA.p, mb, c->bPtDM.p + size_t(b) * 12 * n,
                               c->bPtDMl.p + size_t(b) * 12 * n, c->stream);
            launch_mixed_nodes(tree_dev(c), nmb, mb, c->bNodeDC.p + size_t(b) * 12 * nn,
                               c->bNodeDCl.p + size_t(b) * 12 * nn, c->bNodeDn.p + size_t(b) * nn, c->bRef.p + 24 * b,
                               c->stream);
        } else {
            const int B = kBatchWalk;
            launch_mixed_nodal(n, tree_dev(c), nmb, c->ptXA.p, mb, c->bPtDM.p + 12 * b, c->bPtDMl.p + 12 * b,
                               c->stream, 12 * B);
            launch_mixed_nodes(tree_dev(c), nmb, mb, c->bNodeDC.p + 12 * b, c->bNodeDCl.p + 12 * b, c->bNodeDn.p + b,
                               c->bRef.p + 24 * b, c->stream, 12 * B, B);
        }
    }
    int rc = check_launch(c, "batch nodal properties");
    if (rc) return rc;
    EvalConsts k;
    k.law = make_law(c);
    k.errTol = c->opt.errTol;
    k.sym = c->sym;
    k.slotStats = 0;
    k.exactSchedule = c->opt.exactSchedule;
    k.precGate = tangent ? tangentGate : mixed_gate(c);
    const TreeDevF tf = tree_devf(c);
    PointsDevF pf;
    pf.da = c->ptDA.p;
    pf.dl = c->ptDL.p;
    pf.dm = c->bPtDM.p;
    pf.dml = c->bPtDMl.p;
    NodeAggF af;
    af.dc = c->bNodeDC.p;
    af.dcl = c->bNodeDCl.p;
    af.dn = c->bNodeDn.p;
    af.ref = c->bRef.p;
    WalkRecF rec;
    rec.hi = c->recHi.p;
    rec.lo = c->recLo.p;
    {
        // the gate's denominators depend on the weights only: the
        // single-surface walk on the context's own arrays gives them
        PointsDevF p1 = pf;
        p1.dm = c->ptDM.p;
        p1.dml = c->ptDMl.p;
        NodeAggF a1 = af;
        a1.dc = c->nodeDC.p;
        a1.dcl = c->nodeDCl.p;
        a1.dn = c->nodeDn.p;
        a1.ref = c->refDB.p;
        a1.rr = c->replayRec.p;
        rc = ensure_walk_lists(c, tf, rec, k);
        if (rc) return rc;
        rc = ensure_gate_den(c, tf, p1, a1, rec, k, exact);
        if (rc) return rc;
    }
    rec.gden = c->gden.p;
    if (k.lists.list && !tiledExact && !exact) launch_add_walk_counters(c->counters.p, k.lists.counters, c->stream);
    CK(cudaEventRecord(c->ev0, c->stream));
    if (tiledExact) {
        // exact mode on a mesh that fills the GPU: the tiled kernel per surface
        // (no decisions to share between surfaces)
        const MixedParams mp = make_mixed_params(k);
        for (int b = 0; b < nb; ++b) {
            PointsDevF pb = pf;
            pb.dm += size_t(b) * 12 * n;
            pb.dml += size_t(b) * 12 * n;
            NodeAggF ab = af;
            ab.dc += size_t(b) * 12 * nn;
            ab.dcl += size_t(b) * 12 * nn;
            ab.dn += size_t(b) * nn;
            ab.ref += 24 * b;
            launch_exact_mixed(tf, pb, ab, vol_dev(c), rec, mp, k.law, c->bAcc.p + size_t(b) * 2 * c->nVol,
                               c->counters.p, c->stream);
        }
    } else {
        launch_walk_mixed_batch(nb, tree_dev(c), tf, pf, af, vol_dev(c), rec, k, exact, c->bAcc.p, 2 * c->nVol,
                                c->counters.p, c->stream);
    }
    for (int b = 0; b < nb; ++b)
        launch_finalize_mixed(vol_dev(c), rec, c->bAcc.p + size_t(b) * 2 * c->nVol, k.law.bExp,
                              outDev + size_t(b) * vdof, c->stream, tangent);
    CK(cudaEventRecord(c->ev1, c->stream));
    c->eventsRecorded = true;
    return check_launch(c, "batch walk");
}

extern "C" {

int idw_warp_mesh_batch(void *ctx, const double *coords, int32_t nbatch, double *out, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (int e0 = ensure_den0(c)) return e0;
    if (nbatch < 0 || !coords || !out) return fail(c, IDW_ERR_ARG, "bad batch arguments");
    CK(cudaSetDevice(c->device));
    const size_t sdof = 3 * size_t(c->nPts), vdof = 3 * size_t(c->nVol);
    if (c->opt.precision == IDW_PREC_MIXED && nbatch > 0) {
        // surfaces in groups of up to kBatchWalk per walk
        CK(cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream));
        DevBuf<double> tin, tout;
        const int g = std::min<int>(nbatch, kBatchWalk);
        if (where != IDW_DEVICE) {
            CKA(tin.alloc(size_t(g) * sdof));
            CKA(tout.alloc(size_t(g) * vdof));
        }
        const int G = std::max(1, std::min(c->batchGroup, kBatchWalk));
        for (int b0 = 0; b0 < nbatch; b0 += G) {
            const int nb = std::min<int>(G, nbatch - b0);
            const double *cin = coords + size_t(b0) * sdof;
            double *cout = out + size_t(b0) * vdof;
            if (where != IDW_DEVICE) {
                if (!all_finite(cin, size_t(nb) * sdof)) return fail(c, IDW_ERR_NONFINITE, "non-finite coordinates");
                int rc = copy_in(c, tin.p, cin, size_t(nb) * sdof, IDW_HOST);
                if (rc) return rc;
                cin = tin.p;
            }
            int rc = run_warp_batch_mixed(c, cin, nb, where != IDW_DEVICE ? tout.p : cout);
            if (rc) return rc;
            if (where != IDW_DEVICE) {
                rc = copy_out(c, out + size_t(b0) * vdof, tout.p, size_t(nb) * vdof, IDW_HOST);
                if (rc) return rc;
            }
        }
        CK(cudaStreamSynchronize(c->stream));
        return IDW_OK;
    }
    // keep the context's own surface: stage it and restore afterwards
    DevBuf<double> keep, tmpOut;
    CKA(keep.alloc(sdof));
    CK(cudaMemcpyAsync(keep.p, c->xs.p, sdof * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if (where != IDW_DEVICE) CKA(tmpOut.alloc(vdof));
    for (int b = 0; b < nbatch; ++b) {
        int rc = copy_in(c, c->xs.p, coords + b * sdof, sdof, where);
        if (rc) return rc;
        double *dst = (where == IDW_DEVICE) ? out + b * vdof : tmpOut.p;
        rc = run_warp(c, dst, nullptr);
        if (rc) return rc;
        if (where != IDW_DEVICE) {
            rc = copy_out(c, out + b * vdof, tmpOut.p, vdof, IDW_HOST);
            if (rc) return rc;
        }
    }
    CK(cudaMemcpyAsync(c->xs.p, keep.p, sdof * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->nodalValid = false;
    return IDW_OK;
}

int idw_get_volume_coordinates(void *ctx, double *out, int64_t ndof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (ndof != 3 * c->nVol) return fail(c, IDW_ERR_ARG, "ndof mismatch: %lld vs %lld", (long long)ndof, (long long)(3 * c->nVol));
    CK(cudaSetDevice(c->device));
    return copy_out(c, out, c->xv.p, size_t(ndof), where);
}

int idw_get_common_volume_coordinates(void *ctx, double *out, int64_t ndof, int where) {
    return idw_get_volume_coordinates(ctx, out, ndof, where);
}

int idw_get_volume_coordinates_async(void *ctx, double *out, int64_t ndof) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (ndof != 3 * c->nVol) return fail(c, IDW_ERR_ARG, "ndof mismatch: %lld vs %lld", (long long)ndof, (long long)(3 * c->nVol));
    if (ndof > 0 && !out) return fail(c, IDW_ERR_ARG, "null output pointer");
    CK(cudaSetDevice(c->device));
    if (!c->copyStream) {
        CK(cudaStreamCreateWithFlags(&c->copyStream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&c->evReady, cudaEventDisableTiming));
        for (auto &r : c->rd) CK(cudaEventCreateWithFlags(&r.ev, cudaEventDisableTiming));
    }
    // the read of this buffer's slot (or the slot of the other buffer's older read)
    Ctx::PendingRead *slot = nullptr;
    for (auto &r : c->rd)
        if (r.p == c->xv.p) slot = &r;
    if (!slot)
        for (auto &r : c->rd)
            if (!r.on || r.p != c->xvAlt.p) slot = &r;
    if (!slot) return fail(c, IDW_ERR_STATE, "no free read slot");
    CK(cudaEventRecord(c->evReady, c->stream));
    CK(cudaStreamWaitEvent(c->copyStream, c->evReady, 0));
    if (ndof > 0)
        CK(cudaMemcpyAsync(out, c->xv.p, sizeof(double) * size_t(ndof), cudaMemcpyDeviceToHost, c->copyStream));
    CK(cudaEventRecord(slot->ev, c->copyStream));
    slot->p = c->xv.p;
    slot->on = true;
    return IDW_OK;
}

int idw_set_volume_coordinates(void *ctx, const double *in, int64_t ndof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (ndof != 3 * c->nVol) return fail(c, IDW_ERR_ARG, "ndof mismatch");
    CK(cudaSetDevice(c->device));
    int rc = prepare_xv_write(c);
    if (rc) return rc;
    rc = copy_in(c, c->xv.p, in, size_t(ndof), where);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return IDW_OK;
}

int idw_get_stats(void *ctx, idw_stats *out) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c || !out) return IDW_ERR_ARG;
    CK(cudaSetDevice(c->device));
    int rc = read_counters(c);
    if (rc) return rc;
    *out = c->stats;
    return IDW_OK;
}

int idw_get_denominator0(void *ctx, double *out, int64_t nvol, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (int e0 = ensure_den0(c)) return e0;
    if (nvol != c->nVol) return fail(c, IDW_ERR_ARG, "nvol mismatch");
    CK(cudaSetDevice(c->device));
    return copy_out(c, out, c->den0.p, size_t(nvol), where);
}

int idw_compute_denominator0(void *ctx) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (int e0 = ensure_den0(c)) return e0;
    CK(cudaStreamSynchronize(c->stream));
    return IDW_OK;
}

int idw_set_denominator0(void *ctx, const double *den0, int64_t nvol, int64_t checkStride, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (nvol != c->nVol) return fail(c, IDW_ERR_ARG, "nvol mismatch: expected %lld, received %lld",
                                     (long long)c->nVol, (long long)nvol);
    if (nvol > 0 && !den0) return fail(c, IDW_ERR_ARG, "null denominator pointer");
    if (where != IDW_DEVICE && !all_finite(den0, size_t(nvol)))
        return fail(c, IDW_ERR_NONFINITE, "non-finite denominator estimate");
    CK(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    DevBuf<double> tmp;
    CKA(tmp.alloc(size_t(nvol)));
    int rc = copy_in(c, tmp.p, den0, size_t(nvol), where);
    if (rc) return rc;
    if (checkStride > 0 && nvol > 0) {
        // initializeWarping.F90:190-209: re-estimate every checkStride-th node
        const int64_t m = (nvol + checkStride - 1) / checkStride;
        DevBuf<double> est;
        CKA(est.alloc(size_t(m)));
        launch_denominator0_strided(tree_dev(c), c->nodeRec.p, c->ptXA.p, vol_dev(c), make_init_law(c), c->sym, checkStride,
                                    est.p, st);
        rc = check_launch(c, "denominator0 check");
        if (rc) return rc;
        std::vector<double> e(m), l(m);
        CK(cudaMemcpyAsync(e.data(), est.p, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpy2DAsync(l.data(), sizeof(double), tmp.p, sizeof(double) * size_t(checkStride), sizeof(double),
                             size_t(m), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int64_t k = 0; k < m; ++k)
            if (1.0 - e[k] / l[k] > 1e-15)
                return fail(c, IDW_ERR_RESTART, "denominator0 of node %lld: loaded %.17g, estimate %.17g",
                            (long long)(k * checkStride), l[k], e[k]);
    }
    CK(cudaMemcpyAsync(c->den0.p, tmp.p, sizeof(double) * size_t(nvol), cudaMemcpyDeviceToDevice, st));
    c->haveWarp = c->haveDxs = false;
    rc = finish_den0(c);
    if (rc) return rc;
    CK(cudaStreamSynchronize(st));
    return IDW_OK;
}

int idw_dry_run_costs(void *ctx, double *costs, int64_t nvol, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (int e0 = ensure_den0(c)) return e0;
    if (nvol != c->nVol) return fail(c, IDW_ERR_ARG, "nvol mismatch");
    CK(cudaSetDevice(c->device));
    DevBuf<double> out;
    CKA(out.alloc(size_t(nvol)));
    if (nvol > 0) CK(cudaMemsetAsync(out.p, 0, sizeof(double) * size_t(nvol), c->stream));
    launch_dry_run(tree_dev(c), vol_dev(c), c->sym, c->opt.errTol, c->nUnique, out.p, c->stream);
    int rc = check_launch(c, "dryRun costs");
    if (rc) return rc;
    return copy_out(c, costs, out.p, size_t(nvol), where);
}

int idw_get_denominator(void *ctx, double *out, int64_t nvol, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveWarp) return fail(c, IDW_ERR_STATE, "warpMesh has not been called");
    if (nvol != c->nVol) return fail(c, IDW_ERR_ARG, "nvol mismatch");
    CK(cudaSetDevice(c->device));
    return copy_out(c, out, c->den.p, size_t(nvol), where);
}

}  // extern "C"

// ---- order-independent landings (option deterministic, idw_land.cuh) ----

// Deterministic reverse products run one at a time in the process: the
// landing state is one constant per translation unit.
std::mutex g_landMu;

__global__ void k_land_convert(double *d, int64_t len, const int *expo, const unsigned long long *fix) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= len) return;
    const int E = expo[t];
    if (E == kLandNone) return;
    if (E == kLandNonFinite) {
        d[t] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    unsigned long long u0 = fix[3 * t], u1 = fix[3 * t + 1], u2 = fix[3 * t + 2];
    const bool neg = (u2 >> 63) != 0ull;
    if (neg) {
        u0 = ~u0 + 1ull;
        const unsigned long long c0 = u0 == 0ull ? 1ull : 0ull;
        u1 = ~u1 + c0;
        const unsigned long long c1 = (c0 && u1 == 0ull) ? 1ull : 0ull;
        u2 = ~u2 + c1;
    }
    // 2^E sits at bit 126
    const double r = ldexp(double(u2), 2 + E) + ldexp(double(u1), E - 62) + ldexp(double(u0), E - 126);
    d[t] += neg ? -r : r;
}

int land_set_all(Ctx *c, const LandState &s) {
    cudaError_t e = land_set_adjoint(s, c->stream);
    if (e == cudaSuccess) e = land_set_precise(s, c->stream);
    if (e == cudaSuccess) e = land_set_walk(s, c->stream);
    if (e == cudaSuccess) e = land_set_nodal(s, c->stream);
    if (e == cudaSuccess) e = land_set_exact(s, c->stream);
    if (e != cudaSuccess) return fail(c, IDW_ERR_CUDA, "landing state: %s", cudaGetErrorString(e));
    return IDW_OK;
}

// Clears the landing state and waits for the stream when a deterministic
// call ends, on every path out of it (quietly: an error that ended the call
// keeps its message).
struct LandClear {
    Ctx *c;
    bool on;
    ~LandClear() {
        if (!on) return;
        LandState z{};
        land_set_adjoint(z, c->stream);
        land_set_precise(z, c->stream);
        land_set_walk(z, c->stream);
        land_set_nodal(z, c->stream);
        land_set_exact(z, c->stream);
        cudaStreamSynchronize(c->stream);
    }
};

// One scattering stage with order-independent landings into the nArr
// accumulators (base[a], len[a] doubles): `stage(pass)` launches it, once
// per pass; the fixed-point sums are then added to the accumulators.
template <class F>
int land_stage(Ctx *c, int nArr, double *const *base, const int64_t *len, F &&stage) {
    int64_t total = 0;
    for (int a = 0; a < nArr; ++a) total += len[a];
    if (total <= 0) return stage(0);
    CKA(c->landExpo.alloc(size_t(total)));
    CKA(c->landFix.alloc(3 * size_t(total)));
    CK(cudaMemsetAsync(c->landExpo.p, 0x80, sizeof(int) * size_t(total), c->stream));
    CK(cudaMemsetAsync(c->landFix.p, 0, 3 * sizeof(unsigned long long) * size_t(total), c->stream));
    LandState s{};
    s.nArr = nArr;
    int64_t off = 0;
    for (int a = 0; a < nArr; ++a) {
        s.base[a] = base[a];
        s.len[a] = len[a];
        s.expo[a] = c->landExpo.p + off;
        s.fix[a] = c->landFix.p + 3 * off;
        off += len[a];
    }
    for (int pass = 1; pass <= 2; ++pass) {
        s.pass = pass;
        if (int rc = land_set_all(c, s)) return rc;
        if (int rc = stage(pass)) return rc;
    }
    LandState z{};
    if (int rc = land_set_all(c, z)) return rc;
    off = 0;
    for (int a = 0; a < nArr; ++a) {
        if (len[a] > 0)
            k_land_convert<<<int((len[a] + 255) / 256), 256, 0, c->stream>>>(base[a], len[a], c->landExpo.p + off,
                                                                              c->landFix.p + 3 * off);
        off += len[a];
    }
    return check_launch(c, "order-independent landing");
}

extern "C" {

static int run_deriv(Ctx *c, const double *dxvDev, int nSeeds, int64_t seedStride, double *dxsOut, int where,
                     int64_t dxsStride) {
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    const bool det = c->opt.deterministic != 0;
    if (det) {
        // the passes set constant memory and wait for the stream: not inside a capture
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(c->stream, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return fail(c, IDW_ERR_STATE, "deterministic reverse products cannot be captured in a CUDA graph");
    }
    if (int e0 = ensure_den0(c)) return e0;
    if (!c->haveWarp) return fail(c, IDW_ERR_STATE, "warpMesh must be called before warpDeriv");
    int rc = refresh_nodal(c);
    if (rc) return rc;
    EvalConsts k;
    k.law = make_law(c);
    k.errTol = c->opt.errTol;
    k.sym = c->sym;
    k.slotStats = 0;
    k.exactSchedule = c->opt.exactSchedule;
    k.precGate = 0.0;
    PointsDev p;
    p.xa = c->ptXA.p;
    p.mb = c->ptMB.p;
    const int n = c->nUnique, nn = c->nNodes;
    const int exact = c->opt.evalMode == IDW_EVAL_EXACT;
    const int mixed = c->opt.precision == IDW_PREC_MIXED;
    // accumulators owned by the context (grown on demand): a call with device
    // pointers and a seed count already seen allocates nothing, so it can be
    // captured in a CUDA graph
    if (c->adjSeeds < nSeeds) {
        CKA(c->adjPt.alloc(size_t(nSeeds) * 12 * n));
        CKA(c->adjNode.alloc(size_t(nSeeds) * 12 * nn));
        CKA(c->adjRel.alloc(size_t(nSeeds) * 12 * n));
        c->adjSeeds = nSeeds;
    }
    DevView ptAdj{c->adjPt.p}, nodeAdj{c->adjNode.p}, ptRel{c->adjRel.p};
    CK(cudaMemsetAsync(ptAdj.p, 0, sizeof(double) * size_t(nSeeds) * 12 * n, c->stream));
    CK(cudaMemsetAsync(nodeAdj.p, 0, sizeof(double) * size_t(nSeeds) * 12 * nn, c->stream));
    CK(cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream));
    // deterministic: one such call at a time, the landing state cleared on every way out
    std::unique_lock<std::mutex> detLock;
    if (det) detLock = std::unique_lock<std::mutex>(g_landMu);
    LandClear landClear{c, det};
    CK(cudaEventRecord(c->ev0, c->stream));
    const TreeDevF tf = tree_devf(c);
    PointsDevF pf;
    pf.da = c->ptDA.p;
    pf.dl = c->ptDL.p;
    pf.dm = c->ptDM.p;
    pf.dml = c->ptDMl.p;
    WalkRecF rec;
    rec.hi = c->recHi.p;
    rec.lo = c->recLo.p;
    bool precise = false;
    if (mixed) {
        rc = ensure_walk_lists(c, tf, rec, k);
        if (rc) return rc;
        precise = c->opt.adjointPrecision == IDW_ADJ_PRECISE && precise_adjoint_supported(k.law);
        // the precise form's denominator to double-float accuracy: once per weight law and mode
        if (precise && !(c->denPValid && c->denPLdefFact == c->opt.LdefFact && c->denPAlpha == c->opt.alpha &&
                         c->denPMode == c->opt.evalMode)) {
            CKA(c->denP.alloc(size_t(c->nVol)));
            launch_precise_denominator(tree_dev(c), tf, pf, vol_dev(c), rec, k, exact, c->denP.p, c->stream);
            rc = check_launch(c, "precise denominator");
            if (rc) return rc;
            c->denPValid = true;
            c->denPLdefFact = c->opt.LdefFact;
            c->denPAlpha = c->opt.alpha;
            c->denPMode = c->opt.evalMode;
            CK(cudaEventRecord(c->ev0, c->stream));
        }
    }
    // the reverse walk: point and cluster moments land in ptAdj / nodeAdj
    auto walk = [&](int) -> int {
        if (mixed && precise)
            launch_adjoint_precise(tree_dev(c), tf, pf, vol_dev(c), rec, k, exact, dxvDev, nSeeds, seedStride,
                                   c->denP.p, ptAdj.p, nodeAdj.p, n, c->counters.p, c->stream, det);
        else if (mixed)
            launch_adjoint_mixed(tree_dev(c), tf, pf, vol_dev(c), rec, k, exact, dxvDev, nSeeds, seedStride, c->den.p,
                                 ptAdj.p, nodeAdj.p, ptRel.p, c->ptXA.p, n, c->counters.p, c->stream,
                                 c->adjMaxGroup, 0, det);
        else
            launch_walk_adjoint_fp64(tree_dev(c), p, vol_dev(c), k, exact, n, dxvDev, c->den.p, nSeeds, seedStride,
                                     ptAdj.p, nodeAdj.p, int64_t(12) * n, int64_t(12) * nn, c->counters.p,
                                     c->stream, det);
        return check_launch(c, "adjoint walk");
    };
    if (det) {
        // the second pass counts its work again: keep one pass's counters
        double *base[2] = {ptAdj.p, nodeAdj.p};
        const int64_t len[2] = {int64_t(nSeeds) * 12 * n, int64_t(nSeeds) * 12 * nn};
        rc = land_stage(c, 2, base, len, [&](int pass) {
            if (pass == 2) {
                const cudaError_t e = cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream);
                if (e != cudaSuccess) return fail(c, IDW_ERR_CUDA, "counters: %s", cudaGetErrorString(e));
            }
            return walk(pass);
        });
    } else {
        rc = walk(0);
    }
    if (rc) return rc;
    // the relative moments and the cluster shares (setData_b folded in)
    if (mixed) launch_adjoint_combine(tree_dev(c), c->ptXA.p, n, nSeeds, ptAdj.p, nodeAdj.p, ptRel.p, c->stream);
    CK(cudaEventRecord(c->ev1, c->stream));
    c->eventsRecorded = true;
    rc = check_launch(c, "adjoint walk");
    if (rc) return rc;
    SurfaceDev s = surf_dev(c);
    const bool faceLandings = c->opt.useRotations && c->nFaces > 0;
    for (int sd = 0; sd < nSeeds; ++sd) {
        double *pa = (mixed ? ptRel.p : ptAdj.p) + size_t(sd) * 12 * n;
        if (!mixed) launch_set_data_b(tree_dev(c), nodeAdj.p + size_t(sd) * 12 * nn, pa, n, c->stream);
        CK(cudaMemsetAsync(c->xub.p, 0, sizeof(double) * 3 * n, c->stream));
        if (det && faceLandings) {
            // node part: area and normal adjoints land in the faces' scratch
            // (Xub += Bb is the node's own write: from zero in each pass)
            double *faceAdj[1] = {c->faceScratch.p + 4 * size_t(c->nFaces)};
            const int64_t faceLen[1] = {4 * int64_t(c->nFaces)};
            rc = land_stage(c, 1, faceAdj, faceLen, [&](int pass) {
                if (pass == 2) {
                    const cudaError_t e = cudaMemsetAsync(c->xub.p, 0, sizeof(double) * 3 * n, c->stream);
                    if (e != cudaSuccess) return fail(c, IDW_ERR_CUDA, "Xub: %s", cudaGetErrorString(e));
                }
                launch_nodal_b_nodes(s, c->xu.p, c->ptXA.p, c->normals0.p, c->isCorner.p, c->opt.useRotations, pa,
                                     mixed, c->xub.p, c->stream, sd == 0 && pass <= 1, 1);
                return check_launch(c, "reverse nodal properties");
            });
            if (rc) return rc;
            // face part: each face's element adjoint lands in Xub of its vertices
            double *xubArr[1] = {c->xub.p};
            const int64_t xubLen[1] = {3 * int64_t(n)};
            rc = land_stage(c, 1, xubArr, xubLen, [&](int) {
                launch_nodal_b_faces(s, c->xu.p, c->opt.useRotations, c->xub.p, c->stream, 1);
                return check_launch(c, "reverse nodal properties");
            });
            if (rc) return rc;
        } else {
            launch_nodal_b(s, c->xu.p, c->ptXA.p, c->normals0.p, c->isCorner.p, c->opt.useRotations, pa, mixed,
                           c->xub.p, c->stream, sd == 0);
        }
        double *dst = (where == IDW_DEVICE) ? dxsOut + sd * dxsStride : c->dxs.p;
        CK(cudaMemsetAsync(dst, 0, sizeof(double) * 3 * c->nPts, c->stream));
        launch_scatter_dxs(n, c->xuInd.p, c->xub.p, dst, c->stream);
        rc = check_launch(c, "reverse nodal properties");
        if (rc) return rc;
        if (where != IDW_DEVICE && dxsOut) {
            rc = copy_out(c, dxsOut + sd * dxsStride, c->dxs.p, 3 * size_t(c->nPts), IDW_HOST);
            if (rc) return rc;
        }
    }
    return IDW_OK;
}

int idw_warp_deriv(void *ctx, const double *dxv, int64_t ndof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (ndof != 3 * c->nVol) return fail(c, IDW_ERR_ARG, "dXv has %lld entries, expected %lld", (long long)ndof, (long long)(3 * c->nVol));
    CK(cudaSetDevice(c->device));
    const double *d = dxv;
    DevBuf<double> tmp;
    if (where != IDW_DEVICE) {
        CKA(tmp.alloc(size_t(ndof)));
        int rc = copy_in(c, tmp.p, dxv, size_t(ndof), IDW_HOST);
        if (rc) return rc;
        d = tmp.p;
    }
    int rc = run_deriv(c, d, 1, ndof, c->dxs.p, IDW_DEVICE, 3 * int64_t(c->nPts));
    if (rc) return rc;
    if (where != IDW_DEVICE) CK(cudaStreamSynchronize(c->stream));
    c->haveDxs = true;
    return IDW_OK;
}

int idw_get_dxs(void *ctx, double *out, int64_t ndof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (ndof != 3 * int64_t(c->nPts)) return fail(c, IDW_ERR_ARG, "ndof mismatch");
    if (!c->haveDxs) return fail(c, IDW_ERR_STATE, "warpDeriv has not been called");
    CK(cudaSetDevice(c->device));
    return copy_out(c, out, c->dxs.p, size_t(ndof), where);
}

int idw_warp_deriv_batch(void *ctx, const double *dxv, int32_t nseeds, double *dxs, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (nseeds < 1 || !dxv || !dxs) return fail(c, IDW_ERR_ARG, "bad seed arguments");
    CK(cudaSetDevice(c->device));
    const size_t vdof = 3 * size_t(c->nVol);
    const double *d = dxv;
    DevBuf<double> tmp;
    if (where != IDW_DEVICE) {
        CKA(tmp.alloc(vdof * nseeds));
        int rc = copy_in(c, tmp.p, dxv, vdof * nseeds, IDW_HOST);
        if (rc) return rc;
        d = tmp.p;
    }
    int rc = run_deriv(c, d, nseeds, int64_t(vdof), dxs, where, 3 * int64_t(c->nPts));
    if (rc) return rc;
    // host results were synchronised by the copies; device results are
    // ordered on the stream
    return IDW_OK;
}

int idw_set_external_mesh_indices(void *ctx, const int32_t *ind, int64_t ndof_solver) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (ndof_solver < 0 || (ndof_solver > 0 && !ind)) return fail(c, IDW_ERR_ARG, "bad solver indices");
    for (int64_t k = 0; k < ndof_solver; ++k)
        if (ind[k] < 0 || ind[k] >= 3 * c->nVol)
            return fail(c, IDW_ERR_ARG, "solver index %d out of range", ind[k]);
    CK(cudaSetDevice(c->device));
    CKA(c->solverInd.alloc(std::max<int64_t>(ndof_solver, 1)));
    if (ndof_solver > 0)
        CK(cudaMemcpyAsync(c->solverInd.p, ind, sizeof(int) * ndof_solver, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->nSolver = ndof_solver;
    return IDW_OK;
}

int idw_get_solver_mesh_dof(void *ctx, int64_t *ndof) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c || !ndof) return IDW_ERR_ARG;
    *ndof = c->nSolver;
    return IDW_OK;
}

}  // extern "C"

namespace {
__global__ void k_gather_dof(int64_t n, const int *ind, const double *src, double *dst) {
    int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = src[ind[k]];
}
__global__ void k_scatter_add_dof(int64_t n, const int *ind, const double *src, double *dst) {
    int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < n) atomicAdd(dst + ind[k], src[k]);
}
// max |v| (non-negative doubles order like their bit patterns)
__global__ void k_absmax(int64_t n, const double *v, unsigned long long *out) {
    int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double a = k < n ? fabs(v[k]) : 0.0;
    if (!(a <= 1.7976931348623157e308)) a = 0.0;  // non-finite entries are rejected by the caller
    unsigned long long b = (unsigned long long)__double_as_longlong(a);
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long q = __shfl_down_sync(0xffffffffu, b, o);
        b = q > b ? q : b;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, b);
}

// warpDerivFwd (src/warp/warpDerivFwd.F90:58-97): Xvd = sum w (Md r + bd) / den.
int run_deriv_fwd(Ctx *c, const double *xsdDev, double *xvdDev) {
    const int n = c->nUnique, nn = c->nNodes;
    const int exact = c->opt.evalMode == IDW_EVAL_EXACT;
    const int mixed = c->opt.precision == IDW_PREC_MIXED;
    DevBuf<double> xud, ptMBd, nodeMBd;
    CKA(xud.alloc(3 * size_t(n)));
    CKA(ptMBd.alloc(12 * size_t(n)));
    CKA(nodeMBd.alloc(12 * size_t(nn)));
    // Xu, Xud = Xs, Xsd at the first caller occurrence of each unique point
    launch_gather_xu(n, c->xuInd.p, c->xs.p, c->xu.p, c->stream);
    launch_gather_xu(n, c->xuInd.p, xsdDev, xud.p, c->stream);
    // (Md, bd) for the FP64 walk in tangent mode (S = Md r + bd); (Md + I, bd)
    // for the mixed walk, whose motions are relative to the identity
    launch_nodal_d(surf_dev(c), c->xu.p, xud.p, c->ptXA.p, c->normals0.p, c->tmpAi.p, c->isCorner.p,
                   c->opt.useRotations, mixed ? 1 : 0, ptMBd.p, c->stream);
    launch_set_data(tree_dev(c), ptMBd.p, nodeMBd.p, setdata_scratch(c), c->stream);
    int rc = check_launch(c, "tangent nodal properties");
    if (rc) return rc;
    EvalConsts k;
    k.law = make_law(c);
    k.errTol = c->opt.errTol;
    k.sym = c->sym;
    k.slotStats = 0;
    k.exactSchedule = c->opt.exactSchedule;
    k.precGate = 0.0;
    WalkOut o;
    o.xv = xvdDev;
    o.counters = c->counters.p;
    o.tangent = 1;
    o.denIn = c->den.p;
    CK(cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream));
    if (mixed) {
        // the gate scales with the size of the tangent instead of Ldef
        CK(cudaMemsetAsync(c->counters.p + 7, 0, sizeof(unsigned long long), c->stream));
        const int64_t nd = 3 * int64_t(n);
        k_absmax<<<int((nd + 255) / 256), 256, 0, c->stream>>>(nd, xud.p, c->counters.p + 7);
        unsigned long long bits = 0;
        CK(cudaMemcpyAsync(&bits, c->counters.p + 7, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        double scale;
        std::memcpy(&scale, &bits, sizeof(scale));
        k.precGate = c->opt.mixedGate * scale;
        CK(cudaMemsetAsync(c->counters.p + 7, 0, sizeof(unsigned long long), c->stream));
        // the FP32 walk arrays now describe the tangent; the next warp rebuilds them
        launch_mixed_nodal(n, tree_dev(c), nodeMBd.p, c->ptXA.p, ptMBd.p, c->ptDM.p, c->ptDMl.p, c->stream);
        launch_mixed_nodes(tree_dev(c), nodeMBd.p, ptMBd.p, c->nodeDC.p, c->nodeDCl.p, c->nodeDn.p, c->refDB.p,
                           c->stream);
        launch_replay_records(c->nNodes, c->nodeDC.p, c->nodeDn.p, c->replayRec.p, c->stream);
        c->nodalValid = false;
        const TreeDevF tf = tree_devf(c);
        PointsDevF pf;
        pf.da = c->ptDA.p;
        pf.dl = c->ptDL.p;
        pf.dm = c->ptDM.p;
        pf.dml = c->ptDMl.p;
        NodeAggF af;
        af.dc = c->nodeDC.p;
        af.dcl = c->nodeDCl.p;
        af.dn = c->nodeDn.p;
        af.ref = c->refDB.p;
        af.rr = c->replayRec.p;
        WalkRecF rec;
        rec.hi = c->recHi.p;
        rec.lo = c->recLo.p;
        rec.gden = c->gdenValid ? c->gden.p : nullptr;
        if (c->listState == 1 && c->listErrTol == c->opt.errTol && !exact) {
            k.lists.offs = c->walkOffs.p;
            k.lists.list = c->walkList.p;
            k.lists.counters = c->walkCnt.p;
        }
        CK(cudaEventRecord(c->ev0, c->stream));
        launch_walk_mixed(tree_dev(c), tf, pf, af, vol_dev(c), rec, k, exact, c->acc.p, o, c->stream);
    } else {
        PointsDev p;
        p.xa = c->ptXA.p;
        p.mb = ptMBd.p;
        CK(cudaEventRecord(c->ev0, c->stream));
        launch_walk_fp64(tree_dev(c), p, vol_dev(c), nodeMBd.p, k, exact, n, o, c->stream);
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    c->eventsRecorded = true;
    rc = check_launch(c, "tangent walk");
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return IDW_OK;
}
}  // namespace

extern "C" {

int idw_warp_deriv_fwd(void *ctx, const double *dxs, int64_t cdof, double *dxv, int64_t ndof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (int e0 = ensure_den0(c)) return e0;
    if (!c->haveWarp) return fail(c, IDW_ERR_STATE, "warpMesh must be called before warpDerivFwd");
    if (!dxs || !dxv) return fail(c, IDW_ERR_ARG, "null dXs or dXv");
    if (cdof != 3 * int64_t(c->nPts))
        return fail(c, IDW_ERR_ARG, "dXs has %lld entries, expected %lld", (long long)cdof,
                    (long long)(3 * int64_t(c->nPts)));
    if (ndof != 3 * c->nVol)
        return fail(c, IDW_ERR_ARG, "dXv has %lld entries, expected %lld", (long long)ndof, (long long)(3 * c->nVol));
    if (where != IDW_DEVICE && !all_finite(dxs, size_t(cdof)))
        return fail(c, IDW_ERR_NONFINITE, "non-finite dXs");
    CK(cudaSetDevice(c->device));
    const double *in = dxs;
    double *out = dxv;
    DevBuf<double> tin, tout;
    if (where != IDW_DEVICE) {
        CKA(tin.alloc(size_t(cdof)));
        CKA(tout.alloc(size_t(ndof)));
        int rc = copy_in(c, tin.p, dxs, size_t(cdof), IDW_HOST);
        if (rc) return rc;
        in = tin.p;
        out = tout.p;
    }
    int rc = run_deriv_fwd(c, in, out);
    if (rc) return rc;
    if (where != IDW_DEVICE) return copy_out(c, dxv, tout.p, size_t(ndof), IDW_HOST);
    return IDW_OK;
}

int idw_warp_to_solver_grid(void *ctx, const double *warp, int64_t wdof, double *solver, int64_t sdof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (c->nSolver < 0) return fail(c, IDW_ERR_STATE, "setExternalMeshIndices has not been called");
    if (wdof != 3 * c->nVol || sdof != c->nSolver) return fail(c, IDW_ERR_ARG, "size mismatch");
    CK(cudaSetDevice(c->device));
    DevBuf<double> w, s;
    const double *wp = warp;
    double *sp = solver;
    if (where != IDW_DEVICE) {
        CKA(w.alloc(size_t(wdof)));
        CKA(s.alloc(size_t(sdof)));
        int rc = copy_in(c, w.p, warp, size_t(wdof), IDW_HOST);
        if (rc) return rc;
        wp = w.p;
        sp = s.p;
    }
    if (sdof > 0) k_gather_dof<<<int((sdof + 255) / 256), 256, 0, c->stream>>>(sdof, c->solverInd.p, wp, sp);
    int rc = check_launch(c, "warp_to_solver");
    if (rc) return rc;
    if (where != IDW_DEVICE) return copy_out(c, solver, s.p, size_t(sdof), IDW_HOST);
    return IDW_OK;
}

int idw_solver_to_warp_grid(void *ctx, const double *solver, int64_t sdof, double *warp, int64_t wdof, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (c->nSolver < 0) return fail(c, IDW_ERR_STATE, "setExternalMeshIndices has not been called");
    if (wdof != 3 * c->nVol || sdof != c->nSolver) return fail(c, IDW_ERR_ARG, "size mismatch");
    CK(cudaSetDevice(c->device));
    DevBuf<double> w, s;
    const double *sp = solver;
    double *wp = warp;
    if (where != IDW_DEVICE) {
        CKA(w.alloc(size_t(wdof)));
        CKA(s.alloc(size_t(sdof)));
        int rc = copy_in(c, s.p, solver, size_t(sdof), IDW_HOST);
        if (rc) return rc;
        sp = s.p;
        wp = w.p;
    }
    CK(cudaMemsetAsync(wp, 0, sizeof(double) * wdof, c->stream));
    if (sdof > 0) k_scatter_add_dof<<<int((sdof + 255) / 256), 256, 0, c->stream>>>(sdof, c->solverInd.p, sp, wp);
    int rc = check_launch(c, "solver_to_warp");
    if (rc) return rc;
    if (where != IDW_DEVICE) return copy_out(c, warp, w.p, size_t(wdof), IDW_HOST);
    CK(cudaStreamSynchronize(c->stream));
    return IDW_OK;
}

int idw_get_tree(void *ctx, int32_t *nodeInfo, double *nodeGeom, double *nodeErr, double *nodeAi) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    CK(cudaSetDevice(c->device));
    const int nn = c->nNodes;
    if (nodeInfo) CK(cudaMemcpyAsync(nodeInfo, c->info.p, sizeof(int4) * nn, cudaMemcpyDeviceToHost, c->stream));
    if (nodeGeom) CK(cudaMemcpyAsync(nodeGeom, c->geom.p, sizeof(dbl4) * nn, cudaMemcpyDeviceToHost, c->stream));
    if (nodeErr) CK(cudaMemcpyAsync(nodeErr, c->nodeErr.p, sizeof(double) * kNerr * nn, cudaMemcpyDeviceToHost, c->stream));
    if (nodeAi) CK(cudaMemcpyAsync(nodeAi, c->nodeAi.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return IDW_OK;
}

int idw_get_surface_state(void *ctx, double *xu0, double *ai, double *normals0, int32_t *isCorner, int32_t *xuInd) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    CK(cudaSetDevice(c->device));
    const int n = c->nUnique;
    std::vector<dbl4> xa(n);
    CK(cudaMemcpyAsync(xa.data(), c->ptXA.p, sizeof(dbl4) * n, cudaMemcpyDeviceToHost, c->stream));
    if (normals0) CK(cudaMemcpyAsync(normals0, c->normals0.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    if (isCorner) CK(cudaMemcpyAsync(isCorner, c->isCorner.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    if (xuInd) CK(cudaMemcpyAsync(xuInd, c->xuInd.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < n; ++i) {
        if (xu0) {
            xu0[3 * i] = xa[i].x;
            xu0[3 * i + 1] = xa[i].y;
            xu0[3 * i + 2] = xa[i].z;
        }
        if (ai) ai[i] = xa[i].w;
    }
    return IDW_OK;
}

int idw_get_nodal_properties(void *ctx, double *mi, double *bi) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    CK(cudaSetDevice(c->device));
    if (!c->nodalValid) {
        int rc = refresh_nodal(c);
        if (rc) return rc;
    }
    const int n = c->nUnique;
    std::vector<double> mb(12 * size_t(n));
    CK(cudaMemcpyAsync(mb.data(), c->ptMB.p, sizeof(double) * 12 * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < n; ++i) {
        if (mi) std::memcpy(mi + 9 * i, &mb[12 * i], 9 * sizeof(double));
        if (bi) std::memcpy(bi + 3 * i, &mb[12 * i + 9], 3 * sizeof(double));
    }
    return IDW_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// warpDeriv without any allocation, for callers that cannot allocate device
// memory during the call.  Scratch lives in one file-scope device array whose
// address is looked up once per device; calls that overlap in time (two
// contexts, or two streams, at once) share it and race.
namespace {

constexpr size_t kNoAllocScratchDoubles = size_t(6) << 20;  // 48 MiB
static __device__ __align__(256) double g_noallocScratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_noallocMu;
double *g_noallocPtr[kMaxDevices] = {};

int noalloc_scratch(Ctx *c, double **out) {
    if (c->device < 0 || c->device >= kMaxDevices) return fail(c, IDW_ERR_LIMIT, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noallocMu);
    if (!g_noallocPtr[c->device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) return fail(c, IDW_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        g_noallocPtr[c->device] = static_cast<double *>(p);
    }
    *out = g_noallocPtr[c->device];
    return IDW_OK;
}

}  // namespace

extern "C" {

int idw_warp_deriv_noalloc(void *ctx, const double *dxv, int64_t ndof, double *dxs, int64_t cdof) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (int e0 = ensure_den0(c)) return e0;
    if (!c->haveWarp) return fail(c, IDW_ERR_STATE, "warpMesh must be called before warpDeriv");
    if (!dxv || !dxs) return fail(c, IDW_ERR_ARG, "null dXv or dXs");
    if (ndof != 3 * c->nVol)
        return fail(c, IDW_ERR_ARG, "dXv has %lld entries, expected %lld", (long long)ndof, (long long)(3 * c->nVol));
    if (cdof != 3 * int64_t(c->nPts))
        return fail(c, IDW_ERR_ARG, "dXs has %lld entries, expected %lld", (long long)cdof,
                    (long long)(3 * int64_t(c->nPts)));
    const int n = c->nUnique, nn = c->nNodes;
    const int mixed = c->opt.precision == IDW_PREC_MIXED;
    const size_t need = 12 * size_t(n) + 12 * size_t(nn) + (mixed ? 12 * size_t(n) : 0);
    if (need > kNoAllocScratchDoubles)
        return fail(c, IDW_ERR_LIMIT,
                    "warpDeriv without allocation needs %zu scratch doubles for %d surface nodes and %d tree nodes; "
                    "the static scratch holds %zu",
                    need, n, nn, kNoAllocScratchDoubles);
    CK(cudaSetDevice(c->device));
    double *scratch = nullptr;
    int rc = noalloc_scratch(c, &scratch);
    if (rc) return rc;
    double *ptAdj = scratch, *nodeAdj = scratch + 12 * size_t(n), *ptRel = nodeAdj + 12 * size_t(nn);
    rc = refresh_nodal(c);
    if (rc) return rc;
    EvalConsts k;
    k.law = make_law(c);
    k.errTol = c->opt.errTol;
    k.sym = c->sym;
    k.slotStats = 0;
    k.exactSchedule = c->opt.exactSchedule;
    k.precGate = 0.0;
    const int exact = c->opt.evalMode == IDW_EVAL_EXACT;
    // the accumulators start at zero
    CK(cudaMemsetAsync(ptAdj, 0, sizeof(double) * 12 * size_t(n), c->stream));
    CK(cudaMemsetAsync(nodeAdj, 0, sizeof(double) * 12 * size_t(nn), c->stream));
    CK(cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream));
    if (mixed) {
        const TreeDevF tf = tree_devf(c);
        PointsDevF pf;
        pf.da = c->ptDA.p;
        pf.dl = c->ptDL.p;
        pf.dm = c->ptDM.p;
        pf.dml = c->ptDMl.p;
        WalkRecF rec;
        rec.hi = c->recHi.p;
        rec.lo = c->recLo.p;
        launch_adjoint_mixed(tree_dev(c), tf, pf, vol_dev(c), rec, k, exact, dxv, 1, ndof, c->den.p, ptAdj, nodeAdj,
                             ptRel, c->ptXA.p, n, c->counters.p, c->stream);
    } else {
        PointsDev p;
        p.xa = c->ptXA.p;
        p.mb = c->ptMB.p;
        launch_walk_adjoint_fp64(tree_dev(c), p, vol_dev(c), k, exact, n, dxv, c->den.p, 1, ndof, ptAdj, nodeAdj,
                                 int64_t(12) * n, int64_t(12) * nn, c->counters.p, c->stream);
        launch_set_data_b(tree_dev(c), nodeAdj, ptAdj, n, c->stream);
    }
    rc = check_launch(c, "adjoint walk");
    if (rc) return rc;
    CK(cudaMemsetAsync(c->xub.p, 0, sizeof(double) * 3 * size_t(n), c->stream));
    launch_nodal_b(surf_dev(c), c->xu.p, c->ptXA.p, c->normals0.p, c->isCorner.p, c->opt.useRotations,
                   mixed ? ptRel : ptAdj, mixed, c->xub.p, c->stream);
    CK(cudaMemsetAsync(dxs, 0, sizeof(double) * size_t(cdof), c->stream));
    launch_scatter_dxs(n, c->xuInd.p, c->xub.p, dxs, c->stream);
    return check_launch(c, "reverse nodal properties");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// A small autotuner for the two launch shapes that are free at run time: the
// number of surfaces that share one batched walk and the number of seeds that
// share one adjoint walk.  Each candidate is timed once (after one warm-up) on
// the context's own mesh and current surface.
namespace {
__global__ void k_fill(int64_t n, double v, double *x) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) x[i] = v * double(1 + (i % 7));
}
}  // namespace

extern "C" {

int idw_autotune(void *ctx, int32_t nsurfaces, int32_t nseeds, idw_tuning *out) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveWarp) return fail(c, IDW_ERR_STATE, "warpMesh must be called before idw_autotune");
    if (nsurfaces < 1 || nseeds < 1 || !out) return fail(c, IDW_ERR_ARG, "bad autotune arguments");
    if (c->opt.precision != IDW_PREC_MIXED) return fail(c, IDW_ERR_STATE, "the tuned launches are the mixed ones");
    CK(cudaSetDevice(c->device));
    std::memset(out, 0, sizeof(*out));
    const size_t sdof = 3 * size_t(c->nPts), vdof = 3 * size_t(c->nVol);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    auto timed = [&](auto &&fn, float &ms) -> int {
        int rc = fn();  // warm-up (and growth of any buffers)
        if (rc) return rc;
        CK(cudaEventRecord(e0, c->stream));
        rc = fn();
        if (rc) return rc;
        CK(cudaEventRecord(e1, c->stream));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        return IDW_OK;
    };
    int rc = IDW_OK;
    {
        // batched walk: the current surface, nsurfaces times
        DevBuf<double> xs, xv;
        CKA(xs.alloc(size_t(nsurfaces) * sdof));
        CKA(xv.alloc(size_t(kBatchMax) * vdof));
        for (int b = 0; b < nsurfaces; ++b)
            CK(cudaMemcpyAsync(xs.p + size_t(b) * sdof, c->xs.p, sdof * sizeof(double), cudaMemcpyDeviceToDevice,
                               c->stream));
        float best = 0.f;
        for (int G = 1; G <= kBatchMax && G <= 4; ++G) {
            float ms = 0.f;
            rc = timed([&]() {
                for (int b0 = 0; b0 < nsurfaces; b0 += G) {
                    const int nb = std::min(G, nsurfaces - b0);
                    int r = run_warp_batch_mixed(c, xs.p + size_t(b0) * sdof, nb, xv.p);
                    if (r) return r;
                }
                return int(IDW_OK);
            }, ms);
            if (rc) break;
            out->batchMs[G - 1] = ms;
            if (G == 1 || ms < best) {
                best = ms;
                out->batchGroup = G;
            }
        }
    }
    if (!rc) {
        // adjoint: seed groups of at most 16, 8 or 4
        DevBuf<double> seeds, dxs;
        CKA(seeds.alloc(size_t(nseeds) * vdof));
        CKA(dxs.alloc(size_t(nseeds) * sdof));
        const int64_t nd = int64_t(nseeds) * int64_t(vdof);
        if (nd > 0) k_fill<<<int((nd + 255) / 256), 256, 0, c->stream>>>(nd, 1e-3, seeds.p);
        const int groups[3] = {16, 8, 4};
        float best = 0.f;
        const int keep = c->adjMaxGroup;
        // the seed groups are those of the FP32 form of the adjoint (the
        // double-float form has its own fixed groups of 16, 4 and 1)
        const int keepPrec = c->opt.adjointPrecision;
        c->opt.adjointPrecision = IDW_ADJ_FAST;
        for (int q = 0; q < 3; ++q) {
            c->adjMaxGroup = groups[q];
            float ms = 0.f;
            rc = timed([&]() { return run_deriv(c, seeds.p, nseeds, int64_t(vdof), dxs.p, IDW_DEVICE, int64_t(sdof)); },
                       ms);
            if (rc) break;
            out->adjMs[q] = ms;
            if (q == 0 || ms < best) {
                best = ms;
                out->adjMaxGroup = groups[q];
            }
        }
        c->adjMaxGroup = rc ? keep : out->adjMaxGroup;
        c->opt.adjointPrecision = keepPrec;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    c->batchGroup = out->batchGroup;
    CK(cudaStreamSynchronize(c->stream));
    return IDW_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// warpDerivFwd for several tangent directions: in mixed precision up to four
// directions share one walk (the weights do not depend on the surface), in
// FP64 one walk per direction.
extern "C" {

int idw_warp_deriv_fwd_batch(void *ctx, const double *dxs, int32_t ndir, double *dxv, int where) {
    Ctx *c = static_cast<Ctx *>(ctx);
    if (!c) return IDW_ERR_ARG;
    if (!c->haveTree) return fail(c, IDW_ERR_STATE, "setSurfaceDefinition must come first");
    if (int e0 = ensure_den0(c)) return e0;
    if (!c->haveWarp) return fail(c, IDW_ERR_STATE, "warpMesh must be called before warpDerivFwd");
    if (ndir < 0 || !dxs || !dxv) return fail(c, IDW_ERR_ARG, "bad tangent arguments");
    CK(cudaSetDevice(c->device));
    const size_t sdof = 3 * size_t(c->nPts), vdof = 3 * size_t(c->nVol);
    if (where != IDW_DEVICE && !all_finite(dxs, size_t(ndir) * sdof))
        return fail(c, IDW_ERR_NONFINITE, "non-finite dXs");
    const int G = c->opt.precision == IDW_PREC_MIXED ? std::max(1, std::min(c->batchGroup, kBatchWalk)) : 1;
    DevBuf<double> tin, tout;
    if (where != IDW_DEVICE) {
        CKA(tin.alloc(size_t(std::min<int>(ndir, G)) * sdof));
        CKA(tout.alloc(size_t(std::min<int>(ndir, G)) * vdof));
    }
    for (int b0 = 0; b0 < ndir; b0 += G) {
        const int nb = std::min(G, int(ndir) - b0);
        const double *in = dxs + size_t(b0) * sdof;
        double *out = dxv + size_t(b0) * vdof;
        if (where != IDW_DEVICE) {
            int rc = copy_in(c, tin.p, in, size_t(nb) * sdof, IDW_HOST);
            if (rc) return rc;
            in = tin.p;
            out = tout.p;
        }
        int rc;
        if (c->opt.precision == IDW_PREC_MIXED) {
            // the gate scales with the largest tangent of the group
            CK(cudaMemsetAsync(c->counters.p + 7, 0, sizeof(unsigned long long), c->stream));
            const int64_t nd = int64_t(nb) * int64_t(sdof);
            k_absmax<<<int((nd + 255) / 256), 256, 0, c->stream>>>(nd, in, c->counters.p + 7);
            unsigned long long bits = 0;
            CK(cudaMemcpyAsync(&bits, c->counters.p + 7, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            double scale;
            std::memcpy(&scale, &bits, sizeof(scale));
            CK(cudaMemsetAsync(c->counters.p, 0, 8 * sizeof(unsigned long long), c->stream));
            rc = run_warp_batch_mixed(c, in, nb, out, 1, c->opt.mixedGate * scale);
        } else {
            rc = run_deriv_fwd(c, in, out);
        }
        if (rc) return rc;
        if (where != IDW_DEVICE) {
            rc = copy_out(c, dxv + size_t(b0) * vdof, tout.p, size_t(nb) * vdof, IDW_HOST);
            if (rc) return rc;
        }
    }
    CK(cudaStreamSynchronize(c->stream));
    return IDW_OK;
}

}  // extern "C"
