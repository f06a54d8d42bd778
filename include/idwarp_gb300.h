/*
 * idwarp_gb300.h — C ABI of the GB300 inverse-distance-weighted mesh-warping
 * library (libidwarp_gb300.so).
 *
 * This ABI replaces the f2py module `libidwarp` of IDWarp (mdolab/idwarp,
 * src/f2py/libidwarp.pyf) for the warping path: one opaque context per mesh
 * instance (the reference instead copies the shared object per instance,
 * idwarp/MExt.py:34-55), plain pointers and sizes, an int status on every
 * call (0 = success, negative = error; the message is available through
 * idw_last_error).  The reference aborts the MPI job on error
 * (src/utils/EChk.F90:13-23).
 *
 * Coordinates are xyz-interleaved doubles, i.e. a C-order (N,3) array, which
 * is the Fortran (3,N) layout the reference uses.  Index arrays are 0-based
 * int32 except `link`, which is 1-based as in the reference.
 *
 * Pointers marked `where` may be host (IDW_HOST) or CUDA device (IDW_DEVICE)
 * memory on the context's device.  All work is issued on the context's CUDA
 * stream (idw_set_stream); calls taking host buffers synchronise that stream
 * before returning.
 *
 * Thread safety: distinct contexts may be used from different threads; one
 * context must not be used concurrently.
 */
#ifndef IDWARP_GB300_H
#define IDWARP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IDW_OK 0
#define IDW_ERR_ARG -1       /* bad argument (size mismatch, null pointer, bad option) */
#define IDW_ERR_STATE -2     /* call made in the wrong order */
#define IDW_ERR_CUDA -3      /* a CUDA runtime call failed */
#define IDW_ERR_NONFINITE -4 /* non-finite coordinates detected */
#define IDW_ERR_LIMIT -5     /* a fixed limit was exceeded (face size, symmetry planes) */
#define IDW_ERR_NOMEM -6     /* device allocation failed */
#define IDW_ERR_RESTART -7   /* a loaded denominator estimate failed its check (idw_set_denominator0) */

#define IDW_HOST 0
#define IDW_DEVICE 1

#define IDW_EVAL_EXACT 0 /* gridInput.f90:16 EVAL_EXACT */
#define IDW_EVAL_FAST 1  /* gridInput.f90:17 EVAL_FAST */

#define IDW_PREC_FP64 0  /* FP64 throughout (the plain form) */
#define IDW_PREC_MIXED 1 /* FP32 distances/weights/accumulation, FP64 set-up and normalisation */

#define IDW_EXACT_AUTO 0  /* exact-mode schedule chosen by mesh size */
#define IDW_EXACT_TILED 1 /* shared-memory tiles of surface points, several volume nodes per thread */
#define IDW_EXACT_WALK 2  /* the tree walk with every node opened */

#define IDW_ADJ_PRECISE 0 /* mixed warpDeriv in double-float (FP32 pairs): terms, products and lane sums */
#define IDW_ADJ_FAST 1    /* mixed warpDeriv with FP32 weights, products and lane sums */

#define IDW_WALK_LISTS_AUTO 0 /* mixed fast mode: record the walk's decisions once and replay them
                               * (when the lists fit in half of the free device memory) */
#define IDW_WALK_LISTS_OFF 1  /* every walk takes its decisions as it goes */

#define IDW_TREE_KD 0     /* the reference's surface kd tree (build_tree, src/modules/kd_tree.F90:123-300),
                           * built on the host: every fast-mode decision as the reference's */
#define IDW_TREE_MORTON 1 /* binary radix tree over Morton-ordered surface points, built on the GPU and cut
                           * at bucketSize+1 points; same aggregates, other clusters: fast-mode results
                           * differ from the kd tree's within what errTol allows */

/* Mesh options: the gridinput module variables (src/modules/gridInput.f90:9-18,
 * libidwarp.pyf:148-162) plus kd_tree.bucket_size (libidwarp.pyf:204-206) and
 * the GB300 precision switch.  Semantics follow doc/options.yaml. */
typedef struct idw_options {
    double aExp;          /* default 3 */
    double bExp;          /* default 5 */
    double LdefFact;      /* default 1 */
    double alpha;         /* default 0.25 */
    double errTol;        /* default 5e-4 */
    double symmTol;       /* default 1e-6 (kept for API parity) */
    double cornerAngle;   /* default 30 (degrees) */
    int32_t evalMode;     /* IDW_EVAL_FAST (default) or IDW_EVAL_EXACT */
    int32_t useRotations; /* default 1 */
    int32_t zeroCornerRotations; /* default 1 */
    int32_t bucketSize;   /* default 8 */
    int32_t precision;    /* IDW_PREC_MIXED (default) or IDW_PREC_FP64 */
    int32_t diagnostics;  /* bit 0: count warp-level lane slots in idw_stats */
    double mixedGate;     /* mixed mode: a term w (|S'| + |D'| |r - X|) larger than
                           * mixedGate * Ldef0 * den (times 2/nLoop beyond one symmetry
                           * plane) is summed in double-float (S' = the term's motion
                           * less the mean surface motion, den = the node's
                           * denominator; default 2e-3; 0 = every term) */
    int32_t exactSchedule; /* mixed exact mode: IDW_EXACT_AUTO (default: tiled
                            * kernel when the mesh fills the GPU, else the walk),
                            * IDW_EXACT_TILED or IDW_EXACT_WALK; same sums either way */
    int32_t adjointPrecision; /* mixed warpDeriv: IDW_ADJ_PRECISE (default) or
                               * IDW_ADJ_FAST (FP32 terms, a few 1e-7 relative per
                               * term; real-valued exponents always use FP32) */
    int32_t walkLists;    /* IDW_WALK_LISTS_AUTO (default) or IDW_WALK_LISTS_OFF: the fast
                           * walk's open/approximate decisions depend on the set-up state
                           * and errTol only, so they can be recorded once (per warp of 32
                           * volume nodes: the tree nodes where a lane approximates or sums
                           * a leaf) and replayed by every later warp; same sums either way */
    int32_t treeBuild;    /* IDW_TREE_KD (default) or IDW_TREE_MORTON; read by
                           * idw_initialize_warping, as bucketSize */
    int32_t deterministic; /* 0 (default): reverse products (idw_warp_deriv*) land their sums with
                            * FP64 atomics, whose order varies from run to run; 1: every scattering
                            * stage runs twice and lands order-independent 192-bit fixed-point sums,
                            * so dXs is the same bit for bit on every run (about twice the time;
                            * such calls are serialised within the process, wait for the stream and
                            * refuse stream capture (IDW_ERR_STATE); idw_warp_deriv_noalloc keeps the
                            * atomics).  The forward calls are deterministic either way. */
    int32_t reserved[2];
} idw_options;

/* Work counters of the last warp / warpDeriv call. */
typedef struct idw_stats {
    int64_t leafPairs;    /* exact (volume node, surface node) pair evaluations */
    int64_t approx;       /* cluster approximations */
    int64_t visited;      /* tree nodes whose decision was evaluated */
    int64_t fp64Fallback; /* mixed mode: decisions re-evaluated in FP64 */
    int64_t nUnique;      /* unique surface nodes */
    int64_t nTreeNodes;
    int64_t maxDepth;
    int64_t nVol;
    int64_t nSurfPts;
    int64_t nLoop;
    double Ldef0;
    double lastKernelMs;  /* device time of the last evaluation kernel(s) */
    int64_t warpLeafSlots; /* lane slots of warp-level leaf visits (32 x leaf size); leafPairs / this = lane use */
    int64_t warpNodeSlots; /* lane slots of warp-level interior-node visits (32 per visit) */
    int64_t preciseTerms;  /* mixed mode: cluster terms summed in double-float */
    int64_t walkListEntries; /* recorded walk decisions (8 bytes each; -1: too large, walks decide) */
    double treeBuildMs;   /* host wall time of the last surface tree build (kd or Morton, with its copies) */
} idw_stats;

/* Fill `o` with the reference defaults (idwarp/UnstructuredMesh.py:124-145). */
void idw_default_options(idw_options *o);

/* Create / destroy a context on the current CUDA device.  (replaces MExt +
 * initpetsc, idwarp/UnstructuredMesh.py:93-99, libidwarp.pyf:10-12) */
int idw_create(const idw_options *opts, void **ctx_out);
int idw_destroy(void *ctx);

/* Copy the last error message (NUL-terminated, truncated to len). */
int idw_last_error(void *ctx, char *buf, int len);

/* Use `stream` (a cudaStream_t, NULL = default stream) for all later work. */
int idw_set_stream(void *ctx, void *stream);
int idw_synchronize(void *ctx); /* also waits for asynchronous grid reads */

/* Update options (UnstructuredMesh.py:1051-1069 _setMeshOptions).  As in the
 * reference, aExp/bExp/bucketSize/cornerAngle/zeroCornerRotations take effect
 * only at the next idw_initialize_warping; LdefFact, alpha, errTol, evalMode,
 * useRotations and precision take effect at the next warp. */
int idw_set_options(void *ctx, const idw_options *opts);

/* Volume grid in common (file) order.  (createcommongrid, libidwarp.pyf:14-17,
 * src/IO/createGrid.F90) */
int idw_create_common_grid(void *ctx, const double *volnodes, int64_t nvol, int where);

/* Symmetry planes, at most 6.  (setsymmetryplanes, libidwarp.pyf:69-73,
 * src/warp/initializeWarping.F90:511-531) */
int idw_set_symmetry_planes(void *ctx, const double *pts, const double *normals, int32_t n);

/* Merge surface points within tol (squared distance <= tol^2).  uniquepts
 * (n,3) and link (n, 1-based) are caller-allocated.  (pointreduce,
 * libidwarp.pyf:195-202, src/utils/pointReduce.F90:1-83) */
int idw_point_reduce(const double *pts, int32_t n, double tol, double *uniquepts, int32_t *link,
                     int32_t *nunique);

/* Build the surface tree, nodal-property state, error tables and the
 * denominator estimate.  pts are this process's surface points (n,3, caller
 * order with duplicates); uniquepts are the lexsorted unique points, link maps
 * every point to its unique point (1-based).  faceConn is 0-based into pts.
 * (initializewarping, libidwarp.pyf:55-67, src/warp/initializeWarping.F90:1-247,
 * src/modules/kd_tree.F90:1365-1545) */
int idw_initialize_warping(void *ctx, const double *pts, int32_t npts, const double *uniquepts, int32_t nunique,
                           const int32_t *link, const int32_t *faceSizes, int32_t nfaces,
                           const int32_t *faceConn, int32_t nconn);

/* Surface coordinates (cdof = 3*npts).  (setsurfacecoordinates /
 * getsurfacecoordinates, libidwarp.pyf:78-86) */
int idw_set_surface_coordinates(void *ctx, const double *coords, int64_t cdof, int where);
int idw_get_surface_coordinates(void *ctx, double *coords, int64_t cdof, int where);

/* Warp the volume mesh to the current surface.  (warpmesh, libidwarp.pyf:75,
 * src/warp/warpMesh.F90:1-82) */
int idw_warp_mesh(void *ctx);

/* Complex step: the counterpart of the reference's complexified library
 * (libidwarp_cs, loaded by idwarp/UnstructuredMesh_C.py; its
 * setsurfacecoordinates / warpmesh / getvolumecoordinates take complex
 * arrays).  coords holds 2*cdof doubles, the caller's (npts,3) complex
 * coordinates with real and imaginary parts interleaved (numpy complex128
 * layout); out receives 2*ndof doubles of the warped grid the same way.
 * FP64 precision only (IDW_ERR_STATE otherwise).  The real part is the
 * ordinary warp of the real coordinates; the imaginary part propagates the
 * imaginary coordinates through the nodal properties in complex arithmetic
 * and through the (linear) weighted sums of the same walk. */
int idw_set_surface_coordinates_cs(void *ctx, const double *coords, int64_t cdof, int where);
int idw_warp_mesh_cs(void *ctx);
int idw_get_volume_coordinates_cs(void *ctx, double *out, int64_t ndof, int where);

/* Warp nbatch surfaces (perturbations of the same surface definition) in one
 * call: coords holds nbatch stacked (npts,3) surfaces, out receives nbatch
 * stacked (nvol,3) grids.  In mixed precision up to four surfaces share one
 * tree walk (decisions and weights computed once); in FP64 the surfaces are
 * warped one after the other.  The context's stored surface/grid are left
 * unchanged.  No reference counterpart. */
int idw_warp_mesh_batch(void *ctx, const double *coords, int32_t nbatch, double *out, int where);

/* Current volume grid in warp order (== common order on one GPU).
 * (getvolumecoordinates, libidwarp.pyf:45-48; getcommonvolumecoordinates
 * :50-53) */
int idw_get_volume_coordinates(void *ctx, double *out, int64_t ndof, int where);
/* idw_get_volume_coordinates into host memory without waiting: the copy is
 * queued on a copy stream of the context behind the work queued so far and
 * overlaps whatever is queued next (e.g. the next warp, which then writes a
 * second device buffer).  out is complete after idw_synchronize; for the copy
 * to run asynchronously it should be page-locked (cudaHostAlloc, torch
 * pin_memory).  No reference counterpart (getvolumecoordinates,
 * libidwarp.pyf:45-48, returns when the copy is done). */
int idw_get_volume_coordinates_async(void *ctx, double *out, int64_t ndof);
int idw_get_common_volume_coordinates(void *ctx, double *out, int64_t ndof, int where);
/* (setvolumecoordinates, src/warp/getVolumeCoordinates.F90:25-46) */
int idw_set_volume_coordinates(void *ctx, const double *in, int64_t ndof, int where);

/* Solver ordering: ind are 0-based DOF indices into the common grid.
 * (setexternalmeshindices, libidwarp.pyf:40-43, src/warp/setExternalMeshIndices.F90)
 * warp->solver is a gather; solver->warp is a scatter-add
 * (src/warp/gridTransform.F90:4-99). */
int idw_set_external_mesh_indices(void *ctx, const int32_t *ind, int64_t ndof_solver);
int idw_get_solver_mesh_dof(void *ctx, int64_t *ndof);
int idw_warp_to_solver_grid(void *ctx, const double *warp, int64_t wdof, double *solver, int64_t sdof, int where);
int idw_solver_to_warp_grid(void *ctx, const double *solver, int64_t sdof, double *warp, int64_t wdof, int where);

/* Reverse derivative dXs = (dXv/dXs)^T dXv using the denominator of the last
 * idw_warp_mesh; fetch the result with idw_get_dxs.  (warpderiv,
 * libidwarp.pyf:102-105, src/warp/warpDeriv.F90:1-131; getdxs :114-117) */
int idw_warp_deriv(void *ctx, const double *dxv, int64_t ndof, int where);
int idw_get_dxs(void *ctx, double *out, int64_t ndof, int where);

/* nseeds reverse derivatives in one launch sharing the tree walk: dxv holds
 * nseeds stacked (nvol,3) seeds, dxs receives nseeds stacked (npts,3). */
int idw_warp_deriv_batch(void *ctx, const double *dxv, int32_t nseeds, double *dxs, int where);

/* Forward-mode (tangent) product dXv = (dXv/dXs) dXs.  Replaces the f2py
 * entry warpderivfwd(xsdot, outvec) (src/f2py/libidwarp.pyf:107-112;
 * src/warp/warpDerivFwd.F90:1-111): dxs (npts,3) in the caller's surface
 * order, dxv (nvol,3) in warp (common) order, both on the host or both on
 * the device (where).  Needs a prior idw_warp_mesh; the derivative numerator
 * is divided by that warp's denominator. */
int idw_warp_deriv_fwd(void *ctx, const double *dxs, int64_t cdof, double *dxv, int64_t ndof, int where);

/* idw_warp_deriv_fwd for ndir tangent directions: dxs holds ndir stacked
 * (npts,3) tangents, dxv receives ndir stacked (nvol,3) products.  In mixed
 * precision up to four directions share one tree walk.  No reference
 * counterpart (the reference takes one direction per call). */
int idw_warp_deriv_fwd_batch(void *ctx, const double *dxs, int32_t ndir, double *dxv, int where);

/* idw_warp_deriv for one seed without allocating device memory in the call
 * (in mixed precision its FP32 form, IDW_ADJ_FAST: the double-float form's
 * denominator array would need an allocation),
 * for callers that cannot allocate while they run (memory reserved up front,
 * allocation-free solver loops).  No reference counterpart.  dxv (nvol,3)
 * and dxs (npts,3, receives the result) are device pointers; the work is
 * ordered on the context's stream and not synchronised.  Scratch is one
 * static 48 MiB device array shared by every context of the process:
 * 12 doubles per unique surface node and per tree node, plus 12 per surface
 * node in mixed precision, must fit in 6*2^20 doubles (with bucketSize 8
 * about 210k unique surface nodes in mixed precision, 360k in FP64), else
 * IDW_ERR_LIMIT.  The array belongs to the library's device code, so every
 * process that loads libidwarp_gb300.so holds those 48 MiB on each device it
 * uses the library on, until it exits, whether or not it ever calls this
 * entry point.  Calls that overlap in time
 * (several contexts or streams at once) race on that scratch.  The first
 * call on a device looks the scratch up (cudaGetSymbolAddress): make it
 * before any stream capture. */
int idw_warp_deriv_noalloc(void *ctx, const double *dxv, int64_t ndof, double *dxs, int64_t cdof);

/* Denominator estimate denominator0 (nvol), in common order.
 * (initializeWarping.F90:241-247) */
int idw_get_denominator0(void *ctx, double *out, int64_t nvol, int where);

/* The denominator estimate is computed at the first walk after
 * idw_initialize_warping unless it was computed or loaded before.
 * idw_compute_denominator0 computes it now (the reference does so during
 * initializewarping, initializeWarping.F90:241-247).  */
int idw_compute_denominator0(void *ctx);

/* Load denominator0 (nvol, common order) in place of computing it: the
 * restart-file path of initializeWarping.F90:124-228.  The common-order nodes
 * 0, checkStride, 2 checkStride, ... (the reference checks every 100th) are
 * re-estimated first; if any has 1 - estimate/loaded > 1e-15 the load is
 * refused with IDW_ERR_RESTART and the context is left as it was, otherwise
 * the loaded values replace the estimate and a previous warp is forgotten
 * (warpMesh must run again before warpDeriv).  checkStride <= 0 skips the
 * check.  Non-finite values are refused (IDW_ERR_NONFINITE) when where is
 * IDW_HOST. */
int idw_set_denominator0(void *ctx, const double *den0, int64_t nvol, int64_t checkStride, int where);

/* Load-balancing cost of every volume node (nvol, common order): dryRun
 * (kd_tree.F90:789-830) summed over the mirrors and divided by the number of
 * unique surface points, as initializeWarping.F90:258-266 accumulates it and
 * the restart file stores it.  Uses the denominator estimate in force. */
int idw_dry_run_costs(void *ctx, double *costs, int64_t nvol, int where);

/* Denominator sum(w) of the last idw_warp_mesh (nvol), in common order; the
 * reference's module variable `denominator` (src/warp/warpMesh.F90:59-70),
 * used by idw_warp_deriv. */
int idw_get_denominator(void *ctx, double *out, int64_t nvol, int where);

/* Counters of the last call. */
int idw_get_stats(void *ctx, idw_stats *out);

/* Tree / nodal-property state for inspection (tree order, preorder nodes).
 * nodeInfo: 4 ints per node (l, u, escape, isLeaf); nodeGeom: 4 doubles per
 * node (X, oradius); nodeErr: 12 per node; nodeAi: 1 per node.
 * Surface: Xu0 (3), Ai, normals0 (3), isCorner, XuInd per unique node. */
int idw_get_tree(void *ctx, int32_t *nodeInfo, double *nodeGeom, double *nodeErr, double *nodeAi);
int idw_get_surface_state(void *ctx, double *xu0, double *ai, double *normals0, int32_t *isCorner,
                          int32_t *xuInd);
/* Per-unique-node rotation Mi (9, row-major) and translation Bi (3) of the
 * current surface (computeNodalProperties, kd_tree.F90:1580-1664). */
int idw_get_nodal_properties(void *ctx, double *mi, double *bi);

/* Launch shapes chosen by idw_autotune, and the candidates' times. */
typedef struct idw_tuning {
    int32_t batchGroup;  /* surfaces per batched walk (1..4) */
    int32_t adjMaxGroup; /* largest seed group per walk of the FP32 adjoint (16, 8 or 4) */
    double batchMs[4];   /* nsurfaces warps with 1..4 surfaces per walk */
    double adjMs[3];     /* nseeds reverse products with groups of 16, 8, 4 */
    int32_t reserved[4];
} idw_tuning;

/* Time the run-time launch shapes of the mixed form on this context's mesh
 * and current surface (nsurfaces surfaces for idw_warp_mesh_batch, nseeds
 * seeds for idw_warp_deriv_batch) and keep the fastest for later calls.
 * Needs a prior idw_warp_mesh in mixed precision.  No reference counterpart. */
int idw_autotune(void *ctx, int32_t nsurfaces, int32_t nseeds, idw_tuning *out);

/* Diagnostic: measured FP32 FFMA throughput of the current device (TFLOP/s),
 * the denominator of the mixed walk's roofline.  No reference counterpart. */
int idw_probe_ffma(void *stream, int device, double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* IDWARP_GB300_H */
