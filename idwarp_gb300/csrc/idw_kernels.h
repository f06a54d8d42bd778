// Device-side views and kernel launchers of the GB300 IDW warping library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "idw_common.cuh"

namespace idw {

// Surface connectivity in tree order (CSR), read-only after set-up.
struct SurfaceDev {
    int n;               // unique surface nodes
    const int *facePtr;  // nFaces+1
    const int *faceConn; // tree-order vertex ids
    const int *n2ePtr;   // n+1
    const int *n2e;      // node -> face ids (one entry per occurrence)
    int nFaces = 0;
    double *faceScratch = nullptr;  // 8 per face: area and unit normal of the current surface (4 nFaces),
                                    // then their adjoints (4 nFaces)
};

// Tree nodes in preorder.  info = (l, u, escape, isLeaf).
struct TreeDev {
    int nNodes;
    const int4 *info;
    const dbl4 *geom;  // X, oradius
    const double *err;    // 12 per node
    const double *ai;     // per node
    const int *parent = nullptr;  // per node: parent index, -1 at the root
};

// Scratch of the bottom-up cluster sums: 12 doubles and one arrival counter per node.
struct SetDataScratch {
    double *sum;
    unsigned *flags;
};

// Everything the mixed walks read at a tree node, packed in one 128-byte
// record (one cache line per visit).  Set-up constant.
struct __align__(128) NodeRecF {
    int4 info;       // l, u, escape, isLeaf (as TreeDev::info)
    float4 cHi;      // centroid high part, oradius
    float4 cLo;      // centroid low part, node area A (high part)
    float err[12];   // error table (true weight units)
    float aLo;       // node area A, low part
    float pad[7];
};

struct TreeDevF {
    const NodeRecF *nodes;
    // leaves in preorder: (l, u, node, 0); their point ranges tile [0, n)
    const int4 *leaves = nullptr;
    int nLeaves = 0;
    int nPts = 0;  // unique surface points (tree order)
};

// Surface point data for the evaluation kernels, tree order.
struct PointsDev {
    const dbl4 *xa;   // Xu0, Ai (FP64)
    const double *mb;    // 12 per point: M row-major, b
};

struct PointsDevF {
    const float4 *da;    // Xu0 - centroid(leaf) high part, Ai  (FP32, set-up constant)
    const float4 *dl;    // Xu0 - centroid(leaf) low part, Ai low part
    const float *dm;     // 12 per point: D' = M - I - Dref (9), u' = S'(Xu0) (3), high parts
    const float *dml;    // the same, low parts
};

// Per volume node (Morton order) and mirror: FP32 walk records.
struct WalkRecF {
    const float4 *hi;  // mirrored point, high part; denominator estimate (FP32)
    const float4 *lo;  // mirrored point, low part; scale exponent s (int bits)
    const float *gden = nullptr;  // per node: the walk's own scaled denominator (precision gate), or null
};

struct MixedParams {
    int nLoop, nSym;
    float nrm[kMaxSym][3], nrmLo[kMaxSym][3];
    float LdefF, alphaToBexpF, errTolF;
    double errTol;
    int intExp, dExp;
    float dExpF;
    int slotStats;  // count warp-level lane slots (diagnostics)
    float LdefLo, abH, abL, precGate;
    double bExp;
    float bExpF;
};

struct NodeAggF {
    const float *dc;     // 12 per node: D' = Mbar - I - Dref (9), c' = S'(X) (3), high parts
    const float *dcl;    // the same, low parts
    const float *dn;     // per node: bound on |D'| (max absolute row sum)
    const float *ref;    // reference motion Dref (9), bref (3): high parts, then low parts
    // per node, what a replayed step reads, in one 128-byte record (8 float4):
    // (cHi.xyz, dn), (cLo.xyz, area; a leaf: first point as int bits),
    // dc high parts (12 floats; a leaf: last point as int bits in .x),
    // (leaf flag as int bits, 0, 0, 0), pad
    const float4 *rr = nullptr;
};

struct VolumeDev {
    int64_t nVol;
    const int *perm;       // Morton order -> common index
    const double *xv0;     // (nVol,3) common order
    const double *den0;    // denominator0, common order
};

struct WalkOut {
    double *xv = nullptr;            // (nVol,3) or nullptr
    double *den = nullptr;           // (nVol) true-unit denominators or nullptr
    unsigned long long *counters = nullptr;  // leafPairs, approx, visited, fp64Fallback, ...
    // tangent mode (warpDerivFwd): xv receives num/denIn, without Xv0
    int tangent = 0;
    const double *denIn = nullptr;
};

// Recorded decisions of the mixed fast walk (idw_replay.cu): per warp of 32
// volume nodes and mirror, the tree nodes where some lane approximates or sums
// a leaf, with the lane mask; null when the walks decide as they go.
struct WalkLists {
    const int64_t *offs = nullptr;   // warps x nLoop + 1 entry offsets
    const int2 *list = nullptr;      // entries {node | 0x80000000 for a leaf, lane mask}
    const unsigned long long *counters = nullptr;  // the recording walk's leafPairs, approx, visited, fp64Fallback
};

struct EvalConsts {
    WeightLaw law;
    double errTol;
    SymPlanes sym;
    int slotStats;
    double precGate;  // mixed walk: weight x lever-arm threshold for double-float cluster terms
    int exactSchedule = 0;  // IDW_EXACT_AUTO / _TILED / _WALK (mixed exact mode)
    WalkLists lists;        // fast mode: replay these decisions when set
};

// Nodal properties (idw_nodal.cu)
void launch_gather_xu(int n, const int *xuInd, const double *Xs, double *Xu, cudaStream_t st);
void launch_nodal_init(const SurfaceDev &s, const double *Xu, double *normals0, double *Ai, cudaStream_t st);
void launch_corners(const SurfaceDev &s, const double *Xu, const double *normals0, double threshold, int enabled,
                    int *isCorner, cudaStream_t st);
void launch_nodal(const SurfaceDev &s, const double *Xu, const dbl4 *xa, const double *normals0,
                  const double *Ai, const int *isCorner, int useRotations, double *ptMB, cudaStream_t st);
void launch_set_data(const TreeDev &t, const double *ptMB, double *nodeMB, const SetDataScratch &sc, cudaStream_t st);
void launch_tree_parents(const TreeDev &t, int *parent, cudaStream_t st);
void launch_set_data_b(const TreeDev &t, const double *nodeAdj, double *ptAdj, int nPts, cudaStream_t st);
// faceProps = 0 reuses the face areas and normals of the previous call (same surface)
void launch_nodal_b(const SurfaceDev &s, const double *Xu, const dbl4 *xa, const double *normals0,
                    const int *isCorner, int useRotations, const double *ptAdj, int relative, double *Xub,
                    cudaStream_t st, int faceProps = 1);
void launch_scatter_dxs(int n, const int *xuInd, const double *Xub, double *dXs, cudaStream_t st);

// Complex-step nodal properties (idw_complex.cu): Xu from the interleaved
// complex coordinates xsC, and the imaginary parts of (M + I, b) per node.
struct cplx;
void launch_nodal_cs(const SurfaceDev &s, const int *xuInd, const double *xsC, cplx *xu, const dbl4 *xa,
                     const double *normals0, const double *Ai, const int *isCorner, int useRotations, double *ptMBim,
                     cudaStream_t st);
void launch_interleave(int64_t n, const double *re, const double *im, double *out, cudaStream_t st);
void launch_split(int64_t n, const double *in, double *re, double *im, cudaStream_t st);
// Tangent nodal properties: (Md [+ I], bd) per point, 12 doubles (M row-major, b).
void launch_nodal_d(const SurfaceDev &s, const double *Xu, const double *Xud, const dbl4 *xa, const double *normals0,
                    const double *Ai, const int *isCorner, int useRotations, int plusIdentity, double *ptMBd,
                    cudaStream_t st);

// Set-up kernels (idw_setup.cu)
// Returns 0, -1 on a CUDA error, -2 when its scratch cannot be allocated.
int launch_compute_errors(const TreeDev &t, const dbl4 *ptXA, const WeightLaw &law, double *err, cudaStream_t st);
// rf: the FP32 node records (split centroid, radius) for the guarded FP32 far-field test
void launch_denominator0(const TreeDev &t, const NodeRecF *rf, const dbl4 *ptXA, const VolumeDev &v,
                         const WeightLaw &law, const SymPlanes &sym, double *den0, cudaStream_t st);
// estimate of the common-order nodes 0, stride, 2 stride, ... into out; returns their count
int64_t launch_denominator0_strided(const TreeDev &t, const NodeRecF *rf, const dbl4 *ptXA, const VolumeDev &v,
                                    const WeightLaw &law, const SymPlanes &sym, int64_t stride, double *out,
                                    cudaStream_t st);
void launch_dry_run(const TreeDev &t, const VolumeDev &v, const SymPlanes &sym, double errTol, int nPts,
                    double *costs, cudaStream_t st);
// Bounding box of n points on the device and the number of non-finite
// coordinates (set-up; synchronises st).  Returns 0, or -1 on a CUDA error.
int volume_bbox(int64_t n, const double *x, double *lo, double *hi, int64_t *nonFinite, cudaStream_t st);
void launch_morton_codes(int64_t nVol, const double *xv0, const double *lo, const double *hi,
                         unsigned long long *codes, int *idx, cudaStream_t st);
// pStride / nStride: floats between consecutive points / nodes of ptDM and
// nodeDC (12 for one surface; 12 kBatchMax for the batched walk's
// point-major arrays); dnStride likewise for nodeDn.
void launch_mixed_nodal(int n, const TreeDev &t, const double *nodeMB, const dbl4 *ptXA, const double *ptMB,
                        float *ptDM, float *ptDMl, cudaStream_t st, int pStride = 12);
// The per-surface fields of the replay records (dn, dc) from nodeDn / nodeDC.
void launch_replay_records(int nNodes, const float *nodeDC, const float *nodeDn, float4 *rr, cudaStream_t st);
void launch_mixed_nodes(const TreeDev &t, const double *nodeMB, const double *ptMB, float *nodeDC, float *nodeDCl,
                        float *nodeDn, float *refDB, cudaStream_t st, int nStride = 12, int dnStride = 1);

// Evaluation (idw_walk.cu)
void launch_walk_fp64(const TreeDev &t, const PointsDev &p, const VolumeDev &v, const double *nodeMB,
                      const EvalConsts &k, int exact, int nPts, const WalkOut &o, cudaStream_t st);
void launch_walk_records(const VolumeDev &v, const SymPlanes &sym, double bExp, float4 *hi, float4 *lo,
                         cudaStream_t st);
void launch_walk_mixed(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af,
                       const VolumeDev &v, const WalkRecF &rec, const EvalConsts &k, int exact, float4 *acc,
                       const WalkOut &o, cudaStream_t st);
// Recorded decisions (idw_replay.cu).  count_walk_lists fills offs (warps x
// nLoop + 1) and returns the number of entries (-1 on a CUDA error; it
// synchronises st); launch_walk_record writes them and the walk's counters;
// launch_walk_replay evaluates the forward sums from k.lists into acc.
int64_t walk_list_warps(int64_t nVol);
// dst[0..3] += the recording walk's counters (a replay counts what it replays)
void launch_add_walk_counters(unsigned long long *dst, const unsigned long long *src, cudaStream_t st);
int64_t count_walk_lists(const TreeDev &t, const TreeDevF &tf, const VolumeDev &v, const WalkRecF &rec,
                         const EvalConsts &k, int64_t *offs, cudaStream_t st);
void launch_walk_record(const TreeDev &t, const TreeDevF &tf, const VolumeDev &v, const WalkRecF &rec,
                        const EvalConsts &k, const int64_t *offs, int2 *list, unsigned long long *counters,
                        cudaStream_t st);
void launch_walk_replay(const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af, const VolumeDev &v,
                        const WalkRecF &rec, const EvalConsts &k, float4 *acc, unsigned long long *counters,
                        cudaStream_t st);
// Exact mode as a tiled N-body kernel (idw_exact.cu); launch_walk_mixed uses
// it for exact = 1.  Fills acc like the walk; no finalisation.
void launch_exact_mixed(const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af, const VolumeDev &v,
                        const WalkRecF &rec, const MixedParams &mp, const WeightLaw &wl, float4 *acc,
                        unsigned long long *counters, cudaStream_t st);
// Exact-mode reverse product of one seed (dxv: 3 per volume node, common
// order) into the points' relative moments ptAdj (12 per point, zeroed by the
// caller), tiled as launch_exact_mixed (idw_exact.cu).
void launch_exact_adjoint(const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v, const WalkRecF &rec,
                          const MixedParams &mp, const WeightLaw &wl, const double *dxv, const double *den,
                          double *ptAdj, unsigned long long *counters, cudaStream_t st, int det = 0);
// True when the tiled exact kernel has volume nodes for at least two full
// waves of the device (below that the walk's finer grain is faster).
bool exact_tiled_fills(int64_t nVol);
// Per node (Morton order): the scaled denominator of the last mixed walk (acc).
void launch_gate_den(int64_t nVol, const float4 *acc, float *gden, cudaStream_t st);
int launch_walk_adjoint_fp64(const TreeDev &t, const PointsDev &p, const VolumeDev &v, const EvalConsts &k, int exact,
                             int nPts, const double *dxv, const double *den, int nSeeds, int64_t seedStride,
                             double *ptAdj, double *nodeAdj, int64_t ptStride, int64_t nodeStride,
                             unsigned long long *counters, cudaStream_t st, int det = 0);
MixedParams make_mixed_params(const EvalConsts &k);
// Largest number of surfaces that share one batched walk.
#ifndef IDW_BATCH_MAX
#define IDW_BATCH_MAX 4
#endif
constexpr int kBatchMax = IDW_BATCH_MAX;
// nb (1..kBatchMax) surfaces in one mixed walk (idw_batch.cu).  The point and
// cluster arrays are point-major: surface b's 12 floats of point i at
// pf.dm + 12 (kBatchMax i + b) (likewise dml, af.dc, af.dcl by node), its
// bound at af.dn[kBatchMax q + b]; the reference motions at af.ref + 24 b,
// accumulators at acc + accStrideB * b.
void launch_walk_mixed_batch(int nb, const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const NodeAggF &af,
                             const VolumeDev &v, const WalkRecF &rec, const EvalConsts &k, int exact, float4 *acc,
                             int64_t accStrideB, unsigned long long *counters, cudaStream_t st);
void launch_finalize_mixed(const VolumeDev &v, const WalkRecF &rec, const float4 *acc, double bExp, double *xv,
                           cudaStream_t st, int tangent = 0);
int launch_adjoint_mixed(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v,
                         const WalkRecF &rec, const EvalConsts &k, int exact, const double *dxv, int nSeeds,
                         int64_t dxvStride, const double *den, double *ptAcc, double *nodeAcc, double *ptAdj,
                         const dbl4 *ptXA, int nPts, unsigned long long *counters, cudaStream_t st,
                         int maxGroup = 16, int combine = 1, int det = 0);
// Point and cluster moments of a mixed reverse walk -> the relative point
// adjoints of the reverse nodal properties (setData_b folded in).
void launch_adjoint_combine(const TreeDev &t, const dbl4 *ptXA, int nPts, int nSeeds, const double *ptAcc,
                            const double *nodeAcc, double *ptAdj, cudaStream_t st);
// Precise (double-float) mixed reverse walk and its denominator walk
// (idw_adjoint_precise.cu); integer exponents only.
bool precise_adjoint_supported(const WeightLaw &wl);
void launch_precise_denominator(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v,
                                const WalkRecF &rec, const EvalConsts &k, int exact, double *denOut,
                                cudaStream_t st);
int launch_adjoint_precise(const TreeDev &t, const TreeDevF &tf, const PointsDevF &pf, const VolumeDev &v,
                           const WalkRecF &rec, const EvalConsts &k, int exact, const double *dxv, int nSeeds,
                           int64_t dxvStride, const double *den, double *ptAcc, double *nodeAcc, int nPts,
                           unsigned long long *counters, cudaStream_t st, int det = 0);
int sort_morton(int64_t nVol, unsigned long long *codes, int *idx, unsigned long long *codesAlt, int *perm,
                cudaStream_t st);

// Setters of the landing state (idw_land.cuh), one per translation unit
// that lands FP64 sums; set all of them on the launching stream.
struct LandState;
cudaError_t land_set_adjoint(const LandState &s, cudaStream_t st);
cudaError_t land_set_precise(const LandState &s, cudaStream_t st);
cudaError_t land_set_walk(const LandState &s, cudaStream_t st);
cudaError_t land_set_nodal(const LandState &s, cudaStream_t st);
cudaError_t land_set_exact(const LandState &s, cudaStream_t st);
// The nodal adjoint's two parts (launch_nodal_b runs both): nodes, whose
// area and normal adjoints land in the faces' scratch, then faces, whose
// element adjoints land in Xub; det: order-independent landings.
void launch_nodal_b_nodes(const SurfaceDev &s, const double *Xu, const dbl4 *xa, const double *normals0,
                          const int *isCorner, int useRotations, const double *ptAdj, int relative, double *Xub,
                          cudaStream_t st, int faceProps, int det);
void launch_nodal_b_faces(const SurfaceDev &s, const double *Xu, int useRotations, double *Xub, cudaStream_t st,
                          int det);

// Surface tree built on the device (idw_tree.cu): Morton order, binary radix
// tree cut at bucket-size leaves, in the host kd build's layout.  pts: host
// array of n unique points.  0, -1 (CUDA error), -2 (out of device memory) or
// -3 (more than 2^30 points).
struct FlatTree;
int build_morton_tree(const double *pts, int n, int bucket, FlatTree &t, cudaStream_t st);

}  // namespace idw
