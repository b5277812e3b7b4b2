/*
 * spr_gb300.h -- C ABI of the GB300-native estimate-and-mark pass.
 *
 * The entry points replace, one for one, the PUMI (SCOREC/core) calls of the
 * estimate-and-mark path.  Each declaration names the reference interface it
 * stands in for (paths relative to the SCOREC/core tree).  A C++ shim on the
 * reference side (core_gb300/shim/sprGB300.{h,cc}) flattens an apf::Mesh2
 * into a sprg_mesh_view, calls these functions, and writes the results back
 * into the apf fields and the "ma_flags" tag, so callers keep the unchanged
 * spr::/ma:: signatures.
 *
 * Conventions
 *  - All arrays are in MDS index order: entity i of a dimension is the i-th
 *    entity visited by apf::Mesh::begin/iterate on that dimension.
 *  - Host pointers everywhere (the library copies to and from the device),
 *    except in the *_resident functions, which keep data in device memory.
 *  - Calls are synchronous: outputs are complete when a call returns.
 *  - Every function returns SPRG_OK (0) or a nonzero SPRG_E* code and never
 *    aborts; sprg_last_error() describes the last failure.  The reference
 *    aborts instead (PCU_ALWAYS_ASSERT, apf::fail); the shim maps nonzero
 *    codes back to apf::fail to keep those semantics.
 *  - One host thread per context.  Contexts are independent.
 */
#ifndef SPR_GB300_H
#define SPR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPRG_OK 0
#define SPRG_EINVAL 1   /* bad argument, unsupported mesh or element type */
#define SPRG_EPATCH 2   /* SPR patch cannot be completed (spr/sprRecoverField.cc:383) */
#define SPRG_EFLAGS 3   /* edge already carries the true flag (ma/maAdapt.cc:304) */
#define SPRG_ENOMEM 4   /* device or host allocation failed */
#define SPRG_ECUDA 5    /* CUDA runtime error */
#define SPRG_ESTATE 6   /* call order: an input the call needs is not resident */
#define SPRG_EEIGEN 7   /* mth::eigenQR of a log-metric did not converge (apf/apfMatrix.cc:75 asserts) */

/* precision modes */
#define SPRG_FP64 0  /* FP64 throughout, the reference's arithmetic */
#define SPRG_FP32 1  /* FP32 fits and sweeps with compensated residuals, FP64 guard band (tets); in the
                        anisotropic pass: FP64 recoveries (cached triangle patch weights) and metric,
                        FP32 measure with an FP64 guard band, FP32 qualities */
#define SPRG_LEARNED 2 /* MLP-predicted recovery with SPR fallback, FP32 sweeps (tets, size to 1e-2) */

/* markEntities flag bits (ma/maAdapt.h:17-37) */
#define SPRG_SPLIT (1 << 0)
#define SPRG_DONT_SPLIT (1 << 1)
#define SPRG_COLLAPSE (1 << 2)
#define SPRG_DONT_COLLAPSE (1 << 3)
#define SPRG_NEED_NOT_SPLIT (1 << 17)
#define SPRG_NEED_NOT_COLLAPSE (1 << 18)
#define SPRG_BAD_QUALITY (1 << 5)  /* element flags of ma::markBadQuality (ma/maAdapt.h:23-24) */
#define SPRG_OK_QUALITY (1 << 6)

/* which marking pass */
#define SPRG_MARK_SPLIT 0    /* ma::markEdgesToSplit    (ma/maRefine.cc:395) */
#define SPRG_MARK_COLLAPSE 1 /* ma::markEdgesToCollapse (ma/maCoarsen.cc:287) */

/* Flattened linear simplex mesh (tets in 3D, triangles in 2D).
   Replaces traversal of apf::Mesh / MDS (mds/apfMDS.cc:300-342). */
typedef struct sprg_mesh_view {
  int dim;                       /* 3 (tets) or 2 (triangles) */
  int64_t n_verts;
  int64_t n_elems;
  int64_t n_edges;
  const double* coords;          /* n_verts x 3: apf::Mesh::getPoint */
  const int32_t* elem_verts;     /* n_elems x (dim+1): getDownward(e, 0) order */
  const int32_t* edge_verts;     /* n_edges x 2: getDownward(edge, 0) */
  /* Optional (both NULL or both set): vertex-to-element adjacency in
     getAdjacent(v, dim) order (mds/mds.c:666 get_up).  It fixes the
     summation order of the vertex size average (spr/sprEstimateError.cc:255)
     so results are bitwise those of the reference.  When NULL the library
     builds it in ascending element order. */
  const int32_t* vert_elem_offsets; /* n_verts + 1 */
  const int32_t* vert_elems;
} sprg_mesh_view;

typedef struct sprg_ctx sprg_ctx;

/* Statistics of the last size-field computation. */
typedef struct sprg_size_info {
  double eps_star_norm2;   /* SelfProduct integral, sum over elements (spr/sprEstimateError.cc:98) */
  double error_sum;        /* Error integral G (spr/sprEstimateError.cc:171) */
  double size_factor;      /* spr/sprEstimateError.cc:205-217 */
  int64_t n_expanded;      /* patches that needed growth (spr/sprRecoverField.cc:365) */
  int64_t n_fp64_refits;   /* FP32 mode: patches refit in FP64 (condition estimate > 1e6) */
  int64_t n_guard_edges;   /* FP32 mode: edges within 2e-6 of 0.5 / 1.5, re-decided in FP64 */
  int64_t n_guard_unresolved; /* FP32 mode: guard edges left to the FP32 decision (patch growth needed) */
  int64_t n_learned_fallback; /* learned mode: vertices recovered by plain SPR instead of the network */
  int64_t n_rounding_dominated; /* FP32 mode, one mesh: 1 when the reference's own FP64 rounding of the IP
                                   gradients (about 2^-50 max|u| |J^-1| per element, times 256) could move
                                   its error integral by 1e-7 or more, or that integral is zero or not
                                   finite (a constant field, one offset far above its variation, NaN):
                                   the reference's sizes are then its rounding's, and
                                   sprg_estimate_and_mark runs the pass again in FP64 (the reference's
                                   operation order); the resident entry points leave that to the caller */
} sprg_size_info;

/* ---- context: flatten + upload (the MDS-to-device flattener) ---------- */

/* Uploads the mesh to device `device` and builds the device adjacency.
   Replaces the per-call apf::Mesh traversal of every function below. */
int sprg_create(const sprg_mesh_view* mesh, int device, sprg_ctx** out);
int sprg_destroy(sprg_ctx* ctx);
const char* sprg_last_error(const sprg_ctx* ctx);
/* SPRG_FP64 (default), SPRG_FP32 or SPRG_LEARNED. */
int sprg_set_precision(sprg_ctx* ctx, int precision);
/* Run on this CUDA stream (cudaStream_t, NULL = the context's own). */
int sprg_set_stream(sprg_ctx* ctx, void* stream);

/* ---- spr ------------------------------------------------------------- */

/* spr::getGradIPField(f, name, order) (spr/spr.h:33, spr/sprGetGradIPField.cc:15).
   order must be 1.  ncomp_in 1 (SCALAR f -> VECTOR ip field, 3 per element)
   or 3 (VECTOR f -> MATRIX ip field, 9 per element, row-major).
   f: n_verts x ncomp_in.  ip_out: n_elems x (3*ncomp_in), may be NULL (the
   ip field stays resident for the calls below). */
int sprg_get_grad_ip_field(sprg_ctx* ctx, const double* f, int ncomp_in, int order, double* ip_out);

/* spr::recoverField(ip_field) (spr/spr.h:39, spr/sprRecoverField.cc:419).
   ip: n_elems x ncomp, or NULL to use the resident ip field.
   out: n_verts x ncomp ("spr_<name>" Lagrange-1 field), may be NULL. */
int sprg_recover_field(sprg_ctx* ctx, const double* ip, int ncomp, double* out);

/* spr::getSPRSizeField(eps, adapt_ratio, pcu) (spr/spr.h:47, spr/sprEstimateError.cc:311).
   ip: as above.  size_out: n_verts ("size" Lagrange-1 field), may be NULL
   (stays resident for ma measure / mark / quality).  info may be NULL. */
int sprg_get_spr_size_field(sprg_ctx* ctx, const double* ip, int ncomp, double adapt_ratio,
                            double* size_out, sprg_size_info* info);

/* spr::getTargetSPRSizeField(eps, target, pcu, alpha, beta)
   (spr/spr.h:56, spr/sprEstimateTargetError.cc:241). */
int sprg_get_target_spr_size_field(sprg_ctx* ctx, const double* ip, int ncomp, size_t target,
                                   double alpha, double beta, double* size_out, sprg_size_info* info);

/* ---- ma --------------------------------------------------------------- */

/* ma::makeSizeField(m, size) + MetricSizeField::measure on every edge
   (ma/maSize.cc:649, 208).  size: n_verts, or NULL for the resident size
   field.  lengths: n_edges, may be NULL (lengths stay resident). */
int sprg_measure_edges(sprg_ctx* ctx, const double* size, double* lengths);

/* ma::makeSizeField(m, sizes, frames, false) + measure (ma/maSize.cc:618,
   AnisoSizeField ma/maSize.cc:364-412).  sizes: n_verts x 3; frames:
   n_verts x 9 row-major (principal directions in columns). */
int sprg_measure_edges_aniso(sprg_ctx* ctx, const double* sizes, const double* frames, double* lengths);

/* ma::makeSizeField(m, sizes, frames, true) + measure: LogAnisoSizeField
   (ma/maSize.cc:455-580), the log-metrics f diag(log(1/h^2)) f^T of the
   vertices interpolated and eigen-decomposed (mth::eigenQR) at each Gauss
   point.  Lengths stay resident for sprg_mark_edges.  SPRG_EEIGEN where the
   reference's eigen iteration would assert. */
int sprg_measure_edges_log_aniso(sprg_ctx* ctx, const double* sizes, const double* frames, double* lengths);

/* ma::measureTetQuality / measureTriQuality (useMax = true) under the
   LogAnisoSizeField of sizes and frames; q resident for the quality sweeps. */
int sprg_measure_quality_log_aniso(sprg_ctx* ctx, const double* sizes, const double* frames, double* q);

/* ma::markEdgesToSplit / ma::markEdgesToCollapse through ma::markEntities
   (ma/maAdapt.cc:293) on the resident lengths.  flags: n_edges int words of
   the "ma_flags" tag (0 where the tag is absent), updated in place.
   count: marked edges (all owned on one part). */
int sprg_mark_edges(sprg_ctx* ctx, int which, int32_t* flags, long* count);

/* ma::measureTetQuality / ma::measureTriQuality with useMax = true
   (ma/maShape.h:24-26, ma/maQuality.cc:110-167) for every element, under the
   isotropic size field `size` (NULL = resident) or, when sizes/frames are
   given, the anisotropic one.  q: n_elems. */
int sprg_measure_quality(sprg_ctx* ctx, const double* size, const double* sizes, const double* frames,
                         double* q);

/* ---- MA sweeps around the marks -------------------------------------------
   Size field kinds: SPRG_SIZE_IDENTITY is ma::IdentitySizeField (apf::measure
   of the edge, ma/maSize.cc:49-92); SPRG_SIZE_ISO the isotropic user field
   (`size`: n_verts, or NULL for the resident one); SPRG_SIZE_ANISO the
   AnisoSizeField of `sizes` (n_verts x 3) and `frames` (n_verts x 9)
   (makeSizeField(m, sizes, frames, false)); SPRG_SIZE_LOG_ANISO the
   LogAnisoSizeField of the same inputs (makeSizeField(m, sizes, frames,
   true), ma/maSize.cc:455-580, the default of ma::configure). */
#define SPRG_SIZE_IDENTITY 0
#define SPRG_SIZE_ISO 1
#define SPRG_SIZE_ANISO 2
#define SPRG_SIZE_LOG_ANISO 3

/* SizeField::measure of would-be edges given as vertex pairs (pairs: n x 2),
   e.g. the edges a collapse would create that ma::collapseSizeCheck measures
   (ma/maCoarsen.cc:47-60).  lengths: n. */
int sprg_measure_vertex_pairs(sprg_ctx* ctx, int kind, const double* size, const double* sizes, const double* frames,
                              int64_t n_pairs, const int32_t* pairs, double* lengths);

/* ma::getMaximumEdgeLength(m, sf) (ma/maSize.cc:673-690): the largest edge
   measure, from 0 (all edges owned on one part). */
int sprg_get_maximum_edge_length(sprg_ctx* ctx, int kind, const double* size, const double* sizes,
                                 const double* frames, double* out);

/* ma::getAverageEdgeLength(m) (ma/maSize.cc:652-671): mean apf::measure of
   the edges (summed in a fixed tree order, not the reference's sequence). */
int sprg_get_average_edge_length(sprg_ctx* ctx, double* out);

/* The iteration count ma::configure derives from the maximum metric edge
   length (updateMaxIterBasedOnSize, ma/maInput.cc:174-190):
   ceil(log2(L)) + 1, at most 10. */
int sprg_max_iterations_for_length(double max_metric_length);

/* ma::markBadQuality (ma/maShape.cc:132-136): ma::markEntities over the
   elements with quality < good_quality on the resident qualities of the last
   sprg_measure_quality; flags: n_elems int words, BAD_QUALITY / OK_QUALITY
   set in place (SPRG_EFLAGS if an element already carries BAD_QUALITY). */
int sprg_mark_bad_quality(sprg_ctx* ctx, double good_quality, int32_t* flags, long* count);

/* ma::getMinQuality (ma/maShape.cc:151-169) on the resident qualities: the
   minimum below 1 (1 if none), the value of the first element holding it. */
int sprg_get_min_quality(sprg_ctx* ctx, double* out);

/* ---- mesh files --------------------------------------------------------------
   One part of an MDS .smb file (mds/mds_smb.c:547-606, versions 0-6,
   uncompressed) read into the flattened layout of sprg_mesh_view, in MDS
   index order: counts and connectivity, coordinates; the sections after the
   coordinates (parametric coordinates, remote copies, classification, tags,
   matches, meta) are not read.  Simplex meshes only: files with quads,
   hexes, prisms or pyramids are refused (SPRG_EINVAL).  Element vertices
   follow MDS's derivation from the downward adjacency (mds/mds.c:498,
   627-662), the order getDownward(e, 0) returns.  Host-only calls.
   sprg_smb_counts: dim and counts; sprg_smb_read: coords (n_verts x 3),
   elem_verts (n_elems x (dim + 1)), edge_verts (n_edges x 2). */
int sprg_smb_counts(const char* path, int* dim, int64_t* n_verts, int64_t* n_elems, int64_t* n_edges);
int sprg_smb_read(const char* path, double* coords, int32_t* elem_verts, int32_t* edge_verts);
/* mds_write_smb for one part (mds/mds_smb.c:617-637): version 4 with the
   flattened edges, the elements' triangles numbered in order of first
   appearance (so that the reader's derivation gives back each element's
   vertex order), zero parametric coordinates, every entity classified on
   the model entity of the mesh's dimension with tag 0, no remote copies,
   tags or matches.  The optional averaging CSR of the view is not stored. */
int sprg_smb_write(const char* path, const sprg_mesh_view* mesh);

/* ---- locality renumbering ------------------------------------------------------
   apf::reorderMdsMesh (mds/apfMDS.cc:957, mds_reorder mds/mds_order.c:409) on
   the flattened arrays: vertices numbered breadth-first from a seed (the
   first vertex of the smallest degree: a flattened view has no model to
   pick the reference's model-vertex seed from), neighbours in descending
   edge id, unreached vertices starting new searches in index order; elements
   and edges then numbered in the order the renumbered vertices first reach
   them (elements through the view's getAdjacent CSR when given, else
   ascending).  Outputs the new index of every old entity (vert_new: n_verts,
   elem_new: n_elems, edge_new: n_edges); the caller builds the renumbered
   view (ids mapped, rows moved; each element's and edge's own vertex order
   kept) and maps results back.  Host-only; no context needed. */
int sprg_locality_order(const sprg_mesh_view* mesh, int32_t* vert_new, int32_t* elem_new, int32_t* edge_new);

/* ---- incremental update after host topology changes ------------------------
   The adapt loop modifies the mesh on the host (refine, coarsen, swap, snap)
   and re-marks it every iteration (ma/maRefine.cc:420-448,
   ma/maCoarsen.cc:294-320).  Instead of a new context (a full flatten and
   upload), the caller sends what changed in the flattened arrays: the new
   counts and, per entity kind, the rows (ids) whose values are new --
   moved vertices, new or rewired elements and edges.  Rows below the old
   count keep their values unless listed; rows from the old count up to the
   new one must all be listed; rows beyond the new count are dropped (a
   deleted entity is expressed by moving the last row into its slot).  The
   vertex-element adjacency, the FP32 records, patch weights, bins, caches
   and graphs are rebuilt or invalidated on the device; a batch view is
   cleared.  averaging CSR (optional, both or neither): the reference's
   getAdjacent order for the size average, as in sprg_mesh_view.
   Everything is validated before anything changes (SPRG_EINVAL). */
typedef struct sprg_mesh_delta {
  int64_t n_verts, n_elems, n_edges;           /* counts after the update */
  int64_t n_vert_rows;  const int32_t* vert_ids;  const double* coords;      /* n x 3 */
  int64_t n_elem_rows;  const int32_t* elem_ids;  const int32_t* elem_verts; /* n x (dim + 1) */
  int64_t n_edge_rows;  const int32_t* edge_ids;  const int32_t* edge_verts; /* n x 2 */
  const int32_t* vert_elem_offsets;            /* n_verts + 1, optional */
  const int32_t* vert_elems;                   /* n_elems x (dim + 1), optional */
} sprg_mesh_delta;
int sprg_update_mesh(sprg_ctx* ctx, const sprg_mesh_delta* delta);

/* Anisotropic metric from a nodal Hessian (V x 9 row-major, e.g. the
   recovered field of the gradient of the recovered gradient): sizes (V x 3)
   h_i = clamp(sqrt(eps / |lambda_i|), h_min, h_max) and frames (V x 9,
   row-major, principal directions as columns, ordered by |lambda|
   descending, each signed so its largest component is positive; in 2D the
   second direction is the first turned by +90 degrees and the third is z with
   h_max).  The metric the 2D anisotropic workload feeds to
   ma::makeSizeField(m, sizes, frames, false) (ma/maSize.cc:618); the
   reference's drivers build it with apf::eigen (apf/apfMatrix.cc:68). */
int sprg_hessian_metric(sprg_ctx* ctx, const double* hessian, double eps, double h_min, double h_max,
                        double* sizes_out, double* frames_out);

/* ---- the whole pass ---------------------------------------------------- */

/* getGradIPField(u,"grad",1) -> getSPRSizeField(grad, adapt_ratio) ->
   makeSizeField(m, size) -> markEdgesToCollapse -> markEdgesToSplit, on a
   scalar P1 field u (n_verts).  flags: n_edges, updated in place (may be
   NULL).  size_out may be NULL.  Counts may be NULL. */
int sprg_estimate_and_mark(sprg_ctx* ctx, const double* u, double adapt_ratio, double* size_out,
                           int32_t* flags, long* n_split, long* n_collapse, sprg_size_info* info);

/* Device-resident form of the pass: d_u is a device pointer (n_verts
   doubles); the result is the device edge-mark bitmap, one bit per edge in
   ceil(n_edges/32) uint32 words each: split bit = (length > 1.5), collapse
   bit = (length < 0.5), the ShouldSplit / ShouldCollapse predicates
   (ma/maRefine.cc:382, ma/maCoarsen.cc:275).  Nothing crosses the host
   boundary; asynchronous on the context stream.  sprg_apply_marks turns the
   bitmaps into "ma_flags" words with markEntities semantics. */
int sprg_estimate_and_mark_resident(sprg_ctx* ctx, const double* d_u, double adapt_ratio, uint32_t* d_split_bits,
                                    uint32_t* d_collapse_bits);
/* After an SPRG_FP32 resident pass on one mesh (waits for the context
   stream): *out = 1 when that pass was rounding-dominated (the
   n_rounding_dominated of sprg_size_info), so its bitmaps follow the FP32
   arithmetic rather than the reference's rounding; the caller reruns the
   pass under SPRG_FP64 for the reference's marks.  0 otherwise, and for any
   other precision or a batch. */
int sprg_rounding_dominated(sprg_ctx* ctx, int* out);
/* The anisotropic pass on device buffers (FP64, any precision setting):
   getGradIPField(u) -> recoverField -> getGradIPField of the recovered
   gradient -> recoverField (nodal Hessian) -> sprg_hessian_metric ->
   AnisoSizeField measure (ma/maSize.cc:364-412) -> split/collapse bitmaps
   -> element quality under the metric (d_quality, n_elems doubles, may be
   NULL).  d_u: V doubles. */
int sprg_aniso_estimate_and_mark_resident(sprg_ctx* ctx, const double* d_u, double eps, double h_min, double h_max,
                                          uint32_t* d_split_bits, uint32_t* d_collapse_bits, double* d_quality);

/* Host write-back of the device edge-mark bitmaps into "ma_flags" words
   with markEntities semantics (ma/maAdapt.cc:293-324): collapse pass, then
   split pass (the order ma::adapt runs them, ma/ma.cc:33-36).  Either
   bitmap may be NULL to skip its pass.  Returns SPRG_EFLAGS, leaving flags
   unchanged, if an edge already carries a pass's true flag. */
int sprg_apply_marks(int64_t n_edges, const uint32_t* split_bits, const uint32_t* collapse_bits, int32_t* flags,
                     long* n_split, long* n_collapse);

/* Per-kernel timing: when enabled, each kernel launch is bracketed by CUDA
   events on the context stream.  sprg_profile_report returns a JSON object
   {"kernel": [launches, total_ms], ...} accumulated since the last reset. */
int sprg_profile_enable(sprg_ctx* ctx, int on);
int sprg_profile_flush(sprg_ctx* ctx);
const char* sprg_profile_report(sprg_ctx* ctx, int reset);

/* Copies up to `bytes` of a named internal device buffer to the host
   (instrumentation for accuracy studies; e.g. "size", "err", "q32",
   "size32", "rec32", "tetd", "out3"). */
int sprg_debug_read(sprg_ctx* ctx, const char* name, void* host, size_t bytes);

/* Number of kernel launches issued by the last call (instrumentation). */
int64_t sprg_last_launch_count(const sprg_ctx* ctx);

/* Stage timing of sprg_estimate_and_mark (instrumentation): when on, each
   call records CUDA events at its stage boundaries and host clocks around
   its enqueue and its final wait; on = 1 or 0 also clears the sums.  The
   report is a JSON object of per-call averages since then: calls,
   upload_field_ms, pass_ms, wait_flags_upload_ms, mark_sweep_ms,
   download_flags_ms, tail_ms (size conversion / download when not
   overlapped, counts), upload_flags_overlapped_ms and
   size_download_overlapped_ms (copy stream, beside the pass),
   host_enqueue_ms, host_wait_ms, call_ms. */
int sprg_e2e_timing(sprg_ctx* ctx, int on);
const char* sprg_e2e_timing_report(sprg_ctx* ctx);

/* Test hooks (failure paths, no reference counterpart): wait_polls > 0 makes
   the learned form's network kernel wait, in place of its first layer's
   completion, wait_polls polls on a barrier that nothing completes (0: off);
   that bounded wait runs out and the pass returns SPRG_ECUDA ("a tensor-core
   wait ran out of time") after the kernel has drained the matrix multiplies
   in flight and freed its tensor memory; the context stays usable.  alloc_fail_after >= 0 makes the context's device
   allocation after that many more succeed fail with SPRG_ENOMEM (-1: off). */
int sprg_test_hooks(sprg_ctx* ctx, int wait_polls, int alloc_fail_after);

/* ---- size field without device allocation ------------------------------- */

/* No counterpart in the reference.  The size-field stage of
   getSPRSizeField (element errors, size factor, element sizes, vertex
   average) for callers that cannot allocate device memory: a code whose
   memory manager owns the device heap, or a thread that cannot take the
   synchronisation a cudaMalloc/cudaFree may imply.  All pointers except
   size_factor_out are device pointers supplied by the caller: the mesh
   (coordinates, element vertices, vertex-to-element adjacency whose order
   fixes the averaging order), the integration-point field d_ip (n_elems x
   ncomp) and the recovered field d_rec (n_verts x ncomp, e.g. from
   sprg_recover_field); the result d_size has n_verts doubles.  The call
   allocates nothing: its scratch is a fixed file-scope device array sized for
   SPRG_NOALLOC_MAX_ELEMS elements (about 17 MB, held by every GPU that loads
   the library until exit); larger meshes are rejected with SPRG_EINVAL.  The
   first call on a device resolves that array's address (do it before any
   stream capture); as CUDA loads device code lazily by default, that first
   call also loads the library's module and commits the array's memory, so a
   caller that reserves the device heap should make it before reserving (or
   set CUDA_MODULE_LOADING=EAGER).  Later calls commit nothing.  Calls share
   the array: calls that overlap on the GPU race.  A CUDA error pending from
   the caller's earlier work makes the call return SPRG_ECUDA before any
   launch, leaving that error in place.  Enqueued on `stream` (cudaStream_t,
   NULL = legacy default); when size_factor_out (host) is given, the call
   waits and stores the size factor. */
#define SPRG_NOALLOC_MAX_ELEMS (1 << 20)
int sprg_spr_size_from_recovered_noalloc(int dim, int64_t n_verts, int64_t n_elems, const double* d_coords,
                                         const int32_t* d_elem_verts, const int32_t* d_vert_elem_offsets,
                                         const int32_t* d_vert_elems, const double* d_ip, int ncomp,
                                         const double* d_rec, double adapt_ratio, double* d_size,
                                         double* size_factor_out, void* stream);

/* ---- box meshes --------------------------------------------------------- */

/* Entity counts of apf::makeMdsBox(nx, ny, nz, wx, wy, wz, true)
   (mds/apfBox.cc:330); nz = 0 gives the 2D triangle box. */
int sprg_box_counts(int nx, int ny, int nz, int64_t* n_verts, int64_t* n_elems, int64_t* n_edges);

/* Flattened apf::makeMdsBox(nx, ny, nz, wx, wy, wz, true): coordinates,
   element vertices and edge vertices in exactly the MDS numbering and
   downward order that BoxBuilder (mds/apfBox.cc:68-328) and
   apf::buildElement (apf/apfMesh2.cc:72) produce.  Arrays are caller
   allocated with the sizes from sprg_box_counts. */
int sprg_box_fill(int nx, int ny, int nz, double wx, double wy, double wz,
                  double* coords, int32_t* elem_verts, int32_t* edge_verts);

/* ---- batch of independent meshes; no reference counterpart ------------
   The context's mesh is the disjoint union of n_meshes meshes (entity ids
   of mesh k offset by the sizes of meshes 0..k-1; vert_offsets and
   elem_offsets hold n_meshes + 1 prefix sums).  The pass (SPRG_FP32) then
   computes each mesh's own SelfProduct / Error integrals and size factor
   with its own adapt ratio, as calling spr::getSPRSizeField once per mesh
   does; the adapt_ratio argument of the pass is ignored.  n_meshes = 0
   returns to a single mesh. */
int sprg_set_batch(sprg_ctx* ctx, int n_meshes, const int64_t* vert_offsets, const int64_t* elem_offsets,
                   const double* adapt_ratios);
/* per mesh of the last batch pass: eps_star_norm2, error_sum, size_factor
   (out: 3 n_meshes doubles) */
int sprg_batch_info(sprg_ctx* ctx, double* out);

/* ---- launch shape and graphs; no reference counterpart ----------------
   The FP32 recovery runs over patch-size bins (<= 8, <= 16, <= 32, more
   elements) in one persistent launch; on the first pass of a mesh an
   autotuner times lanes per bin, tile size and blocks per SM on the real
   data (every choice gives bitwise the same result).  The choice is kept
   across sprg_update_mesh; calling this with on = 1 tunes again at the next
   pass.  on = 0 keeps the current configuration. */
int sprg_set_autotune(sprg_ctx* ctx, int on);
/* fix the binned recovery's configuration (lanes per bin in {1, 2, 4} over
   the patch-CSR lists, or 0: one lane per vertex over a sliced copy of the
   lists, 32 patches side by side, which needs a tile size that is a multiple
   of 32; tile size in vertices, blocks per SM); turns the autotuner off */
int sprg_set_tiling(sprg_ctx* ctx, const int* lanes, int tile_verts, int blocks_per_sm);
/* JSON: bin sizes, chosen configuration, the autotuner's timings */
const char* sprg_tuning_report(sprg_ctx* ctx);
/* Capture the resident pass (sprg_estimate_and_mark_resident with these
   device buffers) into a CUDA graph, after one ordinary pass; needs a caller
   stream (sprg_set_stream).  sprg_graph_replay relaunches it on that stream:
   the caller refreshes d_u in place between replays. */
int sprg_graph_capture(sprg_ctx* ctx, const double* d_u, double adapt_ratio, uint32_t* d_split_bits,
                       uint32_t* d_collapse_bits);
int sprg_graph_replay(sprg_ctx* ctx);

/* ---- learned form (SPRG_LEARNED); no reference counterpart ------------
   eps*(v) = g_c + z * s_v / r_v with g_c the least-squares gradient of the
   vertex's neighbours, z an MLP (4 x 32 inputs -> 64 -> 64 -> 3, GELU, BF16
   weights and activations, FP32 accumulation) of the normalised neighbour
   offsets and residuals.  Plain SPR recovers the vertices the network does
   not answer (see sprg_set_learned_options).  Parameters: FP32 vector of
   SPRG_MLP_PARAMS values, W1 [64][128], b1 [64], W2 [64][64], b2 [64],
   W3 [3][64], b3 [3] (weights [output][input]). */
#define SPRG_MLP_PARAMS 12611
#define SPRG_MLP_INPUTS 128
#define SPRG_MLP_AUX 5
int sprg_set_mlp_params(sprg_ctx* ctx, const float* params, int n_params);
/* use_mlp = 0: g_c alone (the method without the network); z_max: vertices
   whose output has a component beyond it take plain SPR (default 8). */
int sprg_set_learned_options(sprg_ctx* ctx, int use_mlp, double z_max);
/* Network inputs of every vertex for field d_u (device, V doubles): d_x
   [V][128] BF16 (row-major), d_aux [V][5] FP32 = g_c (3), s_v / r_v, and 1 where
   the vertex takes plain SPR.  Training-data generation. */
int sprg_learned_features(sprg_ctx* ctx, const double* d_u, uint16_t* d_x, float* d_aux);

/* ---- MLP training kernels (device pointers, stream = cudaStream_t) ----- */
/* scratch bytes for n samples */
size_t sprg_mlp_scratch_bytes(int n);
/* d_out [n][3] = MLP(d_x) with BF16 weights and activations */
int sprg_mlp_forward(const float* d_params, const uint16_t* d_x, int n, float* d_out, void* d_scratch, void* stream);
/* gradient of the mean squared error against d_y [n][3] (d_grad, SPRG_MLP_PARAMS)
   and the sum of squared errors (d_loss, 1 float) */
int sprg_mlp_grad(const float* d_params, const uint16_t* d_x, const float* d_y, int n, float* d_grad, float* d_loss,
                  void* d_scratch, void* stream);
/* one Adam step (step counts from 1) */
int sprg_mlp_adam(float* d_params, float* d_m1, float* d_m2, const float* d_grad, float lr, float beta1, float beta2,
                  float eps, int step, void* stream);

#ifdef __cplusplus
}
#endif
#endif
