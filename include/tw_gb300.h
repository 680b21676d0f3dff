/*
 * tw_gb300.h -- C-ABI of the GB300 (sm_103a) implementation of TetWild's
 * mesh-optimisation query path: conformal-AMIPS energy/gradient/Hessian,
 * exact tet-inversion checks, the sampled envelope test and the Newton
 * vertex-smoothing step.
 *
 * The reference exposes these as C++ member functions of LocalOperations and
 * VertexSmoother, switched at compile time between the scalar code and the
 * ISPC kernel (TETWILD_WITH_ISPC, LocalOperations.h:21-23).  Each entry point
 * below names the reference routine it replaces; a TetWild build binds them
 * behind a switch of the same kind (TETWILD_WITH_GB300).
 *
 * Conventions
 *  - Every call returns an int status: TW_OK (0), a negative error code, or
 *    TW_NEEDS_EXACT_HOST (1) when part of a result must come from the host's
 *    exact-rational state (tets with unrounded vertices, LocalOperations.cpp
 *    :546-548).  tw_last_error() gives a message for the last failure.
 *  - Pointers are host pointers unless the function name ends in _device;
 *    _device calls take device pointers and are asynchronous on the
 *    context's stream (tw_stream()).  Host calls are synchronous.
 *  - A context belongs to one device and one stream; distinct contexts may be
 *    used from distinct threads.
 *  - Coordinates are binary64.  Decisions (signs, in/out, accept/reject) are
 *    exact or bit-identical to the CPU oracle.  In the default energy form
 *    (TW_ENERGY_FORM_REFERENCE) the binary64 energies, gradients and Hessians
 *    perform the reference routines' own operations in their order, so they
 *    agree with the reference's results to its rounding (within 1e-12
 *    relative; a few ulp in practice, the only difference being pow).
 */
#ifndef TW_GB300_H
#define TW_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__) || defined(__clang__)
#define TW_API __attribute__((visibility("default")))
#else
#define TW_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define TW_OK 0
#define TW_NEEDS_EXACT_HOST 1
#define TW_ERR_ARG (-1)
#define TW_ERR_CUDA (-2)
#define TW_ERR_OOM (-3)          /* device allocation failed or budget exceeded */
#define TW_ERR_NO_SURFACE (-4)
#define TW_ERR_NO_MESH (-5)
#define TW_ERR_TIMEOUT (-6)
#define TW_ERR_TOO_LARGE (-7)    /* request exceeds a fixed capacity (tw_amips_soa_noalloc) */
#define TW_ERR_CANCELLED (-8)    /* serving: the request's job was cancelled before it ran  */
#define TW_BUSY 2                /* serving: not admitted now (memory budget), retry later  */

/* AMIPS output modes */
#define TW_ENERGY_RAW 0          /* comformalAMIPSEnergy_new value            */
#define TW_ENERGY_QUALITY 1      /* calTetQuality_AMIPS value (1e50 sentinel) */

/* arithmetic modes (tw_set_precision) */
#define TW_PRECISION_FP64 0            /* every query in binary64 (default)        */
#define TW_PRECISION_FP32_CERTIFIED 1  /* binary32 bulk with certified error bounds;
                                          binary64 recomputation inside the band:
                                          decisions identical to TW_PRECISION_FP64 */

/* energy forms of the binary64 AMIPS evaluations (tw_set_energy_form) */
#define TW_ENERGY_FORM_REFERENCE 0  /* the reference's generated operations, in its
                                       order and with its 15-digit coefficients
                                       (default: agrees with the reference)   */
#define TW_ENERGY_FORM_CLOSED 1     /* closed form of the same function: within a
                                       few ulp of the exact value, ~3x fewer
                                       binary64 operations                     */

/* surfaces */
#define TW_SURFACE_INPUT 0       /* geo_sf_tree (MeshRefinement.cpp:209)      */
#define TW_SURFACE_BOUNDARY 1    /* geo_b_tree  (MeshRefinement.cpp:213)      */

typedef struct tw_ctx tw_ctx;

/* ---- context --------------------------------------------------------------
 * Replaces: the LocalOperations constructor's state (LocalOperations.h:56-64)
 * and State's eps_2 / sampling_dist (State.h:41-43, State.cpp:34-40).     */
TW_API int tw_ctx_create(int device, size_t hbm_budget_bytes, tw_ctx** out);
TW_API int tw_ctx_destroy(tw_ctx* ctx);
TW_API const char* tw_last_error(const tw_ctx* ctx);
/* newton_max_step / newton_max_it: MAX_STEP=15, MAX_IT=20 in the reference
 * (VertexSmoother.cpp:469-470).                                             */
TW_API int tw_set_params(tw_ctx* ctx, double eps_2, double sampling_dist, int newton_max_step,
                  int newton_max_it);
TW_API int tw_stream(tw_ctx* ctx, void** cuda_stream);
TW_API int tw_synchronize(tw_ctx* ctx);
/* Device bytes currently held by the context (mesh, surfaces, scratch).   */
TW_API int tw_memory_used(const tw_ctx* ctx, size_t* bytes);

/* ---- precision mode and statistics -----------------------------------------------
 * No counterpart in the reference (its arithmetic is binary64 throughout).
 * TW_PRECISION_FP32_CERTIFIED evaluates the bulk in binary32 and recomputes
 * in binary64 every query whose binary32 result falls inside a certified
 * error band (envelope: facets whose certified lower distance bound does not
 * exceed eps; AMIPS: tets whose certified relative error bound exceeds
 * 1e-5), so every decision equals the binary64 one.                         */
TW_API int tw_set_precision(tw_ctx* ctx, int mode);
/* Energy form of every binary64 AMIPS evaluation of the context (the batch
 * calls, tet qualities, energy sweeps, Newton steps, smoothing passes and
 * collapse checks): TW_ENERGY_FORM_REFERENCE (default) or
 * TW_ENERGY_FORM_CLOSED.  No counterpart in the reference, whose expressions
 * are the reference form (LocalOperations.cpp:28-291).                      */
TW_API int tw_set_energy_form(tw_ctx* ctx, int form);
typedef struct tw_stats {
    uint64_t exact_orientations;   /* orientation signs that needed the exact path */
    uint64_t env_queries;          /* envelope points and face samples queried      */
    uint64_t env_facet_tests;      /* facets reached by the traversals              */
    uint64_t env_facet_fp64;       /* of those, evaluated in binary64               */
    uint64_t amips_tets;           /* tets evaluated by the AMIPS kernels           */
    uint64_t amips_fp64;           /* of those, recomputed in binary64 (certified)  */
    uint64_t env_warp_fallbacks;   /* point warps that walked the tree per point    */
} tw_stats;
TW_API int tw_get_stats(tw_ctx* ctx, tw_stats* out);
TW_API int tw_reset_stats(tw_ctx* ctx);

/* ---- AMIPS energy / gradient / Hessian -------------------------------------
 * Replaces: LocalOperations::comformalAMIPSEnergy_new (LocalOperations.cpp:28,
 * decl LocalOperations.h:109), comformalAMIPSJacobian_new (:83, decl :110),
 * comformalAMIPSHessian_new (:149, decl :111), the ISPC batch energy_ispc
 * (energy.ispc:7) and the per-tet body of calTetQualities (:695-773).
 * T: SoA [12][n] doubles (the energy_ispc layout: v0x[n] v0y[n] ... v3z[n]).
 * E [n], J SoA [3][n], H SoA [9][n] (row-major 3x3 per tet), flip [n]
 * (1 = orientation not POSITIVE, isTetFlip on rounded coordinates).  Any
 * output may be NULL.  mode: TW_ENERGY_RAW or TW_ENERGY_QUALITY.           */
TW_API int tw_amips_soa(tw_ctx* ctx, const double* T, int64_t n, int mode, double* E, double* J,
                 double* H, uint8_t* flip);
TW_API int tw_amips_soa_device(tw_ctx* ctx, const double* T, int64_t n, int mode, double* E,
                        double* J, double* H, uint8_t* flip);

/* ---- AMIPS batch that allocates nothing -----------------------------------------
 * No counterpart in the reference (TetWild has no GPU code): this is an extra
 * entry point for callers that cannot let a library allocate device memory,
 * such as a host program whose allocator reserves all free HBM at start-up,
 * or one that must not stall its other streams on the device-wide
 * synchronisation of cudaFree.  Same inputs and outputs as tw_amips_soa, and
 * the same results as tw_amips_soa on a context in TW_PRECISION_FP64 with the
 * default energy form, for at most TW_NOALLOC_MAX_TETS tets per call (larger
 * n returns TW_ERR_TOO_LARGE); needs no context.  It calls no cudaMalloc or
 * cudaFree: its scratch is a fixed device array of TW_NOALLOC_SCRATCH_BYTES
 * that every GPU loading this library holds until the process exits.  The
 * first call on a device looks up that array's address (make it before any
 * stream capture).  All calls on a device share the array, so calls whose
 * work overlaps on the GPU race: serialise them.  cuda_stream may be NULL
 * (the legacy default stream); the call waits for its stream before
 * returning.                                                                 */
#define TW_NOALLOC_MAX_TETS 65536
#define TW_NOALLOC_SCRATCH_BYTES (201 * TW_NOALLOC_MAX_TETS + 256)
TW_API int tw_amips_soa_noalloc(const double* T, int64_t n, int mode, double* E, double* J,
                                double* H, uint8_t* flip, void* cuda_stream);

/* ---- resident mesh -----------------------------------------------------------
 * The tet-mesh vertex array (TetVertex::posf / is_rounded,
 * TetmeshElements.h:24-64) kept in HBM for index-based queries.
 * xyz: [nv][3] doubles; rounded: [nv] (NULL = all rounded).                 */
TW_API int tw_mesh_upload(tw_ctx* ctx, const double* xyz, int32_t nv, const uint8_t* rounded);
TW_API int tw_mesh_update_vertices(tw_ctx* ctx, const int32_t* ids, const double* xyz,
                            const uint8_t* rounded, int32_t n);

/* Replaces: LocalOperations::calTetQualities (LocalOperations.cpp:695, decl
 * LocalOperations.h:69) and isTetFlip / isFlip (:535-573, decl :77-79).
 * tets: [n][4] vertex ids into the resident mesh.  energy[n] gets the
 * calTetQuality_AMIPS value, flip[n] the isTetFlip value; either may be NULL.
 * Tets with an unrounded vertex get needs_host[i] = 1 (if non-NULL) and the
 * call returns TW_NEEDS_EXACT_HOST: their orientation must come from the
 * host's exact coordinates (LocalOperations.cpp:546-548).                  */
TW_API int tw_tet_quality(tw_ctx* ctx, const int32_t* tets, int64_t n, double* energy, uint8_t* flip,
                   uint8_t* needs_host);
TW_API int tw_tet_quality_device(tw_ctx* ctx, const int32_t* tets, int64_t n, double* energy,
                          uint8_t* flip, uint8_t* needs_host);

/* ---- envelope -----------------------------------------------------------------
 * Replaces: the MeshFacetsAABBWithEps constructor (mesh_AABB.cpp:356-379):
 * builds an LBVH over the surface on the device.  V: [nv][3], F: [nf][3].   */
TW_API int tw_surface_upload(tw_ctx* ctx, const double* V, int32_t nv, const int32_t* F, int32_t nf,
                      int which);
/* Replaces: LocalOperations::isPointOutEnvelop (LocalOperations.cpp:1034,
 * decl LocalOperations.h:98) and isPointOutBoundaryEnvelop (:1111, decl :100)
 * for which = TW_SURFACE_BOUNDARY.  P: [n][3]; out[i] = 1 iff the squared
 * distance from P[i] to the surface exceeds eps_2.                          */
TW_API int tw_envelope_points(tw_ctx* ctx, const double* P, int64_t n, int which, uint8_t* out);
TW_API int tw_envelope_points_device(tw_ctx* ctx, const double* P, int64_t n, int which, uint8_t* out);
/* Replaces: LocalOperations::isFaceOutEnvelop / isFaceOutEnvelop_sampling
 * (LocalOperations.cpp:967, :1046; decl LocalOperations.h:97,99) with
 * sampleTriangle (Common.cpp:143).  tris: [n][9] (three vertices).
 * out[i] = 0 for a degenerate triangle, else 1 iff some sample is out.     */
TW_API int tw_envelope_faces(tw_ctx* ctx, const double* tris, int64_t n, uint8_t* out);
TW_API int tw_envelope_faces_device(tw_ctx* ctx, const double* tris, int64_t n, uint8_t* out);
/* sampleTriangle (Common.cpp:143-228) evaluated on the device for one
 * triangle: writes min(count, cap) samples [..][3] to out (host) and the
 * full count to *count.  For checking the device sampling arithmetic.     */
TW_API int tw_sample_triangle(tw_ctx* ctx, const double* tri9, double sampling_dist, double* out,
                       int64_t cap, int64_t* count);

/* Replaces: MeshFacetsAABBWithEps::nearest_facet (mesh_AABB.h:130-141,
 * mesh_AABB.cpp:381-480) for a batch of points.  P: [n][3].  Q: [n][3]
 * closest points, D: [n] squared distances, F: [n] input facet indices (any
 * output may be NULL).  Equal distances go to the smallest facet index
 * (geogram keeps the first facet its traversal meets; the distance is the
 * same).                                                                    */
TW_API int tw_nearest_points(tw_ctx* ctx, const double* P, int64_t n, int which, double* Q,
                             double* D, int32_t* F);
TW_API int tw_nearest_points_device(tw_ctx* ctx, const double* P, int64_t n, int which, double* Q,
                                    double* D, int32_t* F);

/* ---- Newton smoothing ---------------------------------------------------------
 * Replaces: VertexSmoother::NewtonsMethod (VertexSmoother.cpp:465, decl
 * VertexSmoother.h:28) with NewtonsUpdate (:627) and getNewEnergy (:544),
 * for a batch of independent one-ring stars over the resident mesh.
 * star_off: [nstars+1] offsets into tets ([.][4] ids, each star's tets in
 * the caller's order, which fixes the summation order); centers: [nstars]
 * vertex ids.  out: [nstars][3] new position, moved: [nstars] is_moved.    */
TW_API int tw_newton_stars(tw_ctx* ctx, const int32_t* star_off, const int32_t* tets,
                    const int32_t* centers, int32_t nstars, double* out, uint8_t* moved);

/* Device-pointer variant (asynchronous on the context stream): star_off,
 * tets, centers, out and moved are device pointers; ids are not checked.  */
TW_API int tw_newton_stars_device(tw_ctx* ctx, const int32_t* star_off, const int32_t* tets,
                                  const int32_t* centers, int32_t nstars, double* out,
                                  uint8_t* moved);
/* Launch shape of the Newton step: lanes per star (1, 8, 16, 32) and block
 * size (64, 128, 256), TW_NEWTON_SHAPES in all; every shape gives
 * bit-identical results.  tw_newton_autotune_device times every shape on
 * the given batch (device pointers, results written to out/moved), keeps the
 * fastest in the context, and reports it and, if ms_per_shape is non-NULL,
 * each shape's time.  No counterpart in the reference.                     */
#define TW_NEWTON_SHAPES 10
TW_API int tw_set_newton_shape(tw_ctx* ctx, int shape);
TW_API int tw_newton_autotune_device(tw_ctx* ctx, const int32_t* star_off, const int32_t* tets,
                                     const int32_t* centers, int32_t nstars, double* out,
                                     uint8_t* moved, int* best_shape, float* ms_per_shape);

/* ---- one smoothing pass over independent stars ---------------------------------
 * Replaces: the per-vertex bodies of VertexSmoother::smoothSingle
 * (VertexSmoother.cpp:114-210, interior vertices) and smoothSurface
 * (:244-450, surface vertices; decl VertexSmoother.h:24-25), for a batch of
 * stars whose centres are not in one another's stars, with every vertex
 * rounded and the stored tet qualities equal to calTetQuality at the current
 * positions.  Per star: all tets POSITIVE (else TW_SMOOTH_INVALID);
 * NewtonsMethod with the context's max_step / max_it (not moved:
 * TW_SMOOTH_NOT_MOVED); interior stars are then TW_SMOOTH_MOVED.  Surface
 * stars project the Newton position on the nearest facet of the input
 * surface (TW_STAR_BOUNDARY: of the boundary surface), then reject on an
 * inverted tet (TW_SMOOTH_REJECT_FLIP), on max energy not decreasing
 * (TW_SMOOTH_REJECT_QUALITY), or on a one-ring surface face outside the
 * envelope of the input surface (TW_SMOOTH_REJECT_ENVELOPE, eps_2 and
 * sampling_dist of tw_set_params).
 * face_flags: [ntets], bit j set when the face of the tet opposite its j-th
 * vertex is a surface face (is_surface_fs != NOT_SURFACE); may be NULL when
 * every star is interior.  kinds: [nstars] TW_STAR_* (NULL: all interior).
 * out: [nstars][3] the new position (the old one unless TW_SMOOTH_MOVED);
 * status: [nstars] TW_SMOOTH_*.  The envelope decisions follow the
 * context's precision mode (identical decisions in both).                  */
#define TW_STAR_INTERIOR 0
#define TW_STAR_SURFACE 1
#define TW_STAR_BOUNDARY 2
#define TW_SMOOTH_INVALID 0
#define TW_SMOOTH_NOT_MOVED 1
#define TW_SMOOTH_MOVED 2
#define TW_SMOOTH_REJECT_FLIP 3
#define TW_SMOOTH_REJECT_QUALITY 4
#define TW_SMOOTH_REJECT_ENVELOPE 5
TW_API int tw_smooth_stars(tw_ctx* ctx, const int32_t* star_off, const int32_t* tets,
                           const uint8_t* face_flags, const int32_t* centers, const uint8_t* kinds,
                           int32_t nstars, double* out, uint8_t* status);
/* Device-pointer variant (asynchronous on the context stream; ids and kinds
 * are not checked, a kind other than 1 or 2 is interior).  ntets must equal
 * star_off[nstars].  Its scratch grows on first use: a CUDA-graph capture
 * must follow one uncaptured call of at least the same sizes.              */
/* Times the whole pass for every Newton launch shape on this batch (device
 * pointers; results written to out/status), keeps the fastest shape in the
 * context and reports it and, if ms_per_shape is non-NULL, each shape's
 * time.  No counterpart in the reference.                                  */
TW_API int tw_smooth_autotune_device(tw_ctx* ctx, const int32_t* star_off, const int32_t* tets,
                                     const uint8_t* face_flags, const int32_t* centers,
                                     const uint8_t* kinds, int32_t nstars, int64_t ntets,
                                     double* out, uint8_t* status, int* best_shape,
                                     float* ms_per_shape);
TW_API int tw_smooth_stars_device(tw_ctx* ctx, const int32_t* star_off, const int32_t* tets,
                                  const uint8_t* face_flags, const int32_t* centers,
                                  const uint8_t* kinds, int32_t nstars, int64_t ntets, double* out,
                                  uint8_t* status);

/* ---- tuning knobs (work only, never results) ---------------------------------------
 * TW_TUNE_GRID_CELL: cell size of the certified envelope grid as a multiple
 *   of the mean facet extent (default 0.2; the grid is rebuilt).
 * TW_TUNE_SORT_POINTS: 1 (default) orders point queries by Morton cell of
 *   the surface box before the test (a counting sort; 2^(3b) cells with the
 *   smallest b in 3..8 that gives at least one cell per point), 2..8 fixes b,
 *   0 keeps the caller's order.  Results never depend on it.
 * TW_TUNE_POINT_BLOCK: threads per block of the certified grid point test
 *   (128, 256, 384 default, or 768; 768 resident threads per SM in each): the
 *   warps of a block test neighbouring sorted points together.  Results never
 *   depend on it.
 * TW_TUNE_BIN_CELL: bin side of the point test's bin index as a multiple of
 *   the mean facet extent (default 0.25, at least 1/250 of the surface box's
 *   largest side; each bin lists its leaves with a mask of the 8x8x8 fine
 *   cells each reaches; the index is rebuilt); 0 turns the index off (the
 *   point test then reads the grid's hashed cell lists).  Point queries are
 *   sorted on the index's bins.  Results never depend on it.
 * TW_TUNE_TIME_KERNELS: 1 records CUDA events around the point-envelope
 *   test kernel of each tw_envelope_points(_device) call (the last 64);
 *   tw_kernel_times returns their durations (ms) and clears the record.
 * No counterpart in the reference.                                          */
#define TW_TUNE_GRID_CELL 0
#define TW_TUNE_SORT_POINTS 1
#define TW_TUNE_TIME_KERNELS 2
#define TW_TUNE_POINT_BLOCK 3
#define TW_TUNE_BIN_CELL 4
TW_API int tw_set_tuning(tw_ctx* ctx, int knob, double value);
TW_API int tw_kernel_times(tw_ctx* ctx, float* ms, int max, int* count);

/* ---- energy sweeps -------------------------------------------------------------------
 * Replaces: LocalOperations::getAvgMaxEnergy, getMaxEnergy, getSecondMaxEnergy
 * and the histogram of getFilterEnergy (LocalOperations.cpp:605-693, decl
 * LocalOperations.h:103-107) over tets (ids into the resident mesh: the tets
 * that are not removed) with calTetQuality_AMIPS at the resident positions.
 * locked[i] != 0 (NULL: none) excludes tet i from avg / max / second max
 * (isTetLocked_ui).  avg is the mean over the unlocked tets (MAX_ENERGY when
 * the sum overflows) from a double-double sum: within a few ulps of the
 * exact mean, where the reference's sequential sum may differ from it by
 * n ulps.  buckets[11]: getFilterEnergy's counts; tw_filter_energy applies
 * its rule to them.                                                        */
TW_API int tw_energy_stats(tw_ctx* ctx, const int32_t* tets, int64_t n, const uint8_t* locked,
                           double filter_energy_thres, double* avg, double* max_e,
                           double* second_max, int64_t* buckets);
TW_API double tw_filter_energy(const int64_t* buckets, double filter_energy_thres,
                               int* is_clean_up);

/* ---- dihedral-angle sweep ------------------------------------------------------------
 * Replaces: LocalOperations::calTetQuality_AD over the live tets
 * (LocalOperations.cpp:783-860, called by outputInfo :350-353) and
 * outputInfo's statistics over them (:483-521) at the resident positions.
 * locked[i] != 0 (NULL: none) excludes tet i from the statistics.
 * out = {smallest min angle (10 when no tet counts), mean min angle, largest
 * max angle, mean max angle} in radians, the means from double-double sums;
 * counts = {min angle < 6, < 12, < 18 degrees, max angle > 162, > 168,
 * > 174 degrees, tets counted}.  min_angle / max_angle (may be NULL): each
 * tet's (min_d_angle, max_d_angle).  Angles use CUDA's acos (within 4 ulp of
 * the host's).                                                             */
TW_API int tw_dihedral_stats(tw_ctx* ctx, const int32_t* tets, int64_t n, const uint8_t* locked,
                             double* out, int64_t* counts, double* min_angle, double* max_angle);

/* ---- edge-collapse checks ------------------------------------------------------------
 * Replaces: the checks of EdgeCollapser::collapseAnEdge (EdgeCollapser.cpp:
 * 284-446, decl EdgeCollapser.h:31) with isCollapsable_epsilon (:727-775)
 * for a batch of candidate collapses v12[i] = (v1, v2) against the resident
 * mesh (checks only; the caller applies the successful ones).  Star i =
 * conn_tets of v1 (tets[off[i]..off[i+1]), caller order), face_flags per tet
 * as for tw_smooth_stars; flags[i] = TW_CV_* of the two vertices (after the
 * reference's isIsolated / isBoundaryPoint updates).  check_quality =
 * is_check_quality; soft_energy >= 0 replaces the old energy (is_soft).
 * result[i] = TW_COLLAPSE_SUCCESS / _FLIP / _QUALITY / _ENVELOP (the
 * reference's codes, EdgeCollapser.h:52-55).                               */
#define TW_CV_V1_SURFACE 1
#define TW_CV_V1_BOUNDARY 2
#define TW_CV_V2_SURFACE 4
#define TW_CV_V2_BOUNDARY 8
#define TW_CV_V1_UNROUNDED 16
#define TW_COLLAPSE_SUCCESS 0
#define TW_COLLAPSE_FLIP 1
#define TW_COLLAPSE_QUALITY 2
#define TW_COLLAPSE_ENVELOP 3
TW_API int tw_collapse_check(tw_ctx* ctx, const int32_t* v12, const uint8_t* flags,
                             const int32_t* off, const int32_t* tets, const uint8_t* face_flags,
                             int32_t n, int check_quality, double soft_energy, uint8_t* result);

/* ---- edge-removal (swap) checks ---------------------------------------------------
 * Replaces: the checks of EdgeRemover::removeAnEdge_32, _44 and _56
 * (EdgeRemover.cpp:125-177, :277-369, :456-600, decl EdgeRemover.h:59-61)
 * for a batch of candidate edges v12[i] = (v1, v2) against the resident mesh
 * (checks only; the caller applies the successful ones).  Shell i = the tets
 * around the edge, tets[off[i]..off[i+1]) in the caller's order (old_t_ids);
 * only the variant for a shell of 3, 4 or 5 tets applies.  budget[i] (NULL:
 * 0) = the remover's equal_buget at the call: while positive, each quality
 * comparison accepts an equal max energy and spends one unit (spent[i]).
 * result[i] = TW_SWAP_SUCCESS (config[i] = the configuration taken: 0 for
 * 3-2, 0-1 for 4-4, 0-4 for 5-6, in the reference's enumeration), _FLIP
 * (every configuration inverts a tet), _QUALITY (not better), _SIZE (a shell
 * of another size, or tets not around the edge), _NEEDS_HOST (a vertex is
 * unrounded: the call returns TW_NEEDS_EXACT_HOST).                        */
#define TW_SWAP_SUCCESS 0
#define TW_SWAP_FLIP 1
#define TW_SWAP_QUALITY 2
#define TW_SWAP_SIZE 3
#define TW_SWAP_NEEDS_HOST 4
TW_API int tw_swap_check(tw_ctx* ctx, const int32_t* v12, const int32_t* off, const int32_t* tets,
                         const int32_t* budget, int32_t n, uint8_t* result, int8_t* config,
                         uint8_t* spent);

/* ---- operator candidates and a conflict-free batch, on the device ------------------
 * No counterpart in the reference, which applies its operators one at a time
 * from priority queues; this is a parallel schedule, a separate mode whose
 * results differ from the reference's sequential passes.  The candidates
 * mirror the queues' (EdgeSplitter.cpp:37-73, EdgeCollapser.cpp:19-81): for
 * op = TW_OP_SPLIT every edge of tets[ntets][4] whose squared length exceeds
 * ideal_weight * s^2, longest first; for TW_OP_COLLAPSE both directions
 * (v1 -> v2) of every edge shorter than that, shortest first (s = the mean of
 * the two vertices' scale[], 1 when scale is NULL; equal lengths in edge
 * order; the caller filters locked or box-bound vertices).  Squared lengths
 * use the resident positions.  The batch: the greedy choice in that priority
 * order of candidates whose tets are pairwise disjoint (a split's tets: those
 * around its edge; a collapse's: those around v1).  out_v12[2 * cap]: the
 * chosen (v1, v2) in priority order (at most cap written); *n_sched: how
 * many were chosen; *n_cand: how many candidates there were.             */
#define TW_OP_SPLIT 0
#define TW_OP_COLLAPSE 1
TW_API int tw_schedule_edges(tw_ctx* ctx, const int32_t* tets, int32_t ntets, const double* scale,
                             double ideal_weight, int op, int32_t* out_v12, int32_t cap,
                             int32_t* n_sched, int32_t* n_cand);

/* ---- CUDA graphs of the context stream -------------------------------------------
 * Capture the _device calls issued between begin and end into an executable
 * graph and replay it with one launch (the inputs are re-read from the same
 * device pointers at every replay).  No counterpart in the reference.      */
TW_API int tw_capture_begin(tw_ctx* ctx);
TW_API int tw_capture_end(tw_ctx* ctx, void** graph_exec);
TW_API int tw_graph_launch(tw_ctx* ctx, void* graph_exec);
TW_API int tw_graph_destroy(void* graph_exec);

/* ---- pinned host memory for fast copies --------------------------------------- */
TW_API int tw_host_alloc(size_t bytes, void** out);
TW_API int tw_host_free(void* p);

/* ---- serving loop ----------------------------------------------------------------
 * No counterpart in the reference (TetWild runs one job per process).  A
 * server holds many meshing jobs resident in HBM (their input and boundary
 * surfaces as LBVHs, their vertex arrays) and serves their query batches as
 * they arrive: a dispatcher thread takes the waiting requests, joins point
 * and face requests of any jobs into one launch (a segment per request), and
 * runs each batch on one of `lanes` CUDA streams, so batches overlap on the
 * device and a request that arrives while others run joins the next batch
 * as soon as a lane is free.  Results are identical to the single-job
 * entry points on the same inputs (alone or in any mix).
 *
 * Jobs are admitted against the HBM budget: tw_server_job_open returns
 * TW_BUSY when the job's estimated footprint does not fit beside the open
 * jobs and the lanes' scratch; the caller retries after a job closes.
 * Request buffers are host (or device-accessible) memory that must stay
 * valid until tw_server_wait returns for the ticket.                        */
typedef struct tw_server tw_server;

#define TW_REQ_POINTS 0   /* isPointOutEnvelop: in0 = P[n][3], out0 = u8[n]             */
#define TW_REQ_FACES 1    /* isFaceOutEnvelop: in0 = tris[n][9], out0 = u8[n]           */
#define TW_REQ_AMIPS 2    /* E/J/H: in0 = T_soa[12][n]; out0 = E, out1 = J, out2 = H,
                             out3 = flip (any may be NULL); flags TW_REQ_RAW = raw energy  */
#define TW_REQ_SMOOTH 3   /* smoothing pass over n stars of the job's resident mesh:
                             in0 = star_off[n+1], in1 = tets, in2 = face_flags, in3 =
                             centers, in4 = kinds; out0 = out[n][3], out1 = status[n];
                             flags TW_REQ_APPLY writes accepted positions into the mesh   */
#define TW_REQ_RAW 1
#define TW_REQ_APPLY 2

typedef struct tw_request {
    int32_t kind;
    int32_t flags;
    int64_t n;
    const void* in0;
    const void* in1;
    const void* in2;
    const void* in3;
    const void* in4;
    void* out0;
    void* out1;
    void* out2;
    void* out3;
} tw_request;

typedef struct tw_server_stats {
    uint64_t jobs_open;
    uint64_t bytes_used;       /* jobs + lanes */
    uint64_t budget;
    uint64_t requests_done;
    uint64_t batches;
    uint64_t queries_done;
    uint64_t max_requests_per_batch;
} tw_server_stats;

TW_API int tw_server_create(int device, size_t hbm_budget, int lanes, tw_server** out);
TW_API int tw_server_destroy(tw_server* srv);
TW_API const char* tw_server_last_error(tw_server* srv);
/* Precision mode, Newton caps and launch shape for every request.          */
TW_API int tw_server_set_params(tw_server* srv, int precision, int newton_max_step,
                                int newton_max_it, int newton_shape);
TW_API int tw_server_job_open(tw_server* srv, const double* V, int32_t nv, const int32_t* F,
                              int32_t nf, double eps_2, double sampling_dist, int32_t* job);
TW_API int tw_server_job_boundary(tw_server* srv, int32_t job, const double* V, int32_t nv,
                                  const int32_t* F, int32_t nf);
/* Resident vertex positions for TW_REQ_SMOOTH (waits for the job's requests
 * in flight, at most timeout_s).                                           */
TW_API int tw_server_job_mesh(tw_server* srv, int32_t job, const double* xyz, int32_t nv,
                              double timeout_s);
TW_API int tw_server_job_read_mesh(tw_server* srv, int32_t job, double* xyz, double timeout_s);
/* Waits (at most timeout_s) for the job's requests, then frees its memory. */
TW_API int tw_server_job_close(tw_server* srv, int32_t job, double timeout_s);
/* Cancels a job mid-flight: its requests still waiting for a batch complete
 * at once with TW_ERR_CANCELLED (tw_server_wait returns it; their outputs are
 * not written), new submissions for it are refused, the batches already on a
 * lane finish (waited for at most timeout_s), then its memory is freed as by
 * tw_server_job_close.  On TW_ERR_TIMEOUT the queued requests are cancelled
 * and the job stays open; call again to free it.  Other jobs are unaffected. */
TW_API int tw_server_job_cancel(tw_server* srv, int32_t job, double timeout_s);
TW_API int tw_server_submit(tw_server* srv, int32_t job, const tw_request* req, uint64_t* ticket);
/* Waits at most timeout_s for the request; returns its status (TW_ERR_TIMEOUT
 * if not done yet: wait again).  latency_ms: submit to completion.          */
TW_API int tw_server_wait(tw_server* srv, uint64_t ticket, double timeout_s, double* latency_ms);
TW_API int tw_server_get_stats(tw_server* srv, tw_server_stats* out);

/* ---- device self-test -----------------------------------------------------------
 * No counterpart in the reference.  Checks, on `samples` pseudo-random bit
 * patterns, the integer-arithmetic binary64 <-> binary32 conversions that the
 * certified mode relies on against the hardware conversions; failures[0]
 * counts round-to-nearest double->float mismatches, failures[1] exact
 * float->double mismatches.  Both must be 0.                               */
TW_API int tw_self_test(tw_ctx* ctx, uint64_t samples, uint64_t* failures);
/* The bounded wait of the bulk-copy AMIPS kernel: a barrier no copy completes
 * must give up after `limit` polls (1 .. 2^20) and one fed by a bulk copy must
 * complete.  result = {1 when the first gave up, 1 when the second completed,
 * clock cycles the first took, the bits of the first copied double (1.5)}.
 * The kernel faults nothing and leaves no copy in flight.                    */
TW_API int tw_self_test_wait(tw_ctx* ctx, int32_t limit, uint64_t* result);

/* ---- measured pipe peaks (roofline denominators) ------------------------------
 * Times a dependent-FMA loop over the whole GPU and returns FP64 and FP32
 * FMA throughput in TFLOP/s (2 flops per FMA).                              */
TW_API int tw_probe_peaks(tw_ctx* ctx, double* fp64_tflops, double* fp32_tflops);

#ifdef __cplusplus
}
#endif
#endif /* TW_GB300_H */
