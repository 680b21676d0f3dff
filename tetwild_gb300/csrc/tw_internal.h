// tw_internal.h -- host-side declarations shared by the .cu files of
// libtw_gb300.so (not part of the public C-ABI; see include/tw_gb300.h).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/tw_gb300.h"

namespace tw {

// Surface BVH (LBVH, Karras 2012) resident in HBM.  Node i (internal,
// 0 <= i < nf-1) stores the boxes of both children and their indices; a
// child index c >= 0 is an internal node, c < 0 is leaf ~c.  Leaves are the
// facets in Morton order; tri holds their 9 coordinates (72 B per facet).
struct alignas(16) BvhNode {
    double lo0[3], hi0[3];
    double lo1[3], hi1[3];
    int32_t child[2];
    int32_t pad[6];
};
static_assert(sizeof(BvhNode) == 128, "BvhNode must be one 128-byte line");

// The same tree with binary32 boxes rounded outward (lo down, hi up), for the
// FP32 culling of the certified precision mode: 64 bytes per node.
struct alignas(16) BvhNode32 {
    float lo0[3], hi0[3];
    float lo1[3], hi1[3];
    int32_t child[2];
    int32_t pad[2];
};
static_assert(sizeof(BvhNode32) == 64, "BvhNode32 must be 64 bytes");

// Per-facet data for certified binary32 bounds of the point-facet distance,
// all computed in FP64 and rounded to binary32: vertex a as a two-float pair
// (ah = nearest binary32, al = a - ah rounded), unit normal n, the in-plane
// outward unit edge normals ne[e] with offsets c[e] = ne[e] . (v_e - a), the
// offsets o[e] = t_e . (v_e - a) along the unit edge directions
// t_e = n x ne[e], and the edge lengths.  ok = 0 for facets whose normal is
// not accurate to far better than binary32 (degenerate or sliver facets):
// they always take the FP64 test.
struct alignas(16) FacetCull {
    float ah[3];
    float al[3];
    float n[3];
    float ne[3][3];
    float c[3];
    float o[3];
    float len[3];
    uint32_t ok;
    float pad[4];
};
static_assert(sizeof(FacetCull) == 128, "FacetCull must be 128 bytes");

// Uniform grid over the surface for the certified envelope test: cell size c
// (the same on every axis), origin lo; cell (i, j, k) lists every leaf within
// R = eps (1 + 2^-18) + 2^-17 M (M = the largest coordinate magnitude of the
// grown box) of the cell: the cells of the leaf's box grown by R that a
// separating-axis test cannot separate from the triangle (the cube of
// half-size c/2 + R around the cell's centre).  Any point within the
// certified culling radius of a leaf finds that leaf in the list of its own
// cell (the margin covers the binary32 cell index), so one cell's list
// replaces the tree walk.  Built for one eps2 (rebuilt when it changes).
// Only the non-empty cells are stored, in an open-addressing hash table
// (power-of-two size, at most half full) of 16-byte slots read in one load:
// key = cell index (i + n0 (j + n1 k), below 2^32 - 1), then the first entry
// in list and the count; a cell's list holds
// its leaves in ascending order.
struct EnvGrid {
    float lo[3] = {0, 0, 0};
    float inv_c = 0.0f;
    int32_t n[3] = {0, 0, 0};
    uint4* slot = nullptr;     // hash slots: (cell index or 0xffffffff (empty), first, count, -)
    uint32_t shift = 32;       // slot = (cell * 0x9E3779B1) >> shift
    uint32_t mask = 0;
    int32_t* list = nullptr;   // leaf indices
    double eps2 = -1.0;        // the eps2 it was built for (-1: none)
    double cell_factor = 0.0;  // and the cell-size factor
    size_t slot_bytes = 0, list_bytes = 0;
    // The bin index of the point test (boff == nullptr: none; the hash grid
    // serves): cubic bins of side 1/binv from blo, bn per axis (at most 256),
    // in the Morton order of their coordinates (bits per axis: bbits); the
    // entries of bin b are boff[b] .. boff[b + 1] - 1 (boff: 2^(3 bbits) + 1
    // exclusive sums, so the entries of consecutive bins are consecutive),
    // its leaves in ascending order, each with the 512-bit mask of the bin's
    // 8x8x8 fine cells whose cube (half-size c/8/2 + R) a separating-axis
    // test cannot separate from the leaf.  A point tests the leaves whose
    // mask holds its fine cell: the same leaves a grid of cell c/8 would list.
    float blo[3] = {0, 0, 0};
    float binv = 0.0f;
    int32_t bn[3] = {0, 0, 0};
    int32_t bbits = 0;
    uint32_t* boff = nullptr;   // first entry of each bin (Morton index), and the total
    uint32_t* bent = nullptr;   // mask words 0..15 [16 x nt] (word-major), then the leaves [nt]
    int64_t bnt = 0;            // entries
    double bin_factor = 0.0;    // bin side / mean facet extent it was built for
    size_t boff_bytes = 0, bent_bytes = 0;
    // dense id of each bin with entries (Morton order), -1 for an empty bin:
    // point queries are sorted on these nocc ids
    int32_t* bid = nullptr;
    int32_t nocc = 0;
    size_t bid_bytes = 0;
};

struct Surface {
    int32_t nf = 0;
    BvhNode* nodes = nullptr;   // nf-1 internal nodes (none when nf == 1)
    BvhNode32* nodes32 = nullptr;
    FacetCull* cull = nullptr;  // per leaf (Morton order)
    double* tri = nullptr;      // 9 * nf, Morton order
    int32_t* facet_id = nullptr;  // input facet index of each leaf
    double scale = 0.0;         // max |coordinate| over the surface
    double lo[3] = {0, 0, 0};   // box of the facet centroids (Morton grid of the tree;
    double hi[3] = {0, 0, 0};   // query points are ordered on the same grid)
    size_t bytes = 0;
    EnvGrid grid;
};

// Device scratch for ordering query points by Morton cell before traversal
// (a counting sort): bin and rank per point, the permutation, the bin counts
// and the scan temporaries.  knob: the sort_points tuning value (1 = bins
// sized from n, 2..8 = bits a side).
size_t env_sort_scratch_bytes(int64_t n, int knob);

// Device memory block owned by a context, grown on demand.
struct Buffer {
    void* ptr = nullptr;
    size_t cap = 0;
};

}  // namespace tw

struct tw_ctx {
    int device = 0;
    size_t budget = 0;     // bytes of HBM the context may hold (0 = unlimited)
    size_t used = 0;       // bytes currently held
    cudaStream_t stream = nullptr;
    cudaStream_t copy_in = nullptr;
    cudaStream_t copy_out = nullptr;
    cudaEvent_t ev[8] = {};
    double eps2 = 0.0;
    double sampling_dist = 0.0;
    int newton_max_step = 15;
    int newton_max_it = 20;
    tw::Surface surf[2];   // TW_SURFACE_INPUT, TW_SURFACE_BOUNDARY
    // resident mesh vertices (SoA) and rounded flags
    double* vx = nullptr;
    double* vy = nullptr;
    double* vz = nullptr;
    uint8_t* rounded = nullptr;
    int32_t nv = 0;
    size_t mesh_bytes = 0;
    int precision = TW_PRECISION_FP64;
    int energy_form = TW_ENERGY_FORM_REFERENCE;   // tw_set_energy_form
    int newton_shape = 5;  // launch shape of the Newton step (tw_newton_autotune)
    double grid_cell = 0.2;   // envelope grid cell size / mean facet extent (TW_TUNE_GRID_CELL)
    double bin_cell = 0.25;   // point-test bin side / mean facet extent (TW_TUNE_BIN_CELL; 0: none)
    // launch timing of the point-envelope test kernel (TW_TUNE_TIME_KERNELS):
    // a ring of event pairs recorded around each launch
    static constexpr int kTimeRing = 64;
    int time_kernels = 0;
    int time_count = 0;
    cudaEvent_t time_ev[2 * kTimeRing] = {};
    int sort_points = 1;     // Morton-order point queries (TW_TUNE_SORT_POINTS)
    int point_block = 384;   // threads per block of the certified grid test (TW_TUNE_POINT_BLOCK)
    tw::Buffer scratch[10];
    // device counters, see the kCnt* indices below
    unsigned long long* counters = nullptr;
    std::string last_error;
};

namespace tw {
constexpr int kNumCounters = 16;
constexpr int kCntExactOrient = 0;    // orientations decided by the exact expansion path
constexpr int kCntUnrounded = 1;      // tets with an unrounded vertex (per call)
constexpr int kCntError = 2;          // device error word (bits, see sync_status)
constexpr int kCntEnvFacetTests = 3;  // facets reached by the traversal
constexpr int kCntEnvFp64 = 4;        // facets evaluated in FP64
constexpr int kCntAmipsTets = 5;      // tets evaluated by the AMIPS kernels
constexpr int kCntAmipsFp64 = 6;      // tets recomputed in FP64 (certified mode)
constexpr int kCntBad = 7;            // host-visible argument check flag
constexpr int kCntEnvQueries = 8;     // envelope sample/point queries
constexpr int kCntEnvWarpFallback = 9;  // warps whose shared candidate list overflowed
// internal star states of a smoothing pass (the final ones are TW_SMOOTH_*)
constexpr uint8_t kSmoothPendingProject = 6;   // surface star moved by Newton, not yet projected
constexpr uint8_t kSmoothPendingEnvelope = 7;  // surface star waiting for its face tests
// internal states of a collapse check (the final ones are the reference's 0..3)
constexpr uint8_t kCollapsePending = 255;
constexpr uint8_t kCollapsePendingEnvelope = 254;
}  // namespace tw

namespace tw {

// Error helpers (implemented in tw_capi.cu).
int fail(tw_ctx* c, int code, const std::string& msg);
// Waits for the context's streams and turns a CUDA error or the device error
// word into a status (and message).
int stream_status(tw_ctx* c, const char* where);
int cuda_fail(tw_ctx* c, cudaError_t e, const char* where);
int ensure(tw_ctx* c, int slot, size_t bytes, void** out);
int dev_alloc(tw_ctx* c, size_t bytes, void** out);
void dev_free(tw_ctx* c, void* p, size_t bytes);

// Grid size for grid-stride kernels: a multiple of the SM count.
int grid_for(int64_t n, int block, int blocks_per_sm);

// ---- launchers (tw_amips.cu) ----
// form: TW_ENERGY_FORM_* of the binary64 AMIPS evaluations (every launcher
// below that evaluates energies takes it last, the reference form by default).
void launch_amips_soa(const double* T, int64_t n, int mode, double* E, double* J, double* H,
                      uint8_t* flip, unsigned long long* exact_count, cudaStream_t s,
                      int form = TW_ENERGY_FORM_REFERENCE);
// certified binary32 variant; counters is the context's counter array;
// recheck_scratch: amips_recheck_scratch_bytes(n) device bytes (256-byte
// aligned) for the list of tets recomputed in FP64 (none may share it while
// the launch runs)
void launch_amips_soa_cert(const double* T, int64_t n, int mode, double* E, double* J, double* H,
                           uint8_t* flip, unsigned long long* counters, void* recheck_scratch,
                           cudaStream_t s, int form = TW_ENERGY_FORM_REFERENCE);
size_t amips_recheck_scratch_bytes(int64_t n);
// the context's recheck scratch (slot 9) for `parts` concurrent launches of
// up to n tets each; part k starts at *out + k * amips_recheck_scratch_bytes(n)
int amips_recheck_scratch(tw_ctx* c, int64_t n, int parts, char** out);
void launch_tet_quality_idx(const int32_t* tets, int64_t n, const double* vx, const double* vy,
                            const double* vz, const uint8_t* rounded, double* E, uint8_t* flip,
                            uint8_t* needs_host, unsigned long long* counters, cudaStream_t s,
                            int form = TW_ENERGY_FORM_REFERENCE);

// Energy sweeps: block_sum holds energy_stats_blocks(n) double-doubles; acc
// 14 words zeroed by the caller (max bits, second-max bits, unlocked count,
// 11 buckets); sum_out the unlocked energies' sum.
int energy_stats_blocks(int64_t n);
// The bounded-wait self-test (tw_amips.cu): src 16 bytes, 16-byte aligned, on
// the device; out 4 words on the device.
void launch_selftest_wait(const double* src, int limit, unsigned long long* out, cudaStream_t s);
// Dihedral sweep: block_sum holds 2 x energy_stats_blocks(n) double-doubles;
// acc 9 words set by the caller (min bits = 10.0's, max bits 0, 6 threshold
// counts, unlocked count); sums_out the unlocked mins' and maxes' sums;
// mins / maxs per tet (may be null).
void launch_dihedral_stats(const int32_t* tets, int64_t n, const double* vx, const double* vy,
                           const double* vz, const uint8_t* locked, double* mins, double* maxs,
                           void* block_sum, unsigned long long* acc, double* sums_out,
                           cudaStream_t s);
void launch_energy_stats(const int32_t* tets, int64_t n, const double* vx, const double* vy,
                         const double* vz, const uint8_t* locked, double thres,
                         void* block_sum, unsigned long long* acc, double* sum_out,
                         cudaStream_t s, int form = TW_ENERGY_FORM_REFERENCE);

// ---- launchers (tw_lbvh.cu) ----
int build_surface(tw_ctx* c, Surface& S, const double* dV, int32_t nv, const int32_t* dF,
                  int32_t nf, cudaStream_t s);
void free_surface(tw_ctx* c, Surface& S);
// (Re)builds S.grid for eps2 when it was built for another one (tw_envelope.cu).
int build_env_grid(tw_ctx* c, Surface& S, double eps2, double cell_factor, cudaStream_t s);
void free_env_grid(tw_ctx* c, EnvGrid& G);

// ---- launchers (tw_envelope.cu) ----
// err: device word; bit 0 = traversal exceeded its bounds, bit 1 = a face
// exceeded the per-row sample bound.
// sort_scratch (env_sort_scratch_bytes(n, sort_knob) bytes) enables Morton-ordered
// traversal; with nullptr the points are traversed in input order.
// precision: TW_PRECISION_FP64 or TW_PRECISION_FP32_CERTIFIED; counters is
// the context's counter array (error word and statistics).
void launch_env_points(const Surface& S, const double* P, int64_t n, double eps2, uint8_t* out,
                       int precision, unsigned long long* counters, void* sort_scratch,
                       int sort_knob, int point_block, cudaStream_t s, cudaEvent_t ev_begin = nullptr,
                       cudaEvent_t ev_end = nullptr);
void launch_env_faces(const Surface& S, const double* tris, int64_t n, double eps2, double sd,
                      uint8_t* out, int precision, unsigned long long* counters, cudaStream_t s);
void launch_sample_triangle(const double* tri, double sd, double* out, int64_t cap,
                            int64_t* count, cudaStream_t s);
// faces whose count *n_dev (<= cap) is known only on the device
void launch_env_faces_dev(const Surface& S, const double* tris, const unsigned long long* n_dev,
                          int64_t cap, double eps2, double sd, uint8_t* out, int precision,
                          unsigned long long* counters, cudaStream_t s);
// Several jobs per launch: segs is a device array of nsegs env_seg_bytes()
// records filled by fill_env_seg (ascending begin offsets, the first 0).
size_t env_seg_bytes();
void fill_env_seg(void* dst, const Surface& S, int64_t begin, double eps2, double sd);
void launch_env_points_segs(const double* P, int64_t n, const void* segs, int nsegs, uint8_t* out,
                            int precision, unsigned long long* counters, cudaStream_t s);
void launch_env_faces_segs(const double* tris, int64_t n, const void* segs, int nsegs, uint8_t* out,
                           int precision, unsigned long long* counters, cudaStream_t s);
// eps2: the grid shortcut applies when a surface's grid was built for it
void launch_nearest_points(const Surface& S, double eps2, const double* P, int64_t n, double* Q,
                           double* D, int32_t* F, unsigned long long* counters, cudaStream_t s);
void launch_smooth_project(const Surface& Sin, const Surface& Sb, double eps2,
                           const uint8_t* kinds, int32_t nstars, uint8_t* status, double* pnew,
                           unsigned long long* counters, cudaStream_t s);

// ---- launchers (tw_newton.cu) ----
void launch_newton_stars(const double* vx, const double* vy, const double* vz,
                         const int32_t* star_off, const int32_t* tets, const int32_t* centers,
                         int32_t nstars, int max_step, int max_it, double* out, uint8_t* moved,
                         cudaStream_t s, int form = TW_ENERGY_FORM_REFERENCE);
// shape in [0, newton_num_shapes()): lanes per star and block size (see
// kNewtonShapes); every shape gives bit-identical results.
int newton_num_shapes();
void newton_shape_info(int shape, int* group, int* block);
void launch_newton_stars_shape(int shape, const double* vx, const double* vy, const double* vz,
                               const int32_t* star_off, const int32_t* tets,
                               const int32_t* centers, int32_t nstars, int max_step, int max_it,
                               double* out, uint8_t* moved, cudaStream_t s,
                               int form = TW_ENERGY_FORM_REFERENCE);

// Smoothing pass (tw_newton.cu): stage 1 = validity + NewtonsMethod (interior
// stars finish here, surface stars become kSmoothPendingProject with their
// Newton position in pnew); stage 2 (after launch_smooth_project) = flip and
// quality checks at the projected position and the list of one-ring surface
// faces (appended at face_count; face_base/face_cnt per star); finalize =
// the face results decide the surface stars.
void launch_smooth_stage1(int shape, const double* vx, const double* vy, const double* vz,
                          const int32_t* star_off, const int32_t* tets, const int32_t* centers,
                          const uint8_t* kinds, int32_t nstars, int max_step, int max_it,
                          double* out, double* pnew, uint8_t* status, cudaStream_t s,
                          int form = TW_ENERGY_FORM_REFERENCE);
void launch_smooth_stage2(int shape, const double* vx, const double* vy, const double* vz,
                          const int32_t* star_off, const int32_t* tets, const uint8_t* face_flags,
                          const int32_t* centers, int32_t nstars, const double* pnew,
                          uint8_t* status, double* faces, unsigned long long* face_count,
                          int64_t face_cap, int32_t* face_base, int32_t* face_cnt,
                          unsigned long long* counters, cudaStream_t s,
                          int form = TW_ENERGY_FORM_REFERENCE);
void launch_smooth_finalize(int32_t nstars, const int32_t* face_base, const int32_t* face_cnt,
                            const uint8_t* face_out, const double* pnew, double* out,
                            uint8_t* status, cudaStream_t s);

// Scratch of a smoothing pass (context slot 8): per star the Newton /
// projected position, face range and state; per possible face (3 per tet)
// its nine coordinates and decision; the face counter (tw_capi.cu).
struct SmoothScratch {
    double* pnew;
    int32_t* face_base;
    int32_t* face_cnt;
    double* faces;
    uint8_t* face_out;
    unsigned long long* face_count;
    int64_t face_cap;
};
int smooth_scratch(tw_ctx* c, int32_t nstars, int64_t ntets, SmoothScratch& S);
// The pass over device arrays with the context's mesh, surfaces, parameters
// and stream; asynchronous.
void smooth_launch(tw_ctx* c, const int32_t* off, const int32_t* tets, const uint8_t* ff,
                   const int32_t* cen, const uint8_t* kinds, int32_t nstars, bool any_surface,
                   double* out, uint8_t* status, const SmoothScratch& S);

// Collapse checks (tw_envelope.cu / tw_newton.cu): point envelopes and the
// degenerate flag, then flip / quality / face list, then the face results.
void launch_collapse_points(const Surface& Sin, const Surface& Sb, double eps2, int precision,
                            const double* vx, const double* vy, const double* vz,
                            const int32_t* v12, const uint8_t* flags, int32_t n, uint8_t* status,
                            uint8_t* degenerate, unsigned long long* counters, cudaStream_t s);
void launch_collapse_stage(int shape, const double* vx, const double* vy, const double* vz,
                           const int32_t* off, const int32_t* tets, const uint8_t* face_flags,
                           const int32_t* v12, const uint8_t* flags, const uint8_t* degenerate,
                           int32_t n, int check_quality, double soft_energy, uint8_t* status,
                           double* faces, unsigned long long* face_count, int64_t face_cap,
                           int32_t* face_base, int32_t* face_cnt, unsigned long long* counters,
                           cudaStream_t s, int form = TW_ENERGY_FORM_REFERENCE);
void launch_collapse_finalize(int32_t n, const int32_t* face_base, const int32_t* face_cnt,
                              const uint8_t* face_out, uint8_t* status, cudaStream_t s);

// ---- edge-removal checks (tw_swap.cu) ----
void launch_swap_check(const double* vx, const double* vy, const double* vz,
                       const uint8_t* rounded, int32_t nv, const int32_t* v12, const int32_t* off,
                       const int32_t* tets, const int32_t* budget, int32_t n, uint8_t* result,
                       int8_t* config, uint8_t* spent, unsigned long long* counters,
                       cudaStream_t s, int form = TW_ENERGY_FORM_REFERENCE);

// ---- operator scheduling (tw_schedule.cu): device tets [nt][4] and scale
// [nv] (may be null); out_v12 device [2 * cap] ----
int schedule_edges(tw_ctx* c, const int32_t* dtets, int64_t nt, const double* dscale,
                   double ideal_weight, int op, int32_t* out_v12, int32_t cap, int32_t* n_sched,
                   int32_t* n_cand, cudaStream_t s);

// ---- peak probes (tw_capi.cu) ----
void launch_fp64_probe(double* out, int iters, int blocks, cudaStream_t s);
void launch_fp32_probe(float* out, int iters, int blocks, cudaStream_t s);

}  // namespace tw
