// tw_envelope.cu -- envelope tests against the device LBVH.
//
// Decision (isPointOutEnvelop, LocalOperations.cpp:1034-1044): a point is
// out iff every facet f has sqdist(p, f) > eps2.  The traversal stops at the
// first facet with sqdist <= eps2, as facet_in_envelope_recursive does
// (mesh_AABB.cpp:482-548), and skips a child box only when its squared
// distance exceeds (eps + tau)^2 with tau = 64 * 2^-53 * max|coord|, which
// covers the rounding of both the box distance and the facet distance: no
// facet that tests <= eps2 is ever skipped, so the decision equals the
// brute-force decision over all facets.
//
// Faces (isFaceOutEnvelop_sampling, :1046-1109): a warp per face; the lanes
// generate sampleTriangle's samples (Common.cpp:143-228) with the same
// arithmetic as the reference order, each lane first retests the facet that
// held its previous sample (the reference's prev_facet hint, :1080-1083),
// and the warp stops at the first sample that is out.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include "tw_device.cuh"
#include "tw_internal.h"

namespace tw {

constexpr int kStack = 64;  // > max depth of a 30-bit LBVH with index tie-break (63)
// fine cells a side of a bin of the point test's bin index, and the 32-bit
// words of an entry's fine-cell mask
constexpr int kFine = 8;
constexpr int kFineWords = kFine * kFine * kFine / 32;

__device__ __forceinline__ double prune_threshold(const V3& p, double eps2, double scale) {
    double m = scale;
    m = fmax(m, fabs(p.x));
    m = fmax(m, fabs(p.y));
    m = fmax(m, fabs(p.z));
    double eps = sqrt(eps2);
    double tau = 64.0 * kEps * m + 4.0 * kEps * eps;
    return (eps + tau) * (eps + tau);
}

__device__ __forceinline__ double leaf_sqdist(const double* __restrict__ tri, int32_t leaf,
                                              const V3& p) {
    const double* t = tri + 9 * (int64_t)leaf;
    V3 a{__ldg(t + 0), __ldg(t + 1), __ldg(t + 2)};
    V3 b{__ldg(t + 3), __ldg(t + 4), __ldg(t + 5)};
    V3 c{__ldg(t + 6), __ldg(t + 7), __ldg(t + 8)};
    return point_tri_sqdist(p, a, b, c);
}

constexpr int32_t kTraversalError = -2;

#include "tw_envcert.cuh"

// One atomic per warp for the traversal statistics.
__device__ __forceinline__ void flush_stats(const TravStats& st, unsigned long long* counters,
                                            uint32_t queries) {
    unsigned long long a = st.facets, b = st.fp64, q = queries;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        q += __shfl_xor_sync(0xffffffffu, q, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (a) atomicAdd(counters + kCntEnvFacetTests, a);
        if (b) atomicAdd(counters + kCntEnvFp64, b);
        if (q) atomicAdd(counters + kCntEnvQueries, q);
    }
}

// Returns the leaf index of a facet within eps2 of p, -1 if none, or
// kTraversalError if the walk exceeded its bounds (a tree that is not a
// tree); every internal node is visited at most once per query.
__device__ __forceinline__ int32_t find_facet_within(const BvhNode* __restrict__ nodes,
                                                     const double* __restrict__ tri, int32_t nf,
                                                     const V3& p, double eps2, double thr,
                                                     TravStats& st) {
    if (nf == 1) {
        ++st.facets;
        ++st.fp64;
        return leaf_sqdist(tri, 0, p) <= eps2 ? 0 : -1;
    }
    int32_t stack[kStack];
    int sp = 0;
    int32_t cur = 0;
    for (int32_t iter = 0; iter < nf; ++iter) {
        if ((uint32_t)cur >= (uint32_t)(nf - 1)) return kTraversalError;
        const double2* nd = reinterpret_cast<const double2*>(nodes + cur);
        double2 q0 = __ldg(nd + 0), q1 = __ldg(nd + 1), q2 = __ldg(nd + 2);
        double2 q3 = __ldg(nd + 3), q4 = __ldg(nd + 4), q5 = __ldg(nd + 5);
        int2 ch = __ldg(reinterpret_cast<const int2*>(nd + 6));
        double lo0[3] = {q0.x, q0.y, q1.x}, hi0[3] = {q1.y, q2.x, q2.y};
        double lo1[3] = {q3.x, q3.y, q4.x}, hi1[3] = {q4.y, q5.x, q5.y};
        double d0 = point_box_sqdist(p, lo0, hi0);
        double d1 = point_box_sqdist(p, lo1, hi1);
        bool h0 = d0 <= thr, h1 = d1 <= thr;
        if (h0 && ch.x < 0) {
            if ((uint32_t)(~ch.x) >= (uint32_t)nf) return kTraversalError;
            ++st.facets;
            ++st.fp64;
            if (leaf_sqdist(tri, ~ch.x, p) <= eps2) return ~ch.x;
            h0 = false;
        }
        if (h1 && ch.y < 0) {
            if ((uint32_t)(~ch.y) >= (uint32_t)nf) return kTraversalError;
            ++st.facets;
            ++st.fp64;
            if (leaf_sqdist(tri, ~ch.y, p) <= eps2) return ~ch.y;
            h1 = false;
        }
        if (h0 && h1) {
            if (sp >= kStack) return kTraversalError;
            int32_t nearc = (d0 <= d1) ? ch.x : ch.y;
            int32_t farc = (d0 <= d1) ? ch.y : ch.x;
            stack[sp++] = farc;
            cur = nearc;
        } else if (h0) {
            cur = ch.x;
        } else if (h1) {
            cur = ch.y;
        } else {
            if (sp == 0) return -1;
            cur = stack[--sp];
        }
    }
    return kTraversalError;
}

// Query i of the launch is point order[i] (order == nullptr: point i).  With
// the points in Morton order, the lanes of a warp query neighbouring points
// and walk the same nodes: the warp stays converged and the nodes it reads
// are shared in L1.
struct EnvTree {
    const BvhNode* nodes;
    const BvhNode32* nodes32;
    const FacetCull* cull;
    const double* tri;
    int32_t nf;
    double scale;
    float scale_hi;  // scale rounded up to binary32
    const int32_t* facet_id;  // input facet index of each leaf
    // the uniform grid of the certified test (gslot == nullptr: none)
    float glo[3];
    float ginv;
    int32_t gn[3];
    const uint4* gslot;   // (cell, first entry, count, -) per hash slot
    uint32_t gshift, gmask;
    const int32_t* glist;
    // the bin index of the point test (boff == nullptr: none)
    float blo[3];
    float binv;
    int32_t bn[3];
    const uint32_t* boff;   // first entry per bin (Morton index of its coordinates)
    const uint32_t* bmask;  // fine-cell mask word w of entry e at bmask[w * bnt + e]
    const int32_t* bleaf;   // leaf per entry
    int64_t bnt;            // entries
    const int32_t* bid;     // dense id per bin with entries, -1 for an empty bin
    int32_t nocc;           // bins with entries
};

template <bool FP32>
__device__ __forceinline__ int32_t query_point(const EnvTree& T, const V3& p, const EpsParams& E,
                                               TravStats& st) {
    if (FP32)
        return find_facet_within32(T.nodes32, T.cull, T.tri, T.nf, p, cert_query(p, E, T.scale_hi),
                                   E.eps2, st);
    return find_facet_within(T.nodes, T.tri, T.nf, p, E.eps2, prune_threshold(p, E.eps2, T.scale),
                             st);
}

// eps = sqrt(eps2) rounded up and down to binary32, and the scale rounded up.
static EpsParams eps_params(double eps2) {
    EpsParams E;
    E.eps2 = eps2;
    double eps = std::sqrt(eps2);
    float f = (float)eps;
    E.eps_hi = ((double)f < eps) ? std::nextafter(f, INFINITY) : f;
    E.eps_lo = ((double)f > eps) ? std::nextafter(f, 0.0f) : f;
    return E;
}
static float round_up_float(double x) {
    float f = (float)x;
    return ((double)f < x) ? std::nextafter(f, INFINITY) : f;
}
static EnvTree env_tree(const Surface& S);
// The tree with its grid when the grid was built for this eps2.
static EnvTree env_tree_for(const Surface& S, double eps2) {
    EnvTree T = env_tree(S);
    if (S.grid.eps2 != eps2) {
        T.gslot = nullptr;
        T.glist = nullptr;
        T.boff = nullptr;
        T.bmask = nullptr;
        T.bleaf = nullptr;
        T.bid = nullptr;
        T.nocc = 0;
    }
    return T;
}
static EnvTree env_tree(const Surface& S) {
    EnvTree T{S.nodes, S.nodes32, S.cull, S.tri, S.nf, S.scale, round_up_float(S.scale),
              S.facet_id};
    for (int k = 0; k < 3; ++k) {
        T.glo[k] = S.grid.lo[k];
        T.gn[k] = S.grid.n[k];
    }
    T.ginv = S.grid.inv_c;
    T.gslot = S.grid.slot;
    T.gshift = S.grid.shift;
    T.gmask = S.grid.mask;
    T.glist = S.grid.list;
    for (int k = 0; k < 3; ++k) {
        T.blo[k] = S.grid.blo[k];
        T.bn[k] = S.grid.bn[k];
    }
    T.binv = S.grid.binv;
    T.boff = S.grid.boff;
    T.bmask = S.grid.bent;
    T.bleaf = S.grid.bent ? (const int32_t*)(S.grid.bent + kFineWords * S.grid.bnt) : nullptr;
    T.bnt = S.grid.bnt;
    T.bid = S.grid.bid;
    T.nocc = S.grid.nocc;
    return T;
}

template <bool FP32, int MINB = 1>
__global__ void __launch_bounds__(128, MINB) k_env_points(const double* __restrict__ P,
                                                    const int32_t* __restrict__ order, int64_t n,
                                                    EnvTree T, EpsParams E,
                                                    uint8_t* __restrict__ out,
                                                    unsigned long long* __restrict__ counters) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    TravStats st;
    uint32_t nq = 0;
    // every lane runs the same number of iterations so the final warp
    // reduction of the statistics is converged
    const int64_t first = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t base0 = first - (threadIdx.x & 31);
    for (int64_t b = base0; b < n; b += stride) {
        const int64_t i = b + (threadIdx.x & 31);
        if (i < n) {
            const int64_t j = order ? (int64_t)__ldg(order + i) : i;
            V3 p{__ldg(P + 3 * j), __ldg(P + 3 * j + 1), __ldg(P + 3 * j + 2)};
            int32_t f = query_point<FP32>(T, p, E, st);
            if (f == kTraversalError) atomicOr(counters + kCntError, 1ULL);
            out[j] = (uint8_t)(f == -1);
            ++nq;
        }
    }
    flush_stats(st, counters, nq);
}

// ---------------------------------------------------------------------------
// Warp-shared candidates (certified mode).  With the points in Morton order
// the 32 points of a warp lie close together: the warp walks the tree once
// for the box of its points grown by the largest per-point culling radius
// (sqrt of CertQuery::thr, rounded up), collecting every leaf whose binary32
// box meets it, and each lane then tests its own point against that list.
// Every leaf that the per-point walk could reach (box within sqrt(thr) of the
// point) meets the grown box, and each leaf test is the same certified test,
// so every decision equals the per-point walk's, i.e. FP64's.  A warp whose
// box meets more than 32 leaves falls back to the per-point walk.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool box_meets(const float* lo, const float* hi, const float* qlo,
                                          const float* qhi) {
    return lo[0] <= qhi[0] && hi[0] >= qlo[0] && lo[1] <= qhi[1] && hi[1] >= qlo[1] &&
           lo[2] <= qhi[2] && hi[2] >= qlo[2];
}

// Lane k receives the k-th leaf in cand; returns the count (the same on every
// lane), -1 when above 32, kTraversalError on a malformed tree.  Every lane
// walks the same nodes (uniform control flow, broadcast loads).
__device__ __forceinline__ int warp_candidates32(const EnvTree& T, const float* qlo,
                                                 const float* qhi, int lane, int32_t& cand) {
    const int32_t nf = T.nf;
    if (nf == 1) {
        cand = 0;
        return 1;
    }
    int32_t stack[kStack];
    int sp = 0, cnt = 0;
    int32_t cur = 0;
    for (int32_t iter = 0; iter < nf; ++iter) {
        if ((uint32_t)cur >= (uint32_t)(nf - 1)) return kTraversalError;
        const float4* nd = reinterpret_cast<const float4*>(T.nodes32 + cur);
        float4 q0 = __ldg(nd + 0), q1 = __ldg(nd + 1), q2 = __ldg(nd + 2);
        int4 q3 = __ldg(reinterpret_cast<const int4*>(nd + 3));
        const float lo0[3] = {q0.x, q0.y, q0.z}, hi0[3] = {q0.w, q1.x, q1.y};
        const float lo1[3] = {q1.z, q1.w, q2.x}, hi1[3] = {q2.y, q2.z, q2.w};
        bool h0 = box_meets(lo0, hi0, qlo, qhi), h1 = box_meets(lo1, hi1, qlo, qhi);
        if (h0 && q3.x < 0) {
            if ((uint32_t)(~q3.x) >= (uint32_t)nf) return kTraversalError;
            if (lane == cnt) cand = ~q3.x;
            if (++cnt > 32) return -1;
            h0 = false;
        }
        if (h1 && q3.y < 0) {
            if ((uint32_t)(~q3.y) >= (uint32_t)nf) return kTraversalError;
            if (lane == cnt) cand = ~q3.y;
            if (++cnt > 32) return -1;
            h1 = false;
        }
        if (h0 && h1) {
            if (sp >= kStack) return kTraversalError;
            stack[sp++] = q3.y;
            cur = q3.x;
        } else if (h0) {
            cur = q3.x;
        } else if (h1) {
            cur = q3.y;
        } else {
            if (sp == 0) return cnt;
            cur = stack[--sp];
        }
    }
    return kTraversalError;
}

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <int MINB>
__global__ void __launch_bounds__(128, MINB) k_env_points_warp(const double* __restrict__ P,
                                                         const int32_t* __restrict__ order,
                                                         int64_t n, EnvTree T, EpsParams E,
                                                         uint8_t* __restrict__ out,
                                                         unsigned long long* __restrict__ counters) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    TravStats st;
    uint32_t nq = 0, fallback = 0;
    const int64_t base0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane;
    for (int64_t b = base0; b < n; b += stride) {
        const int64_t i = b + lane;
        const bool valid = i < n;
        const int64_t j = valid ? (order ? (int64_t)__ldg(order + i) : i) : 0;
        V3 p{0.0, 0.0, 0.0};
        if (valid) p = V3{__ldg(P + 3 * j), __ldg(P + 3 * j + 1), __ldg(P + 3 * j + 2)};
        const CertQuery q = cert_query(p, E, T.scale_hi);
        const float inf = __int_as_float(0x7f800000);
        const float r = valid ? __fsqrt_ru(q.thr) : 0.0f;
        const float R = warp_max(r);
        float qlo[3], qhi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            qlo[k] = __fsub_rd(warp_min(valid ? q.ph[k] : inf), R);
            qhi[k] = __fadd_ru(warp_max(valid ? q.ph[k] : -inf), R);
        }
        int32_t cand = -1;
        const int cnt = warp_candidates32(T, qlo, qhi, lane, cand);
        bool in = false;
        if (cnt >= 0) {
            for (int k = 0; k < cnt; ++k) {
                const int32_t lf = __shfl_sync(0xffffffffu, cand, k);
                if (valid && !in) in = cert_leaf_within(T.cull, T.tri, lf, p, q, E.eps2, st);
                if (__all_sync(0xffffffffu, in || !valid)) break;
            }
        } else {
            if (cnt == kTraversalError && lane == 0) atomicOr(counters + kCntError, 1ULL);
            ++fallback;
            if (valid) {
                int32_t f = query_point<true>(T, p, E, st);
                if (f == kTraversalError) atomicOr(counters + kCntError, 1ULL);
                in = f >= 0;
            }
        }
        if (valid) {
            out[j] = (uint8_t)!in;
            ++nq;
        }
    }
    flush_stats(st, counters, nq);
    if (lane == 0 && fallback) atomicAdd(counters + kCntEnvWarpFallback, (unsigned long long)fallback);
}

// ---------------------------------------------------------------------------
// Test through the uniform grid: the leaves listed in the point's own cell
// (see EnvGrid) are every leaf within its culling radius, so the point is in
// iff one of them tests in.  No tree walk; the lanes of a warp loop over
// their own lists in step.  Both precision modes use it: CERT tests each leaf
// with the certified binary32 bounds (FP64 in the band), !CERT tests each
// leaf in FP64.  A leaf whose FP64 distance tests <= eps2 lies within
// eps (1 + 2^-50) + O(2^-52 M) of the point, well inside the culling radius
// R = eps (1 + 2^-18) + 2^-17 M the cell lists cover, so both decide exactly
// as the FP64 tree walk (some facet with computed d^2 <= eps2).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void grid_cell_range(const EnvTree& T, const CertQuery& q,
                                                uint32_t& b, uint32_t& e) {
    int ix[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float t = __fmul_rn(__fsub_rn(q.ph[k], T.glo[k]), T.ginv);
        int i;
        if (!(t > 0.0f)) i = 0;
        else if (t >= (float)T.gn[k]) i = T.gn[k] - 1;
        else i = min((int)t, T.gn[k] - 1);
        ix[k] = i;
    }
    const uint32_t cell = ((uint32_t)ix[2] * (uint32_t)T.gn[1] + (uint32_t)ix[1]) *
                              (uint32_t)T.gn[0] + (uint32_t)ix[0];
    uint32_t slot = (cell * 0x9E3779B1u) >> T.gshift;
    b = e = 0;
    for (uint32_t probe = 0; probe <= T.gmask; ++probe) {
        const uint4 r = __ldg(T.gslot + slot);   // key and range in one load
        if (r.x == cell) {
            b = r.y;
            e = r.y + r.z;
            return;
        }
        if (r.x == 0xffffffffu) return;   // an empty cell: no leaf within reach
        slot = (slot + 1) & T.gmask;
    }
}

__device__ __forceinline__ bool fp64_leaf_within(const double* __restrict__ tri, int32_t lf,
                                                 const V3& p, double eps2, TravStats& st) {
    ++st.facets;
    ++st.fp64;
    return leaf_sqdist(tri, lf, p) <= eps2;
}

// in iff a leaf of the point's cell tests in; every lane of the warp calls it
template <bool CERT>
__device__ __forceinline__ bool grid_point_in(const EnvTree& T, const EpsParams& E, bool valid,
                                              const V3& p, const CertQuery& q, TravStats& st) {
    uint32_t b = 0, e = 0;
    if (valid) grid_cell_range(T, q, b, e);
    bool in = false;
    // the next list entry is loaded while the current facet is tested, so
    // each test waits on one load (its record) instead of two
    int32_t lf = b < e ? __ldg(T.glist + b) : 0;
    for (uint32_t k = b; k < e; ++k) {
        const int32_t next = k + 1 < e ? __ldg(T.glist + k + 1) : 0;
        if (CERT ? cert_leaf_within(T.cull, T.tri, lf, p, q, E.eps2, st)
                 : fp64_leaf_within(T.tri, lf, p, E.eps2, st)) {
            in = true;
            break;
        }
        lf = next;
    }
    return in;
}

// Block b's warps take 32-point groups b*W .. b*W+W-1 together (W warps per
// block), then stride by the grid: in Morton order the warps of a block test
// neighbouring cells at the same time and share their facet records in L1.
template <int BLOCK, int MINB, bool CERT>
__global__ void __launch_bounds__(BLOCK, MINB) k_env_points_grid(const double* __restrict__ P,
                                                           const int32_t* __restrict__ order,
                                                           int64_t n, EnvTree T, EpsParams E,
                                                           uint8_t* __restrict__ out,
                                                           unsigned long long* __restrict__ counters) {
    TravStats st;
    uint32_t nq = 0;
    const int64_t groups = (n + 31) >> 5;
    const int64_t warps = (int64_t)gridDim.x * (BLOCK / 32);
    for (int64_t g = (int64_t)blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5); g < groups;
         g += warps) {
        const int64_t i = (g << 5) + (threadIdx.x & 31);
        if (i < n) {
            // the points, the order and the answers stream through once
            // (evict-first), so the facet records and cell lists stay in L2
            const int64_t j = order ? (int64_t)__ldcs(order + i) : i;
            const V3 p{__ldcs(P + 3 * j), __ldcs(P + 3 * j + 1), __ldcs(P + 3 * j + 2)};
            const CertQuery q = cert_query(p, E, T.scale_hi);
            __stcs(out + j, (uint8_t)!grid_point_in<CERT>(T, E, true, p, q, st));
            ++nq;
        }
    }
    flush_stats(st, counters, nq);
}

// ---------------------------------------------------------------------------
// Test through the bin index: the point's bin and fine cell come from its
// binary32 coordinates, t = (ph - blo) * binv per axis (round to nearest):
// bin i = floor(t) and fine cell floor(8 (t - i)) (t - i is exact: t and i
// are within a factor 2, and x8 is exact), clamped to the grid, so the
// computed fine index is floor(8 t).  t is within 2^-24 |p| binv (the
// rounding of p) + 2^-23 |t| (the subtraction and the product) of its exact
// value (p - blo) binv; inside the grown box |t| / binv is at most its extent
// (below 2 M + 2 R), so that is a distance of at most 2^-24 |p| + 2^-22 (M +
// R) <= 2^-21 M per axis, well inside the 2^-17 M of the culling radius R the
// masks are built for.  A clamped coordinate (outside the grown box) maps to the
// outer cell, whose cube holds the point's projection onto the box face, no
// farther from any facet than the point.  So every leaf within the certified
// culling radius of the point is in its bin's list with its fine-cell bit set,
// and the point is in iff one of those leaves tests in (in CERT, the
// certified binary32 bounds with FP64 in the band; else FP64).
// ---------------------------------------------------------------------------
// The point's bin (Morton index) and fine cell (fx + 8 fy + 64 fz).
__device__ __forceinline__ void bin_cell_of(const EnvTree& T, const CertQuery& q, uint32_t& bin,
                                            int& fine) {
    uint32_t m = 0;
    fine = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float t = __fmul_rn(__fsub_rn(q.ph[k], T.blo[k]), T.binv);
        int i, f;
        if (!(t > 0.0f)) {   // below the grid, or NaN
            i = 0;
            f = 0;
        } else if (t >= (float)T.bn[k]) {
            i = T.bn[k] - 1;
            f = kFine - 1;
        } else {
            i = min((int)t, T.bn[k] - 1);
            f = min((int)(__fsub_rn(t, (float)i) * (float)kFine), kFine - 1);
        }
        m |= morton_expand10((uint32_t)i) << (2 - k);
        fine += f * (k == 0 ? 1 : (k == 1 ? kFine : kFine * kFine));
    }
    bin = m;
}

// The mask words of the bin's entries (the word that holds the point's fine
// cell) are read first, 32 at a time, as independent loads: the hits form a
// bit set and only the hit leaves are tested, in entry order.  DEFER (CERT
// only): a leaf in the certified band is not evaluated here; the point is in
// when another leaf tests in, and otherwise undecided (2), for the FP64 pass.
template <bool CERT, bool DEFER = false>
__device__ __forceinline__ int bins_point_test(const EnvTree& T, const EpsParams& E, const V3& p,
                                               const CertQuery& q, TravStats& st) {
    uint32_t bin;
    int fine;
    bin_cell_of(T, q, bin, fine);
    const uint32_t a = __ldg(T.boff + bin), b = __ldg(T.boff + bin + 1);
    const uint32_t* mw = T.bmask + (int64_t)(fine >> 5) * T.bnt;
    const uint32_t sh = (uint32_t)fine & 31u;
    bool band = false;
    for (uint32_t base = a; base < b; base += 32) {
        const uint32_t cnt = min(b - base, 32u);
        uint32_t hits = 0;
#pragma unroll 16
        for (uint32_t k = 0; k < cnt; ++k) hits |= ((__ldg(mw + base + k) >> sh) & 1u) << k;
        while (hits) {
            const uint32_t k = (uint32_t)(__ffs(hits) - 1);
            hits &= hits - 1u;
            const int32_t lf = __ldg(T.bleaf + base + k);
            if (DEFER) {
                ++st.facets;
                const int cls = facet_classify(T.cull, lf, q);
                if (cls == kFacetIn) return 1;
                band |= cls == kFacetBand;
            } else if (CERT ? cert_leaf_within(T.cull, T.tri, lf, p, q, E.eps2, st)
                            : fp64_leaf_within(T.tri, lf, p, E.eps2, st)) {
                return 1;
            }
        }
    }
    return band ? 2 : 0;
}

template <bool CERT>
__device__ __forceinline__ bool bins_point_in(const EnvTree& T, const EpsParams& E, const V3& p,
                                              const CertQuery& q, TravStats& st) {
    return bins_point_test<CERT>(T, E, p, q, st) == 1;
}

// recheck: (count, point indices) of the points the certified test left
// undecided (a leaf in the band and none in), for k_env_points_bins_recheck;
// nullptr: the band is evaluated in FP64 on the spot.
// A lane's point through the surface's index: the bins when built, else the
// grid's hashed cells (the same decisions).  No warp collectives: lanes
// without a point (valid false) take no part.  For point queries, of which
// about half lie outside and test every leaf in reach; face samples and
// collapse checks, mostly inside and decided by their first leaf, keep the
// grid's short cell lists (the bins' mask scan measured slower there: 38.1
// against 34.4 ms for the 200k-star smoothing pass).
template <bool CERT>
__device__ __forceinline__ bool index_point_in(const EnvTree& T, const EpsParams& E, bool valid,
                                               const V3& p, const CertQuery& q, TravStats& st) {
    if (T.boff) return valid && bins_point_in<CERT>(T, E, p, q, st);
    return grid_point_in<CERT>(T, E, valid, p, q, st);
}

// n_dev (sorted on the dense bin ids): the number of sorted queries, read on
// the device (the others were decided by the binning pass); else n.
template <int BLOCK, int MINB, bool CERT, bool DEFER>
__global__ void __launch_bounds__(BLOCK, MINB) k_env_points_bins(const double* __restrict__ P,
                                                           const int32_t* __restrict__ order,
                                                           int64_t n, EnvTree T, EpsParams E,
                                                           uint8_t* __restrict__ out,
                                                           unsigned long long* __restrict__ counters,
                                                           uint32_t* __restrict__ recheck,
                                                           const uint32_t* __restrict__ n_dev) {
    TravStats st;
    uint32_t nq = 0;
    if (n_dev) n = min(n, (int64_t)__ldg(n_dev));
    const int64_t groups = (n + 31) >> 5;
    const int64_t warps = (int64_t)gridDim.x * (BLOCK / 32);
    for (int64_t g = (int64_t)blockIdx.x * (BLOCK / 32) + (threadIdx.x >> 5); g < groups;
         g += warps) {
        const int64_t i = (g << 5) + (threadIdx.x & 31);
        if (i < n) {
            // the points, the order and the answers stream through once
            // (evict-first), so the bins, entries and facet records stay in L2
            const int64_t j = order ? (int64_t)__ldcs(order + i) : i;
            const V3 p{__ldcs(P + 3 * j), __ldcs(P + 3 * j + 1), __ldcs(P + 3 * j + 2)};
            const CertQuery q = cert_query(p, E, T.scale_hi);
            const int r = bins_point_test<CERT, DEFER>(T, E, p, q, st);
            if (DEFER && r == 2) {
                const uint32_t at = atomicAdd(recheck, 1u);
                recheck[1 + at] = (uint32_t)j;   // at < n: one entry per point
            } else {
                __stcs(out + j, (uint8_t)(r != 1));
            }
            ++nq;
        }
    }
    flush_stats(st, counters, nq);
}

// The undecided points of a deferred certified test (the decision of
// TW_PRECISION_FP64 for them).  One point per warp (lane 0): the points'
// leaves take different paths through the FP64 distance, which in one warp
// would run one after another on the slow FP64 pipe; spread over warps (and
// SMs) they run side by side.
__global__ void k_env_points_bins_recheck(const double* __restrict__ P,
                                          const uint32_t* __restrict__ recheck, EnvTree T,
                                          EpsParams E, uint8_t* __restrict__ out,
                                          unsigned long long* __restrict__ counters) {
    if ((threadIdx.x & 31) != 0) return;
    TravStats st;
    const uint32_t cnt = *recheck;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < cnt; k += warps) {
        const int64_t j = recheck[1 + k];
        const V3 p{P[3 * j], P[3 * j + 1], P[3 * j + 2]};
        const CertQuery q = cert_query(p, E, T.scale_hi);
        // the certified test again, now evaluating the band in FP64 on the
        // spot: only the leaves in the band cost a binary64 distance
        out[j] = (uint8_t)!bins_point_in<true>(T, E, p, q, st);
    }
    // no flush_stats: the counters count each point's certified tests once;
    // the FP64 evaluations are added per thread
    if (st.fp64) atomicAdd(counters + kCntEnvFp64, (unsigned long long)st.fp64);
}

// ---- grid build ----------------------------------------------------------------------
// Sum over facets of the largest box extent (for the cell size).
__global__ void k_grid_mean_extent(const double* __restrict__ tri, int32_t nf,
                                   double* __restrict__ sum) {
    double acc = 0.0;
    for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf;
         f += (int64_t)gridDim.x * blockDim.x) {
        const double* t = tri + 9 * f;
        double ext = 0.0;
        for (int k = 0; k < 3; ++k) {
            const double lo = fmin(t[k], fmin(t[3 + k], t[6 + k]));
            const double hi = fmax(t[k], fmax(t[3 + k], t[6 + k]));
            ext = fmax(ext, hi - lo);
        }
        acc += ext;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, acc);
}

// Binary32 separating-axis test of one leaf against the cells of a regular
// grid (cell cs from lo, n cells a side): a cell is within reach when no
// axis (the three box axes, the triangle's normal and the nine edge x
// box-axis products) separates the triangle from the cube of half-size
// cs/2 + Rm + slack around the cell's centre, which holds the ball of radius
// Rm around every point of the cell (slack = 2^-30 M covers the cell's
// placement), so a leaf it excludes is farther than Rm from the whole cell.
// Rigorous in binary32: any direction is a valid separating axis, so the
// binary32 axes themselves are used as exact vectors and only the
// projections carry rounding.  The vertices relative to t0 (rounded once) and
// the cell centre relative to t0 (from base = lo - t0 and (x + 1/2) cs) are
// within 2^-20 L of the exact values (L = 2 (M + the grid's extent) bounds
// every coordinate and offset), so each projection onto axis a is within
// |a|_1 2^-19 L; an axis separates only by more than |a|_1 2^-18 L.  Cells no
// axis separates by that margin are kept (a longer list, never a missing leaf).
struct SatTri {
    float basef[3], vf[3][3], ef[3][3], nmf[3];
    float mL, hf, csf;
    bool sat_ok;

    __device__ __forceinline__ void init(const double* t, const double* lo, const int32_t* n,
                                         double cs, double Rm, double slack) {
        double L = 0.0;
        for (int k = 0; k < 3; ++k)
            L = fmax(L, fmax(fabs(lo[k]), fabs(lo[k] + (double)n[k] * cs)) + fabs(t[k]));
        L = 2.0 * L;
        mL = (float)ldexp(L, -18) * 1.0001f;
        hf = (float)(0.5 * cs + Rm + slack) * 1.000001f;
        csf = (float)cs;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            basef[k] = (float)(lo[k] - t[k]);
            vf[0][k] = 0.0f;
            vf[1][k] = (float)(t[3 + k] - t[k]);
            vf[2][k] = (float)(t[6 + k] - t[k]);
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            ef[0][k] = vf[1][k] - vf[0][k];
            ef[1][k] = vf[2][k] - vf[1][k];
            ef[2][k] = vf[0][k] - vf[2][k];
        }
        nmf[0] = ef[0][1] * ef[1][2] - ef[0][2] * ef[1][1];
        nmf[1] = ef[0][2] * ef[1][0] - ef[0][0] * ef[1][2];
        nmf[2] = ef[0][0] * ef[1][1] - ef[0][1] * ef[1][0];
        // 2^-40 <= L < 2^40 and |a|_1 >= 2^-40 keep every product far from
        // binary32 overflow, and underflow far below the margin (else the
        // cell is kept)
        sat_ok = L >= 0x1p-40 && L < 0x1p40;
    }
    // true when axis a (|a|_1 = a1) separates the triangle (projections p) from the cube
    __device__ __forceinline__ bool apart(const float* p, float a1) const {
        if (!(a1 >= 0x1p-40f)) return false;
        const float r = hf * a1 + a1 * mL;
        return fminf(p[0], fminf(p[1], p[2])) > r || fmaxf(p[0], fmaxf(p[1], p[2])) < -r;
    }
    // cell (x, y, z) within reach of the leaf?
    __device__ __forceinline__ bool within(int x, int y, int z) const {
        if (!sat_ok) return true;
        const float w[3] = {basef[0] + ((float)x + 0.5f) * csf, basef[1] + ((float)y + 0.5f) * csf,
                            basef[2] + ((float)z + 0.5f) * csf};
        float u[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) u[i][k] = vf[i][k] - w[k];
        float p[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {   // the box axes
            p[0] = u[0][k];
            p[1] = u[1][k];
            p[2] = u[2][k];
            if (apart(p, 1.0f)) return false;
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)   // the normal
            p[i] = nmf[0] * u[i][0] + nmf[1] * u[i][1] + nmf[2] * u[i][2];
        if (apart(p, fabsf(nmf[0]) + fabsf(nmf[1]) + fabsf(nmf[2]))) return false;
#pragma unroll
        for (int j = 0; j < 3; ++j) {   // unit_k x e_j
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
                const float a1 = -ef[j][k2], a2 = ef[j][k1];
#pragma unroll
                for (int i = 0; i < 3; ++i) p[i] = a1 * u[i][k1] + a2 * u[i][k2];
                if (apart(p, fabsf(a1) + fabsf(a2))) return false;
            }
        }
        return true;
    }
};

// The index range [i0, i1] a side of the cells (cs = 1 / inv_c from lo, n a
// side) that the leaf's box grown by Rm meets, and their number.
__device__ __forceinline__ int64_t leaf_cell_box(const double* t, const double* lo,
                                                 const int32_t* n, double inv_c, double Rm,
                                                 int* i0, int* i1) {
    for (int k = 0; k < 3; ++k) {
        const double a = fmin(t[k], fmin(t[3 + k], t[6 + k])) - Rm;
        const double b = fmax(t[k], fmax(t[3 + k], t[6 + k])) + Rm;
        double u = floor((a - lo[k]) * inv_c), v = floor((b - lo[k]) * inv_c);
        u = fmin(fmax(u, 0.0), (double)(n[k] - 1));
        v = fmin(fmax(v, 0.0), (double)(n[k] - 1));
        i0[k] = (int)u;
        i1[k] = (int)v;
    }
    return (int64_t)(i1[0] - i0[0] + 1) * (i1[1] - i0[1] + 1) * (i1[2] - i0[2] + 1);
}

// The cells within reach of every leaf (SatTri over the cells of its box
// grown by Rm).  Counting (fcnt != nullptr): the leaf's count and the total;
// filling: the (cell << 32 | leaf) pairs from foff[leaf] on.  A leaf whose
// box spans more than 2^16 cells marks the grid unsuitable (*too_big).  One
// warp per leaf; the lanes take the box's cells in turn.
__global__ void k_grid_cells(const double* __restrict__ tri, int32_t nf, double lo0, double lo1,
                             double lo2, double inv_c, int32_t n0, int32_t n1, int32_t n2,
                             double Rm, double slack, unsigned long long* __restrict__ total,
                             uint32_t* __restrict__ fcnt, const uint32_t* __restrict__ foff,
                             unsigned long long* __restrict__ pairs, int* __restrict__ too_big) {
    const int64_t f = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (f >= nf) return;   // whole warps
    double t[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) t[k] = __ldg(tri + 9 * f + k);
    const double lo[3] = {lo0, lo1, lo2};
    const int32_t n[3] = {n0, n1, n2};
    int i0[3], i1[3];
    const int64_t box = leaf_cell_box(t, lo, n, inv_c, Rm, i0, i1);
    if (box > 65536) {
        if (lane == 0) {
            if (too_big) atomicExch(too_big, 1);
            if (fcnt) fcnt[f] = 0;
        }
        return;
    }
    const int bx = i1[0] - i0[0] + 1, by = i1[1] - i0[1] + 1;
    SatTri S;
    S.init(t, lo, n, 1.0 / inv_c, Rm, slack);
    // cell q of the box (x fastest): within reach of the leaf?
    auto within = [&](int q, uint32_t& cell) {
        const int x = i0[0] + q % bx, y = i0[1] + (q / bx) % by, z = i0[2] + q / (bx * by);
        cell = ((uint32_t)z * (uint32_t)n1 + (uint32_t)y) * (uint32_t)n0 + (uint32_t)x;
        return S.within(x, y, z);
    };
    const int nbox = (int)box;
    if (fcnt) {
        uint32_t cnt = 0;
        for (int q = lane; q < nbox; q += 32) {
            uint32_t cell;
            cnt += within(q, cell) ? 1u : 0u;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if (lane == 0) {
            fcnt[f] = cnt;
            if (cnt) atomicAdd(total, (unsigned long long)cnt);
        }
        return;
    }
    // foff: exclusive sums of the counts (nf + 1 entries)
    uint32_t w = __ldg(foff + f);
    const uint32_t end = __ldg(foff + f + 1);
    for (int q0 = 0; q0 < nbox; q0 += 32) {
        const int q = q0 + lane;
        uint32_t cell = 0;
        const bool in = q < nbox && within(q, cell);
        const unsigned bal = __ballot_sync(0xffffffffu, in);
        const uint32_t at = w + __popc(bal & ((1u << lane) - 1u));
        if (in && at < end) pairs[at] = ((unsigned long long)cell << 32) | (uint32_t)f;
        w += __popc(bal);
    }
}

// The bins within reach of every leaf, with their fine-cell masks: SatTri
// over the fine grid (cell cs/8, 8n a side) for the 512 fine cells of each
// bin of the leaf's grown box (mask word w: fine cells 32 w .. 32 w + 31,
// lane l taking cell s = 32 w + l = fx + 8 fy + 64 fz); a bin with an empty
// mask is no entry.  Counting and filling as k_grid_cells; entry at: the key
// (bin << 32 | leaf; bin: the Morton index of its coordinates), its index in
// vals and its mask words in masks[w * ntot + at].  A leaf whose box spans
// more than 4096 bins marks the index unsuitable (*too_big).
__global__ void k_bin_cells(const double* __restrict__ tri, int32_t nf, double lo0, double lo1,
                            double lo2, double inv_c, int32_t n0, int32_t n1, int32_t n2,
                            double Rm, double slack, unsigned long long* __restrict__ total,
                            uint32_t* __restrict__ fcnt, const uint32_t* __restrict__ foff,
                            unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals,
                            uint32_t* __restrict__ masks, int64_t ntot,
                            int* __restrict__ too_big) {
    const int64_t f = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (f >= nf) return;   // whole warps
    double t[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) t[k] = __ldg(tri + 9 * f + k);
    const double lo[3] = {lo0, lo1, lo2};
    const int32_t n[3] = {n0, n1, n2};
    int i0[3], i1[3];
    const int64_t box = leaf_cell_box(t, lo, n, inv_c, Rm, i0, i1);
    if (box > 4096) {
        if (lane == 0) {
            if (too_big) atomicExch(too_big, 1);
            if (fcnt) fcnt[f] = 0;
        }
        return;
    }
    const int bx = i1[0] - i0[0] + 1, by = i1[1] - i0[1] + 1;
    const int32_t nfine[3] = {kFine * n0, kFine * n1, kFine * n2};
    SatTri S;
    S.init(t, lo, nfine, 1.0 / (kFine * inv_c), Rm, slack);
    uint32_t cnt = 0;
    uint32_t at = fcnt ? 0u : __ldg(foff + f);
    const uint32_t end = fcnt ? 0u : __ldg(foff + f + 1);
    for (int q = 0; q < (int)box; ++q) {
        const int x = i0[0] + q % bx, y = i0[1] + (q / bx) % by, z = i0[2] + q / (bx * by);
        uint32_t mine = 0, any = 0;   // lane w keeps word w
#pragma unroll 1
        for (int w = 0; w < kFineWords; ++w) {
            const int c = 32 * w + lane;
            const unsigned bal = __ballot_sync(
                0xffffffffu, S.within(kFine * x + c % kFine, kFine * y + (c / kFine) % kFine,
                                      kFine * z + c / (kFine * kFine)));
            if (lane == w) mine = bal;
            any |= bal;
        }
        if (any == 0u) continue;
        if (fcnt) {
            ++cnt;
        } else {
            if (at < end) {
                if (lane == 0) {
                    const uint32_t bin = (morton_expand10((uint32_t)x) << 2) |
                                         (morton_expand10((uint32_t)y) << 1) |
                                         morton_expand10((uint32_t)z);
                    keys[at] = ((unsigned long long)bin << 32) | (uint32_t)f;
                    vals[at] = at;
                }
                if (lane < kFineWords) masks[(int64_t)lane * ntot + at] = mine;
            }
            ++at;
        }
    }
    if (fcnt && lane == 0) {
        fcnt[f] = cnt;
        if (cnt) atomicAdd(total, (unsigned long long)cnt);
    }
}

// Sorted (bin << 32 | leaf) keys with the indices of their unsorted entries
// -> the entries (kFineWords mask-word arrays of n, then the leaves), and the
// entry count of each bin (zeroed before).
__global__ void k_bin_split(const unsigned long long* __restrict__ keys,
                            const uint32_t* __restrict__ src, const uint32_t* __restrict__ masks,
                            int64_t n, uint32_t* __restrict__ ent, uint32_t* __restrict__ cnt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = keys[i];
    const int64_t from = src[i];
#pragma unroll
    for (int w = 0; w < kFineWords; ++w) ent[w * n + i] = masks[w * n + from];
    ent[kFineWords * n + i] = (uint32_t)k;
    atomicAdd(cnt + (uint32_t)(k >> 32), 1u);
}

// 1 for a bin with entries, else 0 (boff: nb + 1 exclusive sums).
__global__ void k_bin_flags(const uint32_t* __restrict__ boff, int64_t nb,
                            int32_t* __restrict__ flag) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m < nb) flag[m] = boff[m + 1] > boff[m] ? 1 : 0;
}

// Exclusive sums of the flags -> the dense id of each bin with entries, -1
// for the others; *nocc: how many have entries.
__global__ void k_bin_ids(const uint32_t* __restrict__ boff, int64_t nb, int32_t* __restrict__ bid,
                          int32_t* __restrict__ nocc) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nb) return;
    const bool has = boff[m + 1] > boff[m];
    const int32_t v = bid[m];
    if (m == nb - 1) *nocc = v + (has ? 1 : 0);
    bid[m] = has ? v : -1;
}

// Sorted pairs -> the cell of each entry and the leaf list.
__global__ void k_grid_split(const unsigned long long* __restrict__ pairs, int64_t n,
                             uint32_t* __restrict__ cells, int32_t* __restrict__ list) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long v = pairs[i];
    cells[i] = (uint32_t)(v >> 32);
    list[i] = (int32_t)(v & 0xffffffffu);
}

// Inserts the distinct cells into the hash table (bounded linear probing).
__global__ void k_grid_insert(const uint32_t* __restrict__ uniq, const uint32_t* __restrict__ cnt,
                              const uint32_t* __restrict__ start, const int* __restrict__ nuniq,
                              uint4* __restrict__ slots, uint32_t shift, uint32_t mask,
                              int* __restrict__ failed) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nuniq) return;
    const uint32_t c = uniq[i];
    uint32_t slot = (c * 0x9E3779B1u) >> shift;
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const uint32_t prev = atomicCAS(&slots[slot].x, 0xffffffffu, c);
        if (prev == 0xffffffffu || prev == c) {
            slots[slot].y = start[i];
            slots[slot].z = cnt[i];
            slots[slot].w = 0u;
            return;
        }
        slot = (slot + 1) & mask;
    }
    atomicExch(failed, 1);
}

// Point order for the traversal: a counting sort of the query points into the
// 2^(3b) Morton cells of the surface box (b bits a side).  The order only
// changes how much work the traversal does, never its results, so the bin
// is computed in binary32 (integer-rounded inputs) and the order of points
// within a bin is whatever the atomic increments give.
__global__ void k_point_bins(const double* __restrict__ P, int64_t n, float lx, float ly,
                             float lz, float sx, float sy, float sz, float side,
                             uint2* __restrict__ bin_rank, uint32_t* __restrict__ count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c[3] = {(d2f_rn(__ldcs(P + 3 * i)) - lx) * sx,
                        (d2f_rn(__ldcs(P + 3 * i + 1)) - ly) * sy,
                        (d2f_rn(__ldcs(P + 3 * i + 2)) - lz) * sz};
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float v = fminf(fmaxf(c[k] * side, 0.0f), side - 1.0f);   // NaN -> 0
        q[k] = (uint32_t)v;
    }
    const uint32_t bin =
        (morton_expand10(q[0]) << 2) | (morton_expand10(q[1]) << 1) | morton_expand10(q[2]);
    bin_rank[i] = make_uint2(bin, atomicAdd(count + bin, 1u));
}

// The same sort on the bin index's own bins (Morton order of the bin
// coordinates shifted right by sh): consecutive queries then share a bin and
// its entries.  The bin coordinates are computed as in bins_point_in.
__global__ void k_point_bins_idx(const double* __restrict__ P, int64_t n, float lx, float ly,
                                 float lz, float inv, int32_t n0, int32_t n1, int32_t n2, int sh,
                                 uint2* __restrict__ bin_rank, uint32_t* __restrict__ count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c[3] = {__fmul_rn(__fsub_rn(d2f_rn(__ldcs(P + 3 * i)), lx), inv),
                        __fmul_rn(__fsub_rn(d2f_rn(__ldcs(P + 3 * i + 1)), ly), inv),
                        __fmul_rn(__fsub_rn(d2f_rn(__ldcs(P + 3 * i + 2)), lz), inv)};
    const int32_t nb[3] = {n0, n1, n2};
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int v = !(c[k] > 0.0f) ? 0 : (c[k] >= (float)nb[k] ? nb[k] - 1 : min((int)c[k], nb[k] - 1));
        q[k] = (uint32_t)v >> sh;
    }
    const uint32_t bin =
        (morton_expand10(q[0]) << 2) | (morton_expand10(q[1]) << 1) | morton_expand10(q[2]);
    bin_rank[i] = make_uint2(bin, atomicAdd(count + bin, 1u));
}

// The same on the dense ids of the bins with entries (bid): a point whose bin
// has no entry has no leaf within its culling radius, so it is out, decided
// here (marked 0xffffffff for the placing pass, counted as a query).
__global__ void k_point_bins_cid(const double* __restrict__ P, int64_t n, float lx, float ly,
                                 float lz, float inv, int32_t n0, int32_t n1, int32_t n2,
                                 const int32_t* __restrict__ bid, uint2* __restrict__ bin_rank,
                                 uint32_t* __restrict__ count, uint8_t* __restrict__ out,
                                 unsigned long long* __restrict__ counters) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c[3] = {__fmul_rn(__fsub_rn(d2f_rn(__ldcs(P + 3 * i)), lx), inv),
                        __fmul_rn(__fsub_rn(d2f_rn(__ldcs(P + 3 * i + 1)), ly), inv),
                        __fmul_rn(__fsub_rn(d2f_rn(__ldcs(P + 3 * i + 2)), lz), inv)};
    const int32_t nb[3] = {n0, n1, n2};
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int v = !(c[k] > 0.0f) ? 0 : (c[k] >= (float)nb[k] ? nb[k] - 1 : min((int)c[k], nb[k] - 1));
        q[k] = (uint32_t)v;
    }
    const uint32_t m =
        (morton_expand10(q[0]) << 2) | (morton_expand10(q[1]) << 1) | morton_expand10(q[2]);
    const int32_t id = __ldg(bid + m);
    const bool empty = id < 0;
    if (empty) {
        out[i] = 1;
        bin_rank[i] = make_uint2(0xffffffffu, 0u);
    } else {
        bin_rank[i] = make_uint2((uint32_t)id, atomicAdd(count + id, 1u));
    }
    const unsigned act = __activemask();
    const unsigned dec = __ballot_sync(act, empty);
    if (dec && (threadIdx.x & 31) == (unsigned)(__ffs(act) - 1))
        atomicAdd(counters + kCntEnvQueries, (unsigned long long)__popc(dec));
}

// idx[first of bin + rank] = i, with count holding each bin's first position
__global__ void k_point_place(const uint2* __restrict__ bin_rank, int64_t n,
                              const uint32_t* __restrict__ first, int32_t* __restrict__ idx) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint2 br = __ldcs(bin_rank + i);
    if (br.x == 0xffffffffu) return;   // decided by the binning pass
    idx[__ldg(first + br.x) + br.y] = (int32_t)i;
}

// bits a side of the sort grid: the knob (2..8), or the smallest b with
// 2^(3b) >= n, between 3 and 8 (8: cells of 1/256 of the box, about one
// envelope-grid cell on a 100k-facet surface)
static int sort_bits(int64_t n, int knob) {
    if (knob >= 2) return std::min(knob, 8);
    int b = 3;
    while (b < 8 && (int64_t(1) << (3 * b)) < n) ++b;
    return b;
}

struct SortLayout {
    uint2* bin_rank;
    int32_t* idx;
    uint32_t* count;
    int64_t nbins;
    uint32_t* recheck;   // count, then up to n point indices
    void* temp;
    size_t temp_bytes;
};

static size_t cub_scan_bytes(int64_t nbins) {
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, (uint32_t*)nullptr, (int)nbins);
    return b;
}

static SortLayout sort_layout(void* base, int64_t n, int knob) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    char* q = static_cast<char*>(base);
    SortLayout L;
    L.nbins = int64_t(1) << (3 * sort_bits(n, knob));
    L.bin_rank = (uint2*)q; q += al(8 * (size_t)n);
    L.idx = (int32_t*)q; q += al(4 * (size_t)n);
    L.count = (uint32_t*)q; q += al(4 * (size_t)L.nbins);
    L.recheck = (uint32_t*)q; q += al(4 * (size_t)n + 4);
    L.temp = q;
    L.temp_bytes = cub_scan_bytes(L.nbins);
    return L;
}

size_t env_sort_scratch_bytes(int64_t n, int knob) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const int64_t nbins = int64_t(1) << (3 * sort_bits(n, knob));
    return al(8 * (size_t)n) + al(4 * (size_t)n) + al(4 * (size_t)nbins) +
           al(4 * (size_t)n + 4) + al(cub_scan_bytes(nbins)) + 256;
}

// Batches below this size are traversed in input order (sorting would cost
// more than it saves).
constexpr int64_t kSortMin = 4096;

void launch_env_points(const Surface& S, const double* P, int64_t n, double eps2, uint8_t* out,
                       int precision, unsigned long long* counters, void* sort_scratch,
                       int sort_knob, int point_block, cudaStream_t s, cudaEvent_t ev_begin,
                       cudaEvent_t ev_end) {
    if (n <= 0) return;
    const int block = 128;
    const int32_t* order = nullptr;
    uint32_t* recheck = nullptr;
    const uint32_t* n_dev = nullptr;   // sorted queries, when the binning pass decides some
    const EnvTree T = env_tree_for(S, eps2);
    const EpsParams E = eps_params(eps2);
    if (sort_scratch && n >= kSortMin && n <= INT32_MAX) {
        SortLayout L = sort_layout(sort_scratch, n, sort_knob);
        const unsigned nb = (unsigned)((n + 255) / 256);
        const int bits = sort_bits(n, sort_knob);
        if (T.boff && T.bid && sort_knob == 1 && (int64_t)T.nocc + 1 <= L.nbins) {
            // on the dense ids of the bins with entries (a 4-byte count each)
            cudaMemsetAsync(L.count, 0, 4 * ((size_t)T.nocc + 1), s);
            k_point_bins_cid<<<nb, 256, 0, s>>>(P, n, T.blo[0], T.blo[1], T.blo[2], T.binv,
                                                T.bn[0], T.bn[1], T.bn[2], T.bid, L.bin_rank,
                                                L.count, out, counters);
            size_t tb = L.temp_bytes;
            cub::DeviceScan::ExclusiveSum(L.temp, tb, L.count, T.nocc + 1, s);
            n_dev = L.count + T.nocc;
        } else if (T.boff) {
            // on the bin index's own bins (or a coarser Morton prefix of them)
            const int b = std::min(bits, S.grid.bbits);
            cudaMemsetAsync(L.count, 0, 4 * ((size_t)1 << (3 * b)), s);
            k_point_bins_idx<<<nb, 256, 0, s>>>(P, n, T.blo[0], T.blo[1], T.blo[2], T.binv,
                                                T.bn[0], T.bn[1], T.bn[2], S.grid.bbits - b,
                                                L.bin_rank, L.count);
            size_t tb = L.temp_bytes;
            cub::DeviceScan::ExclusiveSum(L.temp, tb, L.count, 1 << (3 * b), s);
        } else {
            double sc[3];
            for (int k = 0; k < 3; ++k) {
                double ext = S.hi[k] - S.lo[k];
                sc[k] = ext > 0.0 ? 1.0 / ext : 0.0;
            }
            cudaMemsetAsync(L.count, 0, 4 * (size_t)L.nbins, s);
            k_point_bins<<<nb, 256, 0, s>>>(P, n, (float)S.lo[0], (float)S.lo[1], (float)S.lo[2],
                                            (float)sc[0], (float)sc[1], (float)sc[2],
                                            std::ldexp(1.0f, bits), L.bin_rank, L.count);
            size_t tb = L.temp_bytes;
            cub::DeviceScan::ExclusiveSum(L.temp, tb, L.count, (int)L.nbins, s);
        }
        k_point_place<<<nb, 256, 0, s>>>(L.bin_rank, n, L.count, L.idx);
        order = L.idx;
        recheck = L.recheck;
    }
    // the tree-walk kernels: at least 6 blocks of 128 threads per SM (85
    // registers), measured best of 1, 6 and 8 on the 10M-point workload (8
    // spills)
    if (ev_begin) cudaEventRecord(ev_begin, s);
    if (T.boff && precision == TW_PRECISION_FP32_CERTIFIED && recheck) {
        // no FP64 code in the bulk kernel (64 registers): 4 blocks of 256 per SM
        // (measured on 10M points: 0.564 ms against 0.592 for 8 of 128, 0.646
        // for 2 of 512, 0.665 for 1 of 1024)
        cudaMemsetAsync(recheck, 0, 4, s);
        k_env_points_bins<256, 4, true, true><<<grid_for(n, 256, 16), 256, 0, s>>>(
            P, order, n, T, E, out, counters, recheck, n_dev);
        k_env_points_bins_recheck<<<grid_for(INT32_MAX, 128, 4), 128, 0, s>>>(P, recheck, T, E,
                                                                             out, counters);
    } else if (T.boff && precision == TW_PRECISION_FP32_CERTIFIED) {
        k_env_points_bins<384, 2, true, false><<<grid_for(n, 384, 6), 384, 0, s>>>(
            P, order, n, T, E, out, counters, nullptr, n_dev);
    } else if (T.boff) {
        k_env_points_bins<384, 2, false, false><<<grid_for(n, 384, 6), 384, 0, s>>>(
            P, order, n, T, E, out, counters, nullptr, n_dev);
    } else if (T.gslot && precision == TW_PRECISION_FP32_CERTIFIED) {
        // 768 resident threads per SM (85 registers) in every block shape
        switch (point_block) {
        case 256:
            k_env_points_grid<256, 3, true><<<grid_for(n, 256, 8), 256, 0, s>>>(P, order, n, T,
                                                                               E, out, counters);
            break;
        case 128:
            k_env_points_grid<128, 6, true><<<grid_for(n, 128, 16), 128, 0, s>>>(P, order, n, T,
                                                                                E, out, counters);
            break;
        case 768:
            k_env_points_grid<768, 1, true><<<grid_for(n, 768, 3), 768, 0, s>>>(P, order, n, T,
                                                                               E, out, counters);
            break;
        default:   // 384: measured best of the four on 10M points (1.11 vs 1.15 ms at 128)
            k_env_points_grid<384, 2, true><<<grid_for(n, 384, 6), 384, 0, s>>>(P, order, n, T,
                                                                               E, out, counters);
        }
    } else if (T.gslot) {
        // FP64 through the same sort and grid
        k_env_points_grid<384, 2, false><<<grid_for(n, 384, 6), 384, 0, s>>>(P, order, n, T, E,
                                                                            out, counters);
    }
    else if (precision == TW_PRECISION_FP32_CERTIFIED && order)
        k_env_points_warp<6><<<grid_for(n, block, 16), block, 0, s>>>(P, order, n, T, E, out,
                                                                      counters);
    else if (precision == TW_PRECISION_FP32_CERTIFIED)
        k_env_points<true, 6><<<grid_for(n, block, 16), block, 0, s>>>(P, order, n, T, E, out,
                                                                       counters);
    else
        k_env_points<false><<<grid_for(n, block, 16), block, 0, s>>>(P, order, n, T, E, out,
                                                                     counters);
    if (ev_end) cudaEventRecord(ev_end, s);
}

// ---------------------------------------------------------------------------
// sampleTriangle arithmetic (geogram vec3 semantics, as in the oracle).
// ---------------------------------------------------------------------------
__device__ __forceinline__ V3 vsub(const V3& a, const V3& b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 vadd(const V3& a, const V3& b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 vmul(const V3& a, double s) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 smul(double s, const V3& a) { return V3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 vdiv(const V3& a, double s) { return V3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ double vlen2(const V3& a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }
__device__ __forceinline__ double vlen(const V3& a) { return sqrt(vlen2(a)); }
__device__ __forceinline__ double vdist(const V3& a, const V3& b) { return vlen(vsub(a, b)); }
__device__ __forceinline__ V3 vnormalize(const V3& a) {
    double s = vlen(a);
    if (s > 1e-30) s = 1.0 / s;
    return smul(s, a);
}
__device__ __forceinline__ int trunc_int(double x) {
    if (!(x == x)) return 0;
    if (x >= 2147483647.0) return 2147483647;
    if (x <= -2147483648.0) return -2147483647 - 1;
    return (int)x;
}

// The per-face constants of sampleTriangle.
struct SampleHeader {
    V3 vs[3];
    V3 v0, v1, v2, n01, n02, n12;
    double ls[3];
    int max_i;
    double N;           // base-row bound after the N == int(N) adjustment
    int trivial;        // N <= 1: the three vertices only
    int M;              // number of candidate rows (M < 1: base row, v1, v2 only)
    double sin_v0, tan_v0, sin_v1;
    double NE, NF;      // edge bounds after the N == int(N) adjustment
    int hasE, hasF;     // the reference samples an edge only when its raw N > 1
    V3 nE, nF;          // edge directions v1->v2, v2->v0
};

__device__ __forceinline__ void sample_header(const double* t, double sd, SampleHeader& h) {
    const double sqrt3_2 = sqrt(3.0) / 2.0;
    h.vs[0] = V3{t[0], t[1], t[2]};
    h.vs[1] = V3{t[3], t[4], t[5]};
    h.vs[2] = V3{t[6], t[7], t[8]};
    for (int i = 0; i < 3; ++i) h.ls[i] = vlen2(vsub(h.vs[i], h.vs[(i + 1) % 3]));
    int max_i = 0;
    for (int i = 1; i < 3; ++i)
        if (!(h.ls[i] < h.ls[max_i])) max_i = i;
    h.max_i = max_i;
    double N = sqrt(h.ls[max_i]) / sd;
    h.trivial = (N <= 1) ? 1 : 0;
    h.M = 0;
    if (h.trivial) return;
    if (N == (double)trunc_int(N)) N -= 1;
    h.N = N;
    h.v0 = h.vs[max_i];
    h.v1 = h.vs[(max_i + 1) % 3];
    h.v2 = h.vs[(max_i + 2) % 3];
    h.n01 = vnormalize(vsub(h.v1, h.v0));
    double hh = vdist(vadd(vdiv(smul(dot3(vsub(h.v2, h.v0), vsub(h.v1, h.v0)), vsub(h.v1, h.v0)),
                               h.ls[max_i]),
                          h.v0),
                     h.v2);
    h.M = trunc_int(hh / (sqrt3_2 * sd));
    if (h.M < 1) return;
    h.n02 = vnormalize(vsub(h.v2, h.v0));
    h.n12 = vnormalize(vsub(h.v2, h.v1));
    double cr0 = vlen(cross3(vsub(h.v2, h.v0), vsub(h.v1, h.v0)));
    double cr1 = vlen(cross3(vsub(h.v2, h.v1), vsub(h.v0, h.v1)));
    h.sin_v0 = cr0 / (vdist(h.v0, h.v2) * vdist(h.v0, h.v1));
    h.tan_v0 = cr0 / dot3(vsub(h.v2, h.v0), vsub(h.v1, h.v0));
    h.sin_v1 = cr1 / (vdist(h.v1, h.v2) * vdist(h.v0, h.v1));
    double NE = sqrt(h.ls[(max_i + 1) % 3]) / sd;
    h.hasE = NE > 1;
    if (h.hasE && NE == (double)trunc_int(NE)) NE -= 1;
    h.NE = NE;
    h.nE = vnormalize(vsub(h.v2, h.v1));
    double NF = sqrt(h.ls[(max_i + 2) % 3]) / sd;
    h.hasF = NF > 1;
    if (h.hasF && NF == (double)trunc_int(NF)) NF -= 1;
    h.NF = NF;
    h.nF = vnormalize(vsub(h.v0, h.v2));
}

// Row m (1 <= m <= M): start point v and last index N1; returns false when
// the row triggers the reference's break (distance(v0_m, v1_m) <= sd).
__device__ __forceinline__ bool sample_row(const SampleHeader& h, double sd, int m, V3& v, int& N1) {
    const double sqrt3_2 = sqrt(3.0) / 2.0;
    int n = trunc_int(sqrt3_2 / h.tan_v0 * m + 0.5);
    int n1 = trunc_int(sqrt3_2 / h.tan_v0 * m);
    if (m % 2 == 0 && n == n1) n += 1;
    V3 v0_m = vadd(h.v0, smul((double)m * sqrt3_2 * sd / h.sin_v0, h.n02));
    V3 v1_m = vadd(h.v1, smul((double)m * sqrt3_2 * sd / h.sin_v1, h.n12));
    if (vdist(v0_m, v1_m) <= sd) return false;
    double delta_d = (((double)n + (m % 2) / 2.0) - (double)m * sqrt3_2 / h.tan_v0) * sd;
    v = vadd(v0_m, smul(delta_d, h.n01));
    N1 = trunc_int(vdist(v, v1_m) / sd);
    return true;
}
__device__ __forceinline__ V3 row_point(const SampleHeader& h, const V3& v, double sd, int i) {
    return vadd(v, vmul(smul((double)i, h.n01), sd));
}
__device__ __forceinline__ V3 base_point(const SampleHeader& h, double sd, int n) {
    return vadd(h.v0, vmul(vmul(h.n01, sd), (double)n));
}
__device__ __forceinline__ V3 edge_point(const V3& o, const V3& dir, double sd, int n) {
    return vadd(o, vmul(vmul(dir, sd), (double)n));
}
// number of integers n with lo <= n <= N (N a double), lo >= 0
__device__ __forceinline__ int count_upto(double N, int lo) {
    if (!(N >= (double)lo)) return 0;
    double f = floor(N);
    if (f > 2147483000.0) f = 2147483000.0;
    return (int)f - lo + 1;
}

// Exact collinearity (Triangle_3f::is_degenerate): the three 2x2 minors of
// [a - c, b - c] vanish.
__device__ __forceinline__ bool minor2_zero(double px, double py, double qx, double qy, double rx,
                                            double ry) {
    double a[2], b[2], c[2], d[2], m[16];
    int na = exp_diff(px, rx, a), nb = exp_diff(qy, ry, b);
    int nc = exp_diff(py, ry, c), nd = exp_diff(qx, rx, d);
    int k = exp_minor(a, na, b, nb, c, nc, d, nd, m);
    return m[k - 1] == 0.0;
}
__device__ __noinline__ bool tri_collinear(const double* t) {
    if (!minor2_zero(t[0], t[1], t[3], t[4], t[6], t[7])) return false;
    if (!minor2_zero(t[0], t[2], t[3], t[5], t[6], t[8])) return false;
    return minor2_zero(t[1], t[2], t[4], t[5], t[7], t[8]);
}

struct FaceCtx {
    EnvTree T;
    EpsParams E;
    unsigned long long* counters;
};

// Largest per-face sample grid the kernel accepts (about 4e6 samples per edge
// row); a larger face would keep one warp busy for seconds, so it is flagged
// as an error instead.
constexpr double kMaxSamplesPerRow = 4.0e6;

__device__ __forceinline__ bool header_too_large(const SampleHeader& h) {
    if (h.trivial) return false;
    if (!(h.N <= kMaxSamplesPerRow)) return true;
    if (h.M > (int)kMaxSamplesPerRow) return true;
    if (h.M >= 1 && h.hasE && !(h.NE <= kMaxSamplesPerRow)) return true;
    if (h.M >= 1 && h.hasF && !(h.NF <= kMaxSamplesPerRow)) return true;
    return false;
}

// Per-lane sample test with the facet hint.
template <bool FP32>
__device__ __forceinline__ bool sample_out(const FaceCtx& F, const V3& p, int32_t& hint,
                                           TravStats& st) {
    if (hint >= 0) {
        ++st.facets;
        if (FP32) {
            int cls = facet_classify(F.T.cull, hint, cert_query(p, F.E, F.T.scale_hi));
            if (cls == kFacetIn) return false;
            if (cls == kFacetBand) {
                ++st.fp64;
                if (leaf_sqdist(F.T.tri, hint, p) <= F.E.eps2) return false;
            }
        } else {
            ++st.fp64;
            if (leaf_sqdist(F.T.tri, hint, p) <= F.E.eps2) return false;
        }
    }
    int32_t f = query_point<FP32>(F.T, p, F.E, st);
    if (f == kTraversalError) {
        atomicOr(F.counters + kCntError, 1ULL);
        return false;
    }
    if (f < 0) return true;
    hint = f;
    return false;
}

// Binary32 box of the face's vertices grown by the largest culling radius of
// any sample (CertQuery::thr with M = the surface's and the face's largest
// coordinate) plus 2^-20 M for the rounding of the sample construction, all
// rounded outward: every sample's binary32 point and everything within its
// culling radius lie inside.
__device__ __forceinline__ void face_query_box(const double* t, const FaceCtx& F, float* qlo,
                                               float* qhi) {
    double m = 0.0;
    for (int k = 0; k < 9; ++k) m = fmax(m, fabs(t[k]));
    const CertQuery q = cert_query(V3{m, m, m}, F.E, F.T.scale_hi);
    const float mu = fmaxf(q.ph[0], F.T.scale_hi);
    const float R = __fadd_ru(__fsqrt_ru(q.thr), __fmul_ru(9.5367431640625e-07f, mu));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double lo = fmin(t[k], fmin(t[3 + k], t[6 + k]));
        const double hi = fmax(t[k], fmax(t[3 + k], t[6 + k]));
        float flo = d2f_rn(lo), fhi = d2f_rn(hi);
        if (f2d_exact(flo) > lo) flo = nextafterf(flo, -__int_as_float(0x7f800000));
        if (f2d_exact(fhi) < hi) fhi = nextafterf(fhi, __int_as_float(0x7f800000));
        qlo[k] = __fsub_rd(flo, R);
        qhi[k] = __fadd_ru(fhi, R);
    }
}

// The samples of one face with its header already computed, the whole warp:
// 1 if some sample is out, 0 otherwise.
template <bool FP32>
__device__ __forceinline__ uint8_t env_face_samples(const SampleHeader& h, const FaceCtx& F,
                                                    double sd, TravStats& st, uint32_t& nq) {
    const int lane = threadIdx.x & 31;
    {
        int32_t hint = -1;
        bool out_found = false;
        // certified mode: the leaves within reach of the face, shared by the
        // warp (see k_env_points_warp); -1 when above 32 (per-sample walks)
        int32_t cand = -1;
        int cnt = -1, kh = 0;
        if (FP32 && !F.T.gslot) {
            float qlo[3], qhi[3];
            const double t[9] = {h.vs[0].x, h.vs[0].y, h.vs[0].z, h.vs[1].x, h.vs[1].y,
                                 h.vs[1].z, h.vs[2].x, h.vs[2].y, h.vs[2].z};
            face_query_box(t, F, qlo, qhi);
            cnt = warp_candidates32(F.T, qlo, qhi, lane, cand);
            if (cnt == kTraversalError) {
                if (lane == 0) atomicOr(F.counters + kCntError, 1ULL);
                cnt = -1;
            }

        }
        // out iff the lane's sample (have) is out; called by the whole warp
        auto lane_out = [&](bool have, const V3& p) -> bool {
            if (F.T.gslot) {
                CertQuery q;
                if (have) q = cert_query(p, F.E, F.T.scale_hi);
                return have && !grid_point_in<FP32>(F.T, F.E, have, p, q, st);
            }
            if (cnt < 0) {
                bool o = false;
                if (have) o = sample_out<FP32>(F, p, hint, st);
                return o;
            }
            bool in = !have;
            CertQuery q;
            if (have) q = cert_query(p, F.E, F.T.scale_hi);
            for (int k = 0; k < cnt; ++k) {
                const int kk = (k + kh) % cnt;
                const int32_t lf = __shfl_sync(0xffffffffu, cand, kk);
                if (!in && cert_leaf_within(F.T.cull, F.T.tri, lf, p, q, F.E.eps2, st)) {
                    in = true;
                    kh = kk;
                }
                if (__all_sync(0xffffffffu, in)) break;
            }
            return !in;
        };
        if (h.trivial) {
            const bool have = lane < 3;
            out_found = lane_out(have, have ? h.vs[lane] : h.vs[0]);
            if (have) ++nq;
            out_found = __any_sync(0xffffffffu, out_found);
            return out_found ? 1 : 0;
        }
        // The samples as flat index ranges that the 32 lanes walk in step (the
        // order of the tests changes only the work: the face is out iff some
        // sample is).  First the base row, v1, v2 and the two other edges...
        const int NA = count_upto(h.N, 0);
        const int NE = (h.M >= 1 && h.hasE) ? count_upto(h.NE, 1) : 0;
        const int NF = (h.M >= 1 && h.hasF) ? count_upto(h.NF, 1) : 0;
        const int NX = NA + 2 + NE + NF;
        for (int s0 = 0; s0 < NX; s0 += 32) {
            const int s = s0 + lane;
            const bool have = s < NX;
            V3 p{0.0, 0.0, 0.0};
            if (have) {
                if (s < NA) p = base_point(h, sd, s);
                else if (s == NA) p = h.v1;
                else if (s == NA + 1) p = h.v2;
                else if (s < NA + 2 + NE) p = edge_point(h.v1, h.nE, sd, s - NA - 1);
                else p = edge_point(h.v2, h.nF, sd, s - NA - 1 - NE);
            }
            const bool o = lane_out(have, p);
            if (have) ++nq;
            if (__any_sync(0xffffffffu, o)) return 1;
        }
        // ...then the rows 1..M, 32 at a time: each lane sets up one row
        // (start point and last index), the reference's break (the first row
        // with distance(v0_m, v1_m) <= sd) ends the rows, and the lanes walk
        // the chunk's samples by flat index.
        for (int base = 1; base <= h.M; base += 32) {
            const int m = base + lane;
            V3 v{0.0, 0.0, 0.0};
            int N1 = -1;
            const bool valid = m <= h.M;
            const bool brk = valid && !sample_row(h, sd, m, v, N1);
            const unsigned bal = __ballot_sync(0xffffffffu, brk);
            const int first_brk = bal ? __ffs(bal) - 1 : 32;
            int cnt = 0;
            if (valid && lane < first_brk) {
                if (N1 > (int)kMaxSamplesPerRow) {
                    atomicOr(F.counters + kCntError, 2ULL);
                } else {
                    cnt = N1 + 1;
                }
            }
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int excl = incl - cnt;
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            for (int s0 = 0; s0 < total; s0 += 32) {
                const int s = s0 + lane;
                const bool have = s < total;
                // the row holding flat index s: the last lane whose first index is
                // <= s (first indices never decrease; empty rows share the next one's)
                int r = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int c = r + step;
                    const int ex = __shfl_sync(0xffffffffu, excl, c & 31);
                    if (c < 32 && ex <= s) r = c;
                }
                const double vx = __shfl_sync(0xffffffffu, v.x, r);
                const double vy = __shfl_sync(0xffffffffu, v.y, r);
                const double vz = __shfl_sync(0xffffffffu, v.z, r);
                const int ex = __shfl_sync(0xffffffffu, excl, r);
                V3 p{0.0, 0.0, 0.0};
                if (have) p = row_point(h, V3{vx, vy, vz}, sd, s - ex);
                const bool o = lane_out(have, p);
                if (have) ++nq;
                if (__any_sync(0xffffffffu, o)) return 1;
            }
            if (bal) break;
        }
        return out_found ? 1 : 0;
    }
}

// Header stage of one face (one thread): 0 = degenerate (not out), 1 = beyond
// the per-row sample bound (error bit 2, counted out), 2 = sample it.
__device__ __forceinline__ int face_prepare(const double* __restrict__ tri, double sd,
                                            SampleHeader& h, unsigned long long* counters) {
    double t[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) t[k] = __ldg(tri + k);
    if (tri_collinear(t)) return 0;
    sample_header(t, sd, h);
    if (header_too_large(h)) {
        atomicOr(counters + kCntError, 2ULL);
        return 1;
    }
    return 2;
}

// One face, the whole warp (every lane computes the header).
template <bool FP32>
__device__ __forceinline__ uint8_t env_face_warp(const double* __restrict__ tri,
                                                 const FaceCtx& F, double sd, TravStats& st,
                                                 uint32_t& nq) {
    SampleHeader h;
    double t[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) t[k] = __ldg(tri + k);
    if (tri_collinear(t)) return 0;
    sample_header(t, sd, h);
    if (header_too_large(h)) {
        if ((threadIdx.x & 31) == 0) atomicOr(F.counters + kCntError, 2ULL);
        return 1;
    }
    return env_face_samples<FP32>(h, F, sd, st, nq);
}

// Faces in blocks of kFaceBlock: first every thread prepares one face's header
// into shared memory (the FP64 header and the exact degeneracy test run once
// per face instead of once per lane), then each warp samples its share of the
// block's faces.  Ctx(f, F, sd) gives face f's tree, eps and sampling distance.
constexpr int kFaceBlock = 128;

struct FaceSlot {
    SampleHeader h;
    int32_t state;  // face_prepare's result, or -1 past the end
    int32_t seg;
};

template <bool FP32, class Ctx>
__device__ __forceinline__ void faces_blocked(const double* __restrict__ tris, int64_t n,
                                              unsigned long long* counters, Ctx ctx,
                                              uint8_t* __restrict__ out) {
    __shared__ FaceSlot slot[kFaceBlock];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    TravStats st;
    uint32_t nq = 0;
    for (int64_t base = (int64_t)blockIdx.x * kFaceBlock; base < n;
         base += (int64_t)gridDim.x * kFaceBlock) {
        for (int k = threadIdx.x; k < kFaceBlock; k += blockDim.x) {
            const int64_t f = base + k;
            FaceSlot& fs = slot[k];
            if (f >= n) {
                fs.state = -1;
                continue;
            }
            FaceCtx F;
            double sd;
            fs.seg = ctx(f, F, sd);
            fs.state = face_prepare(tris + 9 * f, sd, fs.h, counters);
        }
        __syncthreads();
        for (int k = warp; k < kFaceBlock; k += nwarps) {
            const int64_t f = base + k;
            const FaceSlot& fs = slot[k];
            if (fs.state < 0) break;
            uint8_t o = (uint8_t)fs.state;
            if (fs.state == 2) {
                FaceCtx F;
                double sd;
                ctx(f, F, sd);
                o = env_face_samples<FP32>(fs.h, F, sd, st, nq);
            }
            if (lane == 0) out[f] = o;
        }
        __syncthreads();
    }
    flush_stats(st, counters, nq);
}

template <bool FP32>
__device__ __forceinline__ void k_env_faces_body(const double* __restrict__ tris, int64_t n,
                                                 const FaceCtx& F, double sd,
                                                 uint8_t* __restrict__ out) {
    faces_blocked<FP32>(tris, n, F.counters,
                        [&](int64_t, FaceCtx& Fo, double& sdo) {
                            Fo = F;
                            sdo = sd;
                            return 0;
                        },
                        out);
}

template <bool FP32>
__global__ void __launch_bounds__(128, 4) k_env_faces(const double* __restrict__ tris, int64_t n,
                                                   FaceCtx F, double sd, uint8_t* __restrict__ out) {
    k_env_faces_body<FP32>(tris, n, F, sd, out);
}

void launch_env_faces(const Surface& S, const double* tris, int64_t n, double eps2, double sd,
                      uint8_t* out, int precision, unsigned long long* counters, cudaStream_t s) {
    if (n <= 0) return;
    const int block = kFaceBlock;
    int grid = grid_for(n, block, 4);
    FaceCtx F{env_tree_for(S, eps2), eps_params(eps2), counters};
    if (precision == TW_PRECISION_FP32_CERTIFIED) {
        k_env_faces<true><<<grid, block, 0, s>>>(tris, n, F, sd, out);
    } else {
        k_env_faces<false><<<grid, block, 0, s>>>(tris, n, F, sd, out);
    }
}

// Envelope faces whose count is known only on the device (*n_dev, at most
// cap): the grid is sized for cap and the warps beyond *n_dev exit at once.
template <bool FP32>
__global__ void __launch_bounds__(128, 4) k_env_faces_dev(const double* __restrict__ tris,
                                                       const unsigned long long* __restrict__ n_dev,
                                                       int64_t cap, FaceCtx F, double sd,
                                                       uint8_t* __restrict__ out) {
    const int64_t n = (int64_t)min((unsigned long long)cap, *n_dev);
    k_env_faces_body<FP32>(tris, n, F, sd, out);
}

void launch_env_faces_dev(const Surface& S, const double* tris, const unsigned long long* n_dev,
                          int64_t cap, double eps2, double sd, uint8_t* out, int precision,
                          unsigned long long* counters, cudaStream_t s) {
    if (cap <= 0) return;
    const int block = kFaceBlock;
    int grid = grid_for(cap, block, 4);
    FaceCtx F{env_tree_for(S, eps2), eps_params(eps2), counters};
    if (precision == TW_PRECISION_FP32_CERTIFIED)
        k_env_faces_dev<true><<<grid, block, 0, s>>>(tris, n_dev, cap, F, sd, out);
    else
        k_env_faces_dev<false><<<grid, block, 0, s>>>(tris, n_dev, cap, F, sd, out);
}

// ---------------------------------------------------------------------------
// Several jobs in one launch (the serving loop): query i belongs to the last
// segment whose begin is <= i; each segment names its job's tree and eps.
// ---------------------------------------------------------------------------
struct EnvSeg {
    int64_t begin;
    EnvTree T;
    EpsParams E;
    double sd;
};

size_t env_seg_bytes() { return sizeof(EnvSeg); }

void fill_env_seg(void* dst, const Surface& S, int64_t begin, double eps2, double sd) {
    EnvSeg g;
    g.begin = begin;
    g.T = env_tree_for(S, eps2);
    g.E = eps_params(eps2);
    g.sd = sd;
    std::memcpy(dst, &g, sizeof g);
}

__device__ __forceinline__ int find_seg(const EnvSeg* __restrict__ segs, int nsegs, int64_t i) {
    int lo = 0, hi = nsegs - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(&segs[mid].begin) <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <bool FP32>
__global__ void __launch_bounds__(128) k_env_points_segs(const double* __restrict__ P, int64_t n,
                                                         const EnvSeg* __restrict__ segs, int nsegs,
                                                         uint8_t* __restrict__ out,
                                                         unsigned long long* __restrict__ counters) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    TravStats st;
    uint32_t nq = 0;
    const int64_t first = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t base0 = first - (threadIdx.x & 31);
    for (int64_t b = base0; b < n; b += stride) {
        const int64_t i = b + (threadIdx.x & 31);
        if (i < n) {
            const EnvSeg& g = segs[find_seg(segs, nsegs, i)];
            const EnvTree T = g.T;
            const EpsParams E = g.E;
            V3 p{__ldg(P + 3 * i), __ldg(P + 3 * i + 1), __ldg(P + 3 * i + 2)};
            if (T.gslot) {
                const CertQuery q = cert_query(p, E, T.scale_hi);
                out[i] = (uint8_t)!index_point_in<FP32>(T, E, true, p, q, st);
            } else {
                int32_t f = query_point<FP32>(T, p, E, st);
                if (f == kTraversalError) atomicOr(counters + kCntError, 1ULL);
                out[i] = (uint8_t)(f == -1);
            }
            ++nq;
        }
    }
    flush_stats(st, counters, nq);
}

template <bool FP32>
__global__ void __launch_bounds__(128, 4) k_env_faces_segs(const double* __restrict__ tris, int64_t n,
                                                        const EnvSeg* __restrict__ segs, int nsegs,
                                                        uint8_t* __restrict__ out,
                                                        unsigned long long* __restrict__ counters) {
    faces_blocked<FP32>(tris, n, counters,
                        [&](int64_t f, FaceCtx& Fo, double& sdo) {
                            const int k = find_seg(segs, nsegs, f);
                            const EnvSeg& g = segs[k];
                            Fo = FaceCtx{g.T, g.E, counters};
                            sdo = g.sd;
                            return k;
                        },
                        out);
}

void launch_env_points_segs(const double* P, int64_t n, const void* segs, int nsegs, uint8_t* out,
                            int precision, unsigned long long* counters, cudaStream_t s) {
    if (n <= 0 || nsegs <= 0) return;
    const int block = 128;
    const int grid = grid_for(n, block, 6);
    const EnvSeg* g = static_cast<const EnvSeg*>(segs);
    if (precision == TW_PRECISION_FP32_CERTIFIED)
        k_env_points_segs<true><<<grid, block, 0, s>>>(P, n, g, nsegs, out, counters);
    else
        k_env_points_segs<false><<<grid, block, 0, s>>>(P, n, g, nsegs, out, counters);
}

void launch_env_faces_segs(const double* tris, int64_t n, const void* segs, int nsegs, uint8_t* out,
                           int precision, unsigned long long* counters, cudaStream_t s) {
    if (n <= 0 || nsegs <= 0) return;
    const int block = kFaceBlock;
    const int grid = grid_for(n, block, 4);
    const EnvSeg* g = static_cast<const EnvSeg*>(segs);
    if (precision == TW_PRECISION_FP32_CERTIFIED)
        k_env_faces_segs<true><<<grid, block, 0, s>>>(tris, n, g, nsegs, out, counters);
    else
        k_env_faces_segs<false><<<grid, block, 0, s>>>(tris, n, g, nsegs, out, counters);
}

// ---------------------------------------------------------------------------
// Nearest facet (MeshFacetsAABBWithEps::nearest_facet, mesh_AABB.h:130-141,
// mesh_AABB.cpp:381-480): the facet with the smallest computed squared
// distance and its closest point; equal distances go to the smallest input
// facet index.  A child box is skipped only when its squared distance exceeds
// (b + tau)^2, b = sqrt(best so far), tau = 64 * 2^-53 * max|coord| +
// 16 * 2^-53 * b, so no facet that could tie or beat the best is skipped and
// the result is the exact minimum over all facets, independent of the tree.
// Returns the input facet index, or kTraversalError.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double nearest_threshold(double best, double m) {
    if (!(best < INFINITY)) return INFINITY;
    double b = sqrt(best);
    double tau = 64.0 * kEps * m + 16.0 * kEps * b;
    return (b + tau) * (b + tau);
}

__device__ __forceinline__ void nearest_leaf(const EnvTree& T, int32_t leaf, const V3& p,
                                             double& best, int32_t& best_id, V3& best_q) {
    const double* t = T.tri + 9 * (int64_t)leaf;
    V3 a{__ldg(t + 0), __ldg(t + 1), __ldg(t + 2)};
    V3 b{__ldg(t + 3), __ldg(t + 4), __ldg(t + 5)};
    V3 c{__ldg(t + 6), __ldg(t + 7), __ldg(t + 8)};
    V3 q;
    double d = point_tri_nearest(p, a, b, c, q);
    int32_t id = __ldg(T.facet_id + leaf);
    if (d < best || (d == best && id < best_id)) {
        best = d;
        best_id = id;
        best_q = q;
    }
}

__device__ int32_t nearest_facet(const EnvTree& T, const V3& p, V3& q, double& sqd) {
    double m = T.scale;
    m = fmax(m, fabs(p.x));
    m = fmax(m, fabs(p.y));
    m = fmax(m, fabs(p.z));
    double best = INFINITY;
    int32_t best_id = 0x7fffffff;
    V3 best_q{0.0, 0.0, 0.0};
    const int32_t nf = T.nf;
    if (nf == 1) {
        nearest_leaf(T, 0, p, best, best_id, best_q);
        q = best_q;
        sqd = best;
        return best_id;
    }
    int32_t stack[kStack];
    double sdist[kStack];
    int sp = 0;
    int32_t cur = 0;
    for (int32_t iter = 0; iter < 2 * nf; ++iter) {
        if ((uint32_t)cur >= (uint32_t)(nf - 1)) return kTraversalError;
        const double2* nd = reinterpret_cast<const double2*>(T.nodes + cur);
        double2 q0 = __ldg(nd + 0), q1 = __ldg(nd + 1), q2 = __ldg(nd + 2);
        double2 q3 = __ldg(nd + 3), q4 = __ldg(nd + 4), q5 = __ldg(nd + 5);
        int2 ch = __ldg(reinterpret_cast<const int2*>(nd + 6));
        double lo0[3] = {q0.x, q0.y, q1.x}, hi0[3] = {q1.y, q2.x, q2.y};
        double lo1[3] = {q3.x, q3.y, q4.x}, hi1[3] = {q4.y, q5.x, q5.y};
        double d0 = point_box_sqdist(p, lo0, hi0);
        double d1 = point_box_sqdist(p, lo1, hi1);
        // nearer child first
        int32_t cn = ch.x, cf = ch.y;
        double dn = d0, df = d1;
        if (d1 < d0) {
            cn = ch.y; cf = ch.x;
            dn = d1; df = d0;
        }
        bool hn = dn <= nearest_threshold(best, m);
        if (hn && cn < 0) {
            if ((uint32_t)(~cn) >= (uint32_t)nf) return kTraversalError;
            nearest_leaf(T, ~cn, p, best, best_id, best_q);
            hn = false;
        }
        bool hf = df <= nearest_threshold(best, m);
        if (hf && cf < 0) {
            if ((uint32_t)(~cf) >= (uint32_t)nf) return kTraversalError;
            nearest_leaf(T, ~cf, p, best, best_id, best_q);
            hf = false;
        }
        if (hn && hf) {
            if (sp >= kStack) return kTraversalError;
            stack[sp] = cf;
            sdist[sp] = df;
            ++sp;
            cur = cn;
        } else if (hn) {
            cur = cn;
        } else if (hf) {
            cur = cf;
        } else {
            // pop the next subtree still within reach of the best distance
            cur = -1;
            while (sp > 0) {
                --sp;
                if (sdist[sp] <= nearest_threshold(best, m)) {
                    cur = stack[sp];
                    break;
                }
            }
            if (cur < 0) {
                q = best_q;
                sqd = best;
                return best_id;
            }
        }
    }
    return kTraversalError;
}

// The nearest facet through the envelope grid: the minimum over the leaves of
// the point's cell.  When that minimum is <= eps2 it is the minimum over all
// facets (every facet within eps of the point is in the cell's list, see
// EnvGrid), ties included; otherwise it returns false and the tree decides.
__device__ __forceinline__ bool nearest_facet_grid(const EnvTree& T, double eps2, const V3& p,
                                                   V3& q, double& sqd, int32_t& fid) {
    if (!T.gslot) return false;
    CertQuery cq;
    cq.ph[0] = d2f_rn(p.x);
    cq.ph[1] = d2f_rn(p.y);
    cq.ph[2] = d2f_rn(p.z);
    uint32_t b, e;
    grid_cell_range(T, cq, b, e);
    double best = INFINITY;
    int32_t best_id = 0x7fffffff;
    V3 best_q{0.0, 0.0, 0.0};
    for (uint32_t k = b; k < e; ++k) nearest_leaf(T, __ldg(T.glist + k), p, best, best_id, best_q);
    if (!(best <= eps2)) return false;
    q = best_q;
    sqd = best;
    fid = best_id;
    return true;
}

__global__ void k_nearest_points(EnvTree T, double eps2, const double* __restrict__ P, int64_t n,
                                 double* __restrict__ Q, double* __restrict__ D,
                                 int32_t* __restrict__ Fo, unsigned long long* __restrict__ counters) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        V3 p{__ldg(P + 3 * i), __ldg(P + 3 * i + 1), __ldg(P + 3 * i + 2)};
        V3 q;
        double d;
        int32_t f;
        if (!nearest_facet_grid(T, eps2, p, q, d, f)) f = nearest_facet(T, p, q, d);
        if (f == kTraversalError) {
            atomicOr(counters + kCntError, 1ULL);
            q = p;
            d = 0.0;
            f = -1;
        }
        if (Q) {
            Q[3 * i] = q.x;
            Q[3 * i + 1] = q.y;
            Q[3 * i + 2] = q.z;
        }
        if (D) D[i] = d;
        if (Fo) Fo[i] = f;
    }
}

void free_env_grid(tw_ctx* c, EnvGrid& G) {
    if (G.slot) dev_free(c, G.slot, G.slot_bytes);
    if (G.list) dev_free(c, G.list, G.list_bytes);
    if (G.boff) dev_free(c, G.boff, G.boff_bytes);
    if (G.bent) dev_free(c, G.bent, G.bent_bytes);
    if (G.bid) dev_free(c, G.bid, G.bid_bytes);
    G = EnvGrid{};
}

namespace {
// Scratch blocks of a grid build, released on every exit path.
struct BuildScratch {
    tw_ctx* c;
    std::vector<std::pair<void*, size_t>> blocks;
    void* get(size_t bytes, int& st) {
        void* p = nullptr;
        st = dev_alloc(c, bytes, &p);
        if (st == TW_OK) blocks.emplace_back(p, bytes);
        return p;
    }
    ~BuildScratch() {
        for (auto& b : blocks) dev_free(c, b.first, b.second);
    }
};
}  // namespace

// The bin index (EnvGrid::boff, bent) of a surface whose grid was just built:
// bins of side bin_factor x the mean facet extent, but at least 1/250 of the
// grown box's largest side (at most 256 bins a side).  Leaves it absent when
// unsuitable (a leaf over more than 4096 bins, more than 2^27 entries).
static int build_env_bins(tw_ctx* c, Surface& S, const double* blo, const double* bhi,
                          double mean_ext, double M, double Rm, double bin_factor,
                          cudaStream_t s) {
    EnvGrid& g = S.grid;
    g.bin_factor = bin_factor;   // built for it, or found unsuitable
    if (!(bin_factor > 0.0)) return TW_OK;
    const int32_t nf = S.nf;
    double ext = 0.0;
    for (int k = 0; k < 3; ++k) ext = std::max(ext, bhi[k] - blo[k] + 2.0 * Rm);
    double cs = std::max(bin_factor * mean_ext, ext / 250.0);
    if (!(cs > 0.0) || !std::isfinite(cs)) return TW_OK;
    int64_t n[3];
    float lo[3];
    float inv = 0.0f;
    for (int iter = 0; iter < 64; ++iter) {
        inv = (float)(1.0 / cs);
        int64_t nmax = 0;
        for (int k = 0; k < 3; ++k) {
            const double a = blo[k] - Rm;
            float f = (float)a;
            if ((double)f > a) f = std::nextafter(f, -INFINITY);
            lo[k] = f;
            n[k] = (int64_t)std::floor((bhi[k] + Rm - (double)f) * (double)inv) + 2;
            nmax = std::max(nmax, n[k]);
        }
        if (nmax <= 256) break;
        cs *= 1.01;
    }
    if (std::max(n[0], std::max(n[1], n[2])) > 256) return TW_OK;
    int bits = 0;
    while ((int64_t(1) << bits) < std::max(n[0], std::max(n[1], n[2]))) ++bits;
    const int64_t nmorton = int64_t(1) << (3 * bits);
    BuildScratch B{c, {}};
    int st = TW_OK;
    // acc: [0] entry total, [1] too-big flag, [2] bins with entries
    unsigned long long* acc = (unsigned long long*)B.get(32, st);
    if (st != TW_OK) return st;
    cudaMemsetAsync(acc, 0, 32, s);
    uint32_t* fcnt = (uint32_t*)B.get(4 * ((size_t)nf + 1), st);
    if (st != TW_OK) return st;
    uint32_t* foff = (uint32_t*)B.get(4 * ((size_t)nf + 1), st);
    if (st != TW_OK) return st;
    cudaMemsetAsync(fcnt + nf, 0, 4, s);
    const int Bk = 256;
    const int G = (int)(((int64_t)nf * 32 + Bk - 1) / Bk);   // one warp per leaf
    const double slack = std::ldexp(M, -30);
    k_bin_cells<<<G, Bk, 0, s>>>(S.tri, nf, lo[0], lo[1], lo[2], (double)inv, (int32_t)n[0],
                                 (int32_t)n[1], (int32_t)n[2], Rm, slack, acc, fcnt, nullptr,
                                 nullptr, nullptr, nullptr, 0, (int*)(acc + 1));
    unsigned long long hacc[2] = {0, 0};
    cudaMemcpyAsync(hacc, acc, 16, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "bin index build");
    const unsigned long long total = hacc[0];
    if ((hacc[1] & 0xffffffffULL) != 0 || total == 0 || total > (1ULL << 27)) return TW_OK;
    const int64_t nt = (int64_t)total;
    {
        size_t tbs = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tbs, fcnt, foff, nf + 1, s);
        void* tmp = B.get(tbs + 16, st);
        if (st != TW_OK) return st;
        cub::DeviceScan::ExclusiveSum(tmp, tbs, fcnt, foff, nf + 1, s);
    }
    unsigned long long* keys = (unsigned long long*)B.get(8 * (size_t)nt, st);
    if (st != TW_OK) return st;
    unsigned long long* keys2 = (unsigned long long*)B.get(8 * (size_t)nt, st);
    if (st != TW_OK) return st;
    uint32_t* vals = (uint32_t*)B.get(4 * (size_t)nt, st);
    if (st != TW_OK) return st;
    uint32_t* vals2 = (uint32_t*)B.get(4 * (size_t)nt, st);
    if (st != TW_OK) return st;
    uint32_t* masks = (uint32_t*)B.get(4 * (size_t)kFineWords * (size_t)nt, st);
    if (st != TW_OK) return st;
    k_bin_cells<<<G, Bk, 0, s>>>(S.tri, nf, lo[0], lo[1], lo[2], (double)inv, (int32_t)n[0],
                                 (int32_t)n[1], (int32_t)n[2], Rm, slack, nullptr, nullptr, foff,
                                 keys, vals, masks, nt, nullptr);
    const int key_bits = 32 + 3 * bits;
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, keys2, vals, vals2, (int)nt, 0, key_bits,
                                    s);
    size_t tb2 = 0, tb3 = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb2, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                  (int)(nmorton + 1), s);
    cub::DeviceScan::ExclusiveSum(nullptr, tb3, (int32_t*)nullptr, (int32_t*)nullptr,
                                  (int)nmorton, s);
    void* temp = B.get(std::max(tb, std::max(tb2, tb3)) + 16, st);
    if (st != TW_OK) return st;
    uint32_t* bcnt = (uint32_t*)B.get(4 * ((size_t)nmorton + 1), st);
    if (st != TW_OK) return st;
    cub::DeviceRadixSort::SortPairs(temp, tb, keys, keys2, vals, vals2, (int)nt, 0, key_bits, s);
    void* offp = nullptr;
    void* entp = nullptr;
    const size_t off_bytes = 4 * ((size_t)nmorton + 1),
                 ent_bytes = 4 * (size_t)(kFineWords + 1) * (size_t)nt;
    if ((st = dev_alloc(c, off_bytes, &offp)) != TW_OK) return st;
    if ((st = dev_alloc(c, ent_bytes, &entp)) != TW_OK) {
        dev_free(c, offp, off_bytes);
        return st;
    }
    cudaMemsetAsync(bcnt, 0, 4 * ((size_t)nmorton + 1), s);
    k_bin_split<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(keys2, vals2, masks, nt,
                                                             (uint32_t*)entp, bcnt);
    cub::DeviceScan::ExclusiveSum(temp, tb2, bcnt, (uint32_t*)offp, (int)(nmorton + 1), s);
    // the dense ids of the bins with entries, for the point sort
    void* bidp = nullptr;
    const size_t bid_bytes = 4 * (size_t)nmorton;
    if ((st = dev_alloc(c, bid_bytes, &bidp)) != TW_OK) {
        dev_free(c, offp, off_bytes);
        dev_free(c, entp, ent_bytes);
        return st;
    }
    const unsigned gm = (unsigned)((nmorton + 255) / 256);
    k_bin_flags<<<gm, 256, 0, s>>>((const uint32_t*)offp, nmorton, (int32_t*)bidp);
    cub::DeviceScan::ExclusiveSum(temp, tb3, (int32_t*)bidp, (int32_t*)bidp, (int)nmorton, s);
    k_bin_ids<<<gm, 256, 0, s>>>((const uint32_t*)offp, nmorton, (int32_t*)bidp,
                                 (int32_t*)(acc + 2));
    int32_t nocc = 0;
    cudaMemcpyAsync(&nocc, acc + 2, 4, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);   // the scratch is released on return
    if (e != cudaSuccess) {
        dev_free(c, offp, off_bytes);
        dev_free(c, entp, ent_bytes);
        dev_free(c, bidp, bid_bytes);
        return cuda_fail(c, e, "bin index build");
    }
    g.bid = (int32_t*)bidp;
    g.nocc = nocc;
    g.bid_bytes = bid_bytes;
    for (int k = 0; k < 3; ++k) {
        g.blo[k] = lo[k];
        g.bn[k] = (int32_t)n[k];
    }
    g.binv = inv;
    g.bbits = bits;
    g.boff = (uint32_t*)offp;
    g.bent = (uint32_t*)entp;
    g.bnt = nt;
    g.boff_bytes = off_bytes;
    g.bent_bytes = ent_bytes;
    return TW_OK;
}

int build_env_grid(tw_ctx* c, Surface& S, double eps2, double cell_factor, cudaStream_t s) {
    if (S.nf <= 0 || !(eps2 >= 0.0)) return TW_OK;
    if (S.grid.slot && S.grid.eps2 == eps2 && S.grid.cell_factor == cell_factor &&
        S.grid.bin_factor == c->bin_cell)
        return TW_OK;
    free_env_grid(c, S.grid);
    const int32_t nf = S.nf;
    // bounding box of the facets: the root's two child boxes, or the facet
    double blo[3], bhi[3];
    if (nf > 1) {
        BvhNode root;
        cudaMemcpyAsync(&root, S.nodes, sizeof root, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(c, e, "grid build");
        for (int k = 0; k < 3; ++k) {
            blo[k] = std::min(root.lo0[k], root.lo1[k]);
            bhi[k] = std::max(root.hi0[k], root.hi1[k]);
        }
    } else {
        double t[9];
        cudaMemcpyAsync(t, S.tri, sizeof t, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(c, e, "grid build");
        for (int k = 0; k < 3; ++k) {
            blo[k] = std::min(t[k], std::min(t[3 + k], t[6 + k]));
            bhi[k] = std::max(t[k], std::max(t[3 + k], t[6 + k]));
        }
    }
    BuildScratch B{c, {}};
    int st = TW_OK;
    // acc: [0] sum of extents (double), [1] entry total, [2] too-big flag,
    // [3] distinct cells, [4] insert failure
    void* acc = B.get(64, st);
    if (st != TW_OK) return st;
    double* d_sum = (double*)acc;
    unsigned long long* d_total = (unsigned long long*)acc + 1;
    int* d_big = (int*)((unsigned long long*)acc + 2);
    int* d_nuniq = (int*)((unsigned long long*)acc + 3);
    int* d_failed = (int*)((unsigned long long*)acc + 4);
    cudaMemsetAsync(acc, 0, 64, s);
    k_grid_mean_extent<<<grid_for(nf, 256, 4), 256, 0, s>>>(S.tri, nf, d_sum);
    double sum_ext = 0.0;
    cudaMemcpyAsync(&sum_ext, d_sum, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "grid build");
    // culling radius of any point of the grown box, plus the cell-index margin
    const double eps = std::sqrt(eps2);
    double M = S.scale;
    for (int k = 0; k < 3; ++k) M = std::max(M, std::max(std::fabs(blo[k]), std::fabs(bhi[k])));
    M = M + 2.0 * eps + 1e-300;
    const double Rm = eps * (1.0 + std::ldexp(1.0, -18)) + std::ldexp(M, -17);
    double cs = std::max(cell_factor * sum_ext / nf, 2.0 * Rm);
    int64_t n[3];
    float lo[3];
    float inv = 0.0f;
    for (int iter = 0; iter < 64; ++iter) {
        inv = (float)(1.0 / cs);
        int64_t cells = 1;
        for (int k = 0; k < 3; ++k) {
            const double a = blo[k] - Rm;
            float f = (float)a;
            if ((double)f > a) f = std::nextafter(f, -INFINITY);
            lo[k] = f;
            n[k] = (int64_t)std::floor((bhi[k] + Rm - (double)f) * (double)inv) + 2;
            cells *= n[k];
        }
        if (cells < (int64_t(1) << 31)) break;
        cs *= 1.25;
    }
    if (n[0] * n[1] * n[2] >= (int64_t(1) << 31)) return TW_OK;   // the tree walk serves
    const int Bk = 256;
    const int G = (int)(((int64_t)nf * 32 + Bk - 1) / Bk);   // one warp per leaf
    const double slack = std::ldexp(M, -30);
    // per-leaf counts (nf + 1 entries, the last 0) and their exclusive sums
    uint32_t* fcnt = (uint32_t*)B.get(4 * ((size_t)nf + 1), st);
    if (st != TW_OK) return st;
    uint32_t* foff = (uint32_t*)B.get(4 * ((size_t)nf + 1), st);
    if (st != TW_OK) return st;
    cudaMemsetAsync(fcnt + nf, 0, 4, s);
    k_grid_cells<<<G, Bk, 0, s>>>(S.tri, nf, lo[0], lo[1], lo[2], (double)inv, (int32_t)n[0],
                                  (int32_t)n[1], (int32_t)n[2], Rm, slack, d_total, fcnt,
                                  nullptr, nullptr, d_big);
    unsigned long long hacc[2] = {0, 0};
    cudaMemcpyAsync(hacc, d_total, 16, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "grid build");
    const unsigned long long total = hacc[0];
    // unsuitable (a leaf over too many cells, or too many entries): the tree walk serves
    if ((hacc[1] & 0xffffffffULL) != 0 || total == 0 || total > (1ULL << 27)) return TW_OK;
    const int64_t nt = (int64_t)total;
    // pairs (cell << 32 | leaf), sorted: cells in order, leaves ascending within a cell
    unsigned long long* pairs = (unsigned long long*)B.get(8 * (size_t)nt, st);
    if (st != TW_OK) return st;
    unsigned long long* pairs2 = (unsigned long long*)B.get(8 * (size_t)nt, st);
    if (st != TW_OK) return st;
    {
        size_t tbs = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tbs, fcnt, foff, nf + 1, s);
        void* tmp = B.get(tbs + 16, st);
        if (st != TW_OK) return st;
        cub::DeviceScan::ExclusiveSum(tmp, tbs, fcnt, foff, nf + 1, s);
    }
    k_grid_cells<<<G, Bk, 0, s>>>(S.tri, nf, lo[0], lo[1], lo[2], (double)inv, (int32_t)n[0],
                                  (int32_t)n[1], (int32_t)n[2], Rm, slack, nullptr, nullptr,
                                  foff, pairs, nullptr);
    int key_bits = 32;
    while (key_bits < 64 && (1ULL << (key_bits - 32)) < (unsigned long long)(n[0] * n[1] * n[2]))
        ++key_bits;
    size_t tb = 0;
    cub::DeviceRadixSort::SortKeys(nullptr, tb, pairs, pairs2, (int)nt, 0, key_bits, s);
    void* temp = B.get(tb + 16, st);
    if (st != TW_OK) return st;
    cub::DeviceRadixSort::SortKeys(temp, tb, pairs, pairs2, (int)nt, 0, key_bits, s);
    // the entry cells (into the unsorted buffer) and the final leaf list
    uint32_t* ecell = (uint32_t*)pairs;
    void* listp = nullptr;
    if ((st = dev_alloc(c, 4 * (size_t)nt + 16, &listp)) != TW_OK) return st;
    int32_t* list = (int32_t*)listp;
    k_grid_split<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(pairs2, nt, ecell, list);
    // distinct cells, their counts and first entries (in the sorted buffer, read by now)
    uint32_t* uniq = (uint32_t*)pairs2;
    uint32_t* cnt = uniq + nt;
    uint32_t* start = (uint32_t*)B.get(4 * (size_t)nt + 16, st);
    size_t tb2 = 0, tb3 = 0;
    void* temp2 = nullptr;
    if (st == TW_OK) {
        cub::DeviceRunLengthEncode::Encode(nullptr, tb2, ecell, uniq, cnt, d_nuniq, (int)nt, s);
        cub::DeviceScan::ExclusiveSum(nullptr, tb3, cnt, start, (int)nt, s);
        temp2 = B.get(std::max(tb2, tb3) + 16, st);
    }
    if (st != TW_OK) {
        dev_free(c, listp, 4 * (size_t)nt + 16);
        return st;
    }
    cub::DeviceRunLengthEncode::Encode(temp2, tb2, ecell, uniq, cnt, d_nuniq, (int)nt, s);
    int nuniq = 0;
    cudaMemcpyAsync(&nuniq, d_nuniq, 4, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess || nuniq <= 0) {
        dev_free(c, listp, 4 * (size_t)nt + 16);
        return e != cudaSuccess ? cuda_fail(c, e, "grid build") : TW_OK;
    }
    cub::DeviceScan::ExclusiveSum(temp2, tb3, cnt, start, nuniq, s);
    // the hash table: a power of two at least twice the distinct cells
    uint32_t bits = 1;
    while ((1ULL << bits) < 2ULL * (unsigned long long)nuniq) ++bits;
    const size_t H = size_t(1) << bits;
    void* hs = nullptr;
    if ((st = dev_alloc(c, 16 * H, &hs)) != TW_OK) {
        dev_free(c, listp, 4 * (size_t)nt + 16);
        return st;
    }
    cudaMemsetAsync(hs, 0xff, 16 * H, s);
    k_grid_insert<<<(unsigned)((nuniq + 255) / 256), 256, 0, s>>>(
        uniq, cnt, start, d_nuniq, (uint4*)hs, 32 - bits, (uint32_t)(H - 1), d_failed);
    int failed = 0;
    cudaMemcpyAsync(&failed, d_failed, 4, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess || failed) {
        dev_free(c, listp, 4 * (size_t)nt + 16);
        dev_free(c, hs, 16 * H);
        return e != cudaSuccess ? cuda_fail(c, e, "grid build") : TW_OK;
    }
    EnvGrid& g = S.grid;
    for (int k = 0; k < 3; ++k) {
        g.lo[k] = lo[k];
        g.n[k] = (int32_t)n[k];
    }
    g.inv_c = inv;
    g.slot = (uint4*)hs;
    g.shift = 32 - bits;
    g.mask = (uint32_t)(H - 1);
    g.list = list;
    g.eps2 = eps2;
    g.cell_factor = cell_factor;
    g.slot_bytes = 16 * H;
    g.list_bytes = 4 * (size_t)nt + 16;
    return build_env_bins(c, S, blo, bhi, sum_ext / nf, M, Rm, c->bin_cell, s);
}

// Point checks of candidate collapses (EdgeCollapser.cpp:286-329): the
// degenerate-edge flag, then v2 against the boundary envelope when v1 is on
// the boundary and v2 is not, and against the envelope when v1 is on the
// surface and v2 is not.  ENVELOP (3) or kCollapsePending.
template <bool FP32>
__global__ void k_collapse_points(EnvTree Tin, EnvTree Tb, EpsParams E,
                                  const double* __restrict__ vx, const double* __restrict__ vy,
                                  const double* __restrict__ vz, const int32_t* __restrict__ v12,
                                  const uint8_t* __restrict__ flags, int32_t n,
                                  uint8_t* __restrict__ status, uint8_t* __restrict__ degenerate,
                                  unsigned long long* __restrict__ counters) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    TravStats st;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int32_t v1 = v12[2 * i], v2 = v12[2 * i + 1];
        const double dx = vx[v1] - vx[v2], dy = vy[v1] - vy[v2], dz = vz[v1] - vz[v2];
        const bool deg = sqrt((dx * dx + dy * dy) + dz * dz) == 0.0;
        degenerate[i] = deg;
        const uint8_t fl = flags[i];
        const V3 p{vx[v2], vy[v2], vz[v2]};
        uint8_t res = kCollapsePending;
        for (int pass = 0; pass < 2 && res == kCollapsePending; ++pass) {
            const bool bnd = pass == 0;
            const uint8_t need = bnd ? TW_CV_V1_BOUNDARY : TW_CV_V1_SURFACE;
            const uint8_t has = bnd ? TW_CV_V2_BOUNDARY : TW_CV_V2_SURFACE;
            if (!(fl & need) || (fl & has) || deg) continue;
            const EnvTree& T = bnd ? Tb : Tin;
            if (T.nf <= 0) {
                atomicOr(counters + kCntError, 4ULL);
                res = 3;
                break;
            }
            int32_t f;
            if (T.gslot) {
                const CertQuery q = cert_query(p, E, T.scale_hi);
                f = grid_point_in<FP32>(T, E, true, p, q, st) ? 0 : -1;
            } else {
                f = query_point<FP32>(T, p, E, st);
            }
            if (f == kTraversalError) atomicOr(counters + kCntError, 1ULL);
            if (f == -1) res = 3;
        }
        status[i] = res;
    }
}

void launch_collapse_points(const Surface& Sin, const Surface& Sb, double eps2, int precision,
                            const double* vx, const double* vy, const double* vz,
                            const int32_t* v12, const uint8_t* flags, int32_t n, uint8_t* status,
                            uint8_t* degenerate, unsigned long long* counters, cudaStream_t s) {
    if (n <= 0) return;
    const int block = 128;
    const EnvTree Ti = env_tree_for(Sin, eps2), Tb = env_tree_for(Sb, eps2);
    const EpsParams E = eps_params(eps2);
    if (precision == TW_PRECISION_FP32_CERTIFIED)
        k_collapse_points<true><<<grid_for(n, block, 8), block, 0, s>>>(
            Ti, Tb, E, vx, vy, vz, v12, flags, n, status, degenerate, counters);
    else
        k_collapse_points<false><<<grid_for(n, block, 8), block, 0, s>>>(
            Ti, Tb, E, vx, vy, vz, v12, flags, n, status, degenerate, counters);
}

void launch_nearest_points(const Surface& S, double eps2, const double* P, int64_t n, double* Q,
                           double* D, int32_t* F, unsigned long long* counters, cudaStream_t s) {
    if (n <= 0 || S.nf <= 0) return;
    const int block = 128;
    k_nearest_points<<<grid_for(n, block, 8), block, 0, s>>>(env_tree_for(S, eps2), eps2, P, n, Q,
                                                             D, F, counters);
}

// Projection step of surface smoothing (VertexSmoother.cpp:353-363): every
// star whose status is kSmoothPendingProject moves its Newton position to the
// closest point of the nearest facet of the input surface (kind 1) or of the
// boundary surface (kind 2).  A boundary star without a boundary surface is
// an argument error (error bit 4) and is left invalid.
__global__ void k_smooth_project(EnvTree Tin, EnvTree Tb, double eps2,
                                 const uint8_t* __restrict__ kinds,
                                 int32_t nstars, uint8_t* __restrict__ status,
                                 double* __restrict__ pnew,
                                 unsigned long long* __restrict__ counters) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nstars; i += stride) {
        if (status[i] != kSmoothPendingProject) continue;
        const bool bnd = kinds[i] == TW_STAR_BOUNDARY;
        const EnvTree& T = bnd ? Tb : Tin;
        if (T.nf <= 0) {
            atomicOr(counters + kCntError, 4ULL);
            status[i] = TW_SMOOTH_INVALID;
            continue;
        }
        V3 p{pnew[3 * i], pnew[3 * i + 1], pnew[3 * i + 2]};
        V3 q;
        double d;
        int32_t f;
        if (!nearest_facet_grid(T, eps2, p, q, d, f) && nearest_facet(T, p, q, d) == kTraversalError) {
            atomicOr(counters + kCntError, 1ULL);
            status[i] = TW_SMOOTH_INVALID;
            continue;
        }
        pnew[3 * i] = q.x;
        pnew[3 * i + 1] = q.y;
        pnew[3 * i + 2] = q.z;
    }
}

void launch_smooth_project(const Surface& Sin, const Surface& Sb, double eps2,
                           const uint8_t* kinds, int32_t nstars, uint8_t* status, double* pnew,
                           unsigned long long* counters, cudaStream_t s) {
    if (nstars <= 0) return;
    const int block = 128;
    k_smooth_project<<<grid_for(nstars, block, 8), block, 0, s>>>(
        env_tree_for(Sin, eps2), env_tree_for(Sb, eps2), eps2, kinds, nstars, status, pnew,
        counters);
}

// One thread generates the full sample list in the reference order with the
// same helpers (for checking the device sampling arithmetic).  *count = -1
// when the face exceeds the per-row sample bound.
__global__ void k_sample_triangle(const double* __restrict__ t, double sd, double* out,
                                  int64_t cap, int64_t* count) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    {
        double tv[9];
        for (int k = 0; k < 9; ++k) tv[k] = t[k];
        SampleHeader h;
        sample_header(tv, sd, h);
        if (header_too_large(h)) {
            *count = -1;
            return;
        }
    }
    int64_t cnt = 0;
    auto emit = [&](const V3& p) {
        if (cnt < cap) {
            out[3 * cnt] = p.x;
            out[3 * cnt + 1] = p.y;
            out[3 * cnt + 2] = p.z;
        }
        ++cnt;
    };
    double tv[9];
    for (int k = 0; k < 9; ++k) tv[k] = t[k];
    SampleHeader h;
    sample_header(tv, sd, h);
    if (h.trivial) {
        for (int i = 0; i < 3; ++i) emit(h.vs[i]);
        *count = cnt;
        return;
    }
    for (int n = 0; n <= h.N; ++n) emit(base_point(h, sd, n));
    emit(h.v1);
    if (h.M < 1) {
        emit(h.v2);
        *count = cnt;
        return;
    }
    for (int m = 1; m <= h.M; ++m) {
        V3 v;
        int N1;
        if (!sample_row(h, sd, m, v, N1)) break;
        if (N1 > (int)kMaxSamplesPerRow) {
            *count = -1;
            return;
        }
        for (int i = 0; i <= N1; ++i) emit(row_point(h, v, sd, i));
    }
    emit(h.v2);
    if (h.hasE)
        for (int n = 1; n <= h.NE; ++n) emit(edge_point(h.v1, h.nE, sd, n));
    if (h.hasF)
        for (int n = 1; n <= h.NF; ++n) emit(edge_point(h.v2, h.nF, sd, n));
    *count = cnt;
}

void launch_sample_triangle(const double* tri, double sd, double* out, int64_t cap,
                            int64_t* count, cudaStream_t s) {
    k_sample_triangle<<<1, 32, 0, s>>>(tri, sd, out, cap, count);
}

}  // namespace tw
