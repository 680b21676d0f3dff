// tw_schedule.cu -- operator candidates generated on the device and a
// conflict-free batch of them (a parallel schedule of the local operators).
//
// The reference applies its splits and collapses one at a time from a
// priority queue (EdgeSplitter.cpp:37-73: edges longer than
// ideal_weight * s^2, longest first; EdgeCollapser.cpp:19-81: both directions
// of the edges shorter than that, shortest first; s the mean adaptive scale
// of the two vertices, :372-385 and :710-725).  Here the candidates of one
// operator are built on the device from the tet list and the resident
// positions, and a batch of them whose tets are pairwise disjoint is chosen:
// a split touches the tets around its edge (its shell), a collapse v1 -> v2
// the tets around v1.  The batch is the greedy one in priority order (a
// candidate is taken when no earlier-taken candidate shares a tet with it),
// found by rounds: every undecided candidate claims its tets with its rank
// (atomicMin), a candidate that holds the claim on all its tets is taken and
// its tets are marked, and the undecided candidates touching a marked tet are
// dropped.  A candidate holding all its claims precedes every undecided
// neighbour, so the rounds take exactly the candidates the sequential greedy
// pass takes.  Applying such a batch at once is not the reference's order
// (each of its operations sees the mesh the previous one left), so it is a
// separate mode with other results than the reference's sequential passes.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>

#include "tw_device.cuh"
#include "tw_internal.h"

namespace tw {
namespace {

__global__ void k_tet_edges_verts(const int4* __restrict__ tets, int64_t nt, int32_t nv,
                                  unsigned long long* __restrict__ ekey, int32_t* __restrict__ etet,
                                  uint32_t* __restrict__ vkey, int32_t* __restrict__ vtet,
                                  int* __restrict__ bad) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const int4 t = tets[i];
    const int32_t v[4] = {t.x, t.y, t.z, t.w};
    bool ok = true;
#pragma unroll
    for (int j = 0; j < 4; ++j) ok = ok && v[j] >= 0 && v[j] < nv;
    if (!ok) {
        atomicExch(bad, 1);
        for (int j = 0; j < 6; ++j) {
            ekey[6 * i + j] = 0xffffffffffffffffULL;
            etet[6 * i + j] = (int32_t)i;
        }
        for (int j = 0; j < 4; ++j) {
            vkey[4 * i + j] = 0xffffffffu;
            vtet[4 * i + j] = (int32_t)i;
        }
        return;
    }
    int k = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = a + 1; b < 4; ++b) {
            const uint32_t lo = (uint32_t)min(v[a], v[b]), hi = (uint32_t)max(v[a], v[b]);
            ekey[6 * i + k] = ((unsigned long long)lo << 32) | hi;
            etet[6 * i + k] = (int32_t)i;
            ++k;
        }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        vkey[4 * i + j] = (uint32_t)v[j];
        vtet[4 * i + j] = (int32_t)i;
    }
}

__global__ void k_vertex_counts(const uint32_t* __restrict__ vkey, int64_t n, int32_t nv,
                                int32_t* __restrict__ cnt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && vkey[i] < (uint32_t)nv) atomicAdd(cnt + vkey[i], 1);
}

// candidate flags: slot 2e (a -> b, the split of e) and 2e+1 (b -> a)
__global__ void k_candidate_flags(const unsigned long long* __restrict__ uniq,
                                  const int* __restrict__ nuniq, int64_t cap,
                                  const double* __restrict__ vx, const double* __restrict__ vy,
                                  const double* __restrict__ vz, const double* __restrict__ scale,
                                  double ideal, int op, int32_t* __restrict__ flag,
                                  unsigned long long* __restrict__ wbits) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= cap) return;
    int32_t f0 = 0, f1 = 0;
    double w = 0.0;
    if (e < *nuniq && uniq[e] != 0xffffffffffffffffULL) {
        const int32_t a = (int32_t)(uniq[e] >> 32), b = (int32_t)(uniq[e] & 0xffffffffu);
        // CGAL::squared_distance on posf (LocalOperations.cpp:779-781)
        const double dx = vx[a] - vx[b], dy = vy[a] - vy[b], dz = vz[a] - vz[b];
        w = (dx * dx + dy * dy) + dz * dz;
        const double s = scale ? (scale[a] + scale[b]) / 2.0 : 1.0;
        const double thr = ideal * s * s;
        if (op == TW_OP_SPLIT) {
            f0 = w > thr;
        } else {
            f0 = w < thr;
            f1 = f0;
        }
    }
    flag[2 * e] = f0;
    flag[2 * e + 1] = f1;
    wbits[e] = (unsigned long long)__double_as_longlong(w);
}

__global__ void k_candidates(const int32_t* __restrict__ flag, const int32_t* __restrict__ pos,
                             int64_t nslots, const unsigned long long* __restrict__ wbits,
                             int32_t* __restrict__ cand, unsigned long long* __restrict__ ckey,
                             int32_t* __restrict__ cidx) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nslots || !flag[k]) return;
    const int32_t c = pos[k];
    cand[c] = (int32_t)k;   // edge k >> 1, direction k & 1
    ckey[c] = wbits[k >> 1];
    cidx[c] = c;
}

__global__ void k_ranks(const int32_t* __restrict__ order, const int* __restrict__ ncand,
                        int32_t* __restrict__ rank, uint8_t* __restrict__ state) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *ncand) return;
    rank[order[i]] = (int32_t)i;
    state[order[i]] = 0;   // undecided
}

struct CandTets {
    const int32_t* cand;
    const unsigned long long* uniq;
    const int32_t* eoff;
    const int32_t* etet;
    const int32_t* voff;
    const int32_t* vtet;
    int op;
    __device__ void range(int32_t c, const int32_t*& t, int32_t& m) const {
        const int32_t k = cand[c], e = k >> 1;
        if (op == TW_OP_SPLIT) {
            t = etet + eoff[e];
            m = eoff[e + 1] - eoff[e];
        } else {
            const uint32_t a = (uint32_t)(uniq[e] >> 32), b = (uint32_t)(uniq[e] & 0xffffffffu);
            const uint32_t v1 = (k & 1) ? b : a;
            t = vtet + voff[v1];
            m = voff[v1 + 1] - voff[v1];
        }
    }
};

__global__ void k_claim(CandTets C, const int* __restrict__ ncand, const uint8_t* __restrict__ state,
                        const int32_t* __restrict__ rank, uint32_t* __restrict__ claim) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= *ncand || state[c] != 0) return;
    const int32_t* t;
    int32_t m;
    C.range((int32_t)c, t, m);
    for (int32_t j = 0; j < m; ++j) atomicMin(claim + t[j], (uint32_t)rank[c]);
}

__global__ void k_select(CandTets C, const int* __restrict__ ncand, uint8_t* __restrict__ state,
                         const int32_t* __restrict__ rank, const uint32_t* __restrict__ claim,
                         uint8_t* __restrict__ taken) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= *ncand || state[c] != 0) return;
    const int32_t* t;
    int32_t m;
    C.range((int32_t)c, t, m);
    bool all = true;
    for (int32_t j = 0; j < m && all; ++j) all = claim[t[j]] == (uint32_t)rank[c];
    if (!all) return;
    state[c] = 1;
    for (int32_t j = 0; j < m; ++j) taken[t[j]] = 1;
}

__global__ void k_block(CandTets C, const int* __restrict__ ncand, uint8_t* __restrict__ state,
                        const uint8_t* __restrict__ taken, int* __restrict__ undecided) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= *ncand || state[c] != 0) return;
    const int32_t* t;
    int32_t m;
    C.range((int32_t)c, t, m);
    bool hit = false;
    for (int32_t j = 0; j < m && !hit; ++j) hit = taken[t[j]] != 0;
    if (hit)
        state[c] = 2;
    else
        atomicAdd(undecided, 1);
}

// the taken candidates in rank order
__global__ void k_taken_flags(const int32_t* __restrict__ order, const int* __restrict__ ncand,
                              int64_t cap, const uint8_t* __restrict__ state,
                              int32_t* __restrict__ flag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    flag[i] = (i < *ncand && state[order[i]] == 1) ? 1 : 0;
}

__global__ void k_taken_write(const int32_t* __restrict__ order, const int* __restrict__ ncand,
                              const int32_t* __restrict__ flag, const int32_t* __restrict__ pos,
                              const int32_t* __restrict__ cand,
                              const unsigned long long* __restrict__ uniq, int32_t out_cap,
                              int32_t* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *ncand || !flag[i]) return;
    const int32_t p = pos[i];
    if (p >= out_cap) return;
    const int32_t k = cand[order[i]], e = k >> 1;
    const int32_t a = (int32_t)(uniq[e] >> 32), b = (int32_t)(uniq[e] & 0xffffffffu);
    out[2 * p] = (k & 1) ? b : a;
    out[2 * p + 1] = (k & 1) ? a : b;
}

unsigned blocks_for(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + 255) / 256); }

}  // namespace

int schedule_edges(tw_ctx* c, const int32_t* dtets, int64_t nt, const double* dscale,
                   double ideal_weight, int op, int32_t* out_v12, int32_t cap, int32_t* n_sched,
                   int32_t* n_cand, cudaStream_t s) {
    const int64_t ne = 6 * nt, nvt = 4 * nt, nslots = 2 * ne;
    const int32_t nv = c->nv;
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    size_t t_sort_e = 0, t_rle = 0, t_scan_e = 0, t_sort_v = 0, t_scan_v = 0, t_scan_f = 0,
           t_sort_c = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, t_sort_e, (unsigned long long*)nullptr,
                                    (unsigned long long*)nullptr, (int32_t*)nullptr,
                                    (int32_t*)nullptr, (int)ne, 0, 64, s);
    cub::DeviceRunLengthEncode::Encode(nullptr, t_rle, (unsigned long long*)nullptr,
                                       (unsigned long long*)nullptr, (int32_t*)nullptr,
                                       (int*)nullptr, (int)ne, s);
    cub::DeviceScan::ExclusiveSum(nullptr, t_scan_e, (int32_t*)nullptr, (int32_t*)nullptr,
                                  (int)(ne + 1), s);
    cub::DeviceRadixSort::SortPairs(nullptr, t_sort_v, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (int32_t*)nullptr, (int32_t*)nullptr, (int)nvt, 0, 32, s);
    cub::DeviceScan::ExclusiveSum(nullptr, t_scan_v, (int32_t*)nullptr, (int32_t*)nullptr,
                                  (int)(nv + 1), s);
    cub::DeviceScan::ExclusiveSum(nullptr, t_scan_f, (int32_t*)nullptr, (int32_t*)nullptr,
                                  (int)(nslots + 1), s);
    cub::DeviceRadixSort::SortPairsDescending(nullptr, t_sort_c, (unsigned long long*)nullptr,
                                              (unsigned long long*)nullptr, (int32_t*)nullptr,
                                              (int32_t*)nullptr, (int)nslots, 0, 64, s);
    size_t t_sort_c2 = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, t_sort_c2, (unsigned long long*)nullptr,
                                    (unsigned long long*)nullptr, (int32_t*)nullptr,
                                    (int32_t*)nullptr, (int)nslots, 0, 64, s);
    const size_t temp = std::max({t_sort_e, t_rle, t_scan_e, t_sort_v, t_scan_v, t_scan_f,
                                  t_sort_c, t_sort_c2});
    const size_t bytes = 2 * al(8 * ne) + 2 * al(4 * ne) + al(8 * ne) + al(4 * (ne + 1)) +
                         al(4 * (ne + 1)) + 2 * al(4 * nvt) + 2 * al(4 * nvt) +
                         2 * al(4 * ((size_t)nv + 1)) + 2 * al(4 * (nslots + 1)) + al(8 * ne) +
                         al(4 * nslots) + 4 * al(8 * nslots) + al(4 * nslots) + al(nslots) +
                         al(4 * nt) + al(nt) + al(temp) + 4096;
    void* p;
    int st = ensure(c, 7, bytes, &p);
    if (st != TW_OK) return st;
    char* q = static_cast<char*>(p);
    auto take = [&](size_t b) {
        char* r = q;
        q += al(b);
        return r;
    };
    auto* ekey = (unsigned long long*)take(8 * ne);
    auto* ekey_s = (unsigned long long*)take(8 * ne);
    auto* etet = (int32_t*)take(4 * ne);
    auto* etet_s = (int32_t*)take(4 * ne);
    auto* uniq = (unsigned long long*)take(8 * ne);
    auto* ecnt = (int32_t*)take(4 * (ne + 1));
    auto* eoff = (int32_t*)take(4 * (ne + 1));
    auto* vkey = (uint32_t*)take(4 * nvt);
    auto* vkey_s = (uint32_t*)take(4 * nvt);
    auto* vtet = (int32_t*)take(4 * nvt);
    auto* vtet_s = (int32_t*)take(4 * nvt);
    auto* vcnt = (int32_t*)take(4 * ((size_t)nv + 1));
    auto* voff = (int32_t*)take(4 * ((size_t)nv + 1));
    auto* flag = (int32_t*)take(4 * (nslots + 1));
    auto* fpos = (int32_t*)take(4 * (nslots + 1));
    auto* wbits = (unsigned long long*)take(8 * ne);
    auto* cand = (int32_t*)take(4 * nslots);
    auto* ckey = (unsigned long long*)take(8 * nslots);
    auto* ckey_s = (unsigned long long*)take(8 * nslots);
    auto* cidx = (int32_t*)take(8 * nslots);
    auto* order = (int32_t*)take(8 * nslots);
    auto* rank = (int32_t*)take(4 * nslots);
    auto* state = (uint8_t*)take(nslots);
    auto* claim = (uint32_t*)take(4 * nt);
    auto* taken = (uint8_t*)take(nt);
    void* tmp = take(temp);
    int* small = (int*)take(64);   // [0] bad ids, [1] unique edges, [2] candidates, [3] undecided
    cudaMemsetAsync(small, 0, 64, s);
    // edges and vertex stars
    k_tet_edges_verts<<<blocks_for(nt), 256, 0, s>>>(reinterpret_cast<const int4*>(dtets), nt, nv,
                                                     ekey, etet, vkey, vtet, small);
    size_t tb = temp;
    cub::DeviceRadixSort::SortPairs(tmp, tb, ekey, ekey_s, etet, etet_s, (int)ne, 0, 64, s);
    cudaMemsetAsync(ecnt, 0, 4 * (ne + 1), s);
    tb = temp;
    cub::DeviceRunLengthEncode::Encode(tmp, tb, ekey_s, uniq, ecnt, small + 1, (int)ne, s);
    tb = temp;
    cub::DeviceScan::ExclusiveSum(tmp, tb, ecnt, eoff, (int)(ne + 1), s);
    tb = temp;
    cub::DeviceRadixSort::SortPairs(tmp, tb, vkey, vkey_s, vtet, vtet_s, (int)nvt, 0, 32, s);
    cudaMemsetAsync(vcnt, 0, 4 * ((size_t)nv + 1), s);
    k_vertex_counts<<<blocks_for(nvt), 256, 0, s>>>(vkey_s, nvt, nv, vcnt);
    tb = temp;
    cub::DeviceScan::ExclusiveSum(tmp, tb, vcnt, voff, (int)(nv + 1), s);
    // candidates in (edge, direction) order, then by priority
    cudaMemsetAsync(flag, 0, 4 * (nslots + 1), s);
    k_candidate_flags<<<blocks_for(ne), 256, 0, s>>>(uniq, small + 1, ne, c->vx, c->vy, c->vz,
                                                     dscale, ideal_weight, op, flag, wbits);
    tb = temp;
    cub::DeviceScan::ExclusiveSum(tmp, tb, flag, fpos, (int)(nslots + 1), s);
    cudaMemcpyAsync(small + 2, fpos + nslots, sizeof(int), cudaMemcpyDeviceToDevice, s);
    k_candidates<<<blocks_for(nslots), 256, 0, s>>>(flag, fpos, nslots, wbits, cand, ckey, cidx);
    int hs[3] = {0, 0, 0};
    cudaMemcpyAsync(hs, small, 3 * sizeof(int), cudaMemcpyDeviceToHost, s);
    st = stream_status(c, "tw_schedule_edges");
    if (st != TW_OK) return st;
    if (hs[0]) return fail(c, TW_ERR_ARG, "tw_schedule_edges: vertex id out of range");
    const int ncand = hs[2];
    *n_cand = ncand;
    *n_sched = 0;
    if (ncand == 0) return TW_OK;
    tb = temp;
    if (op == TW_OP_SPLIT)   // longest first; equal lengths in (edge, direction) order
        cub::DeviceRadixSort::SortPairsDescending(tmp, tb, ckey, ckey_s, cidx, order, ncand, 0,
                                                  64, s);
    else                     // shortest first
        cub::DeviceRadixSort::SortPairs(tmp, tb, ckey, ckey_s, cidx, order, ncand, 0, 64, s);
    k_ranks<<<blocks_for(ncand), 256, 0, s>>>(order, small + 2, rank, state);
    cudaMemsetAsync(taken, 0, nt, s);
    const CandTets C{cand, uniq, eoff, etet_s, voff, vtet_s, op};
    // rounds: each takes at least the undecided candidate of lowest rank
    for (int round = 0; round <= ncand; ++round) {
        cudaMemsetAsync(claim, 0xff, 4 * nt, s);
        cudaMemsetAsync(small + 3, 0, sizeof(int), s);
        k_claim<<<blocks_for(ncand), 256, 0, s>>>(C, small + 2, state, rank, claim);
        k_select<<<blocks_for(ncand), 256, 0, s>>>(C, small + 2, state, rank, claim, taken);
        k_block<<<blocks_for(ncand), 256, 0, s>>>(C, small + 2, state, taken, small + 3);
        int undecided = 0;
        cudaMemcpyAsync(&undecided, small + 3, sizeof(int), cudaMemcpyDeviceToHost, s);
        st = stream_status(c, "tw_schedule_edges");
        if (st != TW_OK) return st;
        if (undecided == 0) break;
        if (round == ncand) return fail(c, TW_ERR_TIMEOUT, "tw_schedule_edges: rounds exhausted");
    }
    k_taken_flags<<<blocks_for(ncand + 1), 256, 0, s>>>(order, small + 2, ncand + 1, state, flag);
    tb = temp;
    cub::DeviceScan::ExclusiveSum(tmp, tb, flag, fpos, ncand + 1, s);
    k_taken_write<<<blocks_for(ncand), 256, 0, s>>>(order, small + 2, flag, fpos, cand, uniq, cap,
                                                    out_v12);
    int ns = 0;
    cudaMemcpyAsync(&ns, fpos + ncand, sizeof(int), cudaMemcpyDeviceToHost, s);
    st = stream_status(c, "tw_schedule_edges");
    if (st != TW_OK) return st;
    *n_sched = ns;
    return TW_OK;
}

}  // namespace tw
