// tw_amips.cu -- batched AMIPS energy/gradient/Hessian and exact orientation.
//
// k_amips_soa: one tet per thread over the energy_ispc SoA layout
// (energy.ispc:7-65): 12 coalesced FP64 loads per tet, E/J/H written SoA.
// The orientation filter (FP64) runs first; the rare exact fallback is an
// out-of-line call.  The FP64 pipe, not HBM, bounds this kernel on GB300.
//
// k_tet_quality_idx: calTetQualities over ids into the resident mesh
// (LocalOperations.cpp:695-773): gathers the 4 vertices, orientation, energy
// with the calTetQuality_AMIPS sentinel.
#include <atomic>
#include <cstdint>
#include <utility>

#include "tw_device.cuh"
#include "tw_internal.h"

namespace tw {

template <bool WE, bool WJ, bool WH, bool WF, bool QUAL>
__global__ void __launch_bounds__(256) k_amips_soa(const double* __restrict__ T, int64_t n,
                                                   double* __restrict__ E,
                                                   double* __restrict__ J,
                                                   double* __restrict__ H,
                                                   uint8_t* __restrict__ flip,
                                                   unsigned long long* __restrict__ exact_count,
                                                   int form) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double t[12];
#pragma unroll
        for (int c = 0; c < 12; ++c) t[c] = __ldg(T + (int64_t)c * n + i);
        int ori = 1;
        if (WF || QUAL) {
            int ex = 0;
            ori = orient3d(t, t + 3, t + 6, t + 9, &ex);
            if (ex) atomicAdd(exact_count, 1ULL);
        }
        double jv[3], hv[9];
        double e;
        if (WJ || WH) {
            e = amips_egh_f(t, WJ ? jv : nullptr, WH ? hv : nullptr, form);
        } else {
            e = amips_energy_f(t, form);
        }
        if (WE) E[i] = QUAL ? quality_from(ori, e) : e;
        if (WF) flip[i] = (uint8_t)(ori != 1);
        if (WJ) {
#pragma unroll
            for (int c = 0; c < 3; ++c) J[(int64_t)c * n + i] = jv[c];
        }
        if (WH) {
#pragma unroll
            for (int c = 0; c < 9; ++c) H[(int64_t)c * n + i] = hv[c];
        }
    }
}

// TW_PRECISION_FP32_CERTIFIED: the coordinate differences are formed in FP64
// and rounded once; orientation and E/J/H are evaluated in binary32 with the
// certified bounds of tw_device.cuh; a tet whose orientation the binary32
// filter cannot certify takes the FP64 filter (then the exact path), and a tet
// whose certified energy error exceeds 1e-5 relative is recomputed entirely
// in FP64 (in the context's energy form).  Outputs are FP64 like k_amips_soa.
// The FP64 recomputation (about 3e-6 of the tets) is a separate pass: the
// binary32 kernels append the index of each such tet to a list and write its
// flip; k_amips_recheck then evaluates the listed tets in FP64 and writes
// their E / J / H, so the binary32 kernels carry none of the registers of the
// binary64 evaluation.
constexpr float kAmipsTol32 = 1e-5f;

// One tet of the certified kernel: coordinates t in, outputs at index i.
template <bool WE, bool WJ, bool WH, bool WF, bool QUAL>
__device__ __forceinline__ void amips_cert_tet(const double* t, int64_t i, int64_t n,
                                               double* __restrict__ E, double* __restrict__ J,
                                               double* __restrict__ H,
                                               uint8_t* __restrict__ flip, uint32_t& ntet,
                                               uint32_t& nfp64, uint32_t& nexact,
                                               int32_t* __restrict__ recheck,
                                               unsigned long long* __restrict__ nrecheck) {
    {
        float d1[3], d2[3], d3[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            d1[k] = d2f_rn(t[3 + k] - t[k]);
            d2[k] = d2f_rn(t[6 + k] - t[k]);
            d3[k] = d2f_rn(t[9 + k] - t[k]);
        }
        int ori = 1;
        if (WF || QUAL) {
            ori = orient32_filter(d1, d2, d3);
            if (ori == 2) {
                int ex = 0;
                ori = orient3d(t, t + 3, t + 6, t + 9, &ex);
                nexact += ex;
            }
        }
        ++ntet;
        Amips32 R = amips_egh32<WJ, WH>(d1, d2, d3, kAmipsTol32);
        if (WF) flip[i] = (uint8_t)(ori != 1);
        if (!R.ok) {
            // E / J / H of this tet come from k_amips_recheck
            ++nfp64;
            recheck[atomicAdd(nrecheck, 1ULL)] = (int32_t)i;
            return;
        }
        // a certified binary32 energy is finite and positive: only the
        // orientation part of the sentinel rule can apply
        if (WE) E[i] = (QUAL && ori != 1) ? kMaxEnergy : f2d_exact(R.E);
        if (WJ) {
#pragma unroll
            for (int c = 0; c < 3; ++c) J[(int64_t)c * n + i] = f2d_exact(R.J[c]);
        }
        if (WH) {
#pragma unroll
            for (int c = 0; c < 9; ++c) H[(int64_t)c * n + i] = f2d_exact(R.H[c]);
        }
    }
}

__device__ __forceinline__ void flush_amips_stats(uint32_t ntet, uint32_t nfp64, uint32_t nexact,
                                                  unsigned long long* counters) {
    unsigned long long a = ntet, f = nfp64, x = nexact;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        f += __shfl_xor_sync(0xffffffffu, f, o);
        x += __shfl_xor_sync(0xffffffffu, x, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (a) atomicAdd(counters + kCntAmipsTets, a);
        if (f) atomicAdd(counters + kCntAmipsFp64, f);
        if (x) atomicAdd(counters + kCntExactOrient, x);
    }
}

// FP64 pass over the tets the binary32 kernels listed (in any order): E (with
// the calTetQuality_AMIPS sentinel in quality mode), J and H in the context's
// energy form.  The list length is read on the device.  The list is short and
// each evaluation a long chain of binary64 operations on a slow pipe, so the
// work is spread for latency: in the reference form the energy, the gradient
// and the Hessian of a tet are three independent evaluations, each taken by
// its own warp (lane 0); the closed form evaluates all three in one warp.
__global__ void __launch_bounds__(128) k_amips_recheck(
    const double* __restrict__ T, int64_t n, const int32_t* __restrict__ recheck,
    const unsigned long long* __restrict__ nrecheck, double* __restrict__ E,
    double* __restrict__ J, double* __restrict__ H, int qual, int form) {
    if ((threadIdx.x & 31) != 0) return;
    const int64_t m = (int64_t)*nrecheck;
    const int64_t stride = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < 3 * m;
         u += stride) {
        const int64_t k = u / 3;
        const int part = (int)(u - 3 * k);   // 0: E, 1: J, 2: H
        const int64_t i = recheck[k];
        double t[12];
#pragma unroll
        for (int c = 0; c < 12; ++c) t[c] = T[(int64_t)c * n + i];
        if (form == TW_ENERGY_FORM_CLOSED) {
            if (part != 0) continue;
            double jv[3], hv[9];
            const double e = amips_egh(t, J ? jv : nullptr, H ? hv : nullptr);
            if (E) E[i] = qual ? quality_from(orient3d(t, t + 3, t + 6, t + 9), e) : e;
            if (J)
                for (int c = 0; c < 3; ++c) J[(int64_t)c * n + i] = jv[c];
            if (H)
                for (int c = 0; c < 9; ++c) H[(int64_t)c * n + i] = hv[c];
        } else if (part == 0) {
            if (E) {
                const double e = amips_rf_energy(t);
                E[i] = qual ? quality_from(orient3d(t, t + 3, t + 6, t + 9), e) : e;
            }
        } else if (part == 1) {
            if (J) {
                double jv[3];
                amips_rf_jacobian(t, jv);
                for (int c = 0; c < 3; ++c) J[(int64_t)c * n + i] = jv[c];
            }
        } else if (H) {
            double hv[9];
            amips_rf_hessian(t, hv);
            for (int c = 0; c < 9; ++c) H[(int64_t)c * n + i] = hv[c];
        }
    }
}

template <bool WE, bool WJ, bool WH, bool WF, bool QUAL>
__global__ void __launch_bounds__(256) k_amips_soa_cert(const double* __restrict__ T, int64_t n,
                                                        double* __restrict__ E,
                                                        double* __restrict__ J,
                                                        double* __restrict__ H,
                                                        uint8_t* __restrict__ flip,
                                                        unsigned long long* __restrict__ counters,
                                                        int32_t* __restrict__ recheck,
                                                        unsigned long long* __restrict__ nrecheck) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    uint32_t ntet = 0, nfp64 = 0, nexact = 0;
    const int64_t base0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane;
    for (int64_t b = base0; b < n; b += stride) {
        const int64_t i = b + lane;
        if (i >= n) continue;
        double t[12];
#pragma unroll
        for (int c = 0; c < 12; ++c) t[c] = __ldg(T + (int64_t)c * n + i);
        amips_cert_tet<WE, WJ, WH, WF, QUAL>(t, i, n, E, J, H, flip, ntet, nfp64, nexact, recheck,
                                             nrecheck);
    }
    flush_amips_stats(ntet, nfp64, nexact, counters);
}

// ---------------------------------------------------------------------------
// The same with the coordinates staged by the bulk-copy engine: tiles of 256
// tets, the 12 SoA rows of a tile (2 KB each) copied into shared memory by
// cp.async.bulk on an mbarrier, two tiles in flight per block while the
// threads compute the previous one.  Needs n even and T 16-byte aligned (so
// every row segment starts on a 16-byte boundary); partial tail tiles are
// read directly.  A wait that does not complete within its iteration limit
// sets error bit 32 and ends the block.  Three blocks per SM (80 registers,
// 3 x 48 KB of stages): 0.183 ms per 4M tets against 0.214 at two blocks and
// 0.222 at four (64 registers, spilling).
// ---------------------------------------------------------------------------
constexpr int kBulkTile = 256;
constexpr int kBulkStages = 2;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// true when the barrier's phase with this parity completed within the limit
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = 1 << 20) {
    for (int it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Self-test of the bounded wait (one thread): a barrier whose phase needs 16
// bytes that no copy delivers must give up after `limit` polls, and one fed by
// a 16-byte bulk copy must complete.  out = {1 when the first gave up, 1 when
// the second completed, cycles the first took, the first copied word}.
__global__ void k_selftest_wait(const double* __restrict__ src, int limit,
                                unsigned long long* __restrict__ out) {
    __shared__ __align__(16) double buf[2];
    __shared__ __align__(8) uint64_t bar[2];
    if (threadIdx.x != 0) return;
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_expect_tx(&bar[0], 16);   // no copy will complete this phase
    const long long t0 = clock64();
    const bool done0 = mbar_wait(&bar[0], 0, limit);
    const long long t1 = clock64();
    mbar_expect_tx(&bar[1], 16);
    bulk_g2s(buf, src, 16, &bar[1]);
    bool done1 = mbar_wait(&bar[1], 0);
    if (!done1) done1 = mbar_wait(&bar[1], 0);   // no copy may outlive the kernel
    out[0] = done0 ? 0ULL : 1ULL;
    out[1] = done1 ? 1ULL : 0ULL;
    out[2] = (unsigned long long)(t1 - t0);
    out[3] = done1 ? (unsigned long long)__double_as_longlong(buf[0]) : 0ULL;
}

void launch_selftest_wait(const double* src, int limit, unsigned long long* out, cudaStream_t s) {
    k_selftest_wait<<<1, 32, 0, s>>>(src, limit, out);
}

template <bool WE, bool WJ, bool WH, bool WF, bool QUAL>
__global__ void __launch_bounds__(kBulkTile, 3) k_amips_soa_cert_bulk(
    const double* __restrict__ T, int64_t n, double* __restrict__ E, double* __restrict__ J,
    double* __restrict__ H, uint8_t* __restrict__ flip, unsigned long long* __restrict__ counters,
    int32_t* __restrict__ recheck, unsigned long long* __restrict__ nrecheck) {
    extern __shared__ __align__(128) double stage_mem[];   // kBulkStages x 12 x kBulkTile
    double(*stage)[12 * kBulkTile] = reinterpret_cast<double(*)[12 * kBulkTile]>(stage_mem);
    __shared__ __align__(8) uint64_t bar[kBulkStages];
    __shared__ int abort_flag;
    __shared__ int pend[kBulkStages];   // a copy issued into stage k and not yet consumed
    uint32_t ntet = 0, nfp64 = 0, nexact = 0;
    const int64_t full = n / kBulkTile;               // full tiles
    const int64_t ntiles = (n + kBulkTile - 1) / kBulkTile;
    if (threadIdx.x == 0) {
        for (int k = 0; k < kBulkStages; ++k) {
            mbar_init(&bar[k], 1);
            pend[k] = 0;
        }
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int64_t tile, int k) {
        pend[k] = 1;
        mbar_expect_tx(&bar[k], 12 * kBulkTile * 8);
        for (int c = 0; c < 12; ++c)
            bulk_g2s(&stage[k][c * kBulkTile], T + (int64_t)c * n + tile * kBulkTile,
                     kBulkTile * 8, &bar[k]);
    };
    // prologue: the first kBulkStages tiles of this block
    if (threadIdx.x == 0)
        for (int k = 0; k < kBulkStages; ++k) {
            const int64_t tile = blockIdx.x + (int64_t)k * gridDim.x;
            if (tile < full) issue(tile, k);
        }
    uint32_t phase[kBulkStages] = {0, 0};
    int k = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t i = tile * kBulkTile + threadIdx.x;
        double t[12];
        if (tile < full) {
            if (!mbar_wait(&bar[k], phase[k])) atomicExch(&abort_flag, 1);
            __syncthreads();
            if (abort_flag) {
                // leave no copy writing into this block's shared memory: wait
                // again, with the same limit, for every stage still pending
                if (threadIdx.x == 0) {
                    atomicOr(counters + kCntError, 32ULL);
                    for (int s2 = 0; s2 < kBulkStages; ++s2)
                        if (pend[s2]) mbar_wait(&bar[s2], phase[s2]);
                }
                __syncthreads();
                break;
            }
            phase[k] ^= 1u;
            if (threadIdx.x == 0) pend[k] = 0;
#pragma unroll
            for (int c = 0; c < 12; ++c) t[c] = stage[k][c * kBulkTile + threadIdx.x];
            __syncthreads();  // every thread has its coordinates: the stage may be refilled
            if (threadIdx.x == 0) {
                const int64_t next = tile + (int64_t)kBulkStages * gridDim.x;
                if (next < full) issue(next, k);
            }
            k = (k + 1) % kBulkStages;
        } else {
            if (i >= n) continue;
#pragma unroll
            for (int c = 0; c < 12; ++c) t[c] = __ldg(T + (int64_t)c * n + i);
        }
        amips_cert_tet<WE, WJ, WH, WF, QUAL>(t, i, n, E, J, H, flip, ntet, nfp64, nexact, recheck,
                                             nrecheck);
    }
    flush_amips_stats(ntet, nfp64, nexact, counters);
}

// Per-device caches (SM count; kernels whose shared-memory limit was raised),
// indexed by the device ordinal and safe to fill from several threads: both
// values are idempotent, so a race only repeats the query.
constexpr int kMaxDevices = 64;
static std::atomic<int> g_sm_count[kMaxDevices];
static std::atomic<uint32_t> g_bulk_attr_set[kMaxDevices];

static int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        dev = 0;
    }
    return dev;
}

int grid_for(int64_t n, int block, int blocks_per_sm) {
    const int dev = current_device();
    int sms = g_sm_count[dev].load(std::memory_order_relaxed);
    if (sms <= 0) {
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            sms = 0;
        }
        if (sms <= 0) sms = 1;
        else g_sm_count[dev].store(sms, std::memory_order_relaxed);
    }
    int64_t need = (n + block - 1) / block;
    int64_t cap = (int64_t)sms * blocks_per_sm;
    if (need < 1) need = 1;
    return (int)(need < cap ? need : cap);
}

using AmipsKernel = void (*)(const double*, int64_t, double*, double*, double*, uint8_t*,
                             unsigned long long*, int);
using AmipsCertKernel = void (*)(const double*, int64_t, double*, double*, double*, uint8_t*,
                                 unsigned long long*, int32_t*, unsigned long long*);

template <int BITS>
static AmipsKernel pick_amips() {
    return k_amips_soa<(BITS & 1) != 0, (BITS & 2) != 0, (BITS & 4) != 0, (BITS & 8) != 0,
                       (BITS & 16) != 0>;
}

template <int... B>
static AmipsKernel amips_table(int bits, std::integer_sequence<int, B...>) {
    static const AmipsKernel table[] = {pick_amips<B>()...};
    return table[bits];
}

void launch_amips_soa(const double* T, int64_t n, int mode, double* E, double* J, double* H,
                      uint8_t* flip, unsigned long long* exact_count, cudaStream_t s, int form) {
    if (n <= 0) return;
    int bits = (E ? 1 : 0) | (J ? 2 : 0) | (H ? 4 : 0) | (flip ? 8 : 0) |
               ((mode == TW_ENERGY_QUALITY && E) ? 16 : 0);
    AmipsKernel k = amips_table(bits, std::make_integer_sequence<int, 32>{});
    const int block = 256;
    int grid = grid_for(n, block, 8);
    k<<<grid, block, 0, s>>>(T, n, E, J, H, flip, exact_count, form);
}

template <int BITS>
static AmipsCertKernel pick_amips_cert() {
    return k_amips_soa_cert<(BITS & 1) != 0, (BITS & 2) != 0, (BITS & 4) != 0, (BITS & 8) != 0,
                            (BITS & 16) != 0>;
}

template <int... B>
static AmipsCertKernel amips_cert_table(int bits, std::integer_sequence<int, B...>) {
    static const AmipsCertKernel table[] = {pick_amips_cert<B>()...};
    return table[bits];
}

template <int BITS>
static AmipsCertKernel pick_amips_bulk() {
    return k_amips_soa_cert_bulk<(BITS & 1) != 0, (BITS & 2) != 0, (BITS & 4) != 0,
                                 (BITS & 8) != 0, (BITS & 16) != 0>;
}

template <int... B>
static AmipsCertKernel amips_bulk_table(int bits, std::integer_sequence<int, B...>) {
    static const AmipsCertKernel table[] = {pick_amips_bulk<B>()...};
    return table[bits];
}

void launch_amips_soa_cert(const double* T, int64_t n, int mode, double* E, double* J, double* H,
                           uint8_t* flip, unsigned long long* counters, void* recheck_scratch,
                           cudaStream_t s, int form) {
    if (n <= 0) return;
    // recheck list: a count (zeroed here) and n indices
    auto* nrecheck = static_cast<unsigned long long*>(recheck_scratch);
    int32_t* recheck = reinterpret_cast<int32_t*>(static_cast<char*>(recheck_scratch) + 256);
    cudaMemsetAsync(nrecheck, 0, sizeof(unsigned long long), s);
    const bool qual = (mode == TW_ENERGY_QUALITY && E);
    int bits = (E ? 1 : 0) | (J ? 2 : 0) | (H ? 4 : 0) | (flip ? 8 : 0) |
               ((mode == TW_ENERGY_QUALITY && E) ? 16 : 0);
    // bulk staging needs every row segment 16-byte aligned and is worth it
    // for batches of at least a few tiles per SM; the coordinates must be in
    // device memory (the copy engine path, not a host mapping)
    cudaPointerAttributes a;
    const bool device_mem = cudaPointerGetAttributes(&a, T) == cudaSuccess &&
                            a.type == cudaMemoryTypeDevice;
    if (!device_mem) cudaGetLastError();
    if (device_mem && n % 2 == 0 && ((uintptr_t)T & 15) == 0 && n >= 64 * kBulkTile) {
        AmipsCertKernel k = amips_bulk_table(bits, std::make_integer_sequence<int, 32>{});
        const int smem = kBulkStages * 12 * kBulkTile * (int)sizeof(double);
        // the shared-memory limit is a per-device attribute of the kernel
        const int dev = current_device();
        const uint32_t bit = 1u << bits;
        if (!(g_bulk_attr_set[dev].load(std::memory_order_acquire) & bit)) {
            if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) ==
                cudaSuccess)
                g_bulk_attr_set[dev].fetch_or(bit, std::memory_order_acq_rel);
        }
        k<<<grid_for(n, kBulkTile, 3), kBulkTile, smem, s>>>(T, n, E, J, H, flip, counters,
                                                             recheck, nrecheck);
    } else {
        AmipsCertKernel k = amips_cert_table(bits, std::make_integer_sequence<int, 32>{});
        const int block = 256;
        k<<<grid_for(n, block, 8), block, 0, s>>>(T, n, E, J, H, flip, counters, recheck,
                                                   nrecheck);
    }
    if (E || J || H)
        k_amips_recheck<<<grid_for(INT32_MAX, 128, 4), 128, 0, s>>>(T, n, recheck, nrecheck, E,
                                                                    J, H, qual ? 1 : 0, form);
}

size_t amips_recheck_scratch_bytes(int64_t n) { return 256 + 4 * (size_t)(n > 0 ? n : 0); }

__global__ void __launch_bounds__(256) k_tet_quality_idx(
    const int4* __restrict__ tets, int64_t n, const double* __restrict__ vx,
    const double* __restrict__ vy, const double* __restrict__ vz,
    const uint8_t* __restrict__ rounded, double* __restrict__ E, uint8_t* __restrict__ flip,
    uint8_t* __restrict__ needs_host, unsigned long long* __restrict__ counters, int form) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        int4 tv = __ldg(tets + i);
        int id[4] = {tv.x, tv.y, tv.z, tv.w};
        double t[12];
        bool all_rounded = true;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            t[3 * j] = __ldg(vx + id[j]);
            t[3 * j + 1] = __ldg(vy + id[j]);
            t[3 * j + 2] = __ldg(vz + id[j]);
            if (rounded) all_rounded = all_rounded && (__ldg(rounded + id[j]) != 0);
        }
        int ex = 0;
        int ori = orient3d(t, t + 3, t + 6, t + 9, &ex);
        if (ex) atomicAdd(counters, 1ULL);
        if (E) E[i] = quality_from(ori, amips_energy_f(t, form));
        if (flip) flip[i] = (uint8_t)(ori != 1);
        if (needs_host) needs_host[i] = (uint8_t)(!all_rounded);
        if (!all_rounded) atomicAdd(counters + 1, 1ULL);
    }
}

void launch_tet_quality_idx(const int32_t* tets, int64_t n, const double* vx, const double* vy,
                            const double* vz, const uint8_t* rounded, double* E, uint8_t* flip,
                            uint8_t* needs_host, unsigned long long* counters, cudaStream_t s,
                            int form) {
    if (n <= 0) return;
    const int block = 256;
    k_tet_quality_idx<<<grid_for(n, block, 8), block, 0, s>>>(
        reinterpret_cast<const int4*>(tets), n, vx, vy, vz, rounded, E, flip, needs_host,
        counters, form);
}


// ---------------------------------------------------------------------------
// Energy sweeps (LocalOperations.cpp:605-693): per tet the calTetQuality_AMIPS
// value at the resident positions; max and second max (skipping MAX_ENERGY)
// over the unlocked tets as the largest bit pattern of a non-negative double
// (order-free, exact); the sum of the unlocked energies as a double-double
// per thread, per block (fixed tree) and over the blocks in block order
// (deterministic, within a few ulps of the exact sum); getFilterEnergy's
// eleven bucket counts over every tet.
// ---------------------------------------------------------------------------
struct DD {
    double hi, lo;
};
__device__ __forceinline__ DD dd_add(DD a, DD b) {
    double s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    double h, l;
    fast_two_sum(s, e, h, l);
    return DD{h, l};
}

constexpr int kStatsBlock = 256;

__global__ void __launch_bounds__(kStatsBlock) k_energy_stats(
    const int4* __restrict__ tets, int64_t n, const double* __restrict__ vx,
    const double* __restrict__ vy, const double* __restrict__ vz,
    const uint8_t* __restrict__ locked, double thres_m1, DD* __restrict__ block_sum,
    unsigned long long* __restrict__ acc, int form) {
    // acc: [0] max bits, [1] second-max bits, [2] unlocked count, [3..13] buckets
    __shared__ unsigned long long sb[11];
    __shared__ DD ssum[kStatsBlock / 32];
    if (threadIdx.x < 11) sb[threadIdx.x] = 0;
    __syncthreads();
    DD sum{0.0, 0.0};
    unsigned long long mx = 0, mx2 = 0, cnt = 0;
    const double p10[11] = {1.0, 1e1, 1e2, 1e3, 1e4, 1e5, 1e6, 1e7, 1e8, 1e9, 1e10};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int4 tv = __ldg(tets + i);
        const int id[4] = {tv.x, tv.y, tv.z, tv.w};
        double t[12];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            t[3 * j] = __ldg(vx + id[j]);
            t[3 * j + 1] = __ldg(vy + id[j]);
            t[3 * j + 2] = __ldg(vz + id[j]);
        }
        const double e = quality_from(orient3d(t, t + 3, t + 6, t + 9), amips_energy_f(t, form));
        int bk = -1;
        if (e > thres_m1 + 1e10) {
            bk = 10;
        } else {
            for (int j = 0; j < 10; ++j)
                if (e > thres_m1 + p10[j] && e <= thres_m1 + p10[j + 1]) {
                    bk = j;
                    break;
                }
        }
        if (bk >= 0) atomicAdd(&sb[bk], 1ULL);
        if (locked && __ldg(locked + i)) continue;
        const unsigned long long bits = (unsigned long long)__double_as_longlong(e);
        mx = max(mx, bits);
        if (e != kMaxEnergy) mx2 = max(mx2, bits);
        sum = dd_add(sum, DD{e, 0.0});
        ++cnt;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        DD other{__shfl_down_sync(0xffffffffu, sum.hi, o), __shfl_down_sync(0xffffffffu, sum.lo, o)};
        sum = dd_add(sum, other);
        mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
        mx2 = max(mx2, __shfl_down_sync(0xffffffffu, mx2, o));
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0) {
        ssum[threadIdx.x >> 5] = sum;
        atomicMax(acc + 0, mx);
        atomicMax(acc + 1, mx2);
        atomicAdd(acc + 2, cnt);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        DD b = ssum[0];
        for (int w = 1; w < kStatsBlock / 32; ++w) b = dd_add(b, ssum[w]);
        block_sum[blockIdx.x] = b;
    }
    if (threadIdx.x < 11 && sb[threadIdx.x]) atomicAdd(acc + 3 + threadIdx.x, sb[threadIdx.x]);
}

__global__ void k_energy_stats_sum(const DD* __restrict__ block_sum, int nblocks,
                                   double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    DD s{0.0, 0.0};
    for (int b = 0; b < nblocks; ++b) s = dd_add(s, block_sum[b]);
    out[0] = s.hi + s.lo;
}

int energy_stats_blocks(int64_t n) { return grid_for(n > 0 ? n : 1, kStatsBlock, 4); }

// ---------------------------------------------------------------------------
// Dihedral angles (calTetQuality_AD, LocalOperations.cpp:783-860) and
// outputInfo's sweep over them (:483-521).  Per face i (the other vertices
// p, q, r from i+1 on): normal (a, b, c) = (p - r) x (q - r), offset
// d = -(a r.x + b r.y + c r.z); vertex s = v_i projects to s - lambda (a, b, c)
// with lambda = (a s + d) / |(a, b, c)|^2; nv_i = s - projection, rescaled by
// its largest component below 1e-5.  A zero normal, a projection equal to s or
// a zero nv gives (0, pi).  Angles acos(-nv_a . nv_b / (|nv_a| |nv_b|)) over
// the pairs (0,1), (1,2), (0,2), (2,3), (0,3), (3,1).  Operation for operation
// as the oracle; acos is CUDA's.
// ---------------------------------------------------------------------------
constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ void tet_dihedral_minmax(const double* T, double& mn, double& mx) {
    double nv[4][3], len[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const double* sv = T + 3 * i;
        const double* p = T + 3 * ((i + 1) % 4);
        const double* q = T + 3 * ((i + 2) % 4);
        const double* r = T + 3 * ((i + 3) % 4);
        const double rp0 = p[0] - r[0], rp1 = p[1] - r[1], rp2 = p[2] - r[2];
        const double rq0 = q[0] - r[0], rq1 = q[1] - r[1], rq2 = q[2] - r[2];
        const double a = rp1 * rq2 - rq1 * rp2;
        const double b = rp2 * rq0 - rq2 * rp0;
        const double c = rp0 * rq1 - rq0 * rp1;
        if (a == 0.0 && b == 0.0 && c == 0.0) {
            mn = 0.0;
            mx = kPi;
            return;
        }
        const double d = ((-a * r[0]) - b * r[1]) - c * r[2];
        const double num = ((a * sv[0] + b * sv[1]) + c * sv[2]) + d;
        const double den = (a * a + b * b) + c * c;
        const double lam = num / den;
        const double pr0 = sv[0] - lam * a, pr1 = sv[1] - lam * b, pr2 = sv[2] - lam * c;
        if (pr0 == sv[0] && pr1 == sv[1] && pr2 == sv[2]) {
            mn = 0.0;
            mx = kPi;
            return;
        }
        double v0 = sv[0] - pr0, v1 = sv[1] - pr1, v2 = sv[2] - pr2;
        const double h = (v0 * v0 + v1 * v1) + v2 * v2;
        double m = fabs(v0);
        if (fabs(v1) > m) m = fabs(v1);
        if (fabs(v2) > m) m = fabs(v2);
        if (m == 0.0 || h == 0.0) {
            mn = 0.0;
            mx = kPi;
            return;
        }
        if (m < 1e-5) {
            v0 = v0 / m;
            v1 = v1 / m;
            v2 = v2 / m;
            len[i] = sqrt(h / (m * m));
        } else {
            len[i] = sqrt(h);
        }
        nv[i][0] = v0;
        nv[i][1] = v1;
        nv[i][2] = v2;
    }
    const int pa[6] = {0, 1, 0, 2, 0, 3}, pb[6] = {1, 2, 2, 3, 3, 1};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const double* u = nv[pa[k]];
        const double* w = nv[pb[k]];
        const double cs =
            ((-u[0]) * w[0] + (-u[1]) * w[1] + (-u[2]) * w[2]) / (len[pa[k]] * len[pb[k]]);
        const double ang = cs > 1.0 ? 0.0 : cs < -1.0 ? kPi : acos(cs);
        if (k == 0 || ang < mn) mn = ang;
        if (k == 0 || ang > mx) mx = ang;
    }
}

// acc: [0] min bits (initialised to 10.0's), [1] max bits, [2..7] threshold
// counts, [8] unlocked count; block_sum: per block the DD sums of the mins
// and of the maxes.
__global__ void __launch_bounds__(kStatsBlock) k_dihedral_stats(
    const int4* __restrict__ tets, int64_t n, const double* __restrict__ vx,
    const double* __restrict__ vy, const double* __restrict__ vz,
    const uint8_t* __restrict__ locked, double* __restrict__ mins, double* __restrict__ maxs,
    DD* __restrict__ block_sum, unsigned long long* __restrict__ acc) {
    __shared__ DD ssum[2][kStatsBlock / 32];
    const double cmp[6] = {6 / 180.0 * kPi, 12 / 180.0 * kPi, 18 / 180.0 * kPi,
                           162 / 180.0 * kPi, 168 / 180.0 * kPi, 174 / 180.0 * kPi};
    DD smn{0.0, 0.0}, smx{0.0, 0.0};
    unsigned long long bmn = (unsigned long long)__double_as_longlong(10.0), bmx = 0, cnt = 0;
    unsigned long long c6[6] = {0, 0, 0, 0, 0, 0};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int4 tv = __ldg(tets + i);
        const int id[4] = {tv.x, tv.y, tv.z, tv.w};
        double t[12];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            t[3 * j] = __ldg(vx + id[j]);
            t[3 * j + 1] = __ldg(vy + id[j]);
            t[3 * j + 2] = __ldg(vz + id[j]);
        }
        double a = 0.0, b = 0.0;
        tet_dihedral_minmax(t, a, b);
        if (mins) mins[i] = a;
        if (maxs) maxs[i] = b;
        if (locked && __ldg(locked + i)) continue;
        // angles are >= 0: their bit patterns order as the values
        bmn = min(bmn, (unsigned long long)__double_as_longlong(a));
        bmx = max(bmx, (unsigned long long)__double_as_longlong(b));
        smn = dd_add(smn, DD{a, 0.0});
        smx = dd_add(smx, DD{b, 0.0});
        ++cnt;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            c6[j] += a < cmp[j] ? 1 : 0;
            c6[j + 3] += b > cmp[j + 3] ? 1 : 0;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        DD x{__shfl_down_sync(0xffffffffu, smn.hi, o), __shfl_down_sync(0xffffffffu, smn.lo, o)};
        smn = dd_add(smn, x);
        DD y{__shfl_down_sync(0xffffffffu, smx.hi, o), __shfl_down_sync(0xffffffffu, smx.lo, o)};
        smx = dd_add(smx, y);
        bmn = min(bmn, __shfl_down_sync(0xffffffffu, bmn, o));
        bmx = max(bmx, __shfl_down_sync(0xffffffffu, bmx, o));
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
#pragma unroll
        for (int j = 0; j < 6; ++j) c6[j] += __shfl_down_sync(0xffffffffu, c6[j], o);
    }
    if ((threadIdx.x & 31) == 0) {
        ssum[0][threadIdx.x >> 5] = smn;
        ssum[1][threadIdx.x >> 5] = smx;
        atomicMin(acc + 0, bmn);
        atomicMax(acc + 1, bmx);
#pragma unroll
        for (int j = 0; j < 6; ++j)
            if (c6[j]) atomicAdd(acc + 2 + j, c6[j]);
        if (cnt) atomicAdd(acc + 8, cnt);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        DD a = ssum[0][0], b = ssum[1][0];
        for (int w = 1; w < kStatsBlock / 32; ++w) {
            a = dd_add(a, ssum[0][w]);
            b = dd_add(b, ssum[1][w]);
        }
        block_sum[2 * blockIdx.x] = a;
        block_sum[2 * blockIdx.x + 1] = b;
    }
}

__global__ void k_dihedral_stats_sum(const DD* __restrict__ block_sum, int nblocks,
                                     double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    DD a{0.0, 0.0}, b{0.0, 0.0};
    for (int k = 0; k < nblocks; ++k) {
        a = dd_add(a, block_sum[2 * k]);
        b = dd_add(b, block_sum[2 * k + 1]);
    }
    out[0] = a.hi + a.lo;
    out[1] = b.hi + b.lo;
}

void launch_dihedral_stats(const int32_t* tets, int64_t n, const double* vx, const double* vy,
                           const double* vz, const uint8_t* locked, double* mins, double* maxs,
                           void* block_sum, unsigned long long* acc, double* sums_out,
                           cudaStream_t s) {
    const int blocks = energy_stats_blocks(n);
    k_dihedral_stats<<<blocks, kStatsBlock, 0, s>>>(reinterpret_cast<const int4*>(tets), n, vx,
                                                    vy, vz, locked, mins, maxs, (DD*)block_sum,
                                                    acc);
    k_dihedral_stats_sum<<<1, 32, 0, s>>>((const DD*)block_sum, blocks, sums_out);
}

void launch_energy_stats(const int32_t* tets, int64_t n, const double* vx, const double* vy,
                         const double* vz, const uint8_t* locked, double thres,
                         void* block_sum, unsigned long long* acc, double* sum_out,
                         cudaStream_t s, int form) {
    const int blocks = energy_stats_blocks(n);
    k_energy_stats<<<blocks, kStatsBlock, 0, s>>>(reinterpret_cast<const int4*>(tets), n, vx, vy,
                                                  vz, locked, thres - 1, (DD*)block_sum, acc,
                                                  form);
    k_energy_stats_sum<<<1, 32, 0, s>>>((const DD*)block_sum, blocks, sum_out);
}

}  // namespace tw
