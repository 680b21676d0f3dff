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
                                                   unsigned long long* __restrict__ exact_count) {
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
            e = amips_egh(t, WJ ? jv : nullptr, WH ? hv : nullptr);
        } else {
            e = amips_energy(t);
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
// in FP64 (amips_egh).  Outputs are FP64 like k_amips_soa.
constexpr float kAmipsTol32 = 1e-5f;

template <bool WE, bool WJ, bool WH, bool WF, bool QUAL>
__global__ void __launch_bounds__(256) k_amips_soa_cert(const double* __restrict__ T, int64_t n,
                                                        double* __restrict__ E,
                                                        double* __restrict__ J,
                                                        double* __restrict__ H,
                                                        uint8_t* __restrict__ flip,
                                                        unsigned long long* __restrict__ counters) {
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
        double e, jv[3], hv[9];
        if (R.ok) {
            e = f2d_exact(R.E);
            if (WJ)
#pragma unroll
                for (int c = 0; c < 3; ++c) jv[c] = f2d_exact(R.J[c]);
            if (WH)
#pragma unroll
                for (int c = 0; c < 9; ++c) hv[c] = f2d_exact(R.H[c]);
        } else {
            ++nfp64;
            if (WJ || WH)
                e = amips_egh(t, WJ ? jv : nullptr, WH ? hv : nullptr);
            else
                e = amips_energy(t);
        }
        if (WE) {
            // a certified binary32 energy is finite and positive: only the
            // orientation part of the sentinel rule can apply
            if (R.ok)
                E[i] = (QUAL && ori != 1) ? kMaxEnergy : e;
            else
                E[i] = QUAL ? quality_from(ori, e) : e;
        }
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
    unsigned long long a = ntet, f = nfp64, x = nexact;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        f += __shfl_xor_sync(0xffffffffu, f, o);
        x += __shfl_xor_sync(0xffffffffu, x, o);
    }
    if (lane == 0) {
        if (a) atomicAdd(counters + kCntAmipsTets, a);
        if (f) atomicAdd(counters + kCntAmipsFp64, f);
        if (x) atomicAdd(counters + kCntExactOrient, x);
    }
}

int grid_for(int64_t n, int block, int blocks_per_sm) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int64_t need = (n + block - 1) / block;
    int64_t cap = (int64_t)sms * blocks_per_sm;
    if (need < 1) need = 1;
    return (int)(need < cap ? need : cap);
}

using AmipsKernel = void (*)(const double*, int64_t, double*, double*, double*, uint8_t*,
                             unsigned long long*);

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
                      uint8_t* flip, unsigned long long* exact_count, cudaStream_t s) {
    if (n <= 0) return;
    int bits = (E ? 1 : 0) | (J ? 2 : 0) | (H ? 4 : 0) | (flip ? 8 : 0) |
               ((mode == TW_ENERGY_QUALITY && E) ? 16 : 0);
    AmipsKernel k = amips_table(bits, std::make_integer_sequence<int, 32>{});
    const int block = 256;
    int grid = grid_for(n, block, 8);
    k<<<grid, block, 0, s>>>(T, n, E, J, H, flip, exact_count);
}

template <int BITS>
static AmipsKernel pick_amips_cert() {
    return k_amips_soa_cert<(BITS & 1) != 0, (BITS & 2) != 0, (BITS & 4) != 0, (BITS & 8) != 0,
                            (BITS & 16) != 0>;
}

template <int... B>
static AmipsKernel amips_cert_table(int bits, std::integer_sequence<int, B...>) {
    static const AmipsKernel table[] = {pick_amips_cert<B>()...};
    return table[bits];
}

void launch_amips_soa_cert(const double* T, int64_t n, int mode, double* E, double* J, double* H,
                           uint8_t* flip, unsigned long long* counters, cudaStream_t s) {
    if (n <= 0) return;
    int bits = (E ? 1 : 0) | (J ? 2 : 0) | (H ? 4 : 0) | (flip ? 8 : 0) |
               ((mode == TW_ENERGY_QUALITY && E) ? 16 : 0);
    AmipsKernel k = amips_cert_table(bits, std::make_integer_sequence<int, 32>{});
    const int block = 256;
    int grid = grid_for(n, block, 8);
    k<<<grid, block, 0, s>>>(T, n, E, J, H, flip, counters);
}

__global__ void __launch_bounds__(256) k_tet_quality_idx(
    const int4* __restrict__ tets, int64_t n, const double* __restrict__ vx,
    const double* __restrict__ vy, const double* __restrict__ vz,
    const uint8_t* __restrict__ rounded, double* __restrict__ E, uint8_t* __restrict__ flip,
    uint8_t* __restrict__ needs_host, unsigned long long* __restrict__ counters) {
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
        if (E) E[i] = quality_from(ori, amips_energy(t));
        if (flip) flip[i] = (uint8_t)(ori != 1);
        if (needs_host) needs_host[i] = (uint8_t)(!all_rounded);
        if (!all_rounded) atomicAdd(counters + 1, 1ULL);
    }
}

void launch_tet_quality_idx(const int32_t* tets, int64_t n, const double* vx, const double* vy,
                            const double* vz, const uint8_t* rounded, double* E, uint8_t* flip,
                            uint8_t* needs_host, unsigned long long* counters, cudaStream_t s) {
    if (n <= 0) return;
    const int block = 256;
    k_tet_quality_idx<<<grid_for(n, block, 8), block, 0, s>>>(
        reinterpret_cast<const int4*>(tets), n, vx, vy, vz, rounded, E, flip, needs_host,
        counters);
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
    unsigned long long* __restrict__ acc) {
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
        const double e = quality_from(orient3d(t, t + 3, t + 6, t + 9), amips_energy(t));
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

void launch_energy_stats(const int32_t* tets, int64_t n, const double* vx, const double* vy,
                         const double* vz, const uint8_t* locked, double thres,
                         void* block_sum, unsigned long long* acc, double* sum_out,
                         cudaStream_t s) {
    const int blocks = energy_stats_blocks(n);
    k_energy_stats<<<blocks, kStatsBlock, 0, s>>>(reinterpret_cast<const int4*>(tets), n, vx, vy,
                                                  vz, locked, thres - 1, (DD*)block_sum, acc);
    k_energy_stats_sum<<<1, 32, 0, s>>>((const DD*)block_sum, blocks, sum_out);
}

}  // namespace tw
