// tw_capi.cu -- the extern "C" boundary (include/tw_gb300.h).
//
// Host-pointer calls run a chunked pipeline over three streams: chunk k is
// copied in, computed and copied out on stream k % 3, so host<->device
// copies of one chunk overlap the kernels of the others.  _device calls
// enqueue one kernel on the context stream and return.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "tw_device.cuh"
#include "tw_internal.h"

namespace tw {

int fail(tw_ctx* c, int code, const std::string& msg) {
    if (c) c->last_error = msg;
    return code;
}

int cuda_fail(tw_ctx* c, cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return fail(c, e == cudaErrorMemoryAllocation ? TW_ERR_OOM : TW_ERR_CUDA, m);
}

int dev_alloc(tw_ctx* c, size_t bytes, void** out) {
    *out = nullptr;
    if (bytes == 0) bytes = 16;
    if (c->budget && c->used + bytes > c->budget)
        return fail(c, TW_ERR_OOM, "HBM budget of the context exceeded");
    cudaError_t e = cudaMalloc(out, bytes);
    if (e != cudaSuccess) {
        *out = nullptr;
        return cuda_fail(c, e, "cudaMalloc");
    }
    c->used += bytes;
    return TW_OK;
}

void dev_free(tw_ctx* c, void* p, size_t bytes) {
    if (!p) return;
    cudaFree(p);
    if (bytes == 0) bytes = 16;
    c->used -= std::min(c->used, bytes);
}

int ensure(tw_ctx* c, int slot, size_t bytes, void** out) {
    Buffer& b = c->scratch[slot];
    if (b.cap < bytes) {
        if (b.ptr) dev_free(c, b.ptr, b.cap);
        b.ptr = nullptr;
        b.cap = 0;
        size_t want = bytes + bytes / 8;
        int st = dev_alloc(c, want, &b.ptr);
        if (st != TW_OK) return st;
        b.cap = want;
    }
    *out = b.ptr;
    return TW_OK;
}

// ---- pipe peak probes -------------------------------------------------------
__global__ void k_fp64_probe(double* out, int iters) {
    double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
    double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
    const double b = 0.999999, cc = 1e-12;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, b, cc); a1 = fma(a1, b, cc); a2 = fma(a2, b, cc); a3 = fma(a3, b, cc);
        a4 = fma(a4, b, cc); a5 = fma(a5, b, cc); a6 = fma(a6, b, cc); a7 = fma(a7, b, cc);
    }
    double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == 12345.678) out[0] = s;  // keeps the loop live
}
__global__ void k_fp32_probe(float* out, int iters) {
    float a0 = threadIdx.x * 1e-6f, a1 = a0 + 1e-6f, a2 = a0 + 2e-6f, a3 = a0 + 3e-6f;
    float a4 = a0 + 4e-6f, a5 = a0 + 5e-6f, a6 = a0 + 6e-6f, a7 = a0 + 7e-6f;
    const float b = 0.9999f, cc = 1e-7f;
    for (int i = 0; i < iters; ++i) {
        a0 = fmaf(a0, b, cc); a1 = fmaf(a1, b, cc); a2 = fmaf(a2, b, cc); a3 = fmaf(a3, b, cc);
        a4 = fmaf(a4, b, cc); a5 = fmaf(a5, b, cc); a6 = fmaf(a6, b, cc); a7 = fmaf(a7, b, cc);
    }
    float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == 12345.678f) out[0] = s;
}
void launch_fp64_probe(double* out, int iters, int blocks, cudaStream_t s) {
    k_fp64_probe<<<blocks, 256, 0, s>>>(out, iters);
}
void launch_fp32_probe(float* out, int iters, int blocks, cudaStream_t s) {
    k_fp32_probe<<<blocks, 256, 0, s>>>(out, iters);
}

// Self-test of the integer-arithmetic conversions against the hardware
// conversions on pseudo-random bit patterns (all classes: normal, subnormal,
// zero, inf, NaN, out of binary32 range) and on doubles near binary32
// rounding ties.  fail[0]: d2f_rn, fail[1]: f2d_exact.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
__global__ void k_selftest_conv(unsigned long long n, unsigned long long* fail) {
    unsigned long long f0 = 0, f1 = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        unsigned long long r = mix64(i);
        double x;
        switch (i & 3ULL) {
        case 0:  // any pattern
            x = __longlong_as_double((long long)r);
            break;
        case 1: {  // exponent within binary32 range
            unsigned long long e = 1023ULL - 130ULL + ((r >> 52) % 262ULL);
            x = __longlong_as_double((long long)((r & 0x800fffffffffffffULL) | (e << 52)));
            break;
        }
        case 2: {  // near ties: low 29 mantissa bits around the half-way point
            unsigned long long e = 1023ULL - 60ULL + ((r >> 52) % 120ULL);
            unsigned long long m = (r & 0x000fffffe0000000ULL) | (0x10000000ULL + ((r >> 7) & 3ULL) - 1ULL);
            x = __longlong_as_double((long long)((r & 0x8000000000000000ULL) | (e << 52) | m));
            break;
        }
        default: {  // binary32 subnormal range, underflow to zero, and its ties
            unsigned long long e = 1023ULL - 185ULL + ((r >> 52) % 62ULL);
            unsigned long long m = r & 0x000fffffffffffffULL;
            if ((r >> 9) & 1ULL) m &= ~((1ULL << ((r >> 10) % 50ULL)) - 1ULL);
            x = __longlong_as_double((long long)((r & 0x8000000000000000ULL) | (e << 52) | m));
            break;
        }
        }
        float a = d2f_rn(x), b = __double2float_rn(x);
        bool same = (a != a && b != b) || (__float_as_uint(a) == __float_as_uint(b));
        f0 += same ? 0 : 1;
        float g = __uint_as_float((unsigned)(r >> 17));
        double c = f2d_exact(g), d = (double)g;
        bool same2 = (c != c && d != d) || (__double_as_longlong(c) == __double_as_longlong(d));
        f1 += same2 ? 0 : 1;
    }
    if (f0) atomicAdd(fail, f0);
    if (f1) atomicAdd(fail + 1, f1);
}

__global__ void k_aos_to_soa(const double* __restrict__ xyz, int32_t n, double* __restrict__ x,
                             double* __restrict__ y, double* __restrict__ z) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = xyz[3 * (int64_t)i];
    y[i] = xyz[3 * (int64_t)i + 1];
    z[i] = xyz[3 * (int64_t)i + 2];
}
__global__ void k_scatter_vertices(const int32_t* __restrict__ ids, const double* __restrict__ xyz,
                                   const uint8_t* __restrict__ rnd, int32_t n, int32_t nv,
                                   double* __restrict__ x, double* __restrict__ y,
                                   double* __restrict__ z, uint8_t* __restrict__ rounded,
                                   int* __restrict__ bad) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t v = ids[i];
    if (v < 0 || v >= nv) {
        atomicExch(bad, 1);
        return;
    }
    x[v] = xyz[3 * (int64_t)i];
    y[v] = xyz[3 * (int64_t)i + 1];
    z[v] = xyz[3 * (int64_t)i + 2];
    if (rnd) rounded[v] = rnd[i];
}
__global__ void k_check_ids(const int32_t* __restrict__ ids, int64_t n, int32_t lim,
                            int* __restrict__ bad) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t v = ids[i];
    if (v < 0 || v >= lim) atomicExch(bad, 1);
}

int amips_recheck_scratch(tw_ctx* c, int64_t n, int parts, char** out) {
    void* p = nullptr;
    int st = ensure(c, 9, (size_t)parts * amips_recheck_scratch_bytes(n), &p);
    *out = static_cast<char*>(p);
    return st;
}

}  // namespace tw

using namespace tw;

static double __longlong_as_double_host(unsigned long long b) {
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
}

namespace {

constexpr int kNumPipe = 3;
// point chunks of the host-buffer envelope call: the copy of one chunk
// overlaps the test of the one before, and the last chunk's test is the tail
constexpr size_t kPointChunkBytes = 96ull << 20;

struct Guard {
    explicit Guard(int dev) { cudaSetDevice(dev); }
};

// scratch slot layout: pipelines use slots [0, kNumPipe), their point-ordering
// scratch [3, 3 + kNumPipe), misc uses 6, 7
int sync_status(tw_ctx* c, const char* where) {
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->copy_in);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->copy_out);
    if (e != cudaSuccess) return cuda_fail(c, e, where);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, where);
    // device-side error word: read and clear
    unsigned long long err = 0;
    e = cudaMemcpy(&err, c->counters + kCntError, sizeof(err), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, where);
    if (err) {
        cudaMemset(c->counters + kCntError, 0, sizeof(err));
        std::string m = std::string(where) + ": ";
        if (err & 1ULL) m += "surface traversal exceeded its bounds (corrupt tree); ";
        if (err & 2ULL) m += "a face exceeds the per-row sample bound (4e6 samples); ";
        if (err & 4ULL) m += "a boundary star without a boundary surface; ";
        if (err & 8ULL) m += "smoothing face list exceeded its capacity; ";
        return fail(c, TW_ERR_ARG, m);
    }
    return TW_OK;
}

cudaStream_t pipe_stream(tw_ctx* c, int k) {
    if (k == 0) return c->stream;
    return k == 1 ? c->copy_in : c->copy_out;
}

// Device address of page-locked host memory (nullptr for pageable or device
// memory, or nullptr in): on this system the GPU reads and writes it over the
// coherent CPU-GPU link, so kernels can stream it without staging copies.
const void* pinned_device_ptr(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost) return nullptr;
    return a.devicePointer;
}

int64_t chunk_len(int64_t n, size_t bytes_per_item, size_t chunk_bytes = 96ull << 20) {
    // ~chunk_bytes of inputs+outputs per chunk, at least 64k items
    int64_t c = (int64_t)(chunk_bytes / std::max<size_t>(bytes_per_item, 1));
    c = std::max<int64_t>(c, 65536);
    c = (c + 255) & ~int64_t(255);
    return std::min(c, std::max<int64_t>(n, 1));
}

}  // namespace

extern "C" {

int tw_ctx_create(int device, size_t hbm_budget_bytes, tw_ctx** out) {
    if (!out) return TW_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return TW_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) return TW_ERR_ARG;
    Guard g(device);
    tw_ctx* c = new tw_ctx();
    c->device = device;
    c->budget = hbm_budget_bytes;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return TW_ERR_CUDA;
    }
    for (auto& ev : c->ev) cudaEventCreate(&ev);
    void* cnt = nullptr;
    if (dev_alloc(c, kNumCounters * sizeof(unsigned long long), &cnt) != TW_OK) {
        tw_ctx_destroy(c);
        return TW_ERR_OOM;
    }
    c->counters = (unsigned long long*)cnt;
    cudaMemset(c->counters, 0, kNumCounters * sizeof(unsigned long long));
    *out = c;
    return TW_OK;
}

int tw_ctx_destroy(tw_ctx* c) {
    if (!c) return TW_ERR_ARG;
    Guard g(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->copy_in) cudaStreamSynchronize(c->copy_in);
    if (c->copy_out) cudaStreamSynchronize(c->copy_out);
    for (auto& S : c->surf) free_surface(c, S);
    dev_free(c, c->vx, sizeof(double) * (size_t)c->nv);
    dev_free(c, c->vy, sizeof(double) * (size_t)c->nv);
    dev_free(c, c->vz, sizeof(double) * (size_t)c->nv);
    dev_free(c, c->rounded, (size_t)c->nv);
    for (auto& b : c->scratch) dev_free(c, b.ptr, b.cap);
    dev_free(c, c->counters, kNumCounters * sizeof(unsigned long long));
    for (auto& ev : c->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto& ev : c->time_ev)
        if (ev) cudaEventDestroy(ev);
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->copy_in) cudaStreamDestroy(c->copy_in);
    if (c->copy_out) cudaStreamDestroy(c->copy_out);
    delete c;
    return TW_OK;
}

const char* tw_last_error(const tw_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

int tw_set_params(tw_ctx* c, double eps_2, double sampling_dist, int newton_max_step,
                  int newton_max_it) {
    if (!c) return TW_ERR_ARG;
    if (!(eps_2 >= 0.0) || !(sampling_dist >= 0.0) || newton_max_step < 0 || newton_max_it < 0)
        return fail(c, TW_ERR_ARG, "tw_set_params: negative or NaN parameter");
    c->eps2 = eps_2;
    c->sampling_dist = sampling_dist;
    c->newton_max_step = newton_max_step;
    c->newton_max_it = newton_max_it;
    Guard g(c->device);
    for (auto& S : c->surf) {
        int st = build_env_grid(c, S, eps_2, c->grid_cell, c->stream);
        if (st != TW_OK) return st;
    }
    return TW_OK;
}

int tw_set_tuning(tw_ctx* c, int knob, double value) {
    if (!c) return TW_ERR_ARG;
    Guard g(c->device);
    if (knob == TW_TUNE_GRID_CELL) {
        if (!(value >= 0.05 && value <= 64.0)) return fail(c, TW_ERR_ARG, "grid cell factor");
        c->grid_cell = value;
        for (auto& S : c->surf) {
            int st = build_env_grid(c, S, c->eps2, c->grid_cell, c->stream);
            if (st != TW_OK) return st;
        }
        return TW_OK;
    }
    if (knob == TW_TUNE_BIN_CELL) {
        if (!(value == 0.0 || (value >= 0.05 && value <= 64.0)))
            return fail(c, TW_ERR_ARG, "bin cell factor: 0 or 0.05..64");
        c->bin_cell = value;
        for (auto& S : c->surf) {
            int st = build_env_grid(c, S, c->eps2, c->grid_cell, c->stream);
            if (st != TW_OK) return st;
        }
        return TW_OK;
    }
    if (knob == TW_TUNE_SORT_POINTS) {
        if (!(value == 0.0 || value == 1.0 || (value >= 2.0 && value <= 8.0 &&
                                               value == (double)(int)value)))
            return fail(c, TW_ERR_ARG, "sort_points: 0, 1 or 2..8");
        c->sort_points = (int)value;
        return TW_OK;
    }
    if (knob == TW_TUNE_POINT_BLOCK) {
        if (!(value == 128.0 || value == 256.0 || value == 384.0 || value == 768.0))
            return fail(c, TW_ERR_ARG, "point_block: 128, 256, 384 or 768");
        c->point_block = (int)value;
        return TW_OK;
    }
    if (knob == TW_TUNE_TIME_KERNELS) {
        c->time_kernels = value != 0.0;
        c->time_count = 0;
        return TW_OK;
    }
    return fail(c, TW_ERR_ARG, "unknown tuning knob");
}

int tw_kernel_times(tw_ctx* c, float* ms, int max, int* count) {
    if (!c || !count || (max > 0 && !ms)) return TW_ERR_ARG;
    Guard g(c->device);
    const int n = std::min(c->time_count, tw_ctx::kTimeRing);
    const int first = c->time_count - n;
    int k = 0;
    for (int i = first; i < c->time_count && k < max; ++i, ++k) {
        const int r = i % tw_ctx::kTimeRing;
        cudaError_t e = cudaEventSynchronize(c->time_ev[2 * r + 1]);
        if (e != cudaSuccess) return cuda_fail(c, e, "tw_kernel_times");
        cudaEventElapsedTime(ms + k, c->time_ev[2 * r], c->time_ev[2 * r + 1]);
    }
    *count = k;
    c->time_count = 0;
    return TW_OK;
}

int tw_stream(tw_ctx* c, void** s) {
    if (!c || !s) return TW_ERR_ARG;
    *s = (void*)c->stream;
    return TW_OK;
}

int tw_synchronize(tw_ctx* c) {
    if (!c) return TW_ERR_ARG;
    Guard g(c->device);
    return sync_status(c, "tw_synchronize");
}

int tw_memory_used(const tw_ctx* c, size_t* bytes) {
    if (!c || !bytes) return TW_ERR_ARG;
    *bytes = c->used;
    return TW_OK;
}

int tw_set_precision(tw_ctx* c, int mode) {
    if (!c) return TW_ERR_ARG;
    if (mode != TW_PRECISION_FP64 && mode != TW_PRECISION_FP32_CERTIFIED)
        return fail(c, TW_ERR_ARG, "tw_set_precision: unknown mode");
    c->precision = mode;
    return TW_OK;
}

int tw_set_energy_form(tw_ctx* c, int form) {
    if (!c) return TW_ERR_ARG;
    if (form != TW_ENERGY_FORM_REFERENCE && form != TW_ENERGY_FORM_CLOSED)
        return fail(c, TW_ERR_ARG, "tw_set_energy_form: unknown form");
    c->energy_form = form;
    return TW_OK;
}

int tw_get_stats(tw_ctx* c, tw_stats* out) {
    if (!c || !out) return TW_ERR_ARG;
    Guard g(c->device);
    int st = sync_status(c, "tw_get_stats");
    if (st != TW_OK) return st;
    unsigned long long h[kNumCounters] = {};
    cudaError_t e = cudaMemcpy(h, c->counters, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_get_stats");
    out->exact_orientations = h[kCntExactOrient];
    out->env_queries = h[kCntEnvQueries];
    out->env_facet_tests = h[kCntEnvFacetTests];
    out->env_facet_fp64 = h[kCntEnvFp64];
    out->amips_tets = h[kCntAmipsTets];
    out->amips_fp64 = h[kCntAmipsFp64];
    out->env_warp_fallbacks = h[kCntEnvWarpFallback];
    return TW_OK;
}

int tw_reset_stats(tw_ctx* c) {
    if (!c) return TW_ERR_ARG;
    Guard g(c->device);
    int st = sync_status(c, "tw_reset_stats");
    if (st != TW_OK) return st;
    const int keep[] = {kCntExactOrient, kCntEnvQueries, kCntEnvFacetTests, kCntEnvFp64,
                        kCntAmipsTets, kCntAmipsFp64, kCntEnvWarpFallback};
    for (int k : keep) cudaMemset(c->counters + k, 0, sizeof(unsigned long long));
    return sync_status(c, "tw_reset_stats");
}

// ---- AMIPS -------------------------------------------------------------------
int tw_amips_soa_device(tw_ctx* c, const double* T, int64_t n, int mode, double* E, double* J,
                        double* H, uint8_t* flip) {
    if (!c || n < 0 || (n > 0 && !T)) return TW_ERR_ARG;
    if (mode != TW_ENERGY_RAW && mode != TW_ENERGY_QUALITY)
        return fail(c, TW_ERR_ARG, "tw_amips: unknown mode");
    Guard g(c->device);
    if (c->precision == TW_PRECISION_FP32_CERTIFIED) {
        char* rs = nullptr;
        int st = amips_recheck_scratch(c, n, 1, &rs);
        if (st != TW_OK) return st;
        launch_amips_soa_cert(T, n, mode, E, J, H, flip, c->counters, rs, c->stream,
                              c->energy_form);
    } else {
        launch_amips_soa(T, n, mode, E, J, H, flip, c->counters + kCntExactOrient, c->stream,
                         c->energy_form);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_amips_soa_device");
    return TW_OK;
}

int tw_amips_soa(tw_ctx* c, const double* T, int64_t n, int mode, double* E, double* J,
                 double* H, uint8_t* flip) {
    if (!c || n < 0 || (n > 0 && !T)) return TW_ERR_ARG;
    if (mode != TW_ENERGY_RAW && mode != TW_ENERGY_QUALITY)
        return fail(c, TW_ERR_ARG, "tw_amips: unknown mode");
    if (n == 0) return TW_OK;
    Guard g(c->device);
    // every buffer page-locked: the kernel streams them in place
    {
        const void* dT = pinned_device_ptr(T);
        const void* dE = pinned_device_ptr(E);
        const void* dJ = pinned_device_ptr(J);
        const void* dH = pinned_device_ptr(H);
        const void* dF = pinned_device_ptr(flip);
        if (dT && (!E || dE) && (!J || dJ) && (!H || dH) && (!flip || dF)) {
            if (c->precision == TW_PRECISION_FP32_CERTIFIED) {
                char* rs = nullptr;
                int st = amips_recheck_scratch(c, n, 1, &rs);
                if (st != TW_OK) return st;
                launch_amips_soa_cert((const double*)dT, n, mode, (double*)dE, (double*)dJ,
                                      (double*)dH, (uint8_t*)dF, c->counters, rs, c->stream,
                                      c->energy_form);
            } else
                launch_amips_soa((const double*)dT, n, mode, (double*)dE, (double*)dJ,
                                 (double*)dH, (uint8_t*)dF, c->counters + kCntExactOrient,
                                 c->stream, c->energy_form);
            return sync_status(c, "tw_amips_soa");
        }
    }
    const size_t per = 96 + (E ? 8 : 0) + (J ? 24 : 0) + (H ? 72 : 0) + (flip ? 1 : 0);
    const int64_t C = chunk_len(n, per);
    double* dT[kNumPipe];
    double *dE[kNumPipe], *dJ[kNumPipe], *dH[kNumPipe];
    uint8_t* dF[kNumPipe];
    for (int k = 0; k < kNumPipe; ++k) {
        void* p = nullptr;
        int st = ensure(c, k, (size_t)C * per + 1024, &p);
        if (st != TW_OK) return st;
        char* q = (char*)p;
        dT[k] = (double*)q; q += 96 * (size_t)C;
        dE[k] = E ? (double*)q : nullptr; q += E ? 8 * (size_t)C : 0;
        dJ[k] = J ? (double*)q : nullptr; q += J ? 24 * (size_t)C : 0;
        dH[k] = H ? (double*)q : nullptr; q += H ? 72 * (size_t)C : 0;
        dF[k] = flip ? (uint8_t*)q : nullptr;
    }
    char* rs = nullptr;
    if (c->precision == TW_PRECISION_FP32_CERTIFIED) {
        int st = amips_recheck_scratch(c, C, kNumPipe, &rs);
        if (st != TW_OK) return st;
    }
    int64_t chunk = 0;
    for (int64_t i0 = 0; i0 < n; i0 += C, ++chunk) {
        const int k = (int)(chunk % kNumPipe);
        cudaStream_t s = pipe_stream(c, k);
        const int64_t len = std::min<int64_t>(C, n - i0);
        for (int comp = 0; comp < 12; ++comp)
            cudaMemcpyAsync(dT[k] + comp * len, T + comp * n + i0, 8 * (size_t)len,
                            cudaMemcpyHostToDevice, s);
        if (c->precision == TW_PRECISION_FP32_CERTIFIED)
            launch_amips_soa_cert(dT[k], len, mode, dE[k], dJ[k], dH[k], dF[k], c->counters,
                                  rs + k * amips_recheck_scratch_bytes(C), s, c->energy_form);
        else
            launch_amips_soa(dT[k], len, mode, dE[k], dJ[k], dH[k], dF[k],
                             c->counters + kCntExactOrient, s, c->energy_form);
        if (E) cudaMemcpyAsync(E + i0, dE[k], 8 * (size_t)len, cudaMemcpyDeviceToHost, s);
        if (J)
            for (int comp = 0; comp < 3; ++comp)
                cudaMemcpyAsync(J + comp * n + i0, dJ[k] + comp * len, 8 * (size_t)len,
                                cudaMemcpyDeviceToHost, s);
        if (H)
            for (int comp = 0; comp < 9; ++comp)
                cudaMemcpyAsync(H + comp * n + i0, dH[k] + comp * len, 8 * (size_t)len,
                                cudaMemcpyDeviceToHost, s);
        if (flip) cudaMemcpyAsync(flip + i0, dF[k], (size_t)len, cudaMemcpyDeviceToHost, s);
    }
    return sync_status(c, "tw_amips_soa");
}

// ---- resident mesh -------------------------------------------------------------
int tw_mesh_upload(tw_ctx* c, const double* xyz, int32_t nv, const uint8_t* rounded) {
    if (!c || nv < 0 || (nv > 0 && !xyz)) return TW_ERR_ARG;
    Guard g(c->device);
    dev_free(c, c->vx, 8 * (size_t)c->nv);
    dev_free(c, c->vy, 8 * (size_t)c->nv);
    dev_free(c, c->vz, 8 * (size_t)c->nv);
    dev_free(c, c->rounded, (size_t)c->nv);
    c->vx = c->vy = c->vz = nullptr;
    c->rounded = nullptr;
    c->nv = 0;
    if (nv == 0) return TW_OK;
    void *x, *y, *z, *r, *tmp;
    int st;
    if ((st = dev_alloc(c, 8 * (size_t)nv, &x)) != TW_OK) return st;
    if ((st = dev_alloc(c, 8 * (size_t)nv, &y)) != TW_OK) return st;
    if ((st = dev_alloc(c, 8 * (size_t)nv, &z)) != TW_OK) return st;
    if ((st = dev_alloc(c, (size_t)nv, &r)) != TW_OK) return st;
    c->vx = (double*)x;
    c->vy = (double*)y;
    c->vz = (double*)z;
    c->rounded = (uint8_t*)r;
    c->nv = nv;
    if ((st = ensure(c, 6, 24 * (size_t)nv, &tmp)) != TW_OK) return st;
    cudaMemcpyAsync(tmp, xyz, 24 * (size_t)nv, cudaMemcpyHostToDevice, c->stream);
    k_aos_to_soa<<<(nv + 255) / 256, 256, 0, c->stream>>>((const double*)tmp, nv, c->vx, c->vy,
                                                          c->vz);
    if (rounded)
        cudaMemcpyAsync(c->rounded, rounded, (size_t)nv, cudaMemcpyHostToDevice, c->stream);
    else
        cudaMemsetAsync(c->rounded, 1, (size_t)nv, c->stream);
    return sync_status(c, "tw_mesh_upload");
}

int tw_mesh_update_vertices(tw_ctx* c, const int32_t* ids, const double* xyz,
                            const uint8_t* rounded, int32_t n) {
    if (!c || n < 0 || (n > 0 && (!ids || !xyz))) return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    if (n == 0) return TW_OK;
    Guard g(c->device);
    void* tmp;
    const size_t bytes = 4 * (size_t)n + 24 * (size_t)n + (size_t)n + 64;
    int st = ensure(c, 6, bytes, &tmp);
    if (st != TW_OK) return st;
    char* q = (char*)tmp;
    int32_t* dids = (int32_t*)q; q += ((4 * (size_t)n + 15) & ~size_t(15));
    double* dxyz = (double*)q; q += 24 * (size_t)n;
    uint8_t* drnd = rounded ? (uint8_t*)q : nullptr;
    int* bad = (int*)(c->counters + 7);
    cudaMemsetAsync(bad, 0, sizeof(int), c->stream);
    cudaMemcpyAsync(dids, ids, 4 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dxyz, xyz, 24 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
    if (rounded) cudaMemcpyAsync(drnd, rounded, (size_t)n, cudaMemcpyHostToDevice, c->stream);
    k_scatter_vertices<<<(n + 255) / 256, 256, 0, c->stream>>>(dids, dxyz, drnd, n, c->nv, c->vx,
                                                               c->vy, c->vz, c->rounded, bad);
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_mesh_update_vertices");
    if (st != TW_OK) return st;
    if (hbad) return fail(c, TW_ERR_ARG, "vertex id out of range");
    return TW_OK;
}

int tw_tet_quality_device(tw_ctx* c, const int32_t* tets, int64_t n, double* energy,
                          uint8_t* flip, uint8_t* needs_host) {
    if (!c || n < 0 || (n > 0 && !tets)) return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    Guard g(c->device);
    launch_tet_quality_idx(tets, n, c->vx, c->vy, c->vz, c->rounded, energy, flip, needs_host,
                           c->counters, c->stream, c->energy_form);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_tet_quality_device");
    return TW_OK;
}

int tw_tet_quality(tw_ctx* c, const int32_t* tets, int64_t n, double* energy, uint8_t* flip,
                   uint8_t* needs_host) {
    if (!c || n < 0 || (n > 0 && !tets)) return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    if (n == 0) return TW_OK;
    Guard g(c->device);
    void* p;
    const size_t bytes = 16 * (size_t)n + 8 * (size_t)n + 2 * (size_t)n + 256;
    int st = ensure(c, 7, bytes, &p);
    if (st != TW_OK) return st;
    char* q = (char*)p;
    int32_t* dt = (int32_t*)q; q += 16 * (size_t)n;
    double* dE = (double*)q; q += 8 * (size_t)n;
    uint8_t* dF = (uint8_t*)q; q += (size_t)n;
    uint8_t* dN = (uint8_t*)q;
    int* bad = (int*)(c->counters + 7);
    cudaMemsetAsync(bad, 0, sizeof(int), c->stream);
    cudaMemsetAsync(c->counters + 1, 0, sizeof(unsigned long long), c->stream);
    cudaMemcpyAsync(dt, tets, 16 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
    k_check_ids<<<(unsigned)((4 * n + 255) / 256), 256, 0, c->stream>>>(dt, 4 * n, c->nv, bad);
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_tet_quality");
    if (st != TW_OK) return st;
    if (hbad) return fail(c, TW_ERR_ARG, "tet vertex id out of range");
    launch_tet_quality_idx(dt, n, c->vx, c->vy, c->vz, c->rounded, energy ? dE : nullptr,
                           flip ? dF : nullptr, dN, c->counters, c->stream, c->energy_form);
    unsigned long long unrounded = 0;
    cudaMemcpyAsync(&unrounded, c->counters + 1, sizeof(unrounded), cudaMemcpyDeviceToHost,
                    c->stream);
    if (energy) cudaMemcpyAsync(energy, dE, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    if (flip) cudaMemcpyAsync(flip, dF, (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    if (needs_host) cudaMemcpyAsync(needs_host, dN, (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_tet_quality");
    if (st != TW_OK) return st;
    return unrounded ? TW_NEEDS_EXACT_HOST : TW_OK;
}

// ---- envelope -------------------------------------------------------------------
int tw_surface_upload(tw_ctx* c, const double* V, int32_t nv, const int32_t* F, int32_t nf,
                      int which) {
    if (!c || nv < 0 || nf < 0 || (nv > 0 && !V) || (nf > 0 && !F)) return TW_ERR_ARG;
    if (which != TW_SURFACE_INPUT && which != TW_SURFACE_BOUNDARY)
        return fail(c, TW_ERR_ARG, "unknown surface");
    Guard g(c->device);
    if (nf == 0) {
        free_surface(c, c->surf[which]);
        return TW_OK;
    }
    void *dV = nullptr, *dF = nullptr;
    int st = dev_alloc(c, 24 * (size_t)nv, &dV);
    if (st != TW_OK) return st;
    st = dev_alloc(c, 12 * (size_t)nf, &dF);
    if (st != TW_OK) {
        dev_free(c, dV, 24 * (size_t)nv);
        return st;
    }
    cudaMemcpyAsync(dV, V, 24 * (size_t)nv, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dF, F, 12 * (size_t)nf, cudaMemcpyHostToDevice, c->stream);
    st = build_surface(c, c->surf[which], (const double*)dV, nv, (const int32_t*)dF, nf, c->stream);
    dev_free(c, dV, 24 * (size_t)nv);
    dev_free(c, dF, 12 * (size_t)nf);
    if (st == TW_OK) st = build_env_grid(c, c->surf[which], c->eps2, c->grid_cell, c->stream);
    return st;
}

int tw_envelope_points_device(tw_ctx* c, const double* P, int64_t n, int which, uint8_t* out) {
    if (!c || n < 0 || (n > 0 && (!P || !out))) return TW_ERR_ARG;
    if (which != TW_SURFACE_INPUT && which != TW_SURFACE_BOUNDARY) return TW_ERR_ARG;
    if (c->surf[which].nf == 0) return fail(c, TW_ERR_NO_SURFACE, "no surface uploaded");
    Guard g(c->device);
    void* sort = nullptr;
    int st = ensure(c, 3, env_sort_scratch_bytes(n, c->sort_points), &sort);
    if (st != TW_OK) return st;
    cudaEvent_t eb = nullptr, ee = nullptr;
    if (c->time_kernels) {
        const int k = c->time_count % tw_ctx::kTimeRing;
        if (!c->time_ev[2 * k]) {
            cudaEventCreate(&c->time_ev[2 * k]);
            cudaEventCreate(&c->time_ev[2 * k + 1]);
        }
        eb = c->time_ev[2 * k];
        ee = c->time_ev[2 * k + 1];
        ++c->time_count;
    }
    launch_env_points(c->surf[which], P, n, c->eps2, out, c->precision, c->counters,
                      c->sort_points ? sort : nullptr, c->sort_points, c->point_block, c->stream,
                      eb, ee);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_envelope_points_device");
    return TW_OK;
}

int tw_envelope_points(tw_ctx* c, const double* P, int64_t n, int which, uint8_t* out) {
    if (!c || n < 0 || (n > 0 && (!P || !out))) return TW_ERR_ARG;
    if (which != TW_SURFACE_INPUT && which != TW_SURFACE_BOUNDARY) return TW_ERR_ARG;
    if (c->surf[which].nf == 0) return fail(c, TW_ERR_NO_SURFACE, "no surface uploaded");
    if (n == 0) return TW_OK;
    Guard g(c->device);
    const int64_t C = chunk_len(n, 25, kPointChunkBytes);
    double* dP[kNumPipe];
    uint8_t* dO[kNumPipe];
    void* dS[kNumPipe];
    for (int k = 0; k < kNumPipe; ++k) {
        void* p;
        int st = ensure(c, k, 25 * (size_t)C + 256, &p);
        if (st != TW_OK) return st;
        dP[k] = (double*)p;
        dO[k] = (uint8_t*)p + 24 * (size_t)C;
        st = ensure(c, 3 + k, env_sort_scratch_bytes(C, c->sort_points), &dS[k]);
        if (st != TW_OK) return st;
    }
    int64_t chunk = 0;
    for (int64_t i0 = 0; i0 < n; i0 += C, ++chunk) {
        const int k = (int)(chunk % kNumPipe);
        cudaStream_t s = pipe_stream(c, k);
        const int64_t len = std::min<int64_t>(C, n - i0);
        cudaMemcpyAsync(dP[k], P + 3 * i0, 24 * (size_t)len, cudaMemcpyHostToDevice, s);
        launch_env_points(c->surf[which], dP[k], len, c->eps2, dO[k], c->precision, c->counters,
                          c->sort_points ? dS[k] : nullptr, c->sort_points, c->point_block, s);
        cudaMemcpyAsync(out + i0, dO[k], (size_t)len, cudaMemcpyDeviceToHost, s);
    }
    return sync_status(c, "tw_envelope_points");
}

int tw_envelope_faces_device(tw_ctx* c, const double* tris, int64_t n, uint8_t* out) {
    if (!c || n < 0 || (n > 0 && (!tris || !out))) return TW_ERR_ARG;
    if (c->surf[TW_SURFACE_INPUT].nf == 0) return fail(c, TW_ERR_NO_SURFACE, "no surface uploaded");
    if (!(c->sampling_dist > 0.0)) return fail(c, TW_ERR_ARG, "sampling_dist must be > 0");
    Guard g(c->device);
    launch_env_faces(c->surf[TW_SURFACE_INPUT], tris, n, c->eps2, c->sampling_dist, out,
                     c->precision, c->counters, c->stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_envelope_faces_device");
    return TW_OK;
}

int tw_envelope_faces(tw_ctx* c, const double* tris, int64_t n, uint8_t* out) {
    if (!c || n < 0 || (n > 0 && (!tris || !out))) return TW_ERR_ARG;
    if (c->surf[TW_SURFACE_INPUT].nf == 0) return fail(c, TW_ERR_NO_SURFACE, "no surface uploaded");
    if (!(c->sampling_dist > 0.0)) return fail(c, TW_ERR_ARG, "sampling_dist must be > 0");
    if (n == 0) return TW_OK;
    Guard g(c->device);
    void* p;
    int st = ensure(c, 7, 73 * (size_t)n + 256, &p);
    if (st != TW_OK) return st;
    double* dT = (double*)p;
    uint8_t* dO = (uint8_t*)p + 72 * (size_t)n;
    cudaMemcpyAsync(dT, tris, 72 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
    launch_env_faces(c->surf[TW_SURFACE_INPUT], dT, n, c->eps2, c->sampling_dist, dO,
                     c->precision, c->counters, c->stream);
    cudaMemcpyAsync(out, dO, (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    return sync_status(c, "tw_envelope_faces");
}

int tw_sample_triangle(tw_ctx* c, const double* tri9, double sd, double* out, int64_t cap,
                       int64_t* count) {
    if (!c || !tri9 || !count || cap < 0 || (cap > 0 && !out) || !(sd > 0.0)) return TW_ERR_ARG;
    Guard g(c->device);
    void* p;
    int st = ensure(c, 7, 72 + 8 + 24 * (size_t)cap + 256, &p);
    if (st != TW_OK) return st;
    double* dt = (double*)p;
    int64_t* dc = (int64_t*)((char*)p + 72);
    double* dout = (double*)((char*)p + 80);
    cudaMemcpyAsync(dt, tri9, 72, cudaMemcpyHostToDevice, c->stream);
    launch_sample_triangle(dt, sd, dout, cap, dc, c->stream);
    cudaMemcpyAsync(count, dc, 8, cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_sample_triangle");
    if (st != TW_OK) return st;
    if (*count < 0) return fail(c, TW_ERR_ARG, "face exceeds the per-row sample bound (4e6)");
    int64_t k = std::min(*count, cap);
    if (k > 0) {
        cudaMemcpy(out, dout, 24 * (size_t)k, cudaMemcpyDeviceToHost);
        return sync_status(c, "tw_sample_triangle");
    }
    return TW_OK;
}

// ---- Newton stars -----------------------------------------------------------------
int tw_newton_stars(tw_ctx* c, const int32_t* star_off, const int32_t* tets, const int32_t* centers,
                    int32_t nstars, double* out, uint8_t* moved) {
    if (!c || nstars < 0 || (nstars > 0 && (!star_off || !tets || !centers || !out || !moved)))
        return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    if (nstars == 0) return TW_OK;
    for (int32_t i = 0; i < nstars; ++i)
        if (star_off[i + 1] < star_off[i]) return fail(c, TW_ERR_ARG, "star offsets decrease");
    if (star_off[0] != 0) return fail(c, TW_ERR_ARG, "star offsets must start at 0");
    const int64_t nt = star_off[nstars];
    Guard g(c->device);
    void* p;
    const size_t bytes = 4 * (size_t)(nstars + 1) + 16 * (size_t)nt + 4 * (size_t)nstars +
                         24 * (size_t)nstars + (size_t)nstars + 1024;
    int st = ensure(c, 7, bytes, &p);
    if (st != TW_OK) return st;
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    char* q = (char*)p;
    int32_t* doff = (int32_t*)q; q += align(4 * (size_t)(nstars + 1));
    int32_t* dt = (int32_t*)q; q += align(16 * (size_t)nt);
    int32_t* dc = (int32_t*)q; q += align(4 * (size_t)nstars);
    double* dout = (double*)q; q += align(24 * (size_t)nstars);
    uint8_t* dm = (uint8_t*)q;
    int* bad = (int*)(c->counters + 7);
    cudaMemsetAsync(bad, 0, sizeof(int), c->stream);
    cudaMemcpyAsync(doff, star_off, 4 * (size_t)(nstars + 1), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dt, tets, 16 * (size_t)nt, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dc, centers, 4 * (size_t)nstars, cudaMemcpyHostToDevice, c->stream);
    if (nt > 0)
        k_check_ids<<<(unsigned)((4 * nt + 255) / 256), 256, 0, c->stream>>>(dt, 4 * nt, c->nv, bad);
    k_check_ids<<<(unsigned)((nstars + 255) / 256), 256, 0, c->stream>>>(dc, nstars, c->nv, bad);
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_newton_stars");
    if (st != TW_OK) return st;
    if (hbad) return fail(c, TW_ERR_ARG, "star vertex id out of range");
    launch_newton_stars_shape(c->newton_shape, c->vx, c->vy, c->vz, doff, dt, dc, nstars,
                              c->newton_max_step, c->newton_max_it, dout, dm, c->stream, c->energy_form);
    cudaMemcpyAsync(out, dout, 24 * (size_t)nstars, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(moved, dm, (size_t)nstars, cudaMemcpyDeviceToHost, c->stream);
    return sync_status(c, "tw_newton_stars");
}

// ---- nearest facet -------------------------------------------------------------------
int tw_nearest_points_device(tw_ctx* c, const double* P, int64_t n, int which, double* Q,
                             double* D, int32_t* F) {
    if (!c || n < 0 || (n > 0 && !P)) return TW_ERR_ARG;
    if (which != TW_SURFACE_INPUT && which != TW_SURFACE_BOUNDARY) return TW_ERR_ARG;
    if (c->surf[which].nf == 0) return fail(c, TW_ERR_NO_SURFACE, "no surface uploaded");
    Guard g(c->device);
    launch_nearest_points(c->surf[which], c->eps2, P, n, Q, D, F, c->counters, c->stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_nearest_points_device");
    return TW_OK;
}

int tw_nearest_points(tw_ctx* c, const double* P, int64_t n, int which, double* Q, double* D,
                      int32_t* F) {
    if (!c || n < 0 || (n > 0 && !P)) return TW_ERR_ARG;
    if (which != TW_SURFACE_INPUT && which != TW_SURFACE_BOUNDARY) return TW_ERR_ARG;
    if (c->surf[which].nf == 0) return fail(c, TW_ERR_NO_SURFACE, "no surface uploaded");
    if (n == 0) return TW_OK;
    Guard g(c->device);
    void* p;
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t bytes = align(24 * (size_t)n) * 2 + align(8 * (size_t)n) + align(4 * (size_t)n);
    int st = ensure(c, 7, bytes, &p);
    if (st != TW_OK) return st;
    char* q = (char*)p;
    double* dP = (double*)q; q += align(24 * (size_t)n);
    double* dQ = (double*)q; q += align(24 * (size_t)n);
    double* dD = (double*)q; q += align(8 * (size_t)n);
    int32_t* dF = (int32_t*)q;
    cudaMemcpyAsync(dP, P, 24 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
    launch_nearest_points(c->surf[which], c->eps2, dP, n, Q ? dQ : nullptr, D ? dD : nullptr,
                          F ? dF : nullptr, c->counters, c->stream);
    if (Q) cudaMemcpyAsync(Q, dQ, 24 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    if (D) cudaMemcpyAsync(D, dD, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    if (F) cudaMemcpyAsync(F, dF, 4 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    return sync_status(c, "tw_nearest_points");
}

// ---- smoothing pass ----------------------------------------------------------------
}  // extern "C"

namespace tw {
int smooth_scratch(tw_ctx* c, int32_t nstars, int64_t ntets, SmoothScratch& S) {
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    const int64_t cap = 3 * ntets;
    if (cap > (int64_t)INT32_MAX) return fail(c, TW_ERR_TOO_LARGE, "smoothing batch too large");
    const size_t ns = (size_t)nstars, nc = (size_t)cap;
    const size_t bytes = align(24 * ns) + 2 * align(4 * ns) + align(72 * nc) + align(nc) + 256;
    void* p;
    int st = ensure(c, 8, bytes, &p);
    if (st != TW_OK) return st;
    char* q = (char*)p;
    S.pnew = (double*)q; q += align(24 * ns);
    S.face_base = (int32_t*)q; q += align(4 * ns);
    S.face_cnt = (int32_t*)q; q += align(4 * ns);
    S.faces = (double*)q; q += align(72 * nc);
    S.face_out = (uint8_t*)q; q += align(nc);
    S.face_count = (unsigned long long*)q;
    S.face_cap = cap;
    return TW_OK;
}

void smooth_launch(tw_ctx* c, const int32_t* off, const int32_t* tets, const uint8_t* ff,
                   const int32_t* cen, const uint8_t* kinds, int32_t nstars, bool any_surface,
                   double* out, uint8_t* status, const SmoothScratch& S) {
    launch_smooth_stage1(c->newton_shape, c->vx, c->vy, c->vz, off, tets, cen, kinds, nstars,
                         c->newton_max_step, c->newton_max_it, out, S.pnew, status, c->stream, c->energy_form);
    if (!any_surface) return;
    cudaMemsetAsync(S.face_count, 0, sizeof(unsigned long long), c->stream);
    launch_smooth_project(c->surf[TW_SURFACE_INPUT], c->surf[TW_SURFACE_BOUNDARY], c->eps2, kinds,
                          nstars,
                          status, S.pnew, c->counters, c->stream);
    launch_smooth_stage2(c->newton_shape, c->vx, c->vy, c->vz, off, tets, ff, cen, nstars, S.pnew,
                         status, S.faces, S.face_count, S.face_cap, S.face_base, S.face_cnt,
                         c->counters, c->stream, c->energy_form);
    launch_env_faces_dev(c->surf[TW_SURFACE_INPUT], S.faces, S.face_count, S.face_cap, c->eps2,
                         c->sampling_dist, S.face_out, c->precision, c->counters, c->stream);
    launch_smooth_finalize(nstars, S.face_base, S.face_cnt, S.face_out, S.pnew, out, status,
                           c->stream);
}
}  // namespace tw

extern "C" {

int tw_smooth_stars_device(tw_ctx* c, const int32_t* star_off, const int32_t* tets,
                           const uint8_t* face_flags, const int32_t* centers, const uint8_t* kinds,
                           int32_t nstars, int64_t ntets, double* out, uint8_t* status) {
    if (!c || nstars < 0 || ntets < 0 ||
        (nstars > 0 && (!star_off || !centers || !out || !status || (ntets > 0 && !tets))))
        return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    if (nstars == 0) return TW_OK;
    const bool any_surface = kinds != nullptr;
    if (any_surface && !face_flags) return fail(c, TW_ERR_ARG, "surface stars need face_flags");
    if (any_surface && c->surf[TW_SURFACE_INPUT].nf == 0)
        return fail(c, TW_ERR_NO_SURFACE, "no input surface uploaded");
    Guard g(c->device);
    SmoothScratch S;
    int st = smooth_scratch(c, nstars, ntets, S);
    if (st != TW_OK) return st;
    smooth_launch(c, star_off, tets, face_flags, centers, kinds, nstars, any_surface, out, status, S);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_smooth_stars_device");
    return TW_OK;
}

int tw_smooth_stars(tw_ctx* c, const int32_t* star_off, const int32_t* tets,
                    const uint8_t* face_flags, const int32_t* centers, const uint8_t* kinds,
                    int32_t nstars, double* out, uint8_t* status) {
    if (!c || nstars < 0 || (nstars > 0 && (!star_off || !tets || !centers || !out || !status)))
        return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    if (nstars == 0) return TW_OK;
    if (star_off[0] != 0) return fail(c, TW_ERR_ARG, "star offsets must start at 0");
    for (int32_t i = 0; i < nstars; ++i)
        if (star_off[i + 1] < star_off[i]) return fail(c, TW_ERR_ARG, "star offsets decrease");
    bool any_surface = false, any_boundary = false;
    if (kinds) {
        for (int32_t i = 0; i < nstars; ++i) {
            if (kinds[i] > TW_STAR_BOUNDARY) return fail(c, TW_ERR_ARG, "unknown star kind");
            any_surface = any_surface || kinds[i] != TW_STAR_INTERIOR;
            any_boundary = any_boundary || kinds[i] == TW_STAR_BOUNDARY;
        }
    }
    if (any_surface && !face_flags) return fail(c, TW_ERR_ARG, "surface stars need face_flags");
    if (any_surface && c->surf[TW_SURFACE_INPUT].nf == 0)
        return fail(c, TW_ERR_NO_SURFACE, "no input surface uploaded");
    if (any_boundary && c->surf[TW_SURFACE_BOUNDARY].nf == 0)
        return fail(c, TW_ERR_NO_SURFACE, "no boundary surface uploaded");
    const int64_t nt = star_off[nstars];
    Guard g(c->device);
    SmoothScratch S;
    int st = smooth_scratch(c, nstars, nt, S);
    if (st != TW_OK) return st;
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t ns = (size_t)nstars;
    const size_t bytes = align(4 * (ns + 1)) + align(16 * (size_t)nt) + align((size_t)nt) +
                         align(4 * ns) + align(ns) + align(24 * ns) + align(ns) + 256;
    void* p;
    st = ensure(c, 7, bytes, &p);
    if (st != TW_OK) return st;
    char* q = (char*)p;
    int32_t* doff = (int32_t*)q; q += align(4 * (ns + 1));
    int32_t* dt = (int32_t*)q; q += align(16 * (size_t)nt);
    uint8_t* dff = (uint8_t*)q; q += align((size_t)nt);
    int32_t* dc = (int32_t*)q; q += align(4 * ns);
    uint8_t* dk = (uint8_t*)q; q += align(ns);
    double* dout = (double*)q; q += align(24 * ns);
    uint8_t* dst = (uint8_t*)q; q += align(ns);
    int* bad = (int*)q;
    cudaMemsetAsync(bad, 0, sizeof(int), c->stream);
    cudaMemcpyAsync(doff, star_off, 4 * (ns + 1), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dt, tets, 16 * (size_t)nt, cudaMemcpyHostToDevice, c->stream);
    if (any_surface) cudaMemcpyAsync(dff, face_flags, (size_t)nt, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dc, centers, 4 * ns, cudaMemcpyHostToDevice, c->stream);
    if (kinds) cudaMemcpyAsync(dk, kinds, ns, cudaMemcpyHostToDevice, c->stream);
    if (nt > 0)
        k_check_ids<<<(unsigned)((4 * nt + 255) / 256), 256, 0, c->stream>>>(dt, 4 * nt, c->nv, bad);
    k_check_ids<<<(unsigned)((ns + 255) / 256), 256, 0, c->stream>>>(dc, nstars, c->nv, bad);
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_smooth_stars");
    if (st != TW_OK) return st;
    if (hbad) return fail(c, TW_ERR_ARG, "star vertex id out of range");
    smooth_launch(c, doff, dt, any_surface ? dff : nullptr, dc, kinds ? dk : nullptr, nstars,
                  any_surface, dout, dst, S);
    cudaMemcpyAsync(out, dout, 24 * ns, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(status, dst, ns, cudaMemcpyDeviceToHost, c->stream);
    return sync_status(c, "tw_smooth_stars");
}

// ---- energy sweeps -------------------------------------------------------------------
int tw_energy_stats(tw_ctx* c, const int32_t* tets, int64_t n, const uint8_t* locked,
                    double thres, double* avg, double* max_e, double* second_max,
                    int64_t* buckets) {
    if (!c || n < 0 || (n > 0 && !tets) || !avg || !max_e || !second_max || !buckets)
        return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    Guard g(c->device);
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    const int nb = energy_stats_blocks(n);
    const size_t bytes = align(16 * (size_t)n) + align((size_t)n) + align(16 * (size_t)nb) +
                         align(14 * 8) + align(8) + 256;
    void* p;
    int st = ensure(c, 7, bytes, &p);
    if (st != TW_OK) return st;
    char* q = (char*)p;
    int32_t* dt = (int32_t*)q; q += align(16 * (size_t)n);
    uint8_t* dl = (uint8_t*)q; q += align((size_t)n);
    void* dbs = q; q += align(16 * (size_t)nb);
    unsigned long long* dacc = (unsigned long long*)q; q += align(14 * 8);
    double* dsum = (double*)q;
    int* bad = (int*)(c->counters + kCntBad);
    cudaMemsetAsync(bad, 0, sizeof(int), c->stream);
    cudaMemsetAsync(dacc, 0, 14 * 8, c->stream);
    cudaMemsetAsync(dsum, 0, 8, c->stream);
    if (n > 0) {
        cudaMemcpyAsync(dt, tets, 16 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
        if (locked) cudaMemcpyAsync(dl, locked, (size_t)n, cudaMemcpyHostToDevice, c->stream);
        k_check_ids<<<(unsigned)((4 * n + 255) / 256), 256, 0, c->stream>>>(dt, 4 * n, c->nv, bad);
    }
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_energy_stats");
    if (st != TW_OK) return st;
    if (hbad) return fail(c, TW_ERR_ARG, "tet vertex id out of range");
    if (n > 0)
        launch_energy_stats(dt, n, c->vx, c->vy, c->vz, locked ? dl : nullptr, thres, dbs, dacc,
                            dsum, c->stream, c->energy_form);
    unsigned long long hacc[14];
    double hsum = 0.0;
    cudaMemcpyAsync(hacc, dacc, sizeof hacc, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(&hsum, dsum, 8, cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_energy_stats");
    if (st != TW_OK) return st;
    double a = hsum / (double)hacc[2];
    if (std::isinf(a)) a = 1e50;
    *avg = a;
    *max_e = hacc[0] ? __longlong_as_double_host(hacc[0]) : 0.0;
    *second_max = hacc[1] ? __longlong_as_double_host(hacc[1]) : 0.0;
    for (int k = 0; k < 11; ++k) buckets[k] = (int64_t)hacc[3 + k];
    return TW_OK;
}

int tw_dihedral_stats(tw_ctx* c, const int32_t* tets, int64_t n, const uint8_t* locked,
                      double* out, int64_t* counts, double* min_angle, double* max_angle) {
    if (!c || n < 0 || (n > 0 && !tets) || !out || !counts) return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    Guard g(c->device);
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    const int nb = energy_stats_blocks(n);
    const bool per = min_angle || max_angle;
    const size_t bytes = align(16 * (size_t)n) + align((size_t)n) + align(32 * (size_t)nb) +
                         align(9 * 8) + align(16) + (per ? 2 * align(8 * (size_t)n) : 0) + 256;
    void* p;
    int st = ensure(c, 7, bytes, &p);
    if (st != TW_OK) return st;
    char* q = (char*)p;
    int32_t* dt = (int32_t*)q; q += align(16 * (size_t)n);
    uint8_t* dl = (uint8_t*)q; q += align((size_t)n);
    void* dbs = q; q += align(32 * (size_t)nb);
    unsigned long long* dacc = (unsigned long long*)q; q += align(9 * 8);
    double* dsum = (double*)q; q += align(16);
    double* dmin = per ? (double*)q : nullptr; q += per ? align(8 * (size_t)n) : 0;
    double* dmax = per ? (double*)q : nullptr;
    int* bad = (int*)(c->counters + kCntBad);
    unsigned long long init[9] = {0};
    const double ten = 10.0;
    std::memcpy(&init[0], &ten, 8);
    cudaMemsetAsync(bad, 0, sizeof(int), c->stream);
    cudaMemcpyAsync(dacc, init, sizeof init, cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(dsum, 0, 16, c->stream);
    if (n > 0) {
        cudaMemcpyAsync(dt, tets, 16 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
        if (locked) cudaMemcpyAsync(dl, locked, (size_t)n, cudaMemcpyHostToDevice, c->stream);
        k_check_ids<<<(unsigned)((4 * n + 255) / 256), 256, 0, c->stream>>>(dt, 4 * n, c->nv, bad);
    }
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_dihedral_stats");
    if (st != TW_OK) return st;
    if (hbad) return fail(c, TW_ERR_ARG, "tet vertex id out of range");
    if (n > 0)
        launch_dihedral_stats(dt, n, c->vx, c->vy, c->vz, locked ? dl : nullptr, dmin, dmax, dbs,
                              dacc, dsum, c->stream);
    unsigned long long hacc[9];
    double hsum[2] = {0.0, 0.0};
    cudaMemcpyAsync(hacc, dacc, sizeof hacc, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(hsum, dsum, 16, cudaMemcpyDeviceToHost, c->stream);
    if (n > 0 && min_angle)
        cudaMemcpyAsync(min_angle, dmin, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    if (n > 0 && max_angle)
        cudaMemcpyAsync(max_angle, dmax, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_dihedral_stats");
    if (st != TW_OK) return st;
    const double cnt = (double)hacc[8];
    out[0] = __longlong_as_double_host(hacc[0]);
    out[1] = hsum[0] / cnt;
    out[2] = __longlong_as_double_host(hacc[1]);
    out[3] = hsum[1] / cnt;
    for (int k = 0; k < 6; ++k) counts[k] = (int64_t)hacc[2 + k];
    counts[6] = (int64_t)hacc[8];
    return TW_OK;
}

double tw_filter_energy(const int64_t* b, double thres, int* is_clean_up) {
    int64_t t1[10], t2[10];
    for (int i = 0; i < 10; ++i) {
        t1[i] = 0;
        t2[i] = 0;
        for (int k = 0; k <= i; ++k) t1[i] += b[k];
        for (int k = i + 1; k < 11; ++k) t2[i] += b[k];
    }
    if (is_clean_up) *is_clean_up = 0;
    if (t1[0] >= t2[0]) {
        if (is_clean_up) *is_clean_up = t2[5] > 0;
        return 8;
    }
    if (t1[8] <= t2[8]) return 1e11;
    double p = 10.0;
    for (int i = 0; i < 8; ++i, p *= 10.0)
        if (t1[i] < t2[i] && t1[i + 1] > t2[i + 1]) return thres - 1 + 5 * p;
    return 8;
}

// ---- edge-collapse checks ------------------------------------------------------------
int tw_collapse_check(tw_ctx* c, const int32_t* v12, const uint8_t* flags, const int32_t* off,
                      const int32_t* tets, const uint8_t* face_flags, int32_t n, int check_quality,
                      double soft_energy, uint8_t* result) {
    if (!c || n < 0 ||
        (n > 0 && (!v12 || !flags || !off || !tets || !face_flags || !result)))
        return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    if (n == 0) return TW_OK;
    if (off[0] != 0) return fail(c, TW_ERR_ARG, "star offsets must start at 0");
    bool any_surface = false, any_boundary = false;
    for (int32_t i = 0; i < n; ++i) {
        if (off[i + 1] < off[i]) return fail(c, TW_ERR_ARG, "star offsets decrease");
        any_surface = any_surface || (flags[i] & TW_CV_V1_SURFACE);
        any_boundary = any_boundary || (flags[i] & TW_CV_V1_BOUNDARY);
    }
    if (any_surface && c->surf[TW_SURFACE_INPUT].nf == 0)
        return fail(c, TW_ERR_NO_SURFACE, "no input surface uploaded");
    if (any_boundary && c->surf[TW_SURFACE_BOUNDARY].nf == 0)
        return fail(c, TW_ERR_NO_SURFACE, "no boundary surface uploaded");
    const int64_t nt = off[n];
    Guard g(c->device);
    SmoothScratch S;
    int st = smooth_scratch(c, n, nt, S);
    if (st != TW_OK) return st;
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t ns = (size_t)n;
    const size_t bytes = align(8 * ns) + align(ns) + align(4 * (ns + 1)) + align(16 * (size_t)nt) +
                         align((size_t)nt) + 2 * align(ns) + 256;
    void* p;
    st = ensure(c, 7, bytes, &p);
    if (st != TW_OK) return st;
    char* q = (char*)p;
    int32_t* dv = (int32_t*)q; q += align(8 * ns);
    uint8_t* dfl = (uint8_t*)q; q += align(ns);
    int32_t* doff = (int32_t*)q; q += align(4 * (ns + 1));
    int32_t* dt = (int32_t*)q; q += align(16 * (size_t)nt);
    uint8_t* dff = (uint8_t*)q; q += align((size_t)nt);
    uint8_t* dst = (uint8_t*)q; q += align(ns);
    uint8_t* ddeg = (uint8_t*)q; q += align(ns);
    int* bad = (int*)q;
    cudaMemsetAsync(bad, 0, sizeof(int), c->stream);
    cudaMemcpyAsync(dv, v12, 8 * ns, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dfl, flags, ns, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(doff, off, 4 * (ns + 1), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dt, tets, 16 * (size_t)nt, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dff, face_flags, (size_t)nt, cudaMemcpyHostToDevice, c->stream);
    if (nt > 0)
        k_check_ids<<<(unsigned)((4 * nt + 255) / 256), 256, 0, c->stream>>>(dt, 4 * nt, c->nv, bad);
    k_check_ids<<<(unsigned)((2 * ns + 255) / 256), 256, 0, c->stream>>>(dv, 2 * n, c->nv, bad);
    int hbad = 0;
    cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_collapse_check");
    if (st != TW_OK) return st;
    if (hbad) return fail(c, TW_ERR_ARG, "vertex id out of range");
    cudaMemsetAsync(S.face_count, 0, sizeof(unsigned long long), c->stream);
    launch_collapse_points(c->surf[TW_SURFACE_INPUT], c->surf[TW_SURFACE_BOUNDARY], c->eps2,
                           c->precision, c->vx, c->vy, c->vz, dv, dfl, n, dst, ddeg, c->counters,
                           c->stream);
    launch_collapse_stage(c->newton_shape, c->vx, c->vy, c->vz, doff, dt, dff, dv, dfl, ddeg, n,
                          check_quality, soft_energy, dst, S.faces, S.face_count, S.face_cap,
                          S.face_base, S.face_cnt, c->counters, c->stream, c->energy_form);
    if (any_surface)
        launch_env_faces_dev(c->surf[TW_SURFACE_INPUT], S.faces, S.face_count, S.face_cap,
                             c->eps2, c->sampling_dist, S.face_out, c->precision, c->counters,
                             c->stream);
    launch_collapse_finalize(n, S.face_base, S.face_cnt, S.face_out, dst, c->stream);
    cudaMemcpyAsync(result, dst, ns, cudaMemcpyDeviceToHost, c->stream);
    return sync_status(c, "tw_collapse_check");
}

int tw_swap_check(tw_ctx* c, const int32_t* v12, const int32_t* off, const int32_t* tets,
                  const int32_t* budget, int32_t n, uint8_t* result, int8_t* config,
                  uint8_t* spent) {
    if (!c || n < 0 || (n > 0 && (!v12 || !off || !tets || !result || !config || !spent)))
        return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    if (n == 0) return TW_OK;
    if (off[0] != 0) return fail(c, TW_ERR_ARG, "shell offsets must start at 0");
    for (int32_t i = 0; i < n; ++i)
        if (off[i + 1] < off[i]) return fail(c, TW_ERR_ARG, "shell offsets decrease");
    const int64_t nt = off[n];
    Guard g(c->device);
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t ns = (size_t)n;
    const size_t bytes = align(8 * ns) + align(4 * (ns + 1)) + align(16 * (size_t)nt) +
                         align(4 * ns) + 3 * align(ns) + 256;
    void* p;
    int st = ensure(c, 7, bytes, &p);
    if (st != TW_OK) return st;
    char* q = (char*)p;
    int32_t* dv = (int32_t*)q; q += align(8 * ns);
    int32_t* doff = (int32_t*)q; q += align(4 * (ns + 1));
    int32_t* dt = (int32_t*)q; q += align(16 * (size_t)nt);
    int32_t* db = (int32_t*)q; q += align(4 * ns);
    uint8_t* dres = (uint8_t*)q; q += align(ns);
    int8_t* dcfg = (int8_t*)q; q += align(ns);
    uint8_t* dsp = (uint8_t*)q;
    cudaMemsetAsync(c->counters + kCntUnrounded, 0, sizeof(unsigned long long), c->stream);
    cudaMemcpyAsync(dv, v12, 8 * ns, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(doff, off, 4 * (ns + 1), cudaMemcpyHostToDevice, c->stream);
    if (nt > 0) cudaMemcpyAsync(dt, tets, 16 * (size_t)nt, cudaMemcpyHostToDevice, c->stream);
    if (budget) cudaMemcpyAsync(db, budget, 4 * ns, cudaMemcpyHostToDevice, c->stream);
    launch_swap_check(c->vx, c->vy, c->vz, c->rounded, c->nv, dv, doff, dt, budget ? db : nullptr,
                      n, dres, dcfg, dsp, c->counters, c->stream, c->energy_form);
    cudaMemcpyAsync(result, dres, ns, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(config, dcfg, ns, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(spent, dsp, ns, cudaMemcpyDeviceToHost, c->stream);
    unsigned long long unrounded = 0;
    cudaMemcpyAsync(&unrounded, c->counters + kCntUnrounded, sizeof(unsigned long long),
                    cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_swap_check");
    if (st != TW_OK) return st;
    return unrounded ? TW_NEEDS_EXACT_HOST : TW_OK;
}

int tw_schedule_edges(tw_ctx* c, const int32_t* tets, int32_t ntets, const double* scale,
                      double ideal_weight, int op, int32_t* out_v12, int32_t cap, int32_t* n_sched,
                      int32_t* n_cand) {
    if (!c || ntets < 0 || cap < 0 || !n_sched || !n_cand || (ntets > 0 && !tets) ||
        (cap > 0 && !out_v12))
        return TW_ERR_ARG;
    if (op != TW_OP_SPLIT && op != TW_OP_COLLAPSE)
        return fail(c, TW_ERR_ARG, "tw_schedule_edges: unknown operator");
    if (!(ideal_weight >= 0.0)) return fail(c, TW_ERR_ARG, "tw_schedule_edges: ideal_weight");
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    *n_sched = *n_cand = 0;
    if (ntets == 0) return TW_OK;
    if ((int64_t)ntets * 12 > (int64_t)INT32_MAX)
        return fail(c, TW_ERR_TOO_LARGE, "tw_schedule_edges: too many tets");
    Guard g(c->device);
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t bytes = align(16 * (size_t)ntets) + align(8 * (size_t)c->nv) +
                         align(8 * (size_t)std::max(cap, 1)) + 256;
    void* p;
    int st = ensure(c, 6, bytes, &p);
    if (st != TW_OK) return st;
    char* q = (char*)p;
    int32_t* dt = (int32_t*)q; q += align(16 * (size_t)ntets);
    double* ds = (double*)q; q += align(8 * (size_t)c->nv);
    int32_t* dout = (int32_t*)q;
    cudaMemcpyAsync(dt, tets, 16 * (size_t)ntets, cudaMemcpyHostToDevice, c->stream);
    if (scale) cudaMemcpyAsync(ds, scale, 8 * (size_t)c->nv, cudaMemcpyHostToDevice, c->stream);
    int32_t ns = 0, nc = 0;
    st = schedule_edges(c, dt, ntets, scale ? ds : nullptr, ideal_weight, op, dout, cap, &ns, &nc,
                        c->stream);
    if (st != TW_OK) return st;
    const int32_t m = std::min(ns, cap);
    if (m > 0) cudaMemcpyAsync(out_v12, dout, 8 * (size_t)m, cudaMemcpyDeviceToHost, c->stream);
    st = sync_status(c, "tw_schedule_edges");
    if (st != TW_OK) return st;
    *n_sched = ns;
    *n_cand = nc;
    return TW_OK;
}

// ---- misc ---------------------------------------------------------------------------
int tw_newton_stars_device(tw_ctx* c, const int32_t* star_off, const int32_t* tets,
                           const int32_t* centers, int32_t nstars, double* out, uint8_t* moved) {
    if (!c || nstars < 0 || (nstars > 0 && (!star_off || !tets || !centers || !out || !moved)))
        return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    Guard g(c->device);
    launch_newton_stars_shape(c->newton_shape, c->vx, c->vy, c->vz, star_off, tets, centers,
                              nstars, c->newton_max_step, c->newton_max_it, out, moved, c->stream, c->energy_form);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_newton_stars_device");
    return TW_OK;
}

int tw_set_newton_shape(tw_ctx* c, int shape) {
    if (!c) return TW_ERR_ARG;
    if (shape < 0 || shape >= newton_num_shapes())
        return fail(c, TW_ERR_ARG, "tw_set_newton_shape: unknown shape");
    c->newton_shape = shape;
    return TW_OK;
}

}  // extern "C"

namespace {
// Times run(shape) for every launch shape (one untimed launch, then the best
// of two timed ones, CUDA events on the context stream), keeps the fastest
// shape in the context.
template <class Run>
int autotune_shapes(tw_ctx* c, const char* where, int* best_shape, float* ms_per_shape, Run run) {
    int best = c->newton_shape;
    float best_ms = 0.0f;
    for (int sh = 0; sh < newton_num_shapes(); ++sh) {
        float ms = 0.0f;
        for (int rep = 0; rep < 3; ++rep) {
            cudaEventRecord(c->ev[3], c->stream);
            run(sh);
            cudaEventRecord(c->ev[4], c->stream);
            cudaError_t e = cudaEventSynchronize(c->ev[4]);
            if (e != cudaSuccess) return cuda_fail(c, e, where);
            float t = 0.0f;
            cudaEventElapsedTime(&t, c->ev[3], c->ev[4]);
            if (rep == 1 || (rep == 2 && t < ms)) ms = t;
        }
        if (ms_per_shape) ms_per_shape[sh] = ms;
        if (sh == 0 || ms < best_ms) {
            best_ms = ms;
            best = sh;
        }
    }
    c->newton_shape = best;
    *best_shape = best;
    return sync_status(c, where);
}
}  // namespace

extern "C" {

int tw_newton_autotune_device(tw_ctx* c, const int32_t* star_off, const int32_t* tets,
                              const int32_t* centers, int32_t nstars, double* out, uint8_t* moved,
                              int* best_shape, float* ms_per_shape) {
    if (!c || !best_shape || nstars <= 0 || !star_off || !tets || !centers || !out || !moved)
        return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    Guard g(c->device);
    return autotune_shapes(c, "tw_newton_autotune_device", best_shape, ms_per_shape, [&](int sh) {
        launch_newton_stars_shape(sh, c->vx, c->vy, c->vz, star_off, tets, centers, nstars,
                                  c->newton_max_step, c->newton_max_it, out, moved, c->stream, c->energy_form);
    });
}

int tw_smooth_autotune_device(tw_ctx* c, const int32_t* star_off, const int32_t* tets,
                              const uint8_t* face_flags, const int32_t* centers,
                              const uint8_t* kinds, int32_t nstars, int64_t ntets, double* out,
                              uint8_t* status, int* best_shape, float* ms_per_shape) {
    if (!c || !best_shape || nstars <= 0 || ntets < 0 || !star_off || !tets || !centers || !out ||
        !status)
        return TW_ERR_ARG;
    if (!c->vx) return fail(c, TW_ERR_NO_MESH, "no resident mesh");
    const bool any_surface = kinds != nullptr;
    if (any_surface && !face_flags) return fail(c, TW_ERR_ARG, "surface stars need face_flags");
    if (any_surface && c->surf[TW_SURFACE_INPUT].nf == 0)
        return fail(c, TW_ERR_NO_SURFACE, "no input surface uploaded");
    Guard g(c->device);
    SmoothScratch S;
    int st = smooth_scratch(c, nstars, ntets, S);
    if (st != TW_OK) return st;
    const int keep = c->newton_shape;
    st = autotune_shapes(c, "tw_smooth_autotune_device", best_shape, ms_per_shape, [&](int sh) {
        c->newton_shape = sh;
        smooth_launch(c, star_off, tets, face_flags, centers, kinds, nstars, any_surface, out,
                      status, S);
    });
    if (st != TW_OK) c->newton_shape = keep;
    return st;
}

// ---- CUDA graphs of the context stream ---------------------------------------------
int tw_capture_begin(tw_ctx* c) {
    if (!c) return TW_ERR_ARG;
    Guard g(c->device);
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_capture_begin");
    return TW_OK;
}

int tw_capture_end(tw_ctx* c, void** graph_exec) {
    if (!c || !graph_exec) return TW_ERR_ARG;
    Guard g(c->device);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_capture_end");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_capture_end (instantiate)");
    *graph_exec = (void*)exec;
    return TW_OK;
}

int tw_graph_launch(tw_ctx* c, void* graph_exec) {
    if (!c || !graph_exec) return TW_ERR_ARG;
    Guard g(c->device);
    cudaError_t e = cudaGraphLaunch((cudaGraphExec_t)graph_exec, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "tw_graph_launch");
    return TW_OK;
}

int tw_graph_destroy(void* graph_exec) {
    if (!graph_exec) return TW_OK;
    return cudaGraphExecDestroy((cudaGraphExec_t)graph_exec) == cudaSuccess ? TW_OK : TW_ERR_CUDA;
}

int tw_host_alloc(size_t bytes, void** out) {
    if (!out) return TW_ERR_ARG;
    cudaError_t e = cudaMallocHost(out, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return TW_ERR_OOM;
    }
    return TW_OK;
}

int tw_host_free(void* p) {
    if (!p) return TW_OK;
    return cudaFreeHost(p) == cudaSuccess ? TW_OK : TW_ERR_CUDA;
}

int tw_self_test(tw_ctx* c, uint64_t samples, uint64_t* failures) {
    if (!c || !failures) return TW_ERR_ARG;
    Guard g(c->device);
    void* p;
    int st = ensure(c, 6, 64, &p);
    if (st != TW_OK) return st;
    cudaMemsetAsync(p, 0, 16, c->stream);
    k_selftest_conv<<<1024, 256, 0, c->stream>>>((unsigned long long)samples,
                                                 (unsigned long long*)p);
    cudaMemcpyAsync(failures, p, 16, cudaMemcpyDeviceToHost, c->stream);
    return sync_status(c, "tw_self_test");
}

int tw_self_test_wait(tw_ctx* c, int32_t limit, uint64_t* result) {
    if (!c || !result || limit < 1 || limit > (1 << 20)) return TW_ERR_ARG;
    Guard g(c->device);
    void* p;
    int st = ensure(c, 6, 256, &p);
    if (st != TW_OK) return st;
    const double src[2] = {1.5, 2.5};
    double* dsrc = (double*)p;
    unsigned long long* dout = (unsigned long long*)((char*)p + 128);
    cudaMemcpyAsync(dsrc, src, sizeof src, cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(dout, 0, 32, c->stream);
    launch_selftest_wait(dsrc, limit, dout, c->stream);
    cudaMemcpyAsync(result, dout, 32, cudaMemcpyDeviceToHost, c->stream);
    return sync_status(c, "tw_self_test_wait");
}

int tw_probe_peaks(tw_ctx* c, double* fp64_tflops, double* fp32_tflops) {
    if (!c || !fp64_tflops || !fp32_tflops) return TW_ERR_ARG;
    Guard g(c->device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    void* p;
    int st = ensure(c, 6, 64, &p);
    if (st != TW_OK) return st;
    const int blocks = sms * 8;
    const int it64 = 4096, it32 = 65536;
    float ms = 0.0f;
    double best64 = 0.0, best32 = 0.0;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(c->ev[0], c->stream);
        launch_fp64_probe((double*)p, it64, blocks, c->stream);
        cudaEventRecord(c->ev[1], c->stream);
        launch_fp32_probe((float*)p, it32, blocks, c->stream);
        cudaEventRecord(c->ev[2], c->stream);
        cudaEventSynchronize(c->ev[2]);
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
        double f64 = 2.0 * 8.0 * it64 * (double)blocks * 256.0 / (ms * 1e-3) / 1e12;
        cudaEventElapsedTime(&ms, c->ev[1], c->ev[2]);
        double f32 = 2.0 * 8.0 * it32 * (double)blocks * 256.0 / (ms * 1e-3) / 1e12;
        best64 = std::max(best64, f64);
        best32 = std::max(best32, f32);
    }
    *fp64_tflops = best64;
    *fp32_tflops = best32;
    return sync_status(c, "tw_probe_peaks");
}

}  // extern "C"

namespace tw {
int stream_status(tw_ctx* c, const char* where) { return sync_status(c, where); }
}  // namespace tw
