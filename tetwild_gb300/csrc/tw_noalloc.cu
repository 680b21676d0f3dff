// tw_noalloc.cu -- an AMIPS batch entry point that allocates nothing.
//
// tw_amips_soa stages its inputs and outputs in device buffers that the
// context allocates (and grows) with cudaMalloc.  Some callers cannot let a
// library allocate device memory:
//   - applications whose device memory is reserved up front by their own
//     allocator (a host program that hands all free HBM to its own pool at
//     start-up), where a late cudaMalloc fails or fragments that pool;
//   - callers that must not stall the device: cudaFree waits for all work on
//     the device, so a library that frees and re-allocates scratch per call
//     blocks every other stream of the process.
// tw_amips_soa_noalloc serves them.  Its scratch is one file-scope
// __device__ array of TW_NOALLOC_SCRATCH_BYTES (about 12.6 MiB), created when
// the library's device code is loaded on a GPU and held by every GPU that
// loads the library until the process exits.  The caller passes host
// inputs and outputs and a stream; the call copies in, runs the same
// k_amips_soa kernel as tw_amips_soa, copies out and waits for the stream.
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress (with that device current) and keeps it; make
// that first call before any stream capture.  Results are those of
// tw_amips_soa on a context in TW_PRECISION_FP64 with the default (reference)
// energy form.  An error that earlier work of the caller left pending is
// consumed on entry; every copy and the launch are checked as they are queued.  Every call on a
// device shares the one array and leaves the last call's contents in it:
// calls whose work overlaps on the GPU (from several host threads, or on
// several streams) race on it, so serialise them.
#include <mutex>

#include "tw_device.cuh"
#include "tw_internal.h"

namespace {

constexpr int64_t kMaxTets = TW_NOALLOC_MAX_TETS;
static_assert(kMaxTets % 256 == 0, "offsets below stay 256-byte aligned");

// Scratch layout, all offsets multiples of 256 bytes:
//   T [12][kMaxTets] f64 | E [kMaxTets] f64 | J [3][kMaxTets] f64 |
//   H [9][kMaxTets] f64 | flip [kMaxTets] u8 | exact-path counter (u64)
constexpr size_t kOffT = 0;
constexpr size_t kOffE = kOffT + 96 * (size_t)kMaxTets;
constexpr size_t kOffJ = kOffE + 8 * (size_t)kMaxTets;
constexpr size_t kOffH = kOffJ + 24 * (size_t)kMaxTets;
constexpr size_t kOffF = kOffH + 72 * (size_t)kMaxTets;
constexpr size_t kOffC = kOffF + (size_t)kMaxTets;
constexpr size_t kScratchBytes = kOffC + 256;
static_assert(kScratchBytes == TW_NOALLOC_SCRATCH_BYTES, "header and layout disagree");

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up once
// per device).  Returns nullptr on failure.
unsigned char* scratch_on_current_device(int dev) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return nullptr;
        }
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    return g_scratch_ptr[dev];
}

}  // namespace

extern "C" TW_API int tw_amips_soa_noalloc(const double* T, int64_t n, int mode, double* E,
                                           double* J, double* H, uint8_t* flip,
                                           void* cuda_stream) {
    if (n < 0 || (n > 0 && !T)) return TW_ERR_ARG;
    if (mode != TW_ENERGY_RAW && mode != TW_ENERGY_QUALITY) return TW_ERR_ARG;
    if (n > kMaxTets) return TW_ERR_TOO_LARGE;
    if (n == 0) return TW_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return TW_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) return TW_ERR_ARG;
    unsigned char* base = scratch_on_current_device(dev);
    if (!base) return TW_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    double* dT = reinterpret_cast<double*>(base + kOffT);
    double* dE = E ? reinterpret_cast<double*>(base + kOffE) : nullptr;
    double* dJ = J ? reinterpret_cast<double*>(base + kOffJ) : nullptr;
    double* dH = H ? reinterpret_cast<double*>(base + kOffH) : nullptr;
    uint8_t* dF = flip ? reinterpret_cast<uint8_t*>(base + kOffF) : nullptr;
    auto* counter = reinterpret_cast<unsigned long long*>(base + kOffC);
    // An error left pending by earlier work of the caller is not this call's:
    // consume it so that the checks below see only this call's own errors.
    cudaGetLastError();
    // Each step is checked as it is queued; on the first failure nothing more
    // is queued, the stream is drained (so no queued copy outlives the call)
    // and the call fails.
    cudaError_t e = cudaSuccess;
    auto step = [&](cudaError_t r) {
        if (e == cudaSuccess && r != cudaSuccess) e = r;
        return e == cudaSuccess;
    };
    // The counter keeps the previous call's value: it must start at zero.
    step(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s));
    for (int c = 0; c < 12 && e == cudaSuccess; ++c)
        step(cudaMemcpyAsync(dT + c * n, T + c * n, 8 * (size_t)n, cudaMemcpyHostToDevice, s));
    if (e == cudaSuccess) {
        tw::launch_amips_soa(dT, n, mode, dE, dJ, dH, dF, counter, s);
        step(cudaGetLastError());
    }
    if (E && e == cudaSuccess)
        step(cudaMemcpyAsync(E, dE, 8 * (size_t)n, cudaMemcpyDeviceToHost, s));
    for (int c = 0; J && c < 3 && e == cudaSuccess; ++c)
        step(cudaMemcpyAsync(J + c * n, dJ + c * n, 8 * (size_t)n, cudaMemcpyDeviceToHost, s));
    for (int c = 0; H && c < 9 && e == cudaSuccess; ++c)
        step(cudaMemcpyAsync(H + c * n, dH + c * n, 8 * (size_t)n, cudaMemcpyDeviceToHost, s));
    if (flip && e == cudaSuccess)
        step(cudaMemcpyAsync(flip, dF, (size_t)n, cudaMemcpyDeviceToHost, s));
    const cudaError_t es = cudaStreamSynchronize(s);
    step(es);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return TW_ERR_CUDA;
    }
    return TW_OK;
}
