// tw_swap.cu -- the checks of candidate edge removals (EdgeRemover::
// removeAnEdge_32 / _44 / _56, EdgeRemover.cpp:125-177, :277-369, :456-600),
// one candidate per thread.
//
// A candidate is the edge (v1, v2) and its shell, the k tets around it in the
// caller's order (old_t_ids); only the variant for k = 3, 4 or 5 applies.
// Each configuration's quality is the max of its tets' calTetQuality_AMIPS
// (getCheckQuality with use_energy_max, LocalOperations.cpp:575-603; State.h
// :53), the old one the max over the shell.  The steps, their order and the
// reference's early exits are those of the CPU oracle's two_swap_check,
// operation for operation (FP64 in the context's energy form, exact
// orientation), so every result is identical to it.
#include "tw_device.cuh"
#include "tw_internal.h"

namespace tw {
namespace {

struct SwapMesh {
    const double* vx;
    const double* vy;
    const double* vz;
    int form;
};

__device__ __forceinline__ void tet_replace(const int32_t* t, int32_t from, int32_t to,
                                            int32_t* o) {
    bool done = false;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const bool hit = !done && t[j] == from;   // the first occurrence (std::find)
        o[j] = hit ? to : t[j];
        done = done || hit;
    }
}
__device__ __forceinline__ bool tet_has(const int32_t* t, int32_t v) {
    return t[0] == v || t[1] == v || t[2] == v || t[3] == v;
}
__device__ __forceinline__ void tet_coords(const SwapMesh& M, const int32_t* t, double* T) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        T[3 * j] = __ldg(M.vx + t[j]);
        T[3 * j + 1] = __ldg(M.vy + t[j]);
        T[3 * j + 2] = __ldg(M.vz + t[j]);
    }
}
__device__ bool tets_flip(const SwapMesh& M, const int32_t* ts, int m) {
    for (int i = 0; i < m; ++i) {
        double T[12];
        tet_coords(M, ts + 4 * i, T);
        if (orient3d(T, T + 3, T + 6, T + 9) != 1) return true;
    }
    return false;
}
// calTetQuality_AMIPS (LocalOperations.cpp:862-884)
__device__ double tet_q(const SwapMesh& M, const int32_t* t) {
    double T[12];
    tet_coords(M, t, T);
    if (orient3d(T, T + 3, T + 6, T + 9) != 1) return kMaxEnergy;
    return quality_from(1, amips_energy_f(T, M.form));
}
__device__ __forceinline__ bool swap_better(double nq, double oq, int& budget, int& spent) {
    if (budget > 0) {
        --budget;
        ++spent;
        return nq <= oq;
    }
    return nq < oq;
}
// n12_v_ids / n12_t_ids of :278-303 and :457-481
__device__ bool swap_ring(const int32_t* shell, int N, int32_t v1, int32_t v2, int32_t* nv,
                          int* tid) {
    int32_t e[5][2];
    for (int i = 0; i < N; ++i) {
        int c = 0;
        for (int j = 0; j < 4; ++j) {
            const int32_t x = shell[4 * i + j];
            if (x != v1 && x != v2) {
                if (c == 2) return false;
                e[i][c++] = x;
            }
        }
        if (c != 2) return false;
    }
    bool visited[5] = {false, false, false, false, false};
    int m = 2, mt = 1;
    nv[0] = e[0][0];
    nv[1] = e[0][1];
    tid[0] = 0;
    visited[0] = true;
    for (int it = 0; it < N - 2; ++it) {
        for (int j = 0; j < N; ++j) {
            if (visited[j]) continue;
            if (e[j][0] == nv[m - 1]) {
                visited[j] = true;
                nv[m++] = e[j][1];
            } else if (e[j][1] == nv[m - 1]) {
                visited[j] = true;
                nv[m++] = e[j][0];
            }
            if (visited[j]) {
                tid[mt++] = j;
                break;
            }
        }
    }
    if (m != N) return false;
    for (int j = 0; j < N; ++j)
        if (!visited[j]) {
            tid[mt++] = j;
            break;
        }
    return mt == N;
}

__device__ int swap_check(const SwapMesh& M, const int32_t* shell, int k, int32_t v1, int32_t v2,
                          int budget, int& config, int& spent) {
    config = -1;
    spent = 0;
    if (k < 3 || k > 5) return TW_SWAP_SIZE;
    for (int i = 0; i < k; ++i)
        if (!tet_has(shell + 4 * i, v1) || !tet_has(shell + 4 * i, v2)) return TW_SWAP_SIZE;
    double oq = 0.0;
    for (int i = 0; i < k; ++i) {
        const double q = tet_q(M, shell + 4 * i);
        if (q > oq) oq = q;
    }
    int32_t nt[8];
    if (k == 3) {
        int32_t vv[2] = {0, 0};
        int c = 0;
        for (int j = 0; j < 4; ++j)
            if (shell[j] != v1 && shell[j] != v2) vv[c++] = shell[j];
        const int32_t* a = shell + 4;
        const int32_t* b = shell + 8;
        if (!tet_has(a, vv[0])) {
            a = shell + 8;
            b = shell + 4;
        }
        tet_replace(a, v1, vv[1], nt);
        tet_replace(b, v2, vv[0], nt + 4);
        if (tets_flip(M, nt, 2)) return TW_SWAP_FLIP;
        const double q0 = tet_q(M, nt), q1 = tet_q(M, nt + 4);
        double nq = 0.0;
        if (q0 > nq) nq = q0;
        if (q1 > nq) nq = q1;
        if (!swap_better(nq, oq, budget, spent)) return TW_SWAP_QUALITY;
        config = 0;
        return TW_SWAP_SUCCESS;
    }
    int32_t nv[5];
    int tid[5];
    if (!swap_ring(shell, k, v1, v2, nv, tid)) return TW_SWAP_SIZE;
    if (k == 4) {
        bool valid = false;
        for (int i = 0; i < 2; ++i) {
            int32_t ts[16];
            const int32_t a = nv[i], b = nv[2 + i];
            for (int j = 0; j < 4; ++j) {
                const int32_t* t = shell + 4 * j;
                if (tet_has(t, a))
                    tet_replace(t, v2, b, ts + 4 * j);
                else
                    tet_replace(t, v1, a, ts + 4 * j);
            }
            if (tets_flip(M, ts, 4)) continue;
            double nq = 0.0;
            for (int j = 0; j < 4; ++j) {
                const double q = tet_q(M, ts + 4 * j);
                if (q > nq) nq = q;
            }
            if (!swap_better(nq, oq, budget, spent)) return TW_SWAP_QUALITY;
            valid = true;
            oq = nq;
            config = i;
        }
        return valid ? TW_SWAP_SUCCESS : TW_SWAP_FLIP;
    }
    bool vvalid[5] = {true, true, true, true, true};
    double q1[5][2] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
    for (int i = 0; i < 5; ++i) {
        if (!vvalid[(i + 1) % 5] && !vvalid[(i + 4) % 5]) continue;
        const int32_t* t = shell + 4 * tid[i];
        tet_replace(t, v1, nv[(i + 4) % 5], nt);
        tet_replace(t, v2, nv[(i + 4) % 5], nt + 4);
        if (tets_flip(M, nt, 2)) {
            vvalid[(i + 1) % 5] = false;
            vvalid[(i + 4) % 5] = false;
            continue;
        }
        q1[i][0] = tet_q(M, nt);
        q1[i][1] = tet_q(M, nt + 4);
    }
    if (!(vvalid[0] || vvalid[1] || vvalid[2] || vvalid[3] || vvalid[4])) return TW_SWAP_FLIP;
    int sel = -1;
    bool tested = false;
    for (int i = 0; i < 5; ++i) {
        if (!vvalid[i]) continue;
        const int32_t* t = shell + 4 * tid[(i + 2) % 5];
        tet_replace(t, v1, nv[i], nt);
        tet_replace(t, v2, nv[i], nt + 4);
        if (tets_flip(M, nt, 2)) continue;
        tested = true;
        const double qs[6] = {tet_q(M, nt), tet_q(M, nt + 4), q1[(i + 1) % 5][0],
                              q1[(i + 4) % 5][0], q1[(i + 1) % 5][1], q1[(i + 4) % 5][1]};
        double nq = 0.0;
        for (int j = 0; j < 6; ++j)
            if (qs[j] > nq) nq = qs[j];
        if (!swap_better(nq, oq, budget, spent)) continue;
        oq = nq;
        sel = i;
    }
    if (sel < 0) return tested ? TW_SWAP_QUALITY : TW_SWAP_FLIP;
    config = sel;
    return TW_SWAP_SUCCESS;
}

__global__ void __launch_bounds__(128) k_swap_check(SwapMesh M, const uint8_t* __restrict__ rounded,
                                                    const int32_t* __restrict__ v12,
                                                    const int32_t* __restrict__ off,
                                                    const int32_t* __restrict__ tets,
                                                    const int32_t* __restrict__ budget, int32_t n,
                                                    int32_t nv, uint8_t* __restrict__ result,
                                                    int8_t* __restrict__ config,
                                                    uint8_t* __restrict__ spent,
                                                    unsigned long long* __restrict__ counters) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int32_t b = off[i], k = off[i + 1] - b;
        const int32_t v1 = v12[2 * i], v2 = v12[2 * i + 1];
        int cfg = -1, sp = 0;
        int res;
        int32_t shell[20];
        bool ids_ok = k >= 0 && v1 >= 0 && v1 < nv && v2 >= 0 && v2 < nv;
        bool all_rounded = true;
        for (int j = 0; j < 4 * k && j < 20 && ids_ok; ++j) {
            const int32_t v = __ldg(tets + 4 * (int64_t)b + j);
            ids_ok = v >= 0 && v < nv;
            shell[j] = v;
            if (ids_ok && rounded) all_rounded = all_rounded && __ldg(rounded + v) != 0;
        }
        if (!ids_ok) {
            atomicOr(counters + kCntError, 16ULL);
            res = TW_SWAP_SIZE;
        } else if (k < 3 || k > 5) {
            res = TW_SWAP_SIZE;
        } else if (!all_rounded) {
            res = TW_SWAP_NEEDS_HOST;
            atomicAdd(counters + kCntUnrounded, 1ULL);
        } else {
            res = swap_check(M, shell, k, v1, v2, budget ? budget[i] : 0, cfg, sp);
        }
        result[i] = (uint8_t)res;
        config[i] = (int8_t)cfg;
        spent[i] = (uint8_t)sp;
    }
}

}  // namespace

void launch_swap_check(const double* vx, const double* vy, const double* vz,
                       const uint8_t* rounded, int32_t nv, const int32_t* v12, const int32_t* off,
                       const int32_t* tets, const int32_t* budget, int32_t n, uint8_t* result,
                       int8_t* config, uint8_t* spent, unsigned long long* counters,
                       cudaStream_t s, int form) {
    if (n <= 0) return;
    const SwapMesh M{vx, vy, vz, form};
    k_swap_check<<<grid_for(n, 128, 8), 128, 0, s>>>(M, rounded, v12, off, tets, budget, n, nv,
                                                     result, config, spent, counters);
}

}  // namespace tw
