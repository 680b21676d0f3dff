// tw_newton.cu -- damped Newton smoothing of independent one-ring stars.
//
// Restates VertexSmoother::NewtonsMethod (VertexSmoother.cpp:465-542),
// NewtonsUpdate (:627-702) and getNewEnergy (:544-625) of the default scalar
// build: per step, E/J/H summed over the star's tets in caller order (each
// tet rotated so the centre vertex comes first), X = QR(H)^-1 (H X0 - a J)
// with up to max_it halvings of a, each trial rejected if X is not finite,
// if a tet flips (exact orientation) or if the star energy (tets in stored
// order) does not strictly decrease; stop when |dE| < 1e-5.
// The 3x3 solve is Householder QR with column pivoting (Golub & Van Loan,
// Alg. 5.4.1), the same operations as the oracle's, standing in for Eigen's
// ColPivHouseholderQR (:492).
#include "tw_device.cuh"
#include "tw_internal.h"
#include "tw_star.cuh"

namespace tw {

__global__ void __launch_bounds__(128) k_newton_stars(const double* __restrict__ vx,
                                                      const double* __restrict__ vy,
                                                      const double* __restrict__ vz,
                                                      const int32_t* __restrict__ star_off,
                                                      const int4* __restrict__ tets,
                                                      const int32_t* __restrict__ centers,
                                                      int32_t nstars, int max_step, int max_it,
                                                      double* __restrict__ out,
                                                      uint8_t* __restrict__ moved, int form) {
    int32_t sid = blockIdx.x * blockDim.x + threadIdx.x;
    if (sid >= nstars) return;
    int32_t b = star_off[sid], e = star_off[sid + 1];
    StarView S{vx, vy, vz, tets + b, e - b, centers[sid], form};
    double pos[3] = {vx[S.v], vy[S.v], vz[S.v]};
    int is_moved = 0;
    double old_energy = 0.0, new_energy = 0.0, J[3], H[9];
    for (int step = 0; step < max_step; ++step) {
        if (!star_update(S, pos, old_energy, J, H)) break;
        double old_pf[3] = {pos[0], pos[1], pos[2]};
        double X0[3] = {pos[0], pos[1], pos[2]};
        double a = 1.0;
        bool step_taken = false;
        for (int it = 0; it < max_it; ++it) {
            double rhs[3], X[3];
            for (int i = 0; i < 3; ++i)
                rhs[i] = ((H[3 * i] * X0[0] + H[3 * i + 1] * X0[1]) + H[3 * i + 2] * X0[2]) - a * J[i];
            qr_solve3(H, rhs, X);
            if (!isfinite(X[0]) || !isfinite(X[1]) || !isfinite(X[2])) {
                a /= 2.0;
                continue;
            }
            pos[0] = X[0];
            pos[1] = X[1];
            pos[2] = X[2];
            if (star_flip(S, pos)) {
                pos[0] = old_pf[0];
                pos[1] = old_pf[1];
                pos[2] = old_pf[2];
                a /= 2.0;
                continue;
            }
            new_energy = star_new_energy(S, pos);
            if (new_energy >= old_energy || isinf(new_energy) || isnan(new_energy)) {
                pos[0] = old_pf[0];
                pos[1] = old_pf[1];
                pos[2] = old_pf[2];
                a /= 2.0;
                continue;
            }
            step_taken = true;
            break;
        }
        if (fabs(new_energy - old_energy) < 1e-5) step_taken = false;
        if (!step_taken) {
            is_moved = (step != 0);
            break;
        }
        is_moved = 1;
    }
    out[3 * (int64_t)sid] = pos[0];
    out[3 * (int64_t)sid + 1] = pos[1];
    out[3 * (int64_t)sid + 2] = pos[2];
    moved[sid] = (uint8_t)is_moved;
}

template <int G>
__global__ void __launch_bounds__(256) k_newton_group(const double* __restrict__ vx,
                                                      const double* __restrict__ vy,
                                                      const double* __restrict__ vz,
                                                      const int32_t* __restrict__ star_off,
                                                      const int4* __restrict__ tets,
                                                      const int32_t* __restrict__ centers,
                                                      int32_t nstars, int max_step, int max_it,
                                                      double* __restrict__ out,
                                                      uint8_t* __restrict__ moved, int form) {
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const unsigned gm = group_mask<G>(lane);
    const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t sid = gid; sid < nstars; sid += ngroups) {
        const int32_t b = star_off[sid], nt = star_off[sid + 1] - b;
        StarView S{vx, vy, vz, tets + b, nt, centers[sid], form};
        double pos[3] = {vx[S.v], vy[S.v], vz[S.v]};
        const int is_moved = newton_group_star<G>(S, pos, max_step, max_it, gl, gm);
        if (gl == 0) {
            out[3 * sid] = pos[0];
            out[3 * sid + 1] = pos[1];
            out[3 * sid + 2] = pos[2];
            moved[sid] = (uint8_t)is_moved;
        }
    }
}

template <int G>
__global__ void __launch_bounds__(256) k_smooth_stage1(
    const double* __restrict__ vx, const double* __restrict__ vy, const double* __restrict__ vz,
    const int32_t* __restrict__ star_off, const int4* __restrict__ tets,
    const int32_t* __restrict__ centers, const uint8_t* __restrict__ kinds, int32_t nstars,
    int max_step, int max_it, double* __restrict__ out, double* __restrict__ pnew,
    uint8_t* __restrict__ status, int form) {
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const unsigned gm = group_mask<G>(lane);
    const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t sid = gid; sid < nstars; sid += ngroups) {
        const int32_t b = star_off[sid], nt = star_off[sid + 1] - b;
        StarView S{vx, vy, vz, tets + b, nt, centers[sid], form};
        const double p0[3] = {vx[S.v], vy[S.v], vz[S.v]};
        double pos[3] = {p0[0], p0[1], p0[2]};
        const uint8_t kind = kinds ? kinds[sid] : (uint8_t)TW_STAR_INTERIOR;
        const bool surface = (kind == TW_STAR_SURFACE || kind == TW_STAR_BOUNDARY);
        uint8_t st;
        if (!star_positive<G>(S, p0, gl, gm)) {
            st = TW_SMOOTH_INVALID;
        } else if (!newton_group_star<G>(S, pos, max_step, max_it, gl, gm)) {
            st = TW_SMOOTH_NOT_MOVED;
        } else {
            st = surface ? kSmoothPendingProject : (uint8_t)TW_SMOOTH_MOVED;
        }
        if (gl == 0) {
            const bool moved = (st == TW_SMOOTH_MOVED);
            out[3 * sid] = moved ? pos[0] : p0[0];
            out[3 * sid + 1] = moved ? pos[1] : p0[1];
            out[3 * sid + 2] = moved ? pos[2] : p0[2];
            pnew[3 * sid] = pos[0];
            pnew[3 * sid + 1] = pos[1];
            pnew[3 * sid + 2] = pos[2];
            status[sid] = st;
        }
    }
}

template <int G>
__global__ void __launch_bounds__(256) k_smooth_stage2(
    const double* __restrict__ vx, const double* __restrict__ vy, const double* __restrict__ vz,
    const int32_t* __restrict__ star_off, const int4* __restrict__ tets,
    const uint8_t* __restrict__ face_flags, const int32_t* __restrict__ centers, int32_t nstars,
    const double* __restrict__ pnew, uint8_t* __restrict__ status, double* __restrict__ faces,
    unsigned long long* __restrict__ face_count, int64_t face_cap,
    int32_t* __restrict__ face_base, int32_t* __restrict__ face_cnt,
    unsigned long long* __restrict__ counters, int form) {
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const unsigned gm = group_mask<G>(lane);
    const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t sid = gid; sid < nstars; sid += ngroups) {
        if (status[sid] != kSmoothPendingProject) continue;  // uniform within the group
        const int32_t b = star_off[sid], nt = star_off[sid + 1] - b;
        StarView S{vx, vy, vz, tets + b, nt, centers[sid], form};
        const double p0[3] = {vx[S.v], vy[S.v], vz[S.v]};
        const double p[3] = {pnew[3 * sid], pnew[3 * sid + 1], pnew[3 * sid + 2]};
        // isFlip at the projected position (:374-378)
        if (!star_positive<G>(S, p, gl, gm)) {
            if (gl == 0) status[sid] = TW_SMOOTH_REJECT_FLIP;
            continue;
        }
        // max calTetQuality before and after (:379-386); max is exact in any order
        double old_max = 0.0, new_max = 0.0;
        for (int c0 = gl; c0 < nt; c0 += G) {
            double T[12];
            int4 tv = tet_at(S, c0);
            gather_tet(S, tv, 0, p0, T);
            old_max = fmax(old_max, positive_tet_quality(T, S.form));
            gather_tet(S, tv, 0, p, T);
            new_max = fmax(new_max, positive_tet_quality(T, S.form));
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            old_max = fmax(old_max, __shfl_xor_sync(gm, old_max, o, G));
            new_max = fmax(new_max, __shfl_xor_sync(gm, new_max, o, G));
        }
        if (!(new_max < old_max)) {
            if (gl == 0) status[sid] = TW_SMOOTH_REJECT_QUALITY;
            continue;
        }
        // one-ring surface faces (:314-326): the first occurrence of each
        // sorted triple; counted, then written at one reservation per star
        const uint8_t* ff = face_flags + b;
        int nmine = 0;
        for (int c0 = gl; c0 < nt; c0 += G) {
            int4 tv = tet_at(S, c0);
            uint8_t fl = __ldg(ff + c0);
            int32_t key[3];
            for (int j = 0; j < 4; ++j) nmine += first_surface_face(S, ff, c0, tv, fl, j, key);
        }
        int incl = nmine;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            int v = __shfl_up_sync(gm, incl, o, G);
            if (gl >= o) incl += v;
        }
        const int total = __shfl_sync(gm, incl, G - 1, G);
        unsigned long long base = 0;
        if (gl == 0 && total > 0) base = atomicAdd(face_count, (unsigned long long)total);
        base = __shfl_sync(gm, base, 0, G);
        if (total > 0 && base + (unsigned long long)total > (unsigned long long)face_cap) {
            if (gl == 0) {
                atomicOr(counters + kCntError, 8ULL);
                status[sid] = TW_SMOOTH_INVALID;
            }
            continue;
        }
        int64_t w = (int64_t)base + (incl - nmine);
        for (int c0 = gl; c0 < nt; c0 += G) {
            int4 tv = tet_at(S, c0);
            uint8_t fl = __ldg(ff + c0);
            for (int j = 0; j < 4; ++j) {
                int32_t key[3];
                if (!first_surface_face(S, ff, c0, tv, fl, j, key)) continue;
                // the face from the centre onward in the cyclic order of its
                // sorted triple (:427-432)
                const int kv = (key[0] == S.v) ? 0 : (key[1] == S.v) ? 1 : 2;
                const int32_t v1 = key[(kv + 1) % 3], v2 = key[(kv + 2) % 3];
                double* f = faces + 9 * w;
                f[0] = p[0];
                f[1] = p[1];
                f[2] = p[2];
                f[3] = __ldg(vx + v1);
                f[4] = __ldg(vy + v1);
                f[5] = __ldg(vz + v1);
                f[6] = __ldg(vx + v2);
                f[7] = __ldg(vy + v2);
                f[8] = __ldg(vz + v2);
                ++w;
            }
        }
        if (gl == 0) {
            face_base[sid] = (int32_t)base;
            face_cnt[sid] = total;
            status[sid] = kSmoothPendingEnvelope;
        }
    }
}

// ---------------------------------------------------------------------------
// Checks of candidate edge collapses v1 -> v2 (EdgeCollapser.cpp:284-446),
// G lanes per edge; the point-envelope checks ran before
// (launch_collapse_points) and left kCollapsePending where they passed.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool tet_has(int4 tv, int32_t v) {
    return tv.x == v || tv.y == v || tv.z == v || tv.w == v;
}

template <int G>
__global__ void __launch_bounds__(256) k_collapse_stage(
    const double* __restrict__ vx, const double* __restrict__ vy, const double* __restrict__ vz,
    const int32_t* __restrict__ off, const int4* __restrict__ tets,
    const uint8_t* __restrict__ face_flags, const int32_t* __restrict__ v12,
    const uint8_t* __restrict__ flags, const uint8_t* __restrict__ degenerate, int32_t n,
    int check_quality, double soft_energy, uint8_t* __restrict__ status,
    double* __restrict__ faces, unsigned long long* __restrict__ face_count, int64_t face_cap,
    int32_t* __restrict__ face_base, int32_t* __restrict__ face_cnt,
    unsigned long long* __restrict__ counters, int form) {
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const unsigned gm = group_mask<G>(lane);
    const int64_t gid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t e = gid; e < n; e += ngroups) {
        if (status[e] != kCollapsePending) continue;  // uniform within the group
        const int32_t b = off[e], nt = off[e + 1] - b;
        const int32_t v1 = v12[2 * e], v2 = v12[2 * e + 1];
        StarView S{vx, vy, vz, tets + b, nt, v1, form};
        const double p1[3] = {vx[v1], vy[v1], vz[v1]};
        const double p2[3] = {vx[v2], vy[v2], vz[v2]};
        const uint8_t fl = flags[e];
        const bool deg = degenerate[e] != 0;
        // isFlip of the new tets: those without v2, v1 moved onto v2 (:336-384)
        bool bad = false;
        for (int c0 = gl; c0 < nt; c0 += G) {
            const int4 tv = tet_at(S, c0);
            if (tet_has(tv, v2)) continue;
            double T[12];
            gather_tet(S, tv, 0, p2, T);
            bad = bad || (orient3d(T, T + 3, T + 6, T + 9) != 1);
        }
        if (__any_sync(gm, bad)) {
            if (gl == 0) status[e] = 1;  // FLIP
            continue;
        }
        // quality (:390-415): max over the old tets (stored quality) and the new
        if (check_quality) {
            double old_max = 0.0, new_max = 0.0;
            for (int c0 = gl; c0 < nt; c0 += G) {
                const int4 tv = tet_at(S, c0);
                double T[12];
                gather_tet(S, tv, 0, p1, T);
                old_max = fmax(old_max, quality_from(orient3d(T, T + 3, T + 6, T + 9),
                                                     amips_energy_f(T, S.form)));
                if (tet_has(tv, v2)) continue;
                gather_tet(S, tv, 0, p2, T);
                new_max = fmax(new_max, positive_tet_quality(T, S.form));
            }
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) {
                old_max = fmax(old_max, __shfl_xor_sync(gm, old_max, o, G));
                new_max = fmax(new_max, __shfl_xor_sync(gm, new_max, o, G));
            }
            if (soft_energy >= 0.0) old_max = soft_energy;
            if (fl & TW_CV_V1_UNROUNDED) new_max = 0.0;
            if (!deg && !(new_max <= old_max)) {
                if (gl == 0) status[e] = 2;  // QUALITY
                continue;
            }
        }
        if (!(fl & TW_CV_V1_SURFACE) || deg) {
            if (gl == 0) status[e] = 0;  // SUCCESS
            continue;
        }
        // isCollapsable_epsilon (:727-775): the surface faces through v1 as
        // sorted triples without repeats, those through v2 dropped, v1
        // replaced by v2 in place
        const uint8_t* ff = face_flags + b;
        int nmine = 0;
        for (int c0 = gl; c0 < nt; c0 += G) {
            const int4 tv = tet_at(S, c0);
            const uint8_t f8 = __ldg(ff + c0);
            for (int j = 0; j < 4; ++j) {
                int32_t key[3];
                if (!first_surface_face(S, ff, c0, tv, f8, j, key)) continue;
                nmine += (key[0] != v2 && key[1] != v2 && key[2] != v2);
            }
        }
        int incl = nmine;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            int v = __shfl_up_sync(gm, incl, o, G);
            if (gl >= o) incl += v;
        }
        const int total = __shfl_sync(gm, incl, G - 1, G);
        if (total == 0) {
            if (gl == 0) status[e] = 0;
            continue;
        }
        unsigned long long base = 0;
        if (gl == 0) base = atomicAdd(face_count, (unsigned long long)total);
        base = __shfl_sync(gm, base, 0, G);
        if (base + (unsigned long long)total > (unsigned long long)face_cap) {
            if (gl == 0) {
                atomicOr(counters + kCntError, 8ULL);
                status[e] = 3;
            }
            continue;
        }
        int64_t w = (int64_t)base + (incl - nmine);
        for (int c0 = gl; c0 < nt; c0 += G) {
            const int4 tv = tet_at(S, c0);
            const uint8_t f8 = __ldg(ff + c0);
            for (int j = 0; j < 4; ++j) {
                int32_t key[3];
                if (!first_surface_face(S, ff, c0, tv, f8, j, key)) continue;
                if (key[0] == v2 || key[1] == v2 || key[2] == v2) continue;
                double* f = faces + 9 * w;
                for (int k = 0; k < 3; ++k) {
                    if (key[k] == v1) {
                        f[3 * k] = p2[0];
                        f[3 * k + 1] = p2[1];
                        f[3 * k + 2] = p2[2];
                    } else {
                        f[3 * k] = __ldg(vx + key[k]);
                        f[3 * k + 1] = __ldg(vy + key[k]);
                        f[3 * k + 2] = __ldg(vz + key[k]);
                    }
                }
                ++w;
            }
        }
        if (gl == 0) {
            face_base[e] = (int32_t)base;
            face_cnt[e] = total;
            status[e] = kCollapsePendingEnvelope;
        }
    }
}

__global__ void k_collapse_finalize(int32_t n, const int32_t* __restrict__ face_base,
                                    const int32_t* __restrict__ face_cnt,
                                    const uint8_t* __restrict__ face_out,
                                    uint8_t* __restrict__ status) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (status[i] != kCollapsePendingEnvelope) continue;
        bool outside = false;
        const int32_t b = face_base[i], m = face_cnt[i];
        for (int32_t k = 0; k < m && !outside; ++k) outside = face_out[b + k] != 0;
        status[i] = outside ? 3 : 0;
    }
}

__global__ void k_smooth_finalize(int32_t nstars, const int32_t* __restrict__ face_base,
                                  const int32_t* __restrict__ face_cnt,
                                  const uint8_t* __restrict__ face_out,
                                  const double* __restrict__ pnew, double* __restrict__ out,
                                  uint8_t* __restrict__ status) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nstars; i += stride) {
        if (status[i] != kSmoothPendingEnvelope) continue;
        bool outside = false;
        const int32_t b = face_base[i], n = face_cnt[i];
        for (int32_t k = 0; k < n && !outside; ++k) outside = face_out[b + k] != 0;
        if (outside) {
            status[i] = TW_SMOOTH_REJECT_ENVELOPE;
        } else {
            out[3 * i] = pnew[3 * i];
            out[3 * i + 1] = pnew[3 * i + 1];
            out[3 * i + 2] = pnew[3 * i + 2];
            status[i] = TW_SMOOTH_MOVED;
        }
    }
}

// Launch shape of the fused step: lanes per star (8, 16, 32) and threads per
// block (64, 128, 256); variant 0 is the one-thread-per-star kernel.
struct NewtonShape {
    int group;
    int block;
};
static const NewtonShape kNewtonShapes[] = {{1, 128},  {8, 64},   {8, 128},  {8, 256},
                                            {16, 64},  {16, 128}, {16, 256}, {32, 64},
                                            {32, 128}, {32, 256}};
int newton_num_shapes() { return (int)(sizeof(kNewtonShapes) / sizeof(kNewtonShapes[0])); }
void newton_shape_info(int shape, int* group, int* block) {
    if (shape < 0 || shape >= newton_num_shapes()) shape = 5;
    *group = kNewtonShapes[shape].group;
    *block = kNewtonShapes[shape].block;
}

void launch_newton_stars_shape(int shape, const double* vx, const double* vy, const double* vz,
                               const int32_t* star_off, const int32_t* tets,
                               const int32_t* centers, int32_t nstars, int max_step, int max_it,
                               double* out, uint8_t* moved, cudaStream_t s, int form) {
    if (nstars <= 0) return;
    if (shape < 0 || shape >= newton_num_shapes()) shape = 5;
    const NewtonShape sh = kNewtonShapes[shape];
    const int4* t4 = reinterpret_cast<const int4*>(tets);
    if (sh.group == 1) {
        int grid = (nstars + sh.block - 1) / sh.block;
        k_newton_stars<<<grid, sh.block, 0, s>>>(vx, vy, vz, star_off, t4, centers, nstars,
                                                 max_step, max_it, out, moved, form);
        return;
    }
    const int64_t threads = (int64_t)nstars * sh.group;
    const int grid = grid_for(threads, sh.block, 2048 / sh.block);
    if (sh.group == 8)
        k_newton_group<8><<<grid, sh.block, 0, s>>>(vx, vy, vz, star_off, t4, centers, nstars,
                                                    max_step, max_it, out, moved, form);
    else if (sh.group == 16)
        k_newton_group<16><<<grid, sh.block, 0, s>>>(vx, vy, vz, star_off, t4, centers, nstars,
                                                     max_step, max_it, out, moved, form);
    else
        k_newton_group<32><<<grid, sh.block, 0, s>>>(vx, vy, vz, star_off, t4, centers, nstars,
                                                     max_step, max_it, out, moved, form);
}

// Smoothing kernels use the Newton shape's group size; shape 0 (one thread
// per star) runs them with 8 lanes.
static int smooth_group(int shape, int* block) {
    if (shape < 0 || shape >= newton_num_shapes()) shape = 5;
    NewtonShape sh = kNewtonShapes[shape];
    if (sh.group == 1) sh = NewtonShape{8, 128};
    *block = sh.block;
    return sh.group;
}

void launch_smooth_stage1(int shape, const double* vx, const double* vy, const double* vz,
                          const int32_t* star_off, const int32_t* tets, const int32_t* centers,
                          const uint8_t* kinds, int32_t nstars, int max_step, int max_it,
                          double* out, double* pnew, uint8_t* status, cudaStream_t s,
                          int form) {
    if (nstars <= 0) return;
    int block;
    const int G = smooth_group(shape, &block);
    const int grid = grid_for((int64_t)nstars * G, block, 2048 / block);
    const int4* t4 = reinterpret_cast<const int4*>(tets);
    if (G == 8)
        k_smooth_stage1<8><<<grid, block, 0, s>>>(vx, vy, vz, star_off, t4, centers, kinds, nstars,
                                                  max_step, max_it, out, pnew, status, form);
    else if (G == 16)
        k_smooth_stage1<16><<<grid, block, 0, s>>>(vx, vy, vz, star_off, t4, centers, kinds, nstars,
                                                   max_step, max_it, out, pnew, status, form);
    else
        k_smooth_stage1<32><<<grid, block, 0, s>>>(vx, vy, vz, star_off, t4, centers, kinds, nstars,
                                                   max_step, max_it, out, pnew, status, form);
}

void launch_smooth_stage2(int shape, const double* vx, const double* vy, const double* vz,
                          const int32_t* star_off, const int32_t* tets, const uint8_t* face_flags,
                          const int32_t* centers, int32_t nstars, const double* pnew,
                          uint8_t* status, double* faces, unsigned long long* face_count,
                          int64_t face_cap, int32_t* face_base, int32_t* face_cnt,
                          unsigned long long* counters, cudaStream_t s, int form) {
    if (nstars <= 0) return;
    int block;
    const int G = smooth_group(shape, &block);
    const int grid = grid_for((int64_t)nstars * G, block, 2048 / block);
    const int4* t4 = reinterpret_cast<const int4*>(tets);
    if (G == 8)
        k_smooth_stage2<8><<<grid, block, 0, s>>>(vx, vy, vz, star_off, t4, face_flags, centers,
                                                  nstars, pnew, status, faces, face_count, face_cap,
                                                  face_base, face_cnt, counters, form);
    else if (G == 16)
        k_smooth_stage2<16><<<grid, block, 0, s>>>(vx, vy, vz, star_off, t4, face_flags, centers,
                                                   nstars, pnew, status, faces, face_count, face_cap,
                                                   face_base, face_cnt, counters, form);
    else
        k_smooth_stage2<32><<<grid, block, 0, s>>>(vx, vy, vz, star_off, t4, face_flags, centers,
                                                   nstars, pnew, status, faces, face_count, face_cap,
                                                   face_base, face_cnt, counters, form);
}

void launch_smooth_finalize(int32_t nstars, const int32_t* face_base, const int32_t* face_cnt,
                            const uint8_t* face_out, const double* pnew, double* out,
                            uint8_t* status, cudaStream_t s) {
    if (nstars <= 0) return;
    const int block = 256;
    k_smooth_finalize<<<grid_for(nstars, block, 8), block, 0, s>>>(nstars, face_base, face_cnt,
                                                                   face_out, pnew, out, status);
}

void launch_collapse_stage(int shape, const double* vx, const double* vy, const double* vz,
                           const int32_t* off, const int32_t* tets, const uint8_t* face_flags,
                           const int32_t* v12, const uint8_t* flags, const uint8_t* degenerate,
                           int32_t n, int check_quality, double soft_energy, uint8_t* status,
                           double* faces, unsigned long long* face_count, int64_t face_cap,
                           int32_t* face_base, int32_t* face_cnt, unsigned long long* counters,
                           cudaStream_t s, int form) {
    if (n <= 0) return;
    int block;
    const int G = smooth_group(shape, &block);
    const int grid = grid_for((int64_t)n * G, block, 2048 / block);
    const int4* t4 = reinterpret_cast<const int4*>(tets);
#define TW_COLLAPSE_ARGS                                                                      \
    vx, vy, vz, off, t4, face_flags, v12, flags, degenerate, n, check_quality, soft_energy, status, \
        faces, face_count, face_cap, face_base, face_cnt, counters, form
    if (G == 8)
        k_collapse_stage<8><<<grid, block, 0, s>>>(TW_COLLAPSE_ARGS);
    else if (G == 16)
        k_collapse_stage<16><<<grid, block, 0, s>>>(TW_COLLAPSE_ARGS);
    else
        k_collapse_stage<32><<<grid, block, 0, s>>>(TW_COLLAPSE_ARGS);
#undef TW_COLLAPSE_ARGS
}

void launch_collapse_finalize(int32_t n, const int32_t* face_base, const int32_t* face_cnt,
                              const uint8_t* face_out, uint8_t* status, cudaStream_t s) {
    if (n <= 0) return;
    k_collapse_finalize<<<grid_for(n, 256, 8), 256, 0, s>>>(n, face_base, face_cnt, face_out,
                                                            status);
}

void launch_newton_stars(const double* vx, const double* vy, const double* vz,
                         const int32_t* star_off, const int32_t* tets, const int32_t* centers,
                         int32_t nstars, int max_step, int max_it, double* out, uint8_t* moved,
                         cudaStream_t s, int form) {
    launch_newton_stars_shape(5, vx, vy, vz, star_off, tets, centers, nstars, max_step, max_it, out,
                              moved, s, form);
}

}  // namespace tw
