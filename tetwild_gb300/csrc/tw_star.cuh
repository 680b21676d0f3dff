// tw_star.cuh -- device routines of one-ring stars used by the Newton,
// smoothing and collapse kernels (tw_newton.cu):
// the 3x3 solve, the star view and gathers, NewtonsMethod for G lanes, the
// inversion and quality checks and the one-ring surface faces.
#pragma once

#include "tw_device.cuh"
#include "tw_internal.h"

namespace tw {

__device__ __forceinline__ void qr_solve3(const double* Hm, const double* bvec, double* x) {
    double R[3][3], c[3];
    int perm[3] = {0, 1, 2};
    for (int i = 0; i < 3; ++i) {
        c[i] = bvec[i];
        for (int j = 0; j < 3; ++j) R[i][j] = Hm[3 * i + j];
    }
    for (int k = 0; k < 3; ++k) {
        int p = k;
        double best = -1.0;
        for (int j = k; j < 3; ++j) {
            double nrm = 0.0;
            for (int i = k; i < 3; ++i) nrm = nrm + R[i][j] * R[i][j];
            if (nrm > best) {
                best = nrm;
                p = j;
            }
        }
        if (p != k) {
            for (int i = 0; i < 3; ++i) {
                double t = R[i][k];
                R[i][k] = R[i][p];
                R[i][p] = t;
            }
            int t = perm[k];
            perm[k] = perm[p];
            perm[p] = t;
        }
        if (k == 2) break;
        double xn = 0.0;
        for (int i = k; i < 3; ++i) xn = xn + R[i][k] * R[i][k];
        xn = sqrt(xn);
        if (xn == 0.0) continue;
        double alpha = (R[k][k] > 0.0) ? -xn : xn;
        double v[3] = {0.0, 0.0, 0.0};
        for (int i = k; i < 3; ++i) v[i] = R[i][k];
        v[k] = v[k] - alpha;
        double vv = 0.0;
        for (int i = k; i < 3; ++i) vv = vv + v[i] * v[i];
        if (vv == 0.0) continue;
        double beta = 2.0 / vv;
        for (int j = k + 1; j < 3; ++j) {
            double s = 0.0;
            for (int i = k; i < 3; ++i) s = s + v[i] * R[i][j];
            s = s * beta;
            for (int i = k; i < 3; ++i) R[i][j] = R[i][j] - s * v[i];
        }
        {
            double s = 0.0;
            for (int i = k; i < 3; ++i) s = s + v[i] * c[i];
            s = s * beta;
            for (int i = k; i < 3; ++i) c[i] = c[i] - s * v[i];
        }
        R[k][k] = alpha;
        for (int i = k + 1; i < 3; ++i) R[i][k] = 0.0;
    }
    double thr = 3.0 * 2.220446049250313e-16 * fabs(R[0][0]);
    int rank = 0;
    for (int k = 0; k < 3; ++k) {
        if (fabs(R[k][k]) > thr)
            rank = k + 1;
        else
            break;
    }
    double y[3] = {0.0, 0.0, 0.0};
    for (int k = rank - 1; k >= 0; --k) {
        double s = c[k];
        for (int j = k + 1; j < rank; ++j) s = s - R[k][j] * y[j];
        y[k] = s / R[k][k];
    }
    for (int k = 0; k < 3; ++k) x[perm[k]] = y[k];
}

struct StarView {
    const double* vx;
    const double* vy;
    const double* vz;
    const int4* tets;
    int32_t nt;
    int32_t v;
    int form;   // TW_ENERGY_FORM_* of the binary64 AMIPS evaluations
};

__device__ __forceinline__ void gather_tet(const StarView& S, int4 tv, int start, const double* pos,
                                           double* T) {
    int id[4] = {tv.x, tv.y, tv.z, tv.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        int32_t k = id[(start + j) & 3];
        if (k == S.v) {
            T[3 * j] = pos[0];
            T[3 * j + 1] = pos[1];
            T[3 * j + 2] = pos[2];
        } else {
            T[3 * j] = __ldg(S.vx + k);
            T[3 * j + 1] = __ldg(S.vy + k);
            T[3 * j + 2] = __ldg(S.vz + k);
        }
    }
}

static __device__ bool star_flip(const StarView& S, const double* pos) {
    double T[12];
    for (int32_t i = 0; i < S.nt; ++i) {
        gather_tet(S, __ldg(S.tets + i), 0, pos, T);
        if (orient3d(T, T + 3, T + 6, T + 9) != 1) return true;
    }
    return false;
}

static __device__ double star_new_energy(const StarView& S, const double* pos) {
    double s = 0.0, T[12];
    for (int32_t i = 0; i < S.nt; ++i) {
        gather_tet(S, __ldg(S.tets + i), 0, pos, T);
        s += amips_energy_f(T, S.form);
    }
    if (isinf(s) || isnan(s) || s <= 0.0 || s > kMaxEnergy) s = kMaxEnergy;
    return s;
}

static __device__ bool star_update(const StarView& S, const double* pos, double& energy, double* J,
                            double* H) {
    double e = 0.0, T[12], J1[3], H1[9];
    for (int k = 0; k < 3; ++k) J[k] = 0.0;
    for (int k = 0; k < 9; ++k) H[k] = 0.0;
    for (int32_t i = 0; i < S.nt; ++i) {
        int4 tv = __ldg(S.tets + i);
        int start = (tv.x == S.v) ? 0 : (tv.y == S.v) ? 1 : (tv.z == S.v) ? 2 : (tv.w == S.v) ? 3 : 0;
        gather_tet(S, tv, start, pos, T);
        e += amips_egh_f(T, J1, H1, S.form);   // its E is amips_energy_f's, operation for operation
        for (int j = 0; j < 3; ++j) {
            J[j] += J1[j];
            H[3 * j + 0] += H1[3 * j + 0];
            H[3 * j + 1] += H1[3 * j + 1];
            H[3 * j + 2] += H1[3 * j + 2];
        }
    }
    if (isinf(e)) e = kMaxEnergy;
    energy = e;
    if (isnan(e)) return false;
    if (e <= 0.0) return false;
    for (int k = 0; k < 3; ++k)
        if (!isfinite(J[k])) return false;
    for (int k = 0; k < 9; ++k)
        if (!isfinite(H[k])) return false;
    return true;
}

// ---------------------------------------------------------------------------
// Fused Newton step with G lanes per star (G = 8, 16 or 32).
//
// The lanes of a group evaluate the star's tets G at a time; the per-tet
// terms are then added in tet order by broadcasting lane 0's value first,
// lane 1's next, ...: every lane accumulates the same sequence, so every lane
// holds the sum rounded exactly as the sequential loops of the reference
// (VertexSmoother.cpp:654-672 for E/J/H, :606-614 for the trial energy).
// The QR solve, the step logic and the acceptance tests are evaluated
// redundantly by all lanes of the group (uniform within the group); a trial
// position is rejected if any lane finds an inverted tet.
// ---------------------------------------------------------------------------
template <int G>
__device__ __forceinline__ unsigned group_mask(int lane) {
    return (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
}

// NewtonsMethod for the star S with G lanes; every lane returns the same
// position and is_moved.
template <int G>
__device__ __forceinline__ int newton_group_star(const StarView& S, double* pos, int max_step,
                                                 int max_it, int gl, unsigned gm) {
    const int32_t nt = S.nt;
    int is_moved = 0;
    double old_energy = 0.0, new_energy = 0.0, J[3], H[9];
    for (int step = 0; step < max_step; ++step) {
        // NewtonsUpdate: E, J, H summed over the tets in caller order
        double e = 0.0;
        for (int k = 0; k < 3; ++k) J[k] = 0.0;
        for (int k = 0; k < 9; ++k) H[k] = 0.0;
        for (int c0 = 0; c0 < nt; c0 += G) {
            const int cnt = min(G, nt - c0);
            double te = 0.0, tJ[3] = {0.0, 0.0, 0.0}, tH[9];
            for (int k = 0; k < 9; ++k) tH[k] = 0.0;
            if (gl < cnt) {
                int4 tv = __ldg(S.tets + c0 + gl);
                int start = (tv.x == S.v) ? 0 : (tv.y == S.v) ? 1 : (tv.z == S.v) ? 2
                          : (tv.w == S.v) ? 3 : 0;
                double T[12];
                gather_tet(S, tv, start, pos, T);
                te = amips_egh_f(T, tJ, tH, S.form);   // its E is amips_energy_f's
            }
            for (int t = 0; t < cnt; ++t) {
                e += __shfl_sync(gm, te, t, G);
#pragma unroll
                for (int k = 0; k < 3; ++k) J[k] += __shfl_sync(gm, tJ[k], t, G);
#pragma unroll
                for (int k = 0; k < 9; ++k) H[k] += __shfl_sync(gm, tH[k], t, G);
            }
        }
        if (isinf(e)) e = kMaxEnergy;
        old_energy = e;
        bool ok = !isnan(e) && !(e <= 0.0);
        for (int k = 0; k < 3; ++k) ok = ok && isfinite(J[k]);
        for (int k = 0; k < 9; ++k) ok = ok && isfinite(H[k]);
        if (!ok) break;
        double old_pf[3] = {pos[0], pos[1], pos[2]};
        double X0[3] = {pos[0], pos[1], pos[2]};
        double a = 1.0;
        bool step_taken = false;
        for (int it = 0; it < max_it; ++it) {
            double rhs[3], X[3];
            for (int i = 0; i < 3; ++i)
                rhs[i] = ((H[3 * i] * X0[0] + H[3 * i + 1] * X0[1]) + H[3 * i + 2] * X0[2]) -
                         a * J[i];
            qr_solve3(H, rhs, X);
            if (!isfinite(X[0]) || !isfinite(X[1]) || !isfinite(X[2])) {
                a /= 2.0;
                continue;
            }
            pos[0] = X[0];
            pos[1] = X[1];
            pos[2] = X[2];
            bool flip = false;
            for (int c0 = gl; c0 < nt; c0 += G) {
                double T[12];
                gather_tet(S, __ldg(S.tets + c0), 0, pos, T);
                flip = flip || (orient3d(T, T + 3, T + 6, T + 9) != 1);
            }
            if (__any_sync(gm, flip)) {
                pos[0] = old_pf[0];
                pos[1] = old_pf[1];
                pos[2] = old_pf[2];
                a /= 2.0;
                continue;
            }
            double sum = 0.0;
            for (int c0 = 0; c0 < nt; c0 += G) {
                const int cnt = min(G, nt - c0);
                double te = 0.0;
                if (gl < cnt) {
                    double T[12];
                    gather_tet(S, __ldg(S.tets + c0 + gl), 0, pos, T);
                    te = amips_energy_f(T, S.form);
                }
                for (int t = 0; t < cnt; ++t) sum += __shfl_sync(gm, te, t, G);
            }
            if (isinf(sum) || isnan(sum) || sum <= 0.0 || sum > kMaxEnergy) sum = kMaxEnergy;
            new_energy = sum;
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
    return is_moved;
}

// ---------------------------------------------------------------------------
// Smoothing pass (VertexSmoother.cpp:114-210 and :244-450), G lanes per star.
// ---------------------------------------------------------------------------
// True when every tet of the star is POSITIVE with the centre at pos.
template <int G>
__device__ __forceinline__ bool star_positive(const StarView& S, const double* pos, int gl,
                                              unsigned gm) {
    bool bad = false;
    for (int c0 = gl; c0 < S.nt; c0 += G) {
        double T[12];
        gather_tet(S, __ldg(S.tets + c0), 0, pos, T);
        bad = bad || (orient3d(T, T + 3, T + 6, T + 9) != 1);
    }
    return !__any_sync(gm, bad);
}

__device__ __forceinline__ int4 tet_at(const StarView& S, int32_t i) { return __ldg(S.tets + i); }
__device__ __forceinline__ int tet_vertex(int4 tv, int j) {
    return j == 0 ? tv.x : j == 1 ? tv.y : j == 2 ? tv.z : tv.w;
}

// The surface face of tet tv opposite its j-th vertex, as a sorted triple.
__device__ __forceinline__ void face_key(int4 tv, int j, int32_t* k) {
    int32_t id[4] = {tv.x, tv.y, tv.z, tv.w};
    int32_t a = id[(j + 1) & 3], b = id[(j + 2) & 3], c = id[(j + 3) & 3];
    int32_t lo = min(a, min(b, c)), hi = max(a, max(b, c));
    k[0] = lo;
    k[1] = (int32_t)((int64_t)a + b + c - lo - hi);
    k[2] = hi;
}

// calTetQuality_AMIPS for a tet already known to be POSITIVE.
__device__ __forceinline__ double positive_tet_quality(const double* T, int form) {
    return quality_from(1, amips_energy_f(T, form));
}

// True when face j of the star's tet c0 is a surface face through the
// centre whose sorted triple does not occur at an earlier (tet, face) of the
// star; writes the triple.
__device__ __forceinline__ bool first_surface_face(const StarView& S, const uint8_t* ff,
                                                   int32_t c0, int4 tv, uint8_t fl, int j,
                                                   int32_t* key) {
    if (tet_vertex(tv, j) == S.v || !((fl >> j) & 1)) return false;
    face_key(tv, j, key);
    for (int32_t i2 = 0; i2 <= c0; ++i2) {
        int4 t2 = tet_at(S, i2);
        uint8_t f2 = __ldg(ff + i2);
        for (int j2 = 0; j2 < 4; ++j2) {
            if (i2 == c0 && j2 >= j) return true;
            if (tet_vertex(t2, j2) == S.v || !((f2 >> j2) & 1)) continue;
            int32_t k2[3];
            face_key(t2, j2, k2);
            if (k2[0] == key[0] && k2[1] == key[1] && k2[2] == key[2]) return false;
        }
    }
    return true;
}

}  // namespace tw
