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

__device__ bool star_flip(const StarView& S, const double* pos) {
    double T[12];
    for (int32_t i = 0; i < S.nt; ++i) {
        gather_tet(S, __ldg(S.tets + i), 0, pos, T);
        if (orient3d(T, T + 3, T + 6, T + 9) != 1) return true;
    }
    return false;
}

__device__ double star_new_energy(const StarView& S, const double* pos) {
    double s = 0.0, T[12];
    for (int32_t i = 0; i < S.nt; ++i) {
        gather_tet(S, __ldg(S.tets + i), 0, pos, T);
        s += amips_energy(T);
    }
    if (isinf(s) || isnan(s) || s <= 0.0 || s > kMaxEnergy) s = kMaxEnergy;
    return s;
}

__device__ bool star_update(const StarView& S, const double* pos, double& energy, double* J,
                            double* H) {
    double e = 0.0, T[12], J1[3], H1[9];
    for (int k = 0; k < 3; ++k) J[k] = 0.0;
    for (int k = 0; k < 9; ++k) H[k] = 0.0;
    for (int32_t i = 0; i < S.nt; ++i) {
        int4 tv = __ldg(S.tets + i);
        int start = (tv.x == S.v) ? 0 : (tv.y == S.v) ? 1 : (tv.z == S.v) ? 2 : (tv.w == S.v) ? 3 : 0;
        gather_tet(S, tv, start, pos, T);
        e += amips_energy(T);
        amips_egh(T, J1, H1);
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

__global__ void __launch_bounds__(128) k_newton_stars(const double* __restrict__ vx,
                                                      const double* __restrict__ vy,
                                                      const double* __restrict__ vz,
                                                      const int32_t* __restrict__ star_off,
                                                      const int4* __restrict__ tets,
                                                      const int32_t* __restrict__ centers,
                                                      int32_t nstars, int max_step, int max_it,
                                                      double* __restrict__ out,
                                                      uint8_t* __restrict__ moved) {
    int32_t sid = blockIdx.x * blockDim.x + threadIdx.x;
    if (sid >= nstars) return;
    int32_t b = star_off[sid], e = star_off[sid + 1];
    StarView S{vx, vy, vz, tets + b, e - b, centers[sid]};
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

void launch_newton_stars(const double* vx, const double* vy, const double* vz,
                         const int32_t* star_off, const int32_t* tets, const int32_t* centers,
                         int32_t nstars, int max_step, int max_it, double* out, uint8_t* moved,
                         cudaStream_t s) {
    if (nstars <= 0) return;
    const int block = 128;
    int grid = (nstars + block - 1) / block;
    k_newton_stars<<<grid, block, 0, s>>>(vx, vy, vz, star_off, reinterpret_cast<const int4*>(tets),
                                          centers, nstars, max_step, max_it, out, moved);
}

}  // namespace tw
