// tw_device.cuh -- device arithmetic of the TetWild query path on sm_103a.
//
// Every routine evaluates the same operations in the same order as the CPU
// oracle, and all translation units are compiled with -fmad=false, so FP64
// results are bit-identical to the oracle's and every decision derived from
// them (orientation sign, envelope in/out, Newton accept/reject) matches.
#pragma once

#include <cstdint>

#include "../../include/tw_gb300.h"

namespace tw {

constexpr double kMaxEnergy = 1e50;                    // State.h:29
constexpr double kIsq3 = 0.57735026918962576451;       // 1/sqrt(3)
constexpr double kIsq6 = 0.40824829046386301637;       // 1/sqrt(6)
constexpr double kTwoThirds = 0.66666666666666662966;
constexpr double kTenNinths = 1.1111111111111111605;
constexpr double kEps = 1.1102230246251565404e-16;     // 2^-53
constexpr double kO3dBound = (7.0 + 56.0 * kEps) * kEps;  // Shewchuk 1997, orient3d stage A

// ---------------------------------------------------------------------------
// x^(-1/3) for x >= 0: exponent reduction to m in [1,8), three binary32 and
// two binary64 Newton-Raphson steps on y^-3 = m, exact rescale by 2^-q.
// Replaces pow(pow(det,2), -0.333333333333333) (LocalOperations.cpp:78-80).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double icbrt(double x) {
    if (!(x == x)) return x;
    if (x <= 0.0) return (x == 0.0) ? __longlong_as_double(0x7ff0000000000000LL)
                                    : __longlong_as_double(0x7ff8000000000000LL);
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    int e = (int)((u >> 52) & 0x7ff);
    if (e == 0x7ff) return 0.0;  // +inf (NaN handled above)
    int ebias = 0;
    if (e == 0) {
        x = x * 18014398509481984.0;
        u = (unsigned long long)__double_as_longlong(x);
        e = (int)((u >> 52) & 0x7ff);
        ebias = -54;
    }
    int ex = e - 1023 + ebias;
    int q = (ex >= 0) ? ex / 3 : -((-ex + 2) / 3);
    int rem = ex - 3 * q;
    double m = __longlong_as_double((long long)((u & 0x000fffffffffffffULL) |
                                                ((unsigned long long)(1023 + rem) << 52)));
    float mf = __double2float_rn(m);
    float yf = 0.9318f - 0.06015f * mf;
    const float third_f = 0.333333343f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float y3 = (yf * yf) * yf;
        float t = 1.0f - mf * y3;
        yf = yf + (yf * t) * third_f;
    }
    double y = (double)yf;
    const double third = 0.33333333333333331483;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        double y3 = (y * y) * y;
        double t = 1.0 - m * y3;
        y = y + (y * t) * third;
    }
    double s = __longlong_as_double((long long)((unsigned long long)(1023 - q) << 52));
    return y * s;
}

struct V3 {
    double x, y, z;
};

// Spreads the low 10 bits of v so that bit k moves to bit 3k (one axis of a
// 30-bit Morton code).
__device__ __forceinline__ uint32_t morton_expand10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
__device__ __forceinline__ double dot3(const V3& u, const V3& v) {
    return (u.x * v.x + u.y * v.y) + u.z * v.z;
}
__device__ __forceinline__ V3 cross3(const V3& u, const V3& v) {
    return V3{u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x};
}

// Rows of the map from the regular tet (closed form of the generated
// expressions in LocalOperations.cpp:28-291):
//   a = p0 - p3, b = (p0 - 2p1 + p3)/sqrt3, c = (p0 + p1 + p3 - 3p2)/sqrt6.
__device__ __forceinline__ void amips_frame(const double* T, V3& a, V3& b, V3& c) {
    double av[3], bv[3], cv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double x0 = T[k], x1 = T[3 + k], x2 = T[6 + k], x3 = T[9 + k];
        av[k] = x0 - x3;
        bv[k] = ((x0 - x1) + (x3 - x1)) * kIsq3;
        cv[k] = (((x0 - x2) + (x1 - x2)) + (x3 - x2)) * kIsq6;
    }
    a = V3{av[0], av[1], av[2]};
    b = V3{bv[0], bv[1], bv[2]};
    c = V3{cv[0], cv[1], cv[2]};
}

// comformalAMIPSEnergy_new (LocalOperations.cpp:28-81): N * (D^2)^(-1/3).
__device__ __forceinline__ double amips_energy(const double* T) {
    V3 a, b, c;
    amips_frame(T, a, b, c);
    double N = (dot3(a, a) + dot3(b, b)) + dot3(c, c);
    V3 bc = cross3(b, c);
    double D = dot3(a, bc);
    return N * icbrt(D * D);
}

// Energy, gradient (:83-147) and Hessian (:149-291) w.r.t. vertex 0 in one
// pass.  J and H are written only when the pointers are non-null.
__device__ __forceinline__ double amips_egh(const double* T, double* J, double* H) {
    V3 a, b, c;
    amips_frame(T, a, b, c);
    double N = (dot3(a, a) + dot3(b, b)) + dot3(c, c);
    V3 bc = cross3(b, c);
    double D = dot3(a, bc);
    double r = icbrt(D * D);
    double E = N * r;
    if (J || H) {
        V3 ca = cross3(c, a), ab = cross3(a, b);
        double g[3], gN[3];
        g[0] = (bc.x + kIsq3 * ca.x) + kIsq6 * ab.x;
        g[1] = (bc.y + kIsq3 * ca.y) + kIsq6 * ab.y;
        g[2] = (bc.z + kIsq3 * ca.z) + kIsq6 * ab.z;
        gN[0] = 2.0 * ((a.x + kIsq3 * b.x) + kIsq6 * c.x);
        gN[1] = 2.0 * ((a.y + kIsq3 * b.y) + kIsq6 * c.y);
        gN[2] = 2.0 * ((a.z + kIsq3 * b.z) + kIsq6 * c.z);
        double invD = 1.0 / D;
        if (J) {
            double t = (kTwoThirds * N) * invD;
#pragma unroll
            for (int k = 0; k < 3; ++k) J[k] = r * (gN[k] - t * g[k]);
        }
        if (H) {
            double s1 = (kTwoThirds * r) * invD;
            double s2 = (((kTenNinths * N) * r) * invD) * invD;
            double r3 = 3.0 * r;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = i; j < 3; ++j) {
                    double base = (i == j) ? r3 : 0.0;
                    double h = (base - s1 * (gN[i] * g[j] + g[i] * gN[j])) + s2 * (g[i] * g[j]);
                    H[i * 3 + j] = h;
                    H[j * 3 + i] = h;
                }
        }
    }
    return E;
}

// ---------------------------------------------------------------------------
// Reference form of the AMIPS energy, gradient and Hessian
// (LocalOperations.cpp:28-81, :83-147, :149-291).  The reference evaluates
// machine-generated expressions on the absolute coordinates with 15-digit
// coefficients; for a small tet away from the origin their terms cancel by up
// to ~1e4, so its results carry rounding of up to ~5e-12 relative, and
// agreeing with it to 1e-12 takes the same IEEE operations in the same order.
// These routines perform them: every sum and product is grouped as the
// generated code groups it (left to right), with its coefficients (kRf*).
// Addition and multiplication are commutative and negation is exact, so only
// the grouping is kept.  x0..z3: the vertices' coordinates; bx..bz, cx..cz:
// the scaled frame rows, grouped per routine as its generated code does;
// Lx0..Lz3: the numerator's per-coordinate linear forms.  pow(d, 2) is d*d
// and pow(s, -0.333333333333333) is rf_pow_m13.  The CPU oracle performs the
// same operations; its libm build is bit-identical to the reference.
// ---------------------------------------------------------------------------
constexpr double kRfB1 = 0.577350269189626;   // 1/sqrt3 as the generated code spells it
constexpr double kRfB2 = 1.15470053837925;    // 2/sqrt3 (not 2 kRfB1)
constexpr double kRfC1 = 0.408248290463863;   // 1/sqrt6
constexpr double kRfC3 = 1.22474487139159;    // 3/sqrt6
constexpr double kRfS2 = 0.707106781186548;   // 1/sqrt2
constexpr double kRf2_3 = 0.666666666666667;
constexpr double kRf4_3 = 1.33333333333333;
constexpr double kRf4_9 = 0.444444444444444;
constexpr double kRf10_9 = 1.11111111111111;
constexpr double kRfTiny = 1.85037170770859e-17;  // code-generation residue (:267), kept
constexpr double kRfDelta = 3.515706244646329e-16;  // -0.333333333333333 + 1/3
constexpr double kRfLn2 = 0.6931471805599453;

// s^(-0.333333333333333): s^(-1/3) (icbrt) times the first-order factor
// 1 + kRfDelta ln s (a correction below 2.6e-13 over the double range; ln s
// to ~4% from the exponent and one atanh term keeps its error below 1e-17).
__device__ __forceinline__ double rf_pow_m13(double s) {
    const double r = icbrt(s);
    if (!(r > 0.0) || isinf(r)) return r;
    const unsigned long long u = (unsigned long long)__double_as_longlong(s);
    const int e = (int)((u >> 52) & 0x7ff);
    const double m = __longlong_as_double(
        (long long)((u & 0x000fffffffffffffULL) | (1023ULL << 52)));
    const double ln = (double)(e - 1023) * kRfLn2 + (2.0 * (m - 1.0)) / (m + 1.0);
    return r + r * (kRfDelta * ln);
}

__device__ __forceinline__ double amips_rf_energy(const double* T) {
    const double x0 = T[0], y0 = T[1], z0 = T[2], x1 = T[3], y1 = T[4], z1 = T[5];
    const double x2 = T[6], y2 = T[7], z2 = T[8], x3 = T[9], y3 = T[10], z3 = T[11];
    const double bx = (kRfB1 * x0 - kRfB2 * x1) + kRfB1 * x3;
    const double cy = ((kRfC1 * y3 + kRfC1 * y0) + kRfC1 * y1) - kRfC3 * y2;
    const double by = (kRfB1 * y3 + kRfB1 * y0) - kRfB2 * y1;
    const double cx = ((kRfC1 * x0 - kRfC3 * x2) + kRfC1 * x1) + kRfC1 * x3;
    const double cz = ((kRfC1 * z0 + kRfC1 * z1) - kRfC3 * z2) + kRfC1 * z3;
    const double bz = (kRfB1 * z0 - kRfB2 * z1) + kRfB1 * z3;
    const double hx = 0.5 * x2 + 0.5 * x1, hy = 0.5 * y1 + 0.5 * y2, hz = 0.5 * z1 + 0.5 * z2;
    const double num =
        z0 * ((0.5 * z3 - 1.5 * z0) + hz) + y3 * ((hy - 1.5 * y3) + 0.5 * y0) +
        x2 * (((0.5 * x0 - 1.5 * x2) + 0.5 * x1) + 0.5 * x3) +
        z1 * (((0.5 * z0 - 1.5 * z1) + 0.5 * z2) + 0.5 * z3) +
        z2 * (((0.5 * z0 + 0.5 * z1) - 1.5 * z2) + 0.5 * z3) + z3 * ((0.5 * z0 - 1.5 * z3) + hz) +
        x0 * ((hx - 1.5 * x0) + 0.5 * x3) + x1 * (((0.5 * x2 + 0.5 * x0) - 1.5 * x1) + 0.5 * x3) +
        x3 * ((hx + 0.5 * x0) - 1.5 * x3) + y0 * ((0.5 * y3 + hy) - 1.5 * y0) +
        y1 * (((0.5 * y3 + 0.5 * y0) - 1.5 * y1) + 0.5 * y2) +
        y2 * (((0.5 * y3 + 0.5 * y0) + 0.5 * y1) - 1.5 * y2);
    const double det = ((z0 - z3) * (cy * bx - by * cx) - (y0 - y3) * (cz * bx - cx * bz)) +
                       (x0 - x3) * (by * cz - cy * bz);
    return -num * rf_pow_m13((det * det));
}

__device__ __forceinline__ void amips_rf_jacobian(const double* T, double* J) {
    const double x0 = T[0], y0 = T[1], z0 = T[2], x1 = T[3], y1 = T[4], z1 = T[5];
    const double x2 = T[6], y2 = T[7], z2 = T[8], x3 = T[9], y3 = T[10], z3 = T[11];
    const double dy = y0 - y3, dz = z0 - z3, dx = x0 - x3;
    const double bx = (kRfB1 * x0 - kRfB2 * x1) + kRfB1 * x3;
    const double by = (kRfB1 * y0 - kRfB2 * y1) + kRfB1 * y3;
    const double bz = (kRfB1 * z0 - kRfB2 * z1) + kRfB1 * z3;
    const double cx = ((kRfC1 * x0 - kRfC3 * x2) + kRfC1 * x1) + kRfC1 * x3;
    const double cy = ((kRfC1 * y0 + kRfC1 * y1) - kRfC3 * y2) + kRfC1 * y3;
    const double cz = ((kRfC1 * z1 - kRfC3 * z2) + kRfC1 * z3) + kRfC1 * z0;
    const double czbx = cz * bx - bz * cx;
    const double cybx = cy * bx, cxby = cx * by;
    const double det = (czbx * dy - dz * (cybx - cxby)) - dx * (cz * by - bz * cy);
    const double r = rf_pow_m13((det * det));
    const double sz = kRfS2 * z1 - kRfS2 * z2, sy = kRfS2 * y1 - kRfS2 * y2;
    const double sx = kRfS2 * x1 - kRfS2 * x2;
    const double hx = 0.5 * x2 + 0.5 * x1, hy = 0.5 * y1 + 0.5 * y2, hz = 0.5 * z1 + 0.5 * z2;
    const double num =
        y0 * ((0.5 * y3 - 1.5 * y0) + hy) + z1 * (((0.5 * z2 - 1.5 * z1) + 0.5 * z3) + 0.5 * z0) +
        z2 * (((0.5 * z1 - 1.5 * z2) + 0.5 * z3) + 0.5 * z0) + z3 * ((hz - 1.5 * z3) + 0.5 * z0) +
        y3 * ((0.5 * y0 - 1.5 * y3) + hy) + x2 * (((0.5 * x0 - 1.5 * x2) + 0.5 * x1) + 0.5 * x3) +
        y1 * (((0.5 * y0 + 0.5 * y3) - 1.5 * y1) + 0.5 * y2) +
        y2 * (((0.5 * y0 + 0.5 * y3) + 0.5 * y1) - 1.5 * y2) + x0 * ((hx - 1.5 * x0) + 0.5 * x3) +
        x1 * (((0.5 * x2 + 0.5 * x0) - 1.5 * x1) + 0.5 * x3) + x3 * ((0.5 * x0 + hx) - 1.5 * x3) +
        z0 * ((0.5 * z3 + hz) - 1.5 * z0);
    const double w = (kRf2_3 * num) / det;
    const double q0 = ((sz * (y3 - y0) - sy * (z3 - z0)) - bz * cy) + by * cz;
    J[0] = -(r * ((((x2 - 3.0 * x0) + w * q0) + x1) + x3));
    J[1] = r * ((((3.0 * y0 - y3) - y1) - y2) + w * ((czbx + dz * sx) - dx * sz));
    J[2] = r * (((((-z1) - z2) - z3) + w * (((-(dy * sx)) - cybx) + cxby + dx * sy)) + 3.0 * z0);
}

__device__ __forceinline__ void amips_rf_hessian(const double* T, double* H) {
    const double x0 = T[0], y0 = T[1], z0 = T[2], x1 = T[3], y1 = T[4], z1 = T[5];
    const double x2 = T[6], y2 = T[7], z2 = T[8], x3 = T[9], y3 = T[10], z3 = T[11];
    const double dz = z0 - z3, dx = x0 - x3, dy = y0 - y3;
    const double bx = (kRfB1 * x0 - kRfB2 * x1) + kRfB1 * x3;
    const double by = (kRfB1 * y0 - kRfB2 * y1) + kRfB1 * y3;
    const double bz = (kRfB1 * z0 - kRfB2 * z1) + kRfB1 * z3;
    const double cx = ((kRfC1 * x0 + kRfC1 * x1) - kRfC3 * x2) + kRfC1 * x3;
    const double cy = ((kRfC1 * y0 + kRfC1 * y1) - kRfC3 * y2) + kRfC1 * y3;
    const double cz = ((kRfC1 * z0 + kRfC1 * z1) - kRfC3 * z2) + kRfC1 * z3;
    const double bxcy = bx * cy, bycx = by * cx;
    const double mx = dz * (bxcy - bycx);
    const double bycz = by * cz, cybz = cy * bz;
    const double myz = bycz - cybz;
    const double my = dx * myz;
    const double bxcz = bx * cz, cxbz = cx * bz;
    const double mxz = bxcz - cxbz;
    const double mz = dy * mxz;
    const double det = (mx + my) - mz;
    const double det2 = (det * det);
    const double r = rf_pow_m13(det2);
    const double lx = ((x2 - 3.0 * x0) + x1) + x3;
    const double sy = kRfS2 * y1 - kRfS2 * y2;
    const double dzsy = dz * sy;
    const double sz = kRfS2 * z1 - kRfS2 * z2;
    const double dysz = dy * sz;
    const double u = (myz + dzsy) - dysz;
    const double k43 = kRf4_3 / det;
    const double idet2 = 1.0 / det2;
    const double hx = 0.5 * x2 + 0.5 * x1;
    const double Lx0 = (hx - 1.5 * x0) + 0.5 * x3;
    const double Lx3 = (0.5 * x0 + hx) - 1.5 * x3;
    const double Lx2 = ((0.5 * x0 - 1.5 * x2) + 0.5 * x1) + 0.5 * x3;
    const double Lx1 = ((0.5 * x2 + 0.5 * x0) - 1.5 * x1) + 0.5 * x3;
    const double hy = 0.5 * y1 + 0.5 * y2;
    const double Ly0 = (0.5 * y3 - 1.5 * y0) + hy;
    const double Ly3 = (0.5 * y0 - 1.5 * y3) + hy;
    const double Ly2 = ((0.5 * y0 + 0.5 * y1) - 1.5 * y2) + 0.5 * y3;
    const double Ly1 = ((0.5 * y0 - 1.5 * y1) + 0.5 * y2) + 0.5 * y3;
    const double hz = 0.5 * z1 + 0.5 * z2;
    const double Lz0 = (0.5 * z3 - 1.5 * z0) + hz;
    const double Lz3 = (0.5 * z0 - 1.5 * z3) + hz;
    const double Lz2 = ((0.5 * z0 + 0.5 * z3) + 0.5 * z1) - 1.5 * z2;
    const double Lz1 = ((0.5 * z0 + 0.5 * z3) - 1.5 * z1) + 0.5 * z2;
    const double num = z0 * Lz0 + y0 * Ly0 + y1 * Ly1 + y2 * Ly2 + y3 * Ly3 + z3 * Lz3 +
                       x2 * Lx2 + z1 * Lz1 + z2 * Lz2 + x0 * Lx0 + x1 * Lx1 + Lx3 * x3;
    const double k49n = (kRf4_9 * idet2) * num;
    const double nd = idet2 * num;
    const double ineg = 1.0 / (-det);
    const double rneg = ineg * r;
    const double sx = kRfS2 * x1 - kRfS2 * x2;
    const double v1 = (((kRf2_3 * bx) * cz + (kRf2_3 * dz) * sx) - (kRf2_3 * cx) * bz) -
                      (kRf2_3 * dx) * sz;
    const double ly = ((y1 - 3.0 * y0) + y2) + y3;
    const double ey = y3 - y0, ez = z3 - z0;
    const double v2 = (((-kRf2_3 * sy) * ez + (kRf2_3 * sz) * ey) + (kRf2_3 * by) * cz) -
                      (kRf2_3 * bz) * cy;
    const double dzsx = dz * sx, dxsz = dx * sz;
    const double p = (dzsx - dxsz) + mxz;
    const double q = ((sz * ey - sy * ez) + by * cz) - bz * cy;
    const double a1 = ((((kRf4_9 * p) * q) * num) * ineg + lx * v1) - ly * v2;
    const double tiny = (kRfTiny * z0) * Lz0 + (kRfTiny * y0) * Ly0 + (kRfTiny * y1) * Ly1 +
                        (kRfTiny * y2) * Ly2 + (kRfTiny * y3) * Ly3 + (kRfTiny * z3) * Lz3 +
                        (kRfTiny * x2) * Lx2 + (kRfTiny * z1) * Lz1 + (kRfTiny * z2) * Lz2 +
                        (kRfTiny * x0) * Lx0 + (kRfTiny * x1) * Lx1 + (kRfTiny * Lx3) * x3;
    const double un = (u * num) * ineg;
    const double v3 = (((kRf2_3 * by) * cx - (kRf2_3 * bx) * cy) + (kRf2_3 * dx) * sy) -
                      (kRf2_3 * dy) * sx;
    const double lz = ((z3 - 3.0 * z0) + z1) + z2;
    const double t = ((bycx - bxcy) + dx * sy) - dy * sx;
    const double tn = ((kRf4_9 * t) * num) * ineg;
    const double a2 = (q * tn + v3 * lx) - lz * v2;
    const double ex = x3 - x0;
    const double w1 = (num * ineg) * (((ex * sz - sx * ez) + bx * cz) - cx * bz);
    const double s = ((dxsz - dzsx) - bxcz) + cxbz;
    const double a3 = ((-p) * tn + v3 * ly) + lz * v1;
    const double w2 = (num * ineg) * (((ex * (-sy) + sx * ey) - bx * cy) + cx * by);
    H[0] = r * ((((lx * u) * k43 - (u * u) * k49n) + ((kRf2_3 * u) * nd) * (((cybz - bycz) - dzsy) + dysz)) + 3.0);
    H[1] = rneg * ((a1 - tiny * z1) + un * v1);
    H[2] = rneg * (un * v3 + a2);
    H[3] = rneg * (a1 + w1 * v2);
    H[4] = r * ((((-(s * s)) * k49n + (s * k43) * ly) + (s * nd) * v1) + 3.0);
    H[5] = rneg * (((-tiny) * x1 - v3 * w1) + a3);
    H[6] = rneg * (((-tiny) * y1 + a2) + w2 * v2);
    H[7] = rneg * (a3 - w2 * v1);
    H[8] = r * ((((-lz) * t) * k43 - (kRf10_9 * (t * t)) * nd) + 3.0);
}

// Energy form of the FP64 evaluations (TW_ENERGY_FORM_*): the reference form
// (the default: agrees with the reference to its rounding) or the closed form.
__device__ __forceinline__ double amips_energy_f(const double* T, int form) {
    return form == TW_ENERGY_FORM_CLOSED ? amips_energy(T) : amips_rf_energy(T);
}
// E, and J / H when non-null, in the selected form.  In the reference form
// they come from the three separate routines, as NewtonsUpdate calls them
// (VertexSmoother.cpp:654-672).
__device__ __forceinline__ double amips_egh_f(const double* T, double* J, double* H, int form) {
    if (form == TW_ENERGY_FORM_CLOSED) return amips_egh(T, J, H);
    const double e = amips_rf_energy(T);
    if (J) amips_rf_jacobian(T, J);
    if (H) amips_rf_hessian(T, H);
    return e;
}

// ---------------------------------------------------------------------------
// Exact orientation: CGAL::orientation(p,q,r,s) = sign det[q-p, r-p, s-p].
// Floating-point filter with Shewchuk's stage-A bound, then exact
// expansion arithmetic (Two-Sum / Two-Diff / fma Two-Product,
// Grow-Expansion and Scale-Expansion with zero elimination).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(double a, double b, double& x, double& y) {
    double s = a + b, bv = s - a, av = s - bv, br = b - bv, ar = a - av;
    x = s;
    y = ar + br;
}
__device__ __forceinline__ void two_diff(double a, double b, double& x, double& y) {
    double d = a - b, bv = a - d, av = d + bv, br = bv - b, ar = a - av;
    x = d;
    y = ar + br;
}
__device__ __forceinline__ void fast_two_sum(double a, double b, double& x, double& y) {
    double s = a + b, bv = s - a;
    x = s;
    y = b - bv;
}
__device__ __forceinline__ void two_prod(double a, double b, double& x, double& y) {
    double p = a * b;
    x = p;
    y = fma(a, b, -p);
}
__device__ __forceinline__ int exp_grow(const double* e, int n, double b, double* h) {
    double Q = b, hh;
    int k = 0;
    for (int i = 0; i < n; ++i) {
        two_sum(Q, e[i], Q, hh);
        if (hh != 0.0) h[k++] = hh;
    }
    if (Q != 0.0 || k == 0) h[k++] = Q;
    return k;
}
__device__ __forceinline__ int exp_sum(const double* e, int n, const double* f, int m, double* h,
                                       double* tmp) {
    int k = n;
    for (int i = 0; i < n; ++i) h[i] = e[i];
    for (int j = 0; j < m; ++j) {
        k = exp_grow(h, k, f[j], tmp);
        for (int i = 0; i < k; ++i) h[i] = tmp[i];
    }
    return k;
}
__device__ __forceinline__ int exp_scale(const double* e, int n, double b, double* h) {
    double Q, hh, p1, p0, sum;
    int k = 0;
    two_prod(e[0], b, Q, hh);
    if (hh != 0.0) h[k++] = hh;
    for (int i = 1; i < n; ++i) {
        two_prod(e[i], b, p1, p0);
        two_sum(Q, p0, sum, hh);
        if (hh != 0.0) h[k++] = hh;
        fast_two_sum(p1, sum, Q, hh);
        if (hh != 0.0) h[k++] = hh;
    }
    if (Q != 0.0 || k == 0) h[k++] = Q;
    return k;
}
__device__ __forceinline__ int exp_mul22(const double* x, int nx, const double* y, int ny,
                                         double* h) {
    double t0[4], t1[4], tmp[8];
    int k0 = exp_scale(y, ny, x[0], t0);
    if (nx == 1) {
        for (int i = 0; i < k0; ++i) h[i] = t0[i];
        return k0;
    }
    int k1 = exp_scale(y, ny, x[1], t1);
    return exp_sum(t0, k0, t1, k1, h, tmp);
}
__device__ __forceinline__ int exp_diff(double a, double b, double* e) {
    double x, y;
    two_diff(a, b, x, y);
    if (y == 0.0) {
        e[0] = x;
        return 1;
    }
    e[0] = y;
    e[1] = x;
    return 2;
}
__device__ __forceinline__ int exp_minor(const double* u1, int n1, const double* v2, int m2,
                                         const double* u2, int n2, const double* v1, int m1,
                                         double* h) {
    double p[8], q[8], tmp[16];
    int kp = exp_mul22(u1, n1, v2, m2, p);
    int kq = exp_mul22(u2, n2, v1, m1, q);
    for (int i = 0; i < kq; ++i) q[i] = -q[i];
    return exp_sum(p, kp, q, kq, h, tmp);
}

// Rare path (the filter failed): kept out of line so the hot kernels do not
// carry its local-memory arrays.
static __device__ __noinline__ int orient3d_exact(const double* p, const double* q,
                                                  const double* r, const double* s) {
    double u[3][2], v[3][2], w[3][2];
    int nu[3], nv[3], nw[3];
    for (int k = 0; k < 3; ++k) {
        nu[k] = exp_diff(q[k], p[k], u[k]);
        nv[k] = exp_diff(r[k], p[k], v[k]);
        nw[k] = exp_diff(s[k], p[k], w[k]);
    }
    double m[16], t0[32], t1[32], term[64], acc[192], acc2[192], tmp[192];
    int nacc = 0;
    const int ia[3] = {1, 2, 0}, ib[3] = {2, 0, 1};
    for (int k = 0; k < 3; ++k) {
        int i = ia[k], j = ib[k];
        int nm = exp_minor(v[i], nv[i], w[j], nw[j], v[j], nv[j], w[i], nw[i], m);
        int k0 = exp_scale(m, nm, u[k][0], t0);
        int nt;
        if (nu[k] == 2) {
            int k1 = exp_scale(m, nm, u[k][1], t1);
            nt = exp_sum(t0, k0, t1, k1, term, tmp);
        } else {
            for (int z = 0; z < k0; ++z) term[z] = t0[z];
            nt = k0;
        }
        if (nacc == 0) {
            for (int z = 0; z < nt; ++z) acc[z] = term[z];
            nacc = nt;
        } else {
            nacc = exp_sum(acc, nacc, term, nt, acc2, tmp);
            for (int z = 0; z < nacc; ++z) acc[z] = acc2[z];
        }
    }
    double top = acc[nacc - 1];
    return (top > 0.0) - (top < 0.0);
}

// Returns +1 POSITIVE, 0 COPLANAR (or non-finite input), -1 NEGATIVE.
// *exact_used is set when the filter could not decide.
__device__ __forceinline__ int orient3d(const double* p, const double* q, const double* r,
                                        const double* s, int* exact_used = nullptr) {
    double ux = q[0] - p[0], uy = q[1] - p[1], uz = q[2] - p[2];
    double vx = r[0] - p[0], vy = r[1] - p[1], vz = r[2] - p[2];
    double wx = s[0] - p[0], wy = s[1] - p[1], wz = s[2] - p[2];
    double vywz = vy * wz, vzwy = vz * wy;
    double vzwx = vz * wx, vxwz = vx * wz;
    double vxwy = vx * wy, vywx = vy * wx;
    double det = (ux * (vywz - vzwy) + uy * (vzwx - vxwz)) + uz * (vxwy - vywx);
    double perm = (fabs(ux) * (fabs(vywz) + fabs(vzwy)) + fabs(uy) * (fabs(vzwx) + fabs(vxwz))) +
                  fabs(uz) * (fabs(vxwy) + fabs(vywx));
    double bound = kO3dBound * perm;
    if (det > bound) return 1;
    if (-det > bound) return -1;
    // Non-finite coordinates make det or perm non-finite: report COPLANAR.
    if (!isfinite(perm) || !isfinite(det)) return 0;
    bool finite_in = true;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        finite_in = finite_in && isfinite(p[k]) && isfinite(q[k]) && isfinite(r[k]) && isfinite(s[k]);
    if (!finite_in) return 0;
    if (exact_used) *exact_used = 1;
    return orient3d_exact(p, q, r, s);
}

// ---------------------------------------------------------------------------
// binary32 <-> binary64 conversions in integer arithmetic.  On this GPU the
// hardware conversions issue to the (slow) FP64 pipe; these use only the
// integer ALU, for every class of input (normal, subnormal, zero, infinity,
// NaN), and agree with the hardware bit for bit (tw_self_test checks it).
// ---------------------------------------------------------------------------
// Exact: every binary32 value is a binary64 value.
__device__ __forceinline__ double f2d_exact(float f) {
    uint32_t b = __float_as_uint(f);
    uint32_t s = b & 0x80000000u;
    uint32_t e = (b >> 23) & 0xffu;
    uint32_t m = b & 0x7fffffu;
    uint32_t hi, lo;
    if (e == 0xffu) {            // inf / NaN: payload kept
        hi = s | 0x7ff00000u | (m >> 3);
        lo = m << 29;
    } else if (e != 0u) {        // normal
        hi = s | ((e + (1023u - 127u)) << 20) | (m >> 3);
        lo = m << 29;
    } else if (m == 0u) {        // signed zero
        hi = s;
        lo = 0u;
    } else {                     // subnormal: m * 2^-149, top bit at position p
        uint32_t p = 31u - (uint32_t)__clz(m);
        unsigned long long mant = ((unsigned long long)m << (52u - p)) & 0x000fffffffffffffULL;
        hi = s | ((p + 1023u - 149u) << 20) | (uint32_t)(mant >> 32);
        lo = (uint32_t)mant;
    }
    return __hiloint2double((int)hi, (int)lo);
}
// Round to nearest, ties to even (the IEEE default), like __double2float_rn.
__device__ __forceinline__ float d2f_rn(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    uint32_t s = hi & 0x80000000u;
    uint32_t e11 = (hi >> 20) & 0x7ffu;
    if (e11 == 0x7ffu) {                               // inf / NaN (NaN made quiet)
        bool nan = ((hi & 0xfffffu) | lo) != 0u;
        return __uint_as_float(s | 0x7f800000u | (nan ? 0x00400000u | ((hi & 0xfffffu) << 3) | (lo >> 29) : 0u));
    }
    int e = (int)e11 - 1023 + 127;
    if (e >= 255) return __uint_as_float(s | 0x7f800000u);   // overflow: inf
    if (e >= 1) {                                       // normal result
        uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 mantissa bits
        uint32_t rest = lo & 0x1fffffffu;                  // the 29 dropped bits
        uint32_t r = ((uint32_t)e << 23) | m;
        // a carry out of the mantissa increments the exponent (and rounds to
        // inf at the top of the range), as round-to-nearest requires
        r += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
        return __uint_as_float(s | r);
    }
    // subnormal or zero result: value = M53 * 2^(e11 - 1075) = k * 2^-149
    if (e11 == 0u) return __uint_as_float(s);          // double zero or subnormal
    unsigned long long M = (b & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    uint32_t sh = 926u - e11;                           // >= 30 here
    if (sh > 54u) return __uint_as_float(s);            // below half the smallest subnormal
    unsigned long long k = M >> sh;
    unsigned long long rest = M & ((1ULL << sh) - 1ULL);
    unsigned long long half = 1ULL << (sh - 1u);
    k += (rest > half || (rest == half && (k & 1ULL))) ? 1ULL : 0ULL;
    return __uint_as_float(s | (uint32_t)k);            // k = 2^23 is the smallest normal
}

// ---------------------------------------------------------------------------
// Certified binary32 AMIPS (TW_PRECISION_FP32_CERTIFIED).
// ---------------------------------------------------------------------------
constexpr float kU32 = 5.9604644775390625e-08f;  // 2^-24

// x^(-1/3) for a normal positive binary32 x: exponent reduction to [1,8) and
// four Newton-Raphson steps from a linear seed; relative error below 4 u.
__device__ __forceinline__ float icbrt32(float x) {
    unsigned u = __float_as_uint(x);
    int e = (int)((u >> 23) & 0xffu) - 127;
    int q = (e >= 0) ? e / 3 : -((-e + 2) / 3);
    int rem = e - 3 * q;
    float m = __uint_as_float((u & 0x7fffffu) | ((unsigned)(127 + rem) << 23));
    float y = fmaf(-0.06015f, m, 0.9318f);
    const float third = 0.333333343f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float y3 = (y * y) * y;
        y = fmaf(y * fmaf(-m, y3, 1.0f), third, y);
    }
    return y * __uint_as_float((unsigned)(127 - q) << 23);
}

// Result of the binary32 evaluation: ok = false when the certified relative
// error bound of E exceeds tol (or a magnitude leaves the safe binary32 range);
// the caller then recomputes the tet in FP64.
struct Amips32 {
    bool ok;
    float E;
    float J[3];
    float H[9];
};

// d1 = p1 - p0, d2 = p2 - p0, d3 = p3 - p0, each rounded once from FP64.
// Frame (same map as amips_frame): a = -d3, b = (d3 - 2 d1)/sqrt3,
// c = (d1 + d3 - 3 d2)/sqrt6.  Error bound (u = 2^-24, first order):
// the components of a, b, c carry errors <= u A_k, 4u B_k, 5u C_k with
// A = |d3|, B = (|d3| + 2|d1|)/sqrt3, C = (|d1| + |d3| + 3|d2|)/sqrt6 (input
// rounding, fma, constant and product roundings), so with perm(A,B,C) the
// permanent of the rows A, B, C:  |dD| <= 16u perm(A,B,C) (10u from the
// inputs, 5u from the triple product), |dN| <= 10u sum(A^2+B^2+C^2) + 4u N,
// and rel(E) <= rel(N) + 2/3 rel(D) + 6u (icbrt <= 4u, D^2 and N r).
template <bool WJ, bool WH>
__device__ __forceinline__ Amips32 amips_egh32(const float* d1, const float* d2, const float* d3,
                                               float tol) {
    const float isq3 = 0.577350269f, isq6 = 0.408248290f;
    float a[3], b[3], c[3], A[3], B[3], C[3], NB = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a[k] = -d3[k];
        b[k] = fmaf(-2.0f, d1[k], d3[k]) * isq3;
        c[k] = fmaf(-3.0f, d2[k], d1[k] + d3[k]) * isq6;
        A[k] = fabsf(d3[k]);
        B[k] = fmaf(2.0f, fabsf(d1[k]), fabsf(d3[k])) * isq3;
        C[k] = fmaf(3.0f, fabsf(d2[k]), fabsf(d1[k]) + fabsf(d3[k])) * isq6;
        NB = fmaf(A[k], A[k], fmaf(B[k], B[k], fmaf(C[k], C[k], NB)));
    }
    float PD = A[0] * fmaf(B[1], C[2], B[2] * C[1]) + A[1] * fmaf(B[2], C[0], B[0] * C[2]) +
               A[2] * fmaf(B[0], C[1], B[1] * C[0]);
    float N = fmaf(a[2], a[2], fmaf(a[1], a[1], a[0] * a[0])) +
              fmaf(b[2], b[2], fmaf(b[1], b[1], b[0] * b[0])) +
              fmaf(c[2], c[2], fmaf(c[1], c[1], c[0] * c[0]));
    float bc[3] = {fmaf(b[1], c[2], -b[2] * c[1]), fmaf(b[2], c[0], -b[0] * c[2]),
                   fmaf(b[0], c[1], -b[1] * c[0])};
    float D = fmaf(a[2], bc[2], fmaf(a[1], bc[1], a[0] * bc[0]));
    float aD = fabsf(D);
    Amips32 R;
    float bound = 1.01f * (14.0f * kU32 * NB / N + 10.6667f * kU32 * PD / aD + 6.0f * kU32);
    R.ok = (aD > 1e-18f) && (aD < 1e18f) && (N > 1e-30f) && (N < 1e30f) && (bound <= tol);
    if (!R.ok) return R;
    float r = icbrt32(D * D);
    R.E = N * r;
    if (WJ || WH) {
        float ca[3] = {fmaf(c[1], a[2], -c[2] * a[1]), fmaf(c[2], a[0], -c[0] * a[2]),
                       fmaf(c[0], a[1], -c[1] * a[0])};
        float ab[3] = {fmaf(a[1], b[2], -a[2] * b[1]), fmaf(a[2], b[0], -a[0] * b[2]),
                       fmaf(a[0], b[1], -a[1] * b[0])};
        float g[3], gN[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            g[k] = fmaf(isq6, ab[k], fmaf(isq3, ca[k], bc[k]));
            gN[k] = 2.0f * fmaf(isq6, c[k], fmaf(isq3, b[k], a[k]));
        }
        float invD = 1.0f / D;
        if (WJ) {
            float t = (0.666666687f * N) * invD;
#pragma unroll
            for (int k = 0; k < 3; ++k) R.J[k] = r * fmaf(-t, g[k], gN[k]);
        }
        if (WH) {
            float s1 = (0.666666687f * r) * invD;
            float s2 = ((1.11111116f * N * r) * invD) * invD;
            float r3 = 3.0f * r;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = i; j < 3; ++j) {
                    float base = (i == j) ? r3 : 0.0f;
                    float h = fmaf(s2, g[i] * g[j], fmaf(-s1, fmaf(gN[i], g[j], g[i] * gN[j]), base));
                    R.H[i * 3 + j] = h;
                    R.H[j * 3 + i] = h;
                }
        }
    }
    return R;
}

// Orientation sign of det[d1, d2, d3] when binary32 can certify it, else 2.
// The bound adds the rounding of the FP64 differences (3.01 u per term of the
// permanent) to the stage-A bound (7 + 56 u) u of the binary32 evaluation.
__device__ __forceinline__ int orient32_filter(const float* d1, const float* d2, const float* d3) {
    float vywz = d2[1] * d3[2], vzwy = d2[2] * d3[1];
    float vzwx = d2[2] * d3[0], vxwz = d2[0] * d3[2];
    float vxwy = d2[0] * d3[1], vywx = d2[1] * d3[0];
    float det = (d1[0] * (vywz - vzwy) + d1[1] * (vzwx - vxwz)) + d1[2] * (vxwy - vywx);
    float perm = (fabsf(d1[0]) * (fabsf(vywz) + fabsf(vzwy)) +
                  fabsf(d1[1]) * (fabsf(vzwx) + fabsf(vxwz))) +
                 fabsf(d1[2]) * (fabsf(vxwy) + fabsf(vywx));
    if (!(perm > 1e-30f) || !(perm < 1e30f)) return 2;
    float bound = 11.0f * kU32 * perm;
    if (det > bound) return 1;
    if (-det > bound) return -1;
    return 2;
}

// calTetQuality_AMIPS (LocalOperations.cpp:862-884) sentinel rule.
__device__ __forceinline__ double quality_from(int ori, double e) {
    if (ori != 1) return kMaxEnergy;
    if (isinf(e) || isnan(e) || e <= 0.0) return kMaxEnergy;
    return e;
}

// ---------------------------------------------------------------------------
// Point-triangle squared distance, Ericson's Voronoi-region closest point
// (Real-Time Collision Detection, 2005, sec. 5.1.5); degenerate face region
// falls back to the three edges.  Same operation order as the oracle.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double seg_nearest(const V3& p, const V3& a, const V3& b, V3& q) {
    V3 ab{b.x - a.x, b.y - a.y, b.z - a.z};
    V3 ap{p.x - a.x, p.y - a.y, p.z - a.z};
    double t = dot3(ap, ab), l = dot3(ab, ab);
    if (t <= 0.0 || l <= 0.0) {
        q = a;
    } else if (t >= l) {
        q = b;
    } else {
        double s = t / l;
        q = V3{a.x + s * ab.x, a.y + s * ab.y, a.z + s * ab.z};
    }
    V3 d{p.x - q.x, p.y - q.y, p.z - q.z};
    return dot3(d, d);
}

// Closest point q of triangle (a, b, c) to p and the squared distance
// |p - q|^2 (Voronoi regions, Ericson 2005 sec. 5.1.5); a triangle whose face
// region is degenerate falls back to the nearest of its edges ab, bc, ca
// (first one on ties).
__device__ __forceinline__ double point_tri_nearest(const V3& p, const V3& a, const V3& b,
                                                    const V3& c, V3& q) {
    V3 ab{b.x - a.x, b.y - a.y, b.z - a.z};
    V3 ac{c.x - a.x, c.y - a.y, c.z - a.z};
    V3 ap{p.x - a.x, p.y - a.y, p.z - a.z};
    double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) {
        q = a;
    } else {
        V3 bp{p.x - b.x, p.y - b.y, p.z - b.z};
        double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
        if (d3 >= 0.0 && d4 <= d3) {
            q = b;
        } else {
            double vc = d1 * d4 - d3 * d2;
            if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
                double v = d1 / (d1 - d3);
                q = V3{a.x + v * ab.x, a.y + v * ab.y, a.z + v * ab.z};
            } else {
                V3 cp{p.x - c.x, p.y - c.y, p.z - c.z};
                double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
                if (d6 >= 0.0 && d5 <= d6) {
                    q = c;
                } else {
                    double vb = d5 * d2 - d1 * d6;
                    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
                        double w = d2 / (d2 - d6);
                        q = V3{a.x + w * ac.x, a.y + w * ac.y, a.z + w * ac.z};
                    } else {
                        double va = d3 * d6 - d5 * d4;
                        double d43 = d4 - d3, d56 = d5 - d6;
                        if (va <= 0.0 && d43 >= 0.0 && d56 >= 0.0) {
                            double w = d43 / (d43 + d56);
                            q = V3{b.x + w * (c.x - b.x), b.y + w * (c.y - b.y),
                                   b.z + w * (c.z - b.z)};
                        } else {
                            double den = (va + vb) + vc;
                            if (!(den > 0.0)) {
                                V3 qa, qb;
                                double best = seg_nearest(p, a, b, q);
                                double d = seg_nearest(p, b, c, qa);
                                if (d < best) { best = d; q = qa; }
                                d = seg_nearest(p, c, a, qb);
                                if (d < best) { best = d; q = qb; }
                                return best;
                            }
                            double inv = 1.0 / den;
                            double v = vb * inv, w = vc * inv;
                            q = V3{(a.x + ab.x * v) + ac.x * w, (a.y + ab.y * v) + ac.y * w,
                                   (a.z + ab.z * v) + ac.z * w};
                        }
                    }
                }
            }
        }
    }
    V3 d{p.x - q.x, p.y - q.y, p.z - q.z};
    return dot3(d, d);
}

__device__ __forceinline__ double point_tri_sqdist(const V3& p, const V3& a, const V3& b,
                                                   const V3& c) {
    V3 q;
    return point_tri_nearest(p, a, b, c, q);
}

// Outside part of point_box_signed_squared_distance (mesh_AABB.cpp:201-220).
__device__ __forceinline__ double point_box_sqdist(const V3& p, const double* lo,
                                                   const double* hi) {
    double r = 0.0;
    if (p.x < lo[0]) { double d = p.x - lo[0]; r += d * d; }
    else if (p.x > hi[0]) { double d = p.x - hi[0]; r += d * d; }
    if (p.y < lo[1]) { double d = p.y - lo[1]; r += d * d; }
    else if (p.y > hi[1]) { double d = p.y - hi[1]; r += d * d; }
    if (p.z < lo[2]) { double d = p.z - lo[2]; r += d * d; }
    else if (p.z > hi[2]) { double d = p.z - hi[2]; r += d * d; }
    return r;
}

}  // namespace tw
