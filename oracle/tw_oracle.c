/*
 * tw_oracle.c -- CPU oracle (test infrastructure) for the TetWild query path.
 *
 * Build: see oracle/Makefile (-O2 -ffp-contract=off; no -ffast-math).
 * Only the tests, the smoke check and the CPU-baseline leg of bench.py use
 * this file.  See tw_oracle.h for the pinning of each routine.
 *
 * Arithmetic contract shared with the .cuh headers in tetwild_gb300/csrc: every floating
 * point expression below is evaluated left to right exactly as written, with
 * no fused multiply-add except where fma() is called explicitly (exact
 * two-product in the expansion arithmetic).
 */
#include "tw_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* =========================================================================
 * Inverse cube root x^(-1/3), x >= 0.
 *
 * The reference evaluates pow(pow(det, 2), -0.333333333333333)
 * (LocalOperations.cpp:78-80).  libm pow is not correctly rounded on every
 * platform, so the GPU and the oracle share this routine instead: exponent
 * reduction x = m * 2^(3q), m in [1, 8), then Newton-Raphson on
 * f(y) = y^-3 - m, y <- y + y*(1 - m*y^3)/3, three steps in binary32 from a
 * linear seed and two in binary64.  Every step is a plain IEEE operation, so
 * the result is bit-identical on any IEEE machine without FP contraction.
 * Accuracy: within 2 ulp of the exact value (measured against mpmath in the
 * tests); relative difference to the reference's pow(.., -0.333333333333333)
 * is below 3e-13 over the whole double range (the reference's exponent is
 * itself 3.3e-16 away from -1/3).
 * ========================================================================= */
static inline uint64_t tw_bits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double tw_from_bits(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }

double two_icbrt(double x)
{
    if (!(x == x)) return x;                 /* NaN */
    if (x <= 0.0) {
        if (x == 0.0) return INFINITY;       /* pow(0, -1/3) = +inf */
        return NAN;                          /* not reached: x = det^2 */
    }
    if (x == INFINITY) return 0.0;
    uint64_t u = tw_bits(x);
    int e = (int)((u >> 52) & 0x7ff);
    int ebias = 0;
    if (e == 0) {                            /* subnormal: scale by 2^54 */
        x = x * 18014398509481984.0;
        u = tw_bits(x);
        e = (int)((u >> 52) & 0x7ff);
        ebias = -54;
    }
    int ex = e - 1023 + ebias;               /* x = m1 * 2^ex, m1 in [1,2) */
    int q = (ex >= 0) ? ex / 3 : -((-ex + 2) / 3);   /* floor(ex / 3) */
    int rem = ex - 3 * q;                    /* 0, 1, 2 */
    double m = tw_from_bits((u & 0x000fffffffffffffULL) | ((uint64_t)(1023 + rem) << 52));
    /* m in [1, 8).  Seed for m^(-1/3) on [1,8): chord-like linear fit.     */
    float mf = (float)m;                     /* round to nearest binary32 */
    float yf = 0.9318f - 0.06015f * mf;
    const float third_f = 0.333333343f;
    for (int i = 0; i < 3; ++i) {
        float y3 = (yf * yf) * yf;
        float t = 1.0f - mf * y3;
        yf = yf + (yf * t) * third_f;
    }
    double y = (double)yf;
    const double third = 0.33333333333333331483;
    for (int i = 0; i < 2; ++i) {
        double y3 = (y * y) * y;
        double t = 1.0 - m * y3;
        y = y + (y * t) * third;
    }
    /* scale by 2^(-q) exactly */
    double s = tw_from_bits((uint64_t)(1023 - q) << 52);
    return y * s;
}

/* =========================================================================
 * Conformal AMIPS energy of a tet, its gradient and Hessian w.r.t. vertex 0.
 *
 * Reference: LocalOperations.cpp:28-81 (energy), :83-147 (Jacobian),
 * :149-291 (Hessian); the same expression is energy.ispc:39-60.  The
 * reference evaluates machine-generated expressions; this restatement
 * evaluates the same function in closed form:
 *   a = p0 - p3,  b = (p0 - 2 p1 + p3)/sqrt3,  c = (p0 + p1 + p3 - 3 p2)/sqrt6
 *   (rows of the map from the regular tet), N = |a|^2 + |b|^2 + |c|^2,
 *   D = a . (b x c),  E = N * (D^2)^(-1/3).
 * dD/dp0 = g = b x c + (c x a)/sqrt3 + (a x b)/sqrt6 (D is affine in p0),
 * dN/dp0 = gN = 2 (a + b/sqrt3 + c/sqrt6), d2N/dp0^2 = 3 I, so with
 * r = (D^2)^(-1/3):
 *   J = r (gN - (2/3)(N/D) g)
 *   H = 3 r I - (2/3)(r/D)(gN g^T + g gN^T) + (10/9)(N r/D^2) g g^T.
 * This closed form is the accurate one (within a few ulp of the exact
 * function); the reference form below is the one that agrees with the
 * reference's own rounding.  two_set_energy_form selects which one the
 * unsuffixed routines (and every caller in this file) use.
 * ========================================================================= */
#define TW_ISQ3 0.57735026918962576451   /* 1/sqrt(3) */
#define TW_ISQ6 0.40824829046386301637   /* 1/sqrt(6) */
#define TW_2_3  0.66666666666666662966   /* 2/3 */
#define TW_10_9 1.1111111111111111605    /* 10/9 */

static inline void tw_frame(const double* T, double a[3], double b[3], double c[3])
{
    for (int k = 0; k < 3; ++k) {
        double x0 = T[k], x1 = T[3 + k], x2 = T[6 + k], x3 = T[9 + k];
        a[k] = x0 - x3;
        b[k] = ((x0 - x1) + (x3 - x1)) * TW_ISQ3;
        c[k] = (((x0 - x2) + (x1 - x2)) + (x3 - x2)) * TW_ISQ6;
    }
}
static inline double tw_dot(const double u[3], const double v[3])
{
    return (u[0] * v[0] + u[1] * v[1]) + u[2] * v[2];
}
static inline void tw_cross(const double u[3], const double v[3], double w[3])
{
    w[0] = u[1] * v[2] - u[2] * v[1];
    w[1] = u[2] * v[0] - u[0] * v[2];
    w[2] = u[0] * v[1] - u[1] * v[0];
}

double two_amips_energy_cf(const double T[12])
{
    double a[3], b[3], c[3], bc[3];
    tw_frame(T, a, b, c);
    double N = (tw_dot(a, a) + tw_dot(b, b)) + tw_dot(c, c);
    tw_cross(b, c, bc);
    double D = tw_dot(a, bc);
    return N * two_icbrt(D * D);
}

/* Shared body of J and H. */
static void tw_amips_grad_terms(const double* T, double* N_, double* D_, double* r_,
                                double g[3], double gN[3])
{
    double a[3], b[3], c[3], bc[3], ca[3], ab[3];
    tw_frame(T, a, b, c);
    double N = (tw_dot(a, a) + tw_dot(b, b)) + tw_dot(c, c);
    tw_cross(b, c, bc);
    tw_cross(c, a, ca);
    tw_cross(a, b, ab);
    double D = tw_dot(a, bc);
    for (int k = 0; k < 3; ++k) {
        g[k] = (bc[k] + TW_ISQ3 * ca[k]) + TW_ISQ6 * ab[k];
        gN[k] = 2.0 * ((a[k] + TW_ISQ3 * b[k]) + TW_ISQ6 * c[k]);
    }
    *N_ = N;
    *D_ = D;
    *r_ = two_icbrt(D * D);
}

void two_amips_jacobian_cf(const double T[12], double J[3])
{
    double N, D, r, g[3], gN[3];
    tw_amips_grad_terms(T, &N, &D, &r, g, gN);
    double invD = 1.0 / D;
    double t = (TW_2_3 * N) * invD;
    for (int k = 0; k < 3; ++k) J[k] = r * (gN[k] - t * g[k]);
}

void two_amips_hessian_cf(const double T[12], double H[9])
{
    double N, D, r, g[3], gN[3];
    tw_amips_grad_terms(T, &N, &D, &r, g, gN);
    double invD = 1.0 / D;
    double s1 = (TW_2_3 * r) * invD;
    double s2 = (((TW_10_9 * N) * r) * invD) * invD;
    double r3 = 3.0 * r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double base = (i == j) ? r3 : 0.0;
            H[i * 3 + j] = (base - s1 * (gN[i] * g[j] + g[i] * gN[j])) + s2 * (g[i] * g[j]);
        }
}

/* =========================================================================
 * Reference form of the AMIPS energy, gradient and Hessian.
 *
 * LocalOperations.cpp:28-81, :83-147 and :149-291 evaluate machine-generated
 * expressions on the absolute coordinates with 15-digit coefficients.  For a
 * small tet away from the origin their terms cancel by up to ~1e4, so the
 * reference's result carries rounding of up to ~5e-12 relative; agreeing
 * with it to 1e-12 takes the same IEEE operations in the same order.  The
 * routines below perform them: each sum and product is grouped as the
 * generated code groups it (left to right), with its coefficients (RF_*).
 * IEEE addition and multiplication are commutative and negation is exact, so
 * the operand order inside one operation and the placement of signs are free;
 * only the grouping is kept.  Names: x0..z3 the coordinates of vertices 0..3;
 * bx, by, bz and cx, cy, cz the two scaled frame rows, each routine grouping
 * them as its generated code does; Lx0..Lz3 the per-coordinate linear forms
 * of the numerator.
 *
 * pow(d, 2) is d*d (pow is exact to the rounding of d*d), and
 * pow(s, -0.333333333333333) is rf_pow_m13: s^(-1/3) (two_icbrt) times
 * s^RF_DELTA, RF_DELTA = -0.333333333333333 + 1/3 = 3.5157e-16, applied as
 * the first-order factor 1 + RF_DELTA ln s (a correction below 2.6e-13 over
 * the double range; ln s to ~4% keeps its own error below 1e-17 relative).
 * Built with -DTW_RF_LIBM the two powers are libm's, which makes the three
 * routines bit-identical to the reference's own (a CPU test checks it).
 * ========================================================================= */
#define RF_B1   0.577350269189626      /* 1/sqrt3, as the generated code spells it */
#define RF_B2   1.15470053837925       /* 2/sqrt3 (not 2*RF_B1) */
#define RF_C1   0.408248290463863      /* 1/sqrt6 */
#define RF_C3   1.22474487139159       /* 3/sqrt6 */
#define RF_S2   0.707106781186548      /* 1/sqrt2 */
#define RF_2_3  0.666666666666667
#define RF_4_3  1.33333333333333
#define RF_4_9  0.444444444444444
#define RF_10_9 1.11111111111111
#define RF_TINY 1.85037170770859e-17   /* code-generation residue, kept (:267) */
#define RF_EXP  -0.333333333333333
#define RF_DELTA 3.515706244646329e-16 /* RF_EXP + 1/3 */
#define RF_LN2  0.6931471805599453

#ifdef TW_RF_LIBM
#define RF_SQ(d) pow((d), 2)
#define RF_POW_M13(s) pow((s), RF_EXP)
#else
#define RF_SQ(d) ((d) * (d))
#define RF_POW_M13(s) two_rf_pow_m13(s)
#endif

double two_rf_pow_m13(double s)
{
    double r = two_icbrt(s);
    if (!(r > 0.0) || r == INFINITY) return r;   /* NaN, s = inf, s = 0 */
    uint64_t u = tw_bits(s);
    int e = (int)((u >> 52) & 0x7ff);
    double m = tw_from_bits((u & 0x000fffffffffffffULL) | (1023ULL << 52));   /* [1, 2) */
    double ln = (double)(e - 1023) * RF_LN2 + (2.0 * (m - 1.0)) / (m + 1.0);
    return r + r * (RF_DELTA * ln);
}

double two_amips_energy_rf(const double T[12])
{
    const double x0 = T[0], y0 = T[1], z0 = T[2], x1 = T[3], y1 = T[4], z1 = T[5];
    const double x2 = T[6], y2 = T[7], z2 = T[8], x3 = T[9], y3 = T[10], z3 = T[11];
    const double bx = (RF_B1 * x0 - RF_B2 * x1) + RF_B1 * x3;
    const double cy = ((RF_C1 * y3 + RF_C1 * y0) + RF_C1 * y1) - RF_C3 * y2;
    const double by = (RF_B1 * y3 + RF_B1 * y0) - RF_B2 * y1;
    const double cx = ((RF_C1 * x0 - RF_C3 * x2) + RF_C1 * x1) + RF_C1 * x3;
    const double cz = ((RF_C1 * z0 + RF_C1 * z1) - RF_C3 * z2) + RF_C1 * z3;
    const double bz = (RF_B1 * z0 - RF_B2 * z1) + RF_B1 * z3;
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
    return -num * RF_POW_M13(RF_SQ(det));
}

void two_amips_jacobian_rf(const double T[12], double J[3])
{
    const double x0 = T[0], y0 = T[1], z0 = T[2], x1 = T[3], y1 = T[4], z1 = T[5];
    const double x2 = T[6], y2 = T[7], z2 = T[8], x3 = T[9], y3 = T[10], z3 = T[11];
    const double dy = y0 - y3, dz = z0 - z3, dx = x0 - x3;
    const double bx = (RF_B1 * x0 - RF_B2 * x1) + RF_B1 * x3;
    const double by = (RF_B1 * y0 - RF_B2 * y1) + RF_B1 * y3;
    const double bz = (RF_B1 * z0 - RF_B2 * z1) + RF_B1 * z3;
    const double cx = ((RF_C1 * x0 - RF_C3 * x2) + RF_C1 * x1) + RF_C1 * x3;
    const double cy = ((RF_C1 * y0 + RF_C1 * y1) - RF_C3 * y2) + RF_C1 * y3;
    const double cz = ((RF_C1 * z1 - RF_C3 * z2) + RF_C1 * z3) + RF_C1 * z0;
    const double czbx = cz * bx - bz * cx;
    const double cybx = cy * bx, cxby = cx * by;
    const double det = (czbx * dy - dz * (cybx - cxby)) - dx * (cz * by - bz * cy);
    const double r = RF_POW_M13(RF_SQ(det));
    const double sz = RF_S2 * z1 - RF_S2 * z2, sy = RF_S2 * y1 - RF_S2 * y2;
    const double sx = RF_S2 * x1 - RF_S2 * x2;
    const double hx = 0.5 * x2 + 0.5 * x1, hy = 0.5 * y1 + 0.5 * y2, hz = 0.5 * z1 + 0.5 * z2;
    const double num =
        y0 * ((0.5 * y3 - 1.5 * y0) + hy) + z1 * (((0.5 * z2 - 1.5 * z1) + 0.5 * z3) + 0.5 * z0) +
        z2 * (((0.5 * z1 - 1.5 * z2) + 0.5 * z3) + 0.5 * z0) + z3 * ((hz - 1.5 * z3) + 0.5 * z0) +
        y3 * ((0.5 * y0 - 1.5 * y3) + hy) + x2 * (((0.5 * x0 - 1.5 * x2) + 0.5 * x1) + 0.5 * x3) +
        y1 * (((0.5 * y0 + 0.5 * y3) - 1.5 * y1) + 0.5 * y2) +
        y2 * (((0.5 * y0 + 0.5 * y3) + 0.5 * y1) - 1.5 * y2) + x0 * ((hx - 1.5 * x0) + 0.5 * x3) +
        x1 * (((0.5 * x2 + 0.5 * x0) - 1.5 * x1) + 0.5 * x3) + x3 * ((0.5 * x0 + hx) - 1.5 * x3) +
        z0 * ((0.5 * z3 + hz) - 1.5 * z0);
    const double w = (RF_2_3 * num) / det;
    const double q0 = ((sz * (y3 - y0) - sy * (z3 - z0)) - bz * cy) + by * cz;
    J[0] = -(r * ((((x2 - 3.0 * x0) + w * q0) + x1) + x3));
    J[1] = r * ((((3.0 * y0 - y3) - y1) - y2) + w * ((czbx + dz * sx) - dx * sz));
    J[2] = r * (((((-z1) - z2) - z3) + w * (((-(dy * sx)) - cybx) + cxby + dx * sy)) + 3.0 * z0);
}

void two_amips_hessian_rf(const double T[12], double H[9])
{
    const double x0 = T[0], y0 = T[1], z0 = T[2], x1 = T[3], y1 = T[4], z1 = T[5];
    const double x2 = T[6], y2 = T[7], z2 = T[8], x3 = T[9], y3 = T[10], z3 = T[11];
    const double dz = z0 - z3, dx = x0 - x3, dy = y0 - y3;
    const double bx = (RF_B1 * x0 - RF_B2 * x1) + RF_B1 * x3;
    const double by = (RF_B1 * y0 - RF_B2 * y1) + RF_B1 * y3;
    const double bz = (RF_B1 * z0 - RF_B2 * z1) + RF_B1 * z3;
    const double cx = ((RF_C1 * x0 + RF_C1 * x1) - RF_C3 * x2) + RF_C1 * x3;
    const double cy = ((RF_C1 * y0 + RF_C1 * y1) - RF_C3 * y2) + RF_C1 * y3;
    const double cz = ((RF_C1 * z0 + RF_C1 * z1) - RF_C3 * z2) + RF_C1 * z3;
    const double bxcy = bx * cy, bycx = by * cx;
    const double mx = dz * (bxcy - bycx);
    const double bycz = by * cz, cybz = cy * bz;
    const double myz = bycz - cybz;
    const double my = dx * myz;
    const double bxcz = bx * cz, cxbz = cx * bz;
    const double mxz = bxcz - cxbz;
    const double mz = dy * mxz;
    const double det = (mx + my) - mz;
    const double det2 = RF_SQ(det);
    const double r = RF_POW_M13(det2);
    const double lx = ((x2 - 3.0 * x0) + x1) + x3;
    const double sy = RF_S2 * y1 - RF_S2 * y2;
    const double dzsy = dz * sy;
    const double sz = RF_S2 * z1 - RF_S2 * z2;
    const double dysz = dy * sz;
    const double u = (myz + dzsy) - dysz;
    const double k43 = RF_4_3 / det;
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
    const double k49n = (RF_4_9 * idet2) * num;
    const double nd = idet2 * num;
    const double ineg = 1.0 / (-det);
    const double rneg = ineg * r;
    const double sx = RF_S2 * x1 - RF_S2 * x2;
    const double v1 = (((RF_2_3 * bx) * cz + (RF_2_3 * dz) * sx) - (RF_2_3 * cx) * bz) -
                      (RF_2_3 * dx) * sz;
    const double ly = ((y1 - 3.0 * y0) + y2) + y3;
    const double ey = y3 - y0, ez = z3 - z0;
    const double v2 = (((-RF_2_3 * sy) * ez + (RF_2_3 * sz) * ey) + (RF_2_3 * by) * cz) -
                      (RF_2_3 * bz) * cy;
    const double dzsx = dz * sx, dxsz = dx * sz;
    const double p = (dzsx - dxsz) + mxz;
    const double q = ((sz * ey - sy * ez) + by * cz) - bz * cy;
    const double a1 = ((((RF_4_9 * p) * q) * num) * ineg + lx * v1) - ly * v2;
    const double tiny = (RF_TINY * z0) * Lz0 + (RF_TINY * y0) * Ly0 + (RF_TINY * y1) * Ly1 +
                        (RF_TINY * y2) * Ly2 + (RF_TINY * y3) * Ly3 + (RF_TINY * z3) * Lz3 +
                        (RF_TINY * x2) * Lx2 + (RF_TINY * z1) * Lz1 + (RF_TINY * z2) * Lz2 +
                        (RF_TINY * x0) * Lx0 + (RF_TINY * x1) * Lx1 + (RF_TINY * Lx3) * x3;
    const double un = (u * num) * ineg;
    const double v3 = (((RF_2_3 * by) * cx - (RF_2_3 * bx) * cy) + (RF_2_3 * dx) * sy) -
                      (RF_2_3 * dy) * sx;
    const double lz = ((z3 - 3.0 * z0) + z1) + z2;
    const double t = ((bycx - bxcy) + dx * sy) - dy * sx;
    const double tn = ((RF_4_9 * t) * num) * ineg;
    const double a2 = (q * tn + v3 * lx) - lz * v2;
    const double ex = x3 - x0;
    const double w1 = (num * ineg) * (((ex * sz - sx * ez) + bx * cz) - cx * bz);
    const double s = ((dxsz - dzsx) - bxcz) + cxbz;
    const double a3 = ((-p) * tn + v3 * ly) + lz * v1;
    const double w2 = (num * ineg) * (((ex * (-sy) + sx * ey) - bx * cy) + cx * by);
    H[0] = r * ((((lx * u) * k43 - RF_SQ(u) * k49n) + ((RF_2_3 * u) * nd) * (((cybz - bycz) - dzsy) + dysz)) + 3.0);
    H[1] = rneg * ((a1 - tiny * z1) + un * v1);
    H[2] = rneg * (un * v3 + a2);
    H[3] = rneg * (a1 + w1 * v2);
    H[4] = r * ((((-RF_SQ(s)) * k49n + (s * k43) * ly) + (s * nd) * v1) + 3.0);
    H[5] = rneg * (((-tiny) * x1 - v3 * w1) + a3);
    H[6] = rneg * (((-tiny) * y1 + a2) + w2 * v2);
    H[7] = rneg * (a3 - w2 * v1);
    H[8] = r * ((((-lz) * t) * k43 - (RF_10_9 * RF_SQ(t)) * nd) + 3.0);
}

static int tw_energy_form = TWO_FORM_REFERENCE;

void two_set_energy_form(int form) { tw_energy_form = form; }
int two_get_energy_form(void) { return tw_energy_form; }

double two_amips_energy(const double T[12])
{
    return tw_energy_form == TWO_FORM_CLOSED ? two_amips_energy_cf(T) : two_amips_energy_rf(T);
}
void two_amips_jacobian(const double T[12], double J[3])
{
    if (tw_energy_form == TWO_FORM_CLOSED)
        two_amips_jacobian_cf(T, J);
    else
        two_amips_jacobian_rf(T, J);
}
void two_amips_hessian(const double T[12], double H[9])
{
    if (tw_energy_form == TWO_FORM_CLOSED)
        two_amips_hessian_cf(T, H);
    else
        two_amips_hessian_rf(T, H);
}

/* =========================================================================
 * Exact orientation and collinearity.
 *
 * CGAL::orientation(p,q,r,s) on Epick points (LocalOperations.cpp:544,
 * :755, :864; VertexSmoother.cpp:166) is POSITIVE iff det[q-p, r-p, s-p] > 0.
 * Method (Shewchuk, "Adaptive Precision Floating-Point Arithmetic and Fast
 * Robust Geometric Predicates", 1997): a floating-point evaluation with the
 * paper's forward error bound (7 + 56 eps) eps * permanent, and, when the
 * filter cannot decide, an exact evaluation with nonoverlapping expansions
 * (Two-Sum, Two-Diff, Two-Product via fma, Grow-Expansion and
 * Scale-Expansion, both with zero elimination).
 * ========================================================================= */
#define TW_EPS 1.1102230246251565404e-16      /* 2^-53 */
#define TW_O3D_BOUND ((7.0 + 56.0 * TW_EPS) * TW_EPS)

static inline void tw_two_sum(double a, double b, double* x, double* y)
{
    double s = a + b, bv = s - a, av = s - bv, br = b - bv, ar = a - av;
    *x = s;
    *y = ar + br;
}
static inline void tw_two_diff(double a, double b, double* x, double* y)
{
    double d = a - b, bv = a - d, av = d + bv, br = bv - b, ar = a - av;
    *x = d;
    *y = ar + br;
}
static inline void tw_fast_two_sum(double a, double b, double* x, double* y)
{
    double s = a + b, bv = s - a;
    *x = s;
    *y = b - bv;
}
static inline void tw_two_prod(double a, double b, double* x, double* y)
{
    double p = a * b;
    *x = p;
    *y = fma(a, b, -p);
}
/* h = e + b  (Grow-Expansion with zero elimination); returns length. */
static int tw_grow(const double* e, int n, double b, double* h)
{
    double Q = b, hh;
    int k = 0;
    for (int i = 0; i < n; ++i) {
        tw_two_sum(Q, e[i], &Q, &hh);
        if (hh != 0.0) h[k++] = hh;
    }
    if (Q != 0.0 || k == 0) h[k++] = Q;
    return k;
}
/* h = e + f by repeated growth; h must hold n + m entries; tmp likewise. */
static int tw_sum(const double* e, int n, const double* f, int m, double* h, double* tmp)
{
    int k = n;
    for (int i = 0; i < n; ++i) h[i] = e[i];
    for (int j = 0; j < m; ++j) {
        k = tw_grow(h, k, f[j], tmp);
        for (int i = 0; i < k; ++i) h[i] = tmp[i];
    }
    return k;
}
/* h = e * b (Scale-Expansion with zero elimination); h holds 2n entries. */
static int tw_scale(const double* e, int n, double b, double* h)
{
    double Q, hh, p1, p0, sum;
    int k = 0;
    tw_two_prod(e[0], b, &Q, &hh);
    if (hh != 0.0) h[k++] = hh;
    for (int i = 1; i < n; ++i) {
        tw_two_prod(e[i], b, &p1, &p0);
        tw_two_sum(Q, p0, &sum, &hh);
        if (hh != 0.0) h[k++] = hh;
        tw_fast_two_sum(p1, sum, &Q, &hh);
        if (hh != 0.0) h[k++] = hh;
    }
    if (Q != 0.0 || k == 0) h[k++] = Q;
    return k;
}
/* product of two expansions (each <= 2 terms) -> <= 8 terms */
static int tw_mul22(const double* x, int nx, const double* y, int ny, double* h)
{
    double t0[4], t1[4], tmp[8];
    int k0 = tw_scale(y, ny, x[0], t0);
    if (nx == 1) {
        for (int i = 0; i < k0; ++i) h[i] = t0[i];
        return k0;
    }
    int k1 = tw_scale(y, ny, x[1], t1);
    return tw_sum(t0, k0, t1, k1, h, tmp);
}
static inline int tw_diff_exp(double a, double b, double* e)
{
    double x, y;
    tw_two_diff(a, b, &x, &y);
    if (y == 0.0) { e[0] = x; return 1; }
    e[0] = y;
    e[1] = x;
    return 2;
}
static inline int tw_sign_exp(const double* e, int n)
{
    double top = e[n - 1];
    return (top > 0.0) - (top < 0.0);
}
/* exact (u1 * v2 - u2 * v1) with u,v 2-term expansions -> <= 16 terms */
static int tw_minor(const double* u1, int n1, const double* v2, int m2, const double* u2, int n2,
                    const double* v1, int m1, double* h)
{
    double p[8], q[8], tmp[16];
    int kp = tw_mul22(u1, n1, v2, m2, p);
    int kq = tw_mul22(u2, n2, v1, m1, q);
    for (int i = 0; i < kq; ++i) q[i] = -q[i];
    return tw_sum(p, kp, q, kq, h, tmp);
}

int two_orient3d_exact(const double p[3], const double q[3], const double r[3], const double s[3])
{
    double u[3][2], v[3][2], w[3][2];
    int nu[3], nv[3], nw[3];
    for (int k = 0; k < 3; ++k) {
        nu[k] = tw_diff_exp(q[k], p[k], u[k]);
        nv[k] = tw_diff_exp(r[k], p[k], v[k]);
        nw[k] = tw_diff_exp(s[k], p[k], w[k]);
    }
    /* det = ux (vy wz - vz wy) + uy (vz wx - vx wz) + uz (vx wy - vy wx) */
    double m[16], t0[32], t1[32], term[64], acc[192], acc2[192], tmp[192];
    int nacc = 0;
    static const int ia[3] = {1, 2, 0}, ib[3] = {2, 0, 1};
    for (int k = 0; k < 3; ++k) {
        int i = ia[k], j = ib[k];
        int nm = tw_minor(v[i], nv[i], w[j], nw[j], v[j], nv[j], w[i], nw[i], m);
        int k0 = tw_scale(m, nm, u[k][0], t0);
        int nt;
        if (nu[k] == 2) {
            int k1 = tw_scale(m, nm, u[k][1], t1);
            nt = tw_sum(t0, k0, t1, k1, term, tmp);
        } else {
            for (int z = 0; z < k0; ++z) term[z] = t0[z];
            nt = k0;
        }
        if (nacc == 0) {
            for (int z = 0; z < nt; ++z) acc[z] = term[z];
            nacc = nt;
        } else {
            nacc = tw_sum(acc, nacc, term, nt, acc2, tmp);
            for (int z = 0; z < nacc; ++z) acc[z] = acc2[z];
        }
    }
    return tw_sign_exp(acc, nacc);
}

int two_orient3d(const double p[3], const double q[3], const double r[3], const double s[3])
{
    for (int k = 0; k < 3; ++k)
        if (!isfinite(p[k]) || !isfinite(q[k]) || !isfinite(r[k]) || !isfinite(s[k])) return 0;
    double ux = q[0] - p[0], uy = q[1] - p[1], uz = q[2] - p[2];
    double vx = r[0] - p[0], vy = r[1] - p[1], vz = r[2] - p[2];
    double wx = s[0] - p[0], wy = s[1] - p[1], wz = s[2] - p[2];
    double vywz = vy * wz, vzwy = vz * wy;
    double vzwx = vz * wx, vxwz = vx * wz;
    double vxwy = vx * wy, vywx = vy * wx;
    double det = (ux * (vywz - vzwy) + uy * (vzwx - vxwz)) + uz * (vxwy - vywx);
    double perm = (fabs(ux) * (fabs(vywz) + fabs(vzwy)) + fabs(uy) * (fabs(vzwx) + fabs(vxwz))) +
                  fabs(uz) * (fabs(vxwy) + fabs(vywx));
    double bound = TW_O3D_BOUND * perm;
    if (det > bound) return 1;
    if (-det > bound) return -1;
    return two_orient3d_exact(p, q, r, s);
}

/* CGAL collinear(p,q,r) (Triangle_3f::is_degenerate, LocalOperations.cpp:1048):
 * all three 2x2 minors of [p-r, q-r] vanish, decided exactly. */
static int tw_minor2_zero(double px, double py, double qx, double qy, double rx, double ry)
{
    double a[2], b[2], c[2], d[2], m[16];
    int na = tw_diff_exp(px, rx, a), nb = tw_diff_exp(qy, ry, b);
    int nc = tw_diff_exp(py, ry, c), nd = tw_diff_exp(qx, rx, d);
    int k = tw_minor(a, na, b, nb, c, nc, d, nd, m);
    return tw_sign_exp(m, k) == 0;
}
int two_collinear(const double a[3], const double b[3], const double c[3])
{
    if (!tw_minor2_zero(a[0], a[1], b[0], b[1], c[0], c[1])) return 0;
    if (!tw_minor2_zero(a[0], a[2], b[0], b[2], c[0], c[2])) return 0;
    return tw_minor2_zero(a[1], a[2], b[1], b[2], c[1], c[2]);
}

/* ========================================================================= */
int two_tet_flip(const double T[12])
{
    return two_orient3d(T, T + 3, T + 6, T + 9) != 1;
}

double two_tet_quality(const double T[12])
{
    /* calTetQuality_AMIPS, LocalOperations.cpp:862-884 */
    if (two_orient3d(T, T + 3, T + 6, T + 9) != 1) return TWO_MAX_ENERGY;
    double e = two_amips_energy(T);
    if (isinf(e) || isnan(e) || e <= 0.0) return TWO_MAX_ENERGY;
    return e;
}

/* =========================================================================
 * Point-triangle squared distance: closest point by Voronoi regions
 * (Ericson, "Real-Time Collision Detection", 2005, sec. 5.1.5), then
 * d^2 = |p - q|^2.  Stands in for geogram's
 * Geom::point_triangle_squared_distance (DistanceQuery.h:36,
 * mesh_AABB.cpp:168), which is not part of the reference sources.  A
 * triangle whose face region is degenerate (va + vb + vc <= 0) falls back to
 * the nearest of its three edges.
 * ========================================================================= */
static double tw_seg_sqdist(const double p[3], const double a[3], const double b[3], double q[3])
{
    double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    double ap[3] = {p[0] - a[0], p[1] - a[1], p[2] - a[2]};
    double t = tw_dot(ap, ab), l = tw_dot(ab, ab);
    if (t <= 0.0 || l <= 0.0) {
        q[0] = a[0]; q[1] = a[1]; q[2] = a[2];
    } else if (t >= l) {
        q[0] = b[0]; q[1] = b[1]; q[2] = b[2];
    } else {
        double s = t / l;
        for (int k = 0; k < 3; ++k) q[k] = a[k] + s * ab[k];
    }
    double d[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
    return tw_dot(d, d);
}

double two_point_triangle_sqdist(const double p[3], const double a[3], const double b[3],
                                 const double c[3], double q_out[3])
{
    double q[3];
    double ab[3], ac[3], ap[3], bp[3], cp[3];
    for (int k = 0; k < 3; ++k) {
        ab[k] = b[k] - a[k];
        ac[k] = c[k] - a[k];
        ap[k] = p[k] - a[k];
    }
    double d1 = tw_dot(ab, ap), d2 = tw_dot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) {
        q[0] = a[0]; q[1] = a[1]; q[2] = a[2];
        goto done;
    }
    for (int k = 0; k < 3; ++k) bp[k] = p[k] - b[k];
    double d3 = tw_dot(ab, bp), d4 = tw_dot(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) {
        q[0] = b[0]; q[1] = b[1]; q[2] = b[2];
        goto done;
    }
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        double v = d1 / (d1 - d3);
        for (int k = 0; k < 3; ++k) q[k] = a[k] + v * ab[k];
        goto done;
    }
    for (int k = 0; k < 3; ++k) cp[k] = p[k] - c[k];
    double d5 = tw_dot(ab, cp), d6 = tw_dot(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) {
        q[0] = c[0]; q[1] = c[1]; q[2] = c[2];
        goto done;
    }
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        double w = d2 / (d2 - d6);
        for (int k = 0; k < 3; ++k) q[k] = a[k] + w * ac[k];
        goto done;
    }
    double va = d3 * d6 - d5 * d4;
    double d43 = d4 - d3, d56 = d5 - d6;
    if (va <= 0.0 && d43 >= 0.0 && d56 >= 0.0) {
        double w = d43 / (d43 + d56);
        for (int k = 0; k < 3; ++k) q[k] = b[k] + w * (c[k] - b[k]);
        goto done;
    }
    {
        double den = (va + vb) + vc;
        if (!(den > 0.0)) {
            /* degenerate face region: nearest of the three edges */
            double qa[3], qb[3];
            double best = tw_seg_sqdist(p, a, b, q);
            double d = tw_seg_sqdist(p, b, c, qa);
            if (d < best) { best = d; q[0] = qa[0]; q[1] = qa[1]; q[2] = qa[2]; }
            d = tw_seg_sqdist(p, c, a, qb);
            if (d < best) { best = d; q[0] = qb[0]; q[1] = qb[1]; q[2] = qb[2]; }
            if (q_out) { q_out[0] = q[0]; q_out[1] = q[1]; q_out[2] = q[2]; }
            return best;
        }
        double inv = 1.0 / den;
        double v = vb * inv, w = vc * inv;
        for (int k = 0; k < 3; ++k) q[k] = (a[k] + ab[k] * v) + ac[k] * w;
    }
done:
    if (q_out) { q_out[0] = q[0]; q_out[1] = q[1]; q_out[2] = q[2]; }
    {
        double d[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
        return tw_dot(d, d);
    }
}

/* point_box_signed_squared_distance, mesh_AABB.cpp:201-220, outside part
 * (a point inside the box gets 0; the reference returns a negative number
 * there, which prunes identically since both are <= any threshold >= 0). */
double two_point_box_sqdist(const double p[3], const double lo[3], const double hi[3])
{
    double r = 0.0;
    for (int k = 0; k < 3; ++k) {
        if (p[k] < lo[k]) {
            double d = p[k] - lo[k];
            r += d * d;
        } else if (p[k] > hi[k]) {
            double d = p[k] - hi[k];
            r += d * d;
        }
    }
    return r;
}

/* =========================================================================
 * sampleTriangle, Common.cpp:143-228, with geogram vec3 semantics:
 *   length2(v) = (x*x + y*y) + z*z, length = sqrt(length2),
 *   distance(a,b) = sqrt(((a-b).x^2 + (a-b).y^2) + (a-b).z^2),
 *   normalize(v) = (1/length(v)) * v  (when length > 1e-30),
 *   s * v and v * s scale each component, v / s divides each component.
 * Samples are emitted in the reference order.
 * ========================================================================= */
typedef struct { double x, y, z; } tw_v3;
static inline tw_v3 v3(double x, double y, double z) { tw_v3 r = {x, y, z}; return r; }
static inline tw_v3 v3_sub(tw_v3 a, tw_v3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline tw_v3 v3_add(tw_v3 a, tw_v3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline tw_v3 v3_mul(tw_v3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline tw_v3 s_mul(double s, tw_v3 a) { return v3(s * a.x, s * a.y, s * a.z); }
static inline tw_v3 v3_div(tw_v3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline double v3_len2(tw_v3 a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }
static inline double v3_len(tw_v3 a) { return sqrt(v3_len2(a)); }
static inline double v3_dist(tw_v3 a, tw_v3 b) { return v3_len(v3_sub(a, b)); }
static inline double v3_dot(tw_v3 a, tw_v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline tw_v3 v3_cross(tw_v3 a, tw_v3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline tw_v3 v3_normalize(tw_v3 a)
{
    double s = v3_len(a);
    if (s > 1e-30) s = 1.0 / s;
    return s_mul(s, a);
}
/* double -> int conversion as C does for values in range; clamps outside it
 * (the reference's behaviour there is undefined). */
static inline int tw_trunc_int(double x)
{
    if (!(x == x)) return 0;
    if (x >= 2147483647.0) return 2147483647;
    if (x <= -2147483648.0) return -2147483647 - 1;
    return (int)x;
}

#define TW_EMIT(P)                                                         \
    do {                                                                   \
        if (cnt < cap && out) {                                            \
            out[3 * cnt] = (P).x; out[3 * cnt + 1] = (P).y; out[3 * cnt + 2] = (P).z; \
        }                                                                  \
        ++cnt;                                                             \
    } while (0)

int64_t two_sample_triangle(const double vv[9], double sd, double* out, int64_t cap)
{
    int64_t cnt = 0;
    const double sqrt3_2 = sqrt(3.0) / 2.0;
    tw_v3 vs[3] = {v3(vv[0], vv[1], vv[2]), v3(vv[3], vv[4], vv[5]), v3(vv[6], vv[7], vv[8])};
    double ls[3];
    for (int i = 0; i < 3; ++i) ls[i] = v3_len2(v3_sub(vs[i], vs[(i + 1) % 3]));
    /* std::minmax_element: first smallest, LAST largest */
    int max_i = 0;
    for (int i = 1; i < 3; ++i)
        if (!(ls[i] < ls[max_i])) max_i = i;
    double N = sqrt(ls[max_i]) / sd;
    if (N <= 1) {
        for (int i = 0; i < 3; ++i) TW_EMIT(vs[i]);
        return cnt;
    }
    if (N == (double)tw_trunc_int(N)) N -= 1;

    tw_v3 v0 = vs[max_i], v1 = vs[(max_i + 1) % 3], v2 = vs[(max_i + 2) % 3];
    tw_v3 n_v0v1 = v3_normalize(v3_sub(v1, v0));
    for (int n = 0; n <= N; ++n) TW_EMIT(v3_add(v0, v3_mul(v3_mul(n_v0v1, sd), (double)n)));
    TW_EMIT(v1);

    double h = v3_dist(v3_add(v3_div(s_mul(v3_dot(v3_sub(v2, v0), v3_sub(v1, v0)), v3_sub(v1, v0)), ls[max_i]), v0), v2);
    int M = tw_trunc_int(h / (sqrt3_2 * sd));
    if (M < 1) {
        TW_EMIT(v2);
        return cnt;
    }
    tw_v3 n_v0v2 = v3_normalize(v3_sub(v2, v0));
    tw_v3 n_v1v2 = v3_normalize(v3_sub(v2, v1));
    double cr0 = v3_len(v3_cross(v3_sub(v2, v0), v3_sub(v1, v0)));
    double cr1 = v3_len(v3_cross(v3_sub(v2, v1), v3_sub(v0, v1)));
    double sin_v0 = cr0 / (v3_dist(v0, v2) * v3_dist(v0, v1));
    double tan_v0 = cr0 / v3_dot(v3_sub(v2, v0), v3_sub(v1, v0));
    double tan_v1 = cr1 / v3_dot(v3_sub(v2, v1), v3_sub(v0, v1));
    double sin_v1 = cr1 / (v3_dist(v1, v2) * v3_dist(v0, v1));
    (void)tan_v1;
    for (int m = 1; m <= M; ++m) {
        int n = tw_trunc_int(sqrt3_2 / tan_v0 * m + 0.5);
        int n1 = tw_trunc_int(sqrt3_2 / tan_v0 * m);
        if (m % 2 == 0 && n == n1) n += 1;
        tw_v3 v0_m = v3_add(v0, s_mul((double)m * sqrt3_2 * sd / sin_v0, n_v0v2));
        tw_v3 v1_m = v3_add(v1, s_mul((double)m * sqrt3_2 * sd / sin_v1, n_v1v2));
        if (v3_dist(v0_m, v1_m) <= sd) break;
        double delta_d = (((double)n + (m % 2) / 2.0) - (double)m * sqrt3_2 / tan_v0) * sd;
        tw_v3 v = v3_add(v0_m, s_mul(delta_d, n_v0v1));
        int N1 = tw_trunc_int(v3_dist(v, v1_m) / sd);
        for (int i = 0; i <= N1; ++i) TW_EMIT(v3_add(v, v3_mul(s_mul((double)i, n_v0v1), sd)));
    }
    TW_EMIT(v2);

    N = sqrt(ls[(max_i + 1) % 3]) / sd;
    if (N > 1) {
        if (N == (double)tw_trunc_int(N)) N -= 1;
        tw_v3 nv = v3_normalize(v3_sub(v2, v1));
        for (int n = 1; n <= N; ++n) TW_EMIT(v3_add(v1, v3_mul(v3_mul(nv, sd), (double)n)));
    }
    N = sqrt(ls[(max_i + 2) % 3]) / sd;
    if (N > 1) {
        if (N == (double)tw_trunc_int(N)) N -= 1;
        tw_v3 nv = v3_normalize(v3_sub(v0, v2));
        for (int n = 1; n <= N; ++n) TW_EMIT(v3_add(v2, v3_mul(v3_mul(nv, sd), (double)n)));
    }
    return cnt;
}

int64_t two_sample_count(const double v[9], double sd)
{
    return two_sample_triangle(v, sd, NULL, 0);
}

/* =========================================================================
 * Surface tree for the envelope: the layout of geogram's
 * MeshFacetsAABBWithEps (mesh_AABB.cpp:356-379): facets reordered by a
 * recursive median split of their centroids, an implicit binary tree over
 * index ranges (node n covers [b,e), children 2n and 2n+1, split at
 * b + (e-b)/2), boxes = exact min/max of the facet vertices.
 *
 * Query semantics (isPointOutEnvelop, LocalOperations.cpp:1034-1044):
 * out <=> min over facets of sqdist(p, f) > eps2.  The traversal stops at the
 * first facet with sqdist <= eps2 (facet_in_envelope_recursive,
 * mesh_AABB.cpp:482-548) and prunes a box only when its distance exceeds
 * (eps + tau)^2, tau = 64 * 2^-53 * max(|coord|): a box is never pruned
 * while it may hold a facet whose computed distance is <= eps2, so the
 * decision equals the brute-force decision bit for bit.
 * ========================================================================= */
struct two_surface {
    int32_t nf;
    double* tri;      /* 9 doubles per facet, tree order */
    int32_t* fid;     /* input facet index of each tree position */
    double* box;      /* 6 doubles per node (lo, hi), implicit indexing */
    int32_t nbox;
    double scale;     /* max |coordinate| of the surface */
};

typedef struct { double c; int32_t id; } tw_key;
static int tw_key_cmp(const void* x, const void* y)
{
    const tw_key* a = (const tw_key*)x;
    const tw_key* b = (const tw_key*)y;
    if (a->c < b->c) return -1;
    if (a->c > b->c) return 1;
    return (a->id > b->id) - (a->id < b->id);
}
static void tw_median_order(const double* cen, int32_t* ids, int32_t n, int axis, tw_key* scratch)
{
    if (n <= 1) return;
    for (int32_t i = 0; i < n; ++i) {
        scratch[i].c = cen[3 * ids[i] + axis];
        scratch[i].id = ids[i];
    }
    qsort(scratch, (size_t)n, sizeof(tw_key), tw_key_cmp);
    for (int32_t i = 0; i < n; ++i) ids[i] = scratch[i].id;
    int32_t m = n / 2;
    tw_median_order(cen, ids, m, (axis + 1) % 3, scratch);
    tw_median_order(cen, ids + m, n - m, (axis + 1) % 3, scratch);
}
static int32_t tw_max_node(int32_t node, int32_t b, int32_t e)
{
    if (b + 1 == e) return node;
    int32_t m = b + (e - b) / 2;
    int32_t l = tw_max_node(2 * node, b, m), r = tw_max_node(2 * node + 1, m, e);
    return l > r ? l : r;
}
static void tw_init_boxes(two_surface* s, int32_t node, int32_t b, int32_t e)
{
    double* B = s->box + 6 * node;
    if (b + 1 == e) {
        const double* t = s->tri + 9 * b;
        for (int k = 0; k < 3; ++k) {
            double lo = t[k], hi = t[k];
            for (int v = 1; v < 3; ++v) {
                if (t[3 * v + k] < lo) lo = t[3 * v + k];
                if (t[3 * v + k] > hi) hi = t[3 * v + k];
            }
            B[k] = lo;
            B[3 + k] = hi;
        }
        return;
    }
    int32_t m = b + (e - b) / 2;
    tw_init_boxes(s, 2 * node, b, m);
    tw_init_boxes(s, 2 * node + 1, m, e);
    const double* L = s->box + 12 * node;
    const double* R = L + 6;
    for (int k = 0; k < 3; ++k) {
        B[k] = L[k] < R[k] ? L[k] : R[k];
        B[3 + k] = L[3 + k] > R[3 + k] ? L[3 + k] : R[3 + k];
    }
}

two_surface* two_surface_build(const double* V, int32_t nV, const int32_t* F, int32_t nF)
{
    (void)nV;
    if (nF <= 0) return NULL;
    two_surface* s = (two_surface*)calloc(1, sizeof(two_surface));
    s->nf = nF;
    double* cen = (double*)malloc(sizeof(double) * 3 * (size_t)nF);
    int32_t* ids = (int32_t*)malloc(sizeof(int32_t) * (size_t)nF);
    tw_key* scratch = (tw_key*)malloc(sizeof(tw_key) * (size_t)nF);
    double scale = 0.0;
    for (int32_t f = 0; f < nF; ++f) {
        ids[f] = f;
        for (int k = 0; k < 3; ++k) {
            double c = 0.0;
            for (int v = 0; v < 3; ++v) {
                double x = V[3 * F[3 * f + v] + k];
                c += x;
                if (fabs(x) > scale) scale = fabs(x);
            }
            cen[3 * f + k] = c / 3.0;
        }
    }
    tw_median_order(cen, ids, nF, 0, scratch);
    s->tri = (double*)malloc(sizeof(double) * 9 * (size_t)nF);
    s->fid = (int32_t*)malloc(sizeof(int32_t) * (size_t)nF);
    for (int32_t i = 0; i < nF; ++i) s->fid[i] = ids[i];
    for (int32_t i = 0; i < nF; ++i)
        for (int v = 0; v < 3; ++v)
            for (int k = 0; k < 3; ++k) s->tri[9 * i + 3 * v + k] = V[3 * F[3 * ids[i] + v] + k];
    s->nbox = tw_max_node(1, 0, nF) + 1;
    s->box = (double*)calloc((size_t)s->nbox * 6, sizeof(double));
    tw_init_boxes(s, 1, 0, nF);
    s->scale = scale;
    free(cen);
    free(ids);
    free(scratch);
    return s;
}

void two_surface_free(two_surface* s)
{
    if (!s) return;
    free(s->tri);
    free(s->fid);
    free(s->box);
    free(s);
}

static double tw_prune_threshold(const two_surface* s, const double p[3], double eps2)
{
    double m = s->scale;
    for (int k = 0; k < 3; ++k)
        if (fabs(p[k]) > m) m = fabs(p[k]);
    double eps = sqrt(eps2);
    double tau = 64.0 * TW_EPS * m + 4.0 * TW_EPS * eps;
    return (eps + tau) * (eps + tau);
}

static int tw_in_recursive(const two_surface* s, const double p[3], double eps2, double thr,
                           int32_t node, int32_t b, int32_t e)
{
    if (b + 1 == e) {
        const double* t = s->tri + 9 * b;
        return two_point_triangle_sqdist(p, t, t + 3, t + 6, NULL) <= eps2;
    }
    int32_t m = b + (e - b) / 2;
    const double* L = s->box + 12 * node;
    const double* R = L + 6;
    double dl = two_point_box_sqdist(p, L, L + 3);
    double dr = two_point_box_sqdist(p, R, R + 3);
    if (dl < dr) {
        if (dl <= thr && tw_in_recursive(s, p, eps2, thr, 2 * node, b, m)) return 1;
        if (dr <= thr && tw_in_recursive(s, p, eps2, thr, 2 * node + 1, m, e)) return 1;
    } else {
        if (dr <= thr && tw_in_recursive(s, p, eps2, thr, 2 * node + 1, m, e)) return 1;
        if (dl <= thr && tw_in_recursive(s, p, eps2, thr, 2 * node, b, m)) return 1;
    }
    return 0;
}

int two_point_out(const two_surface* s, const double p[3], double eps2)
{
    if (!s) return 1;
    double thr = tw_prune_threshold(s, p, eps2);
    const double* B = s->box + 6;
    if (two_point_box_sqdist(p, B, B + 3) > thr) return 1;
    return !tw_in_recursive(s, p, eps2, thr, 1, 0, s->nf);
}

int two_point_out_brute(const two_surface* s, const double p[3], double eps2)
{
    if (!s) return 1;
    for (int32_t f = 0; f < s->nf; ++f) {
        const double* t = s->tri + 9 * f;
        if (two_point_triangle_sqdist(p, t, t + 3, t + 6, NULL) <= eps2) return 0;
    }
    return 1;
}

/* =========================================================================
 * Nearest facet (MeshFacetsAABBWithEps::nearest_facet, mesh_AABB.h:130-141,
 * mesh_AABB.cpp:381-480): the facet with the smallest point-facet squared
 * distance (the closest-point routine above) and its closest point.  Among
 * facets at exactly the same computed distance, the smallest input facet
 * index wins.  (geogram keeps the first one its traversal meets, and that
 * order follows its own facet reordering, which is not part of the
 * reference sources; the distance is the same either way.)  A child box is
 * skipped only when its squared distance exceeds (b + tau)^2, b = sqrt of
 * the best distance so far, tau = 64 * 2^-53 * max|coord| + 16 * 2^-53 * b:
 * a facet whose computed distance could tie or beat the best is never
 * skipped, so the result is the exact minimum over all facets, whatever the
 * tree.
 * ========================================================================= */
typedef struct {
    double d;
    int32_t id;
    double q[3];
} tw_nearest_t;

static double tw_nearest_threshold(const two_surface* s, const double p[3], double best)
{
    if (!(best < INFINITY)) return INFINITY;
    double m = s->scale;
    for (int k = 0; k < 3; ++k)
        if (fabs(p[k]) > m) m = fabs(p[k]);
    double b = sqrt(best);
    double tau = 64.0 * TW_EPS * m + 16.0 * TW_EPS * b;
    return (b + tau) * (b + tau);
}

static void tw_nearest_recursive(const two_surface* s, const double p[3], tw_nearest_t* best,
                                 int32_t node, int32_t b, int32_t e)
{
    if (b + 1 == e) {
        const double* t = s->tri + 9 * b;
        double q[3];
        double d = two_point_triangle_sqdist(p, t, t + 3, t + 6, q);
        int32_t id = s->fid[b];
        if (d < best->d || (d == best->d && id < best->id)) {
            best->d = d;
            best->id = id;
            best->q[0] = q[0]; best->q[1] = q[1]; best->q[2] = q[2];
        }
        return;
    }
    int32_t m = b + (e - b) / 2;
    const double* L = s->box + 12 * node;
    const double* R = L + 6;
    double dl = two_point_box_sqdist(p, L, L + 3);
    double dr = two_point_box_sqdist(p, R, R + 3);
    if (dl <= dr) {
        if (dl <= tw_nearest_threshold(s, p, best->d)) tw_nearest_recursive(s, p, best, 2 * node, b, m);
        if (dr <= tw_nearest_threshold(s, p, best->d)) tw_nearest_recursive(s, p, best, 2 * node + 1, m, e);
    } else {
        if (dr <= tw_nearest_threshold(s, p, best->d)) tw_nearest_recursive(s, p, best, 2 * node + 1, m, e);
        if (dl <= tw_nearest_threshold(s, p, best->d)) tw_nearest_recursive(s, p, best, 2 * node, b, m);
    }
}

int32_t two_nearest_facet(const two_surface* s, const double p[3], double q[3], double* sqd)
{
    tw_nearest_t best;
    best.d = INFINITY;
    best.id = INT32_MAX;
    best.q[0] = best.q[1] = best.q[2] = 0.0;
    if (s) tw_nearest_recursive(s, p, &best, 1, 0, s->nf);
    if (q) { q[0] = best.q[0]; q[1] = best.q[1]; q[2] = best.q[2]; }
    if (sqd) *sqd = best.d;
    return s ? best.id : -1;
}

int32_t two_nearest_facet_brute(const two_surface* s, const double p[3], double q[3], double* sqd)
{
    tw_nearest_t best;
    best.d = INFINITY;
    best.id = INT32_MAX;
    best.q[0] = best.q[1] = best.q[2] = 0.0;
    for (int32_t f = 0; s && f < s->nf; ++f) {
        const double* t = s->tri + 9 * f;
        double qq[3];
        double d = two_point_triangle_sqdist(p, t, t + 3, t + 6, qq);
        if (d < best.d || (d == best.d && s->fid[f] < best.id)) {
            best.d = d;
            best.id = s->fid[f];
            best.q[0] = qq[0]; best.q[1] = qq[1]; best.q[2] = qq[2];
        }
    }
    if (q) { q[0] = best.q[0]; q[1] = best.q[1]; q[2] = best.q[2]; }
    if (sqd) *sqd = best.d;
    return s ? best.id : -1;
}

/* isFaceOutEnvelop_sampling, LocalOperations.cpp:1046-1109: a degenerate
 * triangle is never out; otherwise out iff some sample is out.  The order in
 * which the reference visits the samples (from the middle, with a facet
 * hint) changes only how much work is done, not the decision. */
int two_face_out(const two_surface* s, const double tri[9], double eps2, double sd)
{
    if (two_collinear(tri, tri + 3, tri + 6)) return 0;
    int64_t n = two_sample_count(tri, sd);
    double* ps = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    two_sample_triangle(tri, sd, ps, n);
    int out = 0;
    for (int64_t i = n / 2, c = 0; c < n; i = (i + 1) % n, ++c)
        if (two_point_out(s, ps + 3 * i, eps2)) { out = 1; break; }
    free(ps);
    return out;
}

/* =========================================================================
 * 3x3 solve by Householder QR with column pivoting (Golub & Van Loan,
 * "Matrix Computations", Alg. 5.4.1), standing in for Eigen's
 * ColPivHouseholderQR::solve (VertexSmoother.cpp:492).  Columns are chosen by
 * largest remaining squared norm (first index on ties); a pivot with
 * |R_kk| <= 3 * 2^-52 * |R_00| ends the rank and the remaining unknowns are
 * set to zero (Eigen's default threshold is diagonal size * machine epsilon).
 * ========================================================================= */
int two_qr_solve3(const double Hm[9], const double bvec[3], double x[3])
{
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
            if (nrm > best) { best = nrm; p = j; }
        }
        if (p != k) {
            for (int i = 0; i < 3; ++i) { double t = R[i][k]; R[i][k] = R[i][p]; R[i][p] = t; }
            int t = perm[k]; perm[k] = perm[p]; perm[p] = t;
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
    for (int k = 0; k < 3; ++k)
        if (fabs(R[k][k]) > thr) rank = k + 1; else break;
    double y[3] = {0.0, 0.0, 0.0};
    for (int k = rank - 1; k >= 0; --k) {
        double s = c[k];
        for (int j = k + 1; j < rank; ++j) s = s - R[k][j] * y[j];
        y[k] = s / R[k][k];
    }
    for (int k = 0; k < 3; ++k) x[perm[k]] = y[k];
    return rank == 3 ? 0 : 1;
}

/* =========================================================================
 * NewtonsMethod / NewtonsUpdate / getNewEnergy, VertexSmoother.cpp:465-702
 * (scalar build: TETWILD_WITH_ISPC off).  Per-tet terms are summed in caller
 * order.  NewtonsUpdate evaluates E/J/H on the tet rotated so the centre
 * vertex comes first (:640-651); getNewEnergy evaluates E on the tet in its
 * stored order (:606-614).
 * ========================================================================= */
static void tw_gather(const double* xyz, const int32_t* t, int32_t v, const double* pos,
                      int start, double T[12])
{
    for (int j = 0; j < 4; ++j) {
        int32_t id = t[(start + j) % 4];
        const double* src = (id == v) ? pos : xyz + 3 * (size_t)id;
        T[3 * j] = src[0];
        T[3 * j + 1] = src[1];
        T[3 * j + 2] = src[2];
    }
}

static int tw_star_flip(const double* xyz, const int32_t* tets, int32_t nt, int32_t v,
                        const double* pos)
{
    double T[12];
    for (int32_t i = 0; i < nt; ++i) {
        tw_gather(xyz, tets + 4 * i, v, pos, 0, T);
        if (two_tet_flip(T)) return 1;
    }
    return 0;
}

static double tw_new_energy(const double* xyz, const int32_t* tets, int32_t nt, int32_t v,
                            const double* pos)
{
    double s = 0.0, T[12];
    for (int32_t i = 0; i < nt; ++i) {
        tw_gather(xyz, tets + 4 * i, v, pos, 0, T);
        s += two_amips_energy(T);
    }
    if (isinf(s) || isnan(s) || s <= 0.0 || s > TWO_MAX_ENERGY) s = TWO_MAX_ENERGY;
    return s;
}

static int tw_newton_update(const double* xyz, const int32_t* tets, int32_t nt, int32_t v,
                            const double* pos, double* energy, double J[3], double H[9])
{
    double e = 0.0, T[12], J1[3], H1[9];
    for (int k = 0; k < 3; ++k) J[k] = 0.0;
    for (int k = 0; k < 9; ++k) H[k] = 0.0;
    for (int32_t i = 0; i < nt; ++i) {
        const int32_t* t = tets + 4 * i;
        int start = 0;
        for (int j = 0; j < 4; ++j)
            if (t[j] == v) { start = j; break; }
        tw_gather(xyz, t, v, pos, start, T);
        e += two_amips_energy(T);
        two_amips_jacobian(T, J1);
        two_amips_hessian(T, H1);
        for (int j = 0; j < 3; ++j) {
            J[j] += J1[j];
            H[3 * j + 0] += H1[3 * j + 0];
            H[3 * j + 1] += H1[3 * j + 1];
            H[3 * j + 2] += H1[3 * j + 2];
        }
    }
    if (isinf(e)) e = TWO_MAX_ENERGY;
    *energy = e;
    if (isnan(e)) return 0;
    if (e <= 0.0) return 0;
    for (int k = 0; k < 3; ++k)
        if (!isfinite(J[k])) return 0;
    for (int k = 0; k < 9; ++k)
        if (!isfinite(H[k])) return 0;
    return 1;
}

int two_newton_star(const double* xyz, const int32_t* tets, int32_t nt, int32_t v, int max_step,
                    int max_it, double out[3])
{
    double pos[3] = {xyz[3 * (size_t)v], xyz[3 * (size_t)v + 1], xyz[3 * (size_t)v + 2]};
    int is_moved = 0;
    double old_energy = 0.0, new_energy = 0.0, J[3], H[9];
    for (int step = 0; step < max_step; ++step) {
        if (!tw_newton_update(xyz, tets, nt, v, pos, &old_energy, J, H)) break;
        double old_pf[3] = {pos[0], pos[1], pos[2]};
        double X0[3] = {pos[0], pos[1], pos[2]};
        double a = 1.0;
        int step_taken = 0;
        for (int it = 0; it < max_it; ++it) {
            double rhs[3], X[3];
            for (int i = 0; i < 3; ++i)
                rhs[i] = ((H[3 * i] * X0[0] + H[3 * i + 1] * X0[1]) + H[3 * i + 2] * X0[2]) - a * J[i];
            two_qr_solve3(H, rhs, X);
            if (!isfinite(X[0]) || !isfinite(X[1]) || !isfinite(X[2])) {
                a /= 2.0;
                continue;
            }
            pos[0] = X[0]; pos[1] = X[1]; pos[2] = X[2];
            if (tw_star_flip(xyz, tets, nt, v, pos)) {
                pos[0] = old_pf[0]; pos[1] = old_pf[1]; pos[2] = old_pf[2];
                a /= 2.0;
                continue;
            }
            new_energy = tw_new_energy(xyz, tets, nt, v, pos);
            if (new_energy >= old_energy || isinf(new_energy) || isnan(new_energy)) {
                pos[0] = old_pf[0]; pos[1] = old_pf[1]; pos[2] = old_pf[2];
                a /= 2.0;
                continue;
            }
            step_taken = 1;
            break;
        }
        if (fabs(new_energy - old_energy) < 1e-5) step_taken = 0;
        if (!step_taken) {
            is_moved = (step != 0);
            break;
        }
        is_moved = 1;
    }
    out[0] = pos[0];
    out[1] = pos[1];
    out[2] = pos[2];
    return is_moved;
}

/* =========================================================================
 * One vertex of a smoothing pass (VertexSmoother.cpp).  Interior vertex:
 * the body of smoothSingle (:114-210); surface vertex: the body of
 * smoothSurface (:244-450) with the defaults use_onering_projection = false
 * and use_energy_max = true (State.h:53,60), isBoundarySlide returning false
 * (LocalOperations.cpp:1123-1124), every vertex already rounded (posf ==
 * pos), and the stored tet qualities equal to calTetQuality at the current
 * positions.
 *   1. every tet of the star must be POSITIVE at the current positions
 *      (:161-170, :289-297), else TWO_SMOOTH_INVALID;
 *   2. NewtonsMethod (:465-542); not moved -> TWO_SMOOTH_NOT_MOVED;
 *   interior: the final isFlip (:189-194) cannot fire (every accepted trial
 *      passed the same exact test) and is kept as a check; -> MOVED;
 *   surface: 3. the Newton position is projected on the nearest facet of the
 *      input surface (boundary vertices: of the boundary surface) (:353-363);
 *   4. isFlip at the projected position -> REJECT_FLIP (:374-378);
 *   5. max calTetQuality after < max before, else REJECT_QUALITY (:379-386);
 *   6. each one-ring surface face (faces through the vertex that the caller
 *      flags as surface faces, as sorted vertex triples without repeats),
 *      written from the vertex onward in the cyclic order of its sorted
 *      triple, must pass isFaceOutEnvelop on the input surface (:417-440),
 *      else REJECT_ENVELOPE.
 * fflags[i] bit j: the face of tet i opposite its j-th vertex is a surface
 * face (is_surface_fs != NOT_SURFACE).  out = the new position when MOVED,
 * else the old one.
 * ========================================================================= */
static int tw_tri_key_cmp(const int32_t* a, const int32_t* b)
{
    for (int k = 0; k < 3; ++k) {
        if (a[k] < b[k]) return -1;
        if (a[k] > b[k]) return 1;
    }
    return 0;
}

int two_smooth_star(const double* xyz, const int32_t* tets, const uint8_t* fflags, int32_t nt,
                    int32_t v, int kind, const two_surface* s_in, const two_surface* s_b,
                    double eps2, double sd, int max_step, int max_it, double out[3])
{
    const double* p0 = xyz + 3 * (size_t)v;
    double T[12];
    out[0] = p0[0]; out[1] = p0[1]; out[2] = p0[2];
    for (int32_t i = 0; i < nt; ++i) {
        tw_gather(xyz, tets + 4 * i, v, p0, 0, T);
        if (two_orient3d(T, T + 3, T + 6, T + 9) != 1) return TWO_SMOOTH_INVALID;
    }
    double pf[3];
    if (!two_newton_star(xyz, tets, nt, v, max_step, max_it, pf)) return TWO_SMOOTH_NOT_MOVED;
    if (kind == TWO_STAR_INTERIOR) {
        if (tw_star_flip(xyz, tets, nt, v, pf)) return TWO_SMOOTH_REJECT_FLIP;
        out[0] = pf[0]; out[1] = pf[1]; out[2] = pf[2];
        return TWO_SMOOTH_MOVED;
    }
    const two_surface* tree = (kind == TWO_STAR_BOUNDARY) ? s_b : s_in;
    if (!tree || !s_in) return -1;
    double p[3];
    two_nearest_facet(tree, pf, p, NULL);
    if (tw_star_flip(xyz, tets, nt, v, p)) return TWO_SMOOTH_REJECT_FLIP;
    double old_max = 0.0, new_max = 0.0;
    for (int32_t i = 0; i < nt; ++i) {
        tw_gather(xyz, tets + 4 * i, v, p0, 0, T);
        double e = two_tet_quality(T);
        if (e > old_max) old_max = e;
        tw_gather(xyz, tets + 4 * i, v, p, 0, T);
        e = two_tet_quality(T);
        if (e > new_max) new_max = e;
    }
    if (!(new_max < old_max)) return TWO_SMOOTH_REJECT_QUALITY;
    for (int32_t i = 0; i < nt; ++i) {
        const int32_t* t = tets + 4 * i;
        for (int j = 0; j < 4; ++j) {
            if (t[j] == v || !((fflags[i] >> j) & 1)) continue;
            int32_t key[3] = {t[(j + 1) % 4], t[(j + 2) % 4], t[(j + 3) % 4]};
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2 - a; ++b)
                    if (key[b] > key[b + 1]) { int32_t x = key[b]; key[b] = key[b + 1]; key[b + 1] = x; }
            /* repeated triple: only its first occurrence is tested */
            int seen = 0;
            for (int32_t i2 = 0; i2 <= i && !seen; ++i2) {
                const int32_t* t2 = tets + 4 * i2;
                for (int j2 = 0; j2 < 4 && !seen; ++j2) {
                    if (i2 == i && j2 >= j) break;
                    if (t2[j2] == v || !((fflags[i2] >> j2) & 1)) continue;
                    int32_t k2[3] = {t2[(j2 + 1) % 4], t2[(j2 + 2) % 4], t2[(j2 + 3) % 4]};
                    for (int a = 0; a < 2; ++a)
                        for (int b = 0; b < 2 - a; ++b)
                            if (k2[b] > k2[b + 1]) { int32_t x = k2[b]; k2[b] = k2[b + 1]; k2[b + 1] = x; }
                    seen = (tw_tri_key_cmp(key, k2) == 0);
                }
            }
            if (seen) continue;
            int k = (key[0] == v) ? 0 : (key[1] == v) ? 1 : 2;
            const double* b1 = xyz + 3 * (size_t)key[(k + 1) % 3];
            const double* b2 = xyz + 3 * (size_t)key[(k + 2) % 3];
            double tri[9] = {p[0], p[1], p[2], b1[0], b1[1], b1[2], b2[0], b2[1], b2[2]};
            if (two_face_out(s_in, tri, eps2, sd)) return TWO_SMOOTH_REJECT_ENVELOPE;
        }
    }
    out[0] = p[0]; out[1] = p[1]; out[2] = p[2];
    return TWO_SMOOTH_MOVED;
}

/* =========================================================================
 * The checks of one edge collapse v1 -> v2 (EdgeCollapser::collapseAnEdge,
 * EdgeCollapser.cpp:284-446, with isCollapsable_epsilon :727-775), with
 * isBoundarySlide returning false (LocalOperations.cpp:1123-1124), energy
 * AMIPS with use_energy_max (State.h:53), the stored qualities equal to
 * calTetQuality at the current positions, and the caller's vertex flags
 * already updated by isIsolated / isBoundaryPoint (:299-308).  tets: the
 * conn_tets of v1 (caller order); fflags as for two_smooth_star.  Returns
 * SUCCESS 0, FLIP 1, QUALITY 2 or ENVELOP 3 (EdgeCollapser.h:52-55).
 *   1. degenerate edge: |v1 - v2| == 0 (skips the envelope and quality tests);
 *   2. v1 on the boundary, v2 not: v2 out of the boundary envelope -> ENVELOP;
 *      v1 on the surface, v2 not: v2 out of the envelope -> ENVELOP;
 *   3. new tets (those without v2, v1 replaced by v2) not all POSITIVE -> FLIP;
 *   4. check_quality: old max (soft_energy >= 0: soft_energy), new max (0 for
 *      an unrounded v1); new > old -> QUALITY;
 *   5. v1 on the surface: the surface faces through v1 (sorted triples without
 *      repeats) not through v2, v1 replaced by v2 in place, each out of the
 *      envelope -> ENVELOP.
 * ========================================================================= */
int two_collapse_check(const double* xyz, const int32_t* tets, const uint8_t* fflags, int32_t nt,
                       int32_t v1, int32_t v2, int flags, const two_surface* s_in,
                       const two_surface* s_b, double eps2, double sd, int check_quality,
                       double soft_energy)
{
    const double* p1 = xyz + 3 * (size_t)v1;
    const double* p2 = xyz + 3 * (size_t)v2;
    double dx = p1[0] - p2[0], dy = p1[1] - p2[1], dz = p1[2] - p2[2];
    const int degenerate = sqrt(dx * dx + dy * dy + dz * dz) == 0.0;
    if ((flags & TWO_CV_V1_BOUNDARY) && !(flags & TWO_CV_V2_BOUNDARY) && !degenerate)
        if (!s_b || two_point_out(s_b, p2, eps2)) return 3;
    if ((flags & TWO_CV_V1_SURFACE) && !(flags & TWO_CV_V2_SURFACE) && !degenerate)
        if (!s_in || two_point_out(s_in, p2, eps2)) return 3;
    double T[12];
    for (int32_t i = 0; i < nt; ++i) {
        const int32_t* t = tets + 4 * i;
        if (t[0] == v2 || t[1] == v2 || t[2] == v2 || t[3] == v2) continue;
        tw_gather(xyz, t, v1, p2, 0, T);
        if (two_orient3d(T, T + 3, T + 6, T + 9) != 1) return 1;
    }
    if (check_quality) {
        double old_max = 0.0, new_max = 0.0;
        for (int32_t i = 0; i < nt; ++i) {
            const int32_t* t = tets + 4 * i;
            tw_gather(xyz, t, v1, p1, 0, T);
            double e = two_tet_quality(T);
            if (e > old_max) old_max = e;
            if (t[0] == v2 || t[1] == v2 || t[2] == v2 || t[3] == v2) continue;
            tw_gather(xyz, t, v1, p2, 0, T);
            e = two_tet_quality(T);
            if (e > new_max) new_max = e;
        }
        if (soft_energy >= 0.0) old_max = soft_energy;
        if (flags & TWO_CV_V1_UNROUNDED) new_max = 0.0;
        if (!degenerate && !(new_max <= old_max)) return 2;
    }
    if ((flags & TWO_CV_V1_SURFACE) && !degenerate) {
        for (int32_t i = 0; i < nt; ++i) {
            const int32_t* t = tets + 4 * i;
            for (int j = 0; j < 4; ++j) {
                if (t[j] == v1 || !((fflags[i] >> j) & 1)) continue;
                int32_t key[3] = {t[(j + 1) % 4], t[(j + 2) % 4], t[(j + 3) % 4]};
                for (int a = 0; a < 2; ++a)
                    for (int b = 0; b < 2 - a; ++b)
                        if (key[b] > key[b + 1]) { int32_t x = key[b]; key[b] = key[b + 1]; key[b + 1] = x; }
                int seen = 0;
                for (int32_t i2 = 0; i2 <= i && !seen; ++i2) {
                    const int32_t* t2 = tets + 4 * i2;
                    for (int j2 = 0; j2 < 4 && !seen; ++j2) {
                        if (i2 == i && j2 >= j) break;
                        if (t2[j2] == v1 || !((fflags[i2] >> j2) & 1)) continue;
                        int32_t k2[3] = {t2[(j2 + 1) % 4], t2[(j2 + 2) % 4], t2[(j2 + 3) % 4]};
                        for (int a = 0; a < 2; ++a)
                            for (int b = 0; b < 2 - a; ++b)
                                if (k2[b] > k2[b + 1]) { int32_t x = k2[b]; k2[b] = k2[b + 1]; k2[b + 1] = x; }
                        seen = (tw_tri_key_cmp(key, k2) == 0);
                    }
                }
                if (seen) continue;
                if (key[0] == v2 || key[1] == v2 || key[2] == v2) continue;
                double tri[9];
                for (int k = 0; k < 3; ++k) {
                    const double* q = (key[k] == v1) ? p2 : xyz + 3 * (size_t)key[k];
                    tri[3 * k] = q[0];
                    tri[3 * k + 1] = q[1];
                    tri[3 * k + 2] = q[2];
                }
                if (!s_in || two_face_out(s_in, tri, eps2, sd)) return 3;
            }
        }
    }
    return 0;
}

/* =========================================================================
 * Energy sweeps over a tet list (LocalOperations.cpp:605-693) on qualities
 * computed by calTetQuality_AMIPS at the current positions; the list holds
 * the tets that are not removed.  avg / max over the tets with no locked
 * vertex (locked[i] != 0 marks one, NULL: none), avg sequential in list
 * order (MAX_ENERGY when it overflows); second max also skips MAX_ENERGY;
 * buckets of getFilterEnergy over every tet.
 * ========================================================================= */
void two_energy_stats(const double* xyz, const int32_t* tets, int64_t n, const uint8_t* locked,
                      double thres, double* avg, double* max_e, double* second_max,
                      int64_t buckets[11])
{
    double sum = 0.0, mx = 0.0, mx2 = 0.0;
    int64_t cnt = 0;
    static const double p10[11] = {1.0, 1e1, 1e2, 1e3, 1e4, 1e5, 1e6, 1e7, 1e8, 1e9, 1e10};
    for (int k = 0; k < 11; ++k) buckets[k] = 0;
    for (int64_t i = 0; i < n; ++i) {
        double T[12];
        for (int j = 0; j < 4; ++j) {
            const double* src = xyz + 3 * (size_t)tets[4 * i + j];
            T[3 * j] = src[0];
            T[3 * j + 1] = src[1];
            T[3 * j + 2] = src[2];
        }
        const double e = two_tet_quality(T);
        if (e > thres - 1 + 1e10) {
            buckets[10]++;
        } else {
            for (int j = 0; j < 10; ++j)
                if (e > thres - 1 + p10[j] && e <= thres - 1 + p10[j + 1]) {
                    buckets[j]++;
                    break;
                }
        }
        if (locked && locked[i]) continue;
        if (e > mx) mx = e;
        if (e != TWO_MAX_ENERGY && e > mx2) mx2 = e;
        sum += e;
        cnt++;
    }
    double a = sum / (double)cnt;
    if (isinf(a)) a = TWO_MAX_ENERGY;
    *avg = a;
    *max_e = mx;
    *second_max = mx2;
}

/* =========================================================================
 * Dihedral angles (calTetQuality_AD, LocalOperations.cpp:783-860) and the
 * outputInfo sweep over them (:483-521).  For face i (the other three
 * vertices p, q, r in cyclic order from i+1): the plane's normal
 * (a, b, c) = (p - r) x (q - r) and offset d = -(a r.x + b r.y + c r.z); a
 * zero normal is a degenerate face.  Vertex s = v_i projects to
 * s - lambda (a, b, c), lambda = (a s + d) / (a a + b b + c c); nv_i = s - proj
 * and its squared length is the height.  A face whose projection equals s,
 * or whose nv or height is 0, gives (0, pi).  nv is rescaled by its largest
 * component when that is below 1e-5.  The six angles are
 * acos(-nv_a . nv_b / (|nv_a| |nv_b|)) over the vertex pairs (0,1), (1,2),
 * (0,2), (2,3), (0,3), (3,1), clamped to [0, pi] outside [-1, 1].
 * ========================================================================= */
#define TWO_PI 3.14159265358979323846   /* M_PI */

void two_dihedral_minmax(const double T[12], double* min_angle, double* max_angle)
{
    double nv[4][3], len[4];
    for (int i = 0; i < 4; ++i) {
        const double* sv = T + 3 * i;
        const double* p = T + 3 * ((i + 1) % 4);
        const double* q = T + 3 * ((i + 2) % 4);
        const double* r = T + 3 * ((i + 3) % 4);
        const double rp[3] = {p[0] - r[0], p[1] - r[1], p[2] - r[2]};
        const double rq[3] = {q[0] - r[0], q[1] - r[1], q[2] - r[2]};
        const double a = rp[1] * rq[2] - rq[1] * rp[2];
        const double b = rp[2] * rq[0] - rq[2] * rp[0];
        const double c = rp[0] * rq[1] - rq[0] * rp[1];
        if (a == 0.0 && b == 0.0 && c == 0.0) {
            *min_angle = 0.0;
            *max_angle = TWO_PI;
            return;
        }
        const double d = ((-a * r[0]) - b * r[1]) - c * r[2];
        const double num = ((a * sv[0] + b * sv[1]) + c * sv[2]) + d;
        const double den = (a * a + b * b) + c * c;
        const double lam = num / den;
        const double pr[3] = {sv[0] - lam * a, sv[1] - lam * b, sv[2] - lam * c};
        if (pr[0] == sv[0] && pr[1] == sv[1] && pr[2] == sv[2]) {
            *min_angle = 0.0;
            *max_angle = TWO_PI;
            return;
        }
        double v[3] = {sv[0] - pr[0], sv[1] - pr[1], sv[2] - pr[2]};
        const double h = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
        double m = fabs(v[0]);
        if (fabs(v[1]) > m) m = fabs(v[1]);
        if (fabs(v[2]) > m) m = fabs(v[2]);
        if (m == 0.0 || h == 0.0) {
            *min_angle = 0.0;
            *max_angle = TWO_PI;
            return;
        }
        if (m < 1e-5) {
            v[0] = v[0] / m;
            v[1] = v[1] / m;
            v[2] = v[2] / m;
            len[i] = sqrt(h / (m * m));
        } else {
            len[i] = sqrt(h);
        }
        nv[i][0] = v[0];
        nv[i][1] = v[1];
        nv[i][2] = v[2];
    }
    static const int pa[6] = {0, 1, 0, 2, 0, 3}, pb[6] = {1, 2, 2, 3, 3, 1};
    double mn = 0.0, mx = 0.0;
    for (int k = 0; k < 6; ++k) {
        const double* u = nv[pa[k]];
        const double* w = nv[pb[k]];
        const double cs = ((-u[0]) * w[0] + (-u[1]) * w[1] + (-u[2]) * w[2]) /
                          (len[pa[k]] * len[pb[k]]);
        const double ang = cs > 1.0 ? 0.0 : cs < -1.0 ? TWO_PI : acos(cs);
        if (k == 0 || ang < mn) mn = ang;
        if (k == 0 || ang > mx) mx = ang;
    }
    *min_angle = mn;
    *max_angle = mx;
}

void two_dihedral_stats(const double* xyz, const int32_t* tets, int64_t n, const uint8_t* locked,
                        double out[4], int64_t counts[7], double* mins, double* maxs)
{
    static const double cmp[6] = {6 / 180.0 * TWO_PI, 12 / 180.0 * TWO_PI, 18 / 180.0 * TWO_PI,
                                  162 / 180.0 * TWO_PI, 168 / 180.0 * TWO_PI, 174 / 180.0 * TWO_PI};
    double mn_all = 10.0, mx_all = 0.0, sum_mn = 0.0, sum_mx = 0.0;
    int64_t cnt = 0;
    for (int k = 0; k < 7; ++k) counts[k] = 0;
    for (int64_t i = 0; i < n; ++i) {
        double T[12];
        for (int j = 0; j < 4; ++j) {
            const double* src = xyz + 3 * (size_t)tets[4 * i + j];
            T[3 * j] = src[0];
            T[3 * j + 1] = src[1];
            T[3 * j + 2] = src[2];
        }
        double a, b;
        two_dihedral_minmax(T, &a, &b);
        if (mins) mins[i] = a;
        if (maxs) maxs[i] = b;
        if (locked && locked[i]) continue;
        cnt++;
        if (a < mn_all) mn_all = a;
        if (b > mx_all) mx_all = b;
        sum_mn += a;
        sum_mx += b;
        for (int j = 0; j < 3; ++j) {
            if (a < cmp[j]) counts[j]++;
            if (b > cmp[j + 3]) counts[j + 3]++;
        }
    }
    counts[6] = cnt;
    out[0] = mn_all;
    out[1] = sum_mn / (double)cnt;
    out[2] = mx_all;
    out[3] = sum_mx / (double)cnt;
}

/* getFilterEnergy's choice over the buckets (LocalOperations.cpp:674-692). */
double two_filter_energy(const int64_t buckets[11], double thres, int* is_clean_up)
{
    int64_t t1[10], t2[10];
    for (int i = 0; i < 10; ++i) {
        t1[i] = 0;
        t2[i] = 0;
        for (int k = 0; k <= i; ++k) t1[i] += buckets[k];
        for (int k = i + 1; k < 11; ++k) t2[i] += buckets[k];
    }
    *is_clean_up = 0;
    if (t1[0] >= t2[0]) {
        *is_clean_up = t2[5] > 0;
        return 8;
    }
    if (t1[8] <= t2[8]) return 1e11;
    for (int i = 0; i < 8; ++i)
        if (t1[i] < t2[i] && t1[i + 1] > t2[i + 1]) return thres - 1 + 5 * pow(10, i + 1);
    return 8;
}

/* =========================================================================
 * Threaded batch drivers.
 * ========================================================================= */
typedef struct {
    int kind;
    int64_t lo, hi;
    const void* a0;
    const void* a1;
    const void* a2;
    const void* a3;
    const void* a4;
    const void* a5;
    const void* a6;
    const void* a7;
    double d0, d1, d2;
    int i0, i1, i2;
    void* o0;
    void* o1;
    void* o2;
    void* o3;
    int64_t n;
} tw_job;

static void tw_run_amips(tw_job* j)
{
    const double* T = (const double*)j->a0;
    int64_t n = j->n;
    double* E = (double*)j->o0;
    double* J = (double*)j->o1;
    double* H = (double*)j->o2;
    uint8_t* flip = (uint8_t*)j->o3;
    for (int64_t i = j->lo; i < j->hi; ++i) {
        double t[12], jj[3], hh[9];
        for (int c = 0; c < 12; ++c) t[c] = T[c * n + i];
        if (flip) flip[i] = (uint8_t)two_tet_flip(t);
        if (E) E[i] = j->i0 ? two_tet_quality(t) : two_amips_energy(t);
        if (J) {
            two_amips_jacobian(t, jj);
            for (int c = 0; c < 3; ++c) J[c * n + i] = jj[c];
        }
        if (H) {
            two_amips_hessian(t, hh);
            for (int c = 0; c < 9; ++c) H[c * n + i] = hh[c];
        }
    }
}
static void tw_run_points(tw_job* j)
{
    const two_surface* s = (const two_surface*)j->a0;
    const double* P = (const double*)j->a1;
    uint8_t* out = (uint8_t*)j->o0;
    for (int64_t i = j->lo; i < j->hi; ++i) out[i] = (uint8_t)two_point_out(s, P + 3 * i, j->d0);
}
static void tw_run_faces(tw_job* j)
{
    const two_surface* s = (const two_surface*)j->a0;
    const double* tris = (const double*)j->a1;
    uint8_t* out = (uint8_t*)j->o0;
    for (int64_t i = j->lo; i < j->hi; ++i)
        out[i] = (uint8_t)two_face_out(s, tris + 9 * i, j->d0, j->d1);
}
static void tw_run_stars(tw_job* j)
{
    const double* xyz = (const double*)j->a0;
    const int32_t* off = (const int32_t*)j->a1;
    const int32_t* tets = (const int32_t*)j->a2;
    const int32_t* cen = (const int32_t*)j->a3;
    double* out = (double*)j->o0;
    uint8_t* moved = (uint8_t*)j->o1;
    for (int64_t i = j->lo; i < j->hi; ++i) {
        int32_t b = off[i], e = off[i + 1];
        double o[3];
        int mv = two_newton_star(xyz, tets + 4 * (size_t)b, e - b, cen[i], j->i0, j->i1, o);
        out[3 * i] = o[0];
        out[3 * i + 1] = o[1];
        out[3 * i + 2] = o[2];
        moved[i] = (uint8_t)mv;
    }
}
static void tw_run_smooth(tw_job* j)
{
    const double* xyz = (const double*)j->a0;
    const int32_t* off = (const int32_t*)j->a1;
    const int32_t* tets = (const int32_t*)j->a2;
    const int32_t* cen = (const int32_t*)j->a3;
    const uint8_t* ff = (const uint8_t*)j->a4;
    const uint8_t* kinds = (const uint8_t*)j->a5;
    double* out = (double*)j->o0;
    int8_t* status = (int8_t*)j->o1;
    for (int64_t i = j->lo; i < j->hi; ++i) {
        int32_t b = off[i], e = off[i + 1];
        status[i] = (int8_t)two_smooth_star(xyz, tets + 4 * (size_t)b, ff ? ff + b : NULL, e - b,
                                            cen[i], kinds ? kinds[i] : TWO_STAR_INTERIOR,
                                            (const two_surface*)j->a6, (const two_surface*)j->a7,
                                            j->d0, j->d1, j->i0, j->i1, out + 3 * i);
    }
}
static void tw_run_nearest(tw_job* j)
{
    const two_surface* s = (const two_surface*)j->a0;
    const double* P = (const double*)j->a1;
    double* Q = (double*)j->o0;
    double* D = (double*)j->o1;
    int32_t* F = (int32_t*)j->o2;
    for (int64_t i = j->lo; i < j->hi; ++i) {
        double q[3], d;
        int32_t f = two_nearest_facet(s, P + 3 * i, q, &d);
        if (Q) { Q[3 * i] = q[0]; Q[3 * i + 1] = q[1]; Q[3 * i + 2] = q[2]; }
        if (D) D[i] = d;
        if (F) F[i] = f;
    }
}
static void tw_run_collapse(tw_job* j)
{
    const double* xyz = (const double*)j->a0;
    const int32_t* off = (const int32_t*)j->a1;
    const int32_t* tets = (const int32_t*)j->a2;
    const int32_t* v12 = (const int32_t*)j->a3;
    const uint8_t* ff = (const uint8_t*)j->a4;
    const uint8_t* fl = (const uint8_t*)j->a5;
    uint8_t* res = (uint8_t*)j->o0;
    for (int64_t i = j->lo; i < j->hi; ++i) {
        int32_t b = off[i], e = off[i + 1];
        res[i] = (uint8_t)two_collapse_check(xyz, tets + 4 * (size_t)b, ff + b, e - b, v12[2 * i],
                                             v12[2 * i + 1], fl[i], (const two_surface*)j->a6,
                                             (const two_surface*)j->a7, j->d0, j->d1, j->i0,
                                             j->d2);
    }
}
static void* tw_thread_main(void* arg)
{
    tw_job* j = (tw_job*)arg;
    switch (j->kind) {
    case 6: tw_run_collapse(j); break;
    case 0: tw_run_amips(j); break;
    case 1: tw_run_points(j); break;
    case 2: tw_run_faces(j); break;
    case 3: tw_run_stars(j); break;
    case 4: tw_run_smooth(j); break;
    case 5: tw_run_nearest(j); break;
    default: break;
    }
    return NULL;
}
static void tw_parallel(tw_job proto, int64_t n, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if ((int64_t)nthreads > n) nthreads = (int)(n > 0 ? n : 1);
    pthread_t th[256];
    tw_job jobs[256];
    /* contiguous chunks, one per thread */
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = proto;
        jobs[t].lo = n * t / nthreads;
        jobs[t].hi = n * (t + 1) / nthreads;
    }
    if (nthreads == 1) {
        tw_thread_main(&jobs[0]);
        return;
    }
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, tw_thread_main, &jobs[t]);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
}

void two_amips_batch_soa(const double* T, int64_t n, int quality, double* E, double* J, double* H,
                         uint8_t* flip, int nthreads)
{
    tw_job j;
    memset(&j, 0, sizeof j);
    j.kind = 0;
    j.a0 = T;
    j.n = n;
    j.i0 = quality;
    j.o0 = E;
    j.o1 = J;
    j.o2 = H;
    j.o3 = flip;
    tw_parallel(j, n, nthreads);
}
void two_points_out_batch(const two_surface* s, const double* P, int64_t n, double eps2,
                          uint8_t* out, int nthreads)
{
    tw_job j;
    memset(&j, 0, sizeof j);
    j.kind = 1;
    j.a0 = s;
    j.a1 = P;
    j.d0 = eps2;
    j.o0 = out;
    tw_parallel(j, n, nthreads);
}
void two_faces_out_batch(const two_surface* s, const double* tris, int64_t n, double eps2,
                         double sd, uint8_t* out, int nthreads)
{
    tw_job j;
    memset(&j, 0, sizeof j);
    j.kind = 2;
    j.a0 = s;
    j.a1 = tris;
    j.d0 = eps2;
    j.d1 = sd;
    j.o0 = out;
    tw_parallel(j, n, nthreads);
}
void two_newton_stars_batch(const double* xyz, const int32_t* star_off, const int32_t* tets,
                            const int32_t* centers, int64_t nstars, int max_step, int max_it,
                            double* out, uint8_t* moved, int nthreads)
{
    tw_job j;
    memset(&j, 0, sizeof j);
    j.kind = 3;
    j.a0 = xyz;
    j.a1 = star_off;
    j.a2 = tets;
    j.a3 = centers;
    j.i0 = max_step;
    j.i1 = max_it;
    j.o0 = out;
    j.o1 = moved;
    tw_parallel(j, nstars, nthreads);
}

void two_smooth_stars_batch(const double* xyz, const int32_t* star_off, const int32_t* tets,
                            const uint8_t* fflags, const int32_t* centers, const uint8_t* kinds,
                            int64_t nstars, const two_surface* s_in, const two_surface* s_b,
                            double eps2, double sd, int max_step, int max_it, double* out,
                            int8_t* status, int nthreads)
{
    tw_job j;
    memset(&j, 0, sizeof j);
    j.kind = 4;
    j.a0 = xyz;
    j.a1 = star_off;
    j.a2 = tets;
    j.a3 = centers;
    j.a4 = fflags;
    j.a5 = kinds;
    j.a6 = s_in;
    j.a7 = s_b;
    j.d0 = eps2;
    j.d1 = sd;
    j.i0 = max_step;
    j.i1 = max_it;
    j.o0 = out;
    j.o1 = status;
    tw_parallel(j, nstars, nthreads);
}

void two_nearest_batch(const two_surface* s, const double* P, int64_t n, double* Q, double* D,
                       int32_t* F, int nthreads)
{
    tw_job j;
    memset(&j, 0, sizeof j);
    j.kind = 5;
    j.a0 = s;
    j.a1 = P;
    j.o0 = Q;
    j.o1 = D;
    j.o2 = F;
    tw_parallel(j, n, nthreads);
}

void two_collapse_check_batch(const double* xyz, const int32_t* off, const int32_t* tets,
                              const uint8_t* fflags, const int32_t* v12, const uint8_t* flags,
                              int64_t n, const two_surface* s_in, const two_surface* s_b,
                              double eps2, double sd, int check_quality, double soft_energy,
                              uint8_t* result, int nthreads)
{
    tw_job j;
    memset(&j, 0, sizeof j);
    j.kind = 6;
    j.a0 = xyz;
    j.a1 = off;
    j.a2 = tets;
    j.a3 = v12;
    j.a4 = fflags;
    j.a5 = flags;
    j.a6 = s_in;
    j.a7 = s_b;
    j.d0 = eps2;
    j.d1 = sd;
    j.d2 = soft_energy;
    j.i0 = check_quality;
    j.o0 = result;
    tw_parallel(j, n, nthreads);
}

/* =========================================================================
 * The checks of one edge removal (EdgeRemover::removeAnEdge_32 / _44 / _56,
 * EdgeRemover.cpp:125-177, :277-369, :456-600) for the edge (v1, v2) whose
 * shell (old_t_ids, in the caller's order) is the k tets shell[4k]; only the
 * variant for k = 3, 4 or 5 applies (the others return false at once).
 * Energy AMIPS with use_energy_max (State.h:53): a configuration's quality is
 * the max of its tets' calTetQuality_AMIPS (getCheckQuality, :575-603), the
 * old one the max over the shell (the stored qualities, equal to
 * calTetQuality at the current positions).  budget: equal_buget at the call;
 * while positive, each comparison accepts an equal max and spends a unit
 * (:169-176).  The vertices must be rounded (isFlip on posf).  Returns
 * SWAP_SUCCESS 0 (config: the configuration taken), SWAP_FLIP 1 (every
 * configuration inverts a tet), SWAP_QUALITY 2 (not better), SWAP_SIZE 3 (a
 * shell of another size or not around the edge); *spent = budget units spent.
 * The reference's order of tests is kept, including its early exits: in 4-4
 * a valid configuration that is not better ends the removal (:356-364), and a
 * later valid configuration must beat the earlier one.
 * ========================================================================= */
static void tw_tet_replace(const int32_t* t, int32_t from, int32_t to, int32_t* o)
{
    for (int j = 0; j < 4; ++j) o[j] = t[j];
    for (int j = 0; j < 4; ++j)
        if (o[j] == from) { o[j] = to; break; }   /* std::find: the first occurrence */
}
static int tw_tet_has(const int32_t* t, int32_t v)
{
    return t[0] == v || t[1] == v || t[2] == v || t[3] == v;
}
static void tw_tet_coords(const double* xyz, const int32_t* t, double T[12])
{
    for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 3; ++k) T[3 * j + k] = xyz[3 * (size_t)t[j] + k];
}
static int tw_tets_flip(const double* xyz, const int32_t* ts, int m)
{
    for (int i = 0; i < m; ++i) {
        double T[12];
        tw_tet_coords(xyz, ts + 4 * i, T);
        if (two_tet_flip(T)) return 1;
    }
    return 0;
}
static double tw_tet_q(const double* xyz, const int32_t* t)
{
    double T[12];
    tw_tet_coords(xyz, t, T);
    return two_tet_quality(T);
}
static int tw_swap_better(double nq, double oq, int* budget, int* spent)
{
    if (*budget > 0) {
        --*budget;
        ++*spent;
        return nq <= oq;
    }
    return nq < oq;
}
/* n12_v_ids / n12_t_ids of :278-303 and :457-481: the ring of the shell's
 * other vertices, walked from tet 0; returns 0 when the shell is not a ring. */
static int tw_swap_ring(const int32_t* shell, int N, int32_t v1, int32_t v2, int32_t* nv,
                        int* tid)
{
    int32_t e[5][2];
    for (int i = 0; i < N; ++i) {
        int c = 0;
        for (int j = 0; j < 4; ++j) {
            const int32_t x = shell[4 * i + j];
            if (x != v1 && x != v2) {
                if (c == 2) return 0;
                e[i][c++] = x;
            }
        }
        if (c != 2) return 0;
    }
    int visited[5] = {0, 0, 0, 0, 0};
    int m = 2, mt = 1;
    nv[0] = e[0][0];
    nv[1] = e[0][1];
    tid[0] = 0;
    visited[0] = 1;
    for (int it = 0; it < N - 2; ++it) {
        for (int j = 0; j < N; ++j) {
            if (visited[j]) continue;
            if (e[j][0] == nv[m - 1]) {
                visited[j] = 1;
                nv[m++] = e[j][1];
            } else if (e[j][1] == nv[m - 1]) {
                visited[j] = 1;
                nv[m++] = e[j][0];
            }
            if (visited[j]) {
                tid[mt++] = j;
                break;
            }
        }
    }
    if (m != N) return 0;
    for (int j = 0; j < N; ++j)
        if (!visited[j]) { tid[mt++] = j; break; }
    return mt == N;
}

int two_swap_check(const double* xyz, const int32_t* shell, int32_t k, int32_t v1, int32_t v2,
                   int budget, int* config, int* spent)
{
    *config = -1;
    *spent = 0;
    if (k < 3 || k > 5) return 3;
    for (int i = 0; i < k; ++i)
        if (!tw_tet_has(shell + 4 * i, v1) || !tw_tet_has(shell + 4 * i, v2)) return 3;
    double oq = 0.0;
    for (int i = 0; i < k; ++i) {
        const double q = tw_tet_q(xyz, shell + 4 * i);
        if (q > oq) oq = q;
    }
    int32_t nt[8];
    if (k == 3) {
        int32_t vv[2];
        int c = 0;
        for (int j = 0; j < 4; ++j)
            if (shell[j] != v1 && shell[j] != v2) vv[c++] = shell[j];
        const int32_t* a = shell + 4;
        const int32_t* b = shell + 8;
        if (!tw_tet_has(a, vv[0])) {
            a = shell + 8;
            b = shell + 4;
        }
        tw_tet_replace(a, v1, vv[1], nt);
        tw_tet_replace(b, v2, vv[0], nt + 4);
        if (tw_tets_flip(xyz, nt, 2)) return 1;
        const double q0 = tw_tet_q(xyz, nt), q1 = tw_tet_q(xyz, nt + 4);
        double nq = 0.0;
        if (q0 > nq) nq = q0;
        if (q1 > nq) nq = q1;
        if (!tw_swap_better(nq, oq, &budget, spent)) return 2;
        *config = 0;
        return 0;
    }
    int32_t nv[5];
    int tid[5];
    if (!tw_swap_ring(shell, k, v1, v2, nv, tid)) return 3;
    if (k == 4) {
        int valid = 0;
        for (int i = 0; i < 2; ++i) {
            int32_t ts[16];
            const int32_t a = nv[i], b = nv[2 + i];
            for (int j = 0; j < 4; ++j) {
                const int32_t* t = shell + 4 * j;
                if (tw_tet_has(t, a))
                    tw_tet_replace(t, v2, b, ts + 4 * j);
                else
                    tw_tet_replace(t, v1, a, ts + 4 * j);
            }
            if (tw_tets_flip(xyz, ts, 4)) continue;
            double nq = 0.0;
            for (int j = 0; j < 4; ++j) {
                const double q = tw_tet_q(xyz, ts + 4 * j);
                if (q > nq) nq = q;
            }
            if (!tw_swap_better(nq, oq, &budget, spent)) return 2;
            valid = 1;
            oq = nq;
            *config = i;
        }
        return valid ? 0 : 1;
    }
    /* k == 5 */
    int vvalid[5] = {1, 1, 1, 1, 1};
    double q1[5][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
    for (int i = 0; i < 5; ++i) {
        if (!vvalid[(i + 1) % 5] && !vvalid[(i + 4) % 5]) continue;
        const int32_t* t = shell + 4 * tid[i];
        tw_tet_replace(t, v1, nv[(i + 4) % 5], nt);
        tw_tet_replace(t, v2, nv[(i + 4) % 5], nt + 4);
        if (tw_tets_flip(xyz, nt, 2)) {
            vvalid[(i + 1) % 5] = 0;
            vvalid[(i + 4) % 5] = 0;
            continue;
        }
        q1[i][0] = tw_tet_q(xyz, nt);
        q1[i][1] = tw_tet_q(xyz, nt + 4);
    }
    if (!(vvalid[0] || vvalid[1] || vvalid[2] || vvalid[3] || vvalid[4])) return 1;
    int sel = -1, tested = 0;
    for (int i = 0; i < 5; ++i) {
        if (!vvalid[i]) continue;
        const int32_t* t = shell + 4 * tid[(i + 2) % 5];
        tw_tet_replace(t, v1, nv[i], nt);
        tw_tet_replace(t, v2, nv[i], nt + 4);
        if (tw_tets_flip(xyz, nt, 2)) continue;
        tested = 1;
        const double qs[6] = {tw_tet_q(xyz, nt), tw_tet_q(xyz, nt + 4), q1[(i + 1) % 5][0],
                              q1[(i + 4) % 5][0], q1[(i + 1) % 5][1], q1[(i + 4) % 5][1]};
        double nq = 0.0;
        for (int j = 0; j < 6; ++j)
            if (qs[j] > nq) nq = qs[j];
        if (!tw_swap_better(nq, oq, &budget, spent)) continue;
        oq = nq;
        sel = i;
    }
    if (sel < 0) return tested ? 2 : 1;
    *config = sel;
    return 0;
}

void two_swap_check_batch(const double* xyz, const int32_t* off, const int32_t* tets,
                          const int32_t* v12, const int32_t* budget, int64_t n, uint8_t* result,
                          int8_t* config, uint8_t* spent)
{
    for (int64_t i = 0; i < n; ++i) {
        int cfg = -1, sp = 0;
        result[i] = (uint8_t)two_swap_check(xyz, tets + 4 * (size_t)off[i], off[i + 1] - off[i],
                                            v12[2 * i], v12[2 * i + 1], budget ? budget[i] : 0,
                                            &cfg, &sp);
        config[i] = (int8_t)cfg;
        spent[i] = (uint8_t)sp;
    }
}
