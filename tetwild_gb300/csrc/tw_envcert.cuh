// tw_envcert.cuh -- certified binary32 envelope traversal
// (TW_PRECISION_FP32_CERTIFIED), included by tw_envelope.cu.
//
// Notation: u = 2^-24 (binary32 unit roundoff), u64 = 2^-53, M = max of the
// query point's |coordinates| and the surface's largest |coordinate|.
//
// Query point: ph = p rounded to binary32, pl = (p - ph) rounded, so
// p = ph + pl up to u^2 |p|.
//
// Boxes (binary32, rounded outward): a child is skipped only when its
// computed squared distance to ph exceeds thr = (eps (1 + 2^-20) + tau +
// slack)^2 evaluated with upward rounding, tau = 2^-21 M + 2^-20 eps: tau
// covers the rounding of the point (sqrt3 u M) and of the distance (3u eps),
// slack = 16 u64 M the rounding of the FP64 facet evaluation.
//
// Facets: r = p - a is formed in binary32 as (ph - ah) + (pl - al), with
// |r32 - r| <= 2u|r| + 4u^2 M per component.  In the orthonormal frame
// (n, ne_e, t_e) of the facet, h = n.r is the distance to the plane,
// s_e = ne_e.r - c_e the signed distance to edge e's line (positive outside)
// and tau_e = t_e.r - o_e the position along edge e, whose segment is at
// distance sqrt(h^2 + s_e^2 + x_e^2), x_e = max(0, -tau_e, tau_e - len_e).
// The exact point-facet distance is |h| when no edge line is crossed, the
// distance to segment e when only edge e's is, and the smaller of the two
// segment distances when two are.  Each quantity is evaluated in binary32
// with a proven bound on its error:
//   delta_h   = 8u R1 + 16u^2 M                 (normal u R1, r 2u R1 + 12u^2 M, dot 3.01u R1)
//   delta_s_e = 10u (R1 + |c_e|) + 16u^2 M      (as delta_h, plus offset and subtraction)
//   delta_t_e = 12u (R1 + |o_e|) + 16u^2 M      (t_e = n x ne_e formed in binary32: 3u)
//   delta_x_e = delta_t_e + 2u (|tau_e| + len_e)
// with R1 = |r|_1.  When every crossing is certain this yields a lower
// bound L and an upper bound U of the exact distance; when a crossing is
// uncertain L falls back to sqrt(h^2 + max(0, max_e s_e)^2) (the facet lies in
// the plane and inside every edge's half-plane) and U to the nearest segment.
// The facet is out when L^2 > (eps + slack)^2 (1 + 2^-18), in when
// U^2 < (eps - slack)^2 (1 - 2^-18) (the margins cover the FP64 evaluation
// and the final binary32 sums), and otherwise, the band, it is evaluated in
// FP64 exactly as in TW_PRECISION_FP64.  So every decision equals FP64's.
// Included by tw_envelope.cu inside namespace tw, after leaf_sqdist, kStack
// and kTraversalError.
#pragma once

struct TravStats {
    uint32_t facets = 0;  // facets reached
    uint32_t fp64 = 0;    // facets evaluated in FP64
};

// eps = sqrt(eps2) rounded up and down to binary32 (computed on the host).
struct EpsParams {
    double eps2;
    float eps_hi, eps_lo;
};

struct CertQuery {
    float ph[3], pl[3];
    float Mu2;   // 16 u^2 M
    float thr;   // box threshold on the squared distance
    float e2hi;  // facet out when L^2 > e2hi
    float e2lo;  // facet in when U^2 < e2lo
};

constexpr float kUf = 5.9604644775390625e-08f;  // 2^-24

__device__ __forceinline__ CertQuery cert_query(const V3& p, const EpsParams& E, float scale_hi) {
    CertQuery q;
    const double pv[3] = {p.x, p.y, p.z};
    float m = scale_hi;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        q.ph[k] = d2f_rn(pv[k]);
        q.pl[k] = d2f_rn(pv[k] - f2d_exact(q.ph[k]));
        m = fmaxf(m, fabsf(q.ph[k]));
    }
    const float mu = __fmul_ru(m, 1.00000012f);                          // >= max |p|, |a|
    const float slack = __fmul_ru(1.7763568394002505e-15f, mu);          // 16 u64 M
    const float tau = __fadd_ru(__fmul_ru(4.76837158203125e-07f, mu),
                                __fmul_ru(9.5367431640625e-07f, E.eps_hi));
    const float eb = __fadd_ru(__fadd_ru(__fmul_ru(E.eps_hi, 1.00000095f), tau), slack);
    q.thr = __fmul_ru(eb, eb);
    const float eh = __fadd_ru(E.eps_hi, slack);
    q.e2hi = __fmul_ru(__fmul_ru(eh, eh), 1.00000381f);                  // (1 + 2^-18)
    const float el = __fsub_rd(E.eps_lo, slack);
    q.e2lo = el > 0.0f ? __fmul_rd(__fmul_rd(el, el), 0.999996185f) : 0.0f;  // (1 - 2^-18)
    q.Mu2 = __fmul_ru(5.684341886080802e-14f, mu);                       // 16 u^2 M
    return q;
}

__device__ __forceinline__ float point_box_sqdist32(float px, float py, float pz, const float* lo,
                                                    const float* hi) {
    float r = 0.0f;
    if (px < lo[0]) { float d = lo[0] - px; r = d * d; }
    else if (px > hi[0]) { float d = px - hi[0]; r = d * d; }
    if (py < lo[1]) { float d = lo[1] - py; r = r + d * d; }
    else if (py > hi[1]) { float d = py - hi[1]; r = r + d * d; }
    if (pz < lo[2]) { float d = lo[2] - pz; r = r + d * d; }
    else if (pz > hi[2]) { float d = pz - hi[2]; r = r + d * d; }
    return r;
}

constexpr int kFacetOut = 0;
constexpr int kFacetIn = 1;
constexpr int kFacetBand = 2;

// The facet record as seven float4:
// ah0 ah1 ah2 al0 | al1 al2 n0 n1 | n2 ne00 ne01 ne02 | ne10 ne11 ne12 ne20 |
// ne21 ne22 c0 c1 | c2 o0 o1 o2 | len0 len1 len2 ok  (ok == 0: always the band)
__device__ __forceinline__ int facet_classify_rec(const float4& w0, const float4& w1,
                                                  const float4& w2, const float4& w3,
                                                  const float4& w4, const float4& w5,
                                                  const float4& w6, const CertQuery& q) {
    if (__float_as_uint(w6.w) == 0u) return kFacetBand;
    const float rx = (q.ph[0] - w0.x) + (q.pl[0] - w0.w);
    const float ry = (q.ph[1] - w0.y) + (q.pl[1] - w1.x);
    const float rz = (q.ph[2] - w0.z) + (q.pl[2] - w1.y);
    const float R1 = fabsf(rx) + fabsf(ry) + fabsf(rz);
    const float n0 = w1.z, n1 = w1.w, n2 = w2.x;
    const float ne[3][3] = {{w2.y, w2.z, w2.w}, {w3.x, w3.y, w3.z}, {w3.w, w4.x, w4.y}};
    const float c[3] = {w4.z, w4.w, w5.x};
    const float o[3] = {w5.y, w5.z, w5.w};
    const float len[3] = {w6.x, w6.y, w6.z};
    const float h = fabsf(fmaf(n2, rz, fmaf(n1, ry, n0 * rx)));
    const float dh = fmaf(8.0f * kUf, R1, q.Mu2);
    const float hlo = fmaxf(h - dh, 0.0f), hhi = h + dh;
    float s[3], ds[3];
    bool maybe[3], sure[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        s[e] = fmaf(ne[e][2], rz, fmaf(ne[e][1], ry, ne[e][0] * rx)) - c[e];
        ds[e] = fmaf(10.0f * kUf, R1 + fabsf(c[e]), q.Mu2);
        maybe[e] = s[e] + ds[e] >= 0.0f;
        sure[e] = s[e] - ds[e] > 0.0f;
    }
    // the generic lower bound first: it excludes most facets near the query
    // without the edge-segment terms
    const float sm = fmaxf(fmaxf(s[0] - ds[0], s[1] - ds[1]), fmaxf(s[2] - ds[2], 0.0f));
    if (fmaf(hlo, hlo, sm * sm) > q.e2hi) return kFacetOut;
    float L2, U2;
    if (!maybe[0] && !maybe[1] && !maybe[2]) {
        L2 = hlo * hlo;
        U2 = hhi * hhi;
    } else {
        float Lx = __int_as_float(0x7f800000), Ux = __int_as_float(0x7f800000);
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            if (!maybe[e]) continue;
            const float t0 = fmaf(n1, ne[e][2], -n2 * ne[e][1]);
            const float t1 = fmaf(n2, ne[e][0], -n0 * ne[e][2]);
            const float t2 = fmaf(n0, ne[e][1], -n1 * ne[e][0]);
            const float tau = fmaf(t2, rz, fmaf(t1, ry, t0 * rx)) - o[e];
            const float dtau = fmaf(12.0f * kUf, R1 + fabsf(o[e]), q.Mu2);
            const float x = fmaxf(fmaxf(-tau, tau - len[e]), 0.0f);
            const float dx = fmaf(2.0f * kUf, fabsf(tau) + len[e], dtau);
            const float as = fabsf(s[e]);
            const float shi = as + ds[e], xhi = x + dx;
            const float slo = fmaxf(as - ds[e], 0.0f), xlo = fmaxf(x - dx, 0.0f);
            Ux = fminf(Ux, fmaf(hhi, hhi, fmaf(shi, shi, xhi * xhi)));
            Lx = fminf(Lx, fmaf(hlo, hlo, fmaf(slo, slo, xlo * xlo)));
        }
        U2 = Ux;
        if (maybe[0] == sure[0] && maybe[1] == sure[1] && maybe[2] == sure[2])
            L2 = Lx;
        else
            L2 = fmaf(hlo, hlo, sm * sm);
    }
    if (L2 > q.e2hi) return kFacetOut;
    if (U2 < q.e2lo) return kFacetIn;
    return kFacetBand;
}

__device__ __forceinline__ int facet_classify(const FacetCull* __restrict__ cull, int32_t f,
                                              const CertQuery& q) {
    const float4* w = reinterpret_cast<const float4*>(cull + f);
    const float4 w6 = __ldg(w + 6);
    if (__float_as_uint(w6.w) == 0u) return kFacetBand;
    return facet_classify_rec(__ldg(w), __ldg(w + 1), __ldg(w + 2), __ldg(w + 3), __ldg(w + 4),
                              __ldg(w + 5), w6, q);
}

// The certified test of one leaf: FP32 classification, FP64 in the band.
__device__ __forceinline__ bool cert_leaf_within(const FacetCull* __restrict__ cull,
                                                 const double* __restrict__ tri, int32_t lf,
                                                 const V3& p, const CertQuery& q, double eps2,
                                                 TravStats& st) {
    ++st.facets;
    int cls = facet_classify(cull, lf, q);
    if (cls == kFacetIn) return true;
    if (cls == kFacetOut) return false;
    ++st.fp64;
    return leaf_sqdist(tri, lf, p) <= eps2;
}

// FP32-culled traversal; decisions identical to find_facet_within (FP64).
__device__ __forceinline__ int32_t find_facet_within32(const BvhNode32* __restrict__ nodes,
                                                       const FacetCull* __restrict__ cull,
                                                       const double* __restrict__ tri, int32_t nf,
                                                       const V3& p, const CertQuery& q,
                                                       double eps2, TravStats& st) {
    auto test_leaf = [&](int32_t lf) -> bool {
        ++st.facets;
        int cls = facet_classify(cull, lf, q);
        if (cls == kFacetIn) return true;
        if (cls == kFacetOut) return false;
        ++st.fp64;
        return leaf_sqdist(tri, lf, p) <= eps2;
    };
    if (nf == 1) return test_leaf(0) ? 0 : -1;
    const float px = q.ph[0], py = q.ph[1], pz = q.ph[2];
    int32_t stack[kStack];
    int sp = 0;
    int32_t cur = 0;
    for (int32_t iter = 0; iter < nf; ++iter) {
        if ((uint32_t)cur >= (uint32_t)(nf - 1)) return kTraversalError;
        const float4* nd = reinterpret_cast<const float4*>(nodes + cur);
        float4 q0 = __ldg(nd + 0), q1 = __ldg(nd + 1), q2 = __ldg(nd + 2);
        int4 q3 = __ldg(reinterpret_cast<const int4*>(nd + 3));
        float lo0[3] = {q0.x, q0.y, q0.z}, hi0[3] = {q0.w, q1.x, q1.y};
        float lo1[3] = {q1.z, q1.w, q2.x}, hi1[3] = {q2.y, q2.z, q2.w};
        int2 ch = make_int2(q3.x, q3.y);
        float d0 = point_box_sqdist32(px, py, pz, lo0, hi0);
        float d1 = point_box_sqdist32(px, py, pz, lo1, hi1);
        bool h0 = d0 <= q.thr, h1 = d1 <= q.thr;
        // leaf children: the nearer box first, so a contained point stops sooner
        const bool second_first = d1 < d0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const bool right = (k == 0) == second_first;
            const int32_t c = right ? ch.y : ch.x;
            if (!(right ? h1 : h0) || c >= 0) continue;
            const int32_t lf = ~c;
            if ((uint32_t)lf >= (uint32_t)nf) return kTraversalError;
            if (test_leaf(lf)) return lf;
            if (right) h1 = false; else h0 = false;
        }
        if (h0 && h1) {
            if (sp >= kStack) return kTraversalError;
            int32_t nearc = (d0 <= d1) ? ch.x : ch.y;
            int32_t farc = (d0 <= d1) ? ch.y : ch.x;
            stack[sp++] = farc;
            cur = nearc;
        } else if (h0) {
            cur = ch.x;
        } else if (h1) {
            cur = ch.y;
        } else {
            if (sp == 0) return -1;
            cur = stack[--sp];
        }
    }
    return kTraversalError;
}
