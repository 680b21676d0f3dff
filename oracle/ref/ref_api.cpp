// ref_api.cpp -- C entry points over the reference's OWN hot-path code.
//
// TEST INFRASTRUCTURE ONLY.  oracle/ref/build_ref.py slices these reference
// sources into oracle/_ref/src (git-ignored) and compiles them with this file
// into oracle/_ref/libtwref.so:
//   LocalOperations.cpp:28-291     comformalAMIPS{Energy,Jacobian,Hessian}_new
//   LocalOperations.cpp:1034-1109  isPointOutEnvelop, isFaceOutEnvelop_sampling
//   Common.cpp:143-255             sampleTriangle
//   LocalOperations.cpp:605-693    getAvgMaxEnergy, getMaxEnergy, getSecondMaxEnergy,
//                                  getFilterEnergy
//   geogram/mesh_AABB.{h,cpp}      MeshFacetsAABBWithEps (whole files)
//   DistanceQuery.h                get_point_facet_nearest_point
// The library is the pin for the oracle restatement and the timed CPU
// implementation of the reference arm of bench.py.  CGAL predicates that the
// slices call (Triangle_3f::is_degenerate) are served by the oracle's exact
// collinearity test, and geogram's point-triangle distance by the oracle's
// (see shim/geo_shim.h).
#include <array>
#include <cmath>
#include <numeric>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include <geogram/mesh/mesh.h>
#include <tetwild/geogram/mesh_AABB.h>
#include <tetwild/DistanceQuery.h>

#include "tw_oracle.h"

#define CHECK_ENVELOP true
#define TIMING_BREAKDOWN false

namespace tetwild {

struct Point_3f {
    double c[3];
    double operator[](int i) const { return c[i]; }
};
struct Triangle_3f {
    Point_3f v[3];
    const Point_3f& operator[](int i) const { return v[i]; }
    bool is_degenerate() const { return two_collinear(v[0].c, v[1].c, v[2].c) != 0; }
};
struct RefState {
    double eps_2 = 0.0;
    double sampling_dist = 0.0;
};
struct RefLogger {
    template <class... A> void trace(A&&...) const {}
    template <class... A> void debug(A&&...) const {}
};
inline RefLogger& logger() {
    static RefLogger l;
    return l;
}

void sampleTriangle(const std::array<GEO::vec3, 3>& vs, std::vector<GEO::vec3>& ps,
                    const double sampling_dist);

struct LocalOperations {
    RefState state;
    const GEO::Mesh& geo_sf_mesh;
    const GEO::MeshFacetsAABBWithEps& geo_sf_tree;
    LocalOperations(const GEO::Mesh& m, const GEO::MeshFacetsAABBWithEps& t)
        : geo_sf_mesh(m), geo_sf_tree(t) {}

    bool isPointOutEnvelop(const Point_3f& p);
    bool isFaceOutEnvelop_sampling(const Triangle_3f& tri);

    static double comformalAMIPSEnergy_new(const double* T);
    static void comformalAMIPSJacobian_new(const double* T, double* result_0);
    static void comformalAMIPSHessian_new(const double* T, double* result_0);
};

#include "amips_slice.inc"
#include "sample_slice.inc"
#include "envelope_slice.inc"

}  // namespace tetwild

// The full-mesh energy sweeps run over a per-tet quality array; their own
// LocalOperations holds just the members they read.
namespace tetwild_sweeps {
struct TetQualityRef {
    double slim_energy = 0.0;
};
struct SweepArgs {
    double filter_energy_thres = 10.0;
};
struct SweepState {
    double MAX_ENERGY = 1e50;   // State.h:29
};
struct LocalOperations {
    std::vector<TetQualityRef> tet_qualities;
    std::vector<bool> t_is_removed;
    const uint8_t* locked = nullptr;
    SweepArgs args;
    SweepState state;
    bool isTetLocked_ui(int i) const { return locked && locked[i]; }
    void getAvgMaxEnergy(double& avg_tq, double& max_tq);
    double getMaxEnergy();
    double getSecondMaxEnergy(double max_energy);
    double getFilterEnergy(bool& is_clean_up);
};
#include "sweeps_slice.inc"
}  // namespace tetwild_sweeps

// geogram's MESH_ORDER_MORTON spatial sort: recursive median split of the
// facet centroids along x, y, z in turn (affects the tree's shape only).
namespace GEO {
static void median_order(const std::vector<vec3>& cen, index_t* ids, index_t n, int axis) {
    if (n <= 1) return;
    index_t m = n / 2;
    std::nth_element(ids, ids + m, ids + n, [&](index_t a, index_t b) {
        if (cen[a][axis] != cen[b][axis]) return cen[a][axis] < cen[b][axis];
        return a < b;
    });
    median_order(cen, ids, m, (axis + 1) % 3);
    median_order(cen, ids + m, n - m, (axis + 1) % 3);
}
void mesh_reorder(Mesh& M, MeshOrder) {
    index_t nf = M.facets.nb();
    std::vector<vec3> cen(nf);
    std::vector<index_t> ids(nf);
    for (index_t f = 0; f < nf; ++f) {
        ids[f] = f;
        vec3 c;
        for (int k = 0; k < 3; ++k) c = c + M.vertices.pts[M.facet_corners.v[3 * f + k]];
        cen[f] = c / 3.0;
    }
    median_order(cen, ids.data(), nf, 0);
    std::vector<index_t> nv(3 * size_t(nf));
    for (index_t i = 0; i < nf; ++i)
        for (int k = 0; k < 3; ++k) nv[3 * i + k] = M.facet_corners.v[3 * ids[i] + k];
    M.facet_corners.v.swap(nv);
}
}  // namespace GEO

namespace {
struct RefSurface {
    GEO::Mesh mesh;
    GEO::MeshFacetsAABBWithEps* tree = nullptr;
};

template <class F> void parallel_for(int64_t n, int nthreads, F f) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads == 1 || n < 2) {
        f(int64_t(0), n);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) {
        int64_t lo = n * t / nthreads, hi = n * (t + 1) / nthreads;
        th.emplace_back([=]() { f(lo, hi); });
    }
    for (auto& x : th) x.join();
}
}  // namespace

extern "C" {

// T: SoA [12][n] (energy_ispc layout); E [n], J [3][n], H [9][n]; any may be NULL.
void twref_amips_batch_soa(const double* T, int64_t n, double* E, double* J, double* H,
                           int nthreads) {
    parallel_for(n, nthreads, [=](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
            double t[12], jj[3], hh[9];
            for (int c = 0; c < 12; ++c) t[c] = T[c * n + i];
            if (E) E[i] = tetwild::LocalOperations::comformalAMIPSEnergy_new(t);
            if (J) {
                tetwild::LocalOperations::comformalAMIPSJacobian_new(t, jj);
                for (int c = 0; c < 3; ++c) J[c * n + i] = jj[c];
            }
            if (H) {
                tetwild::LocalOperations::comformalAMIPSHessian_new(t, hh);
                for (int c = 0; c < 9; ++c) H[c * n + i] = hh[c];
            }
        }
    });
}

int64_t twref_sample_triangle(const double* v, double sd, double* out, int64_t cap) {
    std::array<GEO::vec3, 3> vs = {{GEO::vec3(v[0], v[1], v[2]), GEO::vec3(v[3], v[4], v[5]),
                                    GEO::vec3(v[6], v[7], v[8])}};
    std::vector<GEO::vec3> ps;
    tetwild::sampleTriangle(vs, ps, sd);
    int64_t n = int64_t(ps.size());
    for (int64_t i = 0; i < n && i < cap; ++i) {
        out[3 * i] = ps[i].x;
        out[3 * i + 1] = ps[i].y;
        out[3 * i + 2] = ps[i].z;
    }
    return n;
}

void* twref_surface_build(const double* V, int32_t nV, const int32_t* F, int32_t nF) {
    RefSurface* s = new RefSurface();
    s->mesh.vertices.pts.resize(size_t(nV));
    for (int32_t i = 0; i < nV; ++i) s->mesh.vertices.pts[i] = GEO::vec3(V[3 * i], V[3 * i + 1], V[3 * i + 2]);
    s->mesh.facet_corners.v.assign(F, F + 3 * size_t(nF));
    s->mesh.facets.n = GEO::index_t(nF);
    s->tree = new GEO::MeshFacetsAABBWithEps(s->mesh);
    return s;
}

void twref_surface_free(void* h) {
    RefSurface* s = static_cast<RefSurface*>(h);
    if (!s) return;
    delete s->tree;
    delete s;
}

void twref_points_out(void* h, const double* P, int64_t n, double eps2, uint8_t* out, int nthreads) {
    RefSurface* s = static_cast<RefSurface*>(h);
    parallel_for(n, nthreads, [=](int64_t lo, int64_t hi) {
        tetwild::LocalOperations ops(s->mesh, *s->tree);
        ops.state.eps_2 = eps2;
        for (int64_t i = lo; i < hi; ++i) {
            tetwild::Point_3f p = {{P[3 * i], P[3 * i + 1], P[3 * i + 2]}};
            out[i] = ops.isPointOutEnvelop(p) ? 1 : 0;
        }
    });
}

void twref_faces_out(void* h, const double* tris, int64_t n, double eps2, double sd, uint8_t* out,
                     int nthreads) {
    RefSurface* s = static_cast<RefSurface*>(h);
    parallel_for(n, nthreads, [=](int64_t lo, int64_t hi) {
        tetwild::LocalOperations ops(s->mesh, *s->tree);
        ops.state.eps_2 = eps2;
        ops.state.sampling_dist = sd;
        for (int64_t i = lo; i < hi; ++i) {
            const double* t = tris + 9 * i;
            tetwild::Triangle_3f tri = {{{{t[0], t[1], t[2]}}, {{t[3], t[4], t[5]}}, {{t[6], t[7], t[8]}}}};
            out[i] = ops.isFaceOutEnvelop_sampling(tri) ? 1 : 0;
        }
    });
}

// MeshFacetsAABBWithEps::nearest_facet (mesh_AABB.h:130-141): closest point
// and squared distance (the facet index refers to the tree's reordered facets
// and is not returned).
void twref_nearest(void* h, const double* P, int64_t n, double* Q, double* D, int nthreads) {
    RefSurface* s = static_cast<RefSurface*>(h);
    parallel_for(n, nthreads, [=](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
            GEO::vec3 p(P[3 * i], P[3 * i + 1], P[3 * i + 2]);
            GEO::vec3 q;
            double d = 0.0;
            s->tree->nearest_facet(p, q, d);
            Q[3 * i] = q.x;
            Q[3 * i + 1] = q.y;
            Q[3 * i + 2] = q.z;
            D[i] = d;
        }
    });
}

// The reference's sweeps over per-tet energies E (removed / locked masks may
// be NULL): out = {avg, max (getAvgMaxEnergy), getMaxEnergy, getSecondMaxEnergy
// of that max, getFilterEnergy}; *is_clean_up as getFilterEnergy leaves it (0
// when it does not set it).
void twref_energy_sweeps(const double* E, const uint8_t* removed, const uint8_t* locked,
                         int64_t n, double thres, double* out, int* is_clean_up) {
    tetwild_sweeps::LocalOperations ops;
    ops.tet_qualities.resize(size_t(n));
    ops.t_is_removed.assign(size_t(n), false);
    for (int64_t i = 0; i < n; ++i) {
        ops.tet_qualities[size_t(i)].slim_energy = E[i];
        if (removed) ops.t_is_removed[size_t(i)] = removed[i] != 0;
    }
    ops.locked = locked;
    ops.args.filter_energy_thres = thres;
    double avg = 0.0, mx = 0.0;
    ops.getAvgMaxEnergy(avg, mx);
    const double m = ops.getMaxEnergy();
    const double m2 = ops.getSecondMaxEnergy(m);
    bool clean = false;
    const double f = ops.getFilterEnergy(clean);
    out[0] = avg;
    out[1] = mx;
    out[2] = m;
    out[3] = m2;
    out[4] = f;
    *is_clean_up = clean ? 1 : 0;
}

}  // extern "C"
