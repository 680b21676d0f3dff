// geo_shim.h -- the small part of the geogram API that the reference's
// mesh_AABB.{h,cpp}, DistanceQuery.h and sampleTriangle use, written for this
// repository so those reference files compile without geogram.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref).  The vec3 operators follow
// geogram's documented semantics (component-wise, left-to-right sums,
// normalize = (1/length) * v).  Geom::point_triangle_squared_distance is the
// oracle's point-triangle distance (Ericson's closest-point method), since
// geogram's own routine is not part of the reference sources.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../tw_oracle.h"

#define GEOGRAM_API
#define geo_debug_assert(x) ((void)0)
#define geo_assert(x) ((void)0)

namespace GEO {

typedef unsigned int index_t;
typedef unsigned char coord_index_t;
static const index_t NO_FACET = index_t(-1);

template <class T> inline T geo_sqr(T x) { return x * x; }
enum Sign { NEGATIVE = -1, ZERO = 0, POSITIVE = 1 };
template <class T> inline Sign geo_sgn(T x) { return (x > 0) ? POSITIVE : ((x < 0) ? NEGATIVE : ZERO); }

struct vec3 {
    double x, y, z;
    vec3() : x(0.0), y(0.0), z(0.0) {}
    vec3(double a, double b, double c) : x(a), y(b), z(c) {}
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const double& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    double* data() { return &x; }
    const double* data() const { return &x; }
    double length2() const { return x * x + y * y + z * z; }
    double length() const { return std::sqrt(length2()); }
    double distance2(const vec3& v) const {
        double dx = v.x - x, dy = v.y - y, dz = v.z - z;
        return dx * dx + dy * dy + dz * dz;
    }
    double distance(const vec3& v) const { return std::sqrt(distance2(v)); }
    vec3 operator+(const vec3& v) const { return vec3(x + v.x, y + v.y, z + v.z); }
    vec3 operator-(const vec3& v) const { return vec3(x - v.x, y - v.y, z - v.z); }
    template <class T2> vec3 operator*(T2 s) const {
        return vec3(x * double(s), y * double(s), z * double(s));
    }
    template <class T2> vec3 operator/(T2 s) const {
        return vec3(x / double(s), y / double(s), z / double(s));
    }
};
template <class T2> inline vec3 operator*(T2 s, const vec3& v) {
    return vec3(double(s) * v.x, double(s) * v.y, double(s) * v.z);
}
inline double dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline double length(const vec3& v) { return v.length(); }
inline double length2(const vec3& v) { return v.length2(); }
inline double distance2(const vec3& a, const vec3& b) { return b.distance2(a); }
inline double distance(const vec3& a, const vec3& b) { return b.distance(a); }
inline vec3 normalize(const vec3& v) {
    double s = length(v);
    if (s > 1e-30) s = 1.0 / s;
    return s * v;
}

template <class T> class vector : public std::vector<T> {
public:
    using std::vector<T>::vector;
    index_t size() const { return index_t(std::vector<T>::size()); }
};

struct Box {
    double xyz_min[3];
    double xyz_max[3];
    bool contains(const vec3& p) const {
        for (int c = 0; c < 3; ++c)
            if (p[c] < xyz_min[c] || p[c] > xyz_max[c]) return false;
        return true;
    }
};
inline void bbox_union(Box& t, const Box& a, const Box& b) {
    for (int c = 0; c < 3; ++c) {
        t.xyz_min[c] = std::min(a.xyz_min[c], b.xyz_min[c]);
        t.xyz_max[c] = std::max(a.xyz_max[c], b.xyz_max[c]);
    }
}
inline bool bboxes_overlap(const Box& a, const Box& b) {
    for (int c = 0; c < 3; ++c)
        if (a.xyz_max[c] < b.xyz_min[c] || b.xyz_max[c] < a.xyz_min[c]) return false;
    return true;
}

class Mesh {
public:
    struct Vertices {
        std::vector<vec3> pts;
        const double* point_ptr(index_t v) const { return pts[v].data(); }
        index_t nb() const { return index_t(pts.size()); }
    } vertices;
    struct FacetCorners {
        std::vector<index_t> v;
        index_t vertex(index_t c) const { return v[c]; }
    } facet_corners;
    struct Facets {
        index_t n = 0;
        index_t nb() const { return n; }
        index_t corners_begin(index_t f) const { return 3 * f; }
        index_t corners_end(index_t f) const { return 3 * f + 3; }
        index_t nb_vertices(index_t) const { return 3; }
        bool are_simplices() const { return true; }
    } facets;
};

enum MeshOrder { MESH_ORDER_HILBERT, MESH_ORDER_MORTON };
void mesh_reorder(Mesh& M, MeshOrder order);

enum MeshRepairMode { MESH_REPAIR_TOPOLOGY = 0, MESH_REPAIR_TRIANGULATE = 4, MESH_REPAIR_QUIET = 16 };
inline MeshRepairMode operator|(MeshRepairMode a, MeshRepairMode b) {
    return MeshRepairMode(int(a) | int(b));
}
inline void mesh_repair(Mesh&, MeshRepairMode, double = 0.0) {}

namespace Geom {
inline const vec3& mesh_vertex(const Mesh& M, index_t v) { return M.vertices.pts[v]; }
inline double distance2(const vec3& a, const vec3& b) { return GEO::distance2(a, b); }
inline double point_triangle_squared_distance(const vec3& p, const vec3& p1, const vec3& p2,
                                              const vec3& p3, vec3& nearest_p, double& l1,
                                              double& l2, double& l3) {
    double q[3];
    double d = two_point_triangle_sqdist(p.data(), p1.data(), p2.data(), p3.data(), q);
    nearest_p = vec3(q[0], q[1], q[2]);
    l1 = l2 = l3 = 0.0;
    return d;
}
inline double tetra_signed_volume(const vec3& p1, const vec3& p2, const vec3& p3, const vec3& p4) {
    return dot(p2 - p1, cross(p3 - p1, p4 - p1)) / 6.0;
}
}  // namespace Geom

}  // namespace GEO
