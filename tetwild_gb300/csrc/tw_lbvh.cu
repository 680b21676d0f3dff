// tw_lbvh.cu -- device-built LBVH over the input surface.
//
// Replaces the MeshFacetsAABBWithEps constructor (mesh_AABB.cpp:356-379),
// which Morton-reorders the facets and builds an implicit median-split tree
// on one CPU thread.  Here, on the device:
//   1. gather the facets' coordinates and centroids, reduce the centroid box;
//   2. 30-bit Morton codes (10 bits per axis) of the normalised centroids;
//   3. radix sort (CUB) of (code, facet) pairs;
//   4. binary radix tree (Karras, "Maximizing Parallelism in the
//      Construction of BVHs, Octrees, and k-d Trees", HPG 2012), ties in the
//      codes broken by leaf index;
//   5. bottom-up refit of FP64 boxes.  Boxes are the exact min/max of the
//      facet vertices (min/max do not round), as in get_facet_bbox
//      (mesh_AABB.cpp:63-79).
// Each internal node stores both children's boxes (128-byte record), so a
// traversal step is one line of L2/HBM traffic.
#include <cub/device/device_radix_sort.cuh>

#include "tw_device.cuh"
#include "tw_internal.h"

namespace tw {

__global__ void k_gather_tris(const double* __restrict__ V, int32_t nv,
                              const int32_t* __restrict__ F, int32_t nf,
                              double* __restrict__ tri, double* __restrict__ cen,
                              int* __restrict__ bad) {
    int32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    double c[3] = {0.0, 0.0, 0.0};
    for (int v = 0; v < 3; ++v) {
        int32_t id = F[3 * f + v];
        if (id < 0 || id >= nv) {
            atomicExch(bad, 1);
            id = 0;
        }
        for (int k = 0; k < 3; ++k) {
            double x = V[3 * (int64_t)id + k];
            tri[9 * (int64_t)f + 3 * v + k] = x;
            c[k] += x;
        }
    }
    for (int k = 0; k < 3; ++k) cen[3 * (int64_t)f + k] = c[k] / 3.0;
}

// One block: min/max of the centroids, and max |coordinate| of the facets.
__global__ void k_bounds(const double* __restrict__ cen, const double* __restrict__ tri,
                         int32_t nf, double* __restrict__ out) {
    __shared__ double red[7][1024];
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    double sc = 0.0;
    for (int32_t f = threadIdx.x; f < nf; f += blockDim.x) {
        for (int k = 0; k < 3; ++k) {
            double x = cen[3 * (int64_t)f + k];
            lo[k] = fmin(lo[k], x);
            hi[k] = fmax(hi[k], x);
        }
        for (int k = 0; k < 9; ++k) sc = fmax(sc, fabs(tri[9 * (int64_t)f + k]));
    }
    for (int k = 0; k < 3; ++k) {
        red[k][threadIdx.x] = lo[k];
        red[3 + k][threadIdx.x] = hi[k];
    }
    red[6][threadIdx.x] = sc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            for (int k = 0; k < 3; ++k) {
                red[k][threadIdx.x] = fmin(red[k][threadIdx.x], red[k][threadIdx.x + w]);
                red[3 + k][threadIdx.x] = fmax(red[3 + k][threadIdx.x], red[3 + k][threadIdx.x + w]);
            }
            red[6][threadIdx.x] = fmax(red[6][threadIdx.x], red[6][threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x < 7) out[threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_morton(const double* __restrict__ cen, int32_t nf,
                         const double* __restrict__ bounds, uint32_t* __restrict__ codes,
                         int32_t* __restrict__ ids) {
    int32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
        double lo = bounds[k], hi = bounds[3 + k];
        double ext = hi - lo;
        double t = ext > 0.0 ? (cen[3 * (int64_t)f + k] - lo) / ext : 0.5;
        double s = t * 1024.0;
        s = fmin(fmax(s, 0.0), 1023.0);
        q[k] = (uint32_t)s;
    }
    codes[f] = (morton_expand10(q[0]) << 2) | (morton_expand10(q[1]) << 1) | morton_expand10(q[2]);
    ids[f] = f;
}

__global__ void k_scatter_tris(const double* __restrict__ tri_in, const int32_t* __restrict__ ids,
                               int32_t nf, double* __restrict__ tri_out,
                               int32_t* __restrict__ facet_id, double* __restrict__ leafbox) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    int32_t f = ids[i];
    facet_id[i] = f;
    double t[9];
    for (int k = 0; k < 9; ++k) {
        t[k] = tri_in[9 * (int64_t)f + k];
        tri_out[9 * (int64_t)i + k] = t[k];
    }
    for (int k = 0; k < 3; ++k) {
        double lo = fmin(fmin(t[k], t[3 + k]), t[6 + k]);
        double hi = fmax(fmax(t[k], t[3 + k]), t[6 + k]);
        leafbox[6 * (int64_t)i + k] = lo;
        leafbox[6 * (int64_t)i + 3 + k] = hi;
    }
}

__device__ __forceinline__ int lbvh_delta(const uint32_t* __restrict__ codes, int32_t n, int32_t i,
                                          int32_t j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = codes[i], b = codes[j];
    if (a == b) return 32 + __clz((uint32_t)(i ^ j));
    return __clz(a ^ b);
}

__global__ void k_karras(const uint32_t* __restrict__ codes, int32_t n, BvhNode* __restrict__ nodes,
                         int32_t* __restrict__ iparent, int32_t* __restrict__ lparent) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (lbvh_delta(codes, n, i, i + 1) - lbvh_delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = lbvh_delta(codes, n, i, i - d);
    int32_t lmax = 2;
    while (lbvh_delta(codes, n, i, i + lmax * d) > dmin) lmax *= 2;
    int32_t l = 0;
    for (int32_t t = lmax / 2; t >= 1; t /= 2)
        if (lbvh_delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
    int32_t j = i + l * d;
    int dnode = lbvh_delta(codes, n, i, j);
    int32_t s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (lbvh_delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int32_t gamma = i + s * d + (d < 0 ? d : 0);
    int32_t lo = i < j ? i : j, hi = i < j ? j : i;
    int32_t left, right;
    if (lo == gamma) {
        left = ~gamma;
        lparent[gamma] = i;
    } else {
        left = gamma;
        iparent[gamma] = i;
    }
    if (hi == gamma + 1) {
        right = ~(gamma + 1);
        lparent[gamma + 1] = i;
    } else {
        right = gamma + 1;
        iparent[gamma + 1] = i;
    }
    nodes[i].child[0] = left;
    nodes[i].child[1] = right;
    if (i == 0) iparent[0] = -1;
}

__device__ __forceinline__ void load_box(const double* __restrict__ ibox,
                                         const double* __restrict__ leafbox, int32_t c,
                                         double* b) {
    const double* src = (c >= 0) ? ibox + 6 * (int64_t)c : leafbox + 6 * (int64_t)(~c);
#pragma unroll
    for (int k = 0; k < 6; ++k) b[k] = __ldcg(src + k);
}

__global__ void k_refit(BvhNode* __restrict__ nodes, double* __restrict__ ibox,
                        const double* __restrict__ leafbox, const int32_t* __restrict__ iparent,
                        const int32_t* __restrict__ lparent, int* __restrict__ flags, int32_t n) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t node = lparent[i];
    // a root-to-leaf path has at most n - 1 internal nodes
    for (int32_t hops = 0; node >= 0 && node < n - 1 && hops < n; ++hops) {
        __threadfence();
        if (atomicAdd(flags + node, 1) == 0) return;  // sibling not finished yet
        __threadfence();
        int32_t c0 = nodes[node].child[0], c1 = nodes[node].child[1];
        double b0[6], b1[6];
        load_box(ibox, leafbox, c0, b0);
        load_box(ibox, leafbox, c1, b1);
        BvhNode& N = nodes[node];
        for (int k = 0; k < 3; ++k) {
            N.lo0[k] = b0[k];
            N.hi0[k] = b0[3 + k];
            N.lo1[k] = b1[k];
            N.hi1[k] = b1[3 + k];
            __stcg(ibox + 6 * (int64_t)node + k, fmin(b0[k], b1[k]));
            __stcg(ibox + 6 * (int64_t)node + 3 + k, fmax(b0[3 + k], b1[3 + k]));
        }
        node = iparent[node];
    }
}

// binary32 copy of the tree with outward-rounded boxes
__global__ void k_nodes32(const BvhNode* __restrict__ nodes, int32_t ni,
                          BvhNode32* __restrict__ out) {
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ni) return;
    const BvhNode& N = nodes[i];
    BvhNode32 M;
    for (int k = 0; k < 3; ++k) {
        M.lo0[k] = __double2float_rd(N.lo0[k]);
        M.hi0[k] = __double2float_ru(N.hi0[k]);
        M.lo1[k] = __double2float_rd(N.lo1[k]);
        M.hi1[k] = __double2float_ru(N.hi1[k]);
    }
    M.child[0] = N.child[0];
    M.child[1] = N.child[1];
    M.pad[0] = M.pad[1] = 0;
    out[i] = M;
}

// Culling data of each leaf facet (FacetCull).  The facet is usable for
// culling only when |ab x ac| > 2^-20 |ab| |ac| (the angle between the edges
// is not tiny): then the FP64 normal and edge normals are accurate to far
// better than binary32, which the error bound of the FP32 test assumes.
__global__ void k_facet_cull(const double* __restrict__ tri, int32_t nf,
                             FacetCull* __restrict__ out) {
    int32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const double* t = tri + 9 * (int64_t)f;
    V3 v[3] = {{t[0], t[1], t[2]}, {t[3], t[4], t[5]}, {t[6], t[7], t[8]}};
    V3 ab{v[1].x - v[0].x, v[1].y - v[0].y, v[1].z - v[0].z};
    V3 ac{v[2].x - v[0].x, v[2].y - v[0].y, v[2].z - v[0].z};
    V3 n = cross3(ab, ac);
    double ln = sqrt(dot3(n, n));
    double lab = sqrt(dot3(ab, ab)), lac = sqrt(dot3(ac, ac));
    FacetCull C;
    double a[3] = {v[0].x, v[0].y, v[0].z};
    for (int k = 0; k < 3; ++k) {
        C.ah[k] = __double2float_rn(a[k]);
        C.al[k] = __double2float_rn(a[k] - (double)C.ah[k]);
    }
    C.pad[0] = C.pad[1] = C.pad[2] = C.pad[3] = 0.0f;
    bool ok = ln > 9.5367431640625e-07 * lab * lac && isfinite(ln) && ln > 0.0;
    V3 un{0.0, 0.0, 0.0};
    if (ok) un = V3{n.x / ln, n.y / ln, n.z / ln};
    C.n[0] = (float)un.x;
    C.n[1] = (float)un.y;
    C.n[2] = (float)un.z;
    for (int e = 0; e < 3; ++e) {
        const V3& p0 = v[e];
        const V3& p1 = v[(e + 1) % 3];
        V3 te{p1.x - p0.x, p1.y - p0.y, p1.z - p0.z};
        double le = sqrt(dot3(te, te));
        V3 ne = cross3(te, un);  // outward for a counter-clockwise facet about n
        double l = sqrt(dot3(ne, ne));
        if (!(l > 0.0) || !(le > 0.0)) ok = false;
        if (ok) ne = V3{ne.x / l, ne.y / l, ne.z / l};
        V3 tu = cross3(un, ne);  // unit edge direction (n and ne orthonormal)
        V3 d{p0.x - v[0].x, p0.y - v[0].y, p0.z - v[0].z};
        C.ne[e][0] = (float)ne.x;
        C.ne[e][1] = (float)ne.y;
        C.ne[e][2] = (float)ne.z;
        C.c[e] = ok ? (float)dot3(ne, d) : 0.0f;
        C.o[e] = ok ? (float)dot3(tu, d) : 0.0f;
        C.len[e] = (float)le;
    }
    C.ok = ok ? 1u : 0u;
    out[f] = C;
}

void free_surface(tw_ctx* c, Surface& S) {
    free_env_grid(c, S.grid);
    const size_t ni = (size_t)(S.nf > 1 ? S.nf - 1 : 1);
    if (S.nodes) dev_free(c, S.nodes, sizeof(BvhNode) * ni);
    if (S.nodes32) dev_free(c, S.nodes32, sizeof(BvhNode32) * ni);
    if (S.cull) dev_free(c, S.cull, sizeof(FacetCull) * (size_t)S.nf);
    if (S.tri) dev_free(c, S.tri, sizeof(double) * 9 * (size_t)S.nf);
    if (S.facet_id) dev_free(c, S.facet_id, sizeof(int32_t) * (size_t)S.nf);
    S = Surface{};
}

int build_surface(tw_ctx* c, Surface& S, const double* dV, int32_t nv, const int32_t* dF,
                  int32_t nf, cudaStream_t s) {
    free_surface(c, S);
    if (nf <= 0) return TW_OK;
    const size_t n = (size_t)nf;
    const size_t ni = n > 1 ? n - 1 : 1;
    int st = TW_OK;
    void *nodes = nullptr, *tri = nullptr, *fid = nullptr, *nodes32 = nullptr, *cull = nullptr;
    void *tri_in = nullptr, *cen = nullptr, *codes = nullptr, *codes2 = nullptr, *ids = nullptr,
         *ids2 = nullptr, *leafbox = nullptr, *ibox = nullptr, *ipar = nullptr, *lpar = nullptr,
         *flags = nullptr, *bounds = nullptr, *bad = nullptr, *temp = nullptr;
    size_t temp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (int32_t*)nullptr, (int32_t*)nullptr, (int)n, 0, 30, s);
    struct A {
        void** p;
        size_t b;
    } allocs[] = {
        {&nodes, sizeof(BvhNode) * ni}, {&tri, 72 * n},       {&fid, 4 * n},
        {&nodes32, sizeof(BvhNode32) * ni}, {&cull, sizeof(FacetCull) * n},
        {&tri_in, 72 * n},              {&cen, 24 * n},       {&codes, 4 * n},
        {&codes2, 4 * n},               {&ids, 4 * n},        {&ids2, 4 * n},
        {&leafbox, 48 * n},             {&ibox, 48 * ni},     {&ipar, 4 * ni},
        {&lpar, 4 * n},                 {&flags, 4 * ni},     {&bounds, 8 * 8},
        {&bad, 4},                      {&temp, temp_bytes + 16},
    };
    const int nalloc = (int)(sizeof(allocs) / sizeof(allocs[0]));
    int done = 0;
    for (; done < nalloc; ++done) {
        st = dev_alloc(c, allocs[done].b, allocs[done].p);
        if (st != TW_OK) break;
    }
    if (st == TW_OK) {
        const int B = 256;
        const int G = (int)((n + B - 1) / B);
        cudaMemsetAsync(bad, 0, 4, s);
        cudaMemsetAsync(flags, 0, 4 * ni, s);
        cudaMemsetAsync(nodes, 0, sizeof(BvhNode) * ni, s);
        k_gather_tris<<<G, B, 0, s>>>(dV, nv, dF, nf, (double*)tri_in, (double*)cen, (int*)bad);
        k_bounds<<<1, 1024, 0, s>>>((const double*)cen, (const double*)tri_in, nf, (double*)bounds);
        k_morton<<<G, B, 0, s>>>((const double*)cen, nf, (const double*)bounds, (uint32_t*)codes,
                                 (int32_t*)ids);
        cub::DeviceRadixSort::SortPairs(temp, temp_bytes, (const uint32_t*)codes,
                                        (uint32_t*)codes2, (const int32_t*)ids, (int32_t*)ids2,
                                        (int)n, 0, 30, s);
        k_scatter_tris<<<G, B, 0, s>>>((const double*)tri_in, (const int32_t*)ids2, nf,
                                       (double*)tri, (int32_t*)fid, (double*)leafbox);
        if (n > 1) {
            k_karras<<<G, B, 0, s>>>((const uint32_t*)codes2, nf, (BvhNode*)nodes, (int32_t*)ipar,
                                     (int32_t*)lpar);
            k_refit<<<G, B, 0, s>>>((BvhNode*)nodes, (double*)ibox, (const double*)leafbox,
                                    (const int32_t*)ipar, (const int32_t*)lpar, (int*)flags, nf);
            k_nodes32<<<G, B, 0, s>>>((const BvhNode*)nodes, nf - 1, (BvhNode32*)nodes32);
        }
        k_facet_cull<<<G, B, 0, s>>>((const double*)tri, nf, (FacetCull*)cull);
        int hbad = 0;
        double hb[8] = {0};
        cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hb, bounds, 7 * sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            st = cuda_fail(c, e, "surface build");
        } else if (hbad) {
            st = fail(c, TW_ERR_ARG, "surface facet index out of range");
        } else {
            S.nf = nf;
            S.nodes = (BvhNode*)nodes;
            S.nodes32 = (BvhNode32*)nodes32;
            S.cull = (FacetCull*)cull;
            S.tri = (double*)tri;
            S.facet_id = (int32_t*)fid;
            S.scale = hb[6];
            for (int k = 0; k < 3; ++k) {
                S.lo[k] = hb[k];
                S.hi[k] = hb[3 + k];
            }
            S.bytes = (sizeof(BvhNode) + sizeof(BvhNode32)) * ni + (76 + sizeof(FacetCull)) * n;
            nodes = tri = fid = nodes32 = cull = nullptr;
        }
    }
    // release temporaries (and the outputs on failure)
    for (int k = done - 1; k >= 0; --k)
        if (*allocs[k].p) dev_free(c, *allocs[k].p, allocs[k].b);
    return st;
}

}  // namespace tw
