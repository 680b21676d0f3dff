"""Seeded synthetic inputs with the shapes of the benchmark workloads.

The reference benchmarks on Thingi10k models, which are not available here;
these generators produce inputs with the stated shapes, sizes and value
distributions instead:

* ``energy_batch``: regular tets of edge 0.01, centres uniform in the unit
  cube, uniformly random rotations, every vertex perturbed by N(0, 0.1 edge).
* ``displaced_sphere``: a lat-long sphere (500 longitudes, 100 latitude rings
  plus two poles: 100,000 triangles) with radius 1 + sum of real spherical
  harmonics of degree <= 8, coefficients N(0, 0.02).
* ``envelope_points``: points uniform by area on a surface, offset along the
  facet normal by U(-2 eps, 2 eps).
* ``icosphere``: subdivided icosahedron, vertices jittered radially.
* ``torus``: lat-long torus.
* ``star_batch``: independent one-ring stars (a centre vertex and a fan of
  tets to a jittered convex polyhedron around it), tets per star
  Poisson(24) clamped to [4, 96].
* ``surface_star_batch``: independent stars of surface vertices: a centre
  near a surface, a ring of points in its tangent plane, and an apex above
  and below, so every ring triangle through the centre is a surface face of
  two tets; tets per star Poisson(24) clamped to [6, 96].
"""
from __future__ import annotations

import math

import numpy as np

REGULAR_TET = np.array(
    [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.5, math.sqrt(3.0) / 2.0, 0.0],
     [0.5, math.sqrt(3.0) / 6.0, math.sqrt(2.0 / 3.0)]])


def random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform rotations from normalised Gaussian quaternions, [n, 3, 3]."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def energy_batch(n: int, seed: int = 0, edge: float = 0.01, sigma_rel: float = 0.1,
                 chunk: int = 1 << 20) -> np.ndarray:
    """SoA [12, n] float64 (the energy_ispc layout)."""
    rng = np.random.default_rng(seed)
    T = np.empty((12, n))
    base = REGULAR_TET * edge
    base = base - base.mean(0)
    for i0 in range(0, n, chunk):
        m = min(chunk, n - i0)
        R = random_rotations(rng, m)
        c = rng.random((m, 1, 3))
        pts = np.einsum("nij,kj->nki", R, base) + c + rng.normal(0.0, sigma_rel * edge, (m, 4, 3))
        T[:, i0:i0 + m] = pts.reshape(m, 12).T
    return T


def _real_sh_grid(theta: np.ndarray, phi: np.ndarray, lmax: int, coef: dict) -> np.ndarray:
    """sum_{l<=lmax, |m|<=l} c_lm Y_lm(theta, phi), real orthonormal harmonics, evaluated by
    the standard associated-Legendre recurrences."""
    x = np.cos(theta)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    out = np.zeros(np.broadcast(theta, phi).shape)
    # P[l][m] for m >= 0, Condon-Shortley phase omitted (real basis)
    P = {}
    P[(0, 0)] = np.ones_like(x)
    for m in range(1, lmax + 1):
        P[(m, m)] = P[(m - 1, m - 1)] * (2 * m - 1) * s
    for m in range(0, lmax):
        P[(m + 1, m)] = x * (2 * m + 1) * P[(m, m)]
    for m in range(0, lmax + 1):
        for l in range(m + 2, lmax + 1):
            P[(l, m)] = ((2 * l - 1) * x * P[(l - 1, m)] - (l + m - 1) * P[(l - 2, m)]) / (l - m)
    for l in range(0, lmax + 1):
        for m in range(-l, l + 1):
            am = abs(m)
            K = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
            if m == 0:
                Y = K * P[(l, 0)]
            elif m > 0:
                Y = math.sqrt(2.0) * K * P[(l, am)] * np.cos(am * phi)
            else:
                Y = math.sqrt(2.0) * K * P[(l, am)] * np.sin(am * phi)
            out = out + coef[(l, m)] * Y
    return out


def displaced_sphere(seed: int = 0, n_lon: int = 500, n_rings: int = 100, lmax: int = 8,
                     sigma: float = 0.02):
    """(V [nv,3], F [nf,3]); nf = 2*n_lon*(n_rings-1) + 2*n_lon (100,000 by default)."""
    rng = np.random.default_rng(seed)
    coef = {(l, m): rng.normal(0.0, sigma) for l in range(0, lmax + 1) for m in range(-l, l + 1)}
    j = np.arange(1, n_rings + 1)
    theta = math.pi * j / (n_rings + 1)
    phi = 2 * math.pi * np.arange(n_lon) / n_lon
    TH, PH = np.meshgrid(theta, phi, indexing="ij")
    r = 1.0 + _real_sh_grid(TH, PH, lmax, coef)
    ring = np.stack([r * np.sin(TH) * np.cos(PH), r * np.sin(TH) * np.sin(PH), r * np.cos(TH)], -1)
    rn = 1.0 + _real_sh_grid(np.array([0.0]), np.array([0.0]), lmax, coef)[0]
    rs = 1.0 + _real_sh_grid(np.array([math.pi]), np.array([0.0]), lmax, coef)[0]
    V = np.concatenate([ring.reshape(-1, 3), [[0.0, 0.0, rn]], [[0.0, 0.0, -rs]]])
    north = n_rings * n_lon
    south = north + 1
    F = []
    idx = lambda a, b: a * n_lon + (b % n_lon)
    for a in range(n_rings - 1):
        for b in range(n_lon):
            v00, v01, v10, v11 = idx(a, b), idx(a, b + 1), idx(a + 1, b), idx(a + 1, b + 1)
            F.append((v00, v10, v11))
            F.append((v00, v11, v01))
    for b in range(n_lon):
        F.append((north, idx(0, b), idx(0, b + 1)))
        F.append((south, idx(n_rings - 1, b + 1), idx(n_rings - 1, b)))
    return V, np.asarray(F, np.int32)


def envelope_points(V: np.ndarray, F: np.ndarray, n: int, eps: float, seed: int = 1,
                    chunk: int = 1 << 21) -> np.ndarray:
    """[n, 3] points uniform by area on (V, F), offset along the facet normal by U(-2eps, 2eps)."""
    rng = np.random.default_rng(seed)
    A, B, C = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    nrm = np.cross(B - A, C - A)
    area = np.linalg.norm(nrm, axis=1)
    unit = nrm / np.maximum(area, 1e-300)[:, None]
    cdf = np.cumsum(area)
    cdf /= cdf[-1]
    P = np.empty((n, 3))
    for i0 in range(0, n, chunk):
        m = min(chunk, n - i0)
        f = np.minimum(np.searchsorted(cdf, rng.random(m)), len(F) - 1)
        u, v = rng.random(m), rng.random(m)
        flip = u + v > 1
        u[flip], v[flip] = 1 - u[flip], 1 - v[flip]
        off = rng.uniform(-2 * eps, 2 * eps, m)
        P[i0:i0 + m] = A[f] + u[:, None] * (B[f] - A[f]) + v[:, None] * (C[f] - A[f]) + off[:, None] * unit[f]
    return P


def icosphere(subdiv: int = 3, radius: float = 1.0, jitter: float = 1e-3, seed: int = 0):
    """Subdivided icosahedron (subdiv 3: 642 vertices, 1,280 triangles), jittered radially by
    N(0, jitter)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    V = [np.array(v, float) / np.linalg.norm(v) for v in V]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        F2 = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            F2 += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = F2
    V = np.asarray(V) * radius
    rng = np.random.default_rng(seed)
    V = V * (1.0 + rng.normal(0.0, jitter, (len(V), 1)) / radius)
    return V, np.asarray(F, np.int32)


def torus(R: float = 1.0, r: float = 0.3, n_major: int = 64, n_minor: int = 32):
    u = 2 * math.pi * np.arange(n_major) / n_major
    v = 2 * math.pi * np.arange(n_minor) / n_minor
    U, W = np.meshgrid(u, v, indexing="ij")
    V = np.stack([(R + r * np.cos(W)) * np.cos(U), (R + r * np.cos(W)) * np.sin(U), r * np.sin(W)], -1)
    V = V.reshape(-1, 3)
    F = []
    for i in range(n_major):
        for j in range(n_minor):
            a = i * n_minor + j
            b = ((i + 1) % n_major) * n_minor + j
            c = ((i + 1) % n_major) * n_minor + (j + 1) % n_minor
            d = i * n_minor + (j + 1) % n_minor
            F.append((a, b, c))
            F.append((a, c, d))
    return V, np.asarray(F, np.int32)


def _fib_dirs(k: int) -> np.ndarray:
    i = np.arange(k) + 0.5
    z = 1 - 2 * i / k
    rr = np.sqrt(np.maximum(0, 1 - z * z))
    ph = math.pi * (1 + math.sqrt(5)) * i
    return np.stack([rr * np.cos(ph), rr * np.sin(ph), z], -1)


def star_batch(nstars: int, seed: int = 0, mean_tets: float = 24.0, lo: int = 4, hi: int = 96,
               radius: float = 0.01, jitter_rel: float = 0.1, centres=None):
    """Independent stars sharing no vertices.

    Star i: centre vertex c_i and k = tets/2 + 2 ring points on a jittered sphere of the given
    radius around it; the convex hull of the ring points (scipy qhull) gives 2k - 4 facets, each
    fanned to the centre as one tet oriented POSITIVE; then every vertex (centre included) is
    jittered by N(0, jitter_rel * radius).  Returns (xyz [nv,3], star_off [ns+1], tets [nt,4],
    centers [ns]).  ``centres`` ([ns,3]) places the stars (default: uniform in the unit cube).
    """
    from scipy.spatial import ConvexHull

    rng = np.random.default_rng(seed)
    ntet = np.clip(rng.poisson(mean_tets, nstars), lo, hi)
    ntet += ntet % 2  # 2k - 4 is even
    ntet = np.clip(ntet, lo, hi)
    if centres is None:
        centres = rng.random((nstars, 3))
    centres = np.asarray(centres, np.float64)
    k = ntet // 2 + 2
    nv_star = k + 1
    voff = np.concatenate([[0], np.cumsum(nv_star)])
    toff = np.concatenate([[0], np.cumsum(2 * k - 4)]).astype(np.int32)
    xyz = np.empty((int(voff[-1]), 3))
    tets = np.empty((int(toff[-1]), 4), np.int32)
    for kk in np.unique(k):
        sel = np.nonzero(k == kk)[0]
        m = len(sel)
        d = _fib_dirs(int(kk))
        simp = ConvexHull(d).simplices.astype(np.int32)  # [2kk-4, 3]
        R = random_rotations(rng, m)
        ring = centres[sel, None, :] + radius * np.einsum("kj,mij->mki", d, R)
        c = centres[sel]
        # orient (centre, a, b, c) POSITIVE on the unjittered geometry
        pa, pb, pc = ring[:, simp[:, 0]], ring[:, simp[:, 1]], ring[:, simp[:, 2]]
        det = np.einsum("mfi,mfi->mf", pa - c[:, None], np.cross(pb - c[:, None], pc - c[:, None]))
        pts = np.concatenate([c[:, None], ring], 1)
        pts = pts + rng.normal(0.0, jitter_rel * radius, pts.shape)
        base = voff[sel]
        for j in range(kk + 1):
            xyz[base + j] = pts[:, j]
        a = base[:, None] + 1 + simp[None, :, 0]
        b = base[:, None] + 1 + simp[None, :, 1]
        cc = base[:, None] + 1 + simp[None, :, 2]
        pos = det > 0
        t = np.stack([np.broadcast_to(base[:, None], a.shape), a, np.where(pos, b, cc),
                      np.where(pos, cc, b)], -1)
        idx = toff[sel][:, None] + np.arange(len(simp))[None, :]
        tets[idx.reshape(-1)] = t.reshape(-1, 4)
    return xyz, toff, tets, voff[:-1].astype(np.int32)


def surface_star_batch(V: np.ndarray, F: np.ndarray, nstars: int, eps: float, seed: int = 0,
                       mean_tets: float = 24.0, lo: int = 6, hi: int = 96,
                       radius: float = 0.01, ring_off: float = 0.8, centre_jitter: float = 0.25):
    """Independent surface stars on (V, F), sharing no vertices.

    Star i: a point c on a random facet (uniform by area), the facet's unit normal n and a
    tangent frame; k = tets/2 ring points at angles 2 pi j / k + U(-0.3, 0.3) * 2 pi / k and
    distance radius * U(0.7, 1.3) in the tangent plane, each offset along n by
    U(-ring_off, ring_off) * eps; apexes c +- 0.8 radius n.  Tets (c, r_j, r_j+1, top) and
    (c, r_j+1, r_j, bottom), oriented POSITIVE on the unperturbed geometry; the face opposite the
    apex (vertex 3) is flagged as a surface face.  Finally the centre moves by
    N(0, centre_jitter * radius) in the tangent plane and U(-0.5, 0.5) * eps along n.
    Returns (xyz [nv,3], star_off [ns+1], tets [nt,4], face_flags [nt] uint8, centers [ns]).
    """
    rng = np.random.default_rng(seed)
    ntet = np.clip(rng.poisson(mean_tets, nstars), lo, hi)
    ntet = np.clip(ntet + ntet % 2, lo, hi)
    A, B, C = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    nrm = np.cross(B - A, C - A)
    area = np.linalg.norm(nrm, axis=1)
    cdf = np.cumsum(area)
    cdf /= cdf[-1]
    f = np.minimum(np.searchsorted(cdf, rng.random(nstars)), len(F) - 1)
    u, v = rng.random(nstars), rng.random(nstars)
    flip = u + v > 1
    u[flip], v[flip] = 1 - u[flip], 1 - v[flip]
    c = A[f] + u[:, None] * (B[f] - A[f]) + v[:, None] * (C[f] - A[f])
    n = nrm[f] / area[f, None]
    t1 = np.cross(n, np.where(np.abs(n[:, :1]) < 0.9, [[1.0, 0.0, 0.0]], [[0.0, 1.0, 0.0]]))
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(n, t1)
    k = ntet // 2
    nv_star = k + 3
    voff = np.concatenate([[0], np.cumsum(nv_star)])
    toff = np.concatenate([[0], np.cumsum(2 * k)]).astype(np.int32)
    xyz = np.empty((int(voff[-1]), 3))
    tets = np.empty((int(toff[-1]), 4), np.int32)
    for kk in np.unique(k):
        sel = np.nonzero(k == kk)[0]
        m = len(sel)
        ang = 2 * math.pi * (np.arange(kk)[None, :] + rng.uniform(-0.3, 0.3, (m, kk))) / kk
        rad = radius * rng.uniform(0.7, 1.3, (m, kk))
        off = rng.uniform(-ring_off, ring_off, (m, kk)) * eps
        cs, t1s, t2s, ns = c[sel, None], t1[sel, None], t2[sel, None], n[sel, None]
        ring = cs + rad[..., None] * (np.cos(ang)[..., None] * t1s + np.sin(ang)[..., None] * t2s)
        ring = ring + off[..., None] * ns
        top = c[sel] + 0.8 * radius * n[sel]
        bot = c[sel] - 0.8 * radius * n[sel]
        cj = (rng.normal(0.0, centre_jitter * radius, (m, 2))[:, :1] * t1[sel]
              + rng.normal(0.0, centre_jitter * radius, (m, 1)) * t2[sel]
              + rng.uniform(-0.5, 0.5, (m, 1)) * eps * n[sel])
        base = voff[sel]
        xyz[base] = c[sel] + cj
        for j in range(kk):
            xyz[base + 1 + j] = ring[:, j]
        xyz[base + 1 + kk] = top
        xyz[base + 2 + kk] = bot
        ci = base
        rj = base[:, None] + 1 + np.arange(kk)[None, :]
        rj1 = base[:, None] + 1 + (np.arange(kk)[None, :] + 1) % kk
        tp = base + 1 + kk
        bt = base + 2 + kk
        tb = toff[sel]
        for j in range(kk):
            tets[tb + 2 * j] = np.stack([ci, rj[:, j], rj1[:, j], tp], 1)
            tets[tb + 2 * j + 1] = np.stack([ci, rj1[:, j], rj[:, j], bt], 1)
    ff = np.full(len(tets), 8, np.uint8)  # bit 3: the face opposite the apex
    cen = voff[:-1].astype(np.int32)
    return xyz, toff, tets, ff, cen


def mixed_star_batch(V: np.ndarray, F: np.ndarray, nstars: int, eps: float, seed: int = 0,
                     surface_fraction: float = 0.5, mean_tets: float = 24.0):
    """Interior stars (``star_batch``, centres on the surface's bounding box) followed by
    surface stars (``surface_star_batch``) in one vertex array.  Returns (xyz, star_off, tets,
    face_flags, centers, kinds) with kinds 0 (interior) / 1 (surface)."""
    ns_s = int(round(nstars * surface_fraction))
    ns_i = nstars - ns_s
    lo, hi = V.min(0), V.max(0)
    rng = np.random.default_rng(seed + 7)
    parts = []
    if ns_i:
        cen_i = lo + (hi - lo) * rng.random((ns_i, 3))
        xi, oi, ti, ci = star_batch(ns_i, seed=seed, mean_tets=mean_tets, centres=cen_i)
        parts.append((xi, oi, ti, np.zeros(len(ti), np.uint8), ci, np.zeros(ns_i, np.uint8)))
    if ns_s:
        xs, os_, ts, fs, cs = surface_star_batch(V, F, ns_s, eps, seed=seed + 1, mean_tets=mean_tets)
        parts.append((xs, os_, ts, fs, cs, np.ones(ns_s, np.uint8)))
    xyz, off, tets, ff, cen, kinds = [], [0], [], [], [], []
    nv = 0
    nt = 0
    for x, o, t, f_, c_, k_ in parts:
        xyz.append(x)
        tets.append(t + nv)
        ff.append(f_)
        cen.append(c_ + nv)
        kinds.append(k_)
        off.extend((o[1:] + nt).tolist())
        nv += len(x)
        nt += len(t)
    return (np.vstack(xyz), np.asarray(off, np.int32), np.vstack(tets).astype(np.int32),
            np.concatenate(ff), np.concatenate(cen).astype(np.int32), np.concatenate(kinds))


def icosphere_stage1_mesh(subdiv: int = 3, jitter: float = 1e-3, seed: int = 0,
                          edge_rel: float = 0.05, margin_rel: float = 0.05):
    """A stand-in for TetWild's mesh at the start of refinement on the jittered icosphere.

    The tet mesh is the Delaunay tetrahedralisation (scipy qhull) of the icosphere's vertices,
    a lattice at spacing L = edge_rel * bbox diagonal (the CLI's default -l 0.05) over the
    bounding box grown by margin_rel * diagonal, jittered by N(0, 0.02 L), minus lattice points
    closer than L/2 to the sphere, plus the grown box's corners.  Tets are oriented POSITIVE.  A face is a surface face
    when its vertex triple is an icosphere triangle.  Returns a dict with V, F (the input
    surface), xyz, tets, face_flags (bit j: the face opposite vertex j is a surface face),
    kind (0 interior, 1 surface, 3 locked box corner) and coverage (icosphere triangles found
    among the Delaunay faces).
    """
    from scipy.spatial import Delaunay

    V, F = icosphere(subdiv, jitter=jitter, seed=seed)
    lo, hi = V.min(0), V.max(0)
    diag = float(np.linalg.norm(hi - lo))
    L = edge_rel * diag
    glo, ghi = lo - margin_rel * diag, hi + margin_rel * diag
    axes = [np.arange(glo[k] + L / 2, ghi[k], L) for k in range(3)]
    G = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    # a regular lattice has co-spherical groups whose Delaunay tets are flat
    G = G + np.random.default_rng(seed + 1).normal(0.0, 0.02 * L, G.shape)
    r = np.linalg.norm(G, axis=1)
    G = G[np.abs(r - 1.0) > L / 2]
    corners = np.array([[glo[0] if i & 1 else ghi[0], glo[1] if i & 2 else ghi[1],
                         glo[2] if i & 4 else ghi[2]] for i in range(8)])
    xyz = np.vstack([V, G, corners])
    kind = np.concatenate([np.ones(len(V), np.uint8), np.zeros(len(G), np.uint8),
                           np.full(8, 3, np.uint8)])
    tets = Delaunay(xyz).simplices.astype(np.int32)
    p = xyz[tets]
    det = np.einsum("ij,ij->i", p[:, 1] - p[:, 0], np.cross(p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]))
    neg = det < 0
    tets[neg] = tets[neg][:, [0, 2, 1, 3]]
    surf = {tuple(sorted(map(int, f))) for f in F}
    ff = np.zeros(len(tets), np.uint8)
    found = set()
    for j in range(4):
        tri = np.sort(np.delete(tets, j, axis=1), axis=1)
        for i in np.nonzero(np.all(tri < len(V), axis=1))[0]:
            key = tuple(int(x) for x in tri[i])
            if key in surf:
                ff[i] |= np.uint8(1 << j)
                found.add(key)
    return {"V": V, "F": F, "xyz": xyz, "tets": tets, "face_flags": ff, "kind": kind,
            "coverage": len(found) / len(F), "diag": diag, "edge": L}


def vertex_stars(tets: np.ndarray, nv: int):
    """conn_tets of every vertex in ascending tet order (CSR: off [nv+1], ids)."""
    t = tets.reshape(-1)
    owner = np.repeat(np.arange(len(tets), dtype=np.int64), 4)
    order = np.lexsort((owner, t))
    ids = owner[order].astype(np.int32)
    off = np.zeros(nv + 1, np.int64)
    np.add.at(off, t + 1, 1)
    return np.cumsum(off).astype(np.int64), ids


def greedy_colouring(tets: np.ndarray, nv: int) -> np.ndarray:
    """Vertex colours such that no two vertices of a tet share one: each colour class is a set
    of independent stars (no centre lies in another centre's star)."""
    off, ids = vertex_stars(tets, nv)
    colour = np.full(nv, -1, np.int64)
    for v in range(nv):
        nb = np.unique(tets[ids[off[v]:off[v + 1]]].reshape(-1))
        used = set(colour[nb][colour[nb] >= 0].tolist())
        c = 0
        while c in used:
            c += 1
        colour[v] = c
    return colour
