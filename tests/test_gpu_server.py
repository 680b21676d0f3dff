"""GPU tests of the serving loop (tw_server_*): results identical alone and in
any mix of jobs and request kinds, equal to the single-job entry points, job
admission against the HBM budget, and errors reported per request."""
import threading

import numpy as np
import pytest

import tetwild_gb300 as tw
from tetwild_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _jobs():
    """(V, F, eps) of four seeded surfaces of different shapes and sizes."""
    out = []
    V, F = syn.icosphere(4, seed=1)
    out.append((V, F, 2e-3))
    V, F = syn.torus(1.0, 0.3, 64, 32)
    out.append((V, F, 2e-3))
    V, F = syn.displaced_sphere(seed=2, n_lon=100, n_rings=50)
    out.append((V, F, 1e-3))
    V, F = syn.displaced_sphere(seed=3, n_lon=60, n_rings=30)
    out.append((V, F, 1.5e-3))
    return out


def _faces_near(V, F, n, eps, seed):
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, len(F), n)
    A, B, C = V[F[idx, 0]], V[F[idx, 1]], V[F[idx, 2]]
    cen = (A + B + C) / 3
    nrm = np.cross(B - A, C - A)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    shrink = rng.uniform(0.2, 0.9, (n, 1))
    push = rng.uniform(-1.5, 1.5, (n, 1)) * eps
    return np.hstack([cen + shrink * (A - cen) + push * nrm, cen + shrink * (B - cen) + push * nrm,
                      cen + shrink * (C - cen) + push * nrm])


@pytest.fixture(scope="module")
def workload():
    jobs = _jobs()
    reqs = []   # (job index, kind, args)
    stars = []
    for j, (V, F, eps) in enumerate(jobs):
        rng = np.random.default_rng(10 + j)
        for k in range(2):
            P = syn.envelope_points(V, F, int(rng.integers(2000, 20000)), eps, seed=100 + 7 * j + k)
            reqs.append((j, "points", (P,)))
        reqs.append((j, "faces", (_faces_near(V, F, 300, eps, seed=200 + j),)))
        reqs.append((j, "amips", (syn.energy_batch(5000, seed=300 + j),)))
        xyz, off, tets, ff, cen = syn.surface_star_batch(V, F, 400, eps, seed=400 + j)
        stars.append(xyz)
        reqs.append((j, "smooth", (off, tets, cen, ff, np.ones(len(cen), np.uint8))))
    return jobs, stars, reqs


def _open(srv, jobs, stars):
    ids = []
    for (V, F, eps), xyz in zip(jobs, stars):
        j = srv.job_open(V, F, eps * eps, eps / 2)
        assert j is not None
        srv.job_mesh(j, xyz)
        ids.append(j)
    return ids


def _submit(srv, ids, req):
    j, kind, a = req
    if kind == "points":
        return srv.submit_points(ids[j], *a)
    if kind == "faces":
        return srv.submit_faces(ids[j], *a)
    if kind == "amips":
        return srv.submit_amips(ids[j], *a)
    off, tets, cen, ff, kinds = a
    return srv.submit_smooth(ids[j], off, tets, cen, ff, kinds)


def _flat(res):
    if isinstance(res, tuple):
        return [np.array(x, copy=True) for x in res]
    return [np.array(res, copy=True)]


@pytest.mark.parametrize("precision", [tw.TW_PRECISION_FP32_CERTIFIED, tw.TW_PRECISION_FP64])
def test_same_alone_and_in_the_mix(workload, precision):
    jobs, stars, reqs = workload
    with tw.Server(0, 0, lanes=4) as srv:
        srv.set_params(precision, 1, 8)
        ids = _open(srv, jobs, stars)
        alone = []
        for r in reqs:
            t, res = _submit(srv, ids, r)
            srv.wait(t)
            alone.append(_flat(res))
        assert srv.stats()["max_requests_per_batch"] == 1
        # the mix: four host threads submit everything in shuffled orders
        order = np.random.default_rng(5).permutation(len(reqs))
        mixed = [None] * len(reqs)
        lat = [None] * len(reqs)
        errors = []

        def worker(part):
            try:
                mine = [(i, _submit(srv, ids, reqs[i])) for i in part]
                for i, (t, res) in mine:
                    lat[i] = srv.wait(t)
                    mixed[i] = _flat(res)
            except Exception as e:   # reported below
                errors.append(e)

        th = [threading.Thread(target=worker, args=(order[k::4],)) for k in range(4)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        assert not errors, errors
        for i in range(len(reqs)):
            for a, b in zip(alone[i], mixed[i]):
                assert np.array_equal(a, b), (i, reqs[i][1])
        st = srv.stats()
        assert st["max_requests_per_batch"] > 1      # requests were joined across jobs
        assert st["jobs_open"] == len(jobs)
        assert all(x >= 0 for x in lat)


def test_server_matches_single_job_entry_points(workload, oracle):
    jobs, stars, reqs = workload
    with tw.Server(0, 0, lanes=2) as srv, tw.Context(0) as ctx:
        srv.set_params(tw.TW_PRECISION_FP32_CERTIFIED, 1, 8)
        ids = _open(srv, jobs, stars)
        for r in reqs:
            j, kind, a = r
            V, F, eps = jobs[j]
            t, res = _submit(srv, ids, r)
            srv.wait(t)
            ctx.set_params(eps * eps, eps / 2, 1, 8)
            ctx.surface_upload(V, F)
            if kind == "points":
                assert np.array_equal(res, ctx.envelope_points(a[0]))
            elif kind == "faces":
                assert np.array_equal(res, ctx.envelope_faces(a[0]))
            elif kind == "amips":
                ctx.set_precision(tw.TW_PRECISION_FP32_CERTIFIED)
                want = ctx.amips(a[0])
                ctx.set_precision(tw.TW_PRECISION_FP64)
                assert np.array_equal(res[0], want["E"]) and np.array_equal(res[3], want["flip"])
            else:
                off, tets, cen, ff, kinds = a
                want, wst = oracle.smooth_stars(stars[j], off, tets, cen, ff, kinds,
                                                surface=oracle.surface(V, F),
                                                boundary=oracle.surface(V, F), eps2=eps * eps,
                                                sd=eps / 2, max_step=1, max_it=8, nthreads=8)
                assert np.array_equal(res[1].astype(np.int8), wst)
                assert np.array_equal(res[0], want)


def test_admission_against_the_budget():
    V, F = syn.displaced_sphere(seed=4, n_lon=250, n_rings=100)   # ~50k facets
    budget = 160 << 20   # one job (~137 MB estimated, ~115 MB resident) fits, two do not
    with tw.Server(0, budget, lanes=1) as srv:
        a = srv.job_open(V, F, 1e-6, 5e-4)
        assert a is not None
        b = srv.job_open(V, F, 1e-6, 5e-4)
        assert b is None                                  # TW_BUSY: does not fit now
        assert srv.stats()["bytes_used"] <= budget
        srv.job_close(a)
        b = srv.job_open(V, F, 1e-6, 5e-4)
        assert b is not None
        P = syn.envelope_points(V, F, 1000, 1e-3, seed=1)
        t, out = srv.submit_points(b, P)
        srv.wait(t)
        srv.job_close(b)
        with pytest.raises(tw.TetWildGpuError):
            srv.submit_points(b, P)                        # closed job


def test_errors_are_per_request(workload):
    jobs, stars, reqs = workload
    V, F, eps = jobs[0]
    with tw.Server(0, 0, lanes=2) as srv:
        j = srv.job_open(V, F, eps * eps, eps / 2)
        off, tets, cen, ff, kinds = reqs[4][2]
        with pytest.raises(tw.TetWildGpuError) as e:
            srv.submit_smooth(j, off, tets, cen, ff, kinds)   # no resident mesh yet
        assert e.value.code == tw.TW_ERR_NO_MESH
        srv.job_mesh(j, stars[0])
        bad = tets.copy()
        bad[0, 0] = len(stars[0]) + 5
        t_bad, _ = srv.submit_smooth(j, off, bad, cen, ff, kinds)
        t_ok, out = srv.submit_points(j, syn.envelope_points(V, F, 500, eps, seed=3))
        with pytest.raises(tw.TetWildGpuError) as e:
            srv.wait(t_bad)
        assert e.value.code == tw.TW_ERR_ARG
        srv.wait(t_ok)


def test_smooth_apply_updates_the_resident_mesh(workload):
    jobs, stars, reqs = workload
    V, F, eps = jobs[2]
    off, tets, cen, ff, kinds = reqs[2 * 5 + 4][2]
    xyz = stars[2]
    with tw.Server(0, 0, lanes=2) as srv:
        srv.set_params(tw.TW_PRECISION_FP32_CERTIFIED, 1, 8)
        j = srv.job_open(V, F, eps * eps, eps / 2)
        srv.job_mesh(j, xyz)
        t, (out, st) = srv.submit_smooth(j, off, tets, cen, ff, kinds, apply=True)
        srv.wait(t)
        now = srv.job_read_mesh(j, len(xyz))
        moved = st == tw.TW_SMOOTH_MOVED
        assert moved.any()
        want = xyz.copy()
        want[cen[moved]] = out[moved]
        assert np.array_equal(now, want)


@pytest.mark.timeout(300, method="thread")
def test_job_errors_on_closed_and_unknown_jobs():
    """Every job call on a closed or unknown job returns an error (and the server stays
    usable); none may block.  The thread timeout ends the process if one does."""
    V, F = syn.icosphere(2)
    with tw.Server(0, 0, lanes=1) as srv:
        j = srv.job_open(V, F, 1e-6, 5e-4)
        srv.job_close(j)
        for call in (lambda: srv.job_close(j), lambda: srv.job_cancel(j),
                     lambda: srv.job_close(12345), lambda: srv.job_mesh(j, V),
                     lambda: srv.job_read_mesh(j, len(V)), lambda: srv.job_boundary(j, V, F)):
            with pytest.raises(tw.TetWildGpuError) as e:
                call()
            assert e.value.code == tw.TW_ERR_ARG
        k = srv.job_open(V, F, 1e-6, 5e-4)
        t, out = srv.submit_points(k, syn.envelope_points(V, F, 100, 1e-3, seed=2))
        srv.wait(t)
        srv.job_close(k)


def test_job_cancel_mid_flight(workload):
    """tw_server_job_cancel: with one lane and a burst of requests queued for job A, the
    cancel completes A's waiting requests with TW_ERR_CANCELLED at once, lets the batches
    already on the lane finish (their results correct), frees A's memory and refuses A
    afterwards; job B's requests, queued among A's, all run and are correct."""
    jobs, stars, reqs = workload
    (Va, Fa, ea), (Vb, Fb, eb) = jobs[2], jobs[0]
    Pa = syn.envelope_points(Va, Fa, 200_000, ea, seed=71)
    Pb = syn.envelope_points(Vb, Fb, 50_000, eb, seed=72)
    with tw.Server(0, 0, lanes=1) as srv, tw.Context(0) as ctx:
        srv.set_params(tw.TW_PRECISION_FP32_CERTIFIED, 1, 8)
        a = srv.job_open(Va, Fa, ea * ea, ea / 2)
        b = srv.job_open(Vb, Fb, eb * eb, eb / 2)
        # a burst first, so that the lane's scratch has grown to its largest batch
        warm = [srv.submit_points(a, Pa) for _ in range(45)]
        for t, _ in warm:
            srv.wait(t)
        before = srv.stats()
        ta, tb = [], []
        for k in range(300):
            ta.append(srv.submit_points(a, Pa))
            if k % 30 == 0:
                tb.append(srv.submit_points(b, Pb))
        srv.job_cancel(a)
        after = srv.stats()
        assert after["jobs_open"] == before["jobs_open"] - 1
        assert after["bytes_used"] < before["bytes_used"]
        ctx.set_params(ea * ea, ea / 2)
        ctx.surface_upload(Va, Fa)
        want_a = ctx.envelope_points(Pa)
        ctx.set_params(eb * eb, eb / 2)
        ctx.surface_upload(Vb, Fb)
        want_b = ctx.envelope_points(Pb)
        statuses = []
        for t, out in ta:
            st, _ = srv.wait_status(t)
            statuses.append(st)
            assert st in (tw.TW_OK, tw.TW_ERR_CANCELLED)
            if st == tw.TW_OK:
                assert np.array_equal(out, want_a)
        n_cancelled = statuses.count(tw.TW_ERR_CANCELLED)
        assert 1 <= n_cancelled < len(ta) or statuses.count(tw.TW_OK) == 0, statuses
        assert n_cancelled >= 1
        for t, out in tb:
            srv.wait(t)
            assert np.array_equal(out, want_b)
        with pytest.raises(tw.TetWildGpuError):
            srv.submit_points(a, Pa)                       # the job is gone
        srv.job_cancel(b)                                  # nothing queued: frees at once
        assert srv.stats()["jobs_open"] == before["jobs_open"] - 2
