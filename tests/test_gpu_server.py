"""Serving engine: admission by device footprint, continuous batching, and the
same result for a request alone and in a mix of concurrent requests.

Tolerances: FP64 results are compared bit for bit (the batched kernels do the
same FP64 arithmetic whatever else runs); the mixed form within 1e-10 of the
largest state entry (FP32 parts of two kernel builds may round differently).
"""
import threading
import time

import numpy as np
import pytest

import zisafvm_gb300 as z
from problems import polytrope_2d, vortex_2d, vortex_tube_3d

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-10


def _requests():
    """(mesh, scheme, u0, n_steps, t_end) of a mixed 2D / 3D, FP64 / mixed set."""
    out = []
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=24, amplitude=1e-3, seed=5, precision=z.MIXED)
    out.append((mesh, scheme, u0, 0, 0.02))
    raw, mesh, scheme, u0 = vortex_2d(n=20, halo=3)
    out.append((mesh, scheme, u0, 12, 0.0))
    raw, mesh, scheme, u0 = vortex_tube_3d(n=8)
    scheme.precision = z.MIXED
    out.append((mesh, scheme, u0, 9, 0.0))
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=16, amplitude=1e-2, seed=9)
    out.append((mesh, scheme, u0, 0, 0.015))
    raw, mesh, scheme, u0 = vortex_tube_3d(n=7, order=2)
    out.append((mesh, scheme, u0, 7, 0.0))
    return out


def _same(a, b, scheme):
    if scheme.precision == z.FP64:
        return np.array_equal(a, b)
    return np.abs(a - b).max() <= TOL_MIXED * np.abs(b).max()


def test_footprint_matches_allocation(zlib):
    for mesh, scheme, u0, _, _ in _requests():
        s = z.Solver(mesh, scheme)
        assert z.solver_footprint(mesh, scheme) == s.device_bytes()
        s.close()


def test_request_alone_and_in_mix(zlib):
    reqs = _requests()
    alone = []
    for mesh, scheme, u0, n, t_end in reqs:
        srv = z.Server(max_slots=4, steps_per_round=4)
        rid = srv.submit(mesh, scheme, u0, n_steps=n, t_end=t_end)
        alone.append(srv.wait(rid, timeout_s=120))
        srv.close()
    # all at once, from several threads, with staggered arrivals
    srv = z.Server(max_slots=8, steps_per_round=3)
    ids = [None] * len(reqs)

    def client(k):
        time.sleep(0.01 * k)
        mesh, scheme, u0, n, t_end = reqs[k]
        ids[k] = srv.submit(mesh, scheme, u0, n_steps=n, t_end=t_end)

    th = [threading.Thread(target=client, args=(k,)) for k in range(len(reqs))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    mixed_res = [srv.wait(rid, timeout_s=120) for rid in ids]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["bytes_in_use"] == 0
    for (mesh, scheme, u0, n, t_end), a, m in zip(reqs, alone, mixed_res):
        assert a[2] == m[2]
        if n:
            assert m[2] == n
        else:
            assert abs(m[1] - t_end) <= 1e-12 * t_end
        assert _same(m[0], a[0], scheme)
        # and the same as the solver run by itself (not batched)
        s = z.Solver(mesh, scheme)
        s.set_state(u0)
        s.advance(n_steps=n, t_end=t_end)
        u, t = s.get_state()
        assert abs(t - m[1]) <= 1e-12 * max(t, 1e-300)
        if scheme.precision == z.FP64:
            assert np.array_equal(u, m[0])
        else:
            assert np.abs(u - m[0]).max() <= TOL_MIXED * np.abs(u).max()


def test_admission_respects_budget(zlib):
    reqs = _requests()
    foot = [z.solver_footprint(m, s) for m, s, *_ in reqs]
    budget = max(foot) + min(foot) // 2
    srv = z.Server(hbm_budget_bytes=budget, max_slots=8, steps_per_round=4)
    ids = [srv.submit(m, s, u0, n_steps=n, t_end=te) for m, s, u0, n, te in reqs]
    res = [srv.wait(rid, timeout_s=300) for rid in ids]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["bytes_peak"] <= budget
    assert max(r[3]["queued"] for r in res) > 0.0
    with pytest.raises(z.ZfvmError) as e:
        srv2 = z.Server(hbm_budget_bytes=min(foot) - 1, max_slots=2)
        try:
            srv2.submit(reqs[0][0], reqs[0][1], reqs[0][2], n_steps=1)
        finally:
            srv2.close()
    assert e.value.code == 2


def test_failed_request_does_not_disturb_others(zlib):
    reqs = _requests()[:2]
    mesh, scheme, u0, n, t_end = reqs[1]
    bad = u0.copy()
    inner = np.flatnonzero(mesh.geometry()["flags"] & 1)
    bad[inner[len(inner) // 2], 0] = -1.0
    srv = z.Server(max_slots=4, steps_per_round=2)
    good_id = srv.submit(*reqs[0][:3], n_steps=reqs[0][3], t_end=reqs[0][4])
    bad_id = srv.submit(mesh, scheme, bad, n_steps=5)
    with pytest.raises(z.ZfvmError) as e:
        srv.wait(bad_id, timeout_s=60)
    assert e.value.code == 3
    u, t, steps, _ = srv.wait(good_id, timeout_s=60)
    assert np.isfinite(u).all() and abs(t - reqs[0][4]) <= 1e-12 * reqs[0][4]
    st = srv.stats()
    srv.close()
    assert st["failed"] == 1 and st["completed"] == 1


def test_close_with_requests_in_every_phase(zlib):
    """Closing a server whose requests are queued, being set up and running
    returns and frees their solvers; a new server then runs normally."""
    reqs = _requests()
    srv = z.Server(max_slots=2, steps_per_round=1)
    for mesh, scheme, u0, _, _ in reqs * 2:
        srv.submit(mesh, scheme, u0, n_steps=10000)
    time.sleep(0.5)
    t0 = time.perf_counter()
    srv.close()
    assert time.perf_counter() - t0 < 60
    mesh, scheme, u0, n, t_end = reqs[1]
    srv = z.Server(max_slots=2, steps_per_round=4)
    u, t, steps, _ = srv.wait(srv.submit(mesh, scheme, u0, n_steps=n, t_end=t_end), timeout_s=120)
    srv.close()
    assert steps == n and np.isfinite(u).all()


def test_step_rejection_request(zlib):
    """A request with RejectLargeDensityChange runs in the server's batch and
    returns exactly what the solver's own time loop gives (FP64)."""
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=16, amplitude=1e-1)
    scheme.step_rejection_drho = 2.4e-3
    scheme.step_rejection_max_exponent = 6
    a = z.Solver(mesh, scheme)
    a.set_state(u0)
    t_a, n_a = a.advance(n_steps=12)
    u_a, _ = a.get_state()
    assert n_a == 12 and a.step_rejections() > 0
    srv = z.Server(max_slots=4, steps_per_round=3)
    mesh2, scheme2, u2, n2, t2 = _requests()[1]
    other = srv.submit(mesh2, scheme2, u2, n_steps=n2, t_end=t2)
    rid = srv.submit(mesh, scheme, u0, n_steps=12)
    u, t, steps, _ = srv.wait(rid, timeout_s=120)
    srv.wait(other, timeout_s=120)
    srv.close()
    assert steps == 12 and t == t_a
    assert np.array_equal(u, u_a)
