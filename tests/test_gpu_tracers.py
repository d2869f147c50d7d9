"""Advected variables (mass-weighted tracers) on the GPU against the oracle,
through the C ABI.

Bars: FP64 tendencies within 1e-13 of each variable's largest tendency, FP64
runs within 1e-12 relative L1 and Linf per variable (the conserved-variable
bars).  On the well-balanced polytrope near rest the contact speed s* that
upwinds the tracers is a small difference of O(1) terms and the tendency a
small divergence, so its tendency and change over the run are bounded against
their own size at ten times the errors measured on GB300 (tendency 1.4e-12,
change 6.4e-13), as the conserved variables are there
(test_gpu_parity.py::test_polytrope_*).  The mixed form's tracers within 1e-6 relative L1 of the FP64 oracle
(the mixed form's bar), since their wave speeds come from the mixed form's
face states.  Tracers are passive: the conserved variables must not change
when tracers are added (bit for bit in FP64).
"""
import os

import numpy as np
import pytest

import zisafvm_gb300 as z
from metrics import rel_errors
from problems import polytrope_2d, polytrope_2d_frozen, tracers, vortex_2d, vortex_tube_3d

pytestmark = pytest.mark.gpu

TOL_RHS = 1e-13
TOL_RUN = 1e-12
TOL_MIXED = 1e-6
TOL_WB = 1.4e-11      # tendency; measured 1.4e-12
TOL_WB_RUN = 6.4e-12  # change over the run; measured 6.4e-13
NA = 2
WB_CASES = ("polytrope", "frozen")


def _oracle(olib, raw, mesh, scheme):
    return olib.Oracle(raw, mesh.stencils(), scheme.oracle_vector(), quad=mesh.quad, threads=os.cpu_count())


def _case(name):
    if name == "vortex_hllc":
        raw, mesh, scheme, u0 = vortex_2d(n=24, halo=3, flux=0)
    elif name == "vortex_rusanov":
        raw, mesh, scheme, u0 = vortex_2d(n=24, halo=3, flux=1)
    elif name == "polytrope":
        raw, mesh, scheme, u0 = polytrope_2d(n_rings=20, amplitude=1e-2, seed=5)
    elif name == "frozen":
        raw, mesh, scheme, u0 = polytrope_2d_frozen(n_rings=24, amplitude=1e-2)
    elif name == "tube_o3":
        raw, mesh, scheme, u0 = vortex_tube_3d(n=8)
    else:
        raw, mesh, scheme, u0 = vortex_tube_3d(n=8, order=2)
    scheme.n_avars = NA
    return raw, mesh, scheme, u0, tracers(mesh, u0, NA)


def _inner(raw, n):
    return np.ones(n, bool) if raw.ghost is None else raw.ghost == 0


def _tracer_errors(q, ref, mask):
    l1 = max(np.abs(q[mask, k] - ref[mask, k]).sum() / np.abs(ref[mask, k]).sum() for k in range(q.shape[1]))
    linf = max(np.abs(q[mask, k] - ref[mask, k]).max() / np.abs(ref[mask, k]).max() for k in range(q.shape[1]))
    return l1, linf


CASES = ["vortex_hllc", "vortex_rusanov", "polytrope", "frozen", "tube_o3", "tube_o2"]


@pytest.mark.parametrize("case", CASES)
def test_tracer_rate_of_change(zlib, olib, case):
    raw, mesh, scheme, u0, q0 = _case(case)
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    s.set_avars(q0)
    tu, tq = s.rate_of_change_all()
    s.close()
    ru, rq = _oracle(olib, raw, mesh, scheme).rate_of_change(u0, q0)
    inner = _inner(raw, u0.shape[0])
    tol = TOL_WB if case in WB_CASES else TOL_RHS
    for k in range(NA):
        scale = np.abs(rq[inner, k]).max()
        err = np.abs(tq[inner, k] - rq[inner, k]).max() / scale
        print(f"tracer tendency {case} {k}: {err:.2e}")
        assert err < tol, (k, err)
    assert np.all(tq[~inner] == 0.0)
    cols = (0, 1, 2, 4) if raw.n_dims == 2 else (0, 1, 2, 3, 4)
    for v in cols:
        scale = np.abs(ru[inner, v]).max()
        assert np.abs(tu[inner, v] - ru[inner, v]).max() <= tol * scale


@pytest.mark.parametrize("case", CASES)
def test_tracer_steps(zlib, olib, case):
    raw, mesh, scheme, u0, q0 = _case(case)
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    s.set_avars(q0)
    t_gpu, n_gpu = s.advance(n_steps=8)
    u_gpu, _ = s.get_state()
    q_gpu = s.get_avars()
    s.close()
    u_ref, q_ref, t_ref, n_ref = _oracle(olib, raw, mesh, scheme).run(u0, n_steps=8, avars=q0)
    assert n_gpu == n_ref == 8
    assert abs(t_gpu - t_ref) <= 1e-13 * t_ref
    inner = _inner(raw, u0.shape[0])
    if case in WB_CASES:
        for a, ref, a0 in ((u_gpu, u_ref, u0), (q_gpu, q_ref, q0)):
            d, dref = (a - a0)[inner], (ref - a0)[inner]
            err = np.abs(d - dref).max() / np.abs(dref).max()
            print(f"tracer run {case}: change error {err:.2e}")
            assert err < TOL_WB_RUN, err
        return
    cols = (0, 1, 2, 4) if raw.n_dims == 2 else (0, 1, 2, 3, 4)
    l1, linf = rel_errors(u_gpu, u_ref, inner, cols)
    assert l1 < TOL_RUN and linf < TOL_RUN, (l1, linf)
    l1, linf = _tracer_errors(q_gpu, q_ref, inner)
    assert l1 < TOL_RUN and linf < TOL_RUN, (l1, linf)


def test_tracers_are_passive_and_conserved(zlib):
    raw, mesh, scheme, u0, q0 = _case("vortex_hllc")
    plain = z.Scheme(**{**scheme.__dict__, "n_avars": 0})
    a = z.Solver(mesh, plain)
    a.set_state(u0)
    a.advance(n_steps=6)
    ua, _ = a.get_state()
    b = z.Solver(mesh, scheme)
    b.set_state(u0)
    b.set_avars(q0)
    b.advance(n_steps=6)
    ub, _ = b.get_state()
    qb = b.get_avars()
    assert np.array_equal(ua, ub)
    vol = mesh.geometry()["volumes"]
    inner = _inner(raw, u0.shape[0])
    for k in range(NA):
        m0, m1 = (vol[inner] * q0[inner, k]).sum(), (vol[inner] * qb[inner, k]).sum()
        assert abs(m1 - m0) <= 1e-13 * (vol[inner] * np.abs(q0[inner, k])).sum()
    # each launch of a step is counted: clock + 2 x 3 kernels per stage
    assert b.launches_per_step() == 1 + 2 * 3 * scheme.rk_stages


@pytest.mark.parametrize("case", ["vortex_hllc", "polytrope", "tube_o3"])
def test_mixed_tracers(zlib, olib, case):
    raw, mesh, scheme, u0, q0 = _case(case)
    mixed = z.Scheme(**{**scheme.__dict__, "precision": z.MIXED})
    s = z.Solver(mesh, mixed)
    s.set_state(u0)
    s.set_avars(q0)
    s.advance(n_steps=8)
    q_gpu = s.get_avars()
    s.close()
    _, q_ref, _, _ = _oracle(olib, raw, mesh, scheme).run(u0, n_steps=8, avars=q0)
    l1, _ = _tracer_errors(q_gpu, q_ref, _inner(raw, u0.shape[0]))
    print(f"mixed tracers {case}: rel L1 {l1:.3e}")
    assert l1 < TOL_MIXED


def test_tracers_with_step_rejection(zlib, olib):
    """A rejected step puts the tracers back too (the setup of
    test_gpu_parity.py::test_step_rejection, plus one tracer; the same
    tolerance on the change over the run)."""
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=16, amplitude=1e-1)
    scheme.n_avars = 1
    scheme.step_rejection_drho = 2.4e-3
    scheme.step_rejection_max_exponent = 6
    q0 = tracers(mesh, u0, 1)
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    s.set_avars(q0)
    t_gpu, n_gpu = s.advance(n_steps=12)
    q_gpu = s.get_avars()
    assert n_gpu == 12 and s.step_rejections() > 0
    s.close()
    _, q_ref, t_ref, n_ref = _oracle(olib, raw, mesh, scheme).run(u0, n_steps=12, avars=q0)
    assert n_ref == 12 and abs(t_gpu - t_ref) <= 1e-12 * t_ref
    d_gpu, d_ref = q_gpu - q0, q_ref - q0
    err = np.abs(d_gpu - d_ref).max() / np.abs(d_ref).max()
    print(f"tracers with step rejection: change error {err:.2e}")
    assert err <= TOL_WB_RUN


def test_tracer_snapshot_restart(zlib, tmp_path):
    raw, mesh, scheme, u0, q0 = _case("polytrope")
    a = z.Solver(mesh, scheme)
    a.set_state(u0)
    a.set_avars(q0)
    a.advance(n_steps=5)
    a.write_snapshot(tmp_path / "s.npz", n_steps=5)
    a.advance(n_steps=5)
    qa = a.get_avars()
    snap = z.read_snapshot(tmp_path / "s.npz")
    assert snap["avars"].shape == (mesh.n_cells, NA)
    b = z.Solver(mesh, scheme)
    assert b.read_snapshot(tmp_path / "s.npz") == 5
    b.advance(n_steps=5)
    assert np.array_equal(qa, b.get_avars())
    # server requests carry no advected variables
    srv = z.Server(max_slots=2, steps_per_round=2)
    try:
        with pytest.raises(z.ZfvmError):
            srv.submit(mesh, scheme, u0, n_steps=1)
    finally:
        srv.close()
