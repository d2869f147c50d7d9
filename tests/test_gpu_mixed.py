"""Mixed FP32/FP64 form against the FP64 form (and the oracle).

Bars of the mixed form: relative L1 error of the conserved variables versus FP64
<= 1e-6 after N steps, and on the well-balanced problems also the relative L1
error of the perturbation (the change from the initial equilibrium plus bump)
<= 1e-6; well-balanced residual on the unperturbed equilibrium <= 1e-10 (max
|du/dt| and drift after N steps, relative).
"""
import numpy as np
import pytest

import zisafvm_gb300 as z
from metrics import perturbation_rel_l1, rel_errors, state_rel_l1
from problems import polytrope_2d, polytrope_2d_frozen, polytrope_3d, vortex_2d, vortex_tube_3d

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-6
TOL_WB = 1e-10


def _pair(mesh, scheme, u0):
    s64 = z.Solver(mesh, scheme)
    sch32 = z.Scheme(**{**scheme.__dict__, "precision": z.MIXED})
    s32 = z.Solver(mesh, sch32)
    s64.set_state(u0)
    s32.set_state(u0)
    return s64, s32


def test_mixed_c1_vortex(zlib):
    raw, mesh, scheme, u0 = vortex_2d(n=160, halo=3)
    s64, s32 = _pair(mesh, scheme, u0)
    s64.advance(n_steps=100)
    s32.advance(n_steps=100)
    u64, t64 = s64.get_state()
    u32, t32 = s32.get_state()
    l1, linf = rel_errors(u32, u64, raw.ghost == 0)
    print(f"mixed C1 100 steps: rel L1 {l1:.3e} rel Linf {linf:.3e}")
    assert l1 < TOL_MIXED
    assert abs(t32 - t64) < 1e-6 * t64


def test_mixed_rate_of_change_matches_fp64(zlib):
    raw, mesh, scheme, u0 = vortex_2d(n=32, halo=3, flux=z.FLUX_HLLC)
    s64, s32 = _pair(mesh, scheme, u0)
    t64, t32 = s64.rate_of_change(), s32.rate_of_change()
    inner = raw.ghost == 0
    cols = [0, 1, 2, 4]  # the 2D state has no third momentum
    err = np.abs(t32[inner][:, cols] - t64[inner][:, cols]).max(axis=0) / np.abs(t64[inner][:, cols]).max(axis=0)
    assert err.max() < 1e-5, err


def test_mixed_well_balanced(zlib):
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=40, amplitude=0.0, precision=z.MIXED)
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    t = s.rate_of_change()
    res = np.abs(t).max()
    print(f"mixed WB residual max|du/dt| = {res:.3e}")
    assert res < TOL_WB
    s.advance(n_steps=30)
    u, _ = s.get_state()
    drift = (np.abs(u - u0)[:, [0, 4]].max(axis=0) / np.abs(u0)[:, [0, 4]].max(axis=0)).max()
    print(f"mixed WB drift after 30 steps = {drift:.3e}")
    assert drift < TOL_WB


@pytest.mark.parametrize("amplitude", [1e-4, 1e-2])
def test_mixed_polytrope_perturbation(zlib, amplitude):
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=60, amplitude=amplitude)
    s64, s32 = _pair(mesh, scheme, u0)
    s64.advance(n_steps=40)
    s32.advance(n_steps=40)
    u64, _ = s64.get_state()
    u32, _ = s32.get_state()
    l1 = state_rel_l1(u32, u64)
    pert_err = perturbation_rel_l1(u32, u64, u0)
    print(f"A={amplitude:g}: state rel L1 {l1:.3e}, perturbation rel L1 {pert_err:.3e}")
    assert l1 < TOL_MIXED
    assert pert_err < TOL_MIXED


def test_mixed_tets(zlib):
    raw, mesh, scheme, u0 = vortex_tube_3d(n=8, order=3)
    s64, s32 = _pair(mesh, scheme, u0)
    s64.advance(n_steps=10)
    s32.advance(n_steps=10)
    u64, _ = s64.get_state()
    u32, _ = s32.get_state()
    l1, linf = rel_errors(u32, u64)
    assert l1 < TOL_MIXED, (l1, linf)


def test_mixed_polytrope_3d(zlib):
    """Tetrahedral well-balanced polytrope: residual at rest and the
    perturbation against the FP64 form."""
    raw, mesh, scheme, u0 = polytrope_3d(n=8, amplitude=0.0, precision=z.MIXED)
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    assert np.abs(s.rate_of_change()).max() < TOL_WB
    s.advance(n_steps=20)
    u, _ = s.get_state()
    drift = (np.abs(u - u0)[:, [0, 4]].max(axis=0) / np.abs(u0)[:, [0, 4]].max(axis=0)).max()
    assert drift < TOL_WB
    raw, mesh, scheme, u0 = polytrope_3d(n=8, amplitude=1e-3)
    s64, s32 = _pair(mesh, scheme, u0)
    s64.advance(n_steps=20)
    s32.advance(n_steps=20)
    u64, _ = s64.get_state()
    u32, _ = s32.get_state()
    assert state_rel_l1(u32, u64) < TOL_MIXED
    assert perturbation_rel_l1(u32, u64, u0) < TOL_MIXED


def test_mixed_frozen_ghost_cells(zlib):
    """Frozen ghost cells in the mixed form: balanced at rest, ghosts unchanged,
    the perturbation against the FP64 form."""
    raw, mesh, scheme, u0 = polytrope_2d_frozen(n_rings=40, amplitude=0.0, precision=z.MIXED)
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    assert np.abs(s.rate_of_change()).max() < TOL_WB
    raw, mesh, scheme, u0 = polytrope_2d_frozen(n_rings=40, amplitude=1e-3)
    s64, s32 = _pair(mesh, scheme, u0)
    s64.advance(n_steps=20)
    s32.advance(n_steps=20)
    u64, _ = s64.get_state()
    u32, _ = s32.get_state()
    ghost = raw.ghost == 1
    assert np.array_equal(u32[ghost], u0[ghost])
    assert state_rel_l1(u32, u64) < TOL_MIXED
    assert perturbation_rel_l1(u32, u64, u0) < TOL_MIXED


def test_mixed_weno_ao(zlib):
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=40, amplitude=1e-3)
    scheme.reconstruction = z.RC_WENO_AO
    s64, s32 = _pair(mesh, scheme, u0)
    s64.advance(n_steps=20)
    s32.advance(n_steps=20)
    u64, _ = s64.get_state()
    u32, _ = s32.get_state()
    assert state_rel_l1(u32, u64) < TOL_MIXED
    assert perturbation_rel_l1(u32, u64, u0) < TOL_MIXED


def test_mixed_heating(zlib):
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=40, amplitude=1e-3)
    scheme.heating_rate, scheme.heating_r0, scheme.heating_r1 = 0.3, 0.2, 0.6
    s64, s32 = _pair(mesh, scheme, u0)
    t64, t32 = s64.rate_of_change(), s32.rate_of_change()
    assert np.abs(t32[:, 4] - t64[:, 4]).max() <= 1e-6 * np.abs(t64[:, 4]).max()
    s64.advance(n_steps=20)
    s32.advance(n_steps=20)
    u64, _ = s64.get_state()
    u32, _ = s32.get_state()
    assert state_rel_l1(u32, u64) < TOL_MIXED


@pytest.mark.parametrize("amplitude", [1e-6, 1e-2])
def test_mixed_c4_amplitude_range_ends(zlib, amplitude):
    """The ensemble's instances draw perturbation amplitudes from 1e-6 to 1e-2:
    at both ends the mixed form follows the FP64 form within 1e-6 over 50
    steps, on the state and on the perturbation (at 1e-6 the perturbation is
    a millionth of the state, where FP32 arithmetic on it matters most)."""
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=60, amplitude=amplitude)
    u0 = mesh.initial_conditions("polytrope", gamma=2.0, K=1.0, rho_c=1.0, k_phi=1.0, amplitude=amplitude,
                                 width=0.05, x0=0.35, y0=-0.25)
    s64, s32 = _pair(mesh, scheme, u0)
    s64.advance(n_steps=50)
    s32.advance(n_steps=50)
    u64, _ = s64.get_state()
    u32, _ = s32.get_state()
    l1, pert = state_rel_l1(u32, u64), perturbation_rel_l1(u32, u64, u0)
    print(f"A={amplitude:g}, 50 steps: state rel L1 {l1:.3e}, perturbation rel L1 {pert:.3e}")
    assert l1 < TOL_MIXED and pert < TOL_MIXED


def test_mixed_against_the_oracle(zlib, olib):
    """The mixed form against the FP64 oracle itself (not only the FP64 GPU
    form), 50 steps of the well-balanced disk."""
    import os
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=30, amplitude=1e-4)
    s32 = z.Solver(mesh, z.Scheme(**{**scheme.__dict__, "precision": z.MIXED}))
    s32.set_state(u0)
    s32.advance(n_steps=50)
    u32, _ = s32.get_state()
    o = olib.Oracle(raw, mesh.stencils(), scheme.oracle_vector(), quad=mesh.quad, threads=os.cpu_count())
    u_ref, _, _ = o.run(u0, n_steps=50)
    l1, pert = state_rel_l1(u32, u_ref), perturbation_rel_l1(u32, u_ref, u0)
    print(f"mixed vs oracle, 50 steps: state rel L1 {l1:.3e}, perturbation rel L1 {pert:.3e}")
    assert l1 < TOL_MIXED and pert < TOL_MIXED
