"""The numerical fluxes and the ghost-cell boundary condition as standalone
calls (zfvm_numerical_flux, zfvm_tracer_flux, zfvm_apply_boundary), against
the oracle's HLLCBatten / Rusanov and the reference's boundary semantics."""
import numpy as np
import pytest

from problems import polytrope_2d_frozen, vortex_2d

pytestmark = pytest.mark.gpu


def _states(rng, n, gamma):
    rho = rng.uniform(0.3, 2.0, n)
    v = rng.uniform(-1.5, 1.5, (n, 3))
    p = rng.uniform(0.2, 3.0, n)
    E = p / (gamma - 1.0) + 0.5 * rho * (v * v).sum(axis=1)
    return np.c_[rho, rho[:, None] * v, E]


@pytest.mark.parametrize("kind", [0, 1])
def test_numerical_flux_matches_the_oracle(zlib, olib, kind):
    """HLLCBatten::flux / tracer_flux (flux/hllc.hpp:142-197) and the Rusanov
    flux of 400 random face-state pairs, including supersonic ones, in one
    launch each."""
    z = zlib
    gamma = 1.4
    rng = np.random.default_rng(3 + kind)
    uL, uR = _states(rng, 400, gamma), _states(rng, 400, gamma)
    f, sp = z.numerical_flux(kind, gamma, uL, uR)
    ref = np.array([olib.flux(kind, gamma, a, b) for a, b in zip(uL, uR)])
    assert np.abs(f - ref).max() <= 1e-14 * np.abs(ref).max()
    qL, qR = rng.uniform(0, 1, 400), rng.uniform(0, 1, 400)
    tq = z.tracer_flux(kind, uL, uR, uL[:, 0] * qL, uR[:, 0] * qR, sp)
    tref = np.array([olib.tracer_flux(kind, gamma, a, b, x, y) for a, b, x, y in
                     zip(uL, uR, uL[:, 0] * qL, uR[:, 0] * qR)])
    assert np.abs(tq - tref).max() <= 1e-14 * np.abs(tref).max()
    if kind == 0:
        assert (sp[:, 0] <= sp[:, 1]).all() and (sp[:, 1] <= sp[:, 2]).all()
    else:
        assert np.array_equal(sp[:, 0], -sp[:, 2]) and not sp[:, 1].any()
    # consistency: equal states give the physical flux
    f_same, _ = z.numerical_flux(kind, gamma, uL, uL)
    assert np.abs(f_same - np.array([olib.euler_flux(gamma, a) for a in uL])).max() <= 1e-14 * np.abs(f_same).max()


def test_apply_boundary_periodic_images(zlib):
    """Periodic ghost cells take their source cells' rows; interior rows stay."""
    z = zlib
    raw, mesh, scheme, u0 = vortex_2d(n=16, halo=3)
    s = z.Solver(mesh, scheme)
    ghost = raw.ghost == 1
    u = u0.copy()
    u[ghost] = 123.0
    out = s.apply_boundary(u)
    assert np.array_equal(out[~ghost], u0[~ghost])
    assert np.array_equal(out[ghost], u0[raw.source[ghost]])


def test_apply_boundary_frozen_cells(zlib):
    """FrozenBC::apply (boundary/frozen_boundary_condition.cpp:39-55): frozen
    ghost cells are reset to the frozen rows, with advected variables."""
    z = zlib
    raw, mesh, scheme, u0 = polytrope_2d_frozen(n_rings=16, amplitude=1e-2)
    scheme.n_avars = 1
    s = z.Solver(mesh, scheme)
    ghost = raw.ghost == 1
    q0 = u0[:, :1] * 0.5
    u, q = u0 * 1.01, q0 * 3.0
    out, qout = s.apply_boundary(u, frozen=u0, avars=q, frozen_avars=q0)
    assert np.array_equal(out[ghost], u0[ghost]) and np.array_equal(out[~ghost], u[~ghost])
    assert np.array_equal(qout[ghost], q0[ghost]) and np.array_equal(qout[~ghost], q[~ghost])
    # without frozen rows the ghost rows are kept
    kept, qkept = s.apply_boundary(u, avars=q)
    assert np.array_equal(kept, u) and np.array_equal(qkept, q)
