"""The oracle's advected variables (AllVariables::avars): properties that pin
the restated tracer flux (flux/hllc.hpp:178-197) and the tracer path of the
time loop.  The reference's own tests hold no tracer vectors; the polynomial
fit and hybridisation the tracers go through are the ones the known-answer
tests of test_oracle_kat.py pin for the conserved variables.

Tolerances: flux identities within 1e-13 of the flux scale (a few roundings
apart); conservation within 1e-13 of the total; the Euler state bit for bit."""
import numpy as np
import pytest

from problems import tracers, vortex_2d

GAMMA = 1.4


def _state(rng):
    rho = rng.uniform(0.3, 3.0)
    v = rng.normal(size=3)
    p = rng.uniform(0.2, 3.0)
    return np.array([rho, *(rho * v), p / (GAMMA - 1) + 0.5 * rho * (v @ v)])


@pytest.mark.parametrize("kind", [0, 1])
def test_tracer_flux_consistency(olib, kind):
    """Equal states on both sides: the tracer flux is mq v."""
    rng = np.random.default_rng(3)
    for _ in range(200):
        u = _state(rng)
        q = rng.uniform(-2.0, 2.0)
        v = u[1] / u[0]
        c = np.sqrt(GAMMA * (GAMMA - 1) * (u[4] - 0.5 * (u[1:4] @ u[1:4]) / u[0]) / u[0])
        f = olib.tracer_flux(kind, GAMMA, u, u, q, q)
        assert abs(f - q * v) <= 1e-13 * abs(q) * (1 + abs(v) + c)


@pytest.mark.parametrize("kind", [0, 1])
def test_density_as_tracer_gives_the_mass_flux(olib, kind):
    """mq = rho on both sides: the tracer flux equals the mass flux."""
    rng = np.random.default_rng(4)
    for _ in range(200):
        uL, uR = _state(rng), _state(rng)
        f = olib.flux(kind, GAMMA, uL, uR)
        ft = olib.tracer_flux(kind, GAMMA, uL, uR, uL[0], uR[0])
        scale = abs(f[0]) + abs(uL[1]) + abs(uR[1]) + 1e-300
        assert abs(ft - f[0]) <= 1e-13 * scale


def _oracle(olib, raw, mesh, scheme, threads=4):
    return olib.Oracle(raw, mesh.stencils(), scheme.oracle_vector(), quad=mesh.quad, threads=threads)


def test_tracers_conserved_and_passive(zlib, olib):
    raw, mesh, scheme, u0 = vortex_2d(n=12, halo=3, flux=0)
    # one thread: the face loop's atomic sums then run in a fixed order
    plain = _oracle(olib, raw, mesh, scheme, threads=1)
    u_plain, t_plain, _ = plain.run(u0, n_steps=4)
    scheme.n_avars = 3
    q0 = tracers(mesh, u0, 3)
    o = _oracle(olib, raw, mesh, scheme, threads=1)
    u1, q1, t1, n1 = o.run(u0, n_steps=4, avars=q0)
    assert n1 == 4 and t1 == t_plain
    # the tracers do not feed back into the flow
    assert np.array_equal(u1, u_plain)
    # periodic square: every tracer's total is conserved
    vol = mesh.geometry()["volumes"]
    inner = raw.ghost == 0
    for k in range(3):
        m0 = (vol[inner] * q0[inner, k]).sum()
        m1 = (vol[inner] * q1[inner, k]).sum()
        assert abs(m1 - m0) <= 1e-13 * (vol[inner] * np.abs(q0[inner, k])).sum()
    # they moved
    assert np.abs(q1[inner] - q0[inner]).max() > 1e-3
    # the tendency call agrees with the step's first stage: zero on ghost rows
    tu, tq = o.rate_of_change(u0, q0)
    assert np.array_equal(tu, plain.rate_of_change(u0))
    assert tq.shape == q0.shape and np.all(tq[~inner] == 0.0)


def test_uniform_mass_fraction_in_uniform_flow(zlib, olib):
    """A constant mass fraction in a constant state stays constant."""
    raw, mesh, scheme, u0 = vortex_2d(n=10, halo=3, flux=0)
    u = np.tile(np.array([1.0, 0.7, -0.4, 0.0, 3.0]), (u0.shape[0], 1))
    scheme.n_avars = 1
    q0 = 0.25 * u[:, :1]
    u1, q1, _, _ = _oracle(olib, raw, mesh, scheme).run(u, n_steps=3, avars=q0)
    inner = raw.ghost == 0
    assert np.abs(q1[inner, 0] / u1[inner, 0] - 0.25).max() < 1e-13


def test_missing_avars_is_an_error(zlib, olib):
    raw, mesh, scheme, u0 = vortex_2d(n=8, halo=3)
    scheme.n_avars = 1
    o = _oracle(olib, raw, mesh, scheme)
    with pytest.raises(olib.OracleError):
        o.run(u0, n_steps=1)
