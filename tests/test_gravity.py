"""The reference's radial gravity potentials (model/gravity_decl.hpp,
model/gravity_impl.hpp, built by make_gravity in model/euler_factory.cpp:60-121)
in the oracle and in the product's set-up, without a GPU.

The oracle's potentials are checked against their closed forms and finite
differences; the product's set-up shares them through the initial data of an
isentropic polytrope in each potential (zfvm_initial_conditions kind 2).
"""
import numpy as np
import pytest

import zisafvm_gb300 as z
from oracle import pyoracle

POLYTROPE = dict(gravity=z.GRAVITY_POLYTROPE_RADIAL, gravity_params=[1.0, 1.0, 1.0])
JUMP = dict(gravity=z.GRAVITY_POLYTROPE_JUMP_RADIAL, gravity_params=[0.5, 1.0, 1.0, 2.0, 1.0])
POINT = dict(gravity=z.GRAVITY_POINT_MASS_RADIAL, gravity_params=[1.0, 0.5, 1.0])


def _vector(**kw):
    return z.Scheme(**kw).oracle_vector()


def _points(n=200, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.9, 0.9, size=(n, 3))
    x[:, 2] = 0.0
    return x


def test_polytrope_potential_closed_form():
    """PolytropeGravity (gravity_impl.hpp:29-58): phi = -2 K rhoC sin(a r) / (a r),
    a = sqrt(2 pi G / K), with the r -> 0 limit -2 K rhoC."""
    rhoC, K, G = 1.3, 0.8, 1.1
    x = _points()
    phi, grad = pyoracle.gravity(_vector(gravity=z.GRAVITY_POLYTROPE_RADIAL, gravity_params=[rhoC, K, G]), x)
    a, r = np.sqrt(2 * np.pi * G / K), np.linalg.norm(x, axis=1)
    assert np.allclose(phi, -2 * K * rhoC * np.sin(a * r) / (a * r), rtol=1e-14, atol=0)
    phi0, _ = pyoracle.gravity(_vector(gravity=z.GRAVITY_POLYTROPE_RADIAL, gravity_params=[rhoC, K, G]), [0, 0, 0])
    assert phi0[0] == -2 * K * rhoC


@pytest.mark.parametrize("case", [POLYTROPE, JUMP, POINT])
def test_gradient_is_the_derivative(case):
    """dphi/dx_k = phi'(r) x_k / (r + 1e-50) (Gravity::dphi_dx with
    RadialAlignment::dx): central differences of phi agree."""
    sv = _vector(**case)
    x = _points(50, seed=1)
    x = x[np.abs(np.linalg.norm(x, axis=1) - 0.5) > 1e-3]  # off the jump radius
    _, grad = pyoracle.gravity(sv, x)
    h = 1e-6
    for d in range(2):
        e = np.zeros(3)
        e[d] = h
        fd = (pyoracle.gravity(sv, x + e)[0] - pyoracle.gravity(sv, x - e)[0]) / (2 * h)
        assert np.abs(fd - grad[:, d]).max() < 1e-7 * max(1.0, np.abs(grad).max())


def test_jump_potential_is_continuous_at_r_crit():
    """PolytropeGravityWithJump's constructor scales the outer polytrope so
    phi is continuous at r_crit (gravity_impl.hpp:70-76)."""
    sv = _vector(**JUMP)
    r_crit = JUMP["gravity_params"][0]
    below, _ = pyoracle.gravity(sv, [r_crit * (1 - 1e-12), 0, 0])
    above, _ = pyoracle.gravity(sv, [r_crit, 0, 0])
    assert abs(below[0] - above[0]) < 1e-10 * abs(above[0])
    # the slope jumps (K_inner != K_outer)
    _, g_in = pyoracle.gravity(sv, [r_crit * 0.999, 0, 0])
    _, g_out = pyoracle.gravity(sv, [r_crit * 1.001, 0, 0])
    assert abs(g_in[0, 0] - g_out[0, 0]) > 1e-3 * abs(g_in[0, 0])


def test_table_interpolates_like_the_reference():
    """NonUniformLinearInterpolation (math/linear_interpolation.hpp:14-45):
    linear between tabulated radii, the interval below the first radius >= r,
    the first interval extrapolated below the table."""
    r = np.array([0.0, 0.2, 0.5, 1.0, 1.5])
    phi = np.array([0.0, 0.1, 0.4, 0.3, 1.0])
    sv = _vector(gravity=z.GRAVITY_RADIAL_TABLE, gravity_table=(r, phi))
    q = np.array([0.1, 0.2, 0.35, 0.75, 1.2])
    got, grad = pyoracle.gravity(sv, np.c_[q, np.zeros(5), np.zeros(5)])
    assert np.allclose(got, np.interp(q, r, phi), rtol=0, atol=1e-15)
    slopes = np.diff(phi) / np.diff(r)
    assert np.allclose(grad[:, 0], slopes[[0, 0, 1, 2, 3]], rtol=1e-14)


def test_polytrope_initial_data_in_each_potential(zlib):
    """The product's potentials, through the initial data h + phi = h_c + phi(0):
    the harmonic potential reproduces the existing polytrope initial data, the
    polytrope potential gives the Lane-Emden profile rho_c sin(a r) / (a r)."""
    raw = z.RawMesh.generate("disk", n=20, radius=1.0, jitter=0.2, seed=5)
    mesh = z.Mesh(raw, z.StencilSpec.cweno(3, 2), quad=(3, 3, 2))
    old = mesh.initial_conditions("polytrope", gamma=2.0, K=1.0, rho_c=1.0, k_phi=1.0, amplitude=1e-3)
    new = mesh.initial_conditions("polytrope_in", gamma=2.0, K=1.0, rho_c=1.0, amplitude=1e-3,
                                  gravity=z.GRAVITY_HARMONIC_RADIAL, gravity_strength=1.0)
    assert np.abs(new - old).max() <= 1e-15 * np.abs(old).max()
    le = mesh.initial_conditions("polytrope_in", gamma=2.0, K=1.0, rho_c=1.0, amplitude=0.0, **POLYTROPE)
    c = mesh.geometry()["centers"]
    a, r = np.sqrt(2 * np.pi), np.linalg.norm(c, axis=1)
    h = 1.0 / 20  # ring spacing: cell averages differ from centre values by O(h^2)
    assert np.abs(le[:, 0] - np.sin(a * r) / (a * r)).max() < 2 * h * h
    assert np.allclose(le[:, 4], le[:, 0] ** 2, rtol=2 * h * h)  # p = K rho^2, E = p / (gamma - 1)
    with pytest.raises(z.ZfvmError):
        mesh.initial_conditions("polytrope_in", gravity=z.GRAVITY_RADIAL_TABLE)
