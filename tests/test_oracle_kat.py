"""Known-answer tests of the oracle, restated from the reference's own unit tests.

Each case cites the reference test it pins (paths inside the ZisaFVM repository).
"""
import numpy as np
import pytest


def test_hllc_consistency(olib):
    # test/zisa/unit_test/flux/hllc.cpp:10-26: F_HLLC(u, u) = F(u), gamma = 1.6, tol 1e-12
    u = [1.0, -0.2, 0.3, 0.8, 12.0]
    nf = olib.flux(0, 1.6, u, u)
    pf = olib.euler_flux(1.6, u)
    assert np.allclose(nf, pf, rtol=1e-12, atol=1e-12)


def test_rusanov_consistency(olib):
    # the Rusanov flux is consistent in the same sense
    u = [1.3, 0.4, -0.1, 0.0, 5.0]
    assert np.allclose(olib.flux(1, 1.4, u, u), olib.euler_flux(1.4, u), rtol=1e-14, atol=1e-14)


def test_hllc_supersonic_upwind(olib):
    # s_L >= 0: the HLLC flux is the left physical flux (hllc.hpp:160-176)
    uL = [1.0, 5.0, 0.0, 0.0, 20.0]
    uR = [0.8, 4.0, 0.0, 0.0, 15.0]
    assert np.allclose(olib.flux(0, 1.4, uL, uR), olib.euler_flux(1.4, uL), rtol=1e-14)


def test_poly2d_examples(olib):
    # test/zisa/unit_test/math/poly2d.cpp:133-166, tolerance 1e-14
    coeffs = [1.0, 2.0, 3.0, 4.0, 5.0, 6.0]
    moments = [0.0, 0.0, 0.0, 1.0, 2.0, 3.0]
    x0 = olib.poly_eval(2, coeffs, moments, [0, 0, 0], 1.0, [0, 0, 0])
    assert abs(x0 - (1.0 - 4.0 - 10.0 - 18.0)) <= 1e-14 * 31
    x, y = -3.0, 2.0
    exact = 1.0 + 2.0 * x + 3.0 * y + 4.0 * (x * x - 1.0) + 5.0 * (x * y - 2.0) + 6.0 * (y * y - 3.0)
    assert abs(olib.poly_eval(2, coeffs, moments, [0, 0, 0], 1.0, [x, y, 0]) - exact) <= 1e-14 * abs(exact)


def test_poly3d_example(olib):
    # test/zisa/unit_test/math/poly2d.cpp:201-275 (first variable)
    c = [1.0, 2.0, -1.0, -3.0, 2.0, 4.0, 2.0, 1.0, 1.0, 3.0]
    m = [0.0, 0.0, 0.0, 0.0, 1.0, 2.0, 3.0, 4.0, 5.0, 6.0]
    x, y, z = -3.0, 2.0, 0.2
    exact = (c[0] + c[1] * x + c[2] * y + c[3] * z + c[4] * (x * x - 1.0) + c[5] * (x * y - 2.0)
             + c[6] * (x * z - 3.0) + c[7] * (y * y - 4.0) + c[8] * (y * z - 5.0) + c[9] * (z * z - 6.0))
    assert abs(olib.poly_eval(3, c, m, [0, 0, 0], 1.0, [x, y, z]) - exact) <= 1e-14 * abs(exact)


@pytest.mark.parametrize("stages,window,dts", [(1, (0.9, 1.1), (1e-3, 1e-4)), (2, (1.9, 2.1), (1e-3, 1e-4)),
                                                (3, (2.9, 3.1), (1e-1, 1e-2))])
def test_runge_kutta_rates(olib, stages, window, dts):
    # test/zisa/unit_test/ode/runge_kutta.cpp:91-199
    assert olib.rk_ode_error(stages, 0, 0.01) < 1e-12
    for ode in (1, 2):
        coarse, fine = (olib.rk_ode_error(stages, ode, dt) for dt in dts)
        if fine > 1e-12:
            rate = (np.log(fine) - np.log(coarse)) / (np.log(dts[1]) - np.log(dts[0]))
            assert window[0] <= rate <= window[1], (ode, rate)


def test_local_equilibrium(olib):
    # test/zisa/unit_test/model/local_equilibrium.cpp:15-60: gamma 1.2, R 0.9,
    # ConstantGravityRadial(0.9), quad degree 2, tolerance 1e-9
    tri = [[1.0, 1.0, 0.0], [1.01, 1.0, 0.0], [1.0, 1.01, 0.0]]
    x_ref = [0.5, 0.6, 0.0]
    theta = [10.0, 3.0]
    rhoE_bar = olib.equilibrium_average(1.2, 1, 0.9, theta, x_ref, tri, 2)
    x = [1.1, 2.1, 0.0]
    st, approx, th = olib.local_equilibrium(1.2, 0.9, 1, 0.9, tri, 2, rhoE_bar, x)
    assert st == 0
    assert np.allclose(approx, _isentropic_point(1.2, 0.9, theta, x_ref, x), rtol=1e-9)
    tri2 = [[1.2, 1.1, 0.0], [1.21, 1.1, 0.0], [1.2, 1.11, 0.0]]
    exact2 = olib.equilibrium_average(1.2, 1, 0.9, theta, x_ref, tri2, 2)
    approx2 = olib.equilibrium_average(1.2, 1, 0.9, th, _first_qp(tri), tri2, 2)
    assert np.allclose(approx2, exact2, rtol=1e-9)


def test_eos_round_trips(olib):
    # test/zisa/unit_test/model/eos.cpp:7-23: IdealGasEOS(1.2, 0.9), (rho, E) = (1, 2)
    # through (h, K) and back, and through (rho, p) and back, within 1e-10
    via_hK, via_p = olib.eos_roundtrips(1.2, 0.9, 1.0, 2.0)
    assert np.allclose(via_hK, [1.0, 2.0], rtol=1e-10, atol=0.0)
    assert np.allclose(via_p, [1.0, 2.0], rtol=1e-10, atol=0.0)


def test_quasi_newton_problems(olib):
    # test/zisa/unit_test/math/quasi_newton.cpp:9-54, solved by the quasi-Newton
    # iteration the equilibrium solve uses: converged, within 10 atol = 1e-9
    x, st = olib.quasi_newton_problem(0)
    assert st == 0 and abs(x[0] - 1.2345) <= 1e-9
    x, st = olib.quasi_newton_problem(1)
    assert st == 0 and np.all(np.abs(x) <= 1e-9)


def test_frozen_ghost_cells_keep_their_values(zlib, olib):
    # test/zisa/unit_test/boundary/frozen_boundary_condition.cpp:9-51: ghost
    # cells under FrozenBC keep the values they were set to, bit for bit, here
    # through whole RK steps of the well-balanced polytrope with the reference's
    # experiment mask (ghost cells beyond r = 0.5), each ghost cell set to
    # distinct values
    from problems import polytrope_2d_frozen
    raw, mesh, scheme, u0 = polytrope_2d_frozen(n_rings=12, amplitude=1e-2)
    ghost = np.where(raw.ghost == 1)[0]
    assert len(ghost) > 0
    u = u0.copy()
    u[ghost] *= 1.0 + 1e-3 * (np.arange(len(ghost)) % 7)[:, None]
    o = olib.Oracle(raw, mesh.stencils(), scheme.oracle_vector(), quad=mesh.quad, threads=2)
    out, t, n = o.run(u, n_steps=3)
    assert n == 3 and np.array_equal(out[ghost], u[ghost])
    assert not np.array_equal(out[raw.ghost == 0], u[raw.ghost == 0])


def _isentropic_point(gamma, g, theta, x_ref, x):
    # h(x) = h_ref + phi(x_ref) - phi(x), phi = g |x|; rho = ((gamma-1)/gamma h/K)^(1/(gamma-1))
    h = theta[0] + g * np.linalg.norm(x_ref) - g * np.linalg.norm(x)
    rho = ((gamma - 1.0) / gamma * h / theta[1]) ** (1.0 / (gamma - 1.0))
    return np.array([rho, theta[1] * rho ** gamma / (gamma - 1.0)])


def _first_qp(tri):
    # x_ref of LocalEquilibriumBase::solve_exact is the first quadrature point of
    # the degree-2 rule: barycentric (2/3, 1/6, 1/6)
    t = np.asarray(tri, float)
    return list(2.0 / 3.0 * t[0] + 1.0 / 6.0 * t[1] + 1.0 / 6.0 * t[2])


def test_pseudo_inverse_matches_ldlt_solve(zlib, olib):
    """The product solves the stencil least-squares problems with a precomputed
    pseudo-inverse (host Householder QR); the reference solves the normal
    equations with an LDLT factorisation per call (reconstruction/
    lsq_solver.cpp:40-85).  The oracle's LDLT restatement and the product's
    pseudo-inverses give the same right-hand side to round-off."""
    from problems import polytrope_2d, vortex_2d
    for raw, mesh, scheme, u0 in (vortex_2d(n=12, halo=3), polytrope_2d(n_rings=10, amplitude=1e-2)):
        o = olib.Oracle(raw, mesh.stencils(), scheme.oracle_vector(), quad=mesh.quad, threads=1)
        t_ldlt = o.rate_of_change(u0)
        o.use_pinv(mesh)
        t_pinv = o.rate_of_change(u0)
        scale = np.abs(t_ldlt).max(axis=0)
        for v in range(5):
            if scale[v] > 0:
                assert np.abs(t_pinv[:, v] - t_ldlt[:, v]).max() <= 1e-12 * scale[v], v
