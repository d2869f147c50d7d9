"""The FP64 form against the oracle at the benchmark sizes.

C2: the well-balanced polytrope disk (199,076 cells), 100 steps.  C3: the
tetrahedral vortex tube (2,058,000 cells), orders 2 and 3, 50 steps.  The bar
is 1e-12 relative in L1 and Linf of the conserved variables (over the whole
state; for the equilibrium's density and energy also per variable).  On the
well-balanced disk the momenta and the change of the state are small
differences of O(1) terms, so their error against their own size is also
checked, at ten times the error measured on GB300.
"""
import os

import numpy as np
import pytest

from metrics import conserved_rel_errors, deviation_rel_max, rel_errors
from problems import polytrope_2d, vortex_tube_3d

pytestmark = pytest.mark.gpu

TOL_RUN = 1e-12
# ten times the deviation error measured on GB300: the change of the state is
# a small difference of O(1/h) flux and source terms, so a reordering of FP64
# arithmetic moves it by about one ulp of the O(1) state
DEV_TOL_C2 = 5e-10  # measured 3.6e-11 - 4.8e-11 (the oracle against itself: the same order)


def _run_pair(z, olib, raw, mesh, scheme, u0, n_steps):
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    t_gpu, n_gpu = s.advance(n_steps=n_steps)
    u_gpu, _ = s.get_state()
    s.close()
    o = olib.Oracle(raw, mesh.stencils(), scheme.oracle_vector(), quad=mesh.quad, threads=os.cpu_count())
    u_ref, t_ref, n_ref = o.run(u0, n_steps=n_steps)
    assert n_gpu == n_ref == n_steps
    assert abs(t_gpu - t_ref) <= 1e-12 * t_ref
    return u_gpu, u_ref


def test_c2_full_100_steps(zlib, olib):
    z = zlib
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=178, amplitude=1e-4)
    assert mesh.n_cells == 199076
    u_gpu, u_ref = _run_pair(z, olib, raw, mesh, scheme, u0, 100)
    l1, linf = conserved_rel_errors(u_gpu, u_ref)
    print(f"C2 100 steps: conserved rel L1 {l1:.3e} Linf {linf:.3e}")
    assert l1 < TOL_RUN and linf < TOL_RUN
    l1_rE, linf_rE = rel_errors(u_gpu, u_ref, cols=(0, 4))
    assert l1_rE < TOL_RUN and linf_rE < TOL_RUN
    dev = deviation_rel_max(u_gpu, u_ref, u0)
    print(f"C2 100 steps: deviation rel max {dev:.3e}")
    assert dev < DEV_TOL_C2


@pytest.mark.parametrize("order", [3, 2])
def test_c3_full_50_steps(zlib, olib, order):
    z = zlib
    raw, mesh, scheme, u0 = vortex_tube_3d(n=70, order=order)
    assert mesh.n_cells == 2058000
    u_gpu, u_ref = _run_pair(z, olib, raw, mesh, scheme, u0, 50)
    l1, linf = conserved_rel_errors(u_gpu, u_ref)
    print(f"C3 order {order} 50 steps: conserved rel L1 {l1:.3e} Linf {linf:.3e}")
    assert l1 < TOL_RUN and linf < TOL_RUN
    # per variable, but for the third momentum: the tube's flow is planar and
    # its z-momentum stays at round-off size
    l1, linf = rel_errors(u_gpu, u_ref, cols=(0, 1, 2, 4))
    print(f"C3 order {order} 50 steps: per-variable rel L1 {l1:.3e} Linf {linf:.3e}")
    assert l1 < TOL_RUN and linf < TOL_RUN
