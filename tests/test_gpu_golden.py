"""The CUDA path against the committed golden fixtures (tests/golden/*.npz,
oracle outputs; see tests/test_golden.py), through the C ABI, with no oracle
at test time.

Bars, as in test_gpu_parity.py: tendencies within 1e-13 of each variable's
largest tendency and runs within 1e-12 relative L1 and Linf of the conserved
variables; on the well-balanced polytropes, whose tendency and change are
small residuals of O(1) terms, also 1e-11 of each variable's largest tendency
and 3e-12 of the largest change over the run (ten times the errors measured
on the comparable parity cases)."""
import os
import sys

import numpy as np
import pytest

import zisafvm_gb300 as z
from metrics import conserved_rel_errors, deviation_rel_max, rel_errors

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from cases import CASES  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_golden(zlib, name):
    make, steps, wb = CASES[name]
    f = np.load(os.path.join(GOLDEN, name + ".npz"))
    raw, mesh, scheme, _ = make()
    u0 = f["u0"]
    inner = np.ones(u0.shape[0], bool) if raw.ghost is None else raw.ghost == 0
    cols = (0, 1, 2, 4) if raw.n_dims == 2 else (0, 1, 2, 3, 4)
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    rhs = s.rate_of_change()
    tol_rhs = 1e-11 if wb else 1e-13
    for v in cols:
        scale = np.abs(f["rhs"][inner, v]).max()
        assert np.abs(rhs[inner, v] - f["rhs"][inner, v]).max() <= tol_rhs * scale, v
    s.set_state(u0)
    t, n = s.advance(n_steps=steps)
    u, _ = s.get_state()
    s.close()
    assert n == int(f["steps"]) and abs(t - float(f["t_end"])) <= 1e-13 * t
    if wb:
        l1, linf = conserved_rel_errors(u, f["u_end"], inner)
        dev = deviation_rel_max(u, f["u_end"], u0, inner)
        print(f"{name}: conserved rel L1 {l1:.2e} Linf {linf:.2e}, deviation rel max {dev:.2e}")
        assert l1 < 1e-12 and linf < 1e-12 and dev < 3e-12
    else:
        l1, linf = rel_errors(u, f["u_end"], inner, cols)
        assert l1 < 1e-12 and linf < 1e-12, (l1, linf)
