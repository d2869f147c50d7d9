"""Golden fixtures (tests/golden/*.npz, written by
tests/golden/make_oracle_fixtures.py): the oracle's tendency of a seeded
initial state and its state after a few steps, for small 2D and 3D problems.

Here, on the CPU: the problem set-up (seeded meshes, stencils, initial data)
and the oracle still reproduce them.  Tolerances: initial states within 1e-14
and oracle results within 1e-13 of each variable's largest value -- the
fixtures were written on another host, whose libm may round the initial data's
transcendental functions differently in the last bit."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from cases import CASES  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def close(a, ref, tol):
    scale = np.maximum(np.abs(ref).max(axis=0), 1e-300)
    return (np.abs(a - ref).max(axis=0) / scale).max() <= tol


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(zlib, olib, name):
    make, steps, _ = CASES[name]
    f = load(name)
    raw, mesh, scheme, u0 = make()
    assert close(u0, f["u0"], 1e-14)
    o = olib.Oracle(raw, mesh.stencils(), scheme.oracle_vector(), quad=mesh.quad, threads=1)
    assert close(o.rate_of_change(f["u0"]), f["rhs"], 1e-13)
    u, t, n = o.run(f["u0"], n_steps=steps)
    assert n == int(f["steps"]) and abs(t - float(f["t_end"])) <= 1e-14 * t
    assert close(u, f["u_end"], 1e-13)
