"""Writes tests/golden/<case>.npz: the oracle's tendency of the initial state
and its state after a few steps, for the cases of tests/golden/cases.py.

Run from the repository root (the native library and the oracle are built on
first use):  python tests/golden/make_oracle_fixtures.py
The oracle runs single-threaded so its face-loop sums have a fixed order."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from cases import CASES  # noqa: E402
from oracle import pyoracle  # noqa: E402


def main():
    for name, (make, steps, wb) in CASES.items():
        raw, mesh, scheme, u0 = make()
        o = pyoracle.Oracle(raw, mesh.stencils(), scheme.oracle_vector(), quad=mesh.quad, threads=1)
        rhs = o.rate_of_change(u0)
        u, t, n = o.run(u0, n_steps=steps)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), u0=u0, rhs=rhs, u_end=u, t_end=np.float64(t),
                 steps=np.int64(n), well_balanced=np.bool_(wb))
        print(name, mesh.n_cells, "cells", n, "steps, t =", t)


if __name__ == "__main__":
    main()
