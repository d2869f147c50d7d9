"""The solver set-up fills its tables with OpenMP loops; every entry is
written by one thread from the same inputs, so the device tables, and the
states a solver computes from them, do not depend on the thread count."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import zisafvm_gb300 as z
from problems import polytrope_2d, polytrope_3d

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CHILD = r'''
import sys
sys.path[:0] = [sys.argv[1], sys.argv[1] + "/tests"]
import numpy as np, zisafvm_gb300 as z
from problems import polytrope_2d, polytrope_3d
out = {}
for name, make in (("disk", lambda p: polytrope_2d(n_rings=24, amplitude=1e-2, precision=p)),
                   ("cube", lambda p: polytrope_3d(n=6, precision=p))):
    for prec in (z.FP64, z.MIXED):
        raw, mesh, scheme, u0 = make(prec)
        s = z.Solver(mesh, scheme)
        s.set_state(u0)
        s.advance(n_steps=4)
        out[f"{name}_{prec}"] = s.get_state()[0]
np.savez(sys.argv[2], **out)
'''


def test_setup_tables_do_not_depend_on_the_thread_count(tmp_path):
    res = {}
    for threads in ("1", "7"):
        f = tmp_path / f"run_{threads}.npz"
        env = dict(os.environ, OMP_NUM_THREADS=threads)
        subprocess.run([sys.executable, "-c", CHILD, str(ROOT), str(f)], env=env, check=True, timeout=600)
        res[threads] = np.load(f)
    for k in res["1"].files:
        assert np.array_equal(res["1"][k], res["7"][k]), k
