"""Checkpoint and restart through snapshot files: a run of 2n steps equals n
steps, a snapshot, a restart in a fresh solver and n more steps, bit for bit
in both forms (the device state is a function of the FP64 cell averages and
the time, which the snapshot holds exactly).  The clock comes back too:
LoadSnapshot::do_load sets the time and the step count (io/load_snapshot.cpp:9-13).
"""
import numpy as np
import pytest

import zisafvm_gb300 as z
from problems import polytrope_2d, vortex_tube_3d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["polytrope_2d_fp64", "polytrope_2d_mixed", "tube_3d_mixed"])
def test_restart_continues_bit_for_bit(zlib, tmp_path, case):
    if case.startswith("polytrope"):
        precision = z.MIXED if case.endswith("mixed") else z.FP64
        raw, mesh, scheme, u0 = polytrope_2d(n_rings=30, amplitude=1e-2, seed=3, precision=precision)
    else:
        raw, mesh, scheme, u0 = vortex_tube_3d(n=10)
        scheme.precision = z.MIXED
    n = 12
    a = z.Solver(mesh, scheme)
    a.set_state(u0, 0.0)
    t_half, s = a.advance(n_steps=n)
    assert s == n
    a.write_snapshot(tmp_path / "snapshot_0001.npz", n_steps=n)
    t_a, _ = a.advance(n_steps=n)
    ua, _ = a.get_state()
    a.close()

    snap = z.read_snapshot(tmp_path / "snapshot_0001.npz")
    assert snap["time"] == t_half and snap["n_steps"] == n

    b = z.Solver(mesh, scheme)
    assert b.read_snapshot(tmp_path / "snapshot_0001.npz") == n
    _, t_b0 = b.get_state()
    assert t_b0 == t_half
    t_b, _ = b.advance(n_steps=n)
    ub, _ = b.get_state()
    b.close()
    assert t_b == t_a
    assert np.array_equal(ua, ub)


def test_restart_refuses_other_mesh_and_steady_state(zlib, tmp_path):
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=12)
    z.write_snapshot(tmp_path / "steady_state.npz", u0)
    s = z.Solver(mesh, scheme)
    with pytest.raises(z.ZfvmError, match="steady state"):
        s.read_snapshot(tmp_path / "steady_state.npz")
    z.write_snapshot(tmp_path / "small.npz", u0[:-1], t=0.0, n_steps=0)
    with pytest.raises(z.ZfvmError, match="cells"):
        s.read_snapshot(tmp_path / "small.npz")
    s.close()
