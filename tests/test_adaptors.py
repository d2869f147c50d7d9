"""The C++ drop-in adaptors (include/zfvm_zisa.hpp: GpuLocalCFL, GpuRateOfChange,
GpuRungeKutta, GpuGlobalReconstruction, GpuBoundaryCondition, GpuHLLCBatten,
GpuRusanov, NpzDumpSnapshot, NpzLoadSnapshot) compile against the C ABI, and
on a GPU give the same numbers as the library's other bindings and the oracle."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _build(tmp_path, zlib) -> Path:
    exe = tmp_path / "adaptor_main"
    lib = Path(zlib.library_path())
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", str(ROOT / "include"), str(ROOT / "tests" / "adaptor_main.cpp"),
           "-o", str(exe), "-L", str(lib.parent), "-lzfvm", f"-Wl,-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_adaptors_compile_and_link(tmp_path, zlib):
    assert _build(tmp_path, zlib).exists()


@pytest.mark.gpu
def test_adaptors_match_python_binding(tmp_path, zlib):
    z = zlib
    exe = _build(tmp_path, zlib)
    r = subprocess.run([str(exe), "10", str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {ln.split()[0]: ln.split()[1:] for ln in r.stdout.splitlines()}
    from problems import polytrope_2d
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=10, amplitude=1e-2, seed=7)
    scheme.n_avars = 1
    cx = raw.vertices[raw.vertex_indices].mean(axis=1)[:, 0]
    q0 = u0[:, :1] * (0.25 + 0.5 * cx[:, None])
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    s.set_avars(q0)
    dt = s.cfl_dt()
    assert float(out["dt"][0]) == dt
    tend, tq = s.rate_of_change_all()
    s.set_state(u0)
    s.set_avars(q0)
    s.step(dt)
    u1, _ = s.get_state()
    q1 = s.get_avars()
    assert float(out["sums"][0]) == pytest.approx(tend.sum(), rel=1e-14, abs=1e-14)
    assert float(out["sums"][1]) == pytest.approx(u1.sum(), rel=1e-14)
    assert float(out["avars"][0]) == pytest.approx(tq.sum(), rel=1e-12, abs=1e-12)
    assert float(out["avars"][1]) == pytest.approx(q1.sum(), rel=1e-14)
    # the snapshot holds the stepped state and the clock, and reads back equal
    assert out["snapshot"][0] == "1" and out["snapshot"][2] == "1"
    assert float(out["snapshot"][1]) == dt
    snap = z.read_snapshot(tmp_path / "snapshot_0000.npz")
    assert np.array_equal(snap["cvars"], u1) and snap["n_steps"] == 1
    # the example forms its tracer's centroids in another order: last-bit differences
    assert np.abs(snap["avars"] - q1).max() <= 1e-13 * np.abs(q1).max()
    cell = int(out["cell"][0])
    s.set_state(u0)
    s.reconstruct()
    ux = s.reconstruction_eval([cell], [[0.25, 0.1, 0.0]])[0]
    assert np.allclose([float(a) for a in out["recon"]], ux, rtol=1e-15, atol=0)
    st = mesh.stencils()
    assert out["cell"][1] == "stencil" and int(out["cell"][2]) == int(st["n_l2g"][cell])
    # HLLCBatten's static interface and the Rusanov flux against the oracle's
    from oracle import pyoracle
    fl, fr = [1.0, 0.3, -0.2, 0.1, 2.5], [0.8, 0.1, 0.05, -0.1, 1.9]
    hllc = np.array([float(a) for a in out["hllc"]])
    assert np.allclose(hllc[:5], pyoracle.flux(0, 1.4, fl, fr), rtol=1e-14, atol=1e-15)
    f, sp = z.numerical_flux(z.FLUX_HLLC, 1.4, fl, fr)
    assert np.array_equal(hllc[:5], f[0]) and np.array_equal(hllc[5:], sp[0])
    assert float(out["tracer"][0]) == pytest.approx(pyoracle.tracer_flux(0, 1.4, fl, fr, 0.4, 0.6), rel=1e-14)
    rus = np.array([float(a) for a in out["rusanov"]])
    assert np.allclose(rus[:5], pyoracle.flux(1, 1.4, fl, fr), rtol=1e-14, atol=1e-15)
    assert out["bc"][0] == "1"
