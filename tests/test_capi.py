"""The C-ABI library loads and exports every entry point include/*.h declares."""
import ctypes
import re

import pytest
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(zfvm_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "zfvm_solver_create" in names and "zfvm_last_error" in names
    assert len(names) >= 20


def test_library_exports_every_symbol(zlib):
    lib = ctypes.CDLL(str(zlib.library_path()))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_the_header(zlib):
    """Every declared entry point has argument types in the bindings' table
    (zfvm_last_error, which takes none, is set up on its own)."""
    src = (ROOT / "zisafvm_gb300" / "__init__.py").read_text()
    bound = set(re.findall(r'"(zfvm_\w+)"\s*:', src))
    assert [n for n in declared_symbols() if n not in bound and n != "zfvm_last_error"] == []
    assert sorted(bound - set(declared_symbols())) == []


def test_error_reporting_without_compute(zlib):
    z = zlib
    lib = z.load_library()
    assert lib.zfvm_mesh_create(None, None) == 1
    assert b"null" in lib.zfvm_last_error()


def test_solver_footprint_without_device(zlib):
    """The admission estimate is host arithmetic: available without a GPU."""
    z = zlib
    from problems import polytrope_2d
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=12)
    f64 = z.solver_footprint(mesh, scheme)
    scheme.precision = z.MIXED
    f32 = z.solver_footprint(mesh, scheme)
    raw2, mesh2, scheme2, _ = polytrope_2d(n_rings=24)
    f64_big = z.solver_footprint(mesh2, scheme2)
    assert 0 < f32 < f64 < f64_big
    per_cell = f64_big / mesh2.n_cells
    assert 500 < per_cell < 5000


def test_solver_validation_runs_before_cuda(zlib):
    """zfvm_solver_create checks its configuration before any CUDA call:
    invalid schemes are refused with ZFVM_EINVAL on any host; on a host
    without a GPU a valid one gets as far as the first CUDA call."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    from problems import polytrope_2d
    from conftest import gpu_available
    z = zlib
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=10)
    bad = [dict(steps_per_recompute=0), dict(rk_stages=4), dict(reconstruction=7), dict(n_avars=-1),
           dict(n_avars=1000), dict(heating_rate=1.0, gravity=z.GRAVITY_NONE, equilibrium=z.EQ_NONE,
                                    flux_bc=z.FLUX_BC_NONE), dict(step_rejection_drho=-1.0)]
    for change in bad:
        sc = z.Scheme(**{**scheme.__dict__, **change})
        with pytest.raises(z.ZfvmError) as e:
            z.Solver(mesh, sc)
        assert e.value.code == 1, (change, e.value)
    if not gpu_available():
        for prec in (z.FP64, z.MIXED):
            with pytest.raises(z.ZfvmError) as e:
                z.Solver(mesh, z.Scheme(**{**scheme.__dict__, "precision": prec}))
            assert e.value.code == 6  # ZFVM_ECUDA: validation passed


def test_equilibrium_schedule_footprint_and_validation(zlib):
    """A refresh schedule adds the per-cell schedule state to the footprint;
    steps_per_recompute below 1 is refused before any device work."""
    z = zlib
    from problems import polytrope_2d
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=12)
    every = z.solver_footprint(mesh, scheme)
    scheme.steps_per_recompute = 3
    scheduled = z.solver_footprint(mesh, scheme)
    assert scheduled > every
    scheme.steps_per_recompute = 0
    with pytest.raises(z.ZfvmError) as e:
        z.Solver(mesh, scheme)
    assert e.value.code == 1 and "steps_per_recompute" in str(e.value)
