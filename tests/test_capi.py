"""The C-ABI library loads and exports every entry point include/*.h declares."""
import ctypes
import re
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
