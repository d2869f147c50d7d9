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
