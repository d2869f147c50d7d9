"""Build recipe for the CPU oracle (``oracle/_build/liboracle.so``).

Plain g++ with OpenMP; ``-ffp-contract=off`` keeps results identical on
x86-64 and aarch64.  The reference itself cannot be compiled (it needs Eigen,
Boost, HDF5, nlohmann_json and the unpinned Zisa* sibling libraries), so there
is no ``oracle/_ref`` build.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "zfvm_oracle.cpp"
OUT = HERE / "_build" / "liboracle.so"
FLAGS = ["-std=c++17", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if not force and OUT.exists() and OUT.stat().st_mtime > SRC.stat().st_mtime:
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    r = subprocess.run(["g++", *FLAGS, str(SRC), "-o", str(tmp)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
