"""Build recipe for the native library ``libzfvm.so`` (host C++ + CUDA for sm_103a).

The library is built in-tree (``zisafvm_gb300/libzfvm.so``) with g++ and nvcc
only; translation units compile in parallel.  Host code is compiled with
``-ffp-contract=off`` so the set-up arithmetic (geometry, stencils, LSQ
operators) is bit-identical on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libzfvm.so"
INCLUDE = PKG.parent / "include"

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-std=c++17", "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall"]
NVCCFLAGS = ["-std=c++17", "-O3", "-lineinfo", *ARCH, "--compress-mode=size", "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off",
             "--expt-relaxed-constexpr"]

HOST_SOURCES = ["grid.cpp", "stencil.cpp", "mesh.cpp", "capi_mesh.cpp", "snapshot.cpp"]
CUDA_SOURCES = ["solver.cu", "batch.cu", "server.cu", "noalloc.cu", "flux_api.cu"]
# inst_shape.cu compiled once per stencil shape x precision x (single solver,
# batch of 64, 128 or 256 threads per block): (object name, -D flags)
SHAPES = {"s2o3": "S2o3", "s2o2": "S2o2", "s3o3": "S3o3", "s3o2": "S3o2"}
SHAPE_UNITS = [
    (f"inst_{name}_{'mix' if mixed else 'f64'}{f'_batch{batch}' if batch else ''}",
     [f"-DZFVM_SHAPE_NAME={name}", f"-DZFVM_SHAPE={cls}", f"-DZFVM_MIXED={mixed}", f"-DZFVM_BATCH={batch}"])
    for name, cls in SHAPES.items() for mixed in (0, 1) for batch in (0, 64, 128, 256)
]


def _headers() -> list[Path]:
    return list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "zfvm.h"]


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile every translation unit that changed and link ``libzfvm.so``."""
    if shutil.which(NVCC) is None and not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    BUILD.mkdir(exist_ok=True)
    deps = _headers()
    jobs = []
    objs = []
    for name in HOST_SOURCES:
        src, obj = CSRC / name, BUILD / (name + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append(["g++", *CXXFLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    units = [(name, CSRC / name, []) for name in CUDA_SOURCES]
    units += [(name + ".cu", CSRC / "inst_shape.cu", defs) for name, defs in SHAPE_UNITS]
    for name, src, defs in units:
        obj = BUILD / (name + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append([NVCC, *NVCCFLAGS, *defs, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    if jobs:
        # the slowest units first, so they do not start last
        jobs.sort(key=lambda cmd: (0 if "-DZFVM_BATCH=0" in cmd else 1,
                                   0 if "-DZFVM_SHAPE_NAME=s3o2" in cmd or "-DZFVM_SHAPE_NAME=s3o3" in cmd else 1))
        with ThreadPoolExecutor(max_workers=workers) as ex:
            for cmd, _ in zip(jobs, ex.map(_run, jobs)):
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([NVCC, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose="--verbose" in sys.argv, force="--force" in sys.argv)
    print(LIB)
