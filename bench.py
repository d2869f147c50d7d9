"""Benchmark: cell-stage updates/s of the rate-of-change + SSP-RK step loop.

One cell-stage update is one cell through one RK stage (reconstruction, its
share of the face fluxes, the source and the stage combination); SSP3 makes
three per cell per step.

Default workload (C4, the metric's mixed-batched form): 256 independent
well-balanced polytrope solves (gamma = 2, K = 1, phi = r^2 / 2 on seeded
jittered disks of 5k-200k triangles, perturbation amplitudes 1e-6-1e-2,
CWENO-AO order 3, HLLC, SSP3, CFL 0.45), mixed FP32/FP64, batched into one
persistent launch per phase per RK stage with autotuned launch shapes, next to
the plain FP64 form run one solve at a time on the same instances.  The same
JSON line carries the other workloads as sub-blocks, measured the same way:
  c2   the well-balanced polytrope disk of 199,076 cells, mixed and FP64, its
       run to t = 0.5 and its well-balanced residual
  c3   the 2,058,000-tetrahedron vortex tube, order 3, mixed and FP64
  c5   the serving loop: Poisson arrivals of 2D / 3D solves, p50 / p99
       latency and throughput, mixed and FP64

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c4|c2|c1|c3|c3o2|c5|...] [--precision mixed|fp64]
                  [--no-blocks] [--profile]

value    whole-job cell-stage updates/s of the headline workload, state
         resident in HBM, CUDA events around K graph-replayed steps (max over
         ranks); inputs larger than L2.
e2e      the same metric through the public API with host buffers: every step
         copies the states from pinned host memory to the device, advances one
         CFL step and reads the new states back (C4: Batch.step_host, one host
         round trip for all 256 instances; single meshes: zfvm_step_host).
roofline the dominant kernel (the reconstruction): algorithmic bytes per launch
         / its event-timed launch duration, against the measured HBM copy
         bandwidth; the FP64 form also against its FP64 pipe.
reference (--impl reference) the reference's CPU path (its FP64 restatement,
         the oracle; the reference itself cannot be built) on a sample of the
         same instances, all host cores, from meshes and stencils that build()
         wrote, so the process loads no part of the GPU library.
Multi-GPU: replicas only -- every rank solves its own copy (no data exchange).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

METRIC = "cell-stage updates/s, FP64 vs mixed-batched at ≤1e-6 L1 error; p50/p99 latency"
UNIT = "cell-stage updates/s"
# meshes, stencils and initial states of the reference arm's samples, written
# by build() (write_reference_inputs) and read by --impl reference
REF_INPUTS = ROOT / "oracle" / "_build" / "reference_inputs"
C4_SEED = 2024
# C4 instances the CPU arms time: the ensemble's size quantiles 5, 25, 50, 75 and 95 %
C4_SAMPLE_QUANTILES = (0.05, 0.25, 0.5, 0.75, 0.95)
# FP64 pipe of GB300: 2 DFMA thread-instructions per cycle per SM (ncu's
# sm__sass_thread_inst_executed_op_dfma_pred_on.avg.peak_sustained), 2 flop each
DFMA_PER_CLK_PER_SM = 2.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c4",
                    choices=["c4", "c2", "c1", "c3", "c3o2", "c5", "c2-small", "c1-small", "c3-small", "c4-small",
                             "c5-small"])
    ap.add_argument("--load", type=float, default=0.7, help="c5: offered load as a fraction of throughput")
    ap.add_argument("--budget-gb", type=float, default=24.0, help="c5: device memory budget of the server")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="single-mesh workloads: the form whose throughput is `value` (mixed times FP64 beside it)")
    ap.add_argument("--no-blocks", action="store_true", help="c4: skip the c2 / c3 / c5 sub-blocks")
    ap.add_argument("--profile", action="store_true",
                    help="timed loop only (no CPU baseline, no e2e loop): the command profiled with ncu")
    ap.add_argument("--write-reference-inputs", action="store_true", help=argparse.SUPPRESS)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------------ configs
def c4_config(world: int, n_inst: int = 256) -> dict:
    """The C4 workload as both arms name it."""
    return {"workload": f"C4 batched ensemble of {n_inst} well-balanced polytrope disks", "instances": n_inst,
            "cells_per_instance": "log-uniform 5k-200k", "amplitudes": "log-uniform 1e-6-1e-2", "seed": C4_SEED,
            "precision": "mixed (FP64 beside it)", "batched": True,
            "scheme": "CWENO-AO o3, HLLC, SSP3, CFL 0.45, isentropic well-balancing",
            "parallelism": f"replicas x{world}", "l2": "inputs larger than L2"}


SINGLE_DESC = {
    "c2": {"workload": "C2 well-balanced polytrope disk", "cells": 199076, "gamma": 2.0,
           "scheme": "CWENO-AO o3, HLLC, SSP3, CFL 0.45, isentropic well-balancing"},
    "c2-small": {"workload": "C2 well-balanced polytrope disk (small)"},
    "c1": {"workload": "C1 periodic isentropic vortex", "cells": 51200,
           "scheme": "CWENO-AO o3, Rusanov, SSP3, CFL 0.45"},
    "c1-small": {"workload": "C1 periodic isentropic vortex (small)"},
    "c3": {"workload": "C3 tetrahedral vortex tube", "cells": 2058000, "scheme": "CWENO-AO o3, HLLC, SSP3, CFL 0.3"},
    "c3o2": {"workload": "C3 tetrahedral vortex tube, order 2", "cells": 2058000,
             "scheme": "CWENO-AO o2, HLLC, SSP3, CFL 0.3"},
    "c3-small": {"workload": "C3 tetrahedral vortex tube (small)"},
}


def single_config(name: str, precision: str, world: int) -> dict:
    return {**SINGLE_DESC[name], "precision": precision, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 for c2 / c3 (state, operators and face data > 129 MB)"}


def workload(name: str, precision: str):
    import zisafvm_gb300 as z
    from problems import polytrope_2d, vortex_2d, vortex_tube_3d
    prec = z.MIXED if precision == "mixed" else z.FP64
    if name == "c2":
        raw, mesh, scheme, u0 = polytrope_2d(n_rings=178, amplitude=1e-4)
    elif name == "c2-small":
        raw, mesh, scheme, u0 = polytrope_2d(n_rings=60, amplitude=1e-4)
    elif name == "c1":
        raw, mesh, scheme, u0 = vortex_2d(n=160, halo=3)
    elif name == "c1-small":
        raw, mesh, scheme, u0 = vortex_2d(n=48, halo=3)
    elif name == "c3o2":
        raw, mesh, scheme, u0 = vortex_tube_3d(n=70, order=2)
    elif name == "c3-small":
        raw, mesh, scheme, u0 = vortex_tube_3d(n=24, order=3)
    else:
        raw, mesh, scheme, u0 = vortex_tube_3d(n=70, order=3)
    scheme.precision = prec
    cells = mesh.info["n_interior_cells"] if name.startswith("c1") else mesh.n_cells
    if "cells" in SINGLE_DESC[name]:
        assert cells == SINGLE_DESC[name]["cells"], (name, cells)
    return raw, mesh, scheme, u0, cells


# ------------------------------------------------------------- rooflines
def algorithmic_bytes_per_cell_stage(mesh, scheme, mixed: bool = False) -> int:
    """Compulsory unique HBM traffic of one cell through one stage of the
    reconstruction kernel, from the array sizes the kernel reads and writes.

    FP64 form: stage state (nv words), pseudo-inverse (8-byte words), stencil
    indices, one-sided local indices, geometry (centre, 1/length, moments), face
    ids, face quadrature points (shared by two cells), the face-point values it
    writes and, with well-balancing, the potential and weights at its quadrature
    points and the equilibrium it stores; with gravity the source it writes.
    Mixed form: the pseudo-inverse, moments and scaled quadrature offsets are
    FP32 per cell, the face-point values are written in FP32 beside the FP64
    cell-average deviation (and its FP32 copy), and the gamma = 2 equilibrium
    needs <phi> and var(phi) per cell instead of the quadrature-point arrays
    and is also written as FP32 pairs for the face kernel."""
    nd = mesh.info["n_dims"]
    nv = nd + 2
    nf = nd + 1
    nqf, nqc = mesh.info["n_face_qp"], mesh.info["n_cell_qp"]
    if nd == 2:
        R0, C0, NB, RB, CB = 10, 5, 3, 3, 2
    else:
        R0, C0, NB, RB, CB = 18, 9, 4, 4, 3
    NP = R0 * C0 + NB * RB * CB
    MAXL = R0 + 1 + NB * RB
    NC = max(C0, CB)
    b = nv * 8                      # own state (neighbour states hit L2: SFC order)
    b += MAXL * 4 + NB * RB         # l2g + one-sided local indices
    b += nf * 4                     # face ids
    if not mixed:
        b += NP * 8                     # pseudo-inverse
        b += (nd + 1 + NC) * 8          # centre, 1/length, moments
        b += nf * nqf * nd * 8 / 2      # face quadrature points (shared by two cells)
        b += nf * nqf * nv * 8          # face-point values written
        if scheme.equilibrium:
            b += nqc * 8 * 2 + nqc * nd * 8 * 2 + 3 * 8   # phi, weights, x, grad phi, equilibrium out
            b += nf * nqf * 8 / 2                          # phi at face points
        if scheme.gravity:
            b += nv * 8                                    # source written
    else:
        b += NP * 4                     # pseudo-inverse (FP32)
        b += NC * 4                     # moments (FP32)
        b += nf * nqf * nd * 4          # scaled face-point offsets (FP32, per cell)
        b += nf * nqf * nv * 4 + nv * 8 + nv * 4  # face-point values (FP32), deviation (FP64 and FP32) written
        if scheme.equilibrium:
            b += 3 * 8 + 4 * 8 + 3 * 8  # phi at the reference point, <phi>, var(phi); equilibrium out (FP64, FP32 pairs)
        if scheme.gravity:
            b += nqc * nd * 4 * 2 + nd * 8 + 8 + nv * 4   # offsets, w grad phi, sum, 1/vol, source out
    return int(b)


def _profile_value(key: str, kernel: str, workload_name: str, precision: str):
    """A per-launch figure (DRAM bytes, FP64 flops) of `kernel` from the
    committed ncu summaries (profiles/traffic.txt)."""
    f = ROOT / "profiles" / "traffic.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        kv = dict(x.split("=", 1) for x in line.split() if "=" in x)
        if kv.get("kernel") == kernel and kv.get("workload") == workload_name and kv.get("precision") == precision \
                and key in kv:
            return float(kv[key])
    return None


def measured_peaks() -> dict:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return {"hbm_gbs": float(d.get("hbm_gbs", 6800.0)), "sm_max_mhz": float(d.get("sm_max_mhz", 2070.0)),
                "kind": "measured"}
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0, "kind": "fallback"}


def sm_count() -> int:
    try:
        import torch
        return int(torch.cuda.get_device_properties(0).multi_processor_count)
    except Exception:
        return 152


def fp64_peak_tflops() -> float:
    """FP64 pipe peak: DFMA issue rate x 2 flop x SMs x maximum SM clock."""
    return DFMA_PER_CLK_PER_SM * 2.0 * sm_count() * measured_peaks()["sm_max_mhz"] * 1e6 / 1e12


def roofline_block(mesh, scheme, kt: dict, mixed: bool, workload_name: str, n_cells_launch: int,
                   kernel: str = "k_reconstruct"):
    """HBM roofline of the reconstruction kernel (the dominant launch): the
    algorithmic bytes of one launch over its event-timed duration.  The FP64
    form adds its FP64-pipe roofline: FP64 flops per launch (counted by ncu,
    per cell) over the same duration against the FP64 pipe's peak."""
    b_cell = algorithmic_bytes_per_cell_stage(mesh, scheme, mixed)
    bytes_launch = b_cell * n_cells_launch
    achieved = bytes_launch / (kt["reconstruct"] * 1e-3) / 1e9
    peaks = measured_peaks()
    prec = "mixed" if mixed else "fp64"
    traffic = _profile_value("bytes_per_launch", kernel, workload_name, prec)
    out = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
           "frac": achieved / peaks["hbm_gbs"], "peak_kind": peaks["kind"], "bytes_per_cell_stage": b_cell,
           "bytes_per_launch": bytes_launch, "traffic": traffic, "kernel_ms": kt}
    flops_cell = _profile_value("fp64_flops_per_cell", kernel, workload_name, prec)
    if flops_cell is not None:
        tf = flops_cell * n_cells_launch / (kt["reconstruct"] * 1e-3) / 1e12
        peak = fp64_peak_tflops()
        out["fp64_pipe"] = {"achieved": tf, "peak": peak, "unit": "TFLOP/s", "frac": tf / peak,
                            "flops_per_cell_stage": flops_cell,
                            "peak_from": "2 DFMA/clk/SM x 2 flop x SMs x max SM clock"}
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.samples, self._stop = gpu, [], threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[4 + k].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# -------------------------------------------------- CPU arms (the oracle)
def _oracle_step_rate(problems, threads: int, budget_s: float, min_steps: int = 1):
    """Cell-stage updates/s of the oracle's SSP3 steps over `problems`
    ((raw, stencils, vector, quad, u0, cells) each), one step of every
    problem per round, rounds until the budget is spent."""
    from oracle import pyoracle
    orcs = []
    for raw, st, vec, quad, u0, cells in problems:
        o = pyoracle.Oracle(raw, st, vec, quad=quad, threads=threads)
        orcs.append([o, u0, o.cfl_dt(u0), cells])
    for rec in orcs:  # warm-up round
        rec[1] = rec[0].step(rec[1], rec[2])
    t0 = time.perf_counter()
    rounds = 0
    while rounds < min_steps or time.perf_counter() - t0 < budget_s:
        for rec in orcs:
            rec[1] = rec[0].step(rec[1], rec[2])
        rounds += 1
    el = time.perf_counter() - t0
    cells = sum(rec[3] for rec in orcs)
    return cells * 3 * rounds / el, rounds, cells


def cpu_baseline(problems, label: str, budget_s: float = 12.0, budget_1t_s: float = 6.0) -> dict:
    """The oracle (the FP64 restatement of the reference's OpenMP path) on a
    bounded sample of the workload: every host core, and one thread on the
    sample's smallest problem (when one step of it takes seconds, not minutes)."""
    threads = os.cpu_count() or 1
    rate, rounds, cells = _oracle_step_rate(problems, threads, budget_s)
    out = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{rounds} SSP3 steps of {label} ({cells} cells) with the oracle's OpenMP loops on "
                     f"{threads} threads"}
    smallest = min(problems, key=lambda pr: pr[5])
    if smallest[5] <= 300000:
        rate1, rounds1, cells1 = _oracle_step_rate([smallest], 1, budget_1t_s)
        out["one_thread"] = {"value": rate1, "unit": UNIT, "cores": 1,
                             "sample": f"{rounds1} SSP3 steps of {cells1} cells on one thread"}
    return out


def _problem_of(raw, mesh, scheme, u0, cells):
    return (raw, mesh.stencils(), scheme.oracle_vector(), mesh.quad, u0, cells)


def c4_sample_indices(params) -> list:
    order = sorted(range(len(params)), key=lambda k: params[k]["rings"])
    return sorted({order[min(len(order) - 1, int(q * len(order)))] for q in C4_SAMPLE_QUANTILES})


def write_reference_inputs(out_dir: Path = REF_INPUTS) -> list:
    """Meshes, stencils, scheme vectors and initial states of the CPU arm's
    samples (C4 size quantiles; the C2 disk), written by the product's set-up
    so the reference arm reads them without loading the GPU library."""
    import numpy as np
    from problems import c4_instance, c4_instance_params, polytrope_2d
    out_dir.mkdir(parents=True, exist_ok=True)
    written = []

    def save(name, raw, mesh, scheme, u0, cells):
        st = mesh.stencils()
        width = max(1, int(st["n_l2g"].max()))
        np.savez_compressed(out_dir / f"{name}.npz", n_dims=raw.n_dims, vertices=raw.vertices,
                            vertex_indices=raw.vertex_indices,
                            ghost=raw.ghost if raw.ghost is not None else np.zeros(0, np.uint8),
                            source=raw.source if raw.source is not None else np.zeros(0, np.int64),
                            **{f"st_{k}": (v[:, :width] if k == "l2g" else v) for k, v in st.items()},
                            vector=scheme.oracle_vector(), quad=np.array(mesh.quad), u0=u0, cells=cells)
        written.append(out_dir / f"{name}.npz")

    params = c4_instance_params(256, seed=C4_SEED)
    for k in c4_sample_indices(params):
        raw, mesh, scheme, u0 = c4_instance(params[k])
        save(f"c4_{k:03d}", raw, mesh, scheme, u0, mesh.n_cells)
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=178, amplitude=1e-4)
    save("c2", raw, mesh, scheme, u0, mesh.n_cells)
    return written


def read_reference_inputs(prefix: str, in_dir: Path = REF_INPUTS) -> list:
    import types

    import numpy as np
    out = []
    for f in sorted(in_dir.glob(f"{prefix}*.npz")):
        d = np.load(f)
        raw = types.SimpleNamespace(n_dims=int(d["n_dims"]), vertices=d["vertices"], vertex_indices=d["vertex_indices"],
                                    ghost=d["ghost"] if d["ghost"].size else None,
                                    source=d["source"] if d["source"].size else None)
        st = {k[3:]: d[k] for k in d.files if k.startswith("st_")}
        out.append((raw, st, d["vector"], tuple(int(x) for x in d["quad"]), d["u0"], int(d["cells"])))
    return out


def run_reference(args, rank, world):
    """The reference's CPU implementation of the path (its FP64 restatement,
    the oracle; the reference cannot be built here) on every host core, on a
    bounded sample of the workload: each step is one SSP3 step of every
    sample problem.  The meshes and stencils come from build()'s files, so
    this process loads the oracle only."""
    if rank != 0:
        return
    name = "c4" if args.workload.startswith("c4") else ("c2" if args.workload.startswith("c2") else None)
    problems = read_reference_inputs("c4_" if name == "c4" else "c2") if name else []
    if not problems:
        print(json.dumps({"impl": "reference", "unavailable":
                          f"no reference inputs for {args.workload} under {REF_INPUTS.relative_to(ROOT)} "
                          "(build() writes the c4 and c2 samples)"}), flush=True)
        return
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    orcs = []
    for raw, st, vec, quad, u0, cells in problems:
        o = pyoracle.Oracle(raw, st, vec, quad=quad, threads=threads)
        orcs.append([o, u0, o.cfl_dt(u0), cells])
    for _ in range(args.warmup):
        for rec in orcs:
            rec[1] = rec[0].step(rec[1], rec[2])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for rec in orcs:
            rec[1] = rec[0].step(rec[1], rec[2])
    el = time.perf_counter() - t0
    cells = sum(rec[3] for rec in orcs)
    value = cells * 3 * args.steps / el
    config = c4_config(world) if name == "c4" else single_config("c2", "mixed", world)
    sample = (f"each step: one SSP3 step of each of {len(orcs)} instances ({cells} cells; the ensemble's size "
              f"quantiles {', '.join(str(q) for q in C4_SAMPLE_QUANTILES)}), oracle OpenMP loops on {threads} threads"
              if name == "c4" else f"each step: one SSP3 step of the {cells}-cell disk, oracle OpenMP loops on "
                                   f"{threads} threads")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded meshes and data)",
            "impl": "reference", "config": config,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- GPU arm
def pinned(shape):
    import numpy as np
    try:
        import torch
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        return np.empty(shape)


def e2e_single(solver, mesh, u0, steps, pg):
    """Public-API loop with host buffers (Solver.step_host, zfvm_step_host):
    upload the state from pinned memory, advance one CFL step, read the new
    state back into pinned memory, one call per step."""
    host, host_out = pinned((mesh.n_cells, 5)), pinned((mesh.n_cells, 5))
    solver.set_state(u0)
    solver.advance(n_steps=1)
    state, _ = solver.get_state()
    host[:] = state
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        solver.step_host(host, n_steps=1, out=host_out)
        host, host_out = host_out, host
    return time.perf_counter() - t0


def max_over_ranks(pg, x: float) -> float:
    if not pg:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, x: float) -> float:
    if not pg:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def single_mesh(name, precision, steps, warmup, rank, world, local, pg, profile=False, cpu=True,
                extras=True) -> dict:
    """One mesh: the `precision` form timed over `steps` graph-replayed steps
    (value), its kernels, rooflines and e2e loop; with the mixed form the FP64
    form beside it, the error between them, the well-balanced residual and (C2)
    the run to t = 0.5."""
    import dataclasses

    import zisafvm_gb300 as z
    raw, mesh, scheme, u0, cells = workload(name, precision)
    mixed = precision == "mixed"
    solver = z.Solver(mesh, scheme)
    solver.set_state(u0)
    stages = scheme.rk_stages
    if warmup:
        solver.advance_timed(warmup)
    if pg:
        pg.barrier()
    with ClockSampler(local) as clk:
        ms = solver.advance_timed(steps)
    ms = max_over_ranks(pg, ms)
    value = world * cells * stages * steps / (ms * 1e-3)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": warmup,
           "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32+f64" if mixed else "f64", "data": "synthetic (seeded mesh and initial data)",
           "config": single_config(name, precision, world)}
    if profile:
        out["profile_run"] = True
        return out
    kt = solver.kernel_times(min(steps, 32))
    out["roofline"] = roofline_block(mesh, scheme, kt, mixed, name, mesh.n_cells)
    e2e_steps = max(4, min(steps, 64))
    e2e_s = max_over_ranks(pg, e2e_single(solver, mesh, u0, e2e_steps, pg))
    io_bytes = mesh.n_cells * 5 * 8
    out["e2e"] = {"value": world * cells * stages * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": io_bytes,
                  "d2h_bytes_per_step": io_bytes,
                  "path": "Solver.step_host (zfvm_step_host: upload, one CFL step, download) with pinned host buffers"}
    out["gpu_launches"] = solver.launches_per_step() * steps
    out["clocks"] = clk.summary()
    solver.close()
    if mixed:
        # the plain FP64 form on the same mesh and data, timed the same way
        sch64 = dataclasses.replace(scheme, precision=z.FP64)
        s64 = z.Solver(mesh, sch64)
        s64.set_state(u0)
        if warmup:
            s64.advance_timed(warmup)
        ms64 = max_over_ranks(pg, s64.advance_timed(steps))
        kt64 = s64.kernel_times(min(steps, 32))
        out["fp64"] = {"value": world * cells * stages * steps / (ms64 * 1e-3), "ms_per_step": ms64 / steps,
                       "roofline": roofline_block(mesh, sch64, kt64, False, name, mesh.n_cells)}
        out["mixed_over_fp64"] = value / out["fp64"]["value"]
        if extras:
            # error of the mixed form against the FP64 form after the same steps
            from metrics import perturbation_rel_l1, state_rel_l1
            s64.set_state(u0)
            s32 = z.Solver(mesh, scheme)
            s32.set_state(u0)
            n_cmp = min(max(steps, 20), 100)
            s64.advance(n_steps=n_cmp)
            s32.advance(n_steps=n_cmp)
            u64, _ = s64.get_state()
            u32, _ = s32.get_state()
            s32.close()
            mask = raw.ghost == 0 if raw.ghost is not None else None
            out["error_vs_fp64"] = {"steps": n_cmp, "state_rel_l1": state_rel_l1(u32, u64, mask),
                                    "perturbation_rel_l1": perturbation_rel_l1(u32, u64, u0, mask)}
            if scheme.equilibrium:
                out["well_balanced"] = well_balanced_residual(z, mesh, scheme, n_cmp)
            if name == "c2":
                out["run_to_t_end"] = run_to_t_end(z, mesh, scheme, u0, 0.5)
        s64.close()
    if cpu and rank == 0:
        try:
            out["cpu_baseline"] = cpu_baseline([_problem_of(raw, mesh, scheme, u0, cells)],
                                               f"the full {SINGLE_DESC[name]['workload']} mesh", budget_s=8.0,
                                               budget_1t_s=4.0)
        except Exception as exc:  # the baseline must not hide the GPU number
            out["cpu_baseline"] = {"error": str(exc)}
    return out


def run_to_t_end(z, mesh, scheme, u0, t_end: float) -> dict:
    """The C2 run as specified: both forms from the same data to t_end with CFL
    time steps (device-resident clock, graph replay), wall time of each, and
    the mixed form's error against the FP64 form at t_end."""
    import dataclasses
    from metrics import perturbation_rel_l1, state_rel_l1
    out = {"t_end": t_end}
    states = {}
    for label, prec in (("mixed", z.MIXED), ("fp64", z.FP64)):
        s = z.Solver(mesh, dataclasses.replace(scheme, precision=prec))
        s.set_state(u0)
        t0 = time.perf_counter()
        t, n = s.advance(t_end=t_end)
        wall = time.perf_counter() - t0
        states[label], _ = s.get_state()
        out[label] = {"t": t, "steps": n, "wall_s": wall,
                      "cell_stage_updates_per_s": mesh.n_cells * scheme.rk_stages * n / wall}
        s.close()
    out["error_vs_fp64"] = {"state_rel_l1": state_rel_l1(states["mixed"], states["fp64"]),
                            "perturbation_rel_l1": perturbation_rel_l1(states["mixed"], states["fp64"], u0)}
    return out


def well_balanced_residual(z, mesh, scheme, steps: int) -> dict:
    """max |du/dt| of the unperturbed equilibrium and its relative drift after
    `steps` steps (rho and E), in the given form."""
    import numpy as np
    u_eq = mesh.initial_conditions("polytrope", gamma=2.0, K=1.0, rho_c=1.0, k_phi=1.0, amplitude=0.0)
    s_eq = z.Solver(mesh, scheme)
    s_eq.set_state(u_eq)
    res = float(np.abs(s_eq.rate_of_change()).max())
    s_eq.advance(n_steps=steps)
    u_end, _ = s_eq.get_state()
    s_eq.close()
    cols = [0, 4]  # rho and E (the momenta of the equilibrium are zero)
    drift = float((np.abs(u_end - u_eq)[:, cols].max(axis=0) / np.abs(u_eq)[:, cols].max(axis=0)).max())
    return {"max_abs_dudt": res, "rel_drift": drift, "steps": steps}


def run_ensemble(args, rank, world, local, pg) -> dict:
    """C4: 256 independent well-balanced polytrope solves of uneven size in one
    batch (mixed form, one persistent launch per phase per RK stage, launch
    shapes picked by the autotuner), against the plain FP64 form run one solve
    at a time on the same instances."""
    import dataclasses

    import numpy as np
    import zisafvm_gb300 as z
    from metrics import perturbation_rel_l1, state_rel_l1
    from problems import c4_instance, c4_instance_params
    small = args.workload == "c4-small"
    n_inst = 16 if small else 256
    t_setup = time.perf_counter()
    params = c4_instance_params(n_inst, n_max=40000 if small else 200000, seed=C4_SEED + 7919 * rank)
    inst = [c4_instance(p) for p in params]
    t_setup = time.perf_counter() - t_setup
    total_cells = sum(m.n_cells for _, m, _, _ in inst)
    stages = 3
    batch = z.Batch(n_inst)
    solvers, slots = [], []
    for raw, mesh, scheme, u0 in inst:
        s = z.Solver(mesh, scheme)
        s.set_state(u0)
        slots.append(batch.add(s, n_steps=1 << 40))
        solvers.append(s)
    t_tune = time.perf_counter()
    batch.autotune(trial_steps=4)
    t_tune = time.perf_counter() - t_tune
    if args.warmup:
        batch.advance_timed(args.warmup)
    if pg:
        pg.barrier()
    with ClockSampler(local) as clk:
        ms = batch.advance_timed(args.steps)
    ms = max_over_ranks(pg, ms)
    value = world * total_cells * stages * args.steps / (ms * 1e-3)
    config = c4_config(world, n_inst)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded meshes and data)", "config": config}
    if args.profile:
        line["profile_run"] = True
        return line
    sizes = sorted(m.n_cells for _, m, _, _ in inst)
    kt = batch.kernel_times(min(args.steps, 16))
    roof = roofline_block(inst[0][1], inst[0][2], kt, True, args.workload, total_cells, kernel="km_reconstruct")
    tuned = batch.tuned_shapes() if hasattr(batch, "tuned_shapes") else None

    # end to end: every step uploads all states from pinned host memory, advances
    # the batch one step and reads every state back (Batch.step_host: one host
    # round trip for the whole batch)
    hosts = {slot: pinned((m.n_cells, 5)) for slot, (_, m, _, _) in zip(slots, inst)}
    for slot, s in zip(slots, solvers):
        s.get_state(out=hosts[slot])
    e2e_steps = max(3, min(args.steps, 16))
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        batch.step_host(hosts, hosts, 1)
    e2e_s = max_over_ranks(pg, time.perf_counter() - t0)
    io_bytes = total_cells * 5 * 8
    launches = 1 + stages * 3   # clock + three persistent kernels per stage, one group
    batch.close()
    for s in solvers:
        s.close()
    del solvers, hosts

    # plain FP64 form, one solve at a time, same steps per instance
    k64 = max(3, min(args.steps, 24))
    ms64 = 0.0
    for raw, mesh, scheme, u0 in inst:
        s64 = z.Solver(mesh, dataclasses.replace(scheme, precision=z.FP64))
        s64.set_state(u0)
        s64.advance_timed(3)
        ms64 += s64.advance_timed(k64)
        s64.close()
    ms64 = max_over_ranks(pg, ms64)
    v64 = world * total_cells * stages * k64 / (ms64 * 1e-3)

    # accuracy of the mixed batched form against FP64 on a sample of instances
    # (among them the ends of the amplitude range)
    amps = np.array([p["amplitude"] for p in params])
    pick = sorted({int(j) for j in np.linspace(0, n_inst - 1, 6).astype(int)} | {int(amps.argmin()), int(amps.argmax())})
    n_cmp = 50
    b2 = z.Batch(len(pick))
    pairs = []
    for j in pick:
        raw, mesh, scheme, u0 = inst[j]
        s32 = z.Solver(mesh, scheme)
        s32.set_state(u0)
        b2.add(s32, n_steps=n_cmp)
        s64 = z.Solver(mesh, dataclasses.replace(scheme, precision=z.FP64))
        s64.set_state(u0)
        s64.advance(n_steps=n_cmp)
        pairs.append((s32, s64, u0, params[j]["amplitude"]))
    while b2.advance(8):
        pass
    errs = []
    for s32, s64, u0, amp in pairs:
        u32, _ = s32.get_state()
        u64, _ = s64.get_state()
        errs.append((state_rel_l1(u32, u64, None), perturbation_rel_l1(u32, u64, u0, None), amp))
        s64.close()
    b2.close()
    wb = well_balanced_residual(z, inst[0][1], inst[0][2], n_cmp)

    line.update({
        "cells_total": total_cells, "cells_min": sizes[0], "cells_median": sizes[len(sizes) // 2],
        "cells_max": sizes[-1], "setup_s": t_setup, "autotune_s": t_tune, "launch_shapes": tuned,
        "e2e": {"value": world * total_cells * stages * e2e_steps / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": io_bytes, "d2h_bytes_per_step": io_bytes,
                "path": "Batch.step_host: every slot's state in from pinned host memory, one batched step, "
                        "every state out, one host synchronisation"},
        "roofline": roof, "gpu_launches": launches * args.steps, "clocks": clk.summary(),
        "fp64": {"value": v64, "ms_per_step": ms64 / k64, "form": "plain FP64, one solve at a time",
                 "steps_per_instance": k64},
        "mixed_batched_over_fp64": value / v64,
        "error_vs_fp64": {"instances": len(errs), "steps": n_cmp,
                          "state_rel_l1_max": max(e[0] for e in errs),
                          "perturbation_rel_l1_max": max(e[1] for e in errs),
                          "perturbation_rel_l1_at_amplitude": {f"{e[2]:.2e}": e[1] for e in errs}},
        "well_balanced": wb,
    })
    if rank == 0:
        try:
            sample = [_problem_of(*inst[k], inst[k][1].n_cells) for k in c4_sample_indices(params)]
            line["cpu_baseline"] = cpu_baseline(sample, f"{len(sample)} ensemble instances (size quantiles)")
        except Exception as exc:
            line["cpu_baseline"] = {"error": str(exc)}
    return line


def serving_requests(n_req: int, seed: int, small: bool):
    """C5 request stream: 70% 2D triangle meshes (2k-500k cells, log-uniform;
    a gamma = 2 well-balanced polytrope disk or a gamma = 1.4 periodic vortex),
    30% 3D tetrahedral meshes (50k-2M cells; gamma = 2 well-balanced
    polytrope on the unit cube), seeded perturbation amplitudes 1e-6-1e-2, end
    times U[0.05, 0.5].  Meshes come from a seeded pool (built before the
    arrivals start; set-up is reported apart from latency).  The 3D vortex
    tube of the C3 benchmark is not used here: with the constant flux
    boundary its inflow faces amplify perturbations over hundreds of steps."""
    import numpy as np
    import zisafvm_gb300 as z
    from problems import polytrope_2d, polytrope_3d, vortex_2d
    rng = np.random.default_rng(seed)
    lo2, hi2, lo3, hi3 = (2000, 60000, 20000, 120000) if small else (2000, 500000, 50000, 2000000)

    def logu(lo, hi):
        return float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
    pool = {"disk": [], "square": [], "cube": []}
    for _ in range(3):
        pool["disk"].append(polytrope_2d(n_rings=max(8, int(round(np.sqrt(logu(lo2, hi2) / (2 * np.pi))))),
                                         amplitude=1e-4, seed=int(rng.integers(1 << 30))))
        pool["square"].append(vortex_2d(n=max(12, int(round(np.sqrt(logu(lo2, hi2) / 2)))), halo=3,
                                        flux=z.FLUX_HLLC))
        pool["cube"].append(polytrope_3d(n=max(6, int(round((logu(lo3, hi3) / 6) ** (1 / 3)))),
                                         seed=int(rng.integers(1 << 30))))
    reqs = []
    for _ in range(n_req):
        u = rng.uniform()
        kind = "cube" if u < 0.3 else ("disk" if u < 0.65 else "square")
        raw, mesh, scheme, _ = pool[kind][int(rng.integers(3))]
        amp = float(np.exp(rng.uniform(np.log(1e-6), np.log(1e-2))))
        t_end = float(rng.uniform(0.05, 0.5))
        if kind == "disk":
            r0, ang = float(rng.uniform(0.1, 0.7)), float(rng.uniform(0, 2 * np.pi))
            u0 = mesh.initial_conditions("polytrope", gamma=2.0, K=1.0, rho_c=1.0, k_phi=1.0, amplitude=amp,
                                         width=0.05, x0=r0 * np.cos(ang), y0=r0 * np.sin(ang))
        elif kind == "cube":
            x0, y0 = float(rng.uniform(0.2, 0.8)), float(rng.uniform(0.2, 0.8))
            u0 = mesh.initial_conditions("polytrope", gamma=2.0, K=1.0, rho_c=1.0, k_phi=1.0, amplitude=amp,
                                         width=0.05, x0=x0, y0=y0)
        else:
            # vortex strength scaled by the amplitude draw: beta in [0.5, 5]
            beta = 0.5 + 4.5 * (np.log10(amp) + 6.0) / 4.0
            x0, y0 = float(rng.uniform(0.3, 0.7)), float(rng.uniform(0.3, 0.7))
            u0 = mesh.initial_conditions("vortex", gamma=1.4, beta=beta, x0=x0, y0=y0, length=0.1)
        reqs.append({"kind": kind, "mesh": mesh, "scheme": scheme, "u0": u0, "t_end": t_end, "amp": amp})
    return pool, reqs


def serve_stream(z, reqs, arrivals, precision, budget, max_slots, steps_per_round):
    """Submit every request at its arrival time from a client thread, wait for
    all, and return per-request latencies and the server statistics."""
    import dataclasses
    srv = z.Server(hbm_budget_bytes=budget, max_slots=max_slots, steps_per_round=steps_per_round)
    ids = [None] * len(reqs)
    t_start = time.perf_counter()

    def client():
        for k, r in enumerate(reqs):
            delay = t_start + arrivals[k] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            sc = dataclasses.replace(r["scheme"], precision=precision)
            ids[k] = srv.submit(r["mesh"], sc, r["u0"], t_end=r["t_end"])

    th = threading.Thread(target=client)
    th.start()
    th.join()
    out = [srv.wait(rid) for rid in ids]
    makespan = time.perf_counter() - t_start
    st = srv.stats()
    srv.close()
    return out, st, makespan


def percentile(xs, q):
    import numpy as np
    return float(np.percentile(np.asarray(xs), q)) if xs else None


def run_serving(args, rank, world, local, pg, small: bool) -> dict:
    """C5: Poisson arrivals of uneven 2D / 3D solves, admitted by device
    footprint and batched continuously; mixed form (value) next to the plain
    FP64 form serving the same stream."""
    import numpy as np
    import zisafvm_gb300 as z
    n_req = 12 if small else 32
    t0 = time.perf_counter()
    pool, reqs = serving_requests(n_req, seed=77 + 7919 * rank, small=small)
    setup_s = time.perf_counter() - t0
    # expected work per request from the CFL step of its initial state
    work = []
    for r in reqs:
        s = z.Solver(r["mesh"], r["scheme"])
        s.set_state(r["u0"])
        dt = s.cfl_dt()
        s.close()
        steps = int(np.ceil(r["t_end"] / dt))
        work.append(r["mesh"].n_cells * 3 * steps)
    # offered load: args.load of the mixed form's sustained throughput (~7e8 /s)
    rate = args.load * 7.0e8 / float(np.mean(work))
    rng = np.random.default_rng(1234 + rank)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n_req))
    arrivals -= arrivals[0]
    budget = int(args.budget_gb * (1 << 30))
    if pg:
        pg.barrier()
    with ClockSampler(local) as clk:
        res, st, makespan = serve_stream(z, reqs, arrivals, z.MIXED, budget, 64, 8)
    lat = [r[3]["total"] for r in res]
    queued = [r[3]["queued"] for r in res]
    work_all = sum_over_ranks(pg, float(st["cell_stage_updates"]))
    value = work_all / max_over_ranks(pg, makespan)
    res64, st64, makespan64 = serve_stream(z, reqs, arrivals, z.FP64, budget, 64, 8)
    lat64 = [r[3]["total"] for r in res64]
    # result of each request: mixed against FP64 (perturbation-level agreement)
    from metrics import state_rel_l1
    errs = [state_rel_l1(a[0], b[0], None) for a, b in zip(res, res64)]
    err_by_kind = {k: max([e for e, r in zip(errs, reqs) if r["kind"] == k], default=None)
                   for k in ("disk", "square", "cube")}
    io_in = sum(r["mesh"].n_cells * 5 * 8 for r in reqs)
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": None, "warmup": 0,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic (seeded meshes, data and arrivals)",
        "config": {"workload": "C5 serving loop" + (" (small)" if small else ""), "requests": n_req,
                   "mix": {k: sum(r["kind"] == k for r in reqs) for k in ("disk", "square", "cube")},
                   "cells_per_request": [int(r["mesh"].n_cells) for r in reqs],
                   "t_end": [round(r["t_end"], 4) for r in reqs],
                   "arrival_rate_per_s": rate, "offered_load": args.load, "budget_bytes": budget,
                   "max_slots": 64, "steps_per_round": 8, "mesh_setup_s": setup_s,
                   "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": percentile(lat, 50), "p99": percentile(lat, 99), "mean": float(np.mean(lat)),
                       "queued_p50": percentile(queued, 50), "queued_p99": percentile(queued, 99)},
        "server": {"completed": st["completed"], "failed": st["failed"], "bytes_peak": st["bytes_peak"],
                   "busy_s": st["busy_s"], "setup_s": st["setup_s"], "makespan_s": makespan, "rounds": st["rounds"],
                   "throughput_while_busy": st["cell_stage_updates"] / max(st["busy_s"], 1e-9)},
        "fp64": {"value": st64["cell_stage_updates"] / makespan64,
                 "latency_ms": {"p50": percentile(lat64, 50), "p99": percentile(lat64, 99)},
                 "makespan_s": makespan64, "completed": st64["completed"], "failed": st64["failed"]},
        "error_vs_fp64": {"state_rel_l1_max": max(errs) if errs else None, "by_kind": err_by_kind},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": io_in, "d2h_bytes_per_step": io_in,
                "path": "Server.submit / wait with host states (bytes per stream, not per step)"},
        "clocks": clk.summary(),
    }


BLOCK_DROP = ("metric", "unit", "n_gpus", "higher_is_better", "scaling", "vs_baseline", "data")


def _block(d: dict) -> dict:
    """A workload's result as a sub-block of the headline line."""
    return {k: v for k, v in d.items() if k not in BLOCK_DROP}


def main():
    args = parse()
    if args.write_reference_inputs:
        for f in write_reference_inputs():
            print(f.relative_to(ROOT))
        return
    rank, world, local = dist_env()
    if world > 1:
        # replicas only: one GPU per process, no collective on the data path
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload.startswith("c4"):
        line = run_ensemble(args, rank, world, local, pg)
        # the other workloads as sub-blocks (one GPU: the scaling runs keep the headline only)
        if not args.profile and not args.no_blocks and world == 1 and args.workload == "c4":
            blocks = {}
            for name in ("c2", "c3"):
                blocks[name] = _block(single_mesh(name, "mixed", args.steps, args.warmup, rank, world, local, pg,
                                                  cpu=False))
            blocks["c5"] = _block(run_serving(args, rank, world, local, pg, small=False))
            line.update(blocks)
        if rank == 0:
            print(json.dumps(line), flush=True)
    elif args.workload.startswith("c5"):
        line = run_serving(args, rank, world, local, pg, small=args.workload == "c5-small")
        line["roofline"], line["gpu_launches"] = None, None
        if rank == 0:
            print(json.dumps(line), flush=True)
    else:
        line = single_mesh(args.workload, args.precision, args.steps, args.warmup, rank, world, local, pg,
                           profile=args.profile)
        if rank == 0:
            print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()


if __name__ == "__main__":
    main()
