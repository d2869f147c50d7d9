"""Benchmark: cell-stage updates/s of the rate-of-change + SSP-RK step loop.

Default workload (C2): the well-balanced 2D polytrope (gamma = 2, K = 1,
phi = r^2 / 2 on the unit disk, ~200k jittered Delaunay triangles, CWENO-AO
order 3, HLLC, SSP3, CFL 0.45, perturbation 1e-4), seeded synthetic data.  One
"step" is one SSP3 time step over the whole mesh: 3 cell-stage updates per cell.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c2|c1|c3|c3o2|c4|...] [--precision mixed|fp64]

value    whole-job cell-stage updates/s of the --precision form (default: the
         mixed FP32/FP64 form), state resident in HBM, CUDA events on the
         solver stream around K graph-replayed steps (max over ranks).  With
         the mixed form the plain FP64 form is timed the same way on the same
         mesh ("fp64"), and the mixed form's error against it and its
         well-balanced residual are reported.
c4       256 solves of uneven size batched into one persistent launch per
         phase per RK stage (autotuned grids), against the FP64 form run one
         solve at a time on the same instances.
e2e      the same metric through the public API with host buffers: every step
         copies the state from pinned host memory to the device, advances one
         CFL step and reads the new state back.
roofline dominant kernel (the reconstruction kernel): algorithmic bytes per
         launch / its event-timed launch duration, against the measured HBM
         copy bandwidth; the FP64 pipe bounds these kernels first.
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

FP64_PEAK_TFLOPS = 1.254  # FMA-chain probe on this machine's GB300 (2 flop / DFMA)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=160)
    ap.add_argument("--warmup", type=int, default=16)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2",
                    choices=["c2", "c1", "c3", "c3o2", "c4", "c5", "c2-small", "c1-small", "c3-small", "c4-small",
                             "c5-small"])
    ap.add_argument("--load", type=float, default=0.7, help="c5: offered load as a fraction of throughput")
    ap.add_argument("--budget-gb", type=float, default=24.0, help="c5: device memory budget of the server")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="form whose throughput is `value`; with mixed the FP64 form is timed beside it")
    ap.add_argument("--profile", action="store_true",
                    help="timed loop only (no CPU baseline, no e2e loop): the command profiled with ncu")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(name: str, precision: str):
    import zisafvm_gb300 as z
    from problems import polytrope_2d, vortex_2d, vortex_tube_3d
    prec = z.MIXED if precision == "mixed" else z.FP64
    if name == "c2":
        raw, mesh, scheme, u0 = polytrope_2d(n_rings=178, amplitude=1e-4)
        desc = {"workload": "C2 well-balanced polytrope disk", "cells": mesh.n_cells, "gamma": 2.0,
                "scheme": "CWENO-AO o3, HLLC, SSP3, CFL 0.45, isentropic well-balancing"}
    elif name == "c2-small":
        raw, mesh, scheme, u0 = polytrope_2d(n_rings=60, amplitude=1e-4)
        desc = {"workload": "C2 well-balanced polytrope disk (small)", "cells": mesh.n_cells}
    elif name == "c1":
        raw, mesh, scheme, u0 = vortex_2d(n=160, halo=3)
        desc = {"workload": "C1 periodic isentropic vortex", "cells": mesh.info["n_interior_cells"],
                "scheme": "CWENO-AO o3, Rusanov, SSP3, CFL 0.45"}
    elif name == "c1-small":
        raw, mesh, scheme, u0 = vortex_2d(n=48, halo=3)
        desc = {"workload": "C1 periodic isentropic vortex (small)", "cells": mesh.info["n_interior_cells"]}
    elif name == "c3o2":
        raw, mesh, scheme, u0 = vortex_tube_3d(n=70, order=2)
        desc = {"workload": "C3 tetrahedral vortex tube, order 2", "cells": mesh.n_cells,
                "scheme": "CWENO-AO o2, HLLC, SSP3, CFL 0.3"}
    elif name == "c3-small":
        raw, mesh, scheme, u0 = vortex_tube_3d(n=24, order=3)
        desc = {"workload": "C3 tetrahedral vortex tube (small)", "cells": mesh.n_cells}
    else:
        raw, mesh, scheme, u0 = vortex_tube_3d(n=70, order=3)
        desc = {"workload": "C3 tetrahedral vortex tube", "cells": mesh.n_cells,
                "scheme": "CWENO-AO o3, HLLC, SSP3, CFL 0.3"}
    scheme.precision = prec
    return raw, mesh, scheme, u0, desc


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


def profiles_traffic(kernel: str, workload_name: str, precision: str):
    """DRAM traffic per launch of `kernel` from the committed ncu summary."""
    f = ROOT / "profiles" / "traffic.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        kv = dict(x.split("=", 1) for x in line.split() if "=" in x)
        if kv.get("kernel") == kernel and kv.get("workload") == workload_name and kv.get("precision") == precision:
            return float(kv["bytes_per_launch"])
    return None


def measured_peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def cpu_baseline(raw, mesh, scheme, u0, desc, budget_s=20.0):
    """The oracle (C++ restatement of the reference's OpenMP path) on a bounded
    sample: whole RK steps of the full workload on all host cores."""
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    o = pyoracle.Oracle(raw, mesh.stencils(), scheme.oracle_vector(), quad=mesh.quad, threads=threads)
    dt = o.cfl_dt(u0)
    t0 = time.perf_counter()
    u = o.step(u0, dt)
    one = time.perf_counter() - t0
    n = max(1, min(20, int(budget_s / max(one, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(n):
        u = o.step(u, dt)
    el = time.perf_counter() - t0
    cells = desc["cells"]
    return {"value": cells * scheme.rk_stages * n / el, "unit": "cell-stage updates/s", "cores": threads,
            "kind": "port", "sample": f"{n} SSP3 steps of the full {desc['workload']} mesh ({cells} cells) "
                                      f"with the oracle's OpenMP loops on {threads} threads"}


def reference_sample(workload_name: str):
    """A bounded sample of the workload for the CPU arm: the same scheme on a
    smaller mesh of the same family."""
    from problems import polytrope_2d, vortex_2d, vortex_tube_3d
    if workload_name.startswith("c1"):
        raw, mesh, scheme, u0 = vortex_2d(n=48, halo=3)
        return raw, mesh, scheme, u0, mesh.info["n_interior_cells"], "C1 periodic isentropic vortex"
    if workload_name.startswith("c3"):
        raw, mesh, scheme, u0 = vortex_tube_3d(n=12, order=2 if workload_name == "c3o2" else 3)
        return raw, mesh, scheme, u0, mesh.n_cells, "C3 tetrahedral vortex tube"
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=60, amplitude=1e-4)
    name = {"c4": "C4 polytrope ensemble", "c5": "C5 serving request (polytrope disk)"}.get(
        workload_name[:2], "C2 well-balanced polytrope disk")
    return raw, mesh, scheme, u0, mesh.n_cells, name


def run_reference(args, rank, world):
    """The reference's CPU implementation of the path (its oracle restatement;
    the reference cannot be built here) timed on the host cores."""
    if rank != 0:
        return
    from oracle import pyoracle
    raw, mesh, scheme, u0, cells, wl = reference_sample(args.workload)
    threads = os.cpu_count() or 1
    o = pyoracle.Oracle(raw, mesh.stencils(), scheme.oracle_vector(), quad=mesh.quad, threads=threads)
    dt = o.cfl_dt(u0)
    u = u0
    for _ in range(args.warmup):
        u = o.step(u, dt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        u = o.step(u, dt)
    el = time.perf_counter() - t0
    value = cells * 3 * args.steps / el
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": wl, "cells_per_step_sample": cells, "precision": "fp64"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"each step: one SSP3 step of a {cells}-cell mesh of the same workload "
                                       f"family, oracle OpenMP loops on {threads} threads"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


METRIC = "cell-stage updates/s, FP64 vs mixed-batched at \u22641e-6 L1 error; p50/p99 latency"
UNIT = "cell-stage updates/s"


def roofline_block(mesh, scheme, kt: dict, mixed: bool, workload_name: str, n_cells_launch: int,
                   kernel: str = "k_reconstruct"):
    """HBM roofline of the reconstruction kernel (the dominant launch): the
    algorithmic bytes of one launch over its event-timed duration."""
    b_cell = algorithmic_bytes_per_cell_stage(mesh, scheme, mixed)
    bytes_launch = b_cell * n_cells_launch
    achieved = bytes_launch / (kt["reconstruct"] * 1e-3) / 1e9
    hbm, peak_kind = measured_peaks()
    traffic = profiles_traffic(kernel, workload_name, "mixed" if mixed else "fp64")
    return {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_kind": peak_kind, "bytes_per_cell_stage": b_cell,
            "bytes_per_launch": bytes_launch, "traffic": traffic, "kernel_ms": kt,
            "fp64_pipe_note": "the FP64 pipe (1.25 TFLOP/s measured) bounds these kernels before HBM does"}


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


def run_single_mesh(args, rank, world, local, pg):
    import dataclasses

    import numpy as np
    import zisafvm_gb300 as z
    raw, mesh, scheme, u0, desc = workload(args.workload, args.precision)
    mixed = args.precision == "mixed"
    solver = z.Solver(mesh, scheme)
    solver.set_state(u0)
    cells = desc["cells"]
    stages = scheme.rk_stages

    # warm-up, then K graph-replayed steps timed with CUDA events
    if args.warmup:
        solver.advance_timed(args.warmup)
    if pg:
        pg.barrier()
    with ClockSampler(local) as clk:
        ms = solver.advance_timed(args.steps)
    ms = max_over_ranks(pg, ms)
    value = world * cells * stages * args.steps / (ms * 1e-3)

    if args.profile:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "ms_per_step": ms / args.steps,
                              "config": desc, "profile_run": True}), flush=True)
        return

    kt = solver.kernel_times(min(args.steps, 32))
    roof = roofline_block(mesh, scheme, kt, mixed, args.workload, mesh.n_cells)
    e2e_steps = max(4, min(args.steps, 64))
    e2e_s = max_over_ranks(pg, e2e_single(solver, mesh, u0, e2e_steps, pg))
    e2e_value = world * cells * stages * e2e_steps / e2e_s
    io_bytes = mesh.n_cells * 5 * 8

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64",
        "data": "synthetic (seeded mesh and initial data)",
        "config": {**desc, "precision": args.precision, "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 for c2/c3 (state, operators and face data > 129 MB)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": io_bytes, "d2h_bytes_per_step": io_bytes,
                "path": "Solver.step_host (zfvm_step_host: upload, one CFL step, download) with pinned host buffers"},
        "roofline": roof,
        "gpu_launches": solver.launches_per_step() * args.steps,
        "clocks": clk.summary(),
    }
    if mixed:
        # the plain FP64 form on the same mesh and data, timed the same way
        s64 = z.Solver(mesh, dataclasses.replace(scheme, precision=z.FP64))
        s64.set_state(u0)
        if args.warmup:
            s64.advance_timed(args.warmup)
        ms64 = max_over_ranks(pg, s64.advance_timed(args.steps))
        v64 = world * cells * stages * args.steps / (ms64 * 1e-3)
        kt64 = s64.kernel_times(min(args.steps, 32))
        line["fp64"] = {"value": v64, "ms_per_step": ms64 / args.steps,
                        "roofline": roofline_block(mesh, dataclasses.replace(scheme, precision=z.FP64), kt64,
                                                   False, args.workload, mesh.n_cells)}
        line["mixed_over_fp64"] = value / v64
        # error of the mixed form against the FP64 form after the same steps
        from metrics import perturbation_rel_l1, state_rel_l1
        s64.set_state(u0)
        s32 = z.Solver(mesh, scheme)
        s32.set_state(u0)
        n_cmp = min(args.steps, 100)
        s64.advance(n_steps=n_cmp)
        s32.advance(n_steps=n_cmp)
        u64, _ = s64.get_state()
        u32, _ = s32.get_state()
        mask = raw.ghost == 0 if raw.ghost is not None else None
        line["error_vs_fp64"] = {"steps": n_cmp, "state_rel_l1": state_rel_l1(u32, u64, mask),
                                 "perturbation_rel_l1": perturbation_rel_l1(u32, u64, u0, mask)}
        if scheme.equilibrium:
            line["well_balanced"] = well_balanced_residual(z, mesh, scheme, n_cmp)
        if args.workload == "c2":
            line["run_to_t_end"] = run_to_t_end(z, mesh, scheme, u0, 0.5)
    if rank == 0:
        try:
            line["cpu_baseline"] = cpu_baseline(raw, mesh, scheme, u0, desc)
        except Exception as exc:  # the baseline must not hide the GPU number
            line["cpu_baseline"] = {"error": str(exc)}
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()


def run_to_t_end(z, mesh, scheme, u0, t_end: float) -> dict:
    """The C2 run as specified: both forms from the same data to t_end with CFL
    time steps (device-resident clock, graph replay), wall time of each, and
    the mixed form's error against the FP64 form at t_end."""
    import dataclasses
    from metrics import perturbation_rel_l1, state_rel_l1
    out = {"t_end": t_end}
    states = {}
    for name, prec in (("mixed", z.MIXED), ("fp64", z.FP64)):
        s = z.Solver(mesh, dataclasses.replace(scheme, precision=prec))
        s.set_state(u0)
        t0 = time.perf_counter()
        t, n = s.advance(t_end=t_end)
        wall = time.perf_counter() - t0
        states[name], _ = s.get_state()
        out[name] = {"t": t, "steps": n, "wall_s": wall,
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
    cols = [0, 4]  # rho and E (the momenta of the equilibrium are zero)
    drift = float((np.abs(u_end - u_eq)[:, cols].max(axis=0) / np.abs(u_eq)[:, cols].max(axis=0)).max())
    return {"max_abs_dudt": res, "rel_drift": drift, "steps": steps}


def run_ensemble(args, rank, world, local, pg):
    """C4: 256 independent well-balanced polytrope solves of uneven size in one
    batch (mixed form, one persistent launch per phase per RK stage, grids
    picked by the autotuner), against the plain FP64 form run one solve at a
    time on the same instances."""
    import dataclasses

    import numpy as np
    import zisafvm_gb300 as z
    from metrics import perturbation_rel_l1, state_rel_l1
    from problems import ensemble_c4
    n_inst = 256 if args.workload == "c4" else 16
    t_setup = time.perf_counter()
    inst = ensemble_c4(n_inst, n_max=200000 if args.workload == "c4" else 40000, seed=2024 + 7919 * rank)
    t_setup = time.perf_counter() - t_setup
    total_cells = sum(m.n_cells for _, m, _, _ in inst)
    stages = 3
    batch = z.Batch(n_inst)
    solvers = []
    for raw, mesh, scheme, u0 in inst:
        s = z.Solver(mesh, scheme)
        s.set_state(u0)
        batch.add(s, n_steps=1 << 40)
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
    if args.profile:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "ms_per_step": ms / args.steps,
                              "config": {"workload": "C4", "instances": n_inst}, "profile_run": True}), flush=True)
        return
    kt = batch.kernel_times(min(args.steps, 16))
    roof = roofline_block(inst[0][1], inst[0][2], kt, True, args.workload, total_cells, kernel="km_reconstruct")

    # end to end: every step uploads all states from pinned host memory, advances
    # the batch one step and reads every state back
    hosts = [pinned((m.n_cells, 5)) for _, m, _, _ in inst]
    for h, s in zip(hosts, solvers):
        s.get_state(out=h)
    e2e_steps = max(3, min(args.steps, 16))
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for h, s in zip(hosts, solvers):
            s.set_state(h)
        batch.advance(1)
        for h, s in zip(hosts, solvers):
            s.get_state(out=h)
    e2e_s = max_over_ranks(pg, time.perf_counter() - t0)
    e2e_value = world * total_cells * stages * e2e_steps / e2e_s
    io_bytes = total_cells * 5 * 8
    launches = 1 + stages * 3   # clock + three persistent kernels per stage, one group
    batch.close()
    del solvers

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
    errs = []
    sample = [inst[j] for j in np.linspace(0, n_inst - 1, 6).astype(int)]
    n_cmp = 50
    b2 = z.Batch(len(sample))
    pairs = []
    for raw, mesh, scheme, u0 in sample:
        s32 = z.Solver(mesh, scheme)
        s32.set_state(u0)
        b2.add(s32, n_steps=n_cmp)
        s64 = z.Solver(mesh, dataclasses.replace(scheme, precision=z.FP64))
        s64.set_state(u0)
        s64.advance(n_steps=n_cmp)
        pairs.append((s32, s64, raw, u0))
    while b2.advance(8):
        pass
    for s32, s64, raw, u0 in pairs:
        u32, _ = s32.get_state()
        u64, _ = s64.get_state()
        errs.append((state_rel_l1(u32, u64, None), perturbation_rel_l1(u32, u64, u0, None)))
    b2.close()
    wb = well_balanced_residual(z, sample[0][1], sample[0][2], n_cmp)

    sizes = sorted(m.n_cells for _, m, _, _ in inst)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded meshes and data)",
        "config": {"workload": f"C4 batched ensemble of {n_inst} well-balanced polytrope disks",
                   "instances": n_inst, "cells": total_cells, "cells_min": sizes[0], "cells_median": sizes[len(sizes) // 2],
                   "cells_max": sizes[-1], "precision": "mixed", "batched": True,
                   "scheme": "CWENO-AO o3, HLLC, SSP3, CFL 0.45, isentropic well-balancing",
                   "parallelism": f"replicas x{world}", "l2": "inputs larger than L2",
                   "setup_s": t_setup, "autotune_s": t_tune},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": io_bytes, "d2h_bytes_per_step": io_bytes,
                "path": "set_state of every slot / Batch.advance(1) / get_state of every slot, pinned buffers"},
        "roofline": roof,
        "gpu_launches": launches * args.steps,
        "clocks": clk.summary(),
        "fp64": {"value": v64, "ms_per_step": ms64 / k64, "form": "plain FP64, one solve at a time",
                 "steps_per_instance": k64},
        "mixed_batched_over_fp64": value / v64,
        "error_vs_fp64": {"instances": len(sample), "steps": n_cmp,
                          "state_rel_l1_max": max(e[0] for e in errs),
                          "perturbation_rel_l1_max": max(e[1] for e in errs)},
        "well_balanced": wb,
    }
    if rank == 0:
        raw, mesh, scheme, u0 = inst[len(inst) // 2]
        try:
            line["cpu_baseline"] = cpu_baseline(raw, mesh, scheme, u0,
                                                {"cells": mesh.n_cells, "workload": "C4 ensemble instance"})
        except Exception as exc:
            line["cpu_baseline"] = {"error": str(exc)}
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()


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


def run_serving(args, rank, world, local, pg):
    """C5: Poisson arrivals of uneven 2D / 3D solves, admitted by device
    footprint and batched continuously; mixed form (value) next to the plain
    FP64 form serving the same stream."""
    import numpy as np
    import zisafvm_gb300 as z
    small = args.workload == "c5-small"
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
    # e2e here is the serving path itself: host states in, host states out
    io_in = sum(r["mesh"].n_cells * 5 * 8 for r in reqs)
    line = {
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
        "roofline": None,
        "gpu_launches": None,
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
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
        run_ensemble(args, rank, world, local, pg)
    elif args.workload.startswith("c5"):
        run_serving(args, rank, world, local, pg)
    else:
        run_single_mesh(args, rank, world, local, pg)
    if pg:
        pg.barrier()


if __name__ == "__main__":
    main()
