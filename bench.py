"""Benchmark: cell-stage updates/s of the rate-of-change + SSP-RK step loop.

Default workload: the well-balanced 2D polytrope (gamma = 2, K = 1,
phi = r^2 / 2 on the unit disk, ~200k jittered Delaunay triangles, CWENO-AO
order 3, HLLC, SSP3, CFL 0.45), seeded synthetic data.  One "step" is one SSP3
time step over the whole mesh: 3 cell-stage updates per cell.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c2|c1|c3|c2-small] [--precision fp64|mixed]

value    whole-job cell-stage updates/s, state resident in HBM, CUDA events on
         the solver stream around K graph-replayed steps (max over ranks).
e2e      the same metric through the public API with host buffers: every step
         copies the state from pinned host memory to the device, advances one
         CFL step and reads the new state back.
roofline dominant kernel (the reconstruction kernel): algorithmic bytes per
         launch / its event-timed launch duration, against the measured HBM
         copy bandwidth; FP64 issue rate reported beside it.
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
    ap.add_argument("--workload", default="c2", choices=["c2", "c1", "c3", "c2-small", "c1-small"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
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
    else:
        raw, mesh, scheme, u0 = vortex_tube_3d(n=70, order=3)
        desc = {"workload": "C3 tetrahedral vortex tube", "cells": mesh.n_cells,
                "scheme": "CWENO-AO o3, HLLC, SSP3, CFL 0.3"}
    scheme.precision = prec
    return raw, mesh, scheme, u0, desc


def algorithmic_bytes_per_cell_stage(mesh, scheme, wdt=8) -> int:
    """Compulsory unique HBM traffic of one cell through one stage of the
    reconstruction kernel (per cell, from the array sizes the kernel reads and
    writes): stage state (nv words), pseudo-inverse, stencil indices, one-sided
    local indices, geometry (centre, 1/length, moments), face ids, the face-point
    values it writes and, with well-balancing, potentials at its quadrature
    points and the equilibrium it stores."""
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
    b += NP * wdt                   # pseudo-inverse
    b += MAXL * 4 + NB * RB         # l2g + one-sided local indices
    b += (nd + 1 + NC) * 8 + nf * 4  # centre, 1/length, moments, face ids
    b += nf * nqf * nd * 8 / 2      # face quadrature points (shared by two cells)
    b += nf * nqf * nv * 8          # face-point values written
    if scheme.equilibrium:
        b += nqc * 8 * 2 + nqc * nd * 8 * 2 + 3 * 8   # phi, weights, x, grad phi, equilibrium out
        b += nf * nqf * 8 / 2                          # phi at face points
    if scheme.gravity:
        b += nv * 8                                    # source written
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


def run_reference(args, rank, world):
    """The reference's CPU implementation of the path (its oracle restatement;
    the reference cannot be built here) timed on the host cores."""
    if rank != 0:
        return
    import zisafvm_gb300 as z  # set-up only (host code)
    from oracle import pyoracle
    from problems import polytrope_2d, vortex_2d
    # bounded per-step sample of the same workload: the same scheme on a smaller
    # mesh of the same family, one SSP3 step per timed step
    if args.workload.startswith("c1"):
        raw, mesh, scheme, u0 = vortex_2d(n=48, halo=3)
        cells = mesh.info["n_interior_cells"]
        wl = "C1 periodic isentropic vortex"
    else:
        raw, mesh, scheme, u0 = polytrope_2d(n_rings=60, amplitude=1e-4)
        cells = mesh.n_cells
        wl = "C2 well-balanced polytrope disk"
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
    line = {"metric": "cell-stage updates/s", "value": value, "unit": "cell-stage updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": wl, "cells_per_step_sample": cells, "precision": "fp64"},
            "cpu_baseline": {"value": value, "unit": "cell-stage updates/s", "cores": threads, "kind": "port",
                             "sample": f"each step: one SSP3 step of a {cells}-cell mesh of the same workload "
                                       f"family, oracle OpenMP loops on {threads} threads"},
            "e2e": {"value": value, "unit": "cell-stage updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
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
        if pg:
            pg.barrier()
        return

    import numpy as np
    import zisafvm_gb300 as z
    raw, mesh, scheme, u0, desc = workload(args.workload, args.precision)
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
    if pg:
        import torch
        t = torch.tensor([ms], dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
    value = world * cells * stages * args.steps / (ms * 1e-3)

    if args.profile:
        if rank == 0:
            print(json.dumps({"metric": "cell-stage updates/s", "value": value, "ms_per_step": ms / args.steps,
                              "config": desc, "profile_run": True}), flush=True)
        return

    # per-kernel event timing of the same loop (not graph-replayed)
    kt = solver.kernel_times(min(args.steps, 32))
    wdt = 8
    b_cell = algorithmic_bytes_per_cell_stage(mesh, scheme, wdt)
    n_recon = mesh.n_cells
    bytes_launch = b_cell * n_recon
    achieved = bytes_launch / (kt["reconstruct"] * 1e-3) / 1e9
    hbm, peak_kind = measured_peaks()
    traffic = profiles_traffic("k_reconstruct", args.workload, args.precision)

    # end to end through the public API with host buffers
    try:
        import torch
        host = torch.empty((mesh.n_cells, 5), dtype=torch.float64, pin_memory=True).numpy()
        host_out = torch.empty((mesh.n_cells, 5), dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        host = np.empty((mesh.n_cells, 5))
        host_out = np.empty((mesh.n_cells, 5))
    solver.set_state(u0)
    solver.advance(n_steps=1)
    state, _ = solver.get_state()
    host[:] = state
    e2e_steps = max(4, min(args.steps, 64))
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        solver.set_state(host)
        solver.advance(n_steps=1)
        solver.get_state(out=host_out)
        host, host_out = host_out, host
    e2e_s = time.perf_counter() - t0
    e2e_value = world * cells * stages * e2e_steps / e2e_s
    io_bytes = mesh.n_cells * 5 * 8

    line = {
        "metric": "cell-stage updates/s", "value": value, "unit": "cell-stage updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded mesh and initial data)",
        "config": {**desc, "precision": args.precision, "parallelism": f"replicas x{world}",
                   "l2": "working set of the step loop > L2 for c2/c3; state stays resident across steps"},
        "e2e": {"value": e2e_value, "unit": "cell-stage updates/s", "h2d_bytes_per_step": io_bytes,
                "d2h_bytes_per_step": io_bytes},
        "roofline": {"bound": "hbm", "kernel": "k_reconstruct", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "peak_kind": peak_kind,
                     "bytes_per_cell_stage": b_cell, "traffic": traffic,
                     "kernel_ms": kt},
        "gpu_launches": solver.launches_per_step() * args.steps,
        "clocks": clk.summary(),
    }
    if args.precision == "mixed":
        # error of the mixed form against the FP64 form after the same steps
        import dataclasses
        from metrics import perturbation_rel_l1, state_rel_l1
        s64 = z.Solver(mesh, dataclasses.replace(scheme, precision=z.FP64))
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
            eq_raw, eq_mesh, eq_scheme, eq_u0, _ = workload(args.workload, args.precision)
            u_eq = eq_mesh.initial_conditions("polytrope", gamma=2.0, K=1.0, rho_c=1.0, k_phi=1.0, amplitude=0.0)
            s_eq = z.Solver(eq_mesh, eq_scheme)
            s_eq.set_state(u_eq)
            res = float(np.abs(s_eq.rate_of_change()).max())
            s_eq.advance(n_steps=n_cmp)
            u_end, _ = s_eq.get_state()
            drift = float((np.abs(u_end - u_eq).max(axis=0) / np.abs(u_eq).max(axis=0))[[0, 4]].max())
            line["well_balanced"] = {"max_abs_dudt": res, "rel_drift": drift, "steps": n_cmp}
    if rank == 0:
        try:
            line["cpu_baseline"] = cpu_baseline(raw, mesh, scheme, u0, desc)
        except Exception as exc:  # the baseline must not hide the GPU number
            line["cpu_baseline"] = {"error": str(exc)}
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()


if __name__ == "__main__":
    main()
