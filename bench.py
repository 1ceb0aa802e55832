"""Headline benchmark: steady transonic NACA 0012 solves per second on one GB300.

Workload (the reference's transonic inviscid configuration): NACA 0012 with a
closed trailing edge on a 512 x 256 O-grid to 30 chords (radial growth 1.05,
outer 40 % of the rings triangulated; 183,296 cells, 314,880 faces), M 0.8,
AoA 1.25 deg, HLLC flux, Green-Gauss gradients, Venkatakrishnan limiter
(K = 5).  One step = one complete steady solve from freestream: a first-order
starter solve followed by the second-order solve to an absolute area-weighted
energy-residual norm below 1e-10, with the FP32 stored Jacobian and the FP32
block-colour ILU(0) preconditioner inside FGMRES(30).  Synthetic mesh and
inputs (seeded generator); the working set (states, Jacobian, Krylov basis,
~0.5 GB) exceeds the 126 MB L2, so no explicit flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line on rank 0 (N > 1: one independent solve per rank,
weak scaling, no collective on the data path).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MESH = [512, 256, 30.0, 0, 0, 1.05, 154, 3]
PHYS = dict(Minf=0.8, aoa_deg=1.25)
NUM_MAIN = dict(flux="HLLC", gradient="GREENGAUSS", reconstruction="VENKATAKRISHNAN", limiter_param=5.0)
NUM_START = dict(flux="HLLC", gradient="NONE")
BCS = [(2, "slipwall", ()), (4, "farfield", ())]
STARTER = dict(cfl_min=25, cfl_max=500, tolerance=1e-1, abs_tolerance=0, max_timesteps=100, nl_update=1,
               min_relax=0.3)
MAIN = dict(cfl_min=50, cfl_max=1000, tolerance=1e-10, abs_tolerance=1, max_timesteps=600, nl_update=1,
            min_relax=0.3, pc="ilu0")
WORKLOAD = "naca0012_transonic_512x256_ogrid_hllc_gg_venkat5"
METRIC = "solves/s to ||R||<1e-10 (transonic NACA0012, FP32 Jacobian + FP32 block-colour ILU0)"


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                parts = [p.strip() for p in out.stdout.strip().split(",")]
                if len(parts) >= 7:
                    self.samples.append(parts)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def build_case(fv):
    m = fv.UMesh.generate(fv.MESH_NACA_OGRID, MESH, reorder=1)
    ph = fv.physics_cfg(**PHYS)
    main = fv.FlowFV(m, ph, fv.numerics_cfg(**NUM_MAIN), BCS)
    start = fv.FlowFV(m, ph, fv.numerics_cfg(**NUM_START), BCS)
    return m, main, start


def run_ours(args):
    import torch

    import fvens_gb300 as fv
    from fvens_gb300 import build as fvbuild

    rank, world, local = _dist()
    if not os.path.exists(fv.LIB_PATH):
        fvbuild.build_library()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    m, main, start = build_case(fv)
    prec = 8 if args.plain else 4
    S1 = fv.SteadyBackwardEulerSolver(start, precision=prec, **STARTER)
    S2 = fv.SteadyBackwardEulerSolver(main, precision=prec, **MAIN)
    uinf = main.freestream()[0]
    u0 = np.ascontiguousarray(np.tile(uinf, (m.nelem, 1)))
    ud = torch.empty((m.nelem, 4), dtype=torch.float64, device=dev)
    u0d = torch.tensor(u0, device=dev)

    def solve_device():
        ud.copy_(u0d)
        S1.solve(ud, raise_on_error=False)
        rc, st = S2.solve(ud, raise_on_error=False)
        return rc, st

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        rc, st = solve_device()
    torch.cuda.synchronize()
    launches0 = fv.kernel_launch_count()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    with ClockSampler(local) as clk:
        ev0.record()
        for _ in range(args.steps):
            rc, st = solve_device()
            stats.append(st[0])
        ev1.record()
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = fv.kernel_launch_count() - launches0
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * args.steps / (ms / 1e3)

    # end to end through the host-buffer C-ABI call: pinned host state in,
    # converged state out (starter and main solve)
    hu = torch.empty((m.nelem, 4), dtype=torch.float64).pin_memory()
    hn = hu.numpy()
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        hn[:] = u0
        S1.solve_host(hn, raise_on_error=False)
        S2.solve_host(hn, raise_on_error=False)
    t1 = time.perf_counter()
    e2e_s = t1 - t0
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * args.steps / e2e_s

    # per-kernel timing (roofline) at the converged state
    def timed(which, reps=20):
        import ctypes
        a, b = ctypes.c_double(), ctypes.c_double()
        fv.check(fv.lib().fv_solver_time_kernel(S2._h, fv._vp(fv.dptr(ud)), which, reps, ctypes.byref(a),
                                                ctypes.byref(b)))
        return a.value, b.value

    kern = {}
    for name, which in (("residual", 0), ("face_flux", 1), ("jacobian", 2), ("ilu0_apply", 3), ("spmv", 4),
                        ("ilu0_setup", 5)):
        ms_k, by = timed(which)
        kern[name] = dict(ms=ms_k, bytes=by, gbs=by / (ms_k * 1e-3) / 1e9)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    dom = "ilu0_apply"
    steps_main = statistics.median([s["steps"] for s in stats])
    lin_main = statistics.median([s["lin_iters"] for s in stats])
    nf = m.naface
    nblocks = m.nelem + 2 * (m.naface - m.nbface)
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 residual / f32 jacobian+ilu0" if prec == 4 else "f64",
        "data": "synthetic (seeded NACA 0012 O-grid generator, freestream start)",
        "config": {"workload": WORKLOAD, "cells": m.nelem, "faces": nf, "batch": 1,
                   "parallelism": f"replicas{world}" if world > 1 else "single",
                   "l2": "working set > L2 (no flush needed)",
                   "main_steps_median": steps_main, "linear_iters_median": lin_main,
                   "converged": all(s["status"] == 0 for s in stats),
                   "final_res_max": max(s["res"] for s in stats)},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": 2 * u0.nbytes,
                "d2h_bytes_per_step": 2 * u0.nbytes},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": kern[dom]["gbs"], "peak": hbm_peak,
                     "unit": "GB/s", "frac": kern[dom]["gbs"] / hbm_peak, "traffic": None,
                     "peak_source": peak_src},
        "kernels": kern,
        "residual_gfaces_s": nf / (kern["residual"]["ms"] * 1e-3) / 1e9,
        "jacobian_blocks_s": nblocks / (kern["jacobian"]["ms"] * 1e-3),
        "ilu0_sweep_gbs": kern["ilu0_apply"]["gbs"],
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(m, steps_main, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def cpu_baseline(m, steps_per_solve, budget_s):
    """The oracle (the CPU restatement of the reference's path) on the host
    cores: a bounded number of pseudo-time steps of the same second-order
    solve, scaled to solves/s with the GPU's step count per solve."""
    from oracle import orc
    nthreads = os.cpu_count() or 1
    orc.set_threads(nthreads)
    om = orc.Mesh.from_export(m.export())
    od = orc.Disc(om, **PHYS, **NUM_MAIN, bcs=BCS)
    u0 = np.tile(od.freestream(), (m.nelem, 1))
    nsteps = 1
    t0 = time.perf_counter()
    od.steady_solve(u0, cflmin=MAIN["cfl_min"], cflmax=MAIN["cfl_max"], tol=1e-10, maxiter=nsteps, pc="ilu0",
                    nl_update="robust_flow", min_relax=MAIN["min_relax"])
    per = time.perf_counter() - t0
    nsteps = max(1, min(20, int(budget_s / max(per, 1e-3))))
    t0 = time.perf_counter()
    od.steady_solve(u0, cflmin=MAIN["cfl_min"], cflmax=MAIN["cfl_max"], tol=1e-10, maxiter=nsteps, pc="ilu0",
                    nl_update="robust_flow", min_relax=MAIN["min_relax"])
    per = (time.perf_counter() - t0) / nsteps
    value = 1.0 / (per * max(steps_per_solve, 1))
    return {"value": value, "unit": "solves/s", "cores": nthreads, "kind": "port",
            "sample": f"{nsteps} second-order implicit pseudo-time steps of the same workload on the oracle "
                      f"({per:.2f} s/step, natural-order ILU0, FGMRES(30)), scaled by {steps_per_solve} steps/solve"}


def run_reference(args):
    """The reference's CPU path as restated by the oracle (the reference itself
    does not build here: PETSc, Eigen, Boost and MPI are absent), on all host
    threads; each step is a bounded sample of the workload."""
    rank, world, local = _dist()
    if rank != 0:
        return
    from fvens_gb300 import build as fvbuild
    import fvens_gb300 as fv
    if not os.path.exists(fvbuild.ORACLE_LIB):
        fvbuild.build_oracle()
    if not os.path.exists(fv.LIB_PATH):
        fvbuild.build_library()
    m = fv.UMesh.generate(fv.MESH_NACA_OGRID, MESH, reorder=1)
    steps_per_solve = args.ref_steps_per_solve
    vals = []
    for k in range(args.warmup + args.steps):
        cb = cpu_baseline(m, steps_per_solve, args.cpu_seconds / max(args.steps + args.warmup, 1))
        if k >= args.warmup:
            vals.append(cb)
    value = statistics.median([v["value"] for v in vals])
    cb = dict(vals[-1])
    cb["value"] = value
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded NACA 0012 O-grid generator)",
            "config": {"workload": WORKLOAD, "cells": m.nelem, "faces": m.naface},
            "cpu_baseline": cb, "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain", action="store_true", help="FP64 Jacobian and preconditioner (the plain path)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--ref-steps-per-solve", type=int, default=150)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
