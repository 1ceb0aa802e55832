"""Headline benchmark: steady transonic NACA 0012 solves per second on one GB300.

Workload (the reference's transonic inviscid configuration): NACA 0012 with a
closed trailing edge on a 512 x 256 O-grid to 30 chords (outer 40 % of the
rings triangulated; 183,296 cells, 314,880 faces), M 0.8, AoA 1.25 deg, HLLC
flux, Green-Gauss gradients, Venkatakrishnan limiter (K = 5).  The radial
spacing grows by 1.02 per ring (first cell 3.8e-3 chords): with growth 1.05
the first cell is 5.7e-6 chords and the reference's pseudo-time method does
not reach 1e-10 on it in thousands of steps.  One step = one complete steady
solve from freestream: a first-order starter (100 pseudo-time steps) followed
by the second-order solve to an absolute area-weighted energy-residual norm
below 1e-10, matrix-free FP64 Jacobian-vector products in FGMRES(30) with the
FP32 stored first-order Jacobian and the FP32 block-colour ILU(0)
preconditioner.  Synthetic mesh and inputs (seeded generator); the working set
(states, Jacobian, Krylov basis, ~0.5 GB) exceeds the 126 MB L2, so no
explicit flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --kernel residual|ilu|jacobian|mpnn|fp64peak [--reps R]

--impl reference: the oracle (the CPU FP64 restatement of the reference's
path, natural-order ILU(0) as PETSc's) on all host cores, building the same
mesh with its own generator; it times ONE complete solve of the workload (it
takes minutes), whatever --steps / --warmup ask for, and says so in its line.

--kernel: profiling aid; runs R launches of one kernel family on the workload
(or on the laminar hybrid mesh for mpnn) and prints the mean time per launch.

Prints one JSON line on rank 0 (N > 1: one independent solve per rank,
weak scaling, no collective on the data path).
"""
import argparse
import hashlib
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MESH = [512, 256, 30.0, 0, 0, 1.02, 154, 3]
SMALL_MESH = [64, 32, 30.0, 0, 0, 1.1, 20, 3]
PHYS = dict(Minf=0.8, aoa_deg=1.25)
NUM_MAIN = dict(flux="HLLC", gradient="GREENGAUSS", reconstruction="VENKATAKRISHNAN", limiter_param=5.0)
NUM_START = dict(flux="HLLC", gradient="NONE")
BCS = [(2, "slipwall", ()), (4, "farfield", ())]
STARTER = dict(cfl_min=25, cfl_max=500, tolerance=1e-1, abs_tolerance=0, max_timesteps=100, nl_update=2,
               min_relax=0.2, pc="ilu0")
# Solver options of the main solve (each one the reference's own: PETSc's
# -ksp_rtol, -matrix_free_difference_step, the update's minimum relaxation).
# The Venkatakrishnan-limited transonic solve stalls just above 1e-10 or blows
# up for part of the rounding-level perturbations of its path with the
# reference's defaults (difference step 1e-7, relaxation floor 0.2); a
# difference step of 1e-8 (fewer finite differences across limiter switches)
# and a floor of 0.1 converge for every perturbation tried.
MAIN = dict(cfl_min=100, cfl_max=5000, tolerance=1e-10, abs_tolerance=1, max_timesteps=2000, nl_update=2,
            min_relax=0.1, pc="ilu0", matrix_free=1, ksp_rtol=0.3, mf_eps=1e-8)
WORKLOAD = "naca0012_transonic_512x256_ogrid_g1.02_hllc_gg_venkat5"
METRIC = "solves/s to ||R||<1e-10 (transonic NACA0012, matrix-free FGMRES, FP32 Jacobian + FP32 block-colour ILU0)"
C2_FIXTURE = os.path.join(ROOT, "tests", "golden", "naca0012_transonic_oracle_converged.npz")

# Per-launch counters of the residual's two heavy kernels on this workload
# (ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,
#  sm__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum,
#  sm__thread_inst_executed_pipe_fp64_pred_on.sum on `python bench.py --kernel residual`),
# valid for the kernel sources whose digest is `sources`; any other build reports them as null.
_CAPTURE = ("ncu --metrics ... -k regex:'k_face|k_grad' -c 4 on `python bench.py --kernel residual --reps 20` "
            "(transonic workload, perturbed freestream state); gradients: k_grad alone")
NCU_COUNTS = {
    "sources": "87537eca21f92835",
    "face_flux": {"faces": 314880, "dram_bytes": 38410496, "fp64_flop": 86596608, "fp64_pipe_inst": 59829760,
                  "capture": _CAPTURE},
    "gradients": {"faces": 314880, "dram_bytes": 36154112, "fp64_flop": 65691648, "fp64_pipe_inst": 43585504,
                  "capture": _CAPTURE},
}
KERNEL_SOURCES = ["fvens_gb300/csrc/fv_residual_body.cuh", "fvens_gb300/csrc/fv_device.cuh",
                  "fvens_gb300/csrc/fv_residual.cu", "fvens_gb300/csrc/fv_core.cuh"]
# DRAM traffic of one FP32 ILU(0) apply on this workload (the 10 colour launches
# of k_fwd_parts / k_bwd_parts; ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum
# -k regex:'k_fwd_parts|k_bwd_parts' -s 10 -c 10 on `python bench.py --kernel ilu --reps 5`),
# valid for the sweep sources whose digest is `sources`
NCU_ILU = {"sources": "010e9ef5d94d2cd6", "dram_bytes": 86507520}
ILU_SOURCES = ["fvens_gb300/csrc/fv_linalg.cu", "fvens_gb300/csrc/fv_linalg.cuh"]


def kernel_sources_digest(files=None):
    h = hashlib.sha256()
    for f in files or KERNEL_SOURCES:
        with open(os.path.join(ROOT, f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def _host_threads():
    """Host threads this process may run on (its CPU affinity)."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_config(world, small=False):
    """The workload's description, identical in both arms' lines."""
    mesh = SMALL_MESH if small else MESH
    return {"workload": WORKLOAD if not small else "naca0012_transonic_64x32_ogrid_g1.1_hllc_gg_venkat5_test",
            "mesh": f"NACA 0012 O-grid {mesh[0]} x {mesh[1]} to {mesh[2]:g} chords, radial growth {mesh[5]:g}, "
                    f"rings from {mesh[6]} triangulated (seed {mesh[7]})",
            "cells": 183296 if not small else 2 * 64 * 32 - 20 * 64, "faces": 314880 if not small else None,
            "flow": "inviscid, M 0.8, AoA 1.25 deg", "scheme": "HLLC, Green-Gauss, Venkatakrishnan K=5",
            "solve": "freestream; 100 first-order starter steps (CFL 25->500); second-order solve to "
                     "||R||<1e-10 (CFL 100->5000, matrix-free FGMRES(30), rtol 0.3, difference step 1e-8, "
                     "relaxation floor 0.1)",
            "batch": 1, "parallelism": f"replicas{world}" if world > 1 else "single",
            "l2": "working set > L2 (no flush needed)"}


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


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def build_case(fv, small=False):
    m = fv.UMesh.generate(fv.MESH_NACA_OGRID, SMALL_MESH if small else MESH, reorder=1)
    ph = fv.physics_cfg(**PHYS)
    main = fv.FlowFV(m, ph, fv.numerics_cfg(**NUM_MAIN), BCS)
    start = fv.FlowFV(m, ph, fv.numerics_cfg(**NUM_START), BCS)
    return m, main, start


def run_ours(args):
    import torch

    import fvens_gb300 as fv
    from fvens_gb300 import build as fvbuild
    from fvens_gb300.replicas import Replicas

    rank, world, local = _dist()
    if not os.path.exists(fv.LIB_PATH):
        fvbuild.build_library()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    reps = Replicas("nccl", dev)
    m, main, start = build_case(fv, args.small)
    prec = 8 if args.plain else 4
    S1 = fv.SteadyBackwardEulerSolver(start, precision=prec, **STARTER)
    S2 = fv.SteadyBackwardEulerSolver(main, precision=prec, **MAIN)
    uinf = main.freestream()[0]
    u0 = np.ascontiguousarray(np.tile(uinf, (m.nelem, 1)))
    ud = torch.empty((m.nelem, 4), dtype=torch.float64, device=dev)
    u0d = torch.tensor(u0, device=dev)
    # launch geometry of the residual kernels picked by the autotuner (untimed)
    block_sizes = {"main": main.autotune(u0d), "starter": start.autotune(u0d)}

    def solve_device():
        ud.copy_(u0d)
        _, st1 = S1.solve(ud, raise_on_error=False)
        if args.nvtx:
            torch.cuda.nvtx.range_push("main_solve")
        rc, st2 = S2.solve(ud, raise_on_error=False)
        if args.nvtx:
            torch.cuda.nvtx.range_pop()
        return st1[0], st2[0]

    barrier = reps.barrier

    for _ in range(args.warmup):
        solve_device()
    torch.cuda.synchronize()
    launches0 = fv.kernel_launch_count()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    with ClockSampler(local) as clk:
        ev0.record()
        for _ in range(args.steps):
            stats.append(solve_device())
        ev1.record()
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = fv.kernel_launch_count() - launches0
    value = reps.throughput(args.steps, ms / 1e3)
    ms = reps.max_over_ranks(ms)
    converged = all(s2["status"] == 0 for _, s2 in stats)
    u_conv = ud.clone()

    # end to end through the host-buffer C-ABI call: pinned host state in,
    # converged state out (starter and main solve)
    n_e2e = max(1, min(args.steps, args.e2e_solves))
    hu = torch.empty((m.nelem, 4), dtype=torch.float64).pin_memory()
    hn = hu.numpy()
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        hn[:] = u0
        S1.solve_host(hn, raise_on_error=False)
        S2.solve_host(hn, raise_on_error=False)
    t1 = time.perf_counter()
    e2e_value = reps.throughput(n_e2e, t1 - t0)
    cl = main.surface_data(u_conv, 2)[0]
    variants = {} if args.no_variants else run_variants(fv, torch, dev, m, main, start, u0d, prec, args)
    ud.copy_(u_conv)

    # per-kernel timing at the converged state; time shares of one solve from
    # the launch counts per step / per Krylov iteration
    def timed(S, which, reps=20):
        import ctypes
        a, b = ctypes.c_double(), ctypes.c_double()
        fv.check(fv.lib().fv_solver_time_kernel(S._h, fv._vp(fv.dptr(ud)), which, reps, ctypes.byref(a),
                                                ctypes.byref(b)))
        return a.value, b.value

    kern = {}
    for name, which in (("residual", 0), ("face_flux", 1), ("jacobian", 2), ("ilu0_apply", 3), ("spmv", 4),
                        ("ilu0_setup", 5), ("gradients", 6)):
        ms_k, by = timed(S2, which)
        kern[name] = dict(ms=ms_k, bytes=by, gbs=by / (ms_k * 1e-3) / 1e9)
    s1, s2 = stats[-1]
    steps_main, lin_main = s2["steps"], s2["lin_iters"]
    mf = MAIN.get("matrix_free", 0)
    calls = {"residual": steps_main + (lin_main if mf else 0), "jacobian": steps_main, "ilu0_setup": steps_main,
             "ilu0_apply": lin_main, "spmv": 0 if mf else lin_main}
    share_ms = {k: calls[k] * kern[k]["ms"] for k in calls}
    # the roofline names one kernel: the larger of the residual's two heavy
    # launches (the face kernel, the gradient/limiter pass) or the ILU(0) sweep
    single = {"face_flux": calls["residual"] * kern["face_flux"]["ms"],
              "gradients": calls["residual"] * kern["gradients"]["ms"],
              "ilu0_apply": share_ms["ilu0_apply"]}
    dom = max(single, key=single.get)
    peaks = _peaks()
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    dfma_rate, _ = fv.fp64_peak(5)
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
        "dtype": "f64 residual+krylov / f32 jacobian+ilu0" if prec == 4 else "f64",
        "data": "synthetic (seeded NACA 0012 O-grid generator, freestream start)",
        "config": workload_config(world, args.small),
        "solve": {"starter_steps": s1["steps"], "starter_linear_iters": s1["lin_iters"], "main_steps": steps_main,
                  "linear_iters": lin_main, "converged": converged, "final_res": s2["res"],
                  "cl_cdp": [float(cl[0]), float(cl[1])], "residual_block_sizes": block_sizes,
                  "launches_per_solve": launches / max(args.steps, 1)},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(u0.nbytes),
                "d2h_bytes_per_step": int(u0.nbytes), "solves": n_e2e},
        "gpu_launches": int(launches),
        "roofline": dict(roofline(dom, kern, nf, hbm_peak, peak_src, dfma_rate),
                         others={k: roofline(k, kern, nf, hbm_peak, peak_src, dfma_rate)
                                 for k in single if k != dom}),
        "kernels": kern,
        "solve_time_shares_ms": share_ms,
        "variants": variants,
        "residual_gfaces_s": nf / (kern["residual"]["ms"] * 1e-3) / 1e9,
        "jacobian_blocks_s": nblocks / (kern["jacobian"]["ms"] * 1e-3),
        "ilu0_sweep_gbs": kern["ilu0_apply"]["gbs"],
        "fp64_peak_tflops": 2 * dfma_rate / 1e12,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu:
        u_host = u_conv.cpu().numpy().reshape(m.nelem, 4)
        line["cpu_baseline"] = cpu_baseline(m, args.cpu_seconds, u_host)
        line["oracle_parity"] = oracle_parity(m, main, u_conv)
    if rank == 0:
        print(json.dumps(line), flush=True)
    reps.close()


def roofline(dom, kern, nfaces, hbm_peak, peak_src, dfma_rate):
    """The roofline of the dominant kernel.  The residual's kernels are bound
    by the FP64 pipe on this part: FLOP/s (DADD + DMUL + 2 DFMA per launch,
    from the ncu counters of this build) against twice the measured DFMA rate,
    with the FP64-pipe instruction rate against the DFMA rate beside it; the
    HBM fraction of the model bytes is reported too.  The ILU(0) sweep is
    reported against HBM."""
    k = kern[dom]
    hbm = {"achieved": k["gbs"], "peak": hbm_peak, "unit": "GB/s", "frac": k["gbs"] / hbm_peak,
           "peak_source": peak_src}
    valid = NCU_COUNTS["sources"] == kernel_sources_digest()
    cnt = NCU_COUNTS.get(dom) if valid else None
    traffic = cnt["dram_bytes"] if cnt else None
    if dom == "ilu0_apply" and NCU_ILU["sources"] == kernel_sources_digest(ILU_SOURCES):
        traffic = NCU_ILU["dram_bytes"]
    if dom == "ilu0_apply" or cnt is None:
        out = dict(bound="hbm", kernel=dom, traffic=traffic, **hbm)
        if dom != "ilu0_apply":
            out["note"] = "FP64-pipe bound; no ncu capture of this build's kernel sources to count its FP64 work"
        return out
    sec = k["ms"] * 1e-3
    flops = cnt["fp64_flop"] * nfaces / cnt["faces"]
    pipe = cnt["fp64_pipe_inst"] * nfaces / cnt["faces"]
    peak = 2 * dfma_rate
    return {"bound": "fp64", "kernel": dom, "achieved": flops / sec / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
            "frac": flops / sec / peak, "fp64_pipe_frac": pipe / sec / dfma_rate,
            "traffic": traffic, "peak_source": "measured in this run (fv_fp64_peak: FP64 FMA chains on every SM)",
            "counts_per_launch": {"fp64_flop": flops, "fp64_pipe_inst": pipe, "source": cnt["capture"]},
            "hbm": hbm}


def _timed_solve(torch, S_list, u, all_members=False):
    """Runs the solvers in turn on u; (seconds by CUDA events, the last
    solver's stats of member 0, or of every member)."""
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    sts = [S.solve(u, raise_on_error=False)[1] for S in S_list]
    ev1.record()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1e3, (sts[-1] if all_members else sts[-1][0])


def run_variants(fv, torch, dev, m, main, start, u0d, prec, args):
    """(1) The same solve on the plain path: FP64 Jacobian and FP64 ILU(0),
    freestream start, one timed solve (CUDA events).  (2) Batched laminar
    solves (run_batched).  (3) The learned warm start (run_warm_start).
    (4) The ~4M-cell instance (run_large)."""
    out = {}

    def guarded(name, fn):
        # a variant that fails reports its error instead of ending the benchmark
        try:
            out[name] = fn()
        except Exception as exc:  # noqa: BLE001
            out[name] = {"error": f"{type(exc).__name__}: {exc}"}
        torch.cuda.synchronize()
        return out[name]

    u = torch.empty_like(u0d)
    P1 = fv.SteadyBackwardEulerSolver(start, precision=8, **STARTER)
    P2 = fv.SteadyBackwardEulerSolver(main, precision=8, **MAIN)
    u.copy_(u0d)
    t, st = _timed_solve(torch, [P1, P2], u)
    out["plain_fp64_cold"] = {"solves_s": 1.0 / t, "s_per_solve": t, "main_steps": st["steps"],
                              "linear_iters": st["lin_iters"], "converged": st["status"] == 0, "res": st["res"]}
    del P1, P2
    if args.large:
        guarded("large_4m", lambda: run_large(fv, torch, dev, float(_peaks().get("hbm_gbs", 6800.0)),
                                              args.large_solve))
    if args.batched:
        got = {}

        def batched():
            bl, got["phys"], got["u"] = run_batched(fv, torch, dev, args.laminar_levels, args.batch,
                                                    sgs=args.laminar_sgs)
            return bl
        bl = guarded("batched_laminar", batched)
        if args.warm_test > 0 and (args.warm_train > 0 or got.get("phys")):
            guarded("warm_start_laminar", lambda: run_warm_start(
                fv, torch, dev, args.laminar_levels, args.warm_train, args.warm_test, args.warm_epochs, args.batch,
                plain_single_s=bl["single_plain_fp64"]["seconds"],
                train_set=None if args.warm_train > 0 else (got["phys"], got["u"])))
        got.clear()
    return out


LAMINAR_BCS = [(4, "inflowoutflow", ()), (2, "adiabaticwall", (0.0,))]
LAMINAR_FIXTURE = os.path.join(ROOT, "tests", "golden", "naca0012_laminar_l{}_oracle_converged.npz")


def _laminar_mesh(fv, levels=0):
    """The reference's hybrid NACA 0012 mesh (13,156 cells), uniformly refined
    `levels` times by the rule that makes the reference's level-2 mesh from
    it (13,156 x 4^levels cells), with its boundary-layer lines kept whole in
    the preconditioner's parts."""
    from fvens_gb300 import meshes
    z = np.load(os.path.join(ROOT, "tests", "golden", "naca0012_lam_hybrid_1_mesh.npz"))
    a = meshes.refine(dict(coords=z["coords"], nnode=z["nnode"], inpoel=z["inpoel"], bface=z["bface"],
                           btag=z["btag"]), levels)
    m = fv.UMesh.from_arrays(a["coords"], a["nnode"], a["inpoel"], a["bface"], a["btag"], reorder=1)
    return m, m.find_lines(10.0)[0]


def _laminar_conditions(fv, n, seed):
    """n seeded laminar conditions: M ~ U[0.3, 0.7], AoA ~ U[-4, 4] deg,
    Re ~ U[2000, 10000], Pr 0.72, T 288.15 K."""
    rng = np.random.default_rng(seed)
    M, A, Re = rng.uniform(0.3, 0.7, n), rng.uniform(-4, 4, n), rng.uniform(2000, 10000, n)
    return [fv.physics_cfg(Minf=float(M[k]), aoa_deg=float(A[k]), Reinf=float(Re[k]), Tinf=288.15, Pr=0.72,
                           viscous=True) for k in range(n)]


# the batched laminar main solve stops a member whose residual has not halved
# in 300 steps (the solver's stagnation stop; members that converge halve it
# every few steps): about half of the 64 conditions never converge on this
# mesh (unsteady separated flows) and otherwise run to the step limit
# pc_ordering 2: the preconditioner's parts coloured with one colour fewer
# (one launch fewer per sweep) than the greedy colouring of the headline solve
LAMINAR_MAIN = dict(cfl_min=200, cfl_max=5000, tolerance=1e-10, abs_tolerance=1, max_timesteps=1500, nl_update=2,
                    stall_steps=300, stall_factor=0.5, pc_ordering=2)
LAMINAR_START = dict(cfl_min=200, cfl_max=1000, tolerance=1e-1, abs_tolerance=0, max_timesteps=50, nl_update=2,
                     pc_ordering=2)


def _laminar_solvers(fv, m, plist, prec, starter=True, pc="ilu0"):
    """(discretisation, [starter solver,] main solver) for the conditions plist:
    first-order starter to a relative 1e-1 (at most 50 steps), then the
    second-order main solve to the absolute 1e-10."""
    main = fv.FlowFV(m, plist, fv.numerics_cfg(flux="ROE", gradient="LEASTSQUARES"), LAMINAR_BCS)
    S2 = fv.SteadyBackwardEulerSolver(main, pc=pc, precision=prec, **LAMINAR_MAIN)
    if not starter:
        return main, [S2]
    start = fv.FlowFV(m, plist, fv.numerics_cfg(flux="ROE", gradient="NONE"), LAMINAR_BCS)
    S1 = fv.SteadyBackwardEulerSolver(start, pc=pc, precision=prec, **LAMINAR_START)
    return main, [S1, S2]


def _freestream_field(torch, dev, disc, nelem):
    return torch.tensor(np.concatenate([np.tile(x, (nelem, 1)) for x in disc.freestream()]), device=dev)


def _vs_laminar_fixture(m, levels, main, u, members):
    """Converged states and Cl / CDp / CDsf of the given batch members against
    the oracle's own converged solves of the same conditions (committed
    fixture, solved to `oracle_tolerance`; None when absent)."""
    path = LAMINAR_FIXTURE.format(levels)
    if not os.path.exists(path):
        return None
    z = np.load(path)
    perm = m.export()["perm"]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm))
    uv = u.view(-1, m.nelem, 4).cpu().numpy()
    fun = main.surface_data(u, 2)
    out = []
    for j, k in enumerate(z["members"]):
        if k not in members:
            continue
        ug = uv[k][inv[z["cells"]]]
        uo = z["states"][j]
        out.append({"member": int(k), "oracle_tolerance": float(z["tolerance"]) if "tolerance" in z.files else 1e-10,
                    "state_rel_diff": float(np.abs(ug - uo).max() / np.abs(uo).max()),
                    "cl_cdp_cdsf_rel_diff": [float(abs(fun[k, i] - z["functionals"][j, i]) /
                                                   max(abs(z["functionals"][j, i]), 1e-300)) for i in range(3)]})
    return out


def run_batched(fv, torch, dev, levels=2, B=64, seed=7, sgs=False):
    """Batched solves of B laminar conditions (M ~ U[0.3, 0.7], AoA ~ U[-4, 4] deg,
    Re ~ U[2000, 10000], Pr 0.72, adiabatic wall; Roe, least squares) on the
    reference's hybrid NACA 0012 mesh refined `levels` times, all members in
    the same launches with FP32 Jacobians and ILU(0) (with sgs, also with
    block SGS), against member 0 alone on the FP32 path and on the plain FP64
    path.  Returns (results, conditions and device states of the batch's
    converged members)."""
    import collections
    m, nlines = _laminar_mesh(fv, levels)
    phs = _laminar_conditions(fv, B, seed)
    res = {"mesh_cells": m.nelem, "mesh_faces": m.naface, "refinements": levels, "batch": B, "lines": nlines,
           "max_main_steps": LAMINAR_MAIN["max_timesteps"]}
    runs = [("single_plain_fp64", phs[:1], 8, "ilu0"), ("single", phs[:1], 4, "ilu0"), ("batch", phs, 4, "ilu0")]
    if sgs:
        runs.append(("batch_sgs", phs, 4, "sgs"))
    conv_phys, conv_states = [], None
    for tag, plist, prec, pc in runs:
        main, solvers = _laminar_solvers(fv, m, plist, prec, pc=pc)
        u = _freestream_field(torch, dev, main, m.nelem)
        t, stats = _timed_solve(torch, solvers, u, all_members=True)
        conv = [k for k, st in enumerate(stats) if st["status"] == 0]
        res[tag] = {"seconds": t, "converged": len(conv), "members": len(plist), "converged_solves_s": len(conv) / t,
                    "status_counts": dict(collections.Counter(int(st["status"]) for st in stats)),
                    "main_steps_max": max(st["steps"] for st in stats),
                    "main_steps_mean": float(np.mean([st["steps"] for st in stats])),
                    "main_steps_mean_converged": float(np.mean([stats[k]["steps"] for k in conv])) if conv else None,
                    "linear_iters_mean": float(np.mean([st["lin_iters"] for st in stats]))}
        if tag in ("single_plain_fp64", "batch"):
            res[tag]["vs_oracle"] = _vs_laminar_fixture(m, levels, main, u, conv)
        if tag == "batch" and conv:
            conv_phys = [plist[k] for k in conv]
            conv_states = u.view(len(plist), m.nelem, 4)[torch.as_tensor(conv, device=u.device)].clone()
        del main, solvers, u
    best = max(res[k]["converged_solves_s"] for k in ("batch", "batch_sgs") if k in res)
    res["batch_vs_single_plain_fp64"] = best / max(res["single_plain_fp64"]["converged_solves_s"], 1e-30)
    return res, conv_phys, conv_states


def run_warm_start(fv, torch, dev, levels, n_train, n_test, epochs, B=64, plain_single_s=None, train_set=None):
    """Learned warm start on the laminar hybrid NACA 0012 case.

    Training data: the converged members of a batched solve, given as
    train_set = (conditions, device states), or else n_train conditions (seed 11)
    solved here in batches of B from freestream (starter + main).  They train
    the message-passing network (4 layers, width 64; BF16 tensor-core GEMMs,
    FP32 accumulation, Adam) on the GPU.  n_test held-out conditions (seed
    12, same distributions) are then solved twice in batches of at most B on
    the FP32-preconditioned path: from freestream with the starter, and from
    the network's prediction without it (members that do not converge fall
    back to freestream).  Reported:
    nonlinear steps, wall time (CUDA events), initial-state error relative to
    the converged state, the largest difference of the two converged states
    and of their Cl/Cd, and the warm-started batch's rate against one plain
    FP64 solve."""
    import collections

    from fvens_gb300.mpnn import MPNN, diverged, fallback_solve, output_scale, train
    m, _ = _laminar_mesh(fv, levels)
    phs_tr = _laminar_conditions(fv, n_train, 11)
    phs_te = _laminar_conditions(fv, n_test, 12)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    keep_phys, keep_u, gen_s = [], [], 0.0
    if train_set is not None:
        keep_phys, keep_u = list(train_set[0]), list(train_set[1])
        n_train = 0
    for s in range(0, n_train, B):
        plist = phs_tr[s:s + B]
        main, solvers = _laminar_solvers(fv, m, plist, 4)
        u = _freestream_field(torch, dev, main, m.nelem)
        t, stats = _timed_solve(torch, solvers, u, all_members=True)
        gen_s += t
        uv = u.view(len(plist), m.nelem, 4)
        for k, st in enumerate(stats):
            if st["status"] == 0:
                keep_phys.append(plist[k])
                keep_u.append(uv[k].clone())
        del main, solvers, u
    targets = torch.stack(keep_u)
    uinf = np.array([[1.0, np.cos(p.aoa), np.sin(p.aoa), 1.0 / (p.gamma * p.Minf ** 2) / (p.gamma - 1) + 0.5]
                     for p in keep_phys])
    net = MPNN(m, layers=4, wall_markers=(2,), seed=11)
    net.set_scale(output_scale(targets.cpu().numpy(), uinf))
    a, b = ev(), ev()
    a.record()
    losses = train(net, keep_phys, targets, epochs=epochs, batch=16, lr=2e-3, lr_final=1e-4, seed=0)
    b.record()
    torch.cuda.synchronize()
    train_s = a.elapsed_time(b) / 1e3
    del targets, keep_u
    out = {"mesh_cells": m.nelem, "train_conditions": n_train if train_set is None else "the batched variant's members",
           "train_converged": len(keep_phys),
           "test_conditions": n_test, "epochs": epochs, "train_batch": 16, "params": net.nparams,
           "data_generation_s": gen_s, "training_s": train_s, "loss_first_last": [losses[0], losses[-1]]}
    agg = {k: dict(seconds=0.0, steps=[], res0=[], status=collections.Counter()) for k in ("freestream", "warm")}
    fb = dict(seconds=0.0, members=0, converged=0, stalled_kept=0, free_converged_of_kept=0)
    err_ratio, du, dcl, dcd, pred_s = [], [], [], [], 0.0
    for s in range(0, n_test, B):
        plist = phs_te[s:s + B]
        nb = len(plist)
        main, solvers = _laminar_solvers(fv, m, plist, 4)
        u_free = _freestream_field(torch, dev, main, m.nelem)
        u0_free = u_free.clone()
        t, st_free = _timed_solve(torch, solvers, u_free, all_members=True)
        agg["freestream"]["seconds"] += t
        main_w, solvers_w = _laminar_solvers(fv, m, plist, 4, starter=False)
        u_warm = torch.empty_like(u_free)
        a, b = ev(), ev()
        a.record()
        net.predict(plist, u_warm)
        b.record()
        torch.cuda.synchronize()
        pred_s += a.elapsed_time(b) / 1e3
        u0_warm = u_warm.clone()
        t, st_warm = _timed_solve(torch, solvers_w, u_warm, all_members=True)
        agg["warm"]["seconds"] += t + a.elapsed_time(b) / 1e3
        # the network's result judged: members whose solve from the prediction diverged (or
        # ended no lower than it started) restart from freestream; a stall or the step limit
        # is kept (mpnn.diverged)
        st_fb = [dict(x) for x in st_warm]
        starter_fb = fv.SteadyBackwardEulerSolver(
            fv.FlowFV(m, plist, fv.numerics_cfg(flux="ROE", gradient="NONE"), LAMINAR_BCS), pc="ilu0", precision=4,
            **LAMINAR_START)
        u_fb = u_warm.clone()
        a2, b2 = ev(), ev()
        a2.record()
        fell = fallback_solve(main_w, starter_fb, solvers_w[-1], u_fb, st_fb, judge=diverged)
        fb["stalled_kept"] += sum(1 for x in st_warm if x["status"] != 0) - len(fell)
        fb["free_converged_of_kept"] += sum(1 for k, x in enumerate(st_warm)
                                            if x["status"] != 0 and k not in fell and st_free[k]["status"] == 0)
        b2.record()
        torch.cuda.synchronize()
        fb["seconds"] += a2.elapsed_time(b2) / 1e3
        fb["members"] += len(fell)
        fb["converged"] += sum(1 for x in st_fb if x["status"] == 0)
        del starter_fb, u_fb
        for tag, sts in (("freestream", st_free), ("warm", st_warm)):
            agg[tag]["status"].update(int(x["status"]) for x in sts)
            agg[tag]["steps"] += [int(x["steps"]) for x in sts]
            agg[tag]["res0"] += [float(x["res0"]) for x in sts if x["res0"] > 0]
        uf = u_free.view(nb, m.nelem, 4)
        uw = u_warm.view(nb, m.nelem, 4)
        for k in range(nb):
            if st_free[k]["status"] != 0:
                continue
            ref = uf[k]
            e0 = torch.linalg.norm(u0_free.view(nb, m.nelem, 4)[k] - ref)
            e1 = torch.linalg.norm(u0_warm.view(nb, m.nelem, 4)[k] - ref)
            err_ratio.append(float(e1 / e0))
            if st_warm[k]["status"] == 0:
                du.append(float((uw[k] - ref).abs().max() / ref.abs().max()))
        cf = main.surface_data(u_free, 2)
        cw = main_w.surface_data(u_warm, 2)
        for k in range(nb):
            if st_free[k]["status"] == 0 and st_warm[k]["status"] == 0:
                dcl.append(float(abs(cw[k, 0] - cf[k, 0])))
                dcd.append(float(abs(cw[k, 1] - cf[k, 1]) / abs(cf[k, 1])))
        del main, solvers, main_w, solvers_w, u_free, u0_free, u_warm, u0_warm
    for tag in agg:
        conv = agg[tag]["status"].get(0, 0)
        st = agg[tag]
        out[tag] = {"seconds": st["seconds"], "converged": conv, "converged_solves_s": conv / st["seconds"],
                    "main_steps_mean": float(np.mean(st["steps"])), "main_steps_max": int(np.max(st["steps"])),
                    "main_initial_residual_geomean": float(np.exp(np.mean(np.log(st["res0"])))) if st["res0"] else None,
                    "status_counts": {str(k): v for k, v in st["status"].items()}}
    out["freestream"]["note"] = "main-solve steps; a first-order starter ran before each batch"
    out["warm"]["prediction_s"] = pred_s
    fb_s = out["warm"]["seconds"] + fb["seconds"]
    out["warm_with_fallback"] = {"seconds": fb_s, "converged": fb["converged"], "fallback_members": fb["members"],
                                 "fallback_s": fb["seconds"], "converged_solves_s": fb["converged"] / fb_s,
                                 "judge": "fall back when the solve from the prediction diverged or ended no lower "
                                          "than it started; a stall or the step limit is kept",
                                 "stalled_kept": fb["stalled_kept"],
                                 "stalled_kept_converged_from_freestream": fb["free_converged_of_kept"]}
    out["initial_error_ratio_mean"] = float(np.mean(err_ratio)) if err_ratio else None
    out["initial_error_ratio_max"] = float(np.max(err_ratio)) if err_ratio else None
    q = lambda v, f: float(np.quantile(v, f)) if v else None
    out["converged_state_rel_diff"] = {"median": q(du, 0.5), "p90": q(du, 0.9), "max": q(du, 1.0),
                                       "within_1e-8": sum(1 for x in du if x <= 1e-8), "members": len(du)}
    out["cl_abs_diff"] = {"median": q(dcl, 0.5), "max": q(dcl, 1.0)}
    out["cdp_rel_diff"] = {"median": q(dcd, 0.5), "max": q(dcd, 1.0),
                           "within_1e-8": sum(1 for x in dcd if x <= 1e-8)}
    out["warm_vs_freestream"] = out["warm"]["converged_solves_s"] / max(out["freestream"]["converged_solves_s"], 1e-30)
    out["warm_with_fallback_vs_freestream"] = (out["warm_with_fallback"]["converged_solves_s"] /
                                               max(out["freestream"]["converged_solves_s"], 1e-30))
    if plain_single_s:
        out["warm_batch_vs_single_plain_fp64"] = out["warm"]["converged_solves_s"] * plain_single_s
    return out


LARGE_MESH = [2048, 1024, 20.0, 96, 2e-5, 1.05, 96, 9]


def _large_case(fv):
    m = fv.UMesh.generate(fv.MESH_NACA_OGRID, LARGE_MESH, reorder=1)
    ph = fv.physics_cfg(Minf=0.75, aoa_deg=2.0, Reinf=5000.0, Tinf=288.15, Pr=0.72, viscous=True)
    bcs = [(2, "adiabaticwall", (0.0,)), (4, "farfield", ())]
    main = fv.FlowFV(m, ph, fv.numerics_cfg(flux="HLLC", gradient="LEASTSQUARES", reconstruction="BARTHJESPERSEN"),
                     bcs)
    start = fv.FlowFV(m, ph, fv.numerics_cfg(flux="HLLC", gradient="NONE"), bcs)
    return m, main, start


def run_large(fv, torch, dev, peak_gbs, solve=True):
    """Large single instance: hybrid NACA 0012 viscous mesh of 2048 x 1024
    O-grid cells (96 quad boundary-layer rings from 2e-5 chords, growth 1.05;
    triangles outside; 3,997,696 cells), M 0.75, AoA 2 deg, Re 5000; HLLC,
    least squares, Barth-Jespersen.  Each kernel is timed alone (CUDA events,
    an L2 eviction before every launch) at a perturbed freestream state:
    residual Gfaces/s, Jacobian blocks/s, FP32 ILU(0) apply GB/s, as fractions
    of the HBM copy peak.  With solve: the end-to-end solve from freestream
    (starter + main to ||R|| < 1e-10) on the FP32-preconditioned path and on
    the plain FP64 path."""
    import ctypes
    t0 = time.perf_counter()
    m, main, start = _large_case(fv)
    t_mesh = time.perf_counter() - t0
    S = fv.SteadyBackwardEulerSolver(main, cfl_min=100, cfl_max=5000, tolerance=1e-10, abs_tolerance=1,
                                     max_timesteps=1, pc="ilu0", precision=4, matrix_free=1)
    rng = np.random.default_rng(3)
    u = torch.tensor(np.tile(main.freestream()[0], (m.nelem, 1)) * (1 + 0.02 * rng.uniform(-1, 1, (m.nelem, 4))),
                     device=dev)
    block_sizes = main.autotune(u)
    out = {"cells": m.nelem, "faces": m.naface, "boundary_faces": m.nbface, "mesh_setup_s": t_mesh,
           "residual_block_sizes": block_sizes}
    for name, which in (("residual", 0), ("face_flux", 1), ("gradients", 6), ("jacobian", 2), ("ilu0_setup", 5),
                        ("ilu0_apply", 3)):
        a, b = ctypes.c_double(), ctypes.c_double()
        fv.check(fv.lib().fv_solver_time_kernel(S._h, fv._vp(fv.dptr(u)), which, 10, ctypes.byref(a), ctypes.byref(b)))
        gbs = b.value / (a.value * 1e-3) / 1e9
        out[name] = {"ms": a.value, "model_bytes": b.value, "gbs": gbs, "frac_hbm": gbs / peak_gbs}
    nb = m.nelem + 2 * (m.naface - m.nbface)
    out["residual_gfaces_s"] = m.naface / (out["residual"]["ms"] * 1e-3) / 1e9
    out["jacobian_blocks_s"] = nb / (out["jacobian"]["ms"] * 1e-3)
    out["ilu0_sweep_gbs"] = out["ilu0_apply"]["gbs"]
    del S
    if solve:
        for tag, prec in (("solve_fp32_precond", 4), ("solve_plain_fp64", 8)):
            S1 = fv.SteadyBackwardEulerSolver(start, precision=prec, **LARGE_STARTER)
            S2 = fv.SteadyBackwardEulerSolver(main, precision=prec, **LARGE_MAIN)
            u.copy_(torch.tensor(np.tile(main.freestream()[0], (m.nelem, 1)), device=dev))
            t, st = _timed_solve(torch, [S1, S2], u)
            cl = main.surface_data(u, 2)[0]
            out[tag] = {"solve_s": t, "main_steps": st["steps"], "linear_iters": st["lin_iters"],
                        "status": st["status"], "res0": st["res0"], "res": st["res"],
                        "max_main_steps": LARGE_MAIN["max_timesteps"], "cl_cdp_cdsf": [float(x) for x in cl]}
            del S1, S2
        a, b = out["solve_fp32_precond"], out["solve_plain_fp64"]
        if a["status"] == 0 and b["status"] == 0:
            out["fp32_vs_plain_fp64"] = b["solve_s"] / a["solve_s"]
    return out


LARGE_STARTER = dict(cfl_min=25, cfl_max=500, tolerance=1e-1, abs_tolerance=0, max_timesteps=100, nl_update=2,
                     min_relax=0.2, pc="ilu0")
LARGE_MAIN = dict(cfl_min=100, cfl_max=5000, tolerance=1e-10, abs_tolerance=1, max_timesteps=100, nl_update=2,
                  min_relax=0.2, pc="ilu0", matrix_free=1)


# ----------------------------- oracle legs ----------------------------------

def _oracle_case_from_arrays(arrs):
    from oracle import orc
    om = orc.Mesh(arrs["coords"], arrs["nnode"], arrs["inpoel"], arrs["bface"], arrs["btag"])
    od1 = orc.Disc(om, **PHYS, **NUM_START, bcs=BCS)
    od2 = orc.Disc(om, **PHYS, **NUM_MAIN, bcs=BCS)
    return om, od1, od2


def _oracle_case(m):
    """Oracle discretisations on the product mesh m (same cell order)."""
    _, od1, od2 = _oracle_case_from_arrays(m.export())
    return od1, od2


def oracle_solve(od1, od2, u, order=None):
    """One complete solve of the workload on the oracle: the starter and the
    main solve with the workload's settings, ILU(0) in the elimination order
    `order` (cell at each position; None: natural order, as PETSc's).
    Returns (u, starter stats, main stats, starter seconds, main seconds)."""
    S, M = STARTER, MAIN
    t0 = time.perf_counter()
    u, st1 = od1.steady_solve(u, cflmin=S["cfl_min"], cflmax=S["cfl_max"], tol=S["tolerance"],
                              maxiter=S["max_timesteps"], abs_tol=bool(S["abs_tolerance"]), pc="ilu0",
                              nl_update="bounded", min_relax=S["min_relax"], lin_rtol=S.get("ksp_rtol", 0.1),
                              order=order)
    t1 = time.perf_counter()
    u, st2 = od2.steady_solve(u, cflmin=M["cfl_min"], cflmax=M["cfl_max"], tol=M["tolerance"],
                              maxiter=M["max_timesteps"], abs_tol=bool(M["abs_tolerance"]), pc="ilu0",
                              nl_update="bounded", min_relax=M["min_relax"], matrix_free=bool(M["matrix_free"]),
                              lin_rtol=M.get("ksp_rtol", 0.1), mf_eps=M.get("mf_eps", 1e-7), order=order)
    t2 = time.perf_counter()
    return u, st1, st2, t1 - t0, t2 - t1


def _oracle_steps(od, cfg, u, nsteps, lin_maxit):
    """nsteps pseudo-time steps on the oracle with every linear solve running
    exactly lin_maxit FGMRES iterations (relative tolerance out of reach)."""
    t0 = time.perf_counter()
    od.steady_solve(u, cflmin=cfg["cfl_min"], cflmax=cfg["cfl_max"], tol=1e-30, maxiter=nsteps, pc="ilu0",
                    matrix_free=bool(cfg.get("matrix_free", 0)), nl_update="bounded", min_relax=cfg["min_relax"],
                    abs_tol=True, lin_rtol=1e-14, lin_maxit=lin_maxit, mf_eps=cfg.get("mf_eps", 1e-7))
    return (time.perf_counter() - t0) / nsteps


def _oracle_step_model(od, cfg, u, budget_s):
    """Per-step and per-Krylov-iteration cost of the oracle: timed steps with 1
    and with 8 FGMRES iterations each, fitted to t = a + b * iterations."""
    t1 = _oracle_steps(od, cfg, u, 1, 1)
    n = max(1, min(10, int(0.25 * budget_s / max(t1, 1e-3))))
    t1 = _oracle_steps(od, cfg, u, n, 1)
    t8 = _oracle_steps(od, cfg, u, n, 8)
    b = max((t8 - t1) / 7.0, 0.0)
    return t1 - b, b, n


def _fixture_counts():
    """Step and Krylov counts of the oracle's own complete solve of the
    workload (recorded with the committed converged-state fixture)."""
    if not os.path.exists(C2_FIXTURE):
        return None
    z = np.load(C2_FIXTURE)
    s = z["solve_counts"]
    return {"starter": {"steps": int(s[0]), "lin_iters": int(s[1])}, "main": {"steps": int(s[2]),
                                                                              "lin_iters": int(s[3])},
            "recorded_seconds": float(z["solve_seconds"]), "recorded_threads": int(z["solve_threads"])}


def oracle_parity(m, main, ud):
    """The GPU's numbers on this workload against the oracle: the
    second-order residual at the GPU's converged state and at a seeded 5 %
    perturbation of freestream (max |difference| over the largest sum of
    |face flux x length| of a cell), Cl, CDp at the converged state, and the
    converged state and Cl, CDp against the oracle's own complete solve of
    the workload (committed fixture: the state at sampled cells)."""
    import torch
    _, od2 = _oracle_case(m)
    out = {}
    u_conv = ud.detach().cpu().numpy().reshape(m.nelem, 4)
    rng = np.random.default_rng(1234)
    u_pert = np.tile(od2.freestream(), (m.nelem, 1)) * (1 + 0.05 * rng.uniform(-1, 1, (m.nelem, 4)))
    area = m.geometry()["area"]
    for tag, u in (("converged", u_conv), ("perturbed", u_pert)):
        udev = torch.tensor(u, device=ud.device)
        r = torch.zeros_like(udev)
        main.compute_residual(udev, r)
        main.synchronize()
        ro, _ = od2.residual(u)
        out[f"residual_{tag}_max_rel_err"] = float(np.abs(r.cpu().numpy() - ro).max() / od2.flux_scale(u).max())
        if tag == "converged":
            # the solver's norm (area-weighted energy residual) of the oracle's
            # residual at the GPU's converged state
            out["oracle_residual_norm_at_gpu_state"] = float(np.sqrt(np.sum(ro[:, 3] ** 2 * area)))
    cg = main.surface_data(ud, 2)[0]
    co = od2.surface_data(u_conv, 2)
    out["cl_cdp_rel_err"] = [float(abs(cg[k] - co[k]) / abs(co[k])) for k in (0, 1)]
    if os.path.exists(C2_FIXTURE) and m.nelem == 183296:
        z = np.load(C2_FIXTURE)
        perm = m.export()["perm"]
        inv = np.empty_like(perm)
        inv[perm] = np.arange(len(perm))
        ug = u_conv[inv[z["cells"]]]
        uo = z["states"]
        out["vs_oracle_converged_solve"] = {
            "state_rel_diff": float(np.abs(ug - uo).max() / np.abs(uo).max()),
            "cells_compared": int(len(z["cells"])),
            "cl_cdp_rel_diff": [float(abs(cg[k] - z["functionals"][k]) / abs(z["functionals"][k])) for k in (0, 1)]}
    return out


def cpu_baseline(m, budget_s, u_state=None, counts=None):
    """The oracle (the CPU restatement of the reference's path, natural-order
    ILU(0) as PETSc's) on the host cores, on a bounded sample: pseudo-time
    steps of the starter and of the main solve with pinned FGMRES iteration
    counts give the cost per step and per Krylov iteration, scaled to the step
    and Krylov counts of the oracle's own complete solve of the workload
    (counts: {"starter": {...}, "main": {...}}; default: the committed
    fixture's record).  With u_state (host array of the state the GPU kernels
    were timed at), the oracle's residual, FP64 Jacobian assembly, ILU(0)
    factorisation and ILU(0) apply are timed there too."""
    from oracle import orc
    nthreads = _host_threads()
    orc.set_threads(nthreads)
    counts = counts or _fixture_counts()
    if counts is None:
        return {"unavailable": "no record of the oracle's complete solve (tests/golden fixture absent)"}
    od1, od2 = _oracle_case(m)
    u0 = np.tile(od2.freestream(), (m.nelem, 1))
    a1, b1, n1 = _oracle_step_model(od1, STARTER, u0, 0.4 * budget_s)
    a2, b2, n2 = _oracle_step_model(od2, MAIN, u0, 0.6 * budget_s)
    st, mn = counts["starter"], counts["main"]
    solve_s = (a1 * st["steps"] + b1 * st["lin_iters"]) + (a2 * mn["steps"] + b2 * mn["lin_iters"])
    kernels = {}
    if u_state is not None:
        t = od2.time_kernels(u_state, "ilu0", reps=5)
        kernels = {"kernels_ms": {"residual": 1e3 * t["residual"], "jacobian": 1e3 * t["jacobian"],
                                  "ilu0_setup": 1e3 * t["pc_setup"], "ilu0_apply": 1e3 * t["pc_apply"]},
                   "kernels_note": f"oracle at the state the GPU kernels were timed at, median of 5 after one "
                                   f"untimed call; residual and FP64 Jacobian on {nthreads} threads, ILU(0) "
                                   f"factorisation and apply sequential in natural order (as PETSc's)"}
    return {"value": 1.0 / solve_s, "unit": "solves/s", "cores": nthreads, "kind": "port",
            "sample": f"2 x {n1} starter + 2 x {n2} main pseudo-time steps of the same workload on the oracle with "
                      f"1 and 8 FGMRES(30) iterations per step (natural-order ILU(0)); per step {a1:.3f} / {a2:.3f} s "
                      f"+ per Krylov iteration {b1:.3f} / {b2:.3f} s, scaled to the oracle's own complete solve: "
                      f"{st['steps']} + {mn['steps']} steps and {st['lin_iters']} + {mn['lin_iters']} Krylov "
                      f"iterations (the reference arm times that solve whole)", **kernels}


def run_reference(args):
    """The reference's CPU path as restated by the oracle (the reference itself
    does not build here: PETSc, Eigen, Boost and MPI are absent), on all host
    threads: ONE complete solve of the workload from freestream, timed whole
    (mesh built by the oracle's own generator; the product library is not
    loaded).  Under torchrun only rank 0 runs."""
    rank, world, local = _dist()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from fvens_gb300 import build as fvbuild
    if not os.path.exists(fvbuild.ORACLE_LIB):
        fvbuild.build_oracle()
    from oracle import meshgen, orc
    nthreads = _host_threads()
    orc.set_threads(nthreads)
    t0 = time.perf_counter()
    arrs = meshgen.naca_ogrid(*(SMALL_MESH if args.small else MESH))
    om, od1, od2 = _oracle_case_from_arrays(arrs)
    t_mesh = time.perf_counter() - t0
    u = np.tile(od2.freestream(), (om.nelem, 1))
    # ILU(0) in the GPU's block-colour elimination order, stored with the
    # committed fixture (PETSc's natural order diverges on this workload)
    order, order_note = None, "natural order (as PETSc's)"
    if os.path.exists(C2_FIXTURE) and not args.small:
        order = np.load(C2_FIXTURE)["order"]
        order_note = "the GPU's block-colour elimination order (parts of <= 128 cells)"
    u, st1, st2, ts, tm = oracle_solve(od1, od2, u, order)
    solve_s = ts + tm
    value = 1.0 / solve_s
    fun = od2.surface_data(u, 2)
    solve = {"starter_steps": st1["steps"], "starter_linear_iters": st1["lin_iters"], "main_steps": st2["steps"],
             "linear_iters": st2["lin_iters"], "converged": st2["status"] == 0, "final_res": float(st2["res"]),
             "cl_cdp": [float(fun[0]), float(fun[1])], "starter_s": ts, "main_s": tm, "mesh_setup_s": t_mesh,
             "ilu0_order": order_note}
    if os.path.exists(C2_FIXTURE) and not args.small:
        z = np.load(C2_FIXTURE)
        solve["vs_committed_oracle_solve"] = {
            "state_rel_diff": float(np.abs(u[z["cells"]] - z["states"]).max() / np.abs(z["states"]).max()),
            "cl_cdp_rel_diff": [float(abs(fun[k] - z["functionals"][k]) / abs(z["functionals"][k])) for k in (0, 1)]}
    cpu = f"{platform.machine()}, {nthreads} threads"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": 1, "warmup": 0, "ms_per_step": solve_s * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded NACA 0012 O-grid, the oracle's own generator; freestream start)",
            "config": workload_config(world, args.small),
            "solve": solve,
            "note": f"one complete solve timed whole (it takes minutes); the requested --steps {args.steps} "
                    f"--warmup {args.warmup} are not repeated",
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nthreads, "kind": "port",
                             "sample": f"one complete solve of the workload on the oracle ({cpu}; ILU(0) in "
                                       f"{order_note}): {st1['steps']} + {st2['steps']} steps, "
                                       f"{st1['lin_iters']} + {st2['lin_iters']} Krylov iterations"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------- kernel micro-benchmarks ------------------------

def run_kernel(args):
    """Profiling aid: R launches of one kernel family, mean time per launch
    (CUDA events) after three untimed launches."""
    import torch

    import fvens_gb300 as fv
    from fvens_gb300 import build as fvbuild
    if not os.path.exists(fv.LIB_PATH):
        fvbuild.build_library()
    dev = torch.device("cuda", 0)
    R = args.reps
    if args.kernel == "fp64peak":
        rate, ms = fv.fp64_peak(R)
        print(f"fp64 peak: {rate / 1e9:.1f} G FMA/s = {2 * rate / 1e12:.4f} TFLOP/s (best launch {ms:.3f} ms)")
        return
    if args.kernel == "mpnn":
        return _kernel_mpnn(fv, torch, dev, args.batch_members, R)
    m, main, start = build_case(fv)
    rng = np.random.default_rng(1234)
    u = torch.tensor(np.tile(main.freestream()[0], (m.nelem, 1)) * (1 + 0.05 * rng.uniform(-1, 1, (m.nelem, 4))),
                     device=dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    if args.kernel == "residual":
        r = torch.zeros_like(u)
        dt = torch.zeros(m.nelem, dtype=torch.float64, device=dev)
        call = lambda: main.compute_residual(u, r, True, dt)
        what = f"residual ({m.nelem} cells, {m.naface} faces)"
    else:
        A = fv.BlockMatrix(start, 4)
        if args.kernel == "jacobian":
            call = lambda: start.assemble_jacobian(u, A)
            what = f"FP32 first-order Jacobian ({m.nelem} cells)"
        else:
            B = args.ilu_batch
            disc = start
            if B > 1:  # B copies of the workload's condition in one batched discretisation
                disc = fv.FlowFV(m, [fv.physics_cfg(**PHYS)] * B, fv.numerics_cfg(**NUM_START), BCS)
                u = u.repeat(B, 1)
                A = fv.BlockMatrix(disc, 4)
            disc.assemble_jacobian(u, A)
            A.add_diagonal(torch.tensor(np.tile(m.geometry()["area"] / 0.01, B), device=dev))  # pseudo-time term
            P = fv.Preconditioner(disc, A, "ilu0", part_size=args.part)
            P.setup()
            x = torch.tensor(rng.normal(size=(B * m.nelem, 4)), device=dev)
            z = torch.zeros_like(x)
            call = lambda: P.apply(x, z)
            what = f"FP32 ILU(0) apply ({B} x {m.nelem} cells, parts of <= {args.part})"
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    a, b = ev(), ev()
    a.record()
    for _ in range(R):
        call()
    b.record()
    torch.cuda.synchronize()
    print(f"{what}: {a.elapsed_time(b) / R:.4f} ms per launch sequence")


def _kernel_mpnn(fv, torch, dev, B, steps):
    from fvens_gb300.mpnn import MPNN
    m, _ = _laminar_mesh(fv, 0)
    phs = _laminar_conditions(fv, B, 11)
    net = MPNN(m, layers=4, wall_markers=(2,), seed=11)
    net.set_scale(np.array([0.05, 0.1, 0.1, 0.2], np.float32))
    tgt = torch.empty((B * m.nelem, 4), dtype=torch.float64, device=dev)
    net.predict(phs, tgt)
    tgt *= 1.01
    u = torch.empty_like(tgt)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for path in ("mma_sync", "tcgen05"):  # the default path first (a launch list of the first launches covers it)
        net.set_gemm_path(path)
        for _ in range(3):
            net.train_step(phs, tgt, 1e-4)
        torch.cuda.synchronize()
        a.record()
        for _ in range(steps):
            net.train_step(phs, tgt, 1e-4)
        b.record()
        torch.cuda.synchronize()
        t_train = a.elapsed_time(b) / steps
        a.record()
        for _ in range(steps):
            net.predict(phs, u)
        b.record()
        torch.cuda.synchronize()
        print(f"mpnn ({path} forward GEMMs): train step {t_train:.3f} ms, predict {a.elapsed_time(b) / steps:.3f} ms, "
              f"{B} conditions x {m.nelem} cells")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--kernel", choices=["residual", "ilu", "jacobian", "mpnn", "fp64peak"],
                    help="profiling aid: time one kernel family instead of the benchmark")
    ap.add_argument("--reps", type=int, default=5, help="launches timed by --kernel")
    ap.add_argument("--part", type=int, default=128, help="--kernel ilu: cells per part of the block-colour order")
    ap.add_argument("--batch-members", type=int, default=16, help="--kernel mpnn: conditions per training step")
    ap.add_argument("--ilu-batch", type=int, default=1, help="--kernel ilu: batch members (copies of the condition)")
    ap.add_argument("--small", action="store_true",
                    help="a 64 x 32 O-grid of the workload's family (CPU tests of the launch path; named so in "
                         "config.workload)")
    ap.add_argument("--plain", action="store_true", help="FP64 Jacobian and preconditioner (the plain path)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--nvtx", action="store_true", help="profiling aid: NVTX range around each main solve")
    ap.add_argument("--no-variants", action="store_true", help="skip every comparison variant")
    ap.add_argument("--no-graph", action="store_true",
                    help="profiling aid: issue every launch from the host instead of replaying a CUDA graph")
    ap.add_argument("--main-steps", type=int, default=0,
                    help="profiling aid: cap the main solve at this many steps (the solve then reports status 4)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--e2e-solves", type=int, default=5, help="solves timed end to end through host buffers")
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="skip the batched laminar and warm-start variants")
    ap.add_argument("--laminar-levels", type=int, default=2,
                    help="refinements of the reference's 13,156-cell hybrid mesh for the laminar variants")
    ap.add_argument("--batch", type=int, default=64, help="conditions per batched laminar solve")
    ap.add_argument("--laminar-sgs", action="store_true", help="batched laminar variant: also block SGS")
    ap.add_argument("--warm-train", type=int, default=0,
                    help="training conditions of the learned warm-start variant, solved for it (0: train on the "
                         "batched variant's converged members)")
    ap.add_argument("--warm-test", type=int, default=16,
                    help="held-out conditions of the warm-start variant (0 skips it)")
    ap.add_argument("--warm-epochs", type=int, default=60, help="training epochs of the warm-start network")
    ap.add_argument("--no-large", dest="large", action="store_false", help="skip the ~4M-cell variant")
    ap.add_argument("--no-large-solve", dest="large_solve", action="store_false",
                    help="~4M-cell variant: kernel times only, no end-to-end solves")
    ap.add_argument("--large-steps", type=int, default=100,
                    help="~4M-cell variant: main-solve step limit of the end-to-end solves (the Barth-Jespersen "
                         "solve does not converge on this mesh; the two paths are compared per step)")
    args = ap.parse_args()
    LARGE_MAIN["max_timesteps"] = args.large_steps
    if args.no_graph:
        STARTER["use_graph"] = 0
        MAIN["use_graph"] = 0
    if args.main_steps > 0:
        MAIN["max_timesteps"] = args.main_steps
    if args.kernel:
        run_kernel(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
