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

MESH = [512, 256, 30.0, 0, 0, 1.02, 154, 3]
PHYS = dict(Minf=0.8, aoa_deg=1.25)
NUM_MAIN = dict(flux="HLLC", gradient="GREENGAUSS", reconstruction="VENKATAKRISHNAN", limiter_param=5.0)
NUM_START = dict(flux="HLLC", gradient="NONE")
BCS = [(2, "slipwall", ()), (4, "farfield", ())]
STARTER = dict(cfl_min=25, cfl_max=500, tolerance=1e-1, abs_tolerance=0, max_timesteps=100, nl_update=2,
               min_relax=0.2, pc="ilu0")
MAIN = dict(cfl_min=100, cfl_max=5000, tolerance=1e-10, abs_tolerance=1, max_timesteps=2000, nl_update=2,
            min_relax=0.2, pc="ilu0", matrix_free=1)
WORKLOAD = "naca0012_transonic_512x256_ogrid_g1.02_hllc_gg_venkat5"
# DRAM bytes (read + write) per launch from one ncu capture of this workload
# (profiles/naca0012_c2_main_solve_launch_list.md; the gradient pass counts k_grad only)
NCU_DRAM_BYTES = {"face_flux": 44611840, "gradients": 37975808}
METRIC = "solves/s to ||R||<1e-10 (transonic NACA0012, matrix-free FGMRES, FP32 Jacobian + FP32 block-colour ILU0)"


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
    from fvens_gb300.replicas import Replicas

    rank, world, local = _dist()
    if not os.path.exists(fv.LIB_PATH):
        fvbuild.build_library()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    reps = Replicas("nccl", dev)
    m, main, start = build_case(fv)
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
    e2e_value = reps.throughput(args.steps, t1 - t0)
    cl = main.surface_data(ud, 2)[0]
    u_conv = ud.clone()
    variants = {} if args.no_variants else run_variants(fv, torch, dev, m, main, start, u0d, prec, args)
    ud.copy_(u_conv)

    # per-kernel timing (roofline) at the converged state; time shares of one
    # solve from the launch counts per step / per Krylov iteration
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
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
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
        "config": {"workload": WORKLOAD, "cells": m.nelem, "faces": nf, "batch": 1,
                   "parallelism": f"replicas{world}" if world > 1 else "single",
                   "l2": "working set > L2 (no flush needed)",
                   "starter_steps": s1["steps"], "main_steps": steps_main, "linear_iters": lin_main,
                   "converged": converged, "final_res": s2["res"],
                   "cl_cdp": [float(cl[0]), float(cl[1])],
                   "residual_block_sizes": block_sizes},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(u0.nbytes),
                "d2h_bytes_per_step": int(u0.nbytes)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": kern[dom]["gbs"], "peak": hbm_peak,
                     "unit": "GB/s", "frac": kern[dom]["gbs"] / hbm_peak,
                     "traffic": NCU_DRAM_BYTES.get(dom), "peak_source": peak_src,
                     "note": "FP64-pipe bound (ncu: FP64 pipe 87 % busy, DRAM 4 %)" if dom != "ilu0_apply" else
                             "latency bound level walk"},
        "kernels": kern,
        "solve_time_shares_ms": share_ms,
        "variants": variants,
        "residual_gfaces_s": nf / (kern["residual"]["ms"] * 1e-3) / 1e9,
        "jacobian_blocks_s": nblocks / (kern["jacobian"]["ms"] * 1e-3),
        "ilu0_sweep_gbs": kern["ilu0_apply"]["gbs"],
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu:
        u_host = u_conv.cpu().numpy().reshape(m.nelem, 4)
        line["cpu_baseline"] = cpu_baseline(m, s1, s2, args.cpu_seconds, u_host)
        line["oracle_parity"] = oracle_parity(m, main, u_conv)
    if rank == 0:
        print(json.dumps(line), flush=True)
    reps.close()


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
    solves (run_batched)."""
    out = {}
    u = torch.empty_like(u0d)
    P1 = fv.SteadyBackwardEulerSolver(start, precision=8, **STARTER)
    P2 = fv.SteadyBackwardEulerSolver(main, precision=8, **MAIN)
    u.copy_(u0d)
    t, st = _timed_solve(torch, [P1, P2], u)
    out["plain_fp64_cold"] = {"solves_s": 1.0 / t, "s_per_solve": t, "main_steps": st["steps"],
                              "linear_iters": st["lin_iters"], "converged": st["status"] == 0, "res": st["res"]}
    del P1, P2
    if args.large:
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        out["large_4m_kernels"] = run_large(fv, torch, dev, float(peaks.get("hbm_gbs", 6800.0)))
    out["batched_laminar"] = bl = run_batched(fv, torch, dev)
    if args.warm_train > 0:
        out["warm_start_laminar"] = run_warm_start(fv, torch, dev, args.warm_train, args.warm_test, args.warm_epochs,
                                                   plain_single_s=bl["single_plain_fp64"]["seconds"])
    return out


LAMINAR_BCS = [(4, "inflowoutflow", ()), (2, "adiabaticwall", (0.0,))]


def _laminar_mesh(fv):
    """The reference's hybrid NACA 0012 mesh (13,156 cells) with its
    boundary-layer lines kept whole in the preconditioner's parts."""
    z = np.load(os.path.join(ROOT, "tests", "golden", "naca0012_lam_hybrid_1_mesh.npz"))
    m = fv.UMesh.from_arrays(z["coords"], z["nnode"].astype(np.int32), z["inpoel"], z["bface"],
                             z["btag"].astype(np.int32), reorder=1)
    return m, m.find_lines(10.0)[0]


def _laminar_conditions(fv, n, seed):
    """n seeded laminar conditions: M ~ U[0.3, 0.7], AoA ~ U[-4, 4] deg,
    Re ~ U[2000, 10000], Pr 0.72, T 288.15 K."""
    rng = np.random.default_rng(seed)
    M, A, Re = rng.uniform(0.3, 0.7, n), rng.uniform(-4, 4, n), rng.uniform(2000, 10000, n)
    return [fv.physics_cfg(Minf=float(M[k]), aoa_deg=float(A[k]), Reinf=float(Re[k]), Tinf=288.15, Pr=0.72,
                           viscous=True) for k in range(n)]


def _laminar_solvers(fv, m, plist, prec, starter=True, pc="ilu0"):
    """(discretisation, [starter solver,] main solver) for the conditions plist:
    first-order starter to a relative 1e-1 (at most 50 steps), then the
    second-order main solve to the absolute 1e-10."""
    main = fv.FlowFV(m, plist, fv.numerics_cfg(flux="ROE", gradient="LEASTSQUARES"), LAMINAR_BCS)
    S2 = fv.SteadyBackwardEulerSolver(main, cfl_min=200, cfl_max=5000, tolerance=1e-10, abs_tolerance=1,
                                      max_timesteps=600, pc=pc, nl_update=2, precision=prec)
    if not starter:
        return main, [S2]
    start = fv.FlowFV(m, plist, fv.numerics_cfg(flux="ROE", gradient="NONE"), LAMINAR_BCS)
    S1 = fv.SteadyBackwardEulerSolver(start, cfl_min=200, cfl_max=1000, tolerance=1e-1, abs_tolerance=0,
                                      max_timesteps=50, pc=pc, nl_update=2, precision=prec)
    return main, [S1, S2]


def _freestream_field(torch, dev, disc, nelem):
    return torch.tensor(np.concatenate([np.tile(x, (nelem, 1)) for x in disc.freestream()]), device=dev)


def run_batched(fv, torch, dev, B=64, seed=7):
    """Batched solves of B laminar conditions (M ~ U[0.3, 0.7], AoA ~ U[-4, 4] deg,
    Re ~ U[2000, 10000], Pr 0.72, adiabatic wall; Roe, least squares) on the
    reference's hybrid NACA 0012 mesh (13,156 cells), all members in the same
    launches with FP32 Jacobians and ILU(0) (and with block SGS), against one
    member alone on the FP32 path and on the plain FP64 path."""
    import collections
    m, nlines = _laminar_mesh(fv)
    phs = _laminar_conditions(fv, B, seed)
    res = {"mesh_cells": m.nelem, "batch": B, "lines": nlines}
    for tag, plist, prec, pc in (("single_plain_fp64", phs[:1], 8, "ilu0"), ("single", phs[:1], 4, "ilu0"),
                                 ("batch", phs, 4, "ilu0"), ("batch_sgs", phs, 4, "sgs")):
        main, solvers = _laminar_solvers(fv, m, plist, prec, pc=pc)
        u = _freestream_field(torch, dev, main, m.nelem)
        t, stats = _timed_solve(torch, solvers, u, all_members=True)
        conv = sum(1 for st in stats if st["status"] == 0)
        res[tag] = {"seconds": t, "converged": conv, "members": len(plist), "converged_solves_s": conv / t,
                    "status_counts": dict(collections.Counter(int(st["status"]) for st in stats)),
                    "main_steps_max": max(st["steps"] for st in stats)}
    res["batch_vs_single_plain_fp64"] = (res["batch"]["converged_solves_s"] /
                                         max(res["single_plain_fp64"]["converged_solves_s"], 1e-30))
    return res


def run_warm_start(fv, torch, dev, n_train, n_test, epochs, B=64, plain_single_s=None):
    """Learned warm start on the laminar hybrid NACA 0012 case.

    n_train conditions (seed 11) are solved in batches of B from freestream
    (starter + main); the converged members train the message-passing network
    (4 layers, width 64; BF16 tensor-core GEMMs, FP32 accumulation, Adam) on
    the GPU.  n_test held-out conditions (seed 12, same distributions) are then
    solved twice in batches of B on the FP32-preconditioned path: from
    freestream with the starter, and from the network's prediction without it.
    Reported: nonlinear steps, wall time (CUDA events), initial-state error
    relative to the converged state, the largest difference of the two
    converged states and of their Cl/Cd, and the warm-started batch's rate
    against one plain FP64 solve."""
    import collections

    from fvens_gb300.mpnn import MPNN, fallback_solve, output_scale, train
    m, _ = _laminar_mesh(fv)
    phs_tr = _laminar_conditions(fv, n_train, 11)
    phs_te = _laminar_conditions(fv, n_test, 12)
    # training data: converged states of the batched solver
    ev = lambda: torch.cuda.Event(enable_timing=True)
    keep_phys, keep_u, gen_s = [], [], 0.0
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
        del main, solvers
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
    # held-out conditions: freestream + starter vs prediction, batches of B
    out = {"train_conditions": n_train, "train_converged": len(keep_phys), "test_conditions": n_test,
           "epochs": epochs, "train_batch": 16, "params": net.nparams, "data_generation_s": gen_s,
           "training_s": train_s, "loss_first_last": [losses[0], losses[-1]]}
    agg = {k: dict(seconds=0.0, steps=[], res0=[], status=collections.Counter()) for k in ("freestream", "warm")}
    fb = dict(seconds=0.0, members=0, converged=0)
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
        # the network's result judged: members that did not converge restart from freestream
        st_fb = [dict(x) for x in st_warm]
        starter_fb = fv.SteadyBackwardEulerSolver(
            fv.FlowFV(m, plist, fv.numerics_cfg(flux="ROE", gradient="NONE"), LAMINAR_BCS), cfl_min=200,
            cfl_max=1000, tolerance=1e-1, abs_tolerance=0, max_timesteps=50, pc="ilu0", nl_update=2, precision=4)
        u_fb = u_warm.clone()
        a2, b2 = ev(), ev()
        a2.record()
        fell = fallback_solve(main_w, starter_fb, solvers_w[-1], u_fb, st_fb)
        b2.record()
        torch.cuda.synchronize()
        fb["seconds"] += a2.elapsed_time(b2) / 1e3
        fb["members"] += len(fell)
        fb["converged"] += sum(1 for x in st_fb if x["status"] == 0)
        del starter_fb
        # freestream stats from the main solver (the starter's steps added)
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
        del main, solvers, main_w, solvers_w
    for tag in agg:
        conv = agg[tag]["status"].get(0, 0)
        st = agg[tag]
        out[tag] = {"seconds": st["seconds"], "converged": conv, "converged_solves_s": conv / st["seconds"],
                    "main_steps_mean": float(np.mean(st["steps"])), "main_steps_max": int(np.max(st["steps"])),
                    "main_initial_residual_geomean": float(np.exp(np.mean(np.log(st["res0"])))) if st["res0"] else None,
                    "status_counts": {str(k): v for k, v in st["status"].items()}}
    out["freestream"]["note"] = "main-solve steps; a first-order starter ran before each batch"
    out["warm"]["prediction_s"] = pred_s
    # with the fallback: the members the warm start did not converge, solved again from freestream
    fb_s = out["warm"]["seconds"] + fb["seconds"]
    out["warm_with_fallback"] = {"seconds": fb_s, "converged": fb["converged"], "fallback_members": fb["members"],
                                 "fallback_s": fb["seconds"], "converged_solves_s": fb["converged"] / fb_s}
    out["initial_error_ratio_mean"] = float(np.mean(err_ratio)) if err_ratio else None
    out["initial_error_ratio_max"] = float(np.max(err_ratio)) if err_ratio else None
    # both starts converged: how far apart are the two converged states?
    q = lambda v, f: float(np.quantile(v, f)) if v else None
    out["converged_state_rel_diff"] = {"median": q(du, 0.5), "p90": q(du, 0.9), "max": q(du, 1.0),
                                       "within_1e-8": sum(1 for x in du if x <= 1e-8), "members": len(du)}
    out["cl_abs_diff"] = {"median": q(dcl, 0.5), "max": q(dcl, 1.0)}
    out["cdp_rel_diff"] = {"median": q(dcd, 0.5), "max": q(dcd, 1.0),
                           "within_1e-8": sum(1 for x in dcd if x <= 1e-8)}
    out["warm_vs_freestream"] = out["warm"]["converged_solves_s"] / max(out["freestream"]["converged_solves_s"], 1e-30)
    if plain_single_s:
        out["warm_batch_vs_single_plain_fp64"] = out["warm"]["converged_solves_s"] * plain_single_s
    return out


LARGE_MESH = [2048, 1024, 20.0, 96, 2e-5, 1.05, 96, 9]


def run_large(fv, torch, dev, peak_gbs):
    """Large single-instance kernel throughput: hybrid NACA 0012 viscous mesh of
    2048 x 1024 O-grid cells (96 quad boundary-layer rings from 2e-5 chords,
    growth 1.05; triangles outside; 3,997,696 cells), M 0.75, AoA 2 deg,
    Re 5000; HLLC, least squares, Barth-Jespersen.  Each kernel is timed alone
    (CUDA events, an L2 eviction before every launch) at a perturbed freestream
    state: residual Gfaces/s, Jacobian blocks/s, FP32 ILU(0) apply GB/s, as
    fractions of the HBM copy peak."""
    import ctypes
    t0 = time.perf_counter()
    m = fv.UMesh.generate(fv.MESH_NACA_OGRID, LARGE_MESH, reorder=1)
    t_mesh = time.perf_counter() - t0
    ph = fv.physics_cfg(Minf=0.75, aoa_deg=2.0, Reinf=5000.0, Tinf=288.15, Pr=0.72, viscous=True)
    bcs = [(2, "adiabaticwall", (0.0,)), (4, "farfield", ())]
    main = fv.FlowFV(m, ph, fv.numerics_cfg(flux="HLLC", gradient="LEASTSQUARES", reconstruction="BARTHJESPERSEN"),
                     bcs)
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
    return out


def _oracle_case(m):
    from oracle import orc
    om = orc.Mesh.from_export(m.export())
    od1 = orc.Disc(om, **PHYS, **NUM_START, bcs=BCS)
    od2 = orc.Disc(om, **PHYS, **NUM_MAIN, bcs=BCS)
    return od1, od2


def _oracle_steps(od, cfg, u, nsteps, lin_maxit):
    """nsteps pseudo-time steps on the oracle with every linear solve running
    exactly lin_maxit FGMRES iterations (relative tolerance out of reach)."""
    t0 = time.perf_counter()
    od.steady_solve(u, cflmin=cfg["cfl_min"], cflmax=cfg["cfl_max"], tol=1e-30, maxiter=nsteps, pc="ilu0",
                    matrix_free=bool(cfg.get("matrix_free", 0)), nl_update="bounded", min_relax=cfg["min_relax"],
                    abs_tol=True, lin_rtol=1e-14, lin_maxit=lin_maxit)
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


def oracle_parity(m, main, ud):
    """The GPU's numbers on this workload against the oracle on the same mesh and
    state: the second-order residual at the converged state and at a seeded
    5 % perturbation of freestream (max |difference| over the largest sum of
    |face flux x length| of a cell), and Cl, CDp at the converged state."""
    import torch
    from oracle import orc
    _, od2 = _oracle_case(m)
    out = {}
    u_conv = ud.detach().cpu().numpy().reshape(m.nelem, 4)
    rng = np.random.default_rng(1234)
    u_pert = np.tile(od2.freestream(), (m.nelem, 1)) * (1 + 0.05 * rng.uniform(-1, 1, (m.nelem, 4)))
    for tag, u in (("converged", u_conv), ("perturbed", u_pert)):
        udev = torch.tensor(u, device=ud.device)
        r = torch.zeros_like(udev)
        main.compute_residual(udev, r)
        main.synchronize()
        ro, _ = od2.residual(u)
        out[f"residual_{tag}_max_rel_err"] = float(np.abs(r.cpu().numpy() - ro).max() / od2.flux_scale(u).max())
    cg = main.surface_data(ud, 2)[0]
    co = od2.surface_data(u_conv, 2)
    out["cl_cdp_rel_err"] = [float(abs(cg[k] - co[k]) / abs(co[k])) for k in (0, 1)]
    return out


def cpu_baseline(m, starter, main, budget_s, u_state=None):
    """The oracle (the CPU restatement of the reference's path, natural-order
    ILU(0) as PETSc's) on the host cores: a bounded sample of pseudo-time
    steps of the starter and of the main solve with pinned FGMRES iteration
    counts gives the cost per step and per Krylov iteration, which is applied
    to the step and iteration counts of the GPU solve.  starter / main: the
    GPU's fv_solve_stats of the two solves.  With u_state (host array of the
    state the GPU kernels were timed at), the oracle's residual, FP64 Jacobian
    assembly, ILU(0) factorisation and ILU(0) apply are timed there too."""
    from oracle import orc
    nthreads = os.cpu_count() or 1
    orc.set_threads(nthreads)
    od1, od2 = _oracle_case(m)
    u0 = np.tile(od2.freestream(), (m.nelem, 1))
    a1, b1, n1 = _oracle_step_model(od1, STARTER, u0, 0.4 * budget_s)
    a2, b2, n2 = _oracle_step_model(od2, MAIN, u0, 0.6 * budget_s)
    solve_s = (a1 * starter["steps"] + b1 * starter["lin_iters"]) + (a2 * main["steps"] + b2 * main["lin_iters"])
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
                      f"+ per Krylov iteration {b1:.3f} / {b2:.3f} s, applied to {starter['steps']} + {main['steps']} "
                      f"steps and {starter['lin_iters']} + {main['lin_iters']} Krylov iterations per solve", **kernels}


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
    vals = []
    for k in range(args.warmup + args.steps):
        cb = cpu_baseline(m, {"steps": STARTER["max_timesteps"], "lin_iters": args.ref_starter_iters},
                          {"steps": args.ref_steps_per_solve, "lin_iters": args.ref_iters_per_solve},
                          args.cpu_seconds / max(args.steps + args.warmup, 1))
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
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain", action="store_true", help="FP64 Jacobian and preconditioner (the plain path)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--nvtx", action="store_true", help="profiling aid: NVTX range around each main solve")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the plain-FP64 and warm-start comparison solves")
    ap.add_argument("--no-graph", action="store_true",
                    help="profiling aid: issue every launch from the host instead of replaying a CUDA graph")
    ap.add_argument("--max-main-steps", type=int, default=0,
                    help="profiling aid: cap the main solve's pseudo-time steps (the solve then does not converge)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--ref-steps-per-solve", type=int, default=1100,
                    help="main-solve pseudo-time steps per solve assumed by the reference arm")
    ap.add_argument("--ref-iters-per-solve", type=int, default=26000,
                    help="main-solve Krylov iterations per solve assumed by the reference arm")
    ap.add_argument("--ref-starter-iters", type=int, default=1800,
                    help="starter Krylov iterations per solve assumed by the reference arm")
    ap.add_argument("--warm-train", type=int, default=512,
                    help="training conditions of the learned warm-start variant (0 skips it; 2048 for the full set)")
    ap.add_argument("--warm-test", type=int, default=64, help="held-out conditions of the warm-start variant")
    ap.add_argument("--warm-epochs", type=int, default=60, help="training epochs of the warm-start network")
    ap.add_argument("--no-large", dest="large", action="store_false",
                    help="skip the ~4M-cell kernel-throughput variant")
    args = ap.parse_args()
    if args.max_main_steps > 0:
        MAIN["max_timesteps"] = args.max_main_steps
    if args.no_graph:
        STARTER["use_graph"] = 0
        MAIN["use_graph"] = 0
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
