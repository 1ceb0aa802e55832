"""The multi-rank (replica) path on CPU with gloo, world size 2: each rank
solves its own flow condition (with the oracle standing in for the GPU
solve), the timing is the maximum over ranks and the throughput counts every
rank's solves; bench.py's reference arm under torchrun prints one line
from rank 0 only; and bench.py's CPU-baseline leg runs on a small mesh."""
import json
import os
import socket
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import time

    from fvens_gb300.replicas import Replicas
    from oracle import orc
    from tests import cases
    reps = Replicas("gloo")
    m = cases.channel(24, 8)
    od = orc.Disc(orc.Mesh.from_export(m.export()), Minf=0.4 + 0.1 * rank, flux="ROE", bcs=cases.CHANNEL_BCS)
    u0 = np.tile(od.freestream(), (m.nelem, 1))
    reps.barrier()
    t0 = time.perf_counter()
    u, st = od.steady_solve(u0, cflmin=10, cflmax=1000, tol=1e-10, maxiter=300, pc="ilu0")
    if rank == 1:
        time.sleep(0.3)  # the slower rank sets the time
    dt = time.perf_counter() - t0
    reps.barrier()
    value = reps.throughput(1, dt)
    tmax = reps.max_over_ranks(dt)
    np.save(os.path.join(out_dir, f"u{rank}.npy"), u)
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump(dict(value=value, tmax=tmax, dt=dt, status=st["status"], res=st["res"]), f)
    reps.close()


def test_two_gloo_replicas(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    r = [json.load(open(tmp_path / f"r{k}.json")) for k in range(2)]
    assert all(x["status"] == 0 and x["res"] <= 1e-10 for x in r)
    assert r[0]["tmax"] == r[1]["tmax"] == max(r[0]["dt"], r[1]["dt"])
    assert r[1]["dt"] >= 0.3 and r[0]["tmax"] >= 0.3
    assert abs(r[0]["value"] - 2.0 / r[0]["tmax"]) <= 1e-12 * r[0]["value"]
    u0, u1 = np.load(tmp_path / "u0.npy"), np.load(tmp_path / "u1.npy")
    assert np.abs(u0 - u1).max() > 1e-3  # independent conditions, no exchange


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--small"]
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [x for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    # one complete solve timed whole, on the oracle's own mesh (same workload description as the GPU arm)
    assert line["steps"] == 1 and line["solve"]["main_steps"] > 0
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"] == bench.workload_config(2, small=True)


def test_bench_cpu_baseline_on_small_naca_mesh():
    """bench.py's CPU-baseline leg (the oracle's step model and its kernel
    timings) on a small O-grid of the workload's family: a positive solve rate
    in the metric's unit, the sample described, and every kernel timed."""
    sys.path.insert(0, ROOT)
    import bench
    import fvens_gb300 as fv
    m = fv.UMesh.generate(fv.MESH_NACA_OGRID, [64, 32, 30.0, 0, 0, 1.1, 12, 3], reorder=1)
    _, od2 = bench._oracle_case(m)
    u = np.tile(od2.freestream(), (m.nelem, 1))
    cb = bench.cpu_baseline(m, 1.0, u, counts={"starter": {"steps": 10, "lin_iters": 50},
                                              "main": {"steps": 20, "lin_iters": 200}})
    assert cb["unit"] == "solves/s" and cb["kind"] == "port" and cb["value"] > 0 and cb["cores"] >= 1
    assert "10 + 20 steps" in cb["sample"]
    assert set(cb["kernels_ms"]) == {"residual", "jacobian", "ilu0_setup", "ilu0_apply"}
    assert all(v > 0 for v in cb["kernels_ms"].values())
