"""Kernel micro-benchmarks: small, self-contained drivers of single kernels
for timing with CUDA events and for profiler captures.

    python -m fvens_gb300.kernel_bench ilu [reps] [part] FP32 block-colour ILU(0) apply (parts of
                                                         at most `part` cells, default 128),
                                                         transonic NACA 0012 512 x 256 O-grid
    python -m fvens_gb300.kernel_bench mpnn [B] [steps]  warm-start network: one Adam training
                                                         step and one prediction for B conditions
                                                         on the 13,156-cell laminar hybrid mesh

Each prints the average time per call after three untimed calls.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# transonic NACA 0012 O-grid: 512 x 256, far field 30 chords, growth 1.02, outer rings triangulated
NACA_C2 = [512, 256, 30.0, 0, 0, 1.02, 154, 3]


def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def bench_ilu(reps=5, part=128):
    import torch

    import fvens_gb300 as fv
    dev = torch.device("cuda", 0)
    m = fv.UMesh.generate(fv.MESH_NACA_OGRID, NACA_C2, reorder=1)
    bcs = [(2, "slipwall", ()), (4, "farfield", ())]
    d = fv.FlowFV(m, fv.physics_cfg(Minf=0.8, aoa_deg=1.25), fv.numerics_cfg(flux="HLLC", gradient="NONE"), bcs)
    u = torch.tensor(np.tile(d.freestream()[0], (m.nelem, 1)), device=dev)
    A = fv.BlockMatrix(d, 4)
    d.assemble_jacobian(u, A)
    A.add_diagonal(torch.tensor(m.geometry()["area"] / 0.01, device=dev))  # pseudo-time term, CFL-like scale
    P = fv.Preconditioner(d, A, "ilu0", part_size=part)
    P.setup()
    r = torch.tensor(np.random.default_rng(0).normal(size=(m.nelem, 4)), device=dev)
    z = torch.zeros_like(r)
    for _ in range(3):
        P.apply(r, z)
    torch.cuda.synchronize()
    a, b = _events(torch)
    a.record()
    for _ in range(reps):
        P.apply(r, z)
    b.record()
    torch.cuda.synchronize()
    print(f"ilu0 apply: {a.elapsed_time(b) / reps:.4f} ms per apply, {m.nelem} cells, parts of <= {part}")


def bench_mpnn(B=16, steps=5):
    import torch

    import fvens_gb300 as fv
    from fvens_gb300.mpnn import MPNN
    dev = torch.device("cuda", 0)
    z = np.load(os.path.join(ROOT, "tests", "golden", "naca0012_lam_hybrid_1_mesh.npz"))
    m = fv.UMesh.from_arrays(z["coords"], z["nnode"].astype(np.int32), z["inpoel"], z["bface"],
                             z["btag"].astype(np.int32), reorder=1)
    rng = np.random.default_rng(11)
    phs = [fv.physics_cfg(Minf=float(rng.uniform(0.3, 0.7)), aoa_deg=float(rng.uniform(-4, 4)),
                          Reinf=float(rng.uniform(2000, 10000)), Tinf=288.15, Pr=0.72, viscous=True) for _ in range(B)]
    net = MPNN(m, layers=4, wall_markers=(2,), seed=11)
    net.set_scale(np.array([0.05, 0.1, 0.1, 0.2], np.float32))
    tgt = torch.empty((B * m.nelem, 4), dtype=torch.float64, device=dev)
    net.predict(phs, tgt)
    tgt *= 1.01
    for _ in range(3):
        net.train_step(phs, tgt, 1e-4)
    torch.cuda.synchronize()
    a, b = _events(torch)
    a.record()
    for _ in range(steps):
        net.train_step(phs, tgt, 1e-4)
    b.record()
    torch.cuda.synchronize()
    t_train = a.elapsed_time(b) / steps
    u = torch.empty_like(tgt)
    a.record()
    for _ in range(steps):
        net.predict(phs, u)
    b.record()
    torch.cuda.synchronize()
    print(f"mpnn: train step {t_train:.3f} ms, predict {a.elapsed_time(b) / steps:.3f} ms, "
          f"{B} conditions x {m.nelem} cells")


def main(argv):
    if not argv or argv[0] not in ("ilu", "mpnn"):
        print(__doc__)
        return 2
    args = [int(x) for x in argv[1:]]
    {"ilu": bench_ilu, "mpnn": bench_mpnn}[argv[0]](*args)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
