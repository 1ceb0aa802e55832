"""Writes naca0012_laminar_l{levels}_oracle_converged.npz: the oracle's own
converged solves of the first members of bench.py's batched laminar workload
(seed-7 conditions of a batch of 64: M ~ U[0.3, 0.7], AoA ~ U[-4, 4] deg,
Re ~ U[2000, 10000]) on the reference's hybrid NACA 0012 mesh refined
`levels` times (fvens_gb300.meshes.refine; cells in the refinement's order):
first-order starter, then the second-order solve (Roe, least squares,
adiabatic wall) to an absolute `tol` (1e-12: at the workload's 1e-10 two
converged solves of a member still differ by ~1e-7 in the state and Cl), the
bench's CFL settings and step limit raised to 3,000, ILU(0) in the
GPU's elimination order (block colours with the boundary-layer lines kept
whole, from the product library here, in the refinement's cell numbering;
with the natural order the oracle's solve of member 0 stalls at 1.4e-6 after
1,500 steps).

    python tests/golden/make_laminar_converged.py [levels] [members] [threads] [tol]

The committed fixture holds members 0, 1 and 4 (`2 0,1,4 8 1e-12`; made as
member 0 and members 1,4 in two runs and concatenated, the same arrays).

Stored per member: the converged state at 4,096 seeded cells and at every
cell touching the wall (`cells`, `states`), Cl / CDp / CDsf (`functionals`)
and the step and Krylov counts.  bench.py compares the GPU's converged batch
members with it, and tests/test_gpu_regression.py a GPU batch of the same
members solved to the same tolerance.  On 8 x86 threads at 1e-12: member 0
3,509 s (50 + 1,043 steps), member 1 2,588 s (50 + 1,199), member 4 4,129 s
(50 + 1,613); member 0 at 1e-10: 2,443 s on 7 threads (50 + 681 steps).
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from fvens_gb300 import meshes  # noqa: E402
from oracle import orc  # noqa: E402


def block_order(a):
    """The GPU's elimination order for the bench's laminar mesh (RCM, lines at
    threshold 10, parts of 128 coloured as pc_ordering 2), as cells of the
    array numbering of a."""
    import ctypes

    import fvens_gb300 as fv
    m = fv.UMesh.from_arrays(a["coords"], a["nnode"], a["inpoel"], a["bface"], a["btag"], reorder=1)
    m.find_lines(10.0)
    order = np.zeros(m.nelem, np.int32)
    npart, ncol = ctypes.c_int(), ctypes.c_int()
    fv.check(fv.lib().fv_mesh_block_order_ex(m._h, 128, 1, fv._hp(order, ctypes.c_int), ctypes.byref(npart),
                                             ctypes.byref(ncol)))
    return m.export()["perm"][order].astype(np.int32)


def main(levels, members, threads, tol):
    from fvens_gb300 import build
    build.build_all()
    orc.set_threads(threads)
    z = np.load(os.path.join(HERE, "naca0012_lam_hybrid_1_mesh.npz"))
    a = meshes.refine(dict(coords=z["coords"], nnode=z["nnode"], inpoel=z["inpoel"], bface=z["bface"],
                           btag=z["btag"]), levels)
    order = block_order(a)
    om = orc.Mesh(a["coords"], a["nnode"], a["inpoel"], a["bface"], a["btag"])
    wall_nodes = np.unique(a["bface"][a["btag"] == 2])
    near_wall = np.where(np.isin(a["inpoel"], wall_nodes).any(axis=1))[0]
    rng = np.random.default_rng(2025)
    cells = np.unique(np.concatenate([near_wall, rng.choice(om.nelem, 4096, replace=False)])).astype(np.int32)
    # the bench draws its batch of 64 at once: those draws fix every member's condition
    rng_c = np.random.default_rng(7)
    n = 64
    M, A, Re = rng_c.uniform(0.3, 0.7, n), rng_c.uniform(-4, 4, n), rng_c.uniform(2000, 10000, n)
    states, funs, counts = [], [], []
    S, T = bench.LAMINAR_START, bench.LAMINAR_MAIN
    for k in members:
        ph = dict(Minf=float(M[k]), aoa_deg=float(A[k]), Reinf=float(Re[k]), Tinf=288.15, Pr=0.72, viscous=True)
        bcs = bench.LAMINAR_BCS
        d1 = orc.Disc(om, **ph, flux="ROE", gradient="NONE", bcs=bcs)
        d2 = orc.Disc(om, **ph, flux="ROE", gradient="LEASTSQUARES", bcs=bcs)
        t0 = time.perf_counter()
        u, s1 = d1.steady_solve(np.tile(d2.freestream(), (om.nelem, 1)), cflmin=S["cfl_min"], cflmax=S["cfl_max"],
                                tol=S["tolerance"], maxiter=S["max_timesteps"], abs_tol=False, pc="ilu0",
                                nl_update="bounded", order=order)
        u, s2 = d2.steady_solve(u, cflmin=T["cfl_min"], cflmax=T["cfl_max"], tol=tol, maxiter=3000, abs_tol=True,
                                pc="ilu0", nl_update="bounded", order=order)
        f = d2.surface_data(u, 2)
        print("member", k, "starter", s1["steps"], "main", s2["steps"], s2["lin_iters"], "status", s2["status"],
              f"res {s2['res']:.2e}", "Cl CDp CDsf", f.tolist(), f"{time.perf_counter() - t0:.0f} s", flush=True)
        if s2["status"] != 0:
            sys.exit(f"member {k}: the oracle's solve did not converge; no fixture written")
        states.append(u[cells])
        funs.append(f)
        counts.append([s1["steps"], s1["lin_iters"], s2["steps"], s2["lin_iters"]])
    np.savez_compressed(os.path.join(HERE, f"naca0012_laminar_l{levels}_oracle_converged.npz"),
                        members=np.array(members, np.int32), tolerance=tol, cells=cells, states=np.array(states),
                        functionals=np.array(funs), solve_counts=np.array(counts, np.int64))


if __name__ == "__main__":
    lv = int(sys.argv[1]) if len(sys.argv) > 1 else 2
    mem = [int(x) for x in sys.argv[2].split(",")] if len(sys.argv) > 2 else [0, 1]
    th = int(sys.argv[3]) if len(sys.argv) > 3 else (os.cpu_count() or 1)
    tl = float(sys.argv[4]) if len(sys.argv) > 4 else 1e-12
    main(lv, mem, th, tl)
