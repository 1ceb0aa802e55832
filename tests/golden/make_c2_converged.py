"""Writes naca0012_transonic_oracle_converged.npz: the oracle's own complete
solve of the benchmark workload (bench.py: transonic NACA 0012 on the
512 x 256 O-grid, HLLC / Green-Gauss / Venkatakrishnan, starter + main solve
to ||R|| < 1e-10) on the mesh of the oracle's generator (oracle/meshgen.py,
cells in the generator's order), with ILU(0) in the GPU's block-colour
elimination order (parts of at most 128 cells).

    python tests/golden/make_c2_converged.py [threads]

The block-colour order comes from the product library here (fv_mesh_block_order
on the RCM-ordered mesh, mapped to the generator's cell numbering) and is
stored, so that bench.py's reference arm runs the same solve without the
product library.  With PETSc's natural order instead, the oracle's solve of
this workload diverges (non-finite residual after 1,022 steps).

Stored: the elimination order (`order`), the converged state at every cell of
the wall ring and at 4,096 seeded cells (`cells`, `states`), Cl / CDp / CDsf
(`functionals`), the solve's step and Krylov counts (`solve_counts`: starter
steps, starter Krylov iterations, main steps, main Krylov iterations), its
final residual, and its wall time with the thread count used.  Takes tens of
minutes on a few cores.
"""
import ctypes
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from oracle import meshgen, orc  # noqa: E402

PART = 128


def block_order():
    """The GPU's block-colour elimination order of the workload's mesh, as
    cells of the generator's numbering."""
    import fvens_gb300 as fv
    m = fv.UMesh.generate(fv.MESH_NACA_OGRID, bench.MESH, reorder=1)
    order = np.zeros(m.nelem, np.int32)
    npart, ncol = ctypes.c_int(), ctypes.c_int()
    fv.check(fv.lib().fv_mesh_block_order(m._h, PART, fv._hp(order, ctypes.c_int), ctypes.byref(npart),
                                          ctypes.byref(ncol)))
    perm = m.export()["perm"]  # RCM position -> generator cell
    return perm[order].astype(np.int32)


def main(threads):
    from fvens_gb300 import build
    build.build_all()
    orc.set_threads(threads)
    order = block_order()
    arrs = meshgen.naca_ogrid(*bench.MESH)
    om, od1, od2 = bench._oracle_case_from_arrays(arrs)
    u = np.tile(od2.freestream(), (om.nelem, 1))
    t0 = time.perf_counter()
    u, st1, st2, ts, tm = bench.oracle_solve(od1, od2, u, order)
    print("starter", st1["steps"], st1["lin_iters"], f"{ts:.1f} s", "main", st2["steps"], st2["lin_iters"],
          f"{tm:.1f} s", "status", st2["status"], "res", st2["res"], flush=True)
    if st2["status"] != 0:
        sys.exit("the oracle's solve did not converge; no fixture written")
    fun = od2.surface_data(u, 2)
    nc = bench.MESH[0]
    rng = np.random.default_rng(2024)
    cells = np.unique(np.concatenate([np.arange(nc), rng.choice(om.nelem, 4096, replace=False)])).astype(np.int32)
    np.savez_compressed(os.path.join(HERE, "naca0012_transonic_oracle_converged.npz"),
                        order=order, part_size=np.int64(PART),
                        cells=cells, states=u[cells], functionals=np.asarray(fun, np.float64),
                        solve_counts=np.array([st1["steps"], st1["lin_iters"], st2["steps"], st2["lin_iters"]],
                                              np.int64),
                        final_res=np.float64(st2["res"]), solve_seconds=np.float64(ts + tm),
                        solve_threads=np.int64(threads), host=np.array(platform.machine()),
                        elapsed_total=np.float64(time.perf_counter() - t0))
    print("Cl, CDp, CDsf", fun.tolist(), "cells stored", len(cells))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1))
