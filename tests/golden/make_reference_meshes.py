"""Writes the reference's regression meshes as compact arrays for the tests
(the reference tree is not available where the GPU tests run).

    python tests/golden/make_reference_meshes.py [REFERENCE_ROOT]   (default: $FVENS_REFERENCE)

Reads, with this project's own Gmsh 2.2 reader (cells kept in file order):
  testcases/naca0012/grids/naca0012luo.msh                 -> naca0012luo_mesh.npz
  testcases/visc-naca0012/grids/NACA0012_lam_hybrid_1.msh  -> naca0012_lam_hybrid_1_mesh.npz
  testcases/2dcylinder/grids/2dcylinder{0..3}.msh           -> 2dcylinder_meshes.npz
and the exact lift and drag of the laminar flat plate,
  tests/visc-flatplate/exact_clcd_flatplate.dat            -> flatplate_exact_clcd.npz
The functional-regression values the tests compare with are the reference's
files testcases/naca0012/regr-MUSCL_LeastSquares_HLLC.txt and
testcases/visc-naca0012/regr-LeastSquares_Roe.txt, stored alongside; the
cylinder meshes are the refinement sequence of the reference's entropy-
convergence test (tests/inv-2dcyl/CMakeLists.txt).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import fvens_gb300 as fv  # noqa: E402

CASES = [
    ("testcases/naca0012/grids/naca0012luo.msh", "naca0012luo_mesh.npz",
     "testcases/naca0012/regr-MUSCL_LeastSquares_HLLC.txt"),
    ("testcases/visc-naca0012/grids/NACA0012_lam_hybrid_1.msh", "naca0012_lam_hybrid_1_mesh.npz",
     "testcases/visc-naca0012/regr-LeastSquares_Roe.txt"),
]


def _arrays(e, prefix=""):
    return {prefix + "coords": e["coords"], prefix + "nnode": e["nnode"].astype(np.int8),
            prefix + "inpoel": e["inpoel"], prefix + "bface": e["bface"], prefix + "btag": e["btag"].astype(np.int16)}


def main(root):
    with open(os.path.join(root, "tests/visc-flatplate/exact_clcd_flatplate.dat")) as f:
        exact = [float(x) for x in f.read().split()[:3]]
    np.savez_compressed(os.path.join(HERE, "flatplate_exact_clcd.npz"), exact=np.array(exact))
    print("flat plate exact CL, CDp, CDsf", exact)
    cyl = {}
    for k in range(4):
        m = fv.UMesh.read_gmsh(os.path.join(root, f"testcases/2dcylinder/grids/2dcylinder{k}.msh"), reorder=0)
        cyl.update(_arrays(m.export(), f"m{k}_"))
        print(f"2dcylinder{k}", m.nelem, "cells", m.npoin, "points", m.nbface, "boundary faces")
    np.savez_compressed(os.path.join(HERE, "2dcylinder_meshes.npz"), **cyl)
    for msh, out, regr in CASES:
        m = fv.UMesh.read_gmsh(os.path.join(root, msh), reorder=0)
        e = m.export()
        with open(os.path.join(root, regr)) as f:
            vals = f.read().split()
        cl, cdp = float(vals[0]), float(vals[1])
        cdsf = float(vals[2]) if vals[2].lower().lstrip("-") != "nan" else np.nan
        np.savez_compressed(os.path.join(HERE, out), **_arrays(e), regression=np.array([cl, cdp, cdsf]))
        print(out, m.nelem, "cells", m.npoin, "points", m.nbface, "boundary faces", "regression", cl, cdp, cdsf)


if __name__ == "__main__":
    from oracle import orc
    root = sys.argv[1] if len(sys.argv) > 1 else orc.reference_root()
    if not root:
        sys.exit("usage: make_reference_meshes.py REFERENCE_ROOT (or set FVENS_REFERENCE)")
    main(root)
