"""The reference's functional-regression cases on the reference's own meshes
(arrays in tests/golden/, written by tests/golden/make_reference_meshes.py),
with the control-file settings of the reference's test runs:
  testcases/naca0012/transonic-sanity-test-muscl.ctrl + opts.solverc
  testcases/visc-naca0012/laminar-implicit.ctrl + opts.solverc
and the cylinder refinement sequence of tests/inv-2dcyl."""
import os

import numpy as np

import fvens_gb300 as fv

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

CASES = {
    # HLLC, least squares, MUSCL Van Albada; starter CFL 50-1000, 20 steps, tol 1e-1;
    # main CFL 500-5000, tol 1e-7, 170 steps; robust_flow update; -pc_type sor
    "inviscid_naca0012luo": dict(
        mesh="naca0012luo_mesh.npz", bcs=[(2, "slipwall", ()), (4, "farfield", ())],
        phys=dict(Minf=0.8, aoa_deg=1.25),
        start=dict(flux="HLLC", gradient="NONE"),
        main=dict(flux="HLLC", gradient="LEASTSQUARES", reconstruction="VANALBADA", limiter_param=20.0),
        start_solver=dict(cfl_min=50, cfl_max=1000, tolerance=1e-1, max_timesteps=20),
        main_solver=dict(cfl_min=500, cfl_max=5000, tolerance=1e-7, max_timesteps=170),
        pc="sgs", nl_update="robust_flow"),
    # Roe, least squares, no limiter, laminar (Re 5000, Sutherland); starter CFL
    # 200-1000, 50 steps, tol 1e-1; main CFL 500-5000, tol 1e-6, 80 steps; full
    # update; -pc_type bjacobi -sub_pc_type ilu
    "laminar_naca0012_hybrid1": dict(
        mesh="naca0012_lam_hybrid_1_mesh.npz", bcs=[(4, "inflowoutflow", ()), (2, "adiabaticwall", (0.0,))],
        phys=dict(Minf=0.5, aoa_deg=0.0, Reinf=5000.0, Tinf=288.15, Pr=0.72, viscous=True),
        start=dict(flux="ROE", gradient="NONE"),
        main=dict(flux="ROE", gradient="LEASTSQUARES"),
        start_solver=dict(cfl_min=200, cfl_max=1000, tolerance=1e-1, max_timesteps=50),
        main_solver=dict(cfl_min=500, cfl_max=5000, tolerance=1e-6, max_timesteps=80),
        pc="ilu0", nl_update="full"),
}


def load(name):
    """(UMesh with RCM ordering as -mesh_reorder rcm, case dict, regression (CL, CDp, CDsf))."""
    c = CASES[name]
    z = np.load(os.path.join(GOLDEN, c["mesh"]))
    m = fv.UMesh.from_arrays(z["coords"], z["nnode"].astype(np.int32), z["inpoel"], z["bface"],
                             z["btag"].astype(np.int32), reorder=1)
    return m, c, z["regression"]


# The reference's entropy-convergence test on its cylinder refinements
# (tests/inv-2dcyl: inv-cyl-base.ctrl with inv-cyl-ls-hllc.ctrl or
# inv-cyl-gg-hllc_tri.ctrl, inv_cyl.solverc): M 0.38, slip wall (marker 2),
# far field (marker 4), HLLC, no limiter, first-order starter then the
# second-order main solve, both to a relative tolerance, robust_flow update,
# -pc_type bjacobi -sub_pc_type ilu
CYLINDER = dict(
    bcs=[(2, "slipwall", ()), (4, "farfield", ())], phys=dict(Minf=0.38, aoa_deg=0.0), flux="HLLC",
    solvers={"LEASTSQUARES": (dict(cfl_min=25, cfl_max=500, tolerance=1e-1, max_timesteps=150),
                              dict(cfl_min=250, cfl_max=5000, tolerance=1e-5, max_timesteps=300)),
             "GREENGAUSS": (dict(cfl_min=25, cfl_max=250, tolerance=1e-1, max_timesteps=250),
                            dict(cfl_min=250, cfl_max=1000, tolerance=1e-5, max_timesteps=350))},
    pc="ilu0", nl_update="robust_flow")


def load_cylinders():
    """The four meshes 2dcylinder0..3 (RCM-ordered as -mesh_reorder rcm)."""
    z = np.load(os.path.join(GOLDEN, "2dcylinder_meshes.npz"))
    return [fv.UMesh.from_arrays(z[f"m{k}_coords"], z[f"m{k}_nnode"].astype(np.int32), z[f"m{k}_inpoel"],
                                 z[f"m{k}_bface"], z[f"m{k}_btag"].astype(np.int32), reorder=1) for k in range(4)]


# The explicit variant (tests/inv-2dcyl/expl-inv-cyl-gg-roe_tri.ctrl, three
# meshes): Roe, Green-Gauss, forward-Euler starter (CFL 0.5, relative 1e-1,
# 15000 steps) and main solve (CFL 0.25, relative 1e-4, 60000 steps)
CYLINDER_EXPLICIT = dict(flux="ROE", gradient="GREENGAUSS", start=dict(cfl=0.5, tolerance=1e-1, max_timesteps=15000),
                         main=dict(cfl=0.25, tolerance=1e-4, max_timesteps=60000), nmesh=3)


# The reference's laminar flat-plate skin-friction convergence test
# (tests/visc-flatplate: flatplate.ctrl, flatplate.solverc; CTest
# SpatialFlow_NS_FlatPlate_LeastSquares_Roe_Struct_CDConvergence, driver
# tests/flow_clcd_conv.cpp) on flatplatestructstretched0..2 (fvens_gb300.meshes
# .flat_plate_stretched): M 0.2, Re 8.7e5, T 290.19 K, Pr 0.708, Sutherland
# viscosity; Roe, least squares, no limiter; starter CFL 20-2000, relative
# 1e-1, 50 steps; main CFL 100-4000, relative 1e-5, 500 steps; robust_flow
# update; -pc_type ilu, -mesh_reorder rcm.  Passes when the order of the
# skin-friction drag error between the two finest meshes lies in [0.95, 1.5].
FLAT_PLATE = dict(
    bcs=[(3, "slipwall", ()), (4, "farfield", ()), (5, "inflowoutflow", ()), (2, "adiabaticwall", (0.0,))],
    phys=dict(Minf=0.2, aoa_deg=0.0, Reinf=8.7e5, Tinf=290.19, Pr=0.708, viscous=True),
    flux="ROE", gradient="LEASTSQUARES",
    start_solver=dict(cfl_min=20, cfl_max=2000, tolerance=1e-1, max_timesteps=50),
    main_solver=dict(cfl_min=100, cfl_max=4000, tolerance=1e-5, max_timesteps=500),
    pc="ilu0", nl_update="robust_flow", nmesh=3, band=(0.95, 1.5))


def load_flat_plates():
    """flatplatestructstretched0..2 (RCM-ordered) and the reference's exact
    (CL, CDp, CDsf) of tests/visc-flatplate/exact_clcd_flatplate.dat."""
    from fvens_gb300 import meshes
    out = []
    for lv in range(FLAT_PLATE["nmesh"]):
        a = meshes.flat_plate_stretched(lv)
        out.append(fv.UMesh.from_arrays(a["coords"], a["nnode"], a["inpoel"], a["bface"], a["btag"], reorder=1))
    return out, np.load(os.path.join(GOLDEN, "flatplate_exact_clcd.npz"))["exact"]


def flat_plate_order(meshes_, cdsf, exact):
    """flow_clcd_conv.cpp's order of the skin-friction drag error between the
    last two meshes: h = 1/sqrt(cells) (casesolvers.cpp:96)."""
    lh = [np.log10(1.0 / np.sqrt(m.nelem)) for m in meshes_]
    le = [np.log10(abs(abs(c) - exact[2])) for c in cdsf]
    return (le[-1] - le[-2]) / (lh[-1] - lh[-2])
