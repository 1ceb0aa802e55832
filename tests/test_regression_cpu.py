"""The oracle against the reference's functional-regression values on the
reference's own meshes and control settings (testcases/naca0012 and
testcases/visc-naca0012; values in their regr-*.txt files).  The reference
stops at a relative residual drop of 1e-7 / 1e-6 and compares CL to 1e-6 and
CDp, CDsf to 1e-8 against runs of its own code path; the oracle follows the
same algorithm with its own (natural-order) ILU(0)/SGS, so its drag
coefficients at the same stopping tolerance agree to a few 1e-7."""
import numpy as np
import pytest

from oracle import orc
from tests import regression_cases as rc


def _oracle_solve(name, tol=None, abs_tol=False, maxiter=None):
    m, c, regr = rc.load(name)
    om = orc.Mesh.from_export(m.export())
    d1 = orc.Disc(om, **c["phys"], **c["start"], bcs=c["bcs"])
    d2 = orc.Disc(om, **c["phys"], **c["main"], bcs=c["bcs"])
    u0 = np.tile(d2.freestream(), (m.nelem, 1))
    s1, s2 = c["start_solver"], c["main_solver"]
    u1, _ = d1.steady_solve(u0, cflmin=s1["cfl_min"], cflmax=s1["cfl_max"], tol=s1["tolerance"],
                            maxiter=s1["max_timesteps"], abs_tol=False, pc=c["pc"], nl_update=c["nl_update"])
    u2, st = d2.steady_solve(u1, cflmin=s2["cfl_min"], cflmax=s2["cfl_max"], tol=tol or s2["tolerance"],
                             maxiter=maxiter or s2["max_timesteps"], abs_tol=abs_tol, pc=c["pc"],
                             nl_update=c["nl_update"])
    return st, d2.surface_data(u2, 2), regr


def test_oracle_reproduces_inviscid_naca0012_regression():
    st, f, regr = _oracle_solve("inviscid_naca0012luo")
    assert st["status"] == 0 and st["steps"] <= 170
    assert abs(f[0] - regr[0]) <= 1e-6 * abs(regr[0])      # the reference's CL tolerance
    assert abs(f[1] - regr[1]) <= 3e-7 * abs(regr[1])      # CDp
    assert f[2] == 0.0                                      # inviscid: no skin friction


def test_oracle_reproduces_laminar_naca0012_regression():
    st, f, regr = _oracle_solve("laminar_naca0012_hybrid1")
    assert st["status"] == 0 and st["steps"] <= 80
    assert abs(f[1] - regr[1]) <= 5e-7 * abs(regr[1])      # CDp
    assert abs(f[2] - regr[2]) <= 5e-7 * abs(regr[2])      # CDsf
    # CL of the symmetric aerofoil at zero incidence is mesh-asymmetry noise
    # (3e-5): compared in absolute terms
    assert abs(f[0] - regr[0]) <= 1e-7


@pytest.mark.parametrize("gradient", ["LEASTSQUARES", "GREENGAUSS"])
def test_oracle_entropy_convergence_on_reference_cylinders(gradient):
    """The reference's SpatialFlow_Euler_Cylinder_{LeastSquares,GreenGauss}_HLLC_Tri_EntropyConvergence
    (tests/flow_conv.cpp:42-89 with tests/inv-2dcyl/*): on 2dcylinder0..3 the
    starter and main solves of the control files run from freestream; a solve
    that stops at its step limit is kept, as FlowCase::run_output
    (casesolvers.cpp:98-103) catches that error; h = 1/sqrt(cells)
    (casesolvers.cpp:96) and the entropy error of the final state give the
    orders between refinements, of which the last must lie in [1.65, 2.1].
    Only that one is checked by the reference, and only the two finest meshes
    enter it: the oracle's least-squares solves on the two coarsest meshes
    break down (non-finite residual), as flow_conv.cpp tolerates."""
    c = rc.CYLINDER
    s1, s2 = c["solvers"][gradient]
    logs, statuses = [], []
    for m in rc.load_cylinders():
        om = orc.Mesh.from_export(m.export())
        d1 = orc.Disc(om, **c["phys"], flux=c["flux"], gradient="NONE", bcs=c["bcs"])
        d2 = orc.Disc(om, **c["phys"], flux=c["flux"], gradient=gradient, bcs=c["bcs"])
        u0 = np.tile(d2.freestream(), (m.nelem, 1))
        u1, _ = d1.steady_solve(u0, cflmin=s1["cfl_min"], cflmax=s1["cfl_max"], tol=s1["tolerance"],
                                maxiter=s1["max_timesteps"], abs_tol=False, pc=c["pc"], nl_update=c["nl_update"])
        u2, st = d2.steady_solve(u1, cflmin=s2["cfl_min"], cflmax=s2["cfl_max"], tol=s2["tolerance"],
                                 maxiter=s2["max_timesteps"], abs_tol=False, pc=c["pc"], nl_update=c["nl_update"])
        statuses.append(st["status"])
        logs.append((np.log10(1.0 / np.sqrt(m.nelem)), np.log10(d2.entropy_error(u2))))
    # the two finest meshes: converged (0) or stopped at the step limit (6)
    assert all(s in (0, 6) for s in statuses[2:]), statuses
    slope = (logs[3][1] - logs[2][1]) / (logs[3][0] - logs[2][0])
    assert 1.65 <= slope <= 2.1, (slope, logs, statuses)


def test_oracle_explicit_entropy_convergence_on_reference_cylinders():
    """The reference's Flow_Explicit_Euler_Cylinder_GreenGauss_Roe_Tri_EntropyConvergence
    (tests/flow_conv.cpp with expl-inv-cyl-gg-roe_tri.ctrl, 2dcylinder0..2):
    forward-Euler starter and main solve from freestream; the last order lies
    in [1.65, 2.1].  The oracle's solves all reach their relative tolerance."""
    c, x = rc.CYLINDER, rc.CYLINDER_EXPLICIT
    logs = []
    for m in rc.load_cylinders()[:x["nmesh"]]:
        om = orc.Mesh.from_export(m.export())
        d1 = orc.Disc(om, **c["phys"], flux=x["flux"], gradient="NONE", bcs=c["bcs"])
        d2 = orc.Disc(om, **c["phys"], flux=x["flux"], gradient=x["gradient"], bcs=c["bcs"])
        s1, s2 = x["start"], x["main"]
        u1, a = d1.steady_fe(np.tile(d2.freestream(), (m.nelem, 1)), s1["cfl"], tol=s1["tolerance"],
                             maxiter=s1["max_timesteps"], abs_tol=False)
        u2, b = d2.steady_fe(u1, s2["cfl"], tol=s2["tolerance"], maxiter=s2["max_timesteps"], abs_tol=False)
        assert a["status"] == 0 and b["status"] == 0, (m.nelem, a["status"], b["status"])
        logs.append((np.log10(1.0 / np.sqrt(m.nelem)), np.log10(d2.entropy_error(u2))))
    slope = (logs[-1][1] - logs[-2][1]) / (logs[-1][0] - logs[-2][0])
    assert 1.65 <= slope <= 2.1, (slope, logs)


def _flat_plate_oracle(m, tol, abs_tol, maxiter):
    c = rc.FLAT_PLATE
    om = orc.Mesh.from_export(m.export())
    d1 = orc.Disc(om, **c["phys"], flux=c["flux"], gradient="NONE", bcs=c["bcs"])
    d2 = orc.Disc(om, **c["phys"], flux=c["flux"], gradient=c["gradient"], bcs=c["bcs"])
    s1 = c["start_solver"]
    u1, _ = d1.steady_solve(np.tile(d2.freestream(), (m.nelem, 1)), cflmin=s1["cfl_min"], cflmax=s1["cfl_max"],
                            tol=s1["tolerance"], maxiter=s1["max_timesteps"], abs_tol=False, pc=c["pc"],
                            nl_update=c["nl_update"])
    s2 = c["main_solver"]
    u2, st = d2.steady_solve(u1, cflmin=s2["cfl_min"], cflmax=s2["cfl_max"], tol=tol, maxiter=maxiter,
                             abs_tol=abs_tol, pc=c["pc"], nl_update=c["nl_update"])
    return u2, st, d2.surface_data(u2, 2)


def test_oracle_flat_plate_skin_friction_convergence():
    """The reference's SpatialFlow_NS_FlatPlate_LeastSquares_Roe_Struct_CDConvergence
    (tests/flow_clcd_conv.cpp with tests/visc-flatplate/flatplate.ctrl and
    flatplate.solverc) on flatplatestructstretched0..2: the order of the
    skin-friction drag error against exact_clcd_flatplate.dat between the two
    finest meshes lies in [0.95, 1.5]."""
    c = rc.FLAT_PLATE
    meshes_, exact = rc.load_flat_plates()
    cdsf = []
    for m in meshes_:
        _, st, f = _flat_plate_oracle(m, c["main_solver"]["tolerance"], False, c["main_solver"]["max_timesteps"])
        assert st["status"] in (0, 6), st["status"]   # a step-limited solve is kept, as run_output does
        cdsf.append(f[2])
    order = rc.flat_plate_order(meshes_, cdsf, exact)
    assert c["band"][0] <= order <= c["band"][1], (order, cdsf)
