"""Steady implicit solves on the GPU against the oracle's restatement of
SteadyBackwardEulerSolver::solve: converged states, step counts, failure
reporting."""
import numpy as np
import pytest

import fvens_gb300 as fv
from oracle import orc
from tests import cases

pytestmark = pytest.mark.gpu


def _setup(nx=48, ny=16, **phys):
    m = cases.channel(nx, ny)
    pk = dict(Minf=0.5, **phys)
    gd = fv.FlowFV(m, fv.physics_cfg(**pk), fv.numerics_cfg(flux="ROE"), cases.CHANNEL_BCS)
    od = orc.Disc(orc.Mesh.from_export(m.export()), **pk, flux="ROE", bcs=cases.CHANNEL_BCS)
    return m, gd, od


@pytest.mark.parametrize("prec", [8, 4])
def test_c1_like_solve_matches_oracle(cuda, prec):
    import torch
    m, gd, od = _setup()
    u0 = np.tile(od.freestream(), (m.nelem, 1))
    S = fv.SteadyBackwardEulerSolver(gd, cfl_min=10, cfl_max=1000, tolerance=1e-10, max_timesteps=200,
                                     pc="ilu0", precision=prec)
    ud = torch.tensor(u0, device=cuda)
    rc, st = S.solve(ud)
    P = fv.Preconditioner(gd, fv.BlockMatrix(gd, prec), "ilu0")
    uo, sto = od.steady_solve(u0, cflmin=10, cflmax=1000, tol=1e-10, maxiter=200, pc="ilu0", order=P.order())
    assert st[0]["status"] == 0 and sto["status"] == 0
    assert st[0]["res"] <= 1e-10
    # converged fields agree (both at ||R|| < 1e-10)
    ug = ud.cpu().numpy()
    assert np.abs(ug - uo).max() / np.abs(uo).max() <= 1e-8
    if prec == 8:
        assert abs(st[0]["steps"] - sto["steps"]) <= 2
    res, cfl, lin = S.history()
    assert len(res) == st[0]["steps"] and cfl[0] == 10.0


def test_matrix_free_solve(cuda):
    import torch
    m, gd, od = _setup()
    u0 = np.tile(od.freestream(), (m.nelem, 1))
    S = fv.SteadyBackwardEulerSolver(gd, cfl_min=10, cfl_max=1000, tolerance=1e-10, max_timesteps=200,
                                     pc="ilu0", precision=4, matrix_free=1)
    ud = torch.tensor(u0, device=cuda)
    rc, st = S.solve(ud)
    assert st[0]["status"] == 0
    r = torch.zeros_like(ud)
    gd.compute_residual(ud, r)
    a = m.geometry()["area"]
    assert np.sqrt((r.cpu().numpy()[:, 3] ** 2 * a).sum()) < 1e-9


def test_batched_solve_matches_single(cuda):
    import torch
    m = cases.channel(48, 16)
    plist = [dict(Minf=0.5), dict(Minf=0.4, aoa_deg=1.0), dict(Minf=0.55, aoa_deg=-0.5)]
    gd = fv.FlowFV(m, [fv.physics_cfg(**p) for p in plist], fv.numerics_cfg(flux="ROE"), cases.CHANNEL_BCS)
    u0 = np.concatenate([np.tile(u, (m.nelem, 1)) for u in gd.freestream()])
    ud = torch.tensor(u0, device=cuda)
    S = fv.SteadyBackwardEulerSolver(gd, cfl_min=10, cfl_max=1000, tolerance=1e-10, max_timesteps=200, precision=4)
    rc, st = S.solve(ud)
    assert all(s["status"] == 0 for s in st)
    for k, p in enumerate(plist):
        g1 = fv.FlowFV(m, fv.physics_cfg(**p), fv.numerics_cfg(flux="ROE"), cases.CHANNEL_BCS)
        u1 = torch.tensor(np.tile(g1.freestream()[0], (m.nelem, 1)), device=cuda)
        fv.SteadyBackwardEulerSolver(g1, cfl_min=10, cfl_max=1000, tolerance=1e-10, max_timesteps=200,
                                     precision=4).solve(u1)
        a = ud.cpu().numpy()[k * m.nelem:(k + 1) * m.nelem]
        assert np.abs(a - u1.cpu().numpy()).max() / np.abs(a).max() <= 1e-8


def test_divergence_reports_numerical_error(cuda):
    """PseudotimeFlow_exception_nanorinf (tests/flowpseudotime.cpp): a state
    that makes the residual non-finite ends the solve with
    FV_ERR_NUMERICAL (the reference throws Numerical_error).  The fault is
    injected on the host, in the initial state."""
    import torch
    m, gd, od = _setup()
    u0 = np.tile(od.freestream(), (m.nelem, 1))
    u0[5, 3] = -1.0  # negative energy: negative pressure, sound speed NaN
    S = fv.SteadyBackwardEulerSolver(gd, max_timesteps=20, precision=4)
    rc, st = S.solve(torch.tensor(u0, device=cuda), raise_on_error=False)
    assert rc == fv.FV_ERR_NUMERICAL and st[0]["status"] == fv.FV_ERR_NUMERICAL


def test_max_steps_reports_tolerance_error(cuda):
    import torch
    m, gd, od = _setup()
    u0 = np.tile(od.freestream(), (m.nelem, 1))
    S = fv.SteadyBackwardEulerSolver(gd, max_timesteps=3, precision=4)
    rc, st = S.solve(torch.tensor(u0, device=cuda), raise_on_error=False)
    assert rc == fv.FV_ERR_TOLERANCE and st[0]["steps"] == 3


def test_host_buffer_solve(cuda):
    m, gd, od = _setup()
    u = np.ascontiguousarray(np.tile(od.freestream(), (m.nelem, 1)))
    S = fv.SteadyBackwardEulerSolver(gd, cfl_min=10, cfl_max=1000, tolerance=1e-10, max_timesteps=200, precision=4)
    rc, st = S.solve_host(u)
    assert st[0]["status"] == 0 and np.all(np.isfinite(u))


def test_convergence_history_file_format(cuda, tmp_path):
    """The reference's convergence-history columns (aoutput.cpp:617-636), as
    read by its plotting scripts with numpy.genfromtxt."""
    import torch
    m, gd, od = _setup()
    u0 = np.tile(od.freestream(), (m.nelem, 1))
    S = fv.SteadyBackwardEulerSolver(gd, cfl_min=10, cfl_max=1000, tolerance=1e-10, max_timesteps=200, precision=4)
    rc, st = S.solve(torch.tensor(u0, device=cuda))
    path = tmp_path / "conv.log"
    S.write_convergence_history(str(path), wall_time=1.0)
    data = np.genfromtxt(str(path))
    assert data.shape == (st[0]["steps"], 7)
    assert data[0, 0] == 1 and data[-1, 0] == st[0]["steps"]
    assert data[0, 1] == 0.0 and abs(data[-1, 2] - np.log10(st[0]["res"])) < 1e-4  # 6 significant digits
    assert data[-1, 5] == st[0]["lin_iters"] and data[0, 6] == 10.0


def test_batch_member_failure_is_isolated(cuda):
    """A member that diverges (negative energy injected in its initial state,
    on the host) ends with FV_ERR_NUMERICAL; the other members still converge
    to the same state as their single solves."""
    import torch
    m = cases.channel(48, 16)
    plist = [dict(Minf=0.5), dict(Minf=0.45), dict(Minf=0.4, aoa_deg=1.0)]
    gd = fv.FlowFV(m, [fv.physics_cfg(**p) for p in plist], fv.numerics_cfg(flux="ROE"), cases.CHANNEL_BCS)
    us = [np.tile(u, (m.nelem, 1)) for u in gd.freestream()]
    us[1][11, 3] = -1.0
    ud = torch.tensor(np.concatenate(us), device=cuda)
    S = fv.SteadyBackwardEulerSolver(gd, cfl_min=10, cfl_max=1000, tolerance=1e-10, max_timesteps=200, precision=4)
    rc, st = S.solve(ud, raise_on_error=False)
    assert rc == fv.FV_ERR_NUMERICAL
    assert st[1]["status"] == fv.FV_ERR_NUMERICAL
    assert st[0]["status"] == 0 and st[2]["status"] == 0
    g0 = fv.FlowFV(m, fv.physics_cfg(**plist[0]), fv.numerics_cfg(flux="ROE"), cases.CHANNEL_BCS)
    u0 = torch.tensor(np.tile(g0.freestream()[0], (m.nelem, 1)), device=cuda)
    fv.SteadyBackwardEulerSolver(g0, cfl_min=10, cfl_max=1000, tolerance=1e-10, max_timesteps=200,
                                 precision=4).solve(u0)
    a = ud.cpu().numpy()[:m.nelem]
    assert np.abs(a - u0.cpu().numpy()).max() <= 1e-8 * np.abs(a).max()


def test_cpp_interface_solves(cuda, tmp_path):
    """The C++ host interface (include/fvens_gb300.hpp) drives a steady solve
    through the C ABI with host buffers."""
    import os
    import shutil
    import subprocess
    from tests.test_host_cpu import CPP_DRIVER, ROOT
    if not shutil.which("g++"):
        pytest.skip("no g++")
    src = tmp_path / "driver.cpp"
    src.write_text(CPP_DRIVER)
    exe = tmp_path / "driver"
    libdir = os.path.dirname(fv.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-lfvens_gb300", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe), "solve"], check=True, capture_output=True, text=True).stdout.split()
    steps, res = int(out[3]), float(out[4])
    assert 0 < steps < 1000 and res <= 1e-10


def test_matrix_free_solve_matches_oracle(cuda):
    """MatrixFreeSpatialJacobian::apply (alinalg.cpp:143-237) inside the steady
    solve: the GPU's FP64 matrix-free solve and the oracle's take the same
    number of steps (within two) and reach the same converged state."""
    import torch
    m, gd, od = _setup()
    u0 = np.tile(od.freestream(), (m.nelem, 1))
    S = fv.SteadyBackwardEulerSolver(gd, cfl_min=10, cfl_max=1000, tolerance=1e-10, max_timesteps=200,
                                     pc="ilu0", precision=8, matrix_free=1)
    ud = torch.tensor(u0, device=cuda)
    rc, st = S.solve(ud)
    P = fv.Preconditioner(gd, fv.BlockMatrix(gd, 8), "ilu0")
    uo, sto = od.steady_solve(u0, cflmin=10, cflmax=1000, tol=1e-10, maxiter=200, pc="ilu0", matrix_free=True,
                              order=P.order())
    assert st[0]["status"] == 0 and sto["status"] == 0
    assert abs(st[0]["steps"] - sto["steps"]) <= 2
    ug = ud.cpu().numpy()
    assert np.abs(ug - uo).max() / np.abs(uo).max() <= 1e-8


def test_matrix_free_first_order_matches_matrix_based(cuda):
    """The reference's Flow_Euler_Cylinder_HLLC_MatFreeVsMat
    (tests/solvers/testmatrixfree.cpp, matfree.ctrl): for a first-order HLLC
    discretisation the stored Jacobian is the residual's exact derivative, so
    the matrix-free solve (difference step 1e-6) takes the steps of the
    matrix-based one (M 0.38, CFL 50 -> 3000, relative tolerance 1e-8, FGMRES
    rtol 1e-2; here on the NACA 0012 O-grid with ILU(0))."""
    import torch
    m = cases.naca()
    d = fv.FlowFV(m, fv.physics_cfg(Minf=0.38), fv.numerics_cfg(flux="HLLC", gradient="NONE"), cases.NACA_INV_BCS)
    cfg = dict(cfl_min=50, cfl_max=3000, tolerance=1e-8, abs_tolerance=0, max_timesteps=100, pc="ilu0", precision=8,
               ksp_rtol=1e-2)
    u0 = torch.tensor(np.tile(d.freestream()[0], (m.nelem, 1)), device=cuda)
    ua, ub = u0.clone(), u0.clone()
    _, sa = fv.SteadyBackwardEulerSolver(d, **cfg).solve(ua)
    _, sb = fv.SteadyBackwardEulerSolver(d, matrix_free=1, mf_eps=1e-6, **cfg).solve(ub)
    assert sa[0]["status"] == 0 and sb[0]["status"] == 0
    assert abs(sa[0]["steps"] - sb[0]["steps"]) <= 1, (sa[0]["steps"], sb[0]["steps"])
    assert (ua - ub).abs().max().item() <= 1e-6 * ua.abs().max().item()


def test_stagnation_stop(cuda):
    """stall_steps (not in the reference): a member whose residual stops
    falling ends early with FV_ERR_TOLERANCE; a converging solve is unchanged
    by it.  The unreachable tolerance (1e-30) makes every step after the
    rounding floor a stall."""
    import torch
    m, gd, od = _setup()
    u0 = torch.tensor(np.tile(od.freestream(), (m.nelem, 1)), device=cuda)
    kw = dict(cfl_min=10, cfl_max=1000, pc="ilu0", precision=4)
    ud = u0.clone()
    rc, st = fv.SteadyBackwardEulerSolver(gd, tolerance=1e-30, max_timesteps=2000, stall_steps=20,
                                          **kw).solve(ud, raise_on_error=False)
    assert rc == fv.FV_ERR_TOLERANCE and st[0]["status"] == fv.FV_ERR_TOLERANCE
    assert 20 < st[0]["steps"] < 2000 and st[0]["res"] < 1e-12
    # converging: identical path and state with and without the stop
    ua, ub = u0.clone(), u0.clone()
    _, sa = fv.SteadyBackwardEulerSolver(gd, tolerance=1e-10, max_timesteps=200, **kw).solve(ua)
    _, sb = fv.SteadyBackwardEulerSolver(gd, tolerance=1e-10, max_timesteps=200, stall_steps=20,
                                         **kw).solve(ub)
    assert sa[0]["steps"] == sb[0]["steps"] and torch.equal(ua, ub)
    with pytest.raises(fv.FvensError):
        fv.SteadyBackwardEulerSolver(gd, stall_steps=10, stall_factor=1.5, **kw)
