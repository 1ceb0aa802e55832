"""A steady case run from a control file (fvens_gb300.case.SteadyFlowCase)
against the same solves set up directly through the binding, and the files
that FlowCase::run_output writes."""
import os
import shutil

import numpy as np
import pytest

import fvens_gb300 as fv
from fvens_gb300 import case
from tests import cases

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_control_file_case_matches_direct_solve(cuda, tmp_path, monkeypatch):
    import torch
    m = cases.channel(48, 16)
    cases.write_gmsh(m, str(tmp_path / "channel.msh"))
    shutil.copy(os.path.join(GOLDEN, "channel_case.ctrl"), tmp_path / "channel_case.ctrl")
    monkeypatch.chdir(tmp_path)
    opts = case.parse_flow_controlfile("channel_case.ctrl")
    so = case.parse_solver_options(os.path.join(GOLDEN, "channel_opts.solverc"))
    c = case.SteadyFlowCase(opts, so)
    f, st = c.run_output(log=lambda *a: None)
    assert st["status"] == 0
    # the same solves through the binding
    mr = fv.UMesh.read("channel.msh", reorder=1)
    ph = fv.physics_cfg(Minf=0.5)
    main = fv.FlowFV(mr, ph, fv.numerics_cfg(flux="ROE", gradient="LEASTSQUARES", limiter_param=20.0),
                     cases.CHANNEL_BCS)
    start = fv.FlowFV(mr, ph, fv.numerics_cfg(flux="ROE", gradient="NONE", limiter_param=1.0), cases.CHANNEL_BCS)
    u = torch.tensor(np.tile(main.freestream()[0], (mr.nelem, 1)), device=cuda)
    fv.SteadyBackwardEulerSolver(start, cfl_min=10, cfl_max=500, tolerance=1e-1, max_timesteps=20, abs_tolerance=0,
                                 pc="ilu0", precision=4).solve(u, raise_on_error=False)
    _, st2 = fv.SteadyBackwardEulerSolver(main, cfl_min=10, cfl_max=1000, tolerance=1e-8, max_timesteps=300,
                                          abs_tolerance=0, pc="ilu0", precision=4).solve(u)
    assert st2[0]["steps"] == st["steps"]
    ref = main.surface_data(u, 1)[0]
    assert abs(f.Cl - ref[0]) <= 1e-13 and abs(f.Cdp - ref[1]) <= 1e-13
    assert abs(f.entropy - main.entropy_error(u)[0]) <= 1e-13 * max(f.entropy, 1e-300)
    # outputs of run_output
    hist = open("channel-residual_history.log").read().splitlines()
    assert len([x for x in hist if not x.startswith("#")]) == st["steps"]
    for name in ("channel-surf_w1.out", "channel-surf_w3.out", "channel-surf_o4.out"):
        assert os.path.getsize(name) > 0
    w1 = open("channel-surf_w1.out").read().splitlines()
    assert w1[0].startswith("#  x") and w1[-2] == "# Cl      Cdp      Cdf"
    assert len(w1) - 3 == int((mr.export()["btag"] == 1).sum())


def test_control_file_case_with_warm_start_network(cuda, tmp_path, monkeypatch):
    """The case runner with a warm-start network (saved and loaded again):
    the main solve starts from the prediction (or falls back to freestream)
    and reaches the functionals of the freestream-started case."""
    from fvens_gb300.mpnn import MPNN
    m = cases.channel(48, 16)
    cases.write_gmsh(m, str(tmp_path / "channel.msh"))
    shutil.copy(os.path.join(GOLDEN, "channel_case.ctrl"), tmp_path / "channel_case.ctrl")
    monkeypatch.chdir(tmp_path)
    opts = case.parse_flow_controlfile("channel_case.ctrl")
    so = case.parse_solver_options(os.path.join(GOLDEN, "channel_opts.solverc"))
    c = case.SteadyFlowCase(opts, so)
    mr = c.read_mesh()
    f_free, st_free = c.run_output(mr, surface_files=False, log=lambda *a: None)
    net = MPNN(mr, layers=2, wall_markers=(1, 3), seed=2)
    p = net.params((np.random.default_rng(0).normal(size=net.nparams) * 0.1).astype(np.float32))
    net.set_scale(np.array([0.01, 0.01, 0.01, 0.02], np.float32))
    net.save(str(tmp_path / "net.npz"))
    net2 = MPNN.load(mr, str(tmp_path / "net.npz"))
    assert np.array_equal(net2.params(), p) and np.array_equal(net2.scale, net.scale)
    f_warm, st_warm = c.run_output(mr, surface_files=False, log=lambda *a: None, net=net2)
    assert st_free["status"] == 0 and st_warm["status"] == 0
    assert abs(f_warm.Cl - f_free.Cl) <= 1e-6 * max(abs(f_free.Cl), 1e-3)
    assert abs(f_warm.Cdp - f_free.Cdp) <= 1e-6 * max(abs(f_free.Cdp), 1e-3)
