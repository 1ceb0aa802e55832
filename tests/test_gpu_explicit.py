"""Explicit time stepping on the GPU against the oracle's restatements of
SteadyForwardEulerSolver::solve (aodesolver.cpp:136-282) and
TVDRKSolver::solve (aodesolver.cpp:671-765)."""
import numpy as np
import pytest

import fvens_gb300 as fv
from oracle import orc
from tests import cases

pytestmark = pytest.mark.gpu


def _channel(**phys):
    m = cases.channel(48, 16)
    pk = dict(Minf=0.5, **phys)
    gd = fv.FlowFV(m, fv.physics_cfg(**pk), fv.numerics_cfg(flux="ROE"), cases.CHANNEL_BCS)
    od = orc.Disc(orc.Mesh.from_export(m.export()), **pk, flux="ROE", bcs=cases.CHANNEL_BCS)
    return m, gd, od


def test_forward_euler_steps_match_oracle(cuda):
    import torch
    m, gd, od = _channel()
    u0 = cases.perturbed_state(od.freestream(), m.nelem, amp=0.01)
    ud = torch.tensor(u0, device=cuda)
    rc, st = gd.steady_fe_solve(ud, cfl=0.8, tolerance=1e-14, max_timesteps=60, abs_tolerance=True,
                                raise_on_error=False)
    uo, sto = od.steady_fe(u0, cflinit=0.8, tol=1e-14, maxiter=60, abs_tol=True)
    assert rc == fv.FV_ERR_TOLERANCE and sto["status"] == 4
    assert st[0]["steps"] == sto["steps"] == 60
    assert abs(st[0]["res"] - sto["res"]) <= 1e-10 * sto["res"]
    assert abs(st[0]["res0"] - sto["res0"]) <= 1e-12 * sto["res0"]
    ug = ud.cpu().numpy()
    assert np.abs(ug - uo).max() <= 1e-11 * np.abs(uo).max()


def test_forward_euler_relative_tolerance_stop(cuda):
    """The loop stops once ||R|| / ||R_0|| <= tol, before max_timesteps."""
    import torch
    m, gd, od = _channel()
    u0 = cases.perturbed_state(od.freestream(), m.nelem, amp=0.02)
    ud = torch.tensor(u0, device=cuda)
    rc, st = gd.steady_fe_solve(ud, cfl=0.8, tolerance=0.5, max_timesteps=400, abs_tolerance=False,
                                raise_on_error=False)
    uo, sto = od.steady_fe(u0, cflinit=0.8, tol=0.5, maxiter=400, abs_tol=False)
    assert rc == fv.FV_OK and sto["status"] == 0
    assert st[0]["steps"] == sto["steps"] and st[0]["steps"] < 400
    assert st[0]["res"] <= 0.5 * st[0]["res0"]


def test_forward_euler_divergence_reports_numerical_error(cuda):
    import torch
    m, gd, od = _channel()
    u0 = np.tile(od.freestream(), (m.nelem, 1))
    u0[7, 3] = -1.0
    rc, st = gd.steady_fe_solve(torch.tensor(u0, device=cuda), cfl=0.8, max_timesteps=10, raise_on_error=False)
    assert rc == fv.FV_ERR_NUMERICAL and st[0]["status"] == fv.FV_ERR_NUMERICAL


def test_forward_euler_batch_members_independent(cuda):
    import torch
    m = cases.channel(48, 16)
    plist = [dict(Minf=0.5), dict(Minf=0.35, aoa_deg=1.0)]
    gd = fv.FlowFV(m, [fv.physics_cfg(**p) for p in plist], fv.numerics_cfg(flux="ROE"), cases.CHANNEL_BCS)
    us = [cases.perturbed_state(u, m.nelem, amp=0.01, seed=3 + k) for k, u in enumerate(gd.freestream())]
    ud = torch.tensor(np.concatenate(us), device=cuda)
    gd.steady_fe_solve(ud, cfl=0.8, tolerance=1e-14, max_timesteps=30, raise_on_error=False)
    for k, p in enumerate(plist):
        od = orc.Disc(orc.Mesh.from_export(m.export()), **p, flux="ROE", bcs=cases.CHANNEL_BCS)
        uo, _ = od.steady_fe(us[k], cflinit=0.8, tol=1e-14, maxiter=30)
        ug = ud.cpu().numpy()[k * m.nelem:(k + 1) * m.nelem]
        assert np.abs(ug - uo).max() <= 1e-11 * np.abs(uo).max()


@pytest.mark.parametrize("order", [1, 2, 3])
def test_tvdrk_matches_oracle(cuda, order):
    import torch
    m, gd, od = _channel()
    u0 = cases.perturbed_state(od.freestream(), m.nelem, amp=0.01)
    # a final time of a few steps (dt = cfl * min local time step)
    _, dt = od.residual(u0)
    cfl = 0.2
    final = 4.5 * cfl * dt.min()
    ud = torch.tensor(u0, device=cuda)
    rc, steps, tm = gd.tvdrk_solve(ud, order, cfl, final)
    uo, so, stat, to = od.tvdrk(u0, order, cfl, final)
    assert rc == fv.FV_OK and stat == 0
    assert steps[0] == so and so >= 4
    assert abs(tm[0] - to) <= 1e-12 * to
    ug = ud.cpu().numpy()
    assert np.abs(ug - uo).max() <= 1e-12 * np.abs(uo).max()


def test_tvdrk_step_bound(cuda):
    import torch
    m, gd, od = _channel()
    ud = torch.tensor(np.tile(od.freestream(), (m.nelem, 1)), device=cuda)
    rc, steps, tm = gd.tvdrk_solve(ud, 3, 0.2, 1.0e3, max_steps=5, raise_on_error=False)
    assert rc == fv.FV_ERR_TOLERANCE and steps[0] == 5


def test_explicit_entropy_convergence_on_reference_cylinders(cuda):
    """The reference's explicit entropy-convergence test (expl-inv-cyl-gg-roe_tri.ctrl
    on 2dcylinder1 and 2dcylinder2): the GPU's forward-Euler starter and main
    solve stop at the oracle's step counts with entropy errors within 1e-8 of
    the oracle's, and the order between the meshes lies in [1.65, 2.1]."""
    import torch

    from tests import regression_cases as rcases
    c, x = rcases.CYLINDER, rcases.CYLINDER_EXPLICIT
    s1, s2 = x["start"], x["main"]
    logs = []
    for m in rcases.load_cylinders()[1:3]:
        ph = fv.physics_cfg(**c["phys"])
        start = fv.FlowFV(m, ph, fv.numerics_cfg(flux=x["flux"], gradient="NONE"), c["bcs"])
        main = fv.FlowFV(m, ph, fv.numerics_cfg(flux=x["flux"], gradient=x["gradient"]), c["bcs"])
        ud = torch.tensor(np.tile(main.freestream()[0], (m.nelem, 1)), device=cuda)
        _, st1 = start.steady_fe_solve(ud, cfl=s1["cfl"], tolerance=s1["tolerance"],
                                       max_timesteps=s1["max_timesteps"], abs_tolerance=False)
        _, st2 = main.steady_fe_solve(ud, cfl=s2["cfl"], tolerance=s2["tolerance"],
                                      max_timesteps=s2["max_timesteps"], abs_tolerance=False)
        om = orc.Mesh.from_export(m.export())
        d1 = orc.Disc(om, **c["phys"], flux=x["flux"], gradient="NONE", bcs=c["bcs"])
        d2 = orc.Disc(om, **c["phys"], flux=x["flux"], gradient=x["gradient"], bcs=c["bcs"])
        u1, a = d1.steady_fe(np.tile(d2.freestream(), (m.nelem, 1)), s1["cfl"], tol=s1["tolerance"],
                             maxiter=s1["max_timesteps"], abs_tol=False)
        u2, b = d2.steady_fe(u1, s2["cfl"], tol=s2["tolerance"], maxiter=s2["max_timesteps"], abs_tol=False)
        assert (st1[0]["steps"], st2[0]["steps"]) == (a["steps"], b["steps"])
        e, eo = main.entropy_error(ud)[0], d2.entropy_error(u2)
        assert abs(e - eo) <= 1e-8 * eo, (m.nelem, e, eo)
        logs.append((np.log10(1.0 / np.sqrt(m.nelem)), np.log10(e)))
    slope = (logs[1][1] - logs[0][1]) / (logs[1][0] - logs[0][0])
    assert 1.65 <= slope <= 2.1, (slope, logs)
