"""GPU residual, local time steps and gradients against the CPU oracle on the
same mesh and state.  Parity metric (1e-12): max |R_gpu - R_oracle| divided by
the largest per-cell sum of |F * len| over the cell's faces."""
import numpy as np
import pytest

import fvens_gb300 as fv
from oracle import orc
from tests import cases

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _setup(mesh_fn, phys_kw, num_kw, bcs, batch_phys=None):
    m = mesh_fn()
    om = orc.Mesh.from_export(m.export())
    plist = batch_phys or [phys_kw]
    discs = [orc.Disc(om, **pk, **num_kw, bcs=bcs) for pk in plist]
    gd = fv.FlowFV(m, [fv.physics_cfg(**pk) for pk in plist], fv.numerics_cfg(**num_kw), bcs)
    return m, om, discs, gd


@pytest.mark.parametrize("case", cases.RESIDUAL_CASES, ids=[c[0] for c in cases.RESIDUAL_CASES])
def test_residual_and_timesteps(cuda, case):
    import torch
    name, mesh_fn, phys_kw, num_kw, bcs = case
    m, om, (od,), gd = _setup(mesh_fn, phys_kw, num_kw, bcs)
    u = cases.perturbed_state(od.freestream(), m.nelem)
    r_o, dt_o = od.residual(u)
    scale = od.flux_scale(u).max()
    ud = torch.tensor(u, device=cuda)
    r0 = np.random.default_rng(3).normal(size=u.shape)  # residual is ADDED to the input
    rd = torch.tensor(r0, device=cuda)
    dtd = torch.zeros(m.nelem, dtype=torch.float64, device=cuda)
    gd.compute_residual(ud, rd, True, dtd)
    gd.synchronize()
    err = np.abs(rd.cpu().numpy() - r0 - r_o).max() / scale
    assert err <= TOL, f"{name}: residual parity {err:.3e}"
    dterr = np.abs(dtd.cpu().numpy() - dt_o).max() / np.abs(dt_o).max()
    assert dterr <= TOL, f"{name}: time-step parity {dterr:.3e}"


@pytest.mark.parametrize("scheme", ["LEASTSQUARES", "GREENGAUSS"])
def test_conserved_gradients(cuda, scheme):
    import torch
    m, om, (od,), gd = _setup(cases.naca, dict(Minf=0.8, aoa_deg=1.25), dict(flux="HLLC", gradient=scheme),
                              cases.NACA_INV_BCS)
    u = cases.perturbed_state(od.freestream(), m.nelem)
    g_o = od.conserved_gradients(u)
    g = torch.zeros((m.nelem, 8), dtype=torch.float64, device=cuda)
    gd.get_gradients(torch.tensor(u, device=cuda), g)
    gd.synchronize()
    err = np.abs(g.cpu().numpy() - g_o).max() / np.abs(g_o).max()
    assert err <= 1e-12, err


def test_linear_field_reproduced_by_wls(cuda):
    """testgradientschemes.cpp:36-90: least-squares gradients of a linear
    field are exact, so face values reproduce it to rounding."""
    import torch
    m = cases.naca(nc=48, nr=16)
    geo = m.geometry()
    om = orc.Mesh.from_export(m.export())
    od = orc.Disc(om, Minf=0.5, flux="ROE", gradient="LEASTSQUARES", bcs=[(2, "extrapolation", ()),
                                                                          (4, "extrapolation", ())])
    gd = fv.FlowFV(m, fv.physics_cfg(Minf=0.5), fv.numerics_cfg(flux="ROE"),
                   [(2, "extrapolation", ()), (4, "extrapolation", ())])
    x, y = geo["cc"][:, 0], geo["cc"][:, 1]
    f = 2.0 * x + 0.5 * y + 2.5
    u = np.stack([f, f, f, f + 10], 1)
    g = torch.zeros((m.nelem, 8), dtype=torch.float64, device=cuda)
    gd.get_gradients(torch.tensor(u, device=cuda), g)
    gh = g.cpu().numpy()
    esuel, nnode = om.arrays()["esuel"], m.export()["nnode"]
    interior = np.array([all(0 <= esuel[i, j] < m.nelem for j in range(nnode[i])) for i in range(m.nelem)])
    assert interior.sum() > m.nelem // 2
    np.testing.assert_allclose(gh[interior, 0], 2.0, atol=1e-9)
    np.testing.assert_allclose(gh[interior, 1], 0.5, atol=1e-9)
    go = od.conserved_gradients(u)
    assert np.abs(gh - go).max() <= 1e-12 * np.abs(go).max()


def test_batched_residual(cuda):
    import torch
    plist = [dict(Minf=0.5, aoa_deg=0.0), dict(Minf=0.6, aoa_deg=2.0), dict(Minf=0.4, aoa_deg=-3.0)]
    m, om, ods, gd = _setup(cases.naca, None, dict(flux="ROE", gradient="LEASTSQUARES"), cases.NACA_INV_BCS,
                            batch_phys=plist)
    us = [cases.perturbed_state(od.freestream(), m.nelem, seed=7 + k) for k, od in enumerate(ods)]
    ud = torch.tensor(np.concatenate(us), device=cuda)
    rd = torch.zeros_like(ud)
    dtd = torch.zeros(len(plist) * m.nelem, dtype=torch.float64, device=cuda)
    gd.compute_residual(ud, rd, True, dtd)
    gd.synchronize()
    rh = rd.cpu().numpy().reshape(len(plist), m.nelem, 4)
    for k, od in enumerate(ods):
        r_o, dt_o = od.residual(us[k])
        err = np.abs(rh[k] - r_o).max() / od.flux_scale(us[k]).max()
        assert err <= TOL, (k, err)


def test_freestream_is_steady(cuda):
    """Uniform freestream on a farfield-bounded mesh: every face flux cancels."""
    import torch
    m = cases.naca()
    gd = fv.FlowFV(m, fv.physics_cfg(Minf=0.5, aoa_deg=3.0), fv.numerics_cfg(flux="HLLC"),
                   [(2, "farfield", ()), (4, "farfield", ())])
    uinf = gd.freestream()[0]
    ud = torch.tensor(np.tile(uinf, (m.nelem, 1)), device=cuda)
    rd = torch.zeros_like(ud)
    gd.compute_residual(ud, rd, False, None)
    assert np.abs(rd.cpu().numpy()).max() < 1e-12


def test_autotune_keeps_results(cuda):
    """The block sizes picked by fv_disc_autotune (residual kernels and the
    Jacobian's face kernel) change timing only: the residual, local time steps
    and the FP32 Jacobian are bitwise unchanged."""
    import torch
    name, mesh, phys, num, bcs = cases.RESIDUAL_CASES[1]
    m = mesh()
    gd = fv.FlowFV(m, fv.physics_cfg(**phys), fv.numerics_cfg(**num), bcs)
    u = torch.tensor(cases.perturbed_state(gd.freestream()[0], m.nelem), device=cuda)
    r0, dt0 = torch.zeros_like(u), torch.zeros(m.nelem, dtype=torch.float64, device=cuda)
    gd.compute_residual(u, r0, True, dt0)
    A0 = fv.BlockMatrix(gd, 4)
    gd.assemble_jacobian(u, A0)
    bs = gd.autotune(u)
    assert set(bs) == {"states", "gradients", "faces", "gather", "jacobian_faces"}
    assert all(b in (64, 128, 256) for b in bs.values())
    r1, dt1 = torch.zeros_like(u), torch.zeros_like(dt0)
    gd.compute_residual(u, r1, True, dt1)
    assert torch.equal(r0, r1) and torch.equal(dt0, dt1)
    A1 = fv.BlockMatrix(gd, 4)
    gd.assemble_jacobian(u, A1)
    gd.synchronize()
    assert np.array_equal(A0.to_host()[2], A1.to_host()[2])
