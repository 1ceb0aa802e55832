"""Wall surface functionals (Cl, CDp, CDsf) on the GPU against the oracle's
restatement of FlowFV_base::computeSurfaceData (flow_spatial.cpp:130-310)."""
import numpy as np
import pytest

import fvens_gb300 as fv
from oracle import orc
from tests import cases

pytestmark = pytest.mark.gpu

SURFACE_CASES = [
    ("inviscid_hllc_gg", cases.naca, dict(Minf=0.8, aoa_deg=1.25), dict(flux="HLLC", gradient="GREENGAUSS"),
     cases.NACA_INV_BCS),
    ("viscous_wls_sutherland", cases.naca_visc, dict(Minf=0.5, Reinf=5000.0, viscous=True, aoa_deg=2.0),
     dict(flux="ROE"), cases.NACA_VISC_BCS),
    ("viscous_first_order", cases.naca_visc, dict(Minf=0.4, Reinf=3000.0, viscous=True, aoa_deg=-3.0),
     dict(flux="ROE", gradient="NONE"), cases.NACA_VISC_BCS),
]


@pytest.mark.parametrize("name,mesh,phys,num,bcs", SURFACE_CASES, ids=[c[0] for c in SURFACE_CASES])
def test_surface_data_matches_oracle(cuda, name, mesh, phys, num, bcs):
    import torch
    m = mesh()
    gd = fv.FlowFV(m, fv.physics_cfg(**phys), fv.numerics_cfg(**num), bcs)
    od = orc.Disc(orc.Mesh.from_export(m.export()), **phys, **num, bcs=bcs)
    u = cases.perturbed_state(od.freestream(), m.nelem)
    got = gd.surface_data(torch.tensor(u, device=cuda), 2)[0]
    ref = od.surface_data(u, 2)
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 1e-12 * scale, (got, ref)
    if phys.get("viscous") and num.get("gradient") != "NONE":
        assert abs(ref[2]) > 0  # skin friction from the conserved gradients


def test_surface_data_batch_members_independent(cuda):
    import torch
    m = cases.naca_visc()
    plist = [dict(Minf=0.5, Reinf=5000.0, viscous=True, aoa_deg=1.0),
             dict(Minf=0.3, Reinf=2000.0, viscous=True, aoa_deg=-2.0)]
    gd = fv.FlowFV(m, [fv.physics_cfg(**p) for p in plist], fv.numerics_cfg(flux="ROE"), cases.NACA_VISC_BCS)
    us = [cases.perturbed_state(u, m.nelem, seed=7 + k) for k, u in enumerate(gd.freestream())]
    got = gd.surface_data(torch.tensor(np.concatenate(us), device=cuda), 2)
    for k, p in enumerate(plist):
        od = orc.Disc(orc.Mesh.from_export(m.export()), **p, flux="ROE", bcs=cases.NACA_VISC_BCS)
        ref = od.surface_data(us[k], 2)
        assert np.abs(got[k] - ref).max() <= 1e-12 * np.abs(ref).max()


def test_surface_data_unknown_marker_rejected(cuda):
    import torch
    m = cases.naca()
    gd = fv.FlowFV(m, fv.physics_cfg(Minf=0.5), fv.numerics_cfg(flux="ROE"), cases.NACA_INV_BCS)
    u = torch.tensor(np.tile(gd.freestream()[0], (m.nelem, 1)), device=cuda)
    with pytest.raises(fv.FvensError):
        gd.surface_data(u, 99)


@pytest.mark.parametrize("name,mesh,phys,num,bcs", SURFACE_CASES[:2], ids=[c[0] for c in SURFACE_CASES[:2]])
def test_entropy_error_matches_oracle(cuda, name, mesh, phys, num, bcs):
    import torch
    m = mesh()
    gd = fv.FlowFV(m, fv.physics_cfg(**phys), fv.numerics_cfg(**num), bcs)
    od = orc.Disc(orc.Mesh.from_export(m.export()), **phys, **num, bcs=bcs)
    u = cases.perturbed_state(od.freestream(), m.nelem)
    got = gd.entropy_error(torch.tensor(u, device=cuda))[0]
    ref = od.entropy_error(u)
    assert ref > 0 and abs(got - ref) <= 1e-12 * ref


@pytest.mark.parametrize("name,mesh,phys,num,bcs", SURFACE_CASES[:2], ids=[c[0] for c in SURFACE_CASES[:2]])
def test_surface_distribution_matches_oracle(cuda, name, mesh, phys, num, bcs):
    """Per-face (x, y, Cp, Cf) rows of computeSurfaceData's output array."""
    import torch
    m = mesh()
    gd = fv.FlowFV(m, fv.physics_cfg(**phys), fv.numerics_cfg(**num), bcs)
    od = orc.Disc(orc.Mesh.from_export(m.export()), **phys, **num, bcs=bcs)
    u = cases.perturbed_state(od.freestream(), m.nelem)
    got = gd.surface_distribution(torch.tensor(u, device=cuda), 2)
    ref = od.surface_distribution(u, 2)
    assert got.shape == ref.shape and got.shape[0] == int((m.export()["btag"] == 2).sum())
    assert np.abs(got[:, :2] - ref[:, :2]).max() <= 1e-14
    for k in (2, 3):
        assert np.abs(got[:, k] - ref[:, k]).max() <= 1e-12 * max(np.abs(ref[:, k]).max(), 1e-300)


def test_export_surface_files(cuda, tmp_path):
    """FlowOutput::exportSurfaceData's files: wall rows x, y, Cp, Cf with the
    Cl/Cdp/Cdf trailer; other-marker rows x, y, u, v."""
    import torch
    m = cases.naca_visc()
    phys = dict(Minf=0.5, Reinf=5000.0, viscous=True, aoa_deg=2.0)
    gd = fv.FlowFV(m, fv.physics_cfg(**phys), fv.numerics_cfg(flux="ROE"), cases.NACA_VISC_BCS)
    u = cases.perturbed_state(gd.freestream()[0], m.nelem)
    ud = torch.tensor(u, device=cuda)
    base = str(tmp_path / "case")
    coeffs = gd.export_surface_data(ud, [2], [4], base)
    lines = open(base + "-surf_w2.out").read().splitlines()
    assert lines[0] == "#  x \t y \t Cp  \t Cf " and lines[-2] == "# Cl      Cdp      Cdf"
    rows = np.array([[float(x) for x in ln.split()] for ln in lines[1:-2]])
    np.testing.assert_allclose(rows, gd.surface_distribution(ud, 2), rtol=1e-5, atol=1e-12)
    trailer = [float(x) for x in lines[-1][1:].split()]
    np.testing.assert_allclose(trailer, coeffs[2], rtol=1e-5)
    other = open(base + "-surf_o4.out").read().splitlines()
    assert other[0].startswith("#   x")
    o = np.array([[float(x) for x in ln.split()] for ln in other[1:]])
    ex, geo = m.export(), m.geometry()
    far = np.nonzero(ex["btag"] == 4)[0]
    assert o.shape == (len(far), 4)
    cells = geo["face_lr"][far, 0]
    np.testing.assert_allclose(o[:, 2], u[cells, 1] / u[cells, 0], rtol=1e-5)
