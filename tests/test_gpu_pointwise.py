"""Device pointwise physics (fluxes, flux Jacobians, BC ghost states and
BC Jacobians) against golden vectors produced by the reference's own compiled
code (tests/golden/pointwise.npz)."""
import os

import numpy as np
import pytest

import fvens_gb300 as fv
from tests import cases

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "pointwise.npz"))


@pytest.fixture(scope="module")
def disc(cuda):
    ph = GOLD["phys"]
    m = cases.channel(8, 4)
    return fv.FlowFV(m, fv.physics_cfg(gamma=ph[0], Minf=ph[1], Tinf=ph[2], Reinf=ph[3], Pr=ph[4],
                                       aoa_deg=np.rad2deg(GOLD["aoa"][0])),
                     fv.numerics_cfg(), cases.CHANNEL_BCS)


def _t(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("k", range(7))
def test_device_flux(disc, k):
    import torch
    ul, ur, n = _t(GOLD["ul"]), _t(GOLD["ur"]), _t(GOLD["n"])
    f = torch.zeros_like(ul)
    fv.check(fv.lib().fv_pointwise_flux(disc._h, k, len(GOLD["ul"]), fv._vp(fv.dptr(ul)), fv._vp(fv.dptr(ur)),
                                        fv._vp(fv.dptr(n)), fv._vp(fv.dptr(f))))
    ref = GOLD[f"flux_{k}"]
    err = np.abs(f.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 1e-14, err


@pytest.mark.parametrize("k", [0, 2, 4, 5, 6])
@pytest.mark.parametrize("wall", [False, True])
def test_device_flux_jacobian(disc, k, wall):
    import torch
    if wall and k not in (4, 6):
        pytest.skip("wall pairs generated for Roe and HLLC")
    ul, n = _t(GOLD["ul"]), _t(GOLD["n"])
    ur = _t(GOLD["wall_ur"] if wall else GOLD["ur"])
    N = len(GOLD["ul"])
    dl = torch.zeros((N, 16), dtype=torch.float64, device="cuda")
    dr = torch.zeros_like(dl)
    fv.check(fv.lib().fv_pointwise_flux_jacobian(disc._h, k, N, fv._vp(fv.dptr(ul)), fv._vp(fv.dptr(ur)),
                                                 fv._vp(fv.dptr(n)), fv._vp(fv.dptr(dl)), fv._vp(fv.dptr(dr))))
    pre = "w" if wall else ""
    rl, rr = GOLD[f"{pre}dfdl_{k}"], GOLD[f"{pre}dfdr_{k}"]
    for i in range(N):
        sc = max(np.abs(rl[i]).max(), np.abs(rr[i]).max())
        assert np.abs(dl[i].cpu().numpy() - rl[i]).max() <= 1e-11 * sc
        assert np.abs(dr[i].cpu().numpy() - rr[i]).max() <= 1e-11 * sc


@pytest.mark.parametrize("t", [0, 1, 2, 3, 4, 6, 7])
def test_device_bc(disc, t):
    import torch
    N = len(GOLD["ul"])
    ins, n = _t(GOLD["ul"]), _t(GOLD["n"])
    g = torch.zeros((N, 4), dtype=torch.float64, device="cuda")
    gj = torch.zeros_like(g)
    G = torch.zeros((N, 16), dtype=torch.float64, device="cuda")
    vals = np.ascontiguousarray(GOLD[f"bc_{t}_vals"], np.float64)
    fv.check(fv.lib().fv_pointwise_bc(disc._h, t, fv._hp(vals, fv.ctypes.c_double), N, fv._vp(fv.dptr(ins)),
                                      fv._vp(fv.dptr(n)), fv._vp(fv.dptr(g)), fv._vp(fv.dptr(gj)),
                                      fv._vp(fv.dptr(G))))
    ref = GOLD[f"bc_{t}_ghost"]
    ok = np.all(np.isfinite(ref), axis=1)
    gh = g.cpu().numpy()
    assert np.abs(gh[ok] - ref[ok]).max() <= 1e-13 * np.abs(ref[ok]).max()
    if t == 3:
        return  # the reference has no subsonic-inflow Jacobian (abc.cpp:179-185 exits)
    assert np.abs(gj.cpu().numpy() - GOLD[f"bc_{t}_jghost"]).max() <= 1e-13 * np.abs(GOLD[f"bc_{t}_jghost"]).max()
    Gr = GOLD[f"bc_{t}_dgdu"]
    assert np.abs(G.cpu().numpy() - Gr).max() <= 1e-12 * max(1.0, np.abs(Gr).max())
