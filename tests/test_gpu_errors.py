"""Invalid arguments and configurations on the GPU entry points end with a
status and a message, not a fault: solver configurations outside what the
reference accepts, the Jacobian fluxes the reference does not implement,
null device pointers, unknown markers and members out of range."""
import ctypes

import numpy as np
import pytest

import fvens_gb300 as fv
from tests import cases

pytestmark = pytest.mark.gpu


def _disc(flux="ROE"):
    m = cases.channel(16, 8)
    return m, fv.FlowFV(m, fv.physics_cfg(Minf=0.5), fv.numerics_cfg(flux=flux), cases.CHANNEL_BCS)


@pytest.mark.parametrize("kw,what", [
    (dict(precision=2), "invalid solver configuration"),
    (dict(ksp_restart=0), "invalid solver configuration"),
    (dict(pc_part_size=300), "pc_part_size at most 256"),
    (dict(nl_update=3), "invalid nonlinear update scheme"),
    (dict(nl_update=1, min_relax=0.0), "Minimum relaxation factor is invalid"),
])
def test_solver_configuration_checks(cuda, kw, what):
    _, d = _disc()
    with pytest.raises(fv.FvensError, match=what) as e:
        fv.SteadyBackwardEulerSolver(d, **kw)
    assert e.value.status == fv.FV_ERR_INVALID


def test_jacobian_flux_without_reference_jacobian(cuda):
    m = cases.channel(16, 8)
    d = fv.FlowFV(m, fv.physics_cfg(Minf=0.5), fv.numerics_cfg(flux="ROE", flux_jac="AUSMPLUS"), cases.CHANNEL_BCS)
    with pytest.raises(fv.FvensError) as e:
        fv.SteadyBackwardEulerSolver(d)
    assert e.value.status == fv.FV_ERR_UNSUPPORTED


def test_null_pointers_and_ranges(cuda):
    import torch
    m, d = _disc()
    u = torch.tensor(np.tile(d.freestream()[0], (m.nelem, 1)), device=cuda)
    L = fv.lib()
    assert L.fv_compute_residual(d._h, None, fv._vp(fv.dptr(u)), 0, None) == fv.FV_ERR_INVALID
    assert L.fv_compute_residual(d._h, fv._vp(fv.dptr(u)), fv._vp(fv.dptr(u)), 1, None) == fv.FV_ERR_INVALID
    n = ctypes.c_int()
    assert L.fv_surface_distribution(d._h, None, 1, 3, None, ctypes.byref(n)) == fv.FV_ERR_INVALID
    with pytest.raises(fv.FvensError, match="no boundary face has marker 99"):
        d.surface_distribution(u, 99)
    # the discretisation stays usable after the rejected calls
    r = torch.zeros_like(u)
    d.compute_residual(u, r)
    d.synchronize()
    assert torch.isfinite(r).all()
