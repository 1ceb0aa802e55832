"""fv_compute_residual_static (scratch in the library's static device array,
no allocation) against fv_compute_residual (the handle's own scratch), called
through the C ABI; collected last so it also runs after every other test."""
import ctypes

import numpy as np
import pytest

import fvens_gb300 as fv
from tests import cases

pytestmark = pytest.mark.gpu


def _static_residual(gd, u, r, dt):
    L = fv.lib()
    return L.fv_compute_residual_static(gd._h, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(r.data_ptr()),
                                        1 if dt is not None else 0,
                                        ctypes.c_void_p(dt.data_ptr()) if dt is not None else None)


@pytest.mark.parametrize("mesh,phys,num,bcs", [
    (cases.naca, dict(Minf=0.8, aoa_deg=1.25),
     dict(flux="HLLC", gradient="GREENGAUSS", reconstruction="VENKATAKRISHNAN", limiter_param=5.0), cases.NACA_INV_BCS),
    (cases.naca_visc, dict(Minf=0.5, Reinf=5000.0, viscous=True, aoa_deg=1.0),
     dict(flux="ROE", reconstruction="WENO", limiter_param=20.0), cases.NACA_VISC_BCS),
], ids=["hllc_gg_venkat", "viscous_roe_weno"])
def test_static_scratch_residual_matches_two_calls(cuda, mesh, phys, num, bcs):
    import torch
    m = mesh()
    gd = fv.FlowFV(m, fv.physics_cfg(**phys), fv.numerics_cfg(**num), bcs)
    for call in range(2):
        u = torch.tensor(cases.perturbed_state(gd.freestream()[0], m.nelem, seed=100 + call), device=cuda)
        r_ref = torch.zeros_like(u)
        dt_ref = torch.zeros(m.nelem, dtype=torch.float64, device=cuda)
        gd.compute_residual(u, r_ref, True, dt_ref)
        r = torch.zeros_like(u)
        dt = torch.zeros_like(dt_ref)
        torch.cuda.synchronize()
        if call == 0:
            # the process's first call loads the array with the library's
            # device image (a one-time, load-time reservation); every call
            # from then on must leave the device's free memory as it was
            assert _static_residual(gd, u, torch.zeros_like(u), torch.zeros_like(dt)) == fv.FV_OK
            torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(cuda)[0]
        assert _static_residual(gd, u, r, dt) == fv.FV_OK
        torch.cuda.synchronize()
        # the device's free memory (driver view) is unchanged by the call
        assert torch.cuda.mem_get_info(cuda)[0] == free0, f"call {call}: device memory was allocated"
        assert torch.equal(r, r_ref), f"call {call}: residuals differ"
        assert torch.equal(dt, dt_ref), f"call {call}: time steps differ"
        # the handle's own scratch is untouched: its next evaluation is unchanged
        r2 = torch.zeros_like(u)
        gd.compute_residual(u, r2, True, dt_ref)
        assert torch.equal(r2, r_ref), f"call {call}: the handle's own evaluation changed"


def test_static_scratch_rejects_oversized(cuda):
    import torch
    m = cases.naca()
    B = 200  # about 0.5 MB of scratch per condition on this mesh: beyond the 64 MiB array
    gd = fv.FlowFV(m, [fv.physics_cfg(Minf=0.5)] * B, fv.numerics_cfg(flux="ROE"), cases.NACA_INV_BCS)
    u = torch.tensor(np.concatenate([np.tile(x, (m.nelem, 1)) for x in gd.freestream()]), device=cuda)
    r = torch.zeros_like(u)
    assert _static_residual(gd, u, r, None) == fv.FV_ERR_INVALID
    assert b"static residual scratch" in fv.lib().fv_last_error()
