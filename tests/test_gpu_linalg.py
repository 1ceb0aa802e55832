"""GPU preconditioners, block SpMV and FGMRES against the oracle's
restatement of PETSc's block ILU(0) / SOR(SGS) / point-block Jacobi and
FGMRES, on the same matrix and the same elimination order."""
import numpy as np
import pytest

import fvens_gb300 as fv
from oracle import orc
from tests import cases

pytestmark = pytest.mark.gpu


def _system(cuda, prec, mesh=None):
    """C1-like Jacobian at a perturbed state plus a pseudo-time diagonal
    (as the solver builds it at CFL 50)."""
    import torch
    m = mesh or cases.channel(48, 16)
    gd = fv.FlowFV(m, fv.physics_cfg(Minf=0.5), fv.numerics_cfg(flux="ROE"), cases.CHANNEL_BCS)
    od = orc.Disc(orc.Mesh.from_export(m.export()), Minf=0.5, flux="ROE", bcs=cases.CHANNEL_BCS)
    u = cases.perturbed_state(od.freestream(), m.nelem)
    ud = torch.tensor(u, device=cuda)
    A = fv.BlockMatrix(gd, prec)
    gd.assemble_jacobian(ud, A)
    _, dt = od.residual(u)
    diag = m.geometry()["area"] / (50.0 * dt)
    A.add_diagonal(torch.tensor(diag, device=cuda))
    rp, col, val = A.to_host()
    return m, gd, A, rp, col, val


@pytest.mark.parametrize("prec,tol", [(8, 1e-11), (4, 3e-5)])
@pytest.mark.parametrize("kind", ["jacobi", "sgs", "ilu0"])
@pytest.mark.parametrize("ordering", [1, 2, 0])
def test_precond_apply(cuda, prec, tol, kind, ordering):
    import torch
    m, gd, A, rp, col, val = _system(cuda, prec)
    P = fv.Preconditioner(gd, A, kind, ordering=ordering, part_size=64)
    P.setup()
    rng = np.random.default_rng(5)
    r = rng.normal(size=(m.nelem, 4))
    z = torch.zeros((m.nelem, 4), dtype=torch.float64, device=cuda)
    P.apply(torch.tensor(r, device=cuda), z)
    zo = orc.precond_apply(rp, col, val, kind, r.ravel(), order=P.order()).reshape(-1, 4)
    err = np.abs(z.cpu().numpy() - zo).max() / np.abs(zo).max()
    assert err <= tol, f"{kind} prec {prec} ordering {ordering}: {err:.3e}"


@pytest.mark.parametrize("ordering", [1, 2])
def test_block_order_is_valid(cuda, ordering):
    m, gd, A, rp, col, val = _system(cuda, 8, mesh=cases.channel(96, 32))
    P = fv.Preconditioner(gd, A, "ilu0", ordering=ordering, part_size=128)
    order = P.order()
    assert np.array_equal(np.sort(order), np.arange(m.nelem))


def test_spmv(cuda):
    import torch
    m, gd, A, rp, col, val = _system(cuda, 8)
    x = np.random.default_rng(2).normal(size=(m.nelem, 4))
    y = torch.zeros((m.nelem, 4), dtype=torch.float64, device=cuda)
    fv.matvec(gd, A, torch.tensor(x, device=cuda), y)
    yo = np.zeros_like(x)
    for i in range(m.nelem):
        for k in range(rp[i], rp[i + 1]):
            yo[i] += val[k].reshape(4, 4) @ x[col[k]]
    assert np.abs(y.cpu().numpy() - yo).max() <= 1e-12 * np.abs(yo).max()


@pytest.mark.parametrize("kind", ["ilu0", "sgs"])
def test_fgmres_matches_oracle(cuda, kind):
    """FP64 matrix and factor: same Krylov iterates as the oracle's FGMRES."""
    import torch
    m, gd, A, rp, col, val = _system(cuda, 8)
    P = fv.Preconditioner(gd, A, kind, ordering=1, part_size=64)
    P.setup()
    b = np.random.default_rng(9).normal(size=(m.nelem, 4))
    x = torch.zeros_like(torch.tensor(b, device=cuda))
    its = P.ksp_solve(torch.tensor(b, device=cuda), x, restart=30, maxit=30, rtol=1e-6)
    xo, itso, rno = orc.fgmres(rp, col, val, kind, b.ravel(), restart=30, maxit=30, rtol=1e-6, order=P.order())
    assert its[0] == itso
    err = np.abs(x.cpu().numpy().ravel() - xo).max() / np.abs(xo).max()
    assert err <= 1e-8, err
    # the iterate really reduces the residual by rtol
    res = b.ravel().copy()
    xx = x.cpu().numpy()
    for i in range(m.nelem):
        for k in range(rp[i], rp[i + 1]):
            res[4 * i:4 * i + 4] -= val[k].reshape(4, 4) @ xx[col[k]]
    # classical Gram-Schmidt (PETSc default, no refinement): the recursive residual
    # estimate and the true residual part ways at tight tolerances
    assert np.linalg.norm(res) <= 1e-5 * np.linalg.norm(b)


@pytest.mark.parametrize("kind", ["ilu0", "sgs"])
def test_line_aware_parts_match_oracle(cuda, kind):
    """With lines of strongly coupled cells (findLines) on the reference's
    laminar hybrid mesh, the parts take whole lines; the preconditioner is
    still exactly the oracle's ILU(0) / SGS in the same elimination order."""
    import torch
    from tests import regression_cases as rc
    m, c, regr = rc.load("laminar_naca0012_hybrid1")
    nl, cl = m.find_lines(10.0)
    assert nl > 100
    ph = dict(Minf=0.5, Reinf=5000.0, viscous=True)
    gd = fv.FlowFV(m, fv.physics_cfg(**ph), fv.numerics_cfg(flux="ROE"), c["bcs"])
    od = orc.Disc(orc.Mesh.from_export(m.export()), **ph, flux="ROE", bcs=c["bcs"])
    u = cases.perturbed_state(od.freestream(), m.nelem)
    A = fv.BlockMatrix(gd, 8)
    gd.assemble_jacobian(torch.tensor(u, device=cuda), A)
    _, dt = od.residual(u)
    A.add_diagonal(torch.tensor(m.geometry()["area"] / (100.0 * dt), device=cuda))
    rp, col, val = A.to_host()
    P = fv.Preconditioner(gd, A, kind, ordering=1, part_size=128)
    P.setup()
    order = P.order()
    # every line's first piece (up to 128 cells) sits in consecutive positions of one part
    pos = np.empty(m.nelem, np.int64)
    pos[order] = np.arange(m.nelem)
    first = np.where(cl == 0)[0]
    assert pos[first].max() - pos[first].min() < 128
    r = np.random.default_rng(5).normal(size=(m.nelem, 4))
    z = torch.zeros((m.nelem, 4), dtype=torch.float64, device=cuda)
    P.apply(torch.tensor(r, device=cuda), z)
    zo = orc.precond_apply(rp, col, val, kind, r.ravel(), order=order).reshape(-1, 4)
    assert np.abs(z.cpu().numpy() - zo).max() <= 1e-11 * np.abs(zo).max()


@pytest.mark.parametrize("kind", ["ilu0", "sgs"])
def test_batched_apply_with_compact_staging(cuda, kind):
    """A batch large enough that a colour's sweep launch holds more CTAs than
    four per SM (32 members x ~58 parts of 64 cells), where the sweeps stage
    only the in-part blocks each part has: every member's apply equals the
    single condition's apply (fixed staging slots) bit for bit, and the
    oracle's to the FP32 tolerance."""
    import torch
    m = cases.channel(192, 64)
    B = 32
    ph = fv.physics_cfg(Minf=0.5)
    num = fv.numerics_cfg(flux="ROE")
    g1 = fv.FlowFV(m, ph, num, cases.CHANNEL_BCS)
    gB = fv.FlowFV(m, [ph] * B, num, cases.CHANNEL_BCS)
    od = orc.Disc(orc.Mesh.from_export(m.export()), Minf=0.5, flux="ROE", bcs=cases.CHANNEL_BCS)
    u = cases.perturbed_state(od.freestream(), m.nelem)
    _, dt = od.residual(u)
    diag = m.geometry()["area"] / (50.0 * dt)
    A1, AB = fv.BlockMatrix(g1, 4), fv.BlockMatrix(gB, 4)
    g1.assemble_jacobian(torch.tensor(u, device=cuda), A1)
    gB.assemble_jacobian(torch.tensor(np.tile(u, (B, 1)), device=cuda), AB)
    A1.add_diagonal(torch.tensor(diag, device=cuda))
    AB.add_diagonal(torch.tensor(np.tile(diag, B), device=cuda))
    P1 = fv.Preconditioner(g1, A1, kind, ordering=1, part_size=64)
    PB = fv.Preconditioner(gB, AB, kind, ordering=1, part_size=64)
    P1.setup()
    PB.setup()
    r = np.random.default_rng(11).normal(size=(m.nelem, 4))
    z1 = torch.zeros((m.nelem, 4), dtype=torch.float64, device=cuda)
    zB = torch.zeros((B * m.nelem, 4), dtype=torch.float64, device=cuda)
    P1.apply(torch.tensor(r, device=cuda), z1)
    PB.apply(torch.tensor(np.tile(r, (B, 1)), device=cuda), zB)
    for k in range(B):
        assert torch.equal(zB[k * m.nelem:(k + 1) * m.nelem], z1), k
    rp, col, val = A1.to_host()
    zo = orc.precond_apply(rp, col, val, kind, r.ravel(), order=P1.order()).reshape(-1, 4)
    assert np.abs(z1.cpu().numpy() - zo).max() <= 3e-5 * np.abs(zo).max()
