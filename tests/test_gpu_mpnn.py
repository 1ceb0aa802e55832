"""The warm-start network on the GPU (fv_mpnn.cu): forward pass and gradients
against the CPU oracle (oracle/mpnn_ref.py, with the same bfloat16 rounding
of GEMM operands), Adam training, and what the trained network gains over
the freestream start of a steady solve."""
import numpy as np
import pytest

import fvens_gb300 as fv
from fvens_gb300.mpnn import MPNN, output_scale, train
from oracle import mpnn_ref as M
from tests import cases

pytestmark = pytest.mark.gpu


def _conds(machs, aoas=None):
    aoas = aoas if aoas is not None else [0.0] * len(machs)
    dicts = [dict(Minf=m, aoa_deg=a, Reinf=np.inf, viscous=False) for m, a in zip(machs, aoas)]
    return [fv.physics_cfg(Minf=m, aoa_deg=a) for m, a in zip(machs, aoas)], dicts


def _random_params(net, seed, amp=0.15):
    rng = np.random.default_rng(seed)
    p = (rng.normal(size=net.nparams) * amp).astype(np.float32)
    return net.params(p)


@pytest.mark.parametrize("path", ["tcgen05", "mma_sync"])
def test_forward_and_gradients_match_oracle(cuda, path):
    import torch
    m = cases.channel(24, 8)
    net = MPNN(m, layers=2, wall_markers=(1, 3), seed=5)
    net.set_gemm_path(path)
    p = _random_params(net, 7)
    scale = np.array([0.05, 0.1, 0.08, 0.3], np.float32)
    net.set_scale(scale)
    phys, dicts = _conds([0.45, 0.55], [1.0, -2.0])
    cond, uinf = M.conditions(dicts)
    xs, faces, ea = net.graph()
    assert faces.shape[0] == m.naface - m.nbface and xs.shape == (m.nelem, 4)
    ref = M.Net(xs, faces, ea, 2, bf16_operands=True)
    # forward: u = uinf + scale * y
    u = torch.zeros((2, m.nelem, 4), dtype=torch.float64, device=cuda)
    net.predict(phys, u)
    y_gpu = (u.cpu().numpy() - uinf[:, None, :]) / scale.astype(np.float64)
    y_ref, _ = ref.forward(p.astype(np.float64), cond)
    assert np.linalg.norm(y_gpu - y_ref) <= 2e-3 * np.linalg.norm(y_ref)
    # gradients of the scaled mean squared error against target states
    rng = np.random.default_rng(3)
    tgt = uinf[:, None, :] + rng.normal(size=(2, m.nelem, 4)) * scale * 0.5
    loss, g = net.gradients(phys, torch.tensor(tgt, device=cuda))
    lref, gref = ref.gradients(p.astype(np.float64), cond, M.scaled_targets(tgt, uinf, scale))
    assert abs(loss - lref) <= 1e-3 * lref
    L, _ = M.layout(2)
    for name, (o, s) in L.items():
        n = int(np.prod(s))
        a, b = g[o:o + n], gref[o:o + n]
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b) + 1e-7, name


def test_gemm_paths_agree_over_many_tiles(cuda):
    """tcgen05 and mma.sync forward GEMMs on a batch large enough that every
    CTA of the persistent GEMMs runs several tiles through its ring of staged
    tiles (about 110k cell rows): the same outputs and gradients up to the
    FP32 summation order."""
    import torch
    m = cases.channel(192, 64)
    net = MPNN(m, layers=2, wall_markers=(1, 3), seed=4)
    _random_params(net, 9)
    net.set_scale(np.array([0.05, 0.1, 0.08, 0.3], np.float32))
    phys, dicts = _conds([0.35, 0.42, 0.5, 0.57, 0.63, 0.7], [-2.0, -1.0, 0.0, 1.0, 2.0, 3.0])
    _, uinf = M.conditions(dicts)
    assert len(phys) * m.nelem > 100000
    tgt = torch.tensor(uinf[:, None, :] + 0.02 * np.random.default_rng(1).normal(size=(len(phys), m.nelem, 4)),
                       device=cuda)
    out = {}
    for path in ("tcgen05", "mma_sync"):
        net.set_gemm_path(path)
        u = torch.zeros((len(phys), m.nelem, 4), dtype=torch.float64, device=cuda)
        net.predict(phys, u)
        out[path] = (u.cpu().numpy() - uinf[:, None, :],) + net.gradients(phys, tgt)
    (ya, la, ga), (yb, lb, gb) = out["tcgen05"], out["mma_sync"]
    assert np.linalg.norm(ya - yb) <= 1e-5 * np.linalg.norm(yb)
    assert abs(la - lb) <= 1e-5 * lb
    assert np.linalg.norm(ga - gb) <= 1e-4 * np.linalg.norm(gb)


def test_bounded_waits_report_an_error_and_leave_the_context_usable(cuda):
    """The bulk-copy GEMMs' mbarrier waits are bounded: with the test switch
    the first tile of every CTA is announced and never copied, every wait for
    it runs out, the call reports FV_ERR_CUDA, and the next call on the same
    network and context gives the same prediction as before."""
    import torch
    from fvens_gb300.mpnn import _bind
    m = cases.channel(24, 8)
    net = MPNN(m, layers=2, wall_markers=(1, 3), seed=5)
    _random_params(net, 7)
    net.set_scale(np.array([0.05, 0.1, 0.08, 0.3], np.float32))
    phys, _ = _conds([0.45, 0.55], [1.0, -2.0])
    u = [torch.zeros((2, m.nelem, 4), dtype=torch.float64, device=cuda) for _ in range(3)]
    net.predict(phys, u[0])
    fv.check(_bind().fv_mpnn_test_wait_limit(net._h, 1))
    with pytest.raises(fv.FvensError) as e:
        net.predict(phys, u[1])
    assert e.value.status == fv.FV_ERR_CUDA and "ran out of time" in str(e.value)
    fv.check(_bind().fv_mpnn_test_wait_limit(net._h, 0))
    net.predict(phys, u[2])
    assert torch.equal(u[2], u[0])


def test_gradients_batch_additive(cuda):
    """The gradient of a batch is the count-weighted sum of the members'."""
    import torch
    m = cases.channel(24, 8)
    net = MPNN(m, layers=2, seed=1)
    _random_params(net, 2)
    phys, dicts = _conds([0.4, 0.6])
    _, uinf = M.conditions(dicts)
    tgt = torch.tensor(uinf[:, None, :] + 0.01 * np.random.default_rng(0).normal(size=(2, m.nelem, 4)), device=cuda)
    l2, g2 = net.gradients(phys, tgt)
    la, ga = net.gradients(phys[:1], tgt[:1].contiguous())
    lb, gb = net.gradients(phys[1:], tgt[1:].contiguous())
    assert np.linalg.norm(g2 - 0.5 * (ga + gb)) <= 1e-4 * np.linalg.norm(g2)
    assert abs(l2 - 0.5 * (la + lb)) <= 1e-5 * l2


def test_adam_training_reduces_loss(cuda):
    import torch
    m = cases.channel(24, 8)
    net = MPNN(m, layers=2, wall_markers=(1, 3), seed=3)
    phys, dicts = _conds([0.35, 0.5, 0.62])
    _, uinf = M.conditions(dicts)
    # smooth synthetic targets: freestream plus a field varying with position and Mach
    g = m.geometry()
    x, y = g["cc"][:, 0], g["cc"][:, 1]
    t = np.stack([uinf[b] + np.outer(np.sin(2 * x) * np.cos(3 * y) * (dicts[b]["Minf"] - 0.3),
                                     [0.05, 0.1, 0.05, 0.2]) for b in range(3)])
    net.set_scale(output_scale(t, uinf))
    tgt = torch.tensor(t, device=cuda)
    l0 = net.gradients(phys, tgt)[0]
    for k in range(300):
        net.train_step(phys, tgt, 3e-3)
    l1 = net.gradients(phys, tgt)[0]
    assert l1 < 0.1 * l0, (l0, l1)


def test_warm_start_gains_over_freestream(cuda):
    """Trained on states the solver converged, the network's prediction for
    held-out conditions starts the solve closer to its converged state, and
    the solve from it converges to the same state in fewer steps."""
    import torch
    m = cases.channel(48, 16)
    num = fv.numerics_cfg(flux="ROE", gradient="LEASTSQUARES")
    cfg = dict(cfl_min=10, cfl_max=1000, tolerance=1e-10, abs_tolerance=1, max_timesteps=300, pc="ilu0",
               precision=4)
    train_m = list(np.linspace(0.3, 0.6, 12))
    test_m = [0.37, 0.48, 0.56]

    def solve(machs, u0=None):
        phys, _ = _conds(machs)
        d = fv.FlowFV(m, phys, num, cases.CHANNEL_BCS)
        if u0 is None:
            u0 = torch.tensor(np.repeat(d.freestream()[:, None, :], m.nelem, axis=1), device=cuda)
        u = u0.clone()
        S = fv.SteadyBackwardEulerSolver(d, **cfg)
        _, st = S.solve(u)
        assert all(s["status"] == 0 for s in st)
        return u, u0, [s["steps"] for s in st]

    u_train, _, _ = solve(train_m)
    phys_tr, dicts_tr = _conds(train_m)
    _, uinf_tr = M.conditions(dicts_tr)
    net = MPNN(m, layers=3, wall_markers=(1, 3), seed=11)
    net.set_scale(output_scale(u_train.cpu().numpy(), uinf_tr))
    train(net, phys_tr, u_train, epochs=150, batch=4, lr=3e-3, lr_final=3e-4, seed=0)

    u_free, u0_free, steps_free = solve(test_m)
    phys_te, _ = _conds(test_m)
    u_pred = torch.zeros_like(u0_free)
    net.predict(phys_te, u_pred)
    u_warm, _, steps_warm = solve(test_m, u_pred)
    ref = u_free.cpu().numpy()
    e_free = np.linalg.norm(u0_free.cpu().numpy() - ref)
    e_pred = np.linalg.norm(u_pred.cpu().numpy() - ref)
    assert e_pred < 0.5 * e_free, (e_pred, e_free)
    # same converged state (both at ||R|| < 1e-10)
    assert np.abs(u_warm.cpu().numpy() - ref).max() <= 1e-8 * np.abs(ref).max()
    assert sum(steps_warm) < sum(steps_free), (steps_warm, steps_free)


def test_warm_started_solve_falls_back_to_freestream(cuda):
    """A prediction the solver cannot converge from (an untrained network with
    a huge output scale) is judged and replaced: the member restarts from
    freestream with the starter and ends at the state of the method without
    the network."""
    import torch

    from fvens_gb300.mpnn import warm_started_solve
    m = cases.channel(24, 8)
    phys, _ = _conds([0.45, 0.55])
    num = fv.numerics_cfg(flux="ROE", gradient="LEASTSQUARES")
    main = fv.FlowFV(m, phys, num, cases.CHANNEL_BCS)
    start = fv.FlowFV(m, phys, fv.numerics_cfg(flux="ROE", gradient="NONE"), cases.CHANNEL_BCS)
    cfg = dict(cfl_min=10, cfl_max=1000, tolerance=1e-10, abs_tolerance=1, max_timesteps=300, pc="ilu0")
    S_main = fv.SteadyBackwardEulerSolver(main, **cfg)
    S_start = fv.SteadyBackwardEulerSolver(start, cfl_min=10, cfl_max=500, tolerance=1e-1, abs_tolerance=0,
                                           max_timesteps=20, pc="ilu0")
    net = MPNN(m, layers=2, seed=4)
    _random_params(net, 5, amp=1.0)
    net.set_scale(np.array([50.0, 50.0, 50.0, 50.0], np.float32))
    u = torch.zeros((2 * m.nelem, 4), dtype=torch.float64, device=cuda)
    stats, fell = warm_started_solve(net, phys, main, S_start, S_main, u)
    assert fell and all(st["status"] == 0 for st in stats)
    # the method without the network, from freestream
    u_ref = torch.tensor(np.repeat(main.freestream()[:, None, :], m.nelem, axis=1).reshape(-1, 4), device=cuda)
    S_start.solve(u_ref, raise_on_error=False)
    S_main.solve(u_ref)
    ug, ur = u.view(2, -1, 4).cpu().numpy(), u_ref.view(2, -1, 4).cpu().numpy()
    for k in fell:
        assert np.abs(ug[k] - ur[k]).max() <= 1e-8 * np.abs(ur[k]).max()
