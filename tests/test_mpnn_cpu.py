"""The warm-start network's CPU oracle (oracle/mpnn_ref.py): bfloat16
rounding, and its analytic backward pass against central finite differences
of the loss in float64."""
import numpy as np

from oracle import mpnn_ref as M


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 1.0 + 2.0 ** -7, 3.0e-3, 0.0])
    r = M.bf16(x)
    # ties to even: 1 + 2^-8 -> 1, 1 + 3*2^-8 -> 1 + 2^-6; representable values stay
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2.0 ** -6
    assert r[3] == -2.5 and r[4] == 1.0 + 2.0 ** -7 and r[6] == 0.0
    assert abs(r[5] - 3.0e-3) <= 3.0e-3 * 2.0 ** -8


def _graph(seed=0, nc=14, nf=22):
    rng = np.random.default_rng(seed)
    pairs = set()
    while len(pairs) < nf:
        a, b = rng.integers(0, nc, 2)
        if a != b and (b, a) not in pairs:
            pairs.add((int(a), int(b)))
    faces = np.array(sorted(pairs))
    xs = rng.normal(size=(nc, 4)) * 0.5
    ang = rng.uniform(0, 2 * np.pi, nf)
    ea = np.stack([np.cos(ang), np.sin(ang), rng.normal(size=nf) * 0.3], axis=1)
    return xs, faces, ea


def test_oracle_gradient_matches_finite_differences():
    layers = 2
    xs, faces, ea = _graph()
    net = M.Net(xs, faces, ea, layers, bf16_operands=False)
    rng = np.random.default_rng(1)
    _, n = M.layout(layers)
    p = rng.normal(size=n) * 0.2
    cond = rng.normal(size=(2, 3))
    t = rng.normal(size=(2, xs.shape[0], 4))
    loss, g = net.gradients(p, cond, t)
    assert abs(loss - net.loss(p, cond, t)) <= 1e-14 * loss
    # every parameter block, a few entries each
    L, _ = M.layout(layers)
    idx = []
    for o, s in L.values():
        idx += list(o + rng.choice(int(np.prod(s)), size=min(4, int(np.prod(s))), replace=False))
    eps = 1e-6
    fd = []
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd.append((net.loss(pp, cond, t) - net.loss(pm, cond, t)) / (2 * eps))
    fd = np.array(fd)
    err = np.abs(fd - g[idx])
    assert err.max() <= 1e-6 * max(np.abs(g).max(), 1e-12), (err.max(), np.abs(g).max())


def test_message_directions_and_aggregation():
    # two cells, one face: each cell receives exactly the other's message
    xs = np.array([[0.1, 0.2, 0.3, 0.4], [-0.3, 0.0, 0.2, 0.1]])
    net = M.Net(xs, np.array([[0, 1]]), np.array([[1.0, 0.0, 0.0]]), 1, bf16_operands=False)
    assert list(net.src) == [0, 1] and list(net.dst) == [1, 0]
    assert np.allclose(net.ea, [[1, 0, 0], [-1, 0, 0]])


def test_fallback_judge():
    """The warm start's fallback restarts a member from freestream when its
    solve from the prediction diverged or ended no lower than it started; a
    member that converged, or made progress and then stalled or reached the
    step limit, keeps its result."""
    from fvens_gb300.mpnn import diverged
    assert diverged(dict(status=3, res=float("nan"), res0=1.0))
    assert diverged(dict(status=4, res=2.0, res0=1.0))
    assert diverged(dict(status=4, res=float("nan"), res0=1.0))
    assert not diverged(dict(status=4, res=1e-6, res0=1.0))
    assert not diverged(dict(status=0, res=1e-11, res0=1.0))
