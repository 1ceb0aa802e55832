"""ORACLE (test infrastructure only): numpy restatement of the warm-start
message-passing network of fvens_gb300/csrc/fv_mpnn.cu — forward pass,
mean-squared-error loss and the analytic backward pass.  The network has no
counterpart in the reference; this module is the CPU check of the GPU's
forward and backward kernels.

Arithmetic is float64.  With ``bf16=True`` every GEMM operand is rounded to
bfloat16 (round to nearest even) at the points where the GPU kernels stage
them in shared memory, so the two differ only by the GPU's FP32 accumulation
order and its FP32 intermediates.  The message MLP's first layer is applied
per cell (W_s h and W_d h, gathered per message), which is the same sum of
products; its backward pass goes through per-cell sums of the messages'
gradients, which are rounded to bfloat16 as GEMM operands.  With
``bf16=False`` the backward pass is checked against central finite
differences of the loss.

Parameter layout (flat float32 vector, as fv_mpnn_params):
    We [64][7], be [64], per layer l: Wm [64][131], bm [64], Wu [64][128], bu [64],
    Wd [4][64], bd [4].
"""
import numpy as np

W = 64


def bf16(x):
    """Rounds to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def layout(layers):
    """Offsets of the parameter blocks in the flat vector."""
    o, L = 0, {}

    def take(name, shape):
        nonlocal o
        L[name] = (o, shape)
        o += int(np.prod(shape))

    take("we", (W, 7))
    take("be", (W,))
    for l in range(layers):
        take(f"wm{l}", (W, 2 * W + 3))
        take(f"bm{l}", (W,))
        take(f"wu{l}", (W, 2 * W))
        take(f"bu{l}", (W,))
    take("wd", (4, W))
    take("bd", (4,))
    return L, o


def unpack(p, layers):
    L, n = layout(layers)
    assert p.size == n
    return {k: np.asarray(p[o:o + int(np.prod(s))], dtype=np.float64).reshape(s) for k, (o, s) in L.items()}


def pack(d, layers):
    L, n = layout(layers)
    p = np.zeros(n)
    for k, (o, s) in L.items():
        p[o:o + int(np.prod(s))] = d[k].ravel()
    return p


def conditions(phys):
    """Condition features of fv_mpnn (Minf, aoa, Reinf scaled) and the
    freestream conserved state per condition; phys: list of dicts with
    Minf, aoa_deg, Reinf, viscous, gamma."""
    cond, uinf = [], []
    for c in phys:
        g, M, a = c.get("gamma", 1.4), c["Minf"], np.deg2rad(c["aoa_deg"])
        cond.append([(M - 0.5) / 0.2, a * 180.0 / np.pi / 4.0,
                     np.log10(c["Reinf"]) - 4.0 if c.get("viscous", False) else -1.0])
        pinf = 1.0 / (g * M * M)
        uinf.append([1.0, np.cos(a), np.sin(a), pinf / (g - 1.0) + 0.5])
    return (np.asarray(cond, np.float32).astype(np.float64), np.asarray(uinf, np.float32).astype(np.float64))


class Net:
    """Forward/backward of the network on one graph.

    xs: nelem x 4 static cell features, faces: nf x 2 (L, R) interior faces,
    eattr: nf x 3 (nx, ny, log10 len) — as fv_mpnn_graph returns them."""

    def __init__(self, xs, faces, eattr, layers, bf16_operands=True):
        self.xs = np.asarray(xs, np.float64)
        f = np.asarray(faces, np.int64)
        e = np.asarray(eattr, np.float64)
        self.nc, self.nf, self.layers = self.xs.shape[0], f.shape[0], layers
        # message 2f: L -> R with the face normal, 2f+1: R -> L with its negative
        self.src = np.empty(2 * self.nf, np.int64)
        self.dst = np.empty(2 * self.nf, np.int64)
        self.src[0::2], self.dst[0::2] = f[:, 0], f[:, 1]
        self.src[1::2], self.dst[1::2] = f[:, 1], f[:, 0]
        self.ea = np.empty((2 * self.nf, 3))
        self.ea[0::2] = e
        self.ea[1::2] = e * np.array([-1.0, -1.0, 1.0])
        self.r = bf16 if bf16_operands else (lambda x: np.asarray(x, np.float64))

    def _scatter(self, v, idx):
        out = np.zeros((self.nc, v.shape[1]))
        np.add.at(out, idx, v)
        return out

    def forward(self, p, cond):
        """y (B x nelem x 4) and the saved activations."""
        P = unpack(p, self.layers)
        r = self.r
        ys, saves = [], []
        for b in range(cond.shape[0]):
            X = np.concatenate([self.xs, np.tile(cond[b], (self.nc, 1))], axis=1)
            Z0 = r(X) @ r(P["we"]).T + P["be"]
            h = np.maximum(Z0, 0.0)
            hs, zm, xm, zu, xu = [h], [], [], [], []
            for l in range(self.layers):
                Xm = np.concatenate([h[self.src], h[self.dst], self.ea], axis=1)
                Zm = r(Xm) @ r(P[f"wm{l}"]).T + P[f"bm{l}"]
                a = self._scatter(np.maximum(Zm, 0.0), self.dst)
                Xu = np.concatenate([h, a], axis=1)
                Zu = r(Xu) @ r(P[f"wu{l}"]).T + P[f"bu{l}"]
                h = h + np.maximum(Zu, 0.0)
                hs.append(h); zm.append(Zm); xm.append(Xm); zu.append(Zu); xu.append(Xu)
            y = r(h) @ r(P["wd"]).T + P["bd"]
            ys.append(y)
            saves.append(dict(X=X, Z0=Z0, hs=hs, zm=zm, xm=xm, zu=zu, xu=xu))
        return np.stack(ys), saves

    def loss(self, p, cond, t):
        """Mean squared error of y against the scaled targets t (B x nelem x 4)."""
        y, _ = self.forward(p, cond)
        return float(np.mean((y - t) ** 2))

    def gradients(self, p, cond, t):
        """(loss, gradient as a flat vector in the parameter layout)."""
        P = unpack(p, self.layers)
        r = self.r
        y, saves = self.forward(p, cond)
        n = y.size
        G = {k: np.zeros_like(v) for k, v in P.items()}
        for b, S in enumerate(saves):
            dy = 2.0 * (y[b] - t[b]) / n
            hL = S["hs"][-1]
            G["wd"] += r(dy).T @ r(hL)
            G["bd"] += dy.sum(0)
            dh = r(dy) @ r(P["wd"])
            for l in reversed(range(self.layers)):
                dZu = dh * (S["zu"][l] > 0)
                G[f"wu{l}"] += r(dZu).T @ r(S["xu"][l])
                G[f"bu{l}"] += dZu.sum(0)
                dXu = r(dZu) @ r(P[f"wu{l}"])
                da = dXu[:, W:]
                dh = dh + dXu[:, :W]
                # the message MLP's first layer is linear in h_src and h_dst, so its
                # gradients go through per-cell sums of dZm over outgoing (S_out) and
                # incoming (S_in) messages; these sums are the BF16-rounded operands
                dZm = da[self.dst] * (S["zm"][l] > 0)
                s_out = self._scatter(dZm, self.src)
                s_in = self._scatter(dZm, self.dst)
                h_l = S["hs"][l]
                Wm = P[f"wm{l}"]
                G[f"wm{l}"][:, :W] += r(s_out).T @ r(h_l)
                G[f"wm{l}"][:, W:2 * W] += r(s_in).T @ r(h_l)
                G[f"wm{l}"][:, 2 * W:] += dZm.T @ r(self.ea)
                G[f"bm{l}"] += dZm.sum(0)
                dh = dh + r(s_out) @ r(Wm[:, :W]) + r(s_in) @ r(Wm[:, W:2 * W])
            dZ0 = dh * (S["Z0"] > 0)
            G["we"] += r(dZ0).T @ r(S["X"])
            G["be"] += dZ0.sum(0)
        return float(np.mean((y - t) ** 2)), pack(G, self.layers)


def scaled_targets(u, uinf, scale):
    """t = (u - uinf) / scale per variable; u: B x nelem x 4 conserved states."""
    return (np.asarray(u, np.float64) - uinf[:, None, :]) / np.asarray(scale, np.float32).astype(np.float64)
