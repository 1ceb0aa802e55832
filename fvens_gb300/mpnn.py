"""Learned warm start: the mesh message-passing network of fv_mpnn.cu behind
its C ABI (fv_mpnn_*), and the helpers that train it on states the steady
solver converged and start solves from its predictions.

The network has no counterpart in the reference: it replaces the freestream
initial state (SteadyFlowCase::initializeSystemVector, casesolvers.cpp:52-69)
and the first-order starter solve (execute_starter, casesolvers.cpp:225-314)
of a steady case; the unchanged implicit solver then converges from the
prediction to the same tolerance and judges the result.
"""
import ctypes

import numpy as np

from . import _vp, check, dptr, fv_physics_cfg, lib

_F = ctypes.POINTER(ctypes.c_float)


def _bind():
    L = lib()
    if getattr(L, "_mpnn_bound", False):
        return L
    vp = ctypes.c_void_p
    L.fv_mpnn_create.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_ulonglong,
                                 ctypes.POINTER(vp)]
    L.fv_mpnn_destroy.argtypes = [vp]
    L.fv_mpnn_destroy.restype = None
    L.fv_mpnn_set_scale.argtypes = [vp, _F]
    L.fv_mpnn_set_gemm_path.argtypes = [vp, ctypes.c_int]
    L.fv_mpnn_test_wait_limit.argtypes = [vp, ctypes.c_int]
    L.fv_mpnn_params.argtypes = [vp, _F, _F, ctypes.POINTER(ctypes.c_longlong)]
    L.fv_mpnn_graph.argtypes = [vp, _F, ctypes.POINTER(ctypes.c_int), _F]
    L.fv_mpnn_predict.argtypes = [vp, ctypes.POINTER(fv_physics_cfg), ctypes.c_int, vp]
    L.fv_mpnn_gradients.argtypes = [vp, ctypes.POINTER(fv_physics_cfg), ctypes.c_int, vp, _F, _F]
    L.fv_mpnn_train_step.argtypes = [vp, ctypes.POINTER(fv_physics_cfg), ctypes.c_int, vp, ctypes.c_float, _F]
    L._mpnn_bound = True
    return L


def _fp(a):
    return a.ctypes.data_as(_F)


class MPNN:
    """Warm-start network on one mesh: width 64, `layers` message-passing
    layers; BF16 tensor-core GEMMs with FP32 accumulation; FP32 parameters
    and Adam state on the GPU."""

    def __init__(self, mesh, layers=4, wall_markers=(), seed=0):
        L = _bind()
        self.mesh, self.layers, self.wall_markers = mesh, layers, tuple(wall_markers)
        wm = (ctypes.c_int * max(len(wall_markers), 1))(*wall_markers)
        h = ctypes.c_void_p()
        check(L.fv_mpnn_create(mesh._h, layers, wm, len(wall_markers), seed, ctypes.byref(h)))
        self._h = h
        n = ctypes.c_longlong()
        check(L.fv_mpnn_params(self._h, None, None, ctypes.byref(n)))
        self.nparams = n.value
        self.scale = np.ones(4, np.float32)

    def set_scale(self, scale):
        """Per-variable scale of the output: u = uinf + scale * y."""
        self.scale = np.ascontiguousarray(scale, dtype=np.float32)
        check(_bind().fv_mpnn_set_scale(self._h, _fp(self.scale)))

    def set_gemm_path(self, path):
        """Tensor-core path of the forward cell GEMMs: "tcgen05"
        (tensor-memory accumulators) or "mma_sync" (warp-level; the default,
        faster for these row-bound GEMMs)."""
        check(_bind().fv_mpnn_set_gemm_path(self._h, {"tcgen05": 0, "mma_sync": 1}[path]))

    def params(self, new=None):
        """The flat FP32 parameter vector (after loading `new` when given)."""
        out = np.zeros(self.nparams, np.float32)
        src = None if new is None else np.ascontiguousarray(new, dtype=np.float32)
        check(_bind().fv_mpnn_params(self._h, _fp(out), None if src is None else _fp(src), None))
        return out

    def graph(self):
        """(cell features nelem x 4, interior faces nf x 2, face features nf x 3)."""
        nf = self.mesh.naface - self.mesh.nbface
        xs = np.zeros((self.mesh.nelem, 4), np.float32)
        faces = np.zeros((nf, 2), np.int32)
        ea = np.zeros((nf, 3), np.float32)
        check(_bind().fv_mpnn_graph(self._h, _fp(xs), faces.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _fp(ea)))
        return xs, faces, ea

    @staticmethod
    def _phys(phys):
        phys = list(phys) if isinstance(phys, (list, tuple)) else [phys]
        return (fv_physics_cfg * len(phys))(*phys), len(phys)

    def predict(self, phys, u):
        """Predicted states of the conditions `phys` into the device array u
        (batch x nelem x 4 doubles)."""
        arr, b = self._phys(phys)
        check(_bind().fv_mpnn_predict(self._h, arr, b, _vp(dptr(u))))

    def gradients(self, phys, target):
        """(loss, gradient) of the mean squared scaled error against the device
        array of target states, without an update."""
        arr, b = self._phys(phys)
        g = np.zeros(self.nparams, np.float32)
        loss = ctypes.c_float()
        check(_bind().fv_mpnn_gradients(self._h, arr, b, _vp(dptr(target)), _fp(g), ctypes.byref(loss)))
        return float(loss.value), g

    def train_step(self, phys, target, lr):
        """One Adam step; returns the loss before the step."""
        arr, b = self._phys(phys)
        loss = ctypes.c_float()
        check(_bind().fv_mpnn_train_step(self._h, arr, b, _vp(dptr(target)), float(lr), ctypes.byref(loss)))
        return float(loss.value)

    def save(self, path):
        """Writes the trained network (parameters, output scale, layers, wall
        markers and the mesh's cell count) to an .npz file."""
        np.savez(path, params=self.params(), scale=self.scale, layers=self.layers,
                 wall_markers=np.asarray(self.wall_markers, np.int32), nelem=self.mesh.nelem)

    @classmethod
    def load(cls, mesh, path):
        """A network written by save(), on the same mesh."""
        z = np.load(path)
        if int(z["nelem"]) != mesh.nelem:
            raise ValueError(f"network was trained on a mesh of {int(z['nelem'])} cells, not {mesh.nelem}")
        net = cls(mesh, layers=int(z["layers"]), wall_markers=tuple(int(x) for x in z["wall_markers"]))
        net.params(z["params"])
        net.set_scale(z["scale"])
        return net

    def __del__(self):
        if getattr(self, "_h", None) is not None:
            try:
                _bind().fv_mpnn_destroy(self._h)
            except Exception:
                pass
            self._h = None


def output_scale(states, uinf):
    """Per-variable scale for the network output: the root-mean-square
    deviation of converged states from their freestream (states: B x nelem x 4,
    uinf: B x 4), floored so that no variable is divided by ~0."""
    d = np.asarray(states, np.float64) - np.asarray(uinf, np.float64)[:, None, :]
    s = np.sqrt(np.mean(d ** 2, axis=(0, 1)))
    return np.maximum(s, 1e-3 * max(s.max(), 1e-12)).astype(np.float32)


def train(net, phys, states, epochs, batch, lr, seed=0, lr_final=None, log=None):
    """Adam on (condition, converged state) pairs.  states: device array
    n x nelem x 4 (torch, float64).  The learning rate decays geometrically
    to lr_final over the run.  Returns the per-epoch mean losses."""
    import torch
    n = len(phys)
    rng = np.random.default_rng(seed)
    steps = epochs * ((n + batch - 1) // batch)
    decay = (lr_final / lr) ** (1.0 / max(steps - 1, 1)) if lr_final else 1.0
    losses, k = [], 0
    for ep in range(epochs):
        perm = rng.permutation(n)
        tot, cnt = 0.0, 0
        for s in range(0, n, batch):
            idx = perm[s:s + batch]
            tgt = states[torch.as_tensor(idx, device=states.device)].contiguous()
            tot += net.train_step([phys[i] for i in idx], tgt, lr * decay ** k) * len(idx)
            cnt += len(idx)
            k += 1
        losses.append(tot / cnt)
        if log:
            log(ep, losses[-1])
    return losses


def diverged(st):
    """A judge for fallback_solve: the solve from the prediction failed
    numerically (non-finite residual) or ended no lower than it started.  A
    member that made progress but stalled or reached the step limit keeps its
    result: a stall is a property of the condition (an unsteady or slowly
    converging flow), which a freestream start meets as well."""
    return st["status"] == 3 or (st["status"] != 0 and not st["res"] < st["res0"])


def fallback_solve(main, start_solver, main_solver, u, stats, judge=None):
    """The fallback of a warm-started batch: members whose solve from the
    prediction is rejected -- judge(stats[k]) true; by default every member
    that did not converge -- restart from freestream with the starter and the
    main solve (the method without the network); the others keep their
    states.  Updates stats in place; returns the members that fell back."""
    import torch
    judge = judge or (lambda st: st["status"] != 0)
    failed = [k for k, st in enumerate(stats) if judge(st)]
    if failed:
        mask = np.zeros(len(stats), np.int32)
        mask[failed] = 1
        uv = u.view(len(stats), -1, 4)
        free = torch.tensor(main.freestream(), device=u.device, dtype=u.dtype)
        for k in failed:
            uv[k] = free[k]
        start_solver.solve(u, member_mask=mask, raise_on_error=False)
        _, again = main_solver.solve(u, member_mask=mask, raise_on_error=False)
        for k in failed:
            stats[k] = dict(again[k], fallback=True)
    return failed


def warm_started_solve(net, phys, main, start_solver, main_solver, u, judge=None):
    """Solves the conditions `phys` from the network's prediction and judges
    the result: the main solve runs from the prediction, and members whose
    solve is rejected (judge; by default every member that did not converge)
    fall back to freestream with the starter (fallback_solve).  u: device
    array of the batch (filled here).  Returns (stats per member, members that
    fell back)."""
    net.predict(phys, u)
    _, stats = main_solver.solve(u, raise_on_error=False)
    return stats, fallback_solve(main, start_solver, main_solver, u, stats, judge)
