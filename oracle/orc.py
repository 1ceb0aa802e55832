"""ORACLE (test infrastructure only): ctypes binding of oracle/build/liborc.so,
the CPU FP64 restatement of the reference's hot path, and of the reference's
own compiled pointwise physics in oracle/_ref (present only where the
reference sources were available at build time).

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs use this module; the product never does.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(_HERE, "build", "liborc.so")
REF_LIB = os.path.join(_HERE, "_ref", "libfvens_ref.so")

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_orc = None
_ref = None


def p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


def lib():
    global _orc
    if _orc is None:
        if not os.path.exists(ORACLE_LIB):
            raise RuntimeError("oracle not built: run `python -m fvens_gb300.build`")
        L = ctypes.CDLL(ORACLE_LIB)
        for fn in ("orc_mesh_create", "orc_disc_create"):
            getattr(L, fn).restype = ctypes.c_void_p
        L.orc_entropy_error.restype = ctypes.c_double
        for fn in ("orc_mesh_destroy", "orc_disc_destroy", "orc_set_threads", "orc_mesh_counts",
                   "orc_mesh_arrays", "orc_freestream", "orc_geometry"):
            getattr(L, fn).restype = None
        _orc = L
    return _orc


def ref_lib():
    """The reference's compiled pointwise physics, or None when absent."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        L = ctypes.CDLL(REF_LIB)
        L.ref_delta_pressure.restype = ctypes.c_double
        L.ref_viscosity.restype = ctypes.c_double
        _ref = L
    return _ref


def reference_root():
    """Root of the reference project's sources, for tests and fixture scripts
    that read its own inputs: $FVENS_REFERENCE, else the root recorded by
    oracle/ref/build_ref.sh when it found the sources; None when neither names
    an existing directory."""
    cand = os.environ.get("FVENS_REFERENCE")
    if not cand:
        rec = os.path.join(_HERE, "_ref", "reference_root.txt")
        if os.path.exists(rec):
            cand = open(rec).read().strip()
    return cand if cand and os.path.isdir(cand) else None


def set_threads(n):
    lib().orc_set_threads(int(n))


def max_threads():
    return int(lib().orc_max_threads())


class Mesh:
    def __init__(self, coords, nnode, inpoel, bface, btag):
        coords = np.ascontiguousarray(coords, np.float64)
        nnode = np.ascontiguousarray(nnode, np.int32)
        inpoel = np.ascontiguousarray(inpoel, np.int32)
        bface = np.ascontiguousarray(bface, np.int32)
        btag = np.ascontiguousarray(btag, np.int32)
        L = lib()
        h = L.orc_mesh_create(len(coords), p(coords), len(nnode), p(nnode, ctypes.c_int), p(inpoel, ctypes.c_int),
                              len(btag), p(bface, ctypes.c_int), p(btag, ctypes.c_int))
        if not h:
            raise RuntimeError("oracle mesh construction failed")
        self._h = ctypes.c_void_p(h)
        c = np.zeros(4, np.int32)
        L.orc_mesh_counts(self._h, p(c, ctypes.c_int))
        self.nelem, self.nbface, self.ninface, self.naface = (int(x) for x in c)

    @classmethod
    def from_export(cls, ex):
        return cls(ex["coords"], ex["nnode"], ex["inpoel"], ex["bface"], ex["btag"])

    def arrays(self):
        intfac = np.zeros((self.naface, 4), np.int32)
        esuel = np.zeros((self.nelem, 4), np.int32)
        area = np.zeros(self.nelem)
        fm = np.zeros((self.naface, 3))
        lib().orc_mesh_arrays(self._h, p(intfac, ctypes.c_int), p(esuel, ctypes.c_int), p(area), p(fm))
        return dict(intfac=intfac, esuel=esuel, area=area, facemetric=fm)

    def __del__(self):
        if getattr(self, "_h", None) is not None and _orc is not None:
            _orc.orc_mesh_destroy(self._h)
            self._h = None


FLUX = {"LLF": 0, "VANLEER": 1, "AUSM": 2, "AUSMPLUS": 3, "ROE": 4, "HLL": 5, "HLLC": 6}
GRADIENT = {"NONE": 0, "GREENGAUSS": 1, "LEASTSQUARES": 2}
RECON = {"NONE": 0, "VANALBADA": 1, "BARTHJESPERSEN": 2, "VENKATAKRISHNAN": 3, "WENO": 4}
BCT = {"slipwall": 0, "farfield": 1, "inflowoutflow": 2, "subsonic_inflow": 3, "extrapolation": 4,
       "isothermalwall": 6, "adiabaticwall": 7}


class Disc:
    """Oracle spatial discretisation (one flow condition)."""

    def __init__(self, mesh, gamma=1.4, Minf=0.5, Tinf=288.15, Reinf=float("inf"), Pr=0.72, aoa_deg=0.0,
                 viscous=False, const_visc=False, flux="ROE", flux_jac=None, gradient="LEASTSQUARES",
                 reconstruction="NONE", limiter_param=0.0, bcs=()):
        self.mesh = mesh
        phys = np.array([gamma, Minf, Tinf, Reinf, Pr, np.deg2rad(aoa_deg)])
        order2 = gradient != "NONE"
        flags = np.array([int(viscous), int(const_visc), int(order2)], np.int32)
        fj = flux if flux_jac in (None, "CONSISTENT") else flux_jac
        sch = np.array([FLUX[flux], FLUX[fj], GRADIENT[gradient], RECON[reconstruction]], np.int32)
        bt = np.array([[t, BCT[k] if isinstance(k, str) else k] for (t, k, v) in bcs], np.int32).reshape(-1, 2)
        bv = np.array([(list(v) + [0, 0])[:2] for (t, k, v) in bcs], np.float64).reshape(-1, 2)
        h = lib().orc_disc_create(mesh._h, p(phys), p(flags, ctypes.c_int), p(sch, ctypes.c_int),
                                  ctypes.c_double(limiter_param), len(bt), p(bt, ctypes.c_int), p(bv))
        if not h:
            raise RuntimeError("oracle discretisation setup failed")
        self._h = ctypes.c_void_p(h)
        self.nelem = mesh.nelem

    def freestream(self):
        u = np.zeros(4)
        lib().orc_freestream(self._h, p(u))
        return u

    def geometry(self):
        m = self.mesh
        rc = np.zeros((m.nelem, 2))
        rcbp = np.zeros((m.nbface, 2))
        gr = np.zeros((m.naface, 2))
        lib().orc_geometry(self._h, p(rc), p(rcbp), p(gr))
        return rc, rcbp, gr

    def residual(self, u, gettimesteps=True):
        u = np.ascontiguousarray(u, np.float64)
        r = np.zeros_like(u)
        dt = np.zeros(self.nelem) if gettimesteps else None
        lib().orc_residual(self._h, p(u), p(r), p(dt) if dt is not None else None)
        return r, dt

    def internals(self, u):
        m = self.mesh
        u = np.ascontiguousarray(u, np.float64)
        grad = np.zeros((m.nelem, 8))
        ul = np.zeros((m.naface, 4))
        ur = np.zeros((m.naface, 4))
        lib().orc_residual_internals(self._h, p(u), p(grad), p(ul), p(ur))
        return grad, ul, ur

    def flux_scale(self, u):
        u = np.ascontiguousarray(u, np.float64)
        s = np.zeros(self.nelem)
        lib().orc_flux_scale(self._h, p(u), p(s))
        return s

    def conserved_gradients(self, u):
        u = np.ascontiguousarray(u, np.float64)
        g = np.zeros((self.nelem, 8))
        lib().orc_conserved_gradients(self._h, p(u), p(g))
        return g

    def jacobian(self, u):
        u = np.ascontiguousarray(u, np.float64)
        nnzb = ctypes.c_int()
        L = lib()
        L.orc_jacobian(self._h, p(u), ctypes.byref(nnzb), None, None, None)
        rowptr = np.zeros(self.nelem + 1, np.int32)
        col = np.zeros(nnzb.value, np.int32)
        val = np.zeros((nnzb.value, 16))
        rc = L.orc_jacobian(self._h, p(u), ctypes.byref(nnzb), p(rowptr, ctypes.c_int), p(col, ctypes.c_int), p(val))
        if rc:
            raise RuntimeError(f"oracle jacobian failed ({rc})")
        return rowptr, col, val

    def steady_solve(self, u, cflmin=10, cflmax=1000, tol=1e-10, maxiter=1000, abs_tol=True, pc="ilu0",
                     restart=30, lin_maxit=30, lin_rtol=0.1, matrix_free=False, mf_eps=1e-7, nl_update="full",
                     min_relax=0.2, order=None):
        u = np.array(u, np.float64, copy=True)
        cd = np.array([cflmin, cflmax, tol, lin_rtol, mf_eps, min_relax])
        ci = np.array([maxiter, int(abs_tol), {"none": 0, "jacobi": 1, "sgs": 2, "ilu0": 3}[pc], restart, lin_maxit,
                       int(matrix_free), {"full": 0, "robust_flow": 1, "bounded": 2}[nl_update]], np.int32)
        st = np.zeros(6)
        hist = np.zeros((maxiter, 3))
        o = None if order is None else np.ascontiguousarray(order, np.int32)
        status = lib().orc_steady_solve(self._h, p(cd), p(ci, ctypes.c_int), p(o, ctypes.c_int) if o is not None else None,
                                        p(u), p(st), p(hist))
        steps = int(st[0])
        return u, dict(status=int(status), steps=steps, lin_iters=int(st[1]), res0=st[3], res=st[4], cfl=st[5],
                       history=hist[:steps])

    def steady_fe(self, u, cflinit, tol=1e-10, maxiter=1000, abs_tol=True):
        """SteadyForwardEulerSolver::solve restated: (u, dict(steps, status, res0, res, history))."""
        u = np.array(u, np.float64, copy=True)
        st = np.zeros(4)
        hist = np.zeros(max(maxiter, 1))
        lib().orc_steady_fe(self._h, p(np.array([cflinit, tol])), p(np.array([maxiter, int(abs_tol)], np.int32),
                                                                     ctypes.c_int), p(u), p(st), p(hist))
        steps = int(st[0])
        return u, dict(steps=steps, status=int(st[1]), res0=st[2], res=st[3], history=hist[:steps])

    def tvdrk(self, u, order, cfl, final_time):
        """TVDRKSolver::solve restated: (u, steps, status, time)."""
        u = np.array(u, np.float64, copy=True)
        out = np.zeros(3)
        lib().orc_tvdrk(self._h, int(order), ctypes.c_double(cfl), ctypes.c_double(final_time), p(u), p(out))
        return u, int(out[0]), int(out[1]), out[2]

    def surface_data(self, u, marker):
        out = np.zeros(3)
        lib().orc_surface_data(self._h, p(np.ascontiguousarray(u, np.float64)), int(marker), p(out), None)
        return out

    def surface_distribution(self, u, marker):
        """Per-face rows (x, y, Cp, Cf) of the marker's faces."""
        u = np.ascontiguousarray(u, np.float64)
        out = np.zeros(3)
        n = lib().orc_surface_data(self._h, p(u), int(marker), p(out), None)
        rows = np.zeros((n, 4))
        lib().orc_surface_data(self._h, p(u), int(marker), p(out), p(rows))
        return rows

    def entropy_error(self, u):
        return lib().orc_entropy_error(self._h, p(np.ascontiguousarray(u, np.float64)))

    def time_kernels(self, u, pc="ilu0", reps=5):
        """Median seconds per call of the residual (with local time steps), the
        Jacobian assembly, the preconditioner setup and one preconditioner
        apply (natural order) at state u, over `reps` calls after one untimed."""
        out = np.zeros(4)
        rc = lib().orc_time_kernels(self._h, p(np.ascontiguousarray(u, np.float64)),
                                    {"none": 0, "jacobi": 1, "sgs": 2, "ilu0": 3}[pc], int(reps), p(out))
        if rc:
            raise RuntimeError(f"oracle kernel timing failed ({rc})")
        return dict(zip(("residual", "jacobian", "pc_setup", "pc_apply"), out.tolist()))

    def __del__(self):
        if getattr(self, "_h", None) is not None and _orc is not None:
            _orc.orc_disc_destroy(self._h)
            self._h = None


def precond_apply(rowptr, col, val, pctype, r, order=None):
    n = len(rowptr) - 1
    z = np.zeros_like(r)
    o = None if order is None else np.ascontiguousarray(order, np.int32)
    rc = lib().orc_precond_apply(n, p(rowptr, ctypes.c_int), p(col, ctypes.c_int), p(np.ascontiguousarray(val)),
                                 {"none": 0, "jacobi": 1, "sgs": 2, "ilu0": 3}[pctype],
                                 p(o, ctypes.c_int) if o is not None else None, p(np.ascontiguousarray(r)), p(z))
    if rc:
        raise RuntimeError(f"oracle preconditioner failed ({rc})")
    return z


def fgmres(rowptr, col, val, pctype, b, restart=30, maxit=30, rtol=0.1, order=None):
    n = len(rowptr) - 1
    x = np.zeros_like(b)
    rn = ctypes.c_double()
    o = None if order is None else np.ascontiguousarray(order, np.int32)
    its = lib().orc_fgmres(n, p(rowptr, ctypes.c_int), p(col, ctypes.c_int), p(np.ascontiguousarray(val)),
                           {"none": 0, "jacobi": 1, "sgs": 2, "ilu0": 3}[pctype],
                           p(o, ctypes.c_int) if o is not None else None, p(np.ascontiguousarray(b)), p(x),
                           restart, maxit, ctypes.c_double(rtol), ctypes.byref(rn))
    return x, its, rn.value
