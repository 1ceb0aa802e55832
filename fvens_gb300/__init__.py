"""Python binding of the fvens_gb300 C ABI (include/fvens_gb300.h).

A thin ctypes layer over the CUDA library built by ``fvens_gb300.build``.
Class and method names mirror the reference's host interfaces
(UMesh, FlowFV::compute_residual / assemble_jacobian / getGradients,
SteadyBackwardEulerSolver::solve) so call sites keep their shape.
Device arrays are passed as CUDA tensors (torch) or raw integer addresses;
there is no CPU path: if the CUDA library is missing, loading fails.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libfvens_gb300.so")

FV_OK, FV_ERR_INVALID, FV_ERR_CUDA, FV_ERR_NUMERICAL, FV_ERR_TOLERANCE, FV_ERR_UNSUPPORTED, FV_ERR_MESH = range(7)
FLUX = {"LLF": 0, "VANLEER": 1, "AUSM": 2, "AUSMPLUS": 3, "ROE": 4, "HLL": 5, "HLLC": 6}
GRADIENT = {"NONE": 0, "GREENGAUSS": 1, "LEASTSQUARES": 2}
RECONSTRUCTION = {"NONE": 0, "VANALBADA": 1, "BARTHJESPERSEN": 2, "VENKATAKRISHNAN": 3, "WENO": 4}
BC = {"slipwall": 0, "farfield": 1, "inflowoutflow": 2, "subsonic_inflow": 3, "extrapolation": 4,
      "periodic": 5, "isothermalwall": 6, "adiabaticwall": 7}
PC = {"none": 0, "jacobi": 1, "sgs": 2, "ilu0": 3}
MESH_CHANNEL_BUMP, MESH_NACA_OGRID, MESH_NACA_HYBRID = 1, 2, 3

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class FvensError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"fvens_gb300 status {status}: {message}")
        self.status = status


class fv_mesh_desc(ctypes.Structure):
    _fields_ = [("npoin", ctypes.c_int), ("nelem", ctypes.c_int), ("nbface", ctypes.c_int),
                ("coords", _c_dbl_p), ("nnode", _c_int_p), ("inpoel", _c_int_p),
                ("bface", _c_int_p), ("btag", _c_int_p)]


class fv_physics_cfg(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_double), ("Minf", ctypes.c_double), ("Tinf", ctypes.c_double),
                ("Reinf", ctypes.c_double), ("Pr", ctypes.c_double), ("aoa", ctypes.c_double),
                ("viscous_sim", ctypes.c_int), ("const_visc", ctypes.c_int)]


class fv_numerics_cfg(ctypes.Structure):
    _fields_ = [("conv_numflux", ctypes.c_int), ("conv_numflux_jac", ctypes.c_int),
                ("gradientscheme", ctypes.c_int), ("reconstruction", ctypes.c_int),
                ("limiter_param", ctypes.c_double), ("order2", ctypes.c_int)]


class fv_bc_cfg(ctypes.Structure):
    _fields_ = [("bc_tag", ctypes.c_int), ("bc_type", ctypes.c_int), ("bc_vals", ctypes.c_double * 2)]


_lib = None
ABI_VERSION = 3  # FVENS_GB300_ABI_VERSION of include/fvens_gb300.h


def lib():
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"fvens_gb300 CUDA library not found at {LIB_PATH}; "
                               "run `python -m fvens_gb300.build` (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        L.fv_status_string.restype = ctypes.c_char_p
        L.fv_last_error.restype = ctypes.c_char_p
        L.fv_kernel_launch_count.restype = ctypes.c_longlong
        L.fv_mesh_destroy.restype = None
        L.fv_disc_destroy.restype = None
        L.fv_matrix_destroy.restype = None
        L.fv_precond_destroy.restype = None
        L.fv_solver_destroy.restype = None
        L.fv_solver_cfg_default.restype = None
        ver = L.fv_abi_version() if hasattr(L, "fv_abi_version") else 1
        if ver != ABI_VERSION:
            raise RuntimeError(f"{LIB_PATH} has ABI version {ver}, this binding expects "
                               f"{ABI_VERSION}; rebuild with `python -m fvens_gb300.build`")
        _lib = L
    return _lib


def check(status):
    if status != FV_OK:
        L = lib()
        raise FvensError(status, L.fv_last_error().decode() or L.fv_status_string(status).decode())


def dptr(x):
    """Device address of a CUDA tensor (or a raw integer address)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise ValueError("expected a CUDA tensor")
        if not x.is_contiguous():
            raise ValueError("expected a contiguous tensor")
        return x.data_ptr()
    raise TypeError(f"cannot take a device address of {type(x)}")


def _hp(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


class UMesh:
    """Unstructured 2-D mesh (reference UMesh + preprocessMesh)."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle) if isinstance(handle, int) else handle
        c = (ctypes.c_int * 6)()
        check(lib().fv_mesh_counts(self._h, c))
        self.nelem, self.nbface, self.ninface, self.naface, self.npoin, self.ncolors = list(c)

    @classmethod
    def from_arrays(cls, coords, nnode, inpoel, bface, btag, reorder=0):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        nnode = np.ascontiguousarray(nnode, dtype=np.int32)
        inpoel = np.ascontiguousarray(inpoel, dtype=np.int32)
        bface = np.ascontiguousarray(bface, dtype=np.int32)
        btag = np.ascontiguousarray(btag, dtype=np.int32)
        d = fv_mesh_desc(coords.shape[0], nnode.shape[0], btag.shape[0], _hp(coords, ctypes.c_double),
                         _hp(nnode, ctypes.c_int), _hp(inpoel, ctypes.c_int), _hp(bface, ctypes.c_int),
                         _hp(btag, ctypes.c_int))
        h = ctypes.c_void_p()
        check(lib().fv_mesh_create(ctypes.byref(d), int(reorder), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def generate(cls, kind, params, reorder=1):
        p = np.ascontiguousarray(params, dtype=np.float64)
        h = ctypes.c_void_p()
        check(lib().fv_mesh_generate(int(kind), _hp(p, ctypes.c_double), len(p), int(reorder), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def read_gmsh(cls, path, reorder=0):
        h = ctypes.c_void_p()
        check(lib().fv_mesh_read_gmsh(path.encode(), int(reorder), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def read(cls, path, reorder=0):
        """Gmsh 2.2 (.msh) or SU2 (.su2) by extension (the reference's readMesh)."""
        h = ctypes.c_void_p()
        check(lib().fv_mesh_read(path.encode(), int(reorder), ctypes.byref(h)))
        return cls(h)

    def find_lines(self, threshold):
        """Lines of strongly coupled cells (the reference's findLines); the mesh
        keeps them for preconditioners created afterwards.  Returns
        (number of lines, line index of every cell or -1)."""
        cl = np.zeros(self.nelem, np.int32)
        nl = ctypes.c_int()
        check(lib().fv_mesh_find_lines(self._h, ctypes.c_double(threshold), ctypes.byref(nl), _hp(cl, ctypes.c_int)))
        return nl.value, cl

    def line_ordering(self, rcm=False):
        """The reference's hybrid line ordering on the lines found by
        find_lines, with the natural or the RCM order of the graph of lines
        and remaining cells; returns the cell at each position."""
        order = np.zeros(self.nelem, np.int32)
        check(lib().fv_mesh_line_ordering(self._h, int(bool(rcm)), _hp(order, ctypes.c_int)))
        return order

    def export(self):
        coords = np.zeros((self.npoin, 2))
        nnode = np.zeros(self.nelem, np.int32)
        inpoel = np.zeros((self.nelem, 4), np.int32)
        bface = np.zeros((self.nbface, 2), np.int32)
        btag = np.zeros(self.nbface, np.int32)
        perm = np.zeros(self.nelem, np.int32)
        check(lib().fv_mesh_export(self._h, _hp(coords, ctypes.c_double), _hp(nnode, ctypes.c_int),
                                   _hp(inpoel, ctypes.c_int), _hp(bface, ctypes.c_int), _hp(btag, ctypes.c_int),
                                   _hp(perm, ctypes.c_int)))
        return dict(coords=coords, nnode=nnode, inpoel=inpoel, bface=bface, btag=btag, perm=perm)

    def geometry(self):
        face_lr = np.zeros((self.naface, 2), np.int32)
        fnorm = np.zeros((self.naface, 3))
        area = np.zeros(self.nelem)
        cc = np.zeros((self.nelem, 2))
        color = np.zeros(self.nelem, np.int32)
        check(lib().fv_mesh_geometry(self._h, _hp(face_lr, ctypes.c_int), _hp(fnorm, ctypes.c_double),
                                     _hp(area, ctypes.c_double), _hp(cc, ctypes.c_double), _hp(color, ctypes.c_int)))
        return dict(face_lr=face_lr, fnorm=fnorm, area=area, cc=cc, color=color)

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fv_mesh_destroy(self._h)
            self._h = None


def physics_cfg(gamma=1.4, Minf=0.5, Tinf=288.15, Reinf=float("inf"), Pr=0.72, aoa_deg=0.0, viscous=False,
                const_visc=False):
    return fv_physics_cfg(gamma, Minf, Tinf, Reinf, Pr, np.deg2rad(aoa_deg), int(viscous), int(const_visc))


def numerics_cfg(flux="ROE", flux_jac=None, gradient="LEASTSQUARES", reconstruction="NONE", limiter_param=0.0,
                 order2=None):
    flux_jac = flux if flux_jac in (None, "CONSISTENT") else flux_jac
    if order2 is None:
        order2 = gradient != "NONE"
    return fv_numerics_cfg(FLUX[flux], FLUX[flux_jac], GRADIENT[gradient], RECONSTRUCTION[reconstruction],
                           float(limiter_param), int(order2))


class FlowFV:
    """GPU finite-volume flow discretisation of `batch` conditions on one mesh
    (reference FlowFV<scalar, order2, constVisc>)."""

    def __init__(self, mesh, phys, numerics, bcs):
        self.mesh = mesh
        phys = list(phys) if isinstance(phys, (list, tuple)) else [phys]
        self.batch = len(phys)
        self._phys = (fv_physics_cfg * self.batch)(*phys)
        self._num = numerics
        bl = [fv_bc_cfg(int(t), BC[k] if isinstance(k, str) else int(k), (ctypes.c_double * 2)(*(list(v) + [0, 0])[:2]))
              for (t, k, v) in bcs]
        self._bcs = (fv_bc_cfg * max(len(bl), 1))(*bl)
        h = ctypes.c_void_p()
        check(lib().fv_disc_create(mesh._h, self._phys, self.batch, ctypes.byref(self._num), self._bcs, len(bl),
                                   ctypes.byref(h)))
        self._h = h
        self.nelem = mesh.nelem

    def set_stream(self, stream):
        check(lib().fv_disc_set_stream(self._h, _vp(stream)))

    def synchronize(self):
        check(lib().fv_disc_synchronize(self._h))

    def freestream(self):
        u = np.zeros((self.batch, 4))
        check(lib().fv_disc_freestream(self._h, _hp(u, ctypes.c_double)))
        return u

    def compute_residual(self, u, r, gettimesteps=False, dt=None):
        """r += -R(u) (device arrays); dt receives local time steps when requested."""
        check(lib().fv_compute_residual(self._h, _vp(dptr(u)), _vp(dptr(r)), int(bool(gettimesteps)),
                                        _vp(dptr(dt)) if dt is not None else None))

    def get_gradients(self, u, grad, primitive=False):
        check(lib().fv_get_gradients(self._h, _vp(dptr(u)), _vp(dptr(grad)), int(bool(primitive))))

    def assemble_jacobian(self, u, matrix):
        check(lib().fv_assemble_jacobian(self._h, _vp(dptr(u)), matrix._h))

    def steady_fe_solve(self, u, cfl, tolerance=1e-10, max_timesteps=1000, abs_tolerance=True, raise_on_error=True):
        """SteadyForwardEulerSolver::solve on the device state u (in place);
        returns (status, per-member stats)."""
        c = solver_cfg(cfl_min=cfl, cfl_max=cfl, tolerance=tolerance, max_timesteps=max_timesteps,
                       abs_tolerance=int(bool(abs_tolerance)))
        st = (fv_solve_stats * self.batch)()
        rc = lib().fv_steady_fe_solve(self._h, ctypes.byref(c), _vp(dptr(u)), st)
        if raise_on_error:
            check(rc)
        return rc, [dict(steps=s.steps, status=s.status, res0=s.res0, res=s.res) for s in st]

    def tvdrk_solve(self, u, order, cfl, final_time, max_steps=1000000, raise_on_error=True):
        """TVDRKSolver::solve on the device state u (in place); returns
        (status, steps[batch], time[batch])."""
        steps = np.zeros(self.batch, np.int32)
        tm = np.zeros(self.batch)
        rc = lib().fv_tvdrk_solve(self._h, int(order), ctypes.c_double(cfl), ctypes.c_double(final_time),
                                  int(max_steps), _vp(dptr(u)), _hp(steps, ctypes.c_int), _hp(tm, ctypes.c_double))
        if raise_on_error:
            check(rc)
        return rc, steps, tm

    def autotune(self, u):
        """Picks the block sizes of the residual kernels and of the Jacobian's
        face kernel by timing them at state u (fv_disc_autotune); returns
        {states, gradients, faces, gather, jacobian_faces: block size}."""
        bs = np.zeros(5, np.int32)
        check(lib().fv_disc_autotune(self._h, _vp(dptr(u)), None))
        check(lib().fv_disc_block_sizes(self._h, 5, _hp(bs, ctypes.c_int)))
        return dict(zip(("states", "gradients", "faces", "gather", "jacobian_faces"), bs.tolist()))

    def entropy_error(self, u):
        """FlowOutput::compute_entropy_cell per batch member."""
        out = np.zeros(self.batch)
        check(lib().fv_entropy_error(self._h, _vp(dptr(u)), _hp(out, ctypes.c_double)))
        return out

    def surface_data(self, u, wall_marker):
        """(Cl, CDp, CDsf) over the faces of wall_marker, one row per batch member
        (FlowFV_base::computeSurfaceData)."""
        out = np.zeros((self.batch, 3))
        check(lib().fv_surface_data(self._h, _vp(dptr(u)), int(wall_marker), _hp(out, ctypes.c_double)))
        return out

    def surface_distribution(self, u, wall_marker, member=0):
        """Rows (x, y, Cp, Cf) of the faces of wall_marker (the per-face output
        of computeSurfaceData), for one batch member."""
        n = ctypes.c_int()
        check(lib().fv_surface_distribution(self._h, None, int(wall_marker), int(member), None, ctypes.byref(n)))
        out = np.zeros((n.value, 4))
        check(lib().fv_surface_distribution(self._h, _vp(dptr(u)), int(wall_marker), int(member),
                                            _hp(out, ctypes.c_double), ctypes.byref(n)))
        return out

    def export_surface_data(self, u, wall_markers, other_markers, basename, member=0):
        """FlowOutput::exportSurfaceData (aoutput.cpp:181-298): for each wall
        marker the file <basename>-surf_w<marker>.out with rows x, y, Cp, Cf and
        the Cl, Cdp, Cdf trailer; for each other marker <basename>-surf_o<marker>.out
        with the face centres and the velocity of the faces' cells.  Returns
        {marker: (Cl, Cdp, Cdf)} of the wall markers."""
        g = lambda v: format(float(v), ".6g")
        out = {}
        for wm in wall_markers:
            rows = self.surface_distribution(u, wm, member)
            cl = self.surface_data(u, wm)[member]
            with open(f"{basename}-surf_w{wm}.out", "w") as f:
                f.write("#  x \t y \t Cp  \t Cf \n")
                for r in rows:
                    f.write("".join("  " + g(v) for v in r) + "\n")
                f.write("# Cl      Cdp      Cdf\n")
                f.write(f"# {g(cl[0])}  {g(cl[1])}  {g(cl[2])}\n")
            out[wm] = tuple(float(x) for x in cl)
        if other_markers:
            ex, geo = self.mesh.export(), self.mesh.geometry()
            uh = u.detach().cpu().numpy().reshape(self.batch, self.nelem, 4)[member]
            fc = ex["coords"][ex["bface"]].mean(axis=1)
            for om in other_markers:
                with open(f"{basename}-surf_o{om}.out", "w") as f:
                    f.write("#   x         y          u           v\n")
                    for k in np.nonzero(ex["btag"] == om)[0]:
                        c = uh[geo["face_lr"][k, 0]]
                        f.write("".join("  " + g(v) for v in (fc[k, 0], fc[k, 1], c[1] / c[0], c[2] / c[0])) + "\n")
        return out

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fv_disc_destroy(self._h)
            self._h = None


class BlockMatrix:
    """Jacobian storage (PETSc BAIJ(4) equivalent), FP32 (precision 4) or FP64 (8)."""

    def __init__(self, disc, precision=4):
        self.disc = disc
        h = ctypes.c_void_p()
        check(lib().fv_matrix_create(disc._h, int(precision), ctypes.byref(h)))
        self._h = h
        self.precision = precision

    def add_diagonal(self, diag):
        check(lib().fv_matrix_add_diagonal(self.disc._h, self._h, _vp(dptr(diag))))

    def to_host(self, member=0):
        nnzb = ctypes.c_int()
        L = lib()
        check(L.fv_matrix_to_host(self.disc._h, self._h, int(member), ctypes.byref(nnzb), None, None, None))
        n = self.disc.nelem
        rowptr = np.zeros(n + 1, np.int32)
        col = np.zeros(nnzb.value, np.int32)
        val = np.zeros((nnzb.value, 16))
        check(L.fv_matrix_to_host(self.disc._h, self._h, int(member), ctypes.byref(nnzb), _hp(rowptr, ctypes.c_int),
                                  _hp(col, ctypes.c_int), _hp(val, ctypes.c_double)))
        return rowptr, col, val

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fv_matrix_destroy(self._h)
            self._h = None


def kernel_launch_count():
    return int(lib().fv_kernel_launch_count())


def fp64_peak(reps=5):
    """FP64 throughput ceiling of the current device: (FMA thread-instructions
    per second, best launch in ms) from fv_fp64_peak."""
    rate, ms = ctypes.c_double(), ctypes.c_double()
    check(lib().fv_fp64_peak(int(reps), ctypes.byref(rate), ctypes.byref(ms)))
    return rate.value, ms.value


class Preconditioner:
    """PETSc PC equivalent on a BlockMatrix: 'jacobi', 'sgs' or 'ilu0'."""

    def __init__(self, disc, matrix, kind="ilu0", ordering=1, part_size=128):
        self.disc, self.matrix = disc, matrix
        h = ctypes.c_void_p()
        check(lib().fv_precond_create(disc._h, matrix._h, PC[kind], int(ordering), int(part_size), ctypes.byref(h)))
        self._h = h

    def setup(self):
        check(lib().fv_precond_setup(self._h))

    def apply(self, r, z):
        check(lib().fv_precond_apply(self._h, _vp(dptr(r)), _vp(dptr(z))))

    def order(self):
        o = np.zeros(self.disc.nelem, np.int32)
        check(lib().fv_precond_order(self._h, _hp(o, ctypes.c_int)))
        return o

    def ksp_solve(self, b, x, restart=30, maxit=30, rtol=0.1):
        its = np.zeros(self.disc.batch, np.int32)
        check(lib().fv_ksp_solve(self._h, _vp(dptr(b)), _vp(dptr(x)), int(restart), int(maxit), ctypes.c_double(rtol),
                                 _hp(its, ctypes.c_int)))
        return its

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fv_precond_destroy(self._h)
            self._h = None


def matvec(disc, matrix, x, y):
    check(lib().fv_matvec(disc._h, matrix._h, _vp(dptr(x)), _vp(dptr(y))))


class fv_solver_cfg(ctypes.Structure):
    _fields_ = [("cfl_min", ctypes.c_double), ("cfl_max", ctypes.c_double), ("tolerance", ctypes.c_double),
                ("max_timesteps", ctypes.c_int), ("abs_tolerance", ctypes.c_int), ("pc_type", ctypes.c_int),
                ("ksp_restart", ctypes.c_int), ("ksp_maxit", ctypes.c_int), ("ksp_rtol", ctypes.c_double),
                ("matrix_free", ctypes.c_int), ("mf_eps", ctypes.c_double), ("nl_update", ctypes.c_int),
                ("min_relax", ctypes.c_double), ("precision", ctypes.c_int), ("check_every", ctypes.c_int),
                ("use_graph", ctypes.c_int), ("pc_ordering", ctypes.c_int), ("pc_part_size", ctypes.c_int),
                ("stall_steps", ctypes.c_int), ("stall_factor", ctypes.c_double)]


class fv_solve_stats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("lin_iters", ctypes.c_int), ("status", ctypes.c_int),
                ("res0", ctypes.c_double), ("res", ctypes.c_double), ("cfl", ctypes.c_double)]


def solver_cfg(**kw):
    c = fv_solver_cfg()
    lib().fv_solver_cfg_default(ctypes.byref(c))
    names = {f[0] for f in fv_solver_cfg._fields_}
    for k, v in kw.items():
        if k == "pc":
            c.pc_type = PC[v]
        elif k == "nl_update" and isinstance(v, str):
            c.nl_update = {"full": 0, "robust_flow": 1, "bounded": 2}[v]
        elif k in names:
            setattr(c, k, v)
        else:
            raise KeyError(k)
    return c


class SteadyBackwardEulerSolver:
    """Implicit pseudo-time steady solver (reference SteadyBackwardEulerSolver)."""

    def __init__(self, disc, cfg=None, **kw):
        self.disc = disc
        self.cfg = cfg if cfg is not None else solver_cfg(**kw)
        h = ctypes.c_void_p()
        check(lib().fv_solver_create(disc._h, ctypes.byref(self.cfg), ctypes.byref(h)))
        self._h = h

    def _stats(self, st):
        return [dict(steps=s.steps, lin_iters=s.lin_iters, status=s.status, res0=s.res0, res=s.res, cfl=s.cfl)
                for s in st]

    def solve(self, u, member_mask=None, raise_on_error=True):
        """Solves in place; u is a device array (batch x nelem x 4)."""
        st = (fv_solve_stats * self.disc.batch)()
        mask = None if member_mask is None else np.ascontiguousarray(member_mask, np.int32)
        rc = lib().fv_solver_solve(self._h, _vp(dptr(u)), _hp(mask, ctypes.c_int) if mask is not None else None, st)
        if raise_on_error:
            check(rc)
        return rc, self._stats(st)

    def solve_host(self, u, member_mask=None, raise_on_error=True):
        """Solves a host numpy state in place (copies in and out)."""
        assert u.dtype == np.float64 and u.flags.c_contiguous
        st = (fv_solve_stats * self.disc.batch)()
        mask = None if member_mask is None else np.ascontiguousarray(member_mask, np.int32)
        rc = lib().fv_solver_solve_host(self._h, _hp(u, ctypes.c_double),
                                        _hp(mask, ctypes.c_int) if mask is not None else None, st)
        if raise_on_error:
            check(rc)
        return rc, self._stats(st)

    def history(self, member=0):
        n = ctypes.c_int()
        mx = self.cfg.max_timesteps
        res = np.zeros(mx); cfl = np.zeros(mx); lin = np.zeros(mx, np.int32)
        check(lib().fv_solver_history(self._h, int(member), mx, _hp(res, ctypes.c_double), _hp(cfl, ctypes.c_double),
                                      _hp(lin, ctypes.c_int), ctypes.byref(n)))
        k = n.value
        return res[:k], cfl[:k], lin[:k]

    def write_convergence_history(self, path_or_file, member=0, wall_time=None):
        """Writes the convergence history of one member in the reference's
        format (writeConvergenceHistoryHeader / writeStepToConvergenceHistory,
        aoutput.cpp:617-636): step, log10 relative and absolute residual,
        total and linear wall time, linear iterations (cumulative), CFL.  The
        device loop keeps no per-step clock: the time columns hold the solve's
        wall time spread evenly over its steps when wall_time is given, else 0."""
        res, cfl, lin = self.history(member)
        n = len(res)
        lines = ["#%6s%14s%14s%12s%12s%12s%10s" % ("NStep", "Log rel resi", "Log abs resi", "Tot.Wtime",
                                                   "Lin.Wtime", "Lin.iters", "CFL"),
                 "#" + "-" * 82]
        total = 0
        for k in range(n):
            total += int(lin[k])
            t = (wall_time * (k + 1) / n) if wall_time else 0.0
            lines.append("%7d%14.6g%14.6g%12.4g%12.4g%12d%10.4g" % (
                k + 1, np.log10(res[k] / res[0]), np.log10(res[k]), t, 0.0, total, cfl[k]))
        text = "\n".join(lines) + "\n"
        if hasattr(path_or_file, "write"):
            path_or_file.write(text)
        else:
            with open(path_or_file, "w") as f:
                f.write(text)

    def kernels_per_step(self):
        L = lib()
        L.fv_solver_kernels_per_step.restype = ctypes.c_longlong
        return int(L.fv_solver_kernels_per_step(self._h))

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fv_solver_destroy(self._h)
            self._h = None
