"""Steady flow cases driven by the reference's control files.

The layer above the C ABI that the reference's ``fvens_steady`` executable
provides: parse a control file (boost INFO format, the keys of
``parse_flow_controlfile``, src/utilities/controlparser.cpp:59-215) and its
PETSc options file (``opts.solverc``), read the mesh, run the first-order
starter and the main implicit solve (SteadyFlowCase::execute_starter /
execute_main / execute, src/utilities/casesolvers.cpp:225-422) and write the
outputs of FlowCase::run_output (casesolvers.cpp:86-164): the convergence
history ``<log_file_prefix>-residual_history.log``, the surface files of
``listof_output_wall_boundaries`` / ``listof_output_other_boundaries`` and the
functionals (h, entropy error, Cl, Cdp, Cdf).

    python -m fvens_gb300.case case.ctrl [--options opts.solverc] [--mesh_file m.msh]

Differences from the reference: ``limiter_parameter`` is read (the reference
leaves it unset); implicit pseudo-time only (explicit cases go through
``FlowFV.steady_fe_solve``); no VTU volume output.
"""
import argparse
import math
import shlex
import sys
import time
from dataclasses import dataclass, field

import numpy as np


class ControlFileError(ValueError):
    pass


# ------------------------------------------------------------------ INFO format
def parse_info(text):
    """Parses boost property_tree INFO text into nested dicts
    {key: (value, children)}; repeated keys keep the first occurrence, as
    ptree::get does.  ';' starts a comment outside quotes; a '{' (on the key's
    line or the next) opens the children of the last key."""
    root = {}
    stack = [root]
    last = None  # children dict of the most recent key at the current level

    def tokens(line):
        out, i, n = [], 0, len(line)
        while i < n:
            c = line[i]
            if c.isspace():
                i += 1
            elif c == ";":
                break
            elif c in "{}":
                out.append(c)
                i += 1
            elif c == '"':
                j, buf = i + 1, []
                while j < n and line[j] != '"':
                    if line[j] == "\\" and j + 1 < n:
                        j += 1
                        buf.append({"n": "\n", "t": "\t", "0": "\0"}.get(line[j], line[j]))
                    else:
                        buf.append(line[j])
                    j += 1
                if j >= n:
                    raise ControlFileError("unterminated string: " + line.strip())
                out.append(("str", "".join(buf)))
                i = j + 1
            else:
                j = i
                while j < n and not line[j].isspace() and line[j] not in '{};"':
                    j += 1
                out.append(("str", line[i:j]))
                i = j
        return out

    for lineno, line in enumerate(text.splitlines(), 1):
        toks = tokens(line)
        k = 0
        while k < len(toks):
            t = toks[k]
            if t == "{":
                if last is None:
                    raise ControlFileError(f"line {lineno}: '{{' without a key")
                stack.append(last)
                last = None
            elif t == "}":
                if len(stack) == 1:
                    raise ControlFileError(f"line {lineno}: unbalanced '}}'")
                stack.pop()
                last = None
            else:
                key = t[1]
                val = ""
                if k + 1 < len(toks) and isinstance(toks[k + 1], tuple):
                    val = toks[k + 1][1]
                    k += 1
                children = {}  # a repeated key keeps its first entry; the later one's block is dropped
                if key not in stack[-1]:
                    stack[-1][key] = (val, children)
                last = children
            k += 1
    if len(stack) != 1:
        raise ControlFileError("unbalanced '{'")
    return root


def _get(tree, path, default=KeyError):
    node = (None, tree)
    for part in path.split("."):
        if part not in node[1]:
            if default is KeyError:
                raise ControlFileError(f"control file: no key '{path}'")
            return default
        node = node[1][part]
    return node[0]


def _has(tree, path):
    return _get(tree, path, None) is not None


def _bool(s):
    v = str(s).strip().lower()
    if v in ("true", "1", "yes", "on"):
        return True
    if v in ("false", "0", "no", "off"):
        return False
    raise ControlFileError(f"not a boolean: {s}")


# --------------------------------------------------------------------- options
@dataclass
class FlowParserOptions:
    """The fields of the reference's FlowParserOptions that a steady case uses
    (controlparser.hpp), with its defaults."""
    meshfile: str = ""
    vtu_output_file: str = ""
    logfile: str = ""
    lognres: bool = False
    flowtype: str = "EULER"
    gamma: float = 1.4
    alpha: float = 0.0          # radians
    Minf: float = 0.5
    Tinf: float = 298.0
    Reinf: float = math.inf
    Pr: float = math.nan
    viscsim: bool = False
    useconstvisc: bool = False
    bcconf: list = field(default_factory=list)   # (marker, type, values)
    lwalls: list = field(default_factory=list)
    lothers: list = field(default_factory=list)
    surfnameprefix: str = ""
    sim_type: str = "STEADY"
    invflux: str = "ROE"
    invfluxjac: str = "ROE"
    gradientmethod: str = "NONE"
    order2: bool = True
    limiter: str = "NONE"
    limiter_param: float = 0.0
    pseudotimetype: str = "IMPLICIT"
    initcfl: float = 0.0
    endcfl: float = 0.0
    tolerance: float = 0.0
    maxiter: int = 0
    usestarter: bool = False
    firstinitcfl: float = 0.0
    firstendcfl: float = 0.0
    firsttolerance: float = 0.0
    firstmaxiter: int = 0
    nl_update_scheme: str = "FULL"
    min_nl_update: float = 0.2

    def bcconf_tuples(self):
        """Boundary conditions as (marker, type name, values) for FlowFV."""
        return [(marker, typ, vals) for (marker, typ, vals) in self.bcconf]


# scheme names of the control file (afactory.cpp:103-227)
_LIMITERS = ("NONE", "VANALBADA", "BARTHJESPERSEN", "VENKATAKRISHNAN", "WENO")
_GRADIENTS = ("NONE", "LEASTSQUARES", "GREENGAUSS")
# boundary-condition names of the control file (bcTypeMap, src/spatial/abctypemap.cpp:16-30)
_BC_NAMES = ("slipwall", "isothermalwall", "adiabaticwall", "farfield", "inflowoutflow", "subsonic_inflow",
             "extrapolation", "periodic")
_BCS_NEEDING_VALUES = ("adiabaticwall", "isothermalwall", "subsonic_inflow")


def parse_flow_controlfile(path, mesh_file=None):
    """parse_flow_controlfile (controlparser.cpp:59-215) restated: the same keys,
    defaults and required entries (a missing required key raises
    ControlFileError).  mesh_file overrides io.mesh_file, as the command-line
    option of the reference."""
    with open(path) as f:
        t = parse_info(f.read())
    o = FlowParserOptions()
    o.meshfile = mesh_file or _get(t, "io.mesh_file")
    o.vtu_output_file = _get(t, "io.solution_output_file")
    o.logfile = _get(t, "io.log_file_prefix")
    o.lognres = _bool(_get(t, "io.convergence_history_required"))
    o.flowtype = _get(t, "flow_conditions.flow_type").upper()
    o.gamma = float(_get(t, "flow_conditions.adiabatic_index"))
    o.alpha = math.pi / 180.0 * float(_get(t, "flow_conditions.angle_of_attack"))
    o.Minf = float(_get(t, "flow_conditions.freestream_Mach_number"))
    if o.flowtype in ("NAVIERSTOKES", "RANS"):
        if o.flowtype == "RANS":
            raise ControlFileError("unsupported option: flowtype RANS")
        o.viscsim = True
        o.Tinf = float(_get(t, "flow_conditions.freestream_temperature"))
        o.Reinf = float(_get(t, "flow_conditions.freestream_Reynolds_number"))
        o.Pr = float(_get(t, "flow_conditions.Prandtl_number"))
        o.useconstvisc = _bool(_get(t, "flow_conditions.use_constant_viscosity", "false"))
    else:
        o.viscsim, o.Tinf, o.Reinf, o.Pr = False, 298.0, math.inf, math.nan
    # boundary conditions bc0, bc1, ... numbered consecutively
    k = 0
    while _has(t, f"bc.bc{k}"):
        typ = _get(t, f"bc.bc{k}.type").lower()
        if typ not in _BC_NAMES:
            raise ControlFileError(f"unknown boundary condition type '{typ}'")
        marker = int(_get(t, f"bc.bc{k}.marker"))
        vals = ()
        if typ in _BCS_NEEDING_VALUES:
            vals = tuple(float(x) for x in _get(t, f"bc.bc{k}.boundary_values").split())
        if typ == "periodic":
            vals = tuple(int(x) for x in _get(t, f"bc.bc{k}.options").split())
        o.bcconf.append((marker, typ, vals))
        k += 1
    lw = _get(t, "bc.listof_output_wall_boundaries", None)
    o.lwalls = [int(x) for x in lw.split()] if lw else []
    lo = _get(t, "bc.listof_output_other_boundaries", None)
    o.lothers = [int(x) for x in lo.split()] if lo else []
    if o.lwalls or o.lothers:
        o.surfnameprefix = _get(t, "bc.surface_output_file_prefix")
    o.sim_type = _get(t, "time.simulation_type").upper()
    o.invflux = _get(t, "spatial_discretization.inviscid_flux").upper()
    o.gradientmethod = _get(t, "spatial_discretization.gradient_method").upper()
    if o.gradientmethod not in _GRADIENTS:
        raise ControlFileError(f"unknown gradient method '{o.gradientmethod}'")
    o.order2 = o.gradientmethod != "NONE"
    o.limiter = _get(t, "spatial_discretization.limiter").upper()
    if o.limiter not in _LIMITERS:
        raise ControlFileError(f"unknown limiter '{o.limiter}'")
    o.limiter_param = float(_get(t, "spatial_discretization.limiter_parameter", "0"))
    o.pseudotimetype = _get(t, "pseudotime.pseudotime_stepping_type").upper()
    o.initcfl = float(_get(t, "pseudotime.main.cfl_min"))
    o.endcfl = float(_get(t, "pseudotime.main.cfl_max"))
    o.tolerance = float(_get(t, "pseudotime.main.tolerance"))
    o.maxiter = int(_get(t, "pseudotime.main.max_timesteps"))
    if _has(t, "pseudotime.initialization"):
        o.usestarter = True
        o.firstinitcfl = float(_get(t, "pseudotime.initialization.cfl_min"))
        o.firstendcfl = float(_get(t, "pseudotime.initialization.cfl_max"))
        o.firsttolerance = float(_get(t, "pseudotime.initialization.tolerance"))
        o.firstmaxiter = int(_get(t, "pseudotime.initialization.max_timesteps"))
    if o.pseudotimetype == "IMPLICIT":
        jac = _get(t, "Jacobian_inviscid_flux").upper()
        o.invfluxjac = o.invflux if jac == "CONSISTENT" else jac
        o.nl_update_scheme = _get(t, "pseudotime.nonlinear_update_scheme").upper()
        o.min_nl_update = float(_get(t, "pseudotime.min_nonlinear_relaxation_factor", "0.2"))
    return o


@dataclass
class SolverOptions:
    """The PETSc options of an ``opts.solverc`` file that the GPU solver maps."""
    ksp_type: str = "fgmres"
    ksp_rtol: float = 1e-1
    ksp_max_it: int = 30
    ksp_restart: int = 30
    pc_type: str = "bjacobi"
    sub_pc_type: str = "ilu"
    matrix_free: bool = False
    mf_eps: float = 1e-7
    mesh_reorder: str = "rcm"
    anisotropy_threshold: float = 0.0
    ignored: list = field(default_factory=list)


def parse_solver_options(path):
    """Reads a PETSc options file (one or more '-key [value]' per line, '#'
    comments)."""
    s = SolverOptions()
    if not path:
        return s
    with open(path) as f:
        words = []
        for line in f:
            words += shlex.split(line.split("#", 1)[0])
    i = 0
    while i < len(words):
        key = words[i]
        val = words[i + 1] if i + 1 < len(words) and not words[i + 1].startswith("-") else None
        i += 2 if val is not None else 1
        k = key.lstrip("-")
        if k == "ksp_type":
            s.ksp_type = val
        elif k == "ksp_rtol":
            s.ksp_rtol = float(val)
        elif k == "ksp_max_it":
            s.ksp_max_it = int(val)
        elif k == "ksp_gmres_restart":
            s.ksp_restart = int(val)
        elif k == "pc_type":
            s.pc_type = val
        elif k == "sub_pc_type":
            s.sub_pc_type = val
        elif k == "matrix_free_jacobian":
            s.matrix_free = True
        elif k == "matrix_free_difference_step":
            s.mf_eps = float(val)
        elif k == "mesh_reorder":
            s.mesh_reorder = val
        elif k == "mesh_anisotropy_threshold":
            s.anisotropy_threshold = float(val)
        else:
            s.ignored.append(key)
    return s


def _pc_kind(so):
    """PETSc preconditioner name -> the GPU preconditioner (block ILU(0) for
    bjacobi+ilu, block SGS for sor, point-block Jacobi for pbjacobi/jacobi)."""
    if so.pc_type in ("bjacobi", "asm", "ilu"):
        return "ilu0" if so.sub_pc_type in ("ilu", None) else ("sgs" if so.sub_pc_type == "sor" else "jacobi")
    if so.pc_type == "sor":
        return "sgs"
    if so.pc_type in ("pbjacobi", "jacobi", "bjacobi_point"):
        return "jacobi"
    if so.pc_type == "none":
        return "none"
    raise ControlFileError(f"unsupported preconditioner '{so.pc_type}'")


# ------------------------------------------------------------------------ case
@dataclass
class FlowSolutionFunctionals:
    h: float
    entropy: float
    Cl: float
    Cdp: float
    Cdf: float


class SteadyFlowCase:
    """SteadyFlowCase (casesolvers.cpp:207-422) on the GPU: starter + main
    implicit solves, then the outputs of run_output."""

    def __init__(self, opts, solver_opts=None, precision=4, nl_update=None):
        import fvens_gb300 as fv
        self.fv = fv
        self.opts = opts
        self.so = solver_opts or SolverOptions()
        self.precision = precision
        self.nl_update = nl_update
        if opts.sim_type != "STEADY":
            raise ControlFileError("SteadyFlowCase needs simulation_type steady")
        if opts.pseudotimetype != "IMPLICIT":
            raise ControlFileError("only implicit pseudo-time stepping is driven from control files")

    def physics(self):
        o = self.opts
        return self.fv.physics_cfg(gamma=o.gamma, Minf=o.Minf, Tinf=o.Tinf, Reinf=o.Reinf,
                                   Pr=o.Pr if not math.isnan(o.Pr) else 0.72, aoa_deg=math.degrees(o.alpha),
                                   viscous=o.viscsim, const_visc=o.useconstvisc)

    def read_mesh(self):
        fv = self.fv
        m = fv.UMesh.read(self.opts.meshfile, reorder=1 if self.so.mesh_reorder in ("rcm", "line") else 0)
        if self.so.mesh_reorder == "line":
            m.find_lines(self.so.anisotropy_threshold)
        return m

    def _solver(self, disc, cflmin, cflmax, tol, maxiter):
        o, so = self.opts, self.so
        nl = self.nl_update if self.nl_update is not None else {"FULL": 0, "ROBUST_FLOW": 1}.get(o.nl_update_scheme)
        if nl is None:
            raise ControlFileError(f"unknown nonlinear_update_scheme '{o.nl_update_scheme}'")
        return self.fv.SteadyBackwardEulerSolver(
            disc, cfl_min=cflmin, cfl_max=cflmax, tolerance=tol, max_timesteps=maxiter, abs_tolerance=0,
            pc=_pc_kind(so), precision=self.precision, ksp_restart=so.ksp_restart, ksp_maxit=so.ksp_max_it,
            ksp_rtol=so.ksp_rtol, matrix_free=int(so.matrix_free), mf_eps=so.mf_eps, nl_update=nl,
            min_relax=o.min_nl_update)

    def discretisations(self, m):
        fv, o = self.fv, self.opts
        num = fv.numerics_cfg(flux=o.invflux, flux_jac=o.invfluxjac, gradient=o.gradientmethod,
                              reconstruction=o.limiter, limiter_param=o.limiter_param, order2=o.order2)
        num1 = fv.numerics_cfg(flux=o.invflux, flux_jac=o.invfluxjac, gradient="NONE", reconstruction="NONE",
                               limiter_param=1.0, order2=False)
        main = fv.FlowFV(m, self.physics(), num, o.bcconf_tuples())
        start = fv.FlowFV(m, self.physics(), num1, o.bcconf_tuples()) if o.usestarter else None
        return main, start

    def execute(self, m, u=None, log=print, net=None):
        """Starter (Tolerance errors ignored) and main solve on the device
        state u (freestream when None).  With a warm-start network `net` the
        main solve starts from its prediction instead, and falls back to
        freestream + starter when it does not converge.  Returns (u, main
        stats, starter stats, main solver, discretisation)."""
        import torch
        o = self.opts
        main, start = self.discretisations(m)
        if net is not None:
            from .mpnn import warm_started_solve
            u = torch.empty((m.nelem, 4), dtype=torch.float64, device="cuda")
            S2 = self._solver(main, o.initcfl, o.endcfl, o.tolerance, o.maxiter)
            if start is None:
                start = self.fv.FlowFV(m, self.physics(), self.fv.numerics_cfg(
                    flux=o.invflux, flux_jac=o.invfluxjac, gradient="NONE", limiter_param=1.0, order2=False),
                    o.bcconf_tuples())
            S1 = self._solver(start, o.firstinitcfl or o.initcfl, o.firstendcfl or o.endcfl,
                              o.firsttolerance or 1e-1, o.firstmaxiter or 50)
            stats, fell = warm_started_solve(net, [self.physics()], main, S1, S2, u)
            log(f"SteadyFlowCase: warm start, main {stats[0]['steps']} steps, status {stats[0]['status']}"
                + (" (fell back to freestream)" if fell else ""))
            return u, stats[0], None, S2, main
        if u is None:
            u = torch.tensor(np.tile(main.freestream()[0], (m.nelem, 1)), device="cuda")
        st1 = None
        if start is not None:
            S1 = self._solver(start, o.firstinitcfl, o.firstendcfl, o.firsttolerance, o.firstmaxiter)
            rc, st1 = S1.solve(u, raise_on_error=False)
            st1 = st1[0]
            if rc not in (0, self.fv.FV_ERR_TOLERANCE):
                self.fv.check(rc)
            log(f"SteadyFlowCase: starter {st1['steps']} steps, status {st1['status']}")
        S2 = self._solver(main, o.initcfl, o.endcfl, o.tolerance, o.maxiter)
        rc, st2 = S2.solve(u, raise_on_error=False)
        st2 = st2[0]
        log(f"SteadyFlowCase: main {st2['steps']} steps, {st2['lin_iters']} linear iterations, "
            f"status {st2['status']}, residual {st2['res']:.3e}")
        return u, st2, st1, S2, main

    def run_output(self, m=None, surface_files=True, log=print, net=None):
        """FlowCase::run_output (casesolvers.cpp:86-164): solve (from the
        network's prediction when `net` is given), write the convergence
        history and surface files, return the functionals."""
        o = self.opts
        m = m or self.read_mesh()
        t0 = time.perf_counter()
        u, st, st1, S, main = self.execute(m, log=log, net=net)
        wall = time.perf_counter() - t0
        if st["status"] == self.fv.FV_ERR_NUMERICAL:
            raise self.fv.FvensError(st["status"], "main flow solve failed (non-finite residual)")
        if st["status"] != 0:
            log("SteadyFlowCase: main flow solve did not converge")
        if o.lognres:
            S.write_convergence_history(o.logfile + "-residual_history.log", wall_time=wall)
        entropy = float(main.entropy_error(u)[0])
        if surface_files and (o.lwalls or o.lothers):
            coeffs = main.export_surface_data(u, o.lwalls, o.lothers, o.surfnameprefix)
            for wm, c in coeffs.items():
                log(f"FlowOutput: CL = {c[0]:g}   CDp = {c[1]:g}    CDf = {c[2]:g}")
        cl = main.surface_data(u, o.lwalls[0])[0] if o.lwalls else (math.nan,) * 3
        h = 1.0 / math.sqrt(m.nelem)
        return FlowSolutionFunctionals(h, entropy, float(cl[0]), float(cl[1]), float(cl[2])), st


def main(argv=None):
    ap = argparse.ArgumentParser(description="steady flow case from a control file (GPU)")
    ap.add_argument("control_file")
    ap.add_argument("--options", default=None, help="PETSc-style solver options file (opts.solverc)")
    ap.add_argument("--mesh_file", default=None)
    ap.add_argument("--precision", type=int, default=4, choices=[4, 8],
                    help="stored Jacobian / preconditioner precision (4: FP32, 8: FP64)")
    ap.add_argument("--warm-start", default=None,
                    help="trained network (.npz from fvens_gb300.mpnn.MPNN.save) predicting the initial state")
    a = ap.parse_args(argv)
    opts = parse_flow_controlfile(a.control_file, a.mesh_file)
    case = SteadyFlowCase(opts, parse_solver_options(a.options), precision=a.precision)
    m = case.read_mesh()
    net = None
    if a.warm_start:
        from .mpnn import MPNN
        net = MPNN.load(m, a.warm_start)
    f, st = case.run_output(m, net=net)
    print(f"h {f.h:.6g} entropy {f.entropy:.6g} Cl {f.Cl:.10g} Cdp {f.Cdp:.10g} Cdf {f.Cdf:.10g}")
    return 0 if st["status"] == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
