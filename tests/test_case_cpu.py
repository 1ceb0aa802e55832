"""Control-file layer (fvens_gb300/case.py): the INFO-format parser, the
keys and defaults of parse_flow_controlfile (controlparser.cpp:59-215) and the
PETSc options file; with the reference present, every control file of its
test cases parses."""
import glob
import math
import os

import pytest

from fvens_gb300 import case
from oracle import orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
_REF = orc.reference_root()
REF_TESTCASES = os.path.join(_REF, "testcases") if _REF else ""


def test_info_parser_nesting_comments_quotes():
    t = case.parse_info('''
;; comment line
a 1 ; trailing comment
b "two words ; not a comment"
c
{
    d  3
    e { f "x" }
}
a 5
''')
    assert case._get(t, "a") == "1"          # the first of a repeated key
    assert case._get(t, "b") == "two words ; not a comment"
    assert case._get(t, "c.d") == "3" and case._get(t, "c.e.f") == "x"
    assert case._get(t, "c.nothing", None) is None
    with pytest.raises(case.ControlFileError):
        case._get(t, "c.nothing")
    with pytest.raises(case.ControlFileError):
        case.parse_info("a {\n b 1\n")
    with pytest.raises(case.ControlFileError):
        case.parse_info("}\n")


def test_channel_control_file():
    o = case.parse_flow_controlfile(os.path.join(GOLDEN, "channel_case.ctrl"))
    assert o.meshfile == "channel.msh" and o.logfile == "channel" and o.lognres
    assert o.flowtype == "EULER" and not o.viscsim and math.isinf(o.Reinf) and math.isnan(o.Pr) and o.Tinf == 298.0
    assert o.Minf == 0.5 and o.alpha == 0.0 and o.gamma == 1.4
    assert o.bcconf == [(1, "slipwall", ()), (2, "inflowoutflow", ()), (3, "slipwall", ()), (4, "inflowoutflow", ())]
    assert o.lwalls == [1, 3] and o.lothers == [4] and o.surfnameprefix == "channel"
    assert o.invflux == "ROE" and o.invfluxjac == "ROE" and o.gradientmethod == "LEASTSQUARES" and o.order2
    assert o.limiter == "NONE" and o.limiter_param == 20.0
    assert (o.initcfl, o.endcfl, o.tolerance, o.maxiter) == (10.0, 1000.0, 1e-8, 300)
    assert o.usestarter and (o.firstinitcfl, o.firstendcfl, o.firsttolerance, o.firstmaxiter) == (10.0, 500.0, 0.1, 20)
    assert o.nl_update_scheme == "FULL" and o.min_nl_update == 0.2
    o2 = case.parse_flow_controlfile(os.path.join(GOLDEN, "channel_case.ctrl"), mesh_file="other.msh")
    assert o2.meshfile == "other.msh"


def test_control_file_errors(tmp_path):
    text = open(os.path.join(GOLDEN, "channel_case.ctrl")).read()
    p = tmp_path / "bad.ctrl"
    p.write_text(text.replace("freestream_Mach_number        0.5", ""))
    with pytest.raises(case.ControlFileError, match="freestream_Mach_number"):
        case.parse_flow_controlfile(str(p))
    p.write_text(text.replace("type                     slipwall\n\t\tmarker                   1",
                              "type                     nowall\n\t\tmarker                   1"))
    with pytest.raises(case.ControlFileError, match="nowall"):
        case.parse_flow_controlfile(str(p))
    p.write_text(text.replace("flow_type                     euler", "flow_type rans"))
    with pytest.raises(case.ControlFileError, match="RANS"):
        case.parse_flow_controlfile(str(p))


def test_solver_options_file():
    so = case.parse_solver_options(os.path.join(GOLDEN, "channel_opts.solverc"))
    assert so.ksp_type == "fgmres" and so.ksp_rtol == 0.1 and so.ksp_max_it == 30
    assert so.pc_type == "bjacobi" and so.sub_pc_type == "ilu" and case._pc_kind(so) == "ilu0"
    assert not so.matrix_free and so.mesh_reorder == "rcm"
    assert case._pc_kind(case.SolverOptions(pc_type="sor")) == "sgs"
    assert case._pc_kind(case.SolverOptions(pc_type="pbjacobi")) == "jacobi"
    with pytest.raises(case.ControlFileError):
        case._pc_kind(case.SolverOptions(pc_type="mg"))


@pytest.mark.skipif(not os.path.isdir(REF_TESTCASES), reason="reference test cases not present")
def test_reference_control_files_parse():
    files = sorted(glob.glob(os.path.join(REF_TESTCASES, "*", "*.ctrl")))
    assert files
    for f in files:
        o = case.parse_flow_controlfile(f)
        assert o.meshfile and o.bcconf and o.maxiter > 0, f
    o = case.parse_flow_controlfile(os.path.join(REF_TESTCASES, "visc-naca0012", "laminar-implicit.ctrl"))
    assert o.viscsim and o.Reinf == 5000.0 and o.Pr == 0.72 and o.Tinf == 288.15
    assert (2, "adiabaticwall", (0.0,)) in o.bcconf and o.lwalls == [2]
    assert (o.initcfl, o.endcfl, o.maxiter, o.firstmaxiter) == (500.0, 5000.0, 80, 50)
    so = case.parse_solver_options(os.path.join(REF_TESTCASES, "visc-naca0012", "opts.solverc"))
    assert case._pc_kind(so) == "ilu0" and so.ksp_rtol == 0.1 and so.ksp_max_it == 30
