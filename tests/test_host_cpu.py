"""CPU-only checks: the CUDA library loads and exports its C ABI, the host
mesh module (topology, geometry, orderings, generators, Gmsh reader) agrees
with the oracle's restatement of the reference's UMesh, and the oracle's
solver converges on a small case."""
import os
import re

import numpy as np
import pytest

import fvens_gb300 as fv
from oracle import orc
from tests import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_REF = orc.reference_root()
REF_MESHES = os.path.join(_REF, "tests", "common-input") if _REF else ""


def test_library_exports_every_declared_symbol():
    L = fv.lib()
    hdr = open(os.path.join(ROOT, "include", "fvens_gb300.h")).read()
    names = set(re.findall(r"\b(fv_[a-z0-9_]+)\s*\(", hdr))
    assert len(names) > 30
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_abi_version_matches_header():
    hdr = open(os.path.join(ROOT, "include", "fvens_gb300.h")).read()
    v = int(re.search(r"#define FVENS_GB300_ABI_VERSION (\d+)", hdr).group(1))
    assert fv.lib().fv_abi_version() == v == fv.ABI_VERSION


def test_status_strings():
    L = fv.lib()
    for s in range(7):
        assert L.fv_status_string(s)


@pytest.mark.parametrize("mesh_fn,counts", [
    (lambda: fv.UMesh.generate(fv.MESH_CHANNEL_BUMP, [192, 64, 0.5, 1]), (18432, 512, 30464, 30976)),
    (lambda: fv.UMesh.generate(fv.MESH_NACA_OGRID, [512, 256, 30.0, 0, 0, 1.05, 154, 3]), (183296, 1024, 313856, 314880)),
])
def test_generator_counts(mesh_fn, counts):
    m = mesh_fn()
    assert (m.nelem, m.nbface, m.ninface, m.naface) == counts
    assert m.geometry()["area"].min() > 0


def _compare_topology(m):
    ex = m.export()
    om = orc.Mesh.from_export(ex)
    oa = om.arrays()
    g = m.geometry()
    assert (om.nelem, om.nbface, om.naface) == (m.nelem, m.nbface, m.naface)
    np.testing.assert_array_equal(g["area"], oa["area"])
    # boundary faces: same order, host cell and oriented normal (mesh.cpp:660-700)
    np.testing.assert_array_equal(g["face_lr"][:m.nbface, 0], oa["intfac"][:m.nbface, 0])
    np.testing.assert_array_equal(g["fnorm"][:m.nbface], oa["facemetric"][:m.nbface])
    # interior faces: same set, lower index on the left, same normals and lengths
    np.testing.assert_array_equal(g["face_lr"][m.nbface:], oa["intfac"][m.nbface:, :2])
    np.testing.assert_array_equal(g["fnorm"], oa["facemetric"])


def test_topology_matches_oracle_channel():
    _compare_topology(cases.channel(48, 16))


def test_topology_matches_oracle_naca():
    _compare_topology(cases.naca_visc())


def test_rcm_reduces_bandwidth():
    m0 = fv.UMesh.generate(fv.MESH_NACA_OGRID, [64, 32, 20.0, 0, 0, 1.1, 16, 3], reorder=0)
    m1 = fv.UMesh.generate(fv.MESH_NACA_OGRID, [64, 32, 20.0, 0, 0, 1.1, 16, 3], reorder=1)
    bw = lambda m: np.abs(np.diff(m.geometry()["face_lr"][m.nbface:], axis=1)).max()
    assert bw(m1) < bw(m0)
    perm = m1.export()["perm"]
    assert np.array_equal(np.sort(perm), np.arange(m1.nelem))


def test_colourings_are_proper():
    m = cases.channel(96, 32)
    g = m.geometry()
    fl = g["face_lr"][m.nbface:]
    assert np.all(g["color"][fl[:, 0]] != g["color"][fl[:, 1]])
    import ctypes
    order = np.zeros(m.nelem, np.int32)
    npart, ncol = ctypes.c_int(), ctypes.c_int()
    fv.check(fv.lib().fv_mesh_block_order(m._h, 64, fv._hp(order, ctypes.c_int), ctypes.byref(npart),
                                          ctypes.byref(ncol)))
    assert np.array_equal(np.sort(order), np.arange(m.nelem))
    assert npart.value >= m.nelem // 64 and ncol.value <= 8


def test_fewer_colour_part_colouring():
    """fv_mesh_block_order_ex colouring 1 (DSatur + Kempe interchanges): as
    many parts as the greedy colouring and 4 colours on the transonic NACA 0012
    O-grid where greedy needs 5 (the preconditioners in that order match the
    oracle's: test_gpu_linalg.py)."""
    import ctypes
    m = fv.UMesh.generate(fv.MESH_NACA_OGRID, [512, 256, 30.0, 0, 0, 1.02, 154, 3], reorder=1)
    res = {}
    for col in (0, 1):
        order = np.zeros(m.nelem, np.int32)
        npart, ncol = ctypes.c_int(), ctypes.c_int()
        fv.check(fv.lib().fv_mesh_block_order_ex(m._h, 128, col, fv._hp(order, ctypes.c_int), ctypes.byref(npart),
                                                 ctypes.byref(ncol)))
        assert np.array_equal(np.sort(order), np.arange(m.nelem))
        res[col] = (npart.value, ncol.value, order)
    assert res[0][0] == res[1][0] and (res[0][1], res[1][1]) == (5, 4)


@pytest.mark.skipif(not os.path.isdir(REF_MESHES), reason="reference test meshes not present")
@pytest.mark.parametrize("name", ["testperiodic.msh", "2dcylinderhybrid.msh", "testhybrid.msh"])
def test_gmsh_reader_on_reference_meshes(name):
    m = fv.UMesh.read_gmsh(os.path.join(REF_MESHES, name))
    assert m.nelem > 0 and m.geometry()["area"].min() > 0
    _compare_topology(m)


def _cell_edges(e, c):
    k = int(e["nnode"][c])
    nodes = e["inpoel"][c, :k]
    return {frozenset((int(nodes[j]), int(nodes[(j + 1) % k]))) for j in range(k)}


@pytest.mark.skipif(not os.path.isdir(REF_MESHES), reason="reference test meshes not present")
@pytest.mark.parametrize("name", ["2dcylinderhybrid.msh", "testhybrid.msh"])
def test_faces_belong_to_their_cells(name):
    """The reference's Mesh_Topology_FaceStructure / ElemSurrElem consistency
    checks (tests/mesh/mesh.cpp:14-64): every boundary face is an edge of its
    cell; every interior face is an edge shared by its two cells, and its unit
    normal is perpendicular to that edge, with the edge's length, pointing
    from the left cell to the right one."""
    m = fv.UMesh.read_gmsh(os.path.join(REF_MESHES, name))
    e, g = m.export(), m.geometry()
    xy, lr, fn = e["coords"], g["face_lr"], g["fnorm"]
    for f in range(m.nbface):
        assert frozenset(int(x) for x in e["bface"][f]) in _cell_edges(e, lr[f, 0])
    for f in range(m.nbface, m.naface):
        L, R = lr[f]
        assert 0 <= L < R < m.nelem
        shared = _cell_edges(e, L) & _cell_edges(e, R)
        assert len(shared) == 1
        a, b = sorted(next(iter(shared)))
        d = xy[b] - xy[a]
        assert abs(fn[f, 0] * d[0] + fn[f, 1] * d[1]) <= 1e-12 * fn[f, 2]
        assert abs(np.hypot(*d) - fn[f, 2]) <= 1e-12 * fn[f, 2]
        assert fn[f, 0] * (g["cc"][R, 0] - g["cc"][L, 0]) + fn[f, 1] * (g["cc"][R, 1] - g["cc"][L, 1]) > 0


REF_TESTCASES = os.path.join(_REF, "testcases") if _REF else ""


@pytest.mark.skipif(not os.path.isdir(REF_TESTCASES), reason="reference test cases not present")
def test_su2_reader_matches_gmsh_twin():
    """The reference ships the laminar NACA 0012 hybrid mesh in both formats:
    the SU2 reader (meshreaders.cpp:267-397) must give the same cells,
    boundary faces and markers as the Gmsh reader."""
    base = os.path.join(REF_TESTCASES, "visc-naca0012", "grids", "NACA0012_lam_hybrid_1")
    a = fv.UMesh.read(base + ".su2")
    b = fv.UMesh.read(base + ".msh")
    assert (a.nelem, a.nbface, a.npoin) == (b.nelem, b.nbface, b.npoin)
    ga, gb = a.geometry(), b.geometry()
    assert abs(ga["area"].sum() - gb["area"].sum()) <= 1e-12 * gb["area"].sum()
    ea, eb = a.export(), b.export()
    assert sorted(np.bincount(ea["btag"]).tolist()) == sorted(np.bincount(eb["btag"]).tolist())
    _compare_topology(a)


@pytest.mark.skipif(not os.path.isdir(REF_TESTCASES), reason="reference test cases not present")
def test_su2_reader_inviscid_naca_mesh():
    m = fv.UMesh.read(os.path.join(REF_TESTCASES, "naca0012", "grids", "NACA0012_inv.su2"), reorder=1)
    e = m.export()
    assert m.nelem == 10216 and m.npoin == 5233 and m.nbface == 250
    assert sorted(set(e["btag"].tolist())) == [2, 4]
    assert m.geometry()["area"].min() > 0
    _compare_topology(m)


def test_mesh_reader_rejects_unknown_extension(tmp_path):
    p = tmp_path / "mesh.vtu"
    p.write_text("x")
    with pytest.raises(fv.FvensError):
        fv.UMesh.read(str(p))


def test_oracle_solves_small_channel():
    m = cases.channel(24, 8)
    od = orc.Disc(orc.Mesh.from_export(m.export()), Minf=0.5, flux="ROE", gradient="LEASTSQUARES",
                  bcs=cases.CHANNEL_BCS)
    u0 = np.tile(od.freestream(), (m.nelem, 1))
    u, st = od.steady_solve(u0, cflmin=10, cflmax=1000, tol=1e-10, maxiter=200, pc="ilu0")
    assert st["status"] == 0 and st["res"] <= 1e-10
    r, _ = od.residual(u)
    assert np.sqrt((r[:, 3] ** 2 * m.geometry()["area"]).sum()) < 1e-9


def test_oracle_kernel_timings():
    """The CPU baseline's per-kernel timings: every kernel timed, positive,
    and the timing leaves the oracle's results unchanged."""
    m = cases.channel(24, 8)
    od = orc.Disc(orc.Mesh.from_export(m.export()), Minf=0.5, flux="ROE", gradient="LEASTSQUARES",
                  bcs=cases.CHANNEL_BCS)
    u = np.tile(od.freestream(), (m.nelem, 1)) * (1 + 1e-3 * np.random.default_rng(1).normal(size=(m.nelem, 4)))
    r0, _ = od.residual(u)
    t = od.time_kernels(u, "ilu0", reps=3)
    assert set(t) == {"residual", "jacobian", "pc_setup", "pc_apply"} and all(v > 0 for v in t.values())
    assert np.array_equal(od.residual(u)[0], r0)
    with pytest.raises(RuntimeError):
        od.time_kernels(u, "ilu0", reps=0)


def test_oracle_precond_exact_for_block_diagonal():
    """ILU(0), SGS and Jacobi all invert a block-diagonal matrix exactly."""
    rng = np.random.default_rng(0)
    n = 20
    rp = np.arange(n + 1, dtype=np.int32)
    col = np.arange(n, dtype=np.int32)
    blocks = [np.eye(4) * 3 + rng.normal(0, 0.3, (4, 4)) for _ in range(n)]
    val = np.array([b.ravel() for b in blocks])
    r = rng.normal(size=4 * n)
    for kind in ("jacobi", "sgs", "ilu0"):
        z = orc.precond_apply(rp, col, val, kind, r)
        for i in range(n):
            np.testing.assert_allclose(blocks[i] @ z[4 * i:4 * i + 4], r[4 * i:4 * i + 4], atol=1e-12)


CPP_DRIVER = r"""
#include <cstdio>
#include <vector>
#include "fvens_gb300.hpp"
// A host program written against the reference-shaped C++ interface: mesh,
// FlowFV, Jacobian and steady solver objects.  Built and linked here; it only
// runs the CUDA parts where a GPU exists.
int main(int argc, char **argv)
{
	try {
		fvg::Mesh m = fvg::Mesh::generate(FV_MESH_CHANNEL_BUMP, {24, 8, 0.5, 1});
		std::printf("%d %d %d\n", m.gnelem(), m.gnbface(), m.gnaface());
		if (argc < 2) return 0;  // no GPU work requested
		fv_physics_cfg ph = {1.4, 0.5, 288.15, 1e300, 0.72, 0.0, 0, 0};
		fv_numerics_cfg nu = {FV_FLUX_ROE, FV_FLUX_ROE, FV_GRAD_LEASTSQUARES, FV_REC_NONE, 0.0, 1};
		std::vector<fv_bc_cfg> bcs = {{1, FV_BC_SLIPWALL, {0, 0}}, {2, FV_BC_INFLOW_OUTFLOW, {0, 0}},
		                              {3, FV_BC_SLIPWALL, {0, 0}}, {4, FV_BC_INFLOW_OUTFLOW, {0, 0}}};
		fvg::FlowFV flow(m, {ph}, nu, bcs);
		fv_solver_cfg cfg;
		fv_solver_cfg_default(&cfg);
		fvg::SteadyBackwardEulerSolver solver(flow, cfg);
		std::vector<double> u;
		const std::vector<double> uinf = flow.freestream();
		for (int i = 0; i < m.gnelem(); i++) u.insert(u.end(), uinf.begin(), uinf.end());
		const auto st = solver.solve_host(u);
		std::printf("%d %g\n", st[0].steps, st[0].res);
	} catch (const std::exception &e) {
		std::printf("error: %s\n", e.what());
		return 1;
	}
	return 0;
}
"""


def test_cpp_interface_builds_and_links(tmp_path):
    """include/fvens_gb300.hpp (the C++ layer with the reference's class
    names) compiles against the C ABI and links against the library; the
    mesh part runs without a GPU."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("no g++")
    src = tmp_path / "driver.cpp"
    src.write_text(CPP_DRIVER)
    exe = tmp_path / "driver"
    libdir = os.path.dirname(fv.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-lfvens_gb300", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    m = fv.UMesh.generate(fv.MESH_CHANNEL_BUMP, [24, 8, 0.5, 1])
    assert [int(x) for x in out[:3]] == [m.nelem, m.nbface, m.naface]


@pytest.mark.skipif(not os.path.isdir(REF_MESHES), reason="reference test meshes not present")
def test_periodic_map_on_reference_mesh():
    """tests/mesh/mesh.cpp:test_periodic_map: on testperiodic.msh, marker 4,
    axis 0, boundary faces 8..12 pair with 25..21."""
    import ctypes
    m = fv.UMesh.read_gmsh(os.path.join(REF_MESHES, "testperiodic.msh"))
    pm = np.zeros(m.nbface, np.int32)
    fv.check(fv.lib().fv_mesh_periodic_map(m._h, 4, 0, fv._hp(pm, ctypes.c_int)))
    for a, b in zip([8, 9, 10, 11, 12], [25, 24, 23, 22, 21]):
        assert pm[a] == b and pm[b] == a
    e = m.export()
    assert np.all(pm[e["btag"] != 4] == -1)


def test_find_lines_on_boundary_layer_mesh():
    """findLines (meshordering.cpp:208-262) on the reference's laminar hybrid
    mesh: lines start at boundary cells, follow face neighbours, and every
    step's weight (1/distance over the cell's smallest) exceeds the threshold."""
    from tests import regression_cases as rc
    m, c, regr = rc.load("laminar_naca0012_hybrid1")
    nl, cl = m.find_lines(10.0)
    assert nl > 100
    g = m.geometry()
    cc = g["cc"]
    lr = g["face_lr"]
    nbrs = {}
    for a, b in lr[m.nbface:]:
        nbrs.setdefault(a, set()).add(b)
        nbrs.setdefault(b, set()).add(a)
    wall_cells = set(lr[:m.nbface, 0].tolist())
    for k in range(nl):
        cells = np.where(cl == k)[0]
        assert len(cells) >= 2
    # the cells of one line form a connected chain
    k = int(cl[cl >= 0][0])
    members = set(np.where(cl == k)[0].tolist())
    assert any(x in wall_cells for x in members)
    degree = [len(nbrs[x] & members) for x in members]
    assert max(degree) <= 2 and degree.count(1) == 2
    # no lines on an isotropic mesh
    assert cases.channel(24, 8).find_lines(10.0)[0] == 0
    # threshold <= 0 removes them
    assert m.find_lines(0.0)[0] == 0


def test_hybrid_naca_generator_quality():
    """FV_MESH_NACA_HYBRID at the 400k-cell laminar configuration: 48 quad
    boundary-layer rings from 1e-4 chords (growth 1.12) and near-isotropic
    outer triangles to 20 chords -- every cell positive, no triangle angle
    under 1 degree and fewer than 0.3 % under 10 degrees (the trailing-edge
    fan), far-field nodes at >= 20 chords."""
    m = fv.UMesh.generate(fv.MESH_NACA_HYBRID, [512, 48, 1e-4, 1.12, 20.0, 0.5], reorder=0)
    ex, g = m.export(), m.geometry()
    assert m.nelem == 381952 and int((ex["nnode"] == 4).sum()) == 512 * 48
    assert g["area"].min() > 0
    X, P = ex["coords"], ex["inpoel"]
    tri = P[ex["nnode"] == 3][:, :3]
    pts = X[tri]
    ang = []
    for j in range(3):
        v1, v2 = pts[:, (j + 1) % 3] - pts[:, j], pts[:, (j - 1) % 3] - pts[:, j]
        c = (v1 * v2).sum(1) / np.linalg.norm(v1, axis=1) / np.linalg.norm(v2, axis=1)
        ang.append(np.degrees(np.arccos(np.clip(c, -1, 1))))
    amin = np.min(ang, axis=0)
    assert amin.min() > 1.0 and (amin < 10.0).sum() < 0.003 * len(amin)
    far = ex["bface"][ex["btag"] == 4].ravel()
    assert np.hypot(X[far, 0] - 0.5, X[far, 1]).min() >= 20.0
    with pytest.raises(fv.FvensError):
        fv.UMesh.generate(fv.MESH_NACA_HYBRID, [512, 48, 1e-4, 1.12, 20.0, 1.5])


_SQ = [[0, 0], [1, 0], [0, 1], [1, 1]]


def _mesh(coords, nnode, inpoel, bface, btag):
    return fv.UMesh.from_arrays(np.array(coords, float), np.array(nnode, np.int32), np.array(inpoel, np.int32),
                                np.array(bface, np.int32), np.array(btag, np.int32))


def test_smallest_meshes_and_orientation():
    """One triangle (all faces on the boundary), a clockwise triangle (flipped,
    as preprocessMesh does), two triangles sharing one interior face."""
    m = _mesh(_SQ[:3], [3], [[0, 1, 2, -1]], [[0, 1], [1, 2], [2, 0]], [1, 1, 1])
    assert (m.nelem, m.nbface, m.naface) == (1, 3, 3) and m.geometry()["area"][0] == 0.5
    m = _mesh(_SQ[:3], [3], [[0, 2, 1, -1]], [[0, 1], [1, 2], [2, 0]], [1, 1, 1])
    assert m.geometry()["area"][0] == 0.5
    m = _mesh(_SQ, [3, 3], [[0, 1, 3, -1], [0, 3, 2, -1]], [[0, 1], [1, 3], [3, 2], [2, 0]], [1, 1, 1, 1])
    assert (m.nelem, m.nbface, m.naface) == (2, 4, 5)


@pytest.mark.parametrize("coords,nnode,inpoel,bface,what", [
    (_SQ, [3, 3], [[0, 1, 3, -1], [0, 3, 2, -1]], [[0, 1], [1, 3], [3, 2]], "number of boundary faces"),
    (_SQ, [3, 3], [[0, 1, 3, -1], [0, 3, 2, -1]], [[0, 1], [1, 3], [3, 2], [2, 1]], "not an edge"),
    ([[0, 0], [1, 0], [2, 0]], [3], [[0, 1, 2, -1]], [[0, 1], [1, 2], [2, 0]], "non-positive area"),
    (_SQ, [3, 3], [[0, 1, 3, -1], [0, 3, 7, -1]], [[0, 1], [1, 3], [3, 2], [2, 0]], "out of range"),
    ([[0, 0], [1, 0], [0.5, 1], [0.5, -1], [0.5, 0.5]], [3, 3, 3],
     [[0, 1, 2, -1], [0, 3, 1, -1], [0, 1, 4, -1]], [[1, 2], [2, 0], [0, 3], [3, 1], [1, 4], [4, 0]],
     "non-manifold"),
    (_SQ, [5], [[0, 1, 3, 2]], [[0, 1], [1, 3], [3, 2], [2, 0]], "triangles and quadrilaterals"),
], ids=["missing_boundary_face", "stray_boundary_face", "degenerate_cell", "bad_node_index", "non_manifold_edge",
        "bad_cell_kind"])
def test_invalid_meshes_are_rejected(coords, nnode, inpoel, bface, what):
    with pytest.raises(fv.FvensError, match=what) as e:
        _mesh(coords, nnode, inpoel, bface, [1] * len(bface))
    assert e.value.status == fv.FV_ERR_MESH


def test_disc_and_network_argument_checks():
    """Argument checks that return before any device work: no batch members,
    an unknown scheme index, the periodic BC (not implemented by the
    reference's flow discretisation), a boundary marker without a BC, and a
    warm-start network without layers."""
    import ctypes
    m = cases.channel(8, 4)
    num = fv.numerics_cfg(flux="ROE")
    with pytest.raises(fv.FvensError) as e:
        fv.FlowFV(m, [], num, cases.CHANNEL_BCS)
    assert e.value.status == fv.FV_ERR_INVALID
    bad = fv.numerics_cfg(flux="ROE")
    bad.conv_numflux = 9
    with pytest.raises(fv.FvensError) as e:
        fv.FlowFV(m, fv.physics_cfg(Minf=0.5), bad, cases.CHANNEL_BCS)
    assert e.value.status == fv.FV_ERR_INVALID
    with pytest.raises(fv.FvensError) as e:
        fv.FlowFV(m, fv.physics_cfg(Minf=0.5), num, [(1, "periodic", ())] + cases.CHANNEL_BCS[1:])
    assert e.value.status == fv.FV_ERR_UNSUPPORTED
    with pytest.raises(fv.FvensError, match="no boundary condition for boundary marker 4") as e:
        fv.FlowFV(m, fv.physics_cfg(Minf=0.5), num, cases.CHANNEL_BCS[:3])
    assert e.value.status == fv.FV_ERR_INVALID
    h = ctypes.c_void_p()
    assert fv.lib().fv_mpnn_create(m._h, 0, None, 0, ctypes.c_ulonglong(1), ctypes.byref(h)) == fv.FV_ERR_INVALID


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_MESHES, "testanisotropic-lines.txt")),
                    reason="reference test inputs not present")
def test_find_lines_matches_reference_golden_lines():
    """tests/mesh/testlineordering.cpp (MeshUtils_findLines_smallmesh): on
    testanisotropic.msh with threshold 10 the lines are the cells of
    testanisotropic-lines.txt (Gmsh element numbers, boundary elements first)."""
    m = fv.UMesh.read_gmsh(os.path.join(REF_MESHES, "testanisotropic.msh"), reorder=0)
    nl, cl = m.find_lines(10.0)
    gold = [[int(c) - m.nbface - 1 for c in ln.split()]
            for ln in open(os.path.join(REF_MESHES, "testanisotropic-lines.txt")) if ln.strip()]
    assert nl == len(gold)
    for k, cells in enumerate(gold):
        assert [int(cl[c]) for c in cells] == [k] * len(cells)
    assert int((cl >= 0).sum()) == sum(len(g) for g in gold)


@pytest.mark.skipif(not os.path.isdir(REF_MESHES), reason="reference test meshes not present")
def test_line_ordering_matches_reference_golden_ordering():
    """tests/mesh/testhybridlineordering.cpp (MeshUtils_hybridLineOrdering_{natural,rcm}_smallmesh):
    on testanisotropic.msh with threshold 10 the hybrid line orderings are
    testanisotropic-lineordering.txt and testanisotropic-line_rcm_ordering.txt
    (Gmsh element numbers, boundary elements first).  Without lines the
    natural ordering is the identity."""
    m = fv.UMesh.read_gmsh(os.path.join(REF_MESHES, "testanisotropic.msh"), reorder=0)
    assert np.array_equal(m.line_ordering(), np.arange(m.nelem))
    m.find_lines(10.0)
    for rcm, name in ((False, "testanisotropic-lineordering.txt"), (True, "testanisotropic-line_rcm_ordering.txt")):
        with open(os.path.join(REF_MESHES, name)) as f:
            gold = [int(c) - m.nbface - 1 for c in f.read().split()]
        assert m.line_ordering(rcm).tolist() == gold, name
    # a boundary-layer O-grid, with and without lines: permutations of its cells
    big = cases.naca_visc()
    for thr in (0.0, 10.0):
        big.find_lines(thr)
        for rcm in (False, True):
            assert np.array_equal(np.sort(big.line_ordering(rcm)), np.arange(big.nelem))
