"""Workload meshes.  The oracle-side O-grid generator (oracle/meshgen.py),
used by the CPU baseline and the reference arm of bench.py, builds the same
mesh as the product's generator: nodes to rounding, identical cells and
boundary faces, and an oracle mesh with the same face metrics.  The uniform
refinement (fvens_gb300/meshes.py) that makes the laminar hybrid workload
mesh reproduces the reference's own level-2 hybrid NACA 0012 mesh."""
import os

import numpy as np
import pytest

import fvens_gb300 as fv
from fvens_gb300 import meshes
from oracle import meshgen, orc


@pytest.mark.parametrize("params", [
    [128, 96, 20.0, 24, 1e-4, 1.12, 60, 5],     # boundary-layer block, triangulated outer rings
    [96, 48, 30.0, 0, 0.0, 1.02, 29, 3],        # geometric rings (the benchmark's family, smaller)
])
def test_oracle_ogrid_matches_product_generator(params):
    g = meshgen.naca_ogrid(*params)
    e = fv.UMesh.generate(fv.MESH_NACA_OGRID, params, reorder=0).export()
    scale = np.abs(e["coords"]).max()
    assert np.abs(g["coords"] - e["coords"]).max() <= 1e-14 * scale
    assert np.array_equal(g["nnode"], e["nnode"]) and np.array_equal(g["inpoel"], e["inpoel"])
    # the product orients wall faces when it builds the mesh; compare as node sets
    key = lambda b, t: sorted((min(x), max(x), int(tt)) for x, tt in zip(b, t))
    assert key(g["bface"], g["btag"]) == key(e["bface"], e["btag"])
    om_g = orc.Mesh(**g)
    om_e = orc.Mesh.from_export(e)
    a, b = om_g.arrays(), om_e.arrays()
    assert (om_g.nelem, om_g.naface, om_g.nbface) == (om_e.nelem, om_e.naface, om_e.nbface)
    assert np.allclose(a["area"], b["area"], rtol=1e-12, atol=0)
    assert np.allclose(a["facemetric"], b["facemetric"], rtol=1e-12, atol=1e-15)


def test_benchmark_ogrid_counts():
    g = meshgen.naca_ogrid(512, 256, 30.0, 0, 0.0, 1.02, 154, 3)
    assert (len(g["nnode"]), len(g["coords"]), len(g["btag"])) == (183296, 131584, 1024)


_REF = orc.reference_root()
_HYB = "testcases/visc-naca0012/grids/NACA0012_lam_hybrid_{}.msh"


@pytest.mark.skipif(not (_REF and os.path.exists(os.path.join(_REF, _HYB.format(2)))),
                    reason="reference meshes not present")
def test_refinement_reproduces_reference_level_2_hybrid_mesh():
    """meshes.refine of the reference's NACA0012_lam_hybrid_1 gives its
    NACA0012_lam_hybrid_2: the same nodes (to rounding), cells and boundary
    faces (with markers)."""
    from scipy.spatial import cKDTree
    m1 = fv.UMesh.read_gmsh(os.path.join(_REF, _HYB.format(1)), reorder=0).export()
    m2 = fv.UMesh.read_gmsh(os.path.join(_REF, _HYB.format(2)), reorder=0).export()
    r = meshes.refine(m1)
    assert (len(r["nnode"]), len(r["coords"]), len(r["btag"])) == (len(m2["nnode"]), len(m2["coords"]),
                                                                    len(m2["btag"]))
    d, idx = cKDTree(m2["coords"]).query(r["coords"])
    assert d.max() <= 1e-14 and len(np.unique(idx)) == len(idx)

    def canon(nn, el):
        el = [int(x) for x in el[:nn]]
        k = el.index(min(el))
        return tuple(el[k:] + el[:k])
    assert {canon(n, idx[e]) for n, e in zip(r["nnode"], r["inpoel"])} == \
        {canon(n, e) for n, e in zip(m2["nnode"], m2["inpoel"])}
    bf = lambda b, t, f: {(min(f[x], f[y]), max(f[x], f[y]), int(tt)) for (x, y), tt in zip(b, t)}
    assert bf(r["bface"], r["btag"], idx) == bf(m2["bface"], m2["btag"], np.arange(len(m2["coords"])))


def test_refined_hybrid_mesh_builds():
    """Two refinements of the committed level-1 hybrid mesh (210,496 cells, the
    batched laminar workload's mesh): counts, positive areas, and the total
    area kept."""
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "naca0012_lam_hybrid_1_mesh.npz"))
    m1 = dict(coords=z["coords"], nnode=z["nnode"], inpoel=z["inpoel"], bface=z["bface"], btag=z["btag"])
    base = fv.UMesh.from_arrays(z["coords"], z["nnode"].astype(np.int32), z["inpoel"], z["bface"],
                                z["btag"].astype(np.int32), reorder=0)
    r = meshes.refine(m1, 2)
    m = fv.UMesh.from_arrays(r["coords"], r["nnode"], r["inpoel"], r["bface"], r["btag"], reorder=1)
    assert (m.nelem, m.nbface) == (16 * base.nelem, 4 * base.nbface)
    a, a0 = m.geometry()["area"], base.geometry()["area"]
    assert a.min() > 0 and abs(a.sum() - a0.sum()) <= 1e-12 * a0.sum()


def test_laminar_fixture_samples_the_refined_mesh():
    """The oracle's converged-solve fixture of the laminar workload: solved to
    1e-12, its sampled cells are cells of the twice-refined mesh in the
    refinement's numbering and include every cell touching the wall, and the
    sampled states are physical (positive density and energy)."""
    here = os.path.dirname(os.path.abspath(__file__))
    f = np.load(os.path.join(here, "golden", "naca0012_laminar_l2_oracle_converged.npz"))
    z = np.load(os.path.join(here, "golden", "naca0012_lam_hybrid_1_mesh.npz"))
    r = meshes.refine(dict(coords=z["coords"], nnode=z["nnode"], inpoel=z["inpoel"], bface=z["bface"],
                           btag=z["btag"]), 2)
    nelem = len(r["nnode"])
    assert float(f["tolerance"]) == 1e-12 and list(f["members"]) == [0, 1, 4]
    cells = f["cells"]
    assert cells.min() >= 0 and cells.max() < nelem and len(np.unique(cells)) == len(cells)
    wall_nodes = np.unique(r["bface"][r["btag"] == 2])
    near_wall = np.where(np.isin(r["inpoel"], wall_nodes).any(axis=1))[0]
    assert np.isin(near_wall, cells).all()
    u = f["states"]
    assert u.shape == (3, len(cells), 4) and (u[..., 0] > 0).all() and (u[..., 3] > 0).all()
    assert (f["solve_counts"][:, 2] > 0).all() and np.isfinite(f["functionals"]).all()
