"""Synthetic workload meshes built from mesh arrays (numpy, host side).

refine(): uniform refinement of a hybrid 2-D mesh, the rule by which the
reference's NACA0012_lam_hybrid_2.msh is made from NACA0012_lam_hybrid_1.msh
(testcases/visc-naca0012/grids/): a node at the midpoint of every edge
(boundary edges included, with no projection onto the surface), a node at the
mean of the corners of every quadrilateral; each triangle becomes four
triangles (three corner triangles and the middle one), each quadrilateral four
quadrilaterals, each boundary face two.  Children keep their parent's
orientation and sit at positions 4 i .. 4 i + 3 of the refined cell list.

Mesh arrays are the dict that UMesh.export() returns and UMesh.from_arrays()
takes: coords (npoin x 2), nnode (nelem), inpoel (nelem x 4, -1 padded),
bface (nbface x 2), btag (nbface).
"""
import numpy as np


def refine(mesh, levels=1):
    """The mesh refined `levels` times (see the module docstring)."""
    for _ in range(levels):
        mesh = _refine_once(mesh)
    return mesh


def _refine_once(mesh):
    coords = np.asarray(mesh["coords"], np.float64)
    nnode = np.asarray(mesh["nnode"], np.int64)
    inpoel = np.asarray(mesh["inpoel"], np.int64)
    bface = np.asarray(mesh["bface"], np.int64)
    btag = np.asarray(mesh["btag"])
    npoin, nelem = len(coords), len(nnode)
    # local edges j = (corner j, corner j + 1) of every cell
    a = inpoel[:, :4]
    b = np.where(np.arange(4)[None, :] + 1 < nnode[:, None], np.roll(a, -1, axis=1), a[:, :1])
    valid = np.arange(4)[None, :] < nnode[:, None]
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    keys = np.where(valid, lo * npoin + hi, -1)
    uniq, inv = np.unique(keys[valid], return_inverse=True)
    nedge = len(uniq)
    emid = np.full((nelem, 4), -1, np.int64)
    emid[valid] = npoin + inv
    el, eh = uniq // npoin, uniq % npoin
    mids = 0.5 * (coords[el] + coords[eh])
    quad = nnode == 4
    qidx = np.cumsum(quad) - 1
    centre = np.full(nelem, -1, np.int64)
    centre[quad] = npoin + nedge + qidx[quad]
    qc = coords[inpoel[quad]].mean(axis=1)
    new_coords = np.vstack([coords, mids, qc])
    # children
    out = np.full((nelem, 4, 4), -1, np.int64)
    c0, c1, c2, c3 = (inpoel[:, k] for k in range(4))
    m0, m1, m2, m3 = (emid[:, k] for k in range(4))
    t = ~quad
    # triangle (c0, c1, c2), midpoints m0 = c0c1, m1 = c1c2, m2 = c2c0
    out[t, 0, :3] = np.stack([c0, m0, m2], 1)[t]
    out[t, 1, :3] = np.stack([m0, c1, m1], 1)[t]
    out[t, 2, :3] = np.stack([m2, m1, c2], 1)[t]
    out[t, 3, :3] = np.stack([m0, m1, m2], 1)[t]
    # quadrilateral (c0, c1, c2, c3), midpoints m0..m3 of edges 01, 12, 23, 30, centre o
    o = centre
    out[quad, 0] = np.stack([c0, m0, o, m3], 1)[quad]
    out[quad, 1] = np.stack([m0, c1, m1, o], 1)[quad]
    out[quad, 2] = np.stack([o, m1, c2, m2], 1)[quad]
    out[quad, 3] = np.stack([m3, o, m2, c3], 1)[quad]
    new_nnode = np.repeat(nnode, 4)
    # boundary faces: (p, q) -> (p, m), (m, q)
    blo, bhi = np.minimum(bface[:, 0], bface[:, 1]), np.maximum(bface[:, 0], bface[:, 1])
    pos = np.searchsorted(uniq, blo * npoin + bhi)
    if np.any(pos >= nedge) or np.any(uniq[np.minimum(pos, nedge - 1)] != blo * npoin + bhi):
        raise ValueError("a boundary face is not an edge of any cell")
    bm = npoin + pos
    new_bface = np.stack([np.stack([bface[:, 0], bm], 1), np.stack([bm, bface[:, 1]], 1)], 1).reshape(-1, 2)
    return dict(coords=new_coords, nnode=new_nnode.astype(np.int32), inpoel=out.reshape(-1, 4).astype(np.int32),
                bface=new_bface.astype(np.int32), btag=np.repeat(btag, 2).astype(np.int32))


def _progression(length, npoints, ratio):
    """npoints positions from 0 to length whose successive spacings grow by
    `ratio` (Gmsh's "Using Progression")."""
    seg = ratio ** np.arange(npoints - 1, dtype=np.float64)
    return length * np.concatenate([[0.0], np.cumsum(seg)]) / seg.sum()


def flat_plate_stretched(levels=0):
    """The structured laminar flat-plate mesh of the reference's
    testcases/visc-flatplate/grids/flatplatestructstretched.geo (refinement
    factor 2), refined `levels` times as its RefineMesh steps do (levels 0, 1,
    2 are flatplatestructstretched0/1/2.msh).  Domain [-0.5, 1] x [0, 1] in
    two transfinite blocks of quadrilaterals: ahead of the plate 10 points in
    x with spacing growing by 1.2 away from the leading edge, on the plate 20
    points growing by 1.1 from it, 20 points in y growing by 1.4 from the
    wall.  Markers: 2 the plate (0 <= x <= 1, y = 0), 3 the symmetry line
    ahead of it, 4 the inflow and top sides, 5 the outflow side (x = 1)."""
    ref = 2
    nxi, nxp, ny = 5 * ref, 10 * ref, 10 * ref
    xs = np.concatenate([-_progression(0.5, nxi, 1.2)[::-1], _progression(1.0, nxp, 1.1)[1:]])
    ys = _progression(1.0, ny, 1.4)
    nx = len(xs)
    X, Y = np.meshgrid(xs, ys)
    coords = np.stack([X.ravel(), Y.ravel()], 1)
    node = lambda i, j: j * nx + i
    I, J = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1))
    I, J = I.ravel(), J.ravel()
    inpoel = np.stack([node(I, J), node(I + 1, J), node(I + 1, J + 1), node(I, J + 1)], 1)
    i = np.arange(nx - 1)
    j = np.arange(ny - 1)
    bface = np.concatenate([np.stack([node(i, 0), node(i + 1, 0)], 1),
                            np.stack([node(nx - 1, j), node(nx - 1, j + 1)], 1),
                            np.stack([node(i + 1, ny - 1), node(i, ny - 1)], 1),
                            np.stack([node(0, j + 1), node(0, j)], 1)])
    btag = np.concatenate([np.where(xs[1:] <= 0.0, 3, 2), np.full(ny - 1, 5), np.full(nx - 1, 4),
                           np.full(ny - 1, 4)])
    mesh = dict(coords=coords, nnode=np.full(len(inpoel), 4, np.int32), inpoel=inpoel.astype(np.int32),
                bface=bface.astype(np.int32), btag=btag.astype(np.int32))
    return refine(mesh, levels)
