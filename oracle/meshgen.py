"""ORACLE (test infrastructure only): the benchmark's NACA 0012 O-grid,
generated in numpy without the product library, so that the CPU baseline and
the reference arm of bench.py build their mesh on the oracle side alone.

The grid is the workload's definition, not a reference algorithm (the
reference reads Gmsh meshes).  It is restated here from its description:

  * airfoil: nc points at theta_i = 2 pi i / nc, x = (1 + cos theta) / 2, on
    the closed-trailing-edge NACA 0012 thickness y_t(x) = 0.6 (0.2969 sqrt x
    - 0.1260 x - 0.3516 x^2 + 0.2843 x^3 - 0.1036 x^4), upper surface for
    0 < i < nc / 2, y = 0 at i = 0 and i = nc / 2;
  * outward normals by central differences, smoothed four times with the
    weights (1/4, 1/2, 1/4) and renormalised;
  * far-field angle of column i: half the normal's (unwrapped) angle plus
    half theta_i, on a circle of radius rfar about mid-chord;
  * ring distances: geometric with ratio g from the wall to rfar - 1/2 (no
    boundary-layer block), or nbl rings h0 g^k followed by a geometric
    outer block fitted by bisection and rescaled to end at rfar - 1/2;
  * ring k: the normal offset d_k blended into the straight line to the far
    field with a smoothstep weight over the first two chords;
  * cells: quads below ring tri_from, above it each quad split into two
    triangles along the diagonal chosen by the low bit of a splitmix64 stream
    seeded with `seed`;
  * boundary faces: the wall ring (marker 2), then the far-field ring
    (marker 4).

tests/test_meshgen_cpu.py checks it against the product's generator (the
same nodes to 1e-13, the same cells and boundary faces).
"""
import numpy as np

_M64 = (1 << 64) - 1


def _splitmix64_stream(seed, n):
    """n successive outputs of splitmix64 (Steele, Lea and Flood 2014)."""
    out = np.empty(n, dtype=np.uint64)
    s = int(seed) & _M64
    for k in range(n):
        s = (s + 0x9E3779B97F4A7C15) & _M64
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        out[k] = z ^ (z >> 31)
    return out


def _thickness(x):
    x = np.maximum(x, 0.0)
    return 0.6 * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x * x + 0.2843 * x * x * x - 0.1036 * x * x * x * x)


def _ring_distances(nr, rfar, nbl, h0, g):
    D = rfar - 0.5
    d = np.zeros(nr + 1)
    if nbl <= 0:
        hh = D * (g - 1.0) / (g ** nr - 1.0)
        for k in range(1, nr + 1):
            d[k] = d[k - 1] + hh * g ** (k - 1)
        return d
    for k in range(1, nbl + 1):
        d[k] = d[k - 1] + h0 * g ** (k - 1)
    hl = h0 * g ** (nbl - 1)
    no = nr - nbl
    lo, hi = 1.0 + 1e-12, 2.0
    for _ in range(200):
        gm = 0.5 * (lo + hi)
        if d[nbl] + hl * gm * (gm ** no - 1.0) / (gm - 1.0) > D:
            hi = gm
        else:
            lo = gm
    g2 = 0.5 * (lo + hi)
    for k in range(nbl + 1, nr + 1):
        d[k] = d[k - 1] + hl * g2 ** (k - nbl)
    sc = (D - d[nbl]) / (d[nr] - d[nbl])
    d[nbl + 1:] = d[nbl] + (d[nbl + 1:] - d[nbl]) * sc
    return d


def naca_ogrid(nc, nr, rfar, nbl, h0, g, tri_from, seed):
    """Arrays (coords, nnode, inpoel, bface, btag) of the O-grid, cells ring by
    ring (the generator's own order; the oracle does not reorder)."""
    i = np.arange(nc)
    th = 2.0 * np.pi * i / nc
    px = 0.5 * (1.0 + np.cos(th))
    yt = _thickness(px)
    py = np.where((i == 0) | (2 * i == nc), 0.0, np.where(2 * i < nc, yt, -yt))
    tx = np.roll(px, -1) - np.roll(px, 1)
    ty = np.roll(py, -1) - np.roll(py, 1)
    ln = np.sqrt(tx * tx + ty * ty)
    nx, ny = ty / ln, -tx / ln
    for _ in range(4):
        ax = 0.5 * nx + 0.25 * (np.roll(nx, -1) + np.roll(nx, 1))
        ay = 0.5 * ny + 0.25 * (np.roll(ny, -1) + np.roll(ny, 1))
        ln = np.sqrt(ax * ax + ay * ay)
        nx, ny = ax / ln, ay / ln
    phi = np.zeros(nc)
    prev = 0.0
    for k in range(nc):
        a = float(np.arctan2(ny[k], nx[k]))
        while a < prev - np.pi:
            a += 2 * np.pi
        while a > prev + np.pi:
            a -= 2 * np.pi
        if k == 0:
            a = 0.0
        prev = a
        phi[k] = 0.5 * a + 0.5 * th[k]
    d = _ring_distances(nr, rfar, nbl, h0, g)
    D = rfar - 0.5
    qx, qy = 0.5 + rfar * np.cos(phi), rfar * np.sin(phi)
    coords = np.empty((nr + 1, nc, 2))
    for k in range(nr + 1):
        s = d[k] / D
        t = min(1.0, d[k] / 2.0)
        w = 1.0 if k == nr else t * t * (3.0 - 2.0 * t)
        ax, ay = px + d[k] * nx, py + d[k] * ny
        bx, by = px + s * (qx - px), py + s * (qy - py)
        coords[k, :, 0] = (1 - w) * ax + w * bx
        coords[k, :, 1] = (1 - w) * ay + w * by
    node = lambda ii, kk: kk * nc + (ii % nc)
    ntri_rings = max(nr - tri_from, 0)
    bits = _splitmix64_stream(seed, ntri_rings * nc) & np.uint64(1)
    nnode, inpoel = [], []
    q = 0
    for k in range(nr):
        for ii in range(nc):
            a, b, c, e = node(ii, k), node(ii, k + 1), node(ii + 1, k + 1), node(ii + 1, k)
            if k < tri_from:
                nnode.append(4)
                inpoel.append((a, b, c, e))
            elif bits[q]:
                nnode += [3, 3]
                inpoel += [(a, b, c, -1), (a, c, e, -1)]
            else:
                nnode += [3, 3]
                inpoel += [(a, b, e, -1), (b, c, e, -1)]
            if k >= tri_from:
                q += 1
    bface = [(node(ii, 0), node(ii + 1, 0)) for ii in range(nc)] + \
            [(node(ii, nr), node(ii + 1, nr)) for ii in range(nc)]
    btag = [2] * nc + [4] * nc
    return dict(coords=coords.reshape(-1, 2), nnode=np.array(nnode, np.int32), inpoel=np.array(inpoel, np.int32),
                bface=np.array(bface, np.int32), btag=np.array(btag, np.int32))
