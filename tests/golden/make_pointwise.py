"""Generates tests/golden/pointwise.npz from the reference's own compiled
pointwise physics (oracle/_ref/libfvens_ref.so, built from the reference
sources by oracle/ref/build_ref.sh).

Contents (seeded inputs, reference outputs):
  phys                      gamma, Minf, Tinf, Reinf, Pr
  ul, ur, n                 random states / unit normals (N of each)
  flux_<k>                  reference get_flux for flux kind k (0..6)
  dfdl_<k>, dfdr_<k>        reference get_jacobian for k in {0,2,4,5,6}
  wall_ul, wall_n           states with slip-wall ghost states on the right (entropy fix active)
  wall_ur, wflux_<k>, wdfdl_<k>, wdfdr_<k>
  bc_<t>_vals, bc_<t>_ghost, bc_<t>_jghost, bc_<t>_dgdu   per BC type t
  walltest_*                the reference's wall-BC test state (tests/flow-general/testwallbcs.cpp:73-78)
Run: python tests/golden/make_pointwise.py
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import orc  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pointwise.npz")


def main():
    R = orc.ref_lib()
    if R is None:
        raise SystemExit("reference shim not built (oracle/_ref); run python -m fvens_gb300.build here")
    p = orc.p
    rng = np.random.default_rng(20261203)
    phys = np.array([1.4, 0.5, 288.15, 5000.0, 0.72])
    aoa = 0.03
    N = 96

    def state():
        rho = rng.uniform(0.5, 1.5)
        vx, vy = rng.uniform(-1.2, 1.2, 2)
        pr = rng.uniform(0.6, 1.4) / (1.4 * 0.25)
        return np.array([rho, rho * vx, rho * vy, pr / 0.4 + 0.5 * rho * (vx * vx + vy * vy)])

    ul = np.array([state() for _ in range(N)])
    ur = np.array([state() if k % 2 else ul[k] * (1 + rng.normal(0, 0.05, 4)) for k in range(N)])
    th = rng.uniform(0, 2 * np.pi, N)
    n = np.stack([np.cos(th), np.sin(th)], 1)
    out = dict(phys=phys, aoa=np.array([aoa]), ul=ul, ur=ur, n=n)
    for k in range(7):
        f = np.zeros((N, 4))
        for i in range(N):
            R.ref_flux(k, p(phys), p(ul[i]), p(ur[i]), p(n[i]), p(f[i]))
        out[f"flux_{k}"] = f
        if k in (1, 3):
            continue
        dl = np.zeros((N, 16)); dr = np.zeros((N, 16))
        for i in range(N):
            R.ref_flux_jacobian(k, p(phys), p(ul[i]), p(ur[i]), p(n[i]), p(dl[i]), p(dr[i]))
        out[f"dfdl_{k}"] = dl
        out[f"dfdr_{k}"] = dr
    # slip-wall face pairs: Roe averages have zero normal velocity, entropy fix active
    wur = np.zeros((N, 4))
    z = np.zeros(2)
    for i in range(N):
        R.ref_bc_ghost(0, p(phys), ctypes.c_double(0.0), p(z), p(ul[i]), p(n[i]), p(wur[i]))
    out["wall_ur"] = wur
    for k in (4, 6):
        f = np.zeros((N, 4)); dl = np.zeros((N, 16)); dr = np.zeros((N, 16))
        for i in range(N):
            R.ref_flux(k, p(phys), p(ul[i]), p(wur[i]), p(n[i]), p(f[i]))
            R.ref_flux_jacobian(k, p(phys), p(ul[i]), p(wur[i]), p(n[i]), p(dl[i]), p(dr[i]))
        out[f"wflux_{k}"] = f; out[f"wdfdl_{k}"] = dl; out[f"wdfdr_{k}"] = dr
    bcvals = {0: [0, 0], 1: [0, 0], 2: [0, 0], 3: [2.0 / (1.4 * 0.25) * 0.6, 320.0], 4: [0, 0], 6: [0.1, 290.0],
              7: [0.2, 0]}
    for t, v in bcvals.items():
        v = np.array(v, np.float64)
        g = np.zeros((N, 4)); gj = np.zeros((N, 4)); G = np.zeros((N, 16))
        for i in range(N):
            R.ref_bc_ghost(t, p(phys), ctypes.c_double(aoa), p(v), p(ul[i]), p(n[i]), p(g[i]))
            if t != 3:
                R.ref_bc_ghost_jacobian(t, p(phys), ctypes.c_double(aoa), p(v), p(ul[i]), p(n[i]), p(gj[i]), p(G[i]))
        out[f"bc_{t}_vals"] = v
        out[f"bc_{t}_ghost"] = g
        if t != 3:
            out[f"bc_{t}_jghost"] = gj
            out[f"bc_{t}_dgdu"] = G
    # wall zero-flux test state of the reference (testwallbcs.cpp:73-78)
    uw = np.array([1.0, 0.5, 0.5, 10.0 / (1.4 - 1.0) + 0.5 * 0.5])
    out["walltest_u"] = uw
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
