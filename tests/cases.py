"""Shared mesh / scheme cases for the parity tests (small enough that the
CPU oracle evaluates them in well under a second)."""
import numpy as np

import fvens_gb300 as fv

CHANNEL_BCS = [(1, "slipwall", ()), (2, "inflowoutflow", ()), (3, "slipwall", ()), (4, "inflowoutflow", ())]
NACA_INV_BCS = [(2, "slipwall", ()), (4, "farfield", ())]
NACA_VISC_BCS = [(2, "adiabaticwall", (0.0,)), (4, "farfield", ())]


def channel(nx=48, ny=16, split=0.5, seed=1, reorder=1):
    return fv.UMesh.generate(fv.MESH_CHANNEL_BUMP, [nx, ny, split, seed], reorder=reorder)


def naca(nc=64, nr=24, rfar=20.0, nbl=0, h0=0.0, g=1.15, tri_from=14, seed=3, reorder=1):
    return fv.UMesh.generate(fv.MESH_NACA_OGRID, [nc, nr, rfar, nbl, h0, g, tri_from, seed], reorder=reorder)


def naca_visc(nc=64, nr=28, seed=5):
    return fv.UMesh.generate(fv.MESH_NACA_OGRID, [nc, nr, 20.0, 12, 2e-3, 1.2, 12, seed], reorder=1)


def perturbed_state(uinf, nelem, amp=0.05, seed=1234):
    """Freestream with seeded 5 % per-cell perturbations of every conserved variable."""
    rng = np.random.default_rng(seed)
    u = np.tile(np.asarray(uinf, np.float64), (nelem, 1))
    u *= 1.0 + amp * rng.uniform(-1, 1, size=u.shape)
    return u


# (name, mesh factory, physics kwargs, numerics kwargs, bcs)
RESIDUAL_CASES = [
    ("c1_roe_wls_unlimited", channel, dict(Minf=0.5), dict(flux="ROE", gradient="LEASTSQUARES"), CHANNEL_BCS),
    ("c2_hllc_gg_venkat", naca, dict(Minf=0.8, aoa_deg=1.25),
     dict(flux="HLLC", gradient="GREENGAUSS", reconstruction="VENKATAKRISHNAN", limiter_param=5.0), NACA_INV_BCS),
    ("llf_wls", channel, dict(Minf=0.5), dict(flux="LLF"), CHANNEL_BCS),
    ("vanleer_wls", channel, dict(Minf=0.5), dict(flux="VANLEER", flux_jac="ROE"), CHANNEL_BCS),
    ("ausm_wls", channel, dict(Minf=0.5, aoa_deg=3.0), dict(flux="AUSM"), CHANNEL_BCS),
    ("ausmplus_wls", channel, dict(Minf=0.5), dict(flux="AUSMPLUS", flux_jac="ROE"), CHANNEL_BCS),
    ("hll_wls", channel, dict(Minf=0.5), dict(flux="HLL"), CHANNEL_BCS),
    ("hllc_wls_vanalbada", naca, dict(Minf=0.8, aoa_deg=1.25),
     dict(flux="HLLC", reconstruction="VANALBADA"), NACA_INV_BCS),
    ("hllc_wls_barth", naca, dict(Minf=0.75, aoa_deg=2.0),
     dict(flux="HLLC", reconstruction="BARTHJESPERSEN"), NACA_INV_BCS),
    ("roe_wls_weno", naca, dict(Minf=0.8, aoa_deg=1.25),
     dict(flux="ROE", reconstruction="WENO", limiter_param=20.0), NACA_INV_BCS),
    ("roe_first_order", channel, dict(Minf=0.5), dict(flux="ROE", gradient="NONE"), CHANNEL_BCS),
    ("roe_visc_sutherland", naca_visc, dict(Minf=0.5, Reinf=5000.0, viscous=True, aoa_deg=1.0),
     dict(flux="ROE"), NACA_VISC_BCS),
    ("roe_visc_const", naca_visc, dict(Minf=0.5, Reinf=5000.0, viscous=True, const_visc=True),
     dict(flux="ROE", gradient="GREENGAUSS"), NACA_VISC_BCS),
    ("hllc_visc_first_order", naca_visc, dict(Minf=0.5, Reinf=2000.0, viscous=True),
     dict(flux="HLLC", gradient="NONE"), NACA_VISC_BCS),
    ("roe_visc_isothermal", naca_visc, dict(Minf=0.3, Reinf=3000.0, viscous=True),
     dict(flux="ROE"), [(2, "isothermalwall", (0.0, 1.05)), (4, "farfield", ())]),
    ("hllc_inflow_extrap", channel, dict(Minf=0.4),
     dict(flux="HLLC"), [(1, "slipwall", ()), (2, "extrapolation", ()), (3, "slipwall", ()),
                         (4, "subsonic_inflow", (1.0 / (1.4 * 0.16) * 1.1, 288.15 * 1.032))]),
]


def write_gmsh(m, path):
    """Writes a mesh as Gmsh 2.2 ASCII (boundary faces as lines with their
    markers as physical tags, cells as triangles / quads)."""
    ex = m.export()
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(ex["coords"]))
        for k, (x, y) in enumerate(ex["coords"]):
            f.write("%d %.17g %.17g 0\n" % (k + 1, x, y))
        nb, ne = len(ex["btag"]), len(ex["nnode"])
        f.write("$EndNodes\n$Elements\n%d\n" % (nb + ne))
        k = 1
        for (a, b), t in zip(ex["bface"], ex["btag"]):
            f.write("%d 1 2 %d %d %d %d\n" % (k, t, t, a + 1, b + 1))
            k += 1
        for nn, nodes in zip(ex["nnode"], ex["inpoel"]):
            f.write("%d %d 2 0 1 %s\n" % (k, 2 if nn == 3 else 3, " ".join(str(v + 1) for v in nodes[:nn])))
            k += 1
        f.write("$EndElements\n")
