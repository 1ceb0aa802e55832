// Host-side construction of the device arrays of a mesh and of a
// discretisation (the HBM layout described in fv_core.cuh), kept separate
// from the uploads so it can be checked without a GPU.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>
#include "fv_core.cuh"

namespace fvg {

struct MeshArrays {
	std::vector<double2> cc, fcen, gcen;
	std::vector<double> area, iarea;
	std::vector<int4> cface, cnbr, crev;
	std::vector<int2> flr, fslot;
	std::vector<d4> fgeo;
};

inline MeshArrays mesh_arrays(const HostMesh &h)
{
	MeshArrays a;
	const int ne = h.nelem, nf = h.naface, nb = h.nbface;
	a.cc.resize(ne); a.fcen.resize(nf); a.gcen.resize(std::max(nb, 1));
	a.area.resize(ne); a.iarea.resize(ne);
	a.cface.resize(ne); a.cnbr.resize(ne); a.crev.resize(ne);
	a.flr.resize(nf); a.fslot.resize(nf); a.fgeo.resize(nf);
	for (int i = 0; i < ne; i++) {
		a.cc[i] = make_double2(h.cc[2 * i], h.cc[2 * i + 1]);
		a.area[i] = h.area[i];
		a.iarea[i] = 1.0 / h.area[i];
		int cf[4], cn[4], rv[4];
		for (int j = 0; j < 4; j++) {
			if (j >= h.nnode[i]) { cf[j] = -1; cn[j] = NO_EDGE; rv[j] = -1; continue; }
			const int f = h.elemface[4 * i + j];
			const int side = h.face_l[f] == i ? 0 : 1;
			cf[j] = (f << 1) | side;
			cn[j] = h.esuel[4 * i + j];
			rv[j] = cn[j] >= 0 ? (side ? h.face_sl[f] : h.face_sr[f]) : -1;
		}
		a.cface[i] = make_int4(cf[0], cf[1], cf[2], cf[3]);
		a.cnbr[i] = make_int4(cn[0], cn[1], cn[2], cn[3]);
		a.crev[i] = make_int4(rv[0], rv[1], rv[2], rv[3]);
	}
	for (int f = 0; f < nf; f++) {
		a.flr[f] = make_int2(h.face_l[f], h.face_r[f]);
		a.fslot[f] = make_int2(h.face_sl[f], h.face_sr[f]);
		a.fgeo[f] = d4{h.fnorm[3 * f], h.fnorm[3 * f + 1], h.fnorm[3 * f + 2], 0.0};
		a.fcen[f] = make_double2(h.fc[2 * f], h.fc[2 * f + 1]);
	}
	for (int f = 0; f < nb; f++) a.gcen[f] = make_double2(h.gc[2 * f], h.gc[2 * f + 1]);
	return a;
}

struct DiscArrays {
	std::vector<d4> gcoef_gg, gcoef_ls;  // [nelem][2] (see DiscDev::gcoef)
	std::vector<double2> gself_gg;
	std::vector<d4> fvis;
	std::vector<double> veps2;
};

/* Per-cell gradient coefficients (Green-Gauss and weighted least squares),
 * per-face viscous geometry and per-cell Venkatakrishnan thresholds. */
inline DiscArrays disc_arrays(const HostMesh &h, bool venkat, double limparam)
{
	DiscArrays a;
	const int ne = h.nelem, nf = h.naface, nb = h.nbface;
	std::vector<double2> fwdr(nf), fggw(nf);
	std::vector<d4> vinv(ne);
	a.fvis.resize(nf); a.veps2.assign(ne, 0.0);
	std::vector<double> V(4 * (size_t)ne, 0.0);
	for (int f = 0; f < nf; f++) {
		const int L = h.face_l[f];
		const double xl = h.cc[2 * L], yl = h.cc[2 * L + 1];
		const double xr = f < nb ? h.gc[2 * f] : h.cc[2 * h.face_r[f]];
		const double yr = f < nb ? h.gc[2 * f + 1] : h.cc[2 * h.face_r[f] + 1];
		// weighted least squares (agradientschemes.cpp:219-317)
		const double dx = xl - xr, dy = yl - yr;
		const double w2 = 1.0 / (dx * dx + dy * dy);
		fwdr[f] = make_double2(w2 * dx, w2 * dy);
		const double va = w2 * dx * dx, vb = w2 * dx * dy, vc = w2 * dy * dy;
		V[4 * L] += va; V[4 * L + 1] += vb; V[4 * L + 2] += vb; V[4 * L + 3] += vc;
		if (f >= nb) {
			const int R = h.face_r[f];
			V[4 * R] += va; V[4 * R + 1] += vb; V[4 * R + 2] += vb; V[4 * R + 3] += vc;
		}
		// Green-Gauss inverse-distance weights (agradientschemes.cpp:62-216)
		const double mx = h.fc[2 * f], my = h.fc[2 * f + 1];
		const double dL = 1.0 / std::sqrt((mx - xl) * (mx - xl) + (my - yl) * (my - yl));
		const double dR = 1.0 / std::sqrt((mx - xr) * (mx - xr) + (my - yr) * (my - yr));
		const double len = h.fnorm[3 * f + 2];
		fggw[f] = make_double2(dL / (dL + dR) * len, dR / (dL + dR) * len);
		// viscous face geometry (aspatial.cpp:172-205)
		const double ex = xr - xl, ey = yr - yl, dist = std::sqrt(ex * ex + ey * ey);
		a.fvis[f] = d4{ex / dist, ey / dist, 1.0 / dist, dist};
	}
	for (int i = 0; i < ne; i++) {
		const double va = V[4 * i], vb = V[4 * i + 1], vc = V[4 * i + 2], vd = V[4 * i + 3];
		const double det = va * vd - vb * vc;
		vinv[i] = d4{vd / det, -vb / det, -vc / det, va / det};
	}
	// Per cell and local edge j: the coefficients of the neighbour's value.
	// Green-Gauss (agradientschemes.cpp:62-216): sum over faces of the
	// inverse-distance-weighted face value times the face normal and length,
	// over the area; the cell's own value collects the weights of its side.
	// Weighted least squares (agradientschemes.cpp:219-317): V^-1 w2 dr_ij
	// multiplying (q_j - q_i), dr_ij the neighbour's centre minus the cell's.
	a.gcoef_gg.assign(2 * (size_t)ne, d4{0, 0, 0, 0});
	a.gcoef_ls.assign(2 * (size_t)ne, d4{0, 0, 0, 0});
	a.gself_gg.assign(ne, make_double2(0, 0));
	for (int i = 0; i < ne; i++) {
		const double ia = 1.0 / h.area[i];
		const d4 Vi = vinv[i];
		double sx = 0, sy = 0, gg[8] = {0, 0, 0, 0, 0, 0, 0, 0}, ls[8] = {0, 0, 0, 0, 0, 0, 0, 0};
		for (int j = 0; j < h.nnode[i] && j < 4; j++) {
			const int f = h.elemface[4 * i + j];
			const bool left = h.face_l[f] == i;
			const double nx = h.fnorm[3 * f], ny = h.fnorm[3 * f + 1];
			// the cell's weight and the neighbour's, signed for the outward normal
			const double wself = left ? fggw[f].x : -fggw[f].y;
			const double wnbr = left ? fggw[f].y : -fggw[f].x;
			sx += wself * nx; sy += wself * ny;
			gg[2 * j] = wnbr * nx * ia; gg[2 * j + 1] = wnbr * ny * ia;
			// w2 (r_nbr - r_i): fwdr holds w2 (r_L - r_R)
			const double ex = left ? -fwdr[f].x : fwdr[f].x, ey = left ? -fwdr[f].y : fwdr[f].y;
			ls[2 * j] = Vi.x * ex + Vi.y * ey;
			ls[2 * j + 1] = Vi.z * ex + Vi.w * ey;
		}
		a.gself_gg[i] = make_double2(sx * ia, sy * ia);
		a.gcoef_gg[2 * i] = d4{gg[0], gg[1], gg[2], gg[3]};
		a.gcoef_gg[2 * i + 1] = d4{gg[4], gg[5], gg[6], gg[7]};
		a.gcoef_ls[2 * i] = d4{ls[0], ls[1], ls[2], ls[3]};
		a.gcoef_ls[2 * i + 1] = d4{ls[4], ls[5], ls[6], ls[7]};
	}
	if (venkat) {
		// characteristic length = longest cell edge (limitedlinearreconstruction.cpp:180-205)
		for (int i = 0; i < ne; i++) {
			double l2 = 0;
			for (int j = 0; j < h.nnode[i]; j++) {
				const int p = h.inpoel[4 * i + j], q = h.inpoel[4 * i + (j + 1) % h.nnode[i]];
				const double ex = h.coords[2 * p] - h.coords[2 * q], ey = h.coords[2 * p + 1] - h.coords[2 * q + 1];
				l2 = std::max(l2, ex * ex + ey * ey);
			}
			a.veps2[i] = std::pow(limparam * std::sqrt(l2), 3);
		}
	}
	return a;
}

}  // namespace fvg
