// Per-cell / per-face bodies of the residual evaluation (host/device), used
// by the kernels in fv_residual.cu; see that file for the reference mapping.
#pragma once
#include <cstring>

#include "fv_core.cuh"

namespace fvg {

FV_HD double comp(const d4 &a, int v) { return v == 0 ? a.x : v == 1 ? a.y : v == 2 ? a.z : a.w; }
FV_HD void setc(d4 &a, int v, double x)
{
	if (v == 0) a.x = x; else if (v == 1) a.y = x; else if (v == 2) a.z = x; else a.w = x;
}

FV_HD void prim_of_cons(const Phys &P, const double *uc, double *up)
{
	const double ir = 1.0 / uc[0];
	const double vx = uc[1] * ir, vy = uc[2] * ir;
	up[0] = uc[0];
	up[1] = vx;
	up[2] = vy;
	up[3] = P.gm1 * (uc[3] - 0.5 * (uc[1] * vx + uc[2] * vy));
}

/* 1. primitive cell states; cell-centred ghost states of boundary faces
 *    (flow_spatial.cpp:679-699) */
FV_HD void prep_body(const DiscDev &D, int b, int t, const double *__restrict__ u, const ResidualWork &w)
{
	const Phys &P = D.phys[b];
	const d4 *ub = reinterpret_cast<const d4 *>(u) + (size_t)b * D.nelem;
	if (t < D.nelem) {
		const d4 c = ub[t];
		double uc[4] = {c.x, c.y, c.z, c.w}, up[4];
		prim_of_cons(P, uc, up);
		w.prim[(size_t)b * D.nelem + t] = d4{up[0], up[1], up[2], up[3]};
	} else if (t < D.nelem + D.nbface) {
		const int ib = t - D.nelem;
		const int L = D.flr[ib].x;
		const d4 c = ub[L];
		const double in[4] = {c.x, c.y, c.z, c.w};
		const d4 g = D.fgeo[ib];
		const double n[2] = {g.x, g.y};
		double gs[4], gp[4];
		ghost_cons<double>(P, D.bcs[D.bcid[ib]], in, n, gs, false);
		prim_of_cons(P, gs, gp);
		w.ghost_cons[(size_t)b * D.nbface + ib] = d4{gs[0], gs[1], gs[2], gs[3]};
		w.ghost_prim[(size_t)b * D.nbface + ib] = d4{gp[0], gp[1], gp[2], gp[3]};
	}
}

/* 64-bit integer that orders like the double x (for non-NaN x): its bit
 * pattern with the magnitude bits of negative values flipped, so that the
 * limiter's comparisons run on the integer pipes and leave the FP64 pipe,
 * which bounds these kernels, to the arithmetic. */
FV_HD long long order_key(double x)
{
#ifdef __CUDA_ARCH__
	const long long b = __double_as_longlong(x);
#else
	long long b;
	std::memcpy(&b, &x, sizeof b);
#endif
	return b >= 0 ? b : b ^ 0x7fffffffffffffffLL;
}

/* sign bit of x (true for negative values and -0) */
FV_HD bool sign_bit(double x) { return order_key(x) < 0; }

/* 2. cell gradients (Green-Gauss or weighted least squares) from the cell's
 *    and its neighbours' values with precomputed per-cell coefficients
 *    (DiscDev::gcoef); optionally the Barth-Jespersen / Venkatakrishnan
 *    limiter of the cell, whose limited gradients (the limiter value times
 *    the gradient, per variable) go to lgrad for the face reconstruction.
 *    q: cell states [batch][nelem], qg: ghost states [batch][nbface]. */
FV_HD void grad_body(const DiscDev &D, int b, int i, const d4 *__restrict__ q, const d4 *__restrict__ qg,
                     d4 *__restrict__ grad, d4 *__restrict__ lgrad, int limiter)
{
	const d4 *qb = q + (size_t)b * D.nelem;
	const d4 *qgb = qg + (size_t)b * D.nbface;
	const d4 qi = qb[i];
	const int4 cf = D.cface[i], cn = D.cnbr[i];
	const int fl[4] = {cf.x, cf.y, cf.z, cf.w};
	const int nbr[4] = {cn.x, cn.y, cn.z, cn.w};
	const d4 c01 = D.gcoef[2 * (size_t)i], c23 = D.gcoef[2 * (size_t)i + 1];
	const double cx[4] = {c01.x, c01.z, c23.x, c23.z}, cy[4] = {c01.y, c01.w, c23.y, c23.w};
	d4 qn[4];
	for (int j = 0; j < 4; j++) {
		const int nb = nbr[j];
		qn[j] = fl[j] < 0 ? qi : (nb >= 0 ? qb[nb] : qgb[-1 - nb]);
	}
	double gr[8];
	if (D.gradscheme == GRAD_LEASTSQUARES) {
		// sum_j V^-1 w2 dr_ij (q_j - q_i)   (agradientschemes.cpp:219-317)
#pragma unroll
		for (int v = 0; v < 4; v++) {
			const double uv = comp(qi, v);
			double gx = 0, gy = 0;
#pragma unroll
			for (int j = 0; j < 4; j++) {
				if (fl[j] < 0) continue;
				const double d = comp(qn[j], v) - uv;
				gx = fma(cx[j], d, gx);
				gy = fma(cy[j], d, gy);
			}
			gr[2 * v] = gx;
			gr[2 * v + 1] = gy;
		}
	} else {
		// (sum over faces of the weighted face value x normal x length) / area
		// (agradientschemes.cpp:62-216), split into the cell's and the neighbours' terms
		const double2 sc = D.gself[i];
#pragma unroll
		for (int v = 0; v < 4; v++) {
			const double uv = comp(qi, v);
			double gx = sc.x * uv, gy = sc.y * uv;
#pragma unroll
			for (int j = 0; j < 4; j++) {
				if (fl[j] < 0) continue;
				const double qv = comp(qn[j], v);
				gx = fma(cx[j], qv, gx);
				gy = fma(cy[j], qv, gy);
			}
			gr[2 * v] = gx;
			gr[2 * v + 1] = gy;
		}
	}
	d4 *gb = grad + 2 * ((size_t)b * D.nelem + i);
	gb[0] = d4{gr[0], gr[1], gr[2], gr[3]};
	gb[1] = d4{gr[4], gr[5], gr[6], gr[7]};
	if (!limiter) return;
	// Barth-Jespersen (limitedlinearreconstruction.cpp:117-175) or
	// Venkatakrishnan (:207-268); boundary neighbours are the ghost states.
	const bool venkat = D.recon == REC_VENKATAKRISHNAN;
	const double eps2 = venkat ? D.veps2[i] : 0.0;
	const double2 ci = D.cc[i];
	double dx[4], dy[4];
	for (int j = 0; j < 4; j++) {
		if (fl[j] < 0) { dx[j] = dy[j] = 0; continue; }
		const double2 fc = D.fcen[fl[j] >> 1];
		dx[j] = fc.x - ci.x;
		dy[j] = fc.y - ci.y;
	}
	double lg[8];
#pragma unroll
	for (int v = 0; v < 4; v++) {
		const double uv = comp(qi, v);
		// largest and smallest neighbour difference, each with 0
		double dmin = 0, dmax = 0;
		long long kmin = 0, kmax = 0;
#pragma unroll
		for (int j = 0; j < 4; j++) {
			if (fl[j] < 0) continue;
			const double d = comp(qn[j], v) - uv;
			const long long k = order_key(d);
			if (k > kmax) { kmax = k; dmax = d; }
			if (k < kmin) { kmin = k; dmin = d; }
		}
		// the smallest of 1 and the faces' ratios num/den (den > 0), found by
		// comparing cross products so that only the winner is divided
		double bn = 1.0, bd = 1.0;
#pragma unroll
		for (int j = 0; j < 4; j++) {
			if (fl[j] < 0) continue;
			// unlimited increment to the face centre
			const double dm = fma(gr[2 * v], dx[j], gr[2 * v + 1] * dy[j]);
			const bool neg = sign_bit(dm);
			double num, den;
			if (venkat) {
				const double dp = neg ? dmin : dmax;
				const double t2 = dm + dm;
				num = fma(dp, dp + t2, eps2);                // dp^2 + 2 dp dm + eps^2
				den = fma(dp, dp + dm, fma(t2, dm, eps2));   // dp^2 + dp dm + 2 dm^2 + eps^2
			} else {
				if ((order_key(dm) & 0x7fffffffffffffffLL) == 0) continue;  // dm = 0: ratio 1
				num = neg ? -dmin : dmax;
				den = fabs(dm);
			}
			if (sign_bit(fma(num, bd, -(bn * den)))) { bn = num; bd = den; }
		}
		const double phi = bn == bd ? 1.0 : bn / bd;
		lg[2 * v] = phi * gr[2 * v];
		lg[2 * v + 1] = phi * gr[2 * v + 1];
	}
	d4 *lb = lgrad + 2 * ((size_t)b * D.nelem + i);
	lb[0] = d4{lg[0], lg[1], lg[2], lg[3]};
	lb[1] = d4{lg[4], lg[5], lg[6], lg[7]};
}

/* 3. WENO-blended gradients (limitedlinearreconstruction.cpp:40-80):
 *    w = lambda/(|g|^2+eps)^4 for the cell, 1/(|g|^2+eps)^4 for each
 *    non-ghost neighbour. */
FV_HD void weno_body(const DiscDev &D, int b, int i, const d4 *__restrict__ grad, d4 *__restrict__ lgrad)
{
	const d4 *gb = grad + 2 * (size_t)b * D.nelem;
	const int4 cn = D.cnbr[i];
	const int nbr[4] = {cn.x, cn.y, cn.z, cn.w};
	const double epsw = 1.0e-5;
	double g0[8];
	{
		const d4 a = gb[2 * i], c = gb[2 * i + 1];
		g0[0] = a.x; g0[1] = a.y; g0[2] = a.z; g0[3] = a.w; g0[4] = c.x; g0[5] = c.y; g0[6] = c.z; g0[7] = c.w;
	}
	double ws[4], lg[8];
	for (int v = 0; v < 4; v++) {
		const double m = g0[2 * v] * g0[2 * v] + g0[2 * v + 1] * g0[2 * v + 1] + epsw;
		const double m2 = m * m;
		const double w = D.limparam / (m2 * m2);
		ws[v] = w;
		lg[2 * v] = w * g0[2 * v];
		lg[2 * v + 1] = w * g0[2 * v + 1];
	}
	for (int j = 0; j < 4; j++) {
		const int nb = nbr[j];
		if (nb < 0) continue;
		const d4 a = gb[2 * nb], c = gb[2 * nb + 1];
		const double gn[8] = {a.x, a.y, a.z, a.w, c.x, c.y, c.z, c.w};
		for (int v = 0; v < 4; v++) {
			const double m = gn[2 * v] * gn[2 * v] + gn[2 * v + 1] * gn[2 * v + 1] + epsw;
			const double m2 = m * m;
			const double w = 1.0 / (m2 * m2);
			ws[v] += w;
			lg[2 * v] += w * gn[2 * v];
			lg[2 * v + 1] += w * gn[2 * v + 1];
		}
	}
	for (int v = 0; v < 4; v++) {
		lg[2 * v] /= ws[v];
		lg[2 * v + 1] /= ws[v];
	}
	d4 *o = lgrad + 2 * ((size_t)b * D.nelem + i);
	o[0] = d4{lg[0], lg[1], lg[2], lg[3]};
	o[1] = d4{lg[4], lg[5], lg[6], lg[7]};
}

FV_HD void load_grad(const d4 *g, size_t cell, double *o)
{
	const d4 a = g[2 * cell], c = g[2 * cell + 1];
	o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = c.x; o[5] = c.y; o[6] = c.z; o[7] = c.w;
}

/* primitive-2 cell state and gradients from primitive ones
 * (getPrimitive2StatesAndGradients, viscousphysics.cpp:15-63) */
FV_HD void to_prim2(const Phys &P, const d4 &q, const double *g, double *q2, double *g2)
{
	const double ir = 1.0 / q.x;
	q2[0] = q.x; q2[1] = q.y; q2[2] = q.z; q2[3] = P.tcoef * q.w * ir;
	for (int d = 0; d < 2; d++) {
		g2[d * 4 + 0] = g[0 + d];
		g2[d * 4 + 1] = g[2 + d];
		g2[d * 4 + 2] = g[4 + d];
		g2[d * 4 + 3] = (g[6 + d] * q.x - q.w * g[0 + d]) * ir * ir * P.tcoef;
	}
}

/* 4. face fluxes: reconstruction, ghost state, inviscid + viscous flux,
 *    spectral radii for the local time step. */
template <int FLUX, int VISC>
FV_HD void face_body(const DiscDev &D, int b, int f, const double *__restrict__ u, const ResidualWork &w, int getdt)
{
	const Phys &P = D.phys[b];
	const size_t cb = (size_t)b * D.nelem;
	const int2 lr = D.flr[f];
	const int L = lr.x, Rc = lr.y;
	const bool bnd = Rc < 0;
	const d4 g = D.fgeo[f];
	const double n[2] = {g.x, g.y};
	const double len = g.z;
	const d4 *ub = reinterpret_cast<const d4 *>(u) + cb;
	St<double> sL, sR;
	if (!D.order2) {
		const d4 a = ub[L];
		const double ul[4] = {a.x, a.y, a.z, a.w};
		sL = st_from_cons(P, ul);
		if (bnd) {
			double gs[4];
			ghost_cons<double>(P, D.bcs[D.bcid[f]], ul, n, gs, false);
			sR = st_from_cons(P, gs);
		} else {
			const d4 c = ub[Rc];
			const double ur[4] = {c.x, c.y, c.z, c.w};
			sR = st_from_cons(P, ur);
		}
	} else {
		const d4 qL = w.prim[cb + L];
		const d4 qR = bnd ? w.ghost_prim[(size_t)b * D.nbface + f] : w.prim[cb + Rc];
		const double2 fc = D.fcen[f];
		const double2 cL = D.cc[L];
		const double2 cR = bnd ? D.gcen[f] : D.cc[Rc];
		double qfL[4], qfR[4];
		if (D.recon == REC_VANALBADA) {
			// MUSCL kappa = 1/3 with the Van Albada limiter (musclreconstruction.cpp:34-130)
			const double eps = 1e-8, k = 1.0 / 3.0;
			double gl[8], grr[8];
			load_grad(w.grad, cb + L, gl);
			if (!bnd) load_grad(w.grad, cb + Rc, grr);
			const double drx = cR.x - cL.x, dry = cR.y - cL.y;
			for (int v = 0; v < 4; v++) {
				const double ui = comp(qL, v), uj = comp(qR, v);
				const double dm = 2.0 * (gl[2 * v] * drx + gl[2 * v + 1] * dry) - (uj - ui);
				double pl = (2.0 * dm * (uj - ui) + eps) / (dm * dm + (uj - ui) * (uj - ui) + eps);
				if (pl < 0.0) pl = 0.0;
				qfL[v] = ui + pl / 4.0 * ((1.0 - k * pl) * dm + (1.0 + k * pl) * (uj - ui));
				if (!bnd) {
					const double dp = 2.0 * (grr[2 * v] * drx + grr[2 * v + 1] * dry) - (uj - ui);
					double pr = (2 * dp * (uj - ui) + eps) / (dp * dp + (uj - ui) * (uj - ui) + eps);
					if (pr < 0.0) pr = 0.0;
					qfR[v] = uj - pr / 4.0 * ((1.0 - k * pr) * dp + (1.0 + k * pr) * (uj - ui));
				}
			}
		} else {
			// linear reconstruction with the cell gradients, WENO-blended or
			// already scaled by the limiter values (grad_body)
			const d4 *gsrc = D.recon == REC_NONE ? w.grad : w.lgrad;
			double gl[8];
			load_grad(gsrc, cb + L, gl);
			const double dxl = fc.x - cL.x, dyl = fc.y - cL.y;
			for (int v = 0; v < 4; v++) qfL[v] = fma(gl[2 * v + 1], dyl, fma(gl[2 * v], dxl, comp(qL, v)));
			if (!bnd) {
				double gr[8];
				load_grad(gsrc, cb + Rc, gr);
				const double dxr = fc.x - cR.x, dyr = fc.y - cR.y;
				for (int v = 0; v < 4; v++) qfR[v] = fma(gr[2 * v + 1], dyr, fma(gr[2 * v], dxr, comp(qR, v)));
			}
		}
		if (bnd) {
			sL = st_from_prim(P, qfL);
			double ul[4], gs[4];
			st_cons(sL, ul);
			ghost_cons<double>(P, D.bcs[D.bcid[f]], ul, n, gs, false);
			sR = st_from_cons(P, gs);
		} else {
			st_pair_from_prim(P, qfL, qfR, sL, sR);
		}
	}
	double F[4];
	numflux<FLUX>(P, sL, sR, n, F);
	for (int v = 0; v < 4; v++) F[v] *= len;

	if (VISC) {
		// modified-average face gradient of (rho,u,v,T) (aspatial.cpp:172-205)
		double q2L[4], q2R[4], g2L[8] = {0, 0, 0, 0, 0, 0, 0, 0}, g2R[8] = {0, 0, 0, 0, 0, 0, 0, 0};
		d4 cL, cR;
		if (D.order2) {
			cL = w.prim[cb + L];
			cR = bnd ? w.ghost_prim[(size_t)b * D.nbface + f] : w.prim[cb + Rc];
			double gl[8], gr[8];
			load_grad(w.grad, cb + L, gl);
			load_grad(w.grad, cb + (bnd ? L : Rc), gr);
			to_prim2(P, cL, gl, q2L, g2L);
			to_prim2(P, cR, gr, q2R, g2R);
		} else {
			const d4 a = ub[L];
			double ua[4] = {a.x, a.y, a.z, a.w}, pa[4];
			prim_of_cons(P, ua, pa);
			cL = d4{pa[0], pa[1], pa[2], pa[3]};
			if (bnd) {
				double gs[4], pg[4];
				ghost_cons<double>(P, D.bcs[D.bcid[f]], ua, n, gs, false);
				prim_of_cons(P, gs, pg);
				cR = d4{pg[0], pg[1], pg[2], pg[3]};
			} else {
				const d4 c = ub[Rc];
				double uc[4] = {c.x, c.y, c.z, c.w}, pc[4];
				prim_of_cons(P, uc, pc);
				cR = d4{pc[0], pc[1], pc[2], pc[3]};
			}
			const double z[8] = {0, 0, 0, 0, 0, 0, 0, 0};
			double dummy[8];
			to_prim2(P, cL, z, q2L, dummy);
			to_prim2(P, cR, z, q2R, dummy);
		}
		const d4 fv = D.fvis[f];  // unit vector L->R, 1/dist
		double gf[2][4];
		for (int v = 0; v < 4; v++) {
			const double ax = 0.5 * (g2L[v] + g2R[v]);
			const double ay = 0.5 * (g2L[4 + v] + g2R[4 + v]);
			const double corr = (q2R[v] - q2L[v]) * fv.z;
			const double ddr = ax * fv.x + ay * fv.y;
			gf[0][v] = ax - ddr * fv.x + corr * fv.x;
			gf[1][v] = ay - ddr * fv.y + corr * fv.y;
		}
		double vf[4];
		viscous_flux<double>(P, VISC == 2, n, gf, sL, sR, vf);
		for (int v = 0; v < 4; v++) F[v] += vf[v] * len;
	}
	w.fflux[(size_t)b * D.naface + f] = d4{F[0], F[1], F[2], F[3]};
	if (getdt) {
		const double vni = sL.u * n[0] + sL.v * n[1], vnj = sR.u * n[0] + sR.v * n[1];
		double si = (fabs(vni) + sound_speed(P, sL)) * len;
		double sj = (fabs(vnj) + sound_speed(P, sR)) * len;
		if (VISC) {
			const double mui = VISC == 2 ? P.ivisc : sutherland(P, P.tcoef * sL.p * sL.ir);
			const double muj = VISC == 2 ? P.ivisc : sutherland(P, P.tcoef * sR.p * sR.ir);
			const double coi = fmax(4.0 / 3.0 * sL.ir, P.g * sL.ir);
			const double coj = fmax(4.0 / 3.0 * sR.ir, P.g * sR.ir);
			si += coi * mui / P.Pr * len * len * D.iarea[L];
			if (!bnd) sj += coj * muj / P.Pr * len * len * D.iarea[Rc];
		}
		w.spec[(size_t)b * D.naface + f] = make_double2(si, sj);
	}
}

/* 5. per-cell gather: r_i += sum over faces of -/+ F (left/right), and
 *    dt_i = A_i / sum of spectral radii */
FV_HD void gather_body(const DiscDev &D, int b, int i, const ResidualWork &w, double *__restrict__ r, double *__restrict__ dt)
{
	const int4 cf = D.cface[i];
	const int fl[4] = {cf.x, cf.y, cf.z, cf.w};
	double a0 = 0, a1 = 0, a2 = 0, a3 = 0, integ = 0;
	const d4 *ff = w.fflux + (size_t)b * D.naface;
	const double2 *sp = w.spec + (size_t)b * D.naface;
	for (int j = 0; j < 4; j++) {
		if (fl[j] < 0) continue;
		const int f = fl[j] >> 1, side = fl[j] & 1;
		const d4 F = ff[f];
		if (side) { a0 += F.x; a1 += F.y; a2 += F.z; a3 += F.w; }
		else { a0 -= F.x; a1 -= F.y; a2 -= F.z; a3 -= F.w; }
		if (dt) { const double2 s = sp[f]; integ += side ? s.y : s.x; }
	}
	d4 *rb = reinterpret_cast<d4 *>(r) + (size_t)b * D.nelem + i;
	d4 x = *rb;
	x.x += a0; x.y += a1; x.z += a2; x.w += a3;
	*rb = x;
	if (dt) dt[(size_t)b * D.nelem + i] = D.area[i] / integ;
}

}  // namespace fvg
