// Per-face and per-cell bodies of the Jacobian assembly (host/device), used
// by the kernels in fv_jacobian.cu.
#pragma once
#include "fv_core.cuh"

namespace fvg {

/* F(ul, ur) differentiated w.r.t. one side (SIDE 0: ul, 1: ur); dF[i*4+k]. */
template <int JFLUX, class R, int SIDE>
FV_HD void flux_derivs(const DiscDev &D, const Phys &P, const R *ul, const R *ur,
                                            const double *n, const double2 &rcl, const double2 &rcr, R *dF)
{
	typedef Dual<R, 4> T;
	T a[4], c[4];
	for (int i = 0; i < 4; i++) {
		a[i] = dconst<R, 4>(ul[i]);
		c[i] = dconst<R, 4>(ur[i]);
		if (SIDE == 0) a[i].d[i] = R(1);
		else c[i].d[i] = R(1);
	}
	const St<T> sL = st_from_cons(P, a), sR = st_from_cons(P, c);
	T F[4];
	numflux<JFLUX>(P, sL, sR, n, F);
	if (D.viscous) {
		// thin-layer face gradient of (rho,u,v,T): (q_R - q_L)/d along the centroid line
		double drx = rcr.x - rcl.x, dry = rcr.y - rcl.y;
		const double dist = sqrt(drx * drx + dry * dry);
		drx /= dist;
		dry /= dist;
		const R idist = R(1.0 / dist);
		T qL[4] = {sL.r, sL.u, sL.v, R(P.tcoef) * sL.p * sL.ir};
		T qR[4] = {sR.r, sR.u, sR.v, R(P.tcoef) * sR.p * sR.ir};
		T gf[2][4];
		for (int v = 0; v < 4; v++) {
			const T corr = (qR[v] - qL[v]) * idist;
			gf[0][v] = corr * R(drx);
			gf[1][v] = corr * R(dry);
		}
		T vf[4];
		viscous_flux<T>(P, D.constvisc != 0, n, gf, sL, sR, vf);
		for (int v = 0; v < 4; v++) F[v] = F[v] + vf[v];
	}
	for (int i = 0; i < 4; i++)
		for (int k = 0; k < 4; k++) dF[i * 4 + k] = F[i].d[k];
}

template <class R>
FV_HD void store_block(R *dst, size_t stride_unused, const R *blk)
{
	(void)stride_unused;
	if (sizeof(R) == 4) {
		float4 *d = reinterpret_cast<float4 *>(dst);
		const float *s = reinterpret_cast<const float *>(blk);
		for (int q = 0; q < 4; q++) d[q] = make_float4(s[4 * q], s[4 * q + 1], s[4 * q + 2], s[4 * q + 3]);
	} else {
		double2 *d = reinterpret_cast<double2 *>(dst);
		const double *s = reinterpret_cast<const double *>(blk);
		for (int q = 0; q < 8; q++) d[q] = make_double2(s[2 * q], s[2 * q + 1]);
	}
}

/* face blocks: interior faces write A[R][L] (= L block, -dF/dul*len) and
 * A[L][R] (= U block, dF/dur*len) into their slots; boundary faces write the
 * diagonal contribution len*(dF/dul + dF/dur dG/dul) to bdiag. */
template <int JFLUX, class R>
FV_HD void jac_face_body(const DiscDev &D, int b, int f, const double *__restrict__ u, R *__restrict__ val,
                         double *__restrict__ bdiag, const int2 *__restrict__ fslot)
{
	const Phys &P = D.phys[b];
	const int2 lr = D.flr[f];
	const int L = lr.x, Rc = lr.y;
	const d4 g = D.fgeo[f];
	const double n[2] = {g.x, g.y};
	const R len = R(g.z);
	const d4 *ub = reinterpret_cast<const d4 *>(u) + (size_t)b * D.nelem;
	const d4 a = ub[L];
	R ul[4] = {R(a.x), R(a.y), R(a.z), R(a.w)};
	const size_t N = D.nelem;
	R *vb = val + (size_t)b * 5 * N * 16;
	if (Rc >= 0) {
		const d4 c = ub[Rc];
		R ur[4] = {R(c.x), R(c.y), R(c.z), R(c.w)};
		const double2 rcl = D.cc[L], rcr = D.cc[Rc];
		R blk[16];
		flux_derivs<JFLUX, R, 0>(D, P, ul, ur, n, rcl, rcr, blk);
		for (int q = 0; q < 16; q++) blk[q] = -blk[q] * len;
		const int2 sl = fslot[f];
		store_block(vb + ((size_t)(1 + sl.y) * N + Rc) * 16, 0, blk);  // row R, column L
		flux_derivs<JFLUX, R, 1>(D, P, ul, ur, n, rcl, rcr, blk);
		for (int q = 0; q < 16; q++) blk[q] = blk[q] * len;
		store_block(vb + ((size_t)(1 + sl.x) * N + L) * 16, 0, blk);   // row L, column R
	} else {
		const int ib = -1 - Rc;
		R gs[4], G[16];
		ghost_jacobian<R>(P, D.bcs[D.bcid[ib]], ul, n, gs, G);
		const double2 rcl = D.cc[L], rcr = D.gcen[ib];
		R dl[16], dr[16];
		flux_derivs<JFLUX, R, 0>(D, P, ul, gs, n, rcl, rcr, dl);
		flux_derivs<JFLUX, R, 1>(D, P, ul, gs, n, rcl, rcr, dr);
		double *o = bdiag + ((size_t)b * D.nbface + ib) * 16;
		for (int i = 0; i < 4; i++)
			for (int k = 0; k < 4; k++) {
				R s = dl[4 * i + k];
				for (int j = 0; j < 4; j++) s += dr[4 * i + j] * G[4 * j + k];
				o[4 * i + k] = double(len * s);
			}
	}
}

/* diagonal blocks: A_ii = -sum over interior faces of the neighbour's block
 * in column i, + boundary-face terms. */
template <class R>
FV_HD void jac_diag_body(const DiscDev &D, int b, int i, R *__restrict__ val, const double *__restrict__ bdiag,
                         const int4 *__restrict__ crev)
{
	const size_t N = D.nelem;
	R *vb = val + (size_t)b * 5 * N * 16;
	const int4 cn = D.cnbr[i], rv = crev[i];
	const int nbr[4] = {cn.x, cn.y, cn.z, cn.w};
	const int rev[4] = {rv.x, rv.y, rv.z, rv.w};
	double acc[16];
	for (int q = 0; q < 16; q++) acc[q] = 0;
	for (int j = 0; j < 4; j++) {
		const int nb = nbr[j];
		if (nb == NO_EDGE) continue;
		if (nb >= 0) {
			const R *blk = vb + ((size_t)(1 + rev[j]) * N + nb) * 16;
			for (int q = 0; q < 16; q++) acc[q] -= double(blk[q]);
		} else {
			const double *o = bdiag + ((size_t)b * D.nbface + (-1 - nb)) * 16;
			for (int q = 0; q < 16; q++) acc[q] += o[q];
		}
	}
	R out[16];
	for (int q = 0; q < 16; q++) out[q] = R(acc[q]);
	store_block(vb + (size_t)i * 16, 0, out);
}

}  // namespace fvg
