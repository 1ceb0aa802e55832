// First-order approximate Jacobian assembly on the GPU.
//
// Replaces Spatial::assemble_jacobian (src/spatial/aspatial.cpp:242-340) with
// FlowFV::compute_local_jacobian_interior/_boundary (flow_spatial.cpp:818-875),
// the flux Jacobians (anumericalflux.cpp), BC Jacobians (abc.cpp) and the
// thin-layer viscous Jacobian (flow_spatial.cpp:397-446, aspatial.cpp:207-240,
// viscousphysics.cpp:125-245).
//
// Blocks are obtained by forward-mode differentiation of the Jacobian flux
// (two passes of four directions each, w.r.t. the left and the right state)
// in FP32 (the stored Jacobian of the optimised path) or FP64 (the plain
// path).  No atomics: each off-diagonal block belongs to exactly one face and
// is written by that face's thread; diagonal blocks are gathered per cell from
// the neighbours' off-diagonal blocks (A_ii = -sum_j A_ji) plus boundary-face
// terms, in a second launch.
#include "fv_core.cuh"

namespace fvg {

namespace {

constexpr int BS = 128;

template <class R>
struct BlockOut;

/* F(ul, ur) differentiated w.r.t. one side (SIDE 0: ul, 1: ur); dF[i*4+k]. */
template <int JFLUX, class R, int SIDE>
__device__ __forceinline__ void flux_derivs(const DiscDev &D, const Phys &P, const R *ul, const R *ur,
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
__device__ __forceinline__ void store_block(R *dst, size_t stride_unused, const R *blk)
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
__global__ void __launch_bounds__(BS) k_jac_face(DiscDev D, const double *__restrict__ u, R *__restrict__ val,
                                                 double *__restrict__ bdiag, const int2 *__restrict__ fslot)
{
	const int b = blockIdx.y;
	const int f = blockIdx.x * BS + threadIdx.x;
	if (f >= D.naface) return;
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
__global__ void __launch_bounds__(BS) k_jac_diag(DiscDev D, R *__restrict__ val, const double *__restrict__ bdiag,
                                                 const int4 *__restrict__ crev)
{
	const int b = blockIdx.y;
	const int i = blockIdx.x * BS + threadIdx.x;
	if (i >= D.nelem) return;
	const size_t N = D.nelem;
	R *vb = val + (size_t)b * 5 * N * 16;
	const int4 cn = D.cnbr[i], rv = crev[i];
	const int nbr[4] = {cn.x, cn.y, cn.z, cn.w};
	const int rev[4] = {rv.x, rv.y, rv.z, rv.w};
	double acc[16];
	for (int q = 0; q < 16; q++) acc[q] = 0;
	for (int j = 0; j < 4; j++) {
		const int nb = nbr[j];
		if (nb == -2) continue;
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

template <class R>
__global__ void k_zero_slots(DiscDev D, R *__restrict__ val)
{
	// zero the off-diagonal slots of edges without an interior neighbour
	const int b = blockIdx.y;
	const int i = blockIdx.x * BS + threadIdx.x;
	if (i >= D.nelem) return;
	const size_t N = D.nelem;
	R *vb = val + (size_t)b * 5 * N * 16;
	const int4 cn = D.cnbr[i];
	const int nbr[4] = {cn.x, cn.y, cn.z, cn.w};
	R z[16];
	for (int q = 0; q < 16; q++) z[q] = R(0);
	for (int j = 0; j < 4; j++)
		if (nbr[j] < 0) store_block(vb + ((size_t)(1 + j) * N + i) * 16, 0, z);
}

template <class R>
cudaError_t launch_all(fv_disc_impl *Dh, const double *u, BlockMatrix &A, cudaStream_t s)
{
	const DiscDev &D = Dh->d;
	const int B = Dh->batch;
	R *val = reinterpret_cast<R *>(A.val);
	const int2 *fslot = Dh->mesh->d.fslot;
	const int4 *crev = Dh->mesh->d.cslot_rev;
	const dim3 gf((unsigned)((D.naface + BS - 1) / BS), (unsigned)B);
	const dim3 gc((unsigned)((D.nelem + BS - 1) / BS), (unsigned)B);
	k_zero_slots<R><<<gc, BS, 0, s>>>(D, val);
	switch (D.jflux) {
	case FLUX_LLF: k_jac_face<FLUX_LLF, R><<<gf, BS, 0, s>>>(D, u, val, A.bdiag, fslot); break;
	case FLUX_AUSM: k_jac_face<FLUX_AUSM, R><<<gf, BS, 0, s>>>(D, u, val, A.bdiag, fslot); break;
	case FLUX_ROE: k_jac_face<FLUX_ROE, R><<<gf, BS, 0, s>>>(D, u, val, A.bdiag, fslot); break;
	case FLUX_HLL: k_jac_face<FLUX_HLL, R><<<gf, BS, 0, s>>>(D, u, val, A.bdiag, fslot); break;
	case FLUX_HLLC: k_jac_face<FLUX_HLLC, R><<<gf, BS, 0, s>>>(D, u, val, A.bdiag, fslot); break;
	default: return cudaErrorInvalidValue;
	}
	k_jac_diag<R><<<gc, BS, 0, s>>>(D, val, A.bdiag, crev);
	Dh->kernels_launched += 3;
	return cudaGetLastError();
}

}  // namespace

cudaError_t jacobian_launch(fv_disc_impl *Dh, const double *u, BlockMatrix &A, cudaStream_t s)
{
	if (A.prec == 4) return launch_all<float>(Dh, u, A, s);
	return launch_all<double>(Dh, u, A, s);
}

}  // namespace fvg
