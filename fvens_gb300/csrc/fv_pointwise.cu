// Pointwise device evaluations used to validate the device physics directly
// against the reference's compiled fluxes, flux Jacobians and BCs, and the
// diagonal shift of the block matrix.
#include "fv_abi_internal.hpp"

namespace fvg {

namespace {

template <int FLUX>
__global__ void k_pw_flux(const Phys *P, int n, const double *ul, const double *ur, const double *nrm, double *f)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n) return;
	const St<double> L = st_from_cons(*P, ul + 4 * t), R = st_from_cons(*P, ur + 4 * t);
	numflux<FLUX>(*P, L, R, nrm + 2 * t, f + 4 * t);
}

template <int FLUX>
__global__ void k_pw_fjac(const Phys *P, int n, const double *ul, const double *ur, const double *nrm, double *dl,
                          double *dr)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n) return;
	typedef Dual<double, 8> T;
	T a[4], c[4], F[4];
	for (int i = 0; i < 4; i++) {
		a[i] = dconst<double, 8>(ul[4 * t + i]);
		c[i] = dconst<double, 8>(ur[4 * t + i]);
		a[i].d[i] = 1.0;
		c[i].d[4 + i] = 1.0;
	}
	const St<T> L = st_from_cons(*P, a), R = st_from_cons(*P, c);
	numflux<FLUX>(*P, L, R, nrm + 2 * t, F);
	for (int i = 0; i < 4; i++)
		for (int k = 0; k < 4; k++) {
			dl[16 * t + 4 * i + k] = -F[i].d[k];
			dr[16 * t + 4 * i + k] = F[i].d[4 + k];
		}
}

__global__ void k_pw_bc(const Phys *P, BCDev bc, int n, const double *in, const double *nrm, double *gs, double *gj,
                        double *G)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n) return;
	if (gs) ghost_cons<double>(*P, bc, in + 4 * t, nrm + 2 * t, gs + 4 * t, false);
	if (gj && G) ghost_jacobian<double>(*P, bc, in + 4 * t, nrm + 2 * t, gj + 4 * t, G + 16 * t);
}

template <class R>
__global__ void k_add_diag(int nelem, int batch, R *val, const double *diag)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const int b = blockIdx.y;
	if (i >= nelem) return;
	R *blk = val + ((size_t)b * 5 * nelem + i) * 16;
	const R d = R(diag[(size_t)b * nelem + i]);
	for (int q = 0; q < 4; q++) blk[5 * q] += d;
}

}  // namespace

cudaError_t matrix_add_diag_launch(BlockMatrix &A, const double *diag, cudaStream_t s)
{
	const dim3 g((unsigned)((A.nelem + 127) / 128), (unsigned)A.batch);
	if (A.prec == 4) k_add_diag<float><<<g, 128, 0, s>>>(A.nelem, A.batch, (float *)A.val, diag);
	else k_add_diag<double><<<g, 128, 0, s>>>(A.nelem, A.batch, (double *)A.val, diag);
	return cudaGetLastError();
}

cudaError_t pointwise_flux_launch(fv_disc_impl *D, int kind, int n, const double *ul, const double *ur,
                                  const double *nrm, double *f, cudaStream_t s)
{
	if (n == 0) return cudaSuccess;
	const int g = (n + 127) / 128;
	const Phys *P = D->d.phys;
	switch (kind) {
	case FLUX_LLF: k_pw_flux<FLUX_LLF><<<g, 128, 0, s>>>(P, n, ul, ur, nrm, f); break;
	case FLUX_VANLEER: k_pw_flux<FLUX_VANLEER><<<g, 128, 0, s>>>(P, n, ul, ur, nrm, f); break;
	case FLUX_AUSM: k_pw_flux<FLUX_AUSM><<<g, 128, 0, s>>>(P, n, ul, ur, nrm, f); break;
	case FLUX_AUSMPLUS: k_pw_flux<FLUX_AUSMPLUS><<<g, 128, 0, s>>>(P, n, ul, ur, nrm, f); break;
	case FLUX_ROE: k_pw_flux<FLUX_ROE><<<g, 128, 0, s>>>(P, n, ul, ur, nrm, f); break;
	case FLUX_HLL: k_pw_flux<FLUX_HLL><<<g, 128, 0, s>>>(P, n, ul, ur, nrm, f); break;
	default: k_pw_flux<FLUX_HLLC><<<g, 128, 0, s>>>(P, n, ul, ur, nrm, f); break;
	}
	return cudaGetLastError();
}

cudaError_t pointwise_flux_jac_launch(fv_disc_impl *D, int kind, int n, const double *ul, const double *ur,
                                      const double *nrm, double *dl, double *dr, cudaStream_t s)
{
	if (n == 0) return cudaSuccess;
	const int g = (n + 63) / 64;
	const Phys *P = D->d.phys;
	switch (kind) {
	case FLUX_LLF: k_pw_fjac<FLUX_LLF><<<g, 64, 0, s>>>(P, n, ul, ur, nrm, dl, dr); break;
	case FLUX_AUSM: k_pw_fjac<FLUX_AUSM><<<g, 64, 0, s>>>(P, n, ul, ur, nrm, dl, dr); break;
	case FLUX_ROE: k_pw_fjac<FLUX_ROE><<<g, 64, 0, s>>>(P, n, ul, ur, nrm, dl, dr); break;
	case FLUX_HLL: k_pw_fjac<FLUX_HLL><<<g, 64, 0, s>>>(P, n, ul, ur, nrm, dl, dr); break;
	case FLUX_HLLC: k_pw_fjac<FLUX_HLLC><<<g, 64, 0, s>>>(P, n, ul, ur, nrm, dl, dr); break;
	default: return cudaErrorInvalidValue;
	}
	return cudaGetLastError();
}

cudaError_t pointwise_bc_launch(fv_disc_impl *D, BCDev bc, int n, const double *in, const double *nrm, double *gs,
                                double *gj, double *G, cudaStream_t s)
{
	if (n == 0) return cudaSuccess;
	k_pw_bc<<<(n + 127) / 128, 128, 0, s>>>(D->d.phys, bc, n, in, nrm, gs, gj, G);
	return cudaGetLastError();
}

}  // namespace fvg
