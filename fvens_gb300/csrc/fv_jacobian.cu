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
#include "fv_jacobian_body.cuh"


namespace fvg {

namespace {

constexpr int BS = 128;
constexpr int kMaxJacBS = 256;  // bound of the face kernel's tuned block size (fv_disc_autotune)

template <int JFLUX, class R>
__global__ void __launch_bounds__(kMaxJacBS) k_jac_face(DiscDev D, const double *__restrict__ u, R *__restrict__ val,
                                                        double *__restrict__ bdiag, const int2 *__restrict__ fslot)
{
	const int b = blockIdx.y;
	if (skip_member(D, b)) return;
	const int f = blockIdx.x * blockDim.x + threadIdx.x;
	if (f >= D.naface) return;
	jac_face_body<JFLUX, R>(D, b, f, u, val, bdiag, fslot);
}

template <class R>
__global__ void __launch_bounds__(BS) k_jac_diag(DiscDev D, R *__restrict__ val, const double *__restrict__ bdiag,
                                                 const int4 *__restrict__ crev)
{
	const int b = blockIdx.y;
	if (skip_member(D, b)) return;
	const int i = blockIdx.x * BS + threadIdx.x;
	if (i >= D.nelem) return;
	jac_diag_body<R>(D, b, i, val, bdiag, crev);
}

template <class R>
__global__ void k_zero_slots(DiscDev D, R *__restrict__ val)
{
	// zero the off-diagonal slots of edges without an interior neighbour
	const int b = blockIdx.y;
	if (skip_member(D, b)) return;
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
	const int bj = Dh->bs[KBS_JAC];
	const dim3 gf((unsigned)((D.naface + bj - 1) / bj), (unsigned)B);
	const dim3 gc((unsigned)((D.nelem + BS - 1) / BS), (unsigned)B);
	k_zero_slots<R><<<gc, BS, 0, s>>>(D, val);
	switch (D.jflux) {
	case FLUX_LLF: k_jac_face<FLUX_LLF, R><<<gf, bj, 0, s>>>(D, u, val, A.bdiag, fslot); break;
	case FLUX_AUSM: k_jac_face<FLUX_AUSM, R><<<gf, bj, 0, s>>>(D, u, val, A.bdiag, fslot); break;
	case FLUX_ROE: k_jac_face<FLUX_ROE, R><<<gf, bj, 0, s>>>(D, u, val, A.bdiag, fslot); break;
	case FLUX_HLL: k_jac_face<FLUX_HLL, R><<<gf, bj, 0, s>>>(D, u, val, A.bdiag, fslot); break;
	case FLUX_HLLC: k_jac_face<FLUX_HLLC, R><<<gf, bj, 0, s>>>(D, u, val, A.bdiag, fslot); break;
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
