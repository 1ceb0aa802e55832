// FP64 residual of the finite-volume flow discretisation on the GPU.
//
// Replaces FlowFV::compute_residual (src/spatial/flow_spatial.cpp:636-816)
// and the pieces it calls:
//   ghost states           flow_spatial.cpp:73-93, abc.cpp
//   gradients              agradientschemes.cpp:62-216 (Green-Gauss), :219-440 (WLS)
//   reconstructions        areconstruction.cpp:53-103, musclreconstruction.cpp:71-130,
//                          limitedlinearreconstruction.cpp:28-268
//   face fluxes            flow_spatial.cpp:488-563, anumericalflux.cpp
//   viscous flux           flow_spatial.cpp:348-395, aspatial.cpp:172-205, viscousphysics.cpp:15-122
//   local time steps       flow_spatial.cpp:565-634
// Structure: up to five launches per evaluation (prep, gradient+limiter,
// WENO blend, face flux, cell gather).  Face fluxes are written once per face and gathered
// by cells in a fixed order, so results are deterministic and need no atomics.
#include "fv_residual_body.cuh"

namespace fvg {

namespace {

// block sizes are chosen per discretisation at run time (fv_disc_autotune);
// kMaxBS bounds them for register allocation
constexpr int kMaxBS = 256;

__global__ void __launch_bounds__(kMaxBS) k_prep(DiscDev D, const double *__restrict__ u, ResidualWork w)
{
	const int b = blockIdx.y;
	if (skip_member(D, b)) return;
	prep_body(D, b, blockIdx.x * blockDim.x + threadIdx.x, u, w);
}

/* k_prep at the matrix-free product's perturbed state u + pm x, formed on the
 * fly (the same sum the separate perturbation kernel stores) */
__global__ void __launch_bounds__(kMaxBS) k_prep_mf(DiscDev D, const double *__restrict__ u,
                                                    const double *__restrict__ x, const double *__restrict__ pm,
                                                    ResidualWork w)
{
	const int b = blockIdx.y;
	if (skip_member(D, b)) return;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	const Phys &P = D.phys[b];
	const double p = pm[b];
	const size_t c0 = (size_t)b * D.nelem;
	auto state = [&](int i, double *uc) {
		const d4 a = reinterpret_cast<const d4 *>(u)[c0 + i], v = reinterpret_cast<const d4 *>(x)[c0 + i];
		uc[0] = a.x + p * v.x;
		uc[1] = a.y + p * v.y;
		uc[2] = a.z + p * v.z;
		uc[3] = a.w + p * v.w;
	};
	if (t < D.nelem) {
		double uc[4], up[4];
		state(t, uc);
		prim_of_cons(P, uc, up);
		w.prim[c0 + t] = d4{up[0], up[1], up[2], up[3]};
	} else if (t < D.nelem + D.nbface) {
		const int ib = t - D.nelem;
		double in[4];
		state(D.flr[ib].x, in);
		const d4 g = D.fgeo[ib];
		const double n[2] = {g.x, g.y};
		double gs[4], gp[4];
		ghost_cons<double>(P, D.bcs[D.bcid[ib]], in, n, gs, false);
		prim_of_cons(P, gs, gp);
		w.ghost_cons[(size_t)b * D.nbface + ib] = d4{gs[0], gs[1], gs[2], gs[3]};
		w.ghost_prim[(size_t)b * D.nbface + ib] = d4{gp[0], gp[1], gp[2], gp[3]};
	}
}

__global__ void __launch_bounds__(kMaxBS) k_grad(DiscDev D, const d4 *__restrict__ q, const d4 *__restrict__ qg,
                                                 d4 *__restrict__ grad, d4 *__restrict__ lgrad, int limiter)
{
	const int b = blockIdx.y;
	if (skip_member(D, b)) return;
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= D.nelem) return;
	grad_body(D, b, i, q, qg, grad, lgrad, limiter);
}

__global__ void __launch_bounds__(kMaxBS) k_weno(DiscDev D, const d4 *__restrict__ grad, d4 *__restrict__ lgrad)
{
	const int b = blockIdx.y;
	if (skip_member(D, b)) return;
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= D.nelem) return;
	weno_body(D, b, i, grad, lgrad);
}

template <int FLUX, int VISC>
__global__ void __launch_bounds__(kMaxBS) k_face(DiscDev D, const double *__restrict__ u, ResidualWork w, int getdt)
{
	const int b = blockIdx.y;
	if (skip_member(D, b)) return;
	const int f = blockIdx.x * blockDim.x + threadIdx.x;
	if (f >= D.naface) return;
	face_body<FLUX, VISC>(D, b, f, u, w, getdt);
}

__global__ void __launch_bounds__(kMaxBS) k_gather(DiscDev D, ResidualWork w, double *__restrict__ r,
                                                   double *__restrict__ dt)
{
	const int b = blockIdx.y;
	if (skip_member(D, b)) return;
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= D.nelem) return;
	gather_body(D, b, i, w, r, dt);
}

/* The matrix-free product's last step fused into the gather: with a the
 * gathered -R(u + pm x) of cell i, y_i = dtm_i x_i + (r_i - a) / pm, r = -R(u)
 * (MatrixFreeSpatialJacobian::apply, alinalg.cpp:200-230) */
__global__ void __launch_bounds__(kMaxBS) k_gather_mf(DiscDev D, ResidualWork w, const double *__restrict__ x,
                                                      const double *__restrict__ r, const double *__restrict__ dtm,
                                                      const double *__restrict__ pm, double *__restrict__ y)
{
	const int b = blockIdx.y;
	if (skip_member(D, b)) return;
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= D.nelem) return;
	const int4 cf = D.cface[i];
	const int fl[4] = {cf.x, cf.y, cf.z, cf.w};
	double a[4] = {0, 0, 0, 0};
	const d4 *ff = w.fflux + (size_t)b * D.naface;
	for (int j = 0; j < 4; j++) {
		if (fl[j] < 0) continue;
		const int f = fl[j] >> 1, side = fl[j] & 1;
		const d4 F = ff[f];
		if (side) { a[0] += F.x; a[1] += F.y; a[2] += F.z; a[3] += F.w; }
		else { a[0] -= F.x; a[1] -= F.y; a[2] -= F.z; a[3] -= F.w; }
	}
	const size_t c = (size_t)b * D.nelem + i;
	const d4 xv = reinterpret_cast<const d4 *>(x)[c], rv = reinterpret_cast<const d4 *>(r)[c];
	const double dv = dtm[c], p = pm[b];
	// the gathered value is 0 + a, as in the unfused gather into a zeroed vector
	reinterpret_cast<d4 *>(y)[c] = d4{dv * xv.x + (-(0.0 + a[0]) + rv.x) / p, dv * xv.y + (-(0.0 + a[1]) + rv.y) / p,
	                                 dv * xv.z + (-(0.0 + a[2]) + rv.z) / p, dv * xv.w + (-(0.0 + a[3]) + rv.w) / p};
}

template <int FLUX>
void launch_face(fv_disc_impl *Dh, const ResidualWork &W, const double *u, int getdt, dim3 grid, int bs,
                 cudaStream_t s)
{
	const DiscDev &D = Dh->d;
	const int visc = !D.viscous ? 0 : (D.constvisc ? 2 : 1);
	if (visc == 0) k_face<FLUX, 0><<<grid, bs, 0, s>>>(D, u, W, getdt);
	else if (visc == 1) k_face<FLUX, 1><<<grid, bs, 0, s>>>(D, u, W, getdt);
	else k_face<FLUX, 2><<<grid, bs, 0, s>>>(D, u, W, getdt);
}

/* grid of n items in blocks of bs, one row per batch member */
dim3 grid_of(int n, int bs, int batch) { return dim3((unsigned)((n + bs - 1) / bs), (unsigned)batch); }

}  // namespace

cudaError_t face_launch(fv_disc_impl *Dh, const double *u, int gettimesteps, cudaStream_t s, const ResidualWork *w)
{
	const DiscDev &D = Dh->d;
	const ResidualWork &W = w ? *w : Dh->w;
	const int bs = Dh->bs[KBS_FACE];
	const dim3 gf = grid_of(D.naface, bs, Dh->batch);
	switch (D.flux) {
	case FLUX_LLF: launch_face<FLUX_LLF>(Dh, W, u, gettimesteps, gf, bs, s); break;
	case FLUX_VANLEER: launch_face<FLUX_VANLEER>(Dh, W, u, gettimesteps, gf, bs, s); break;
	case FLUX_AUSM: launch_face<FLUX_AUSM>(Dh, W, u, gettimesteps, gf, bs, s); break;
	case FLUX_AUSMPLUS: launch_face<FLUX_AUSMPLUS>(Dh, W, u, gettimesteps, gf, bs, s); break;
	case FLUX_ROE: launch_face<FLUX_ROE>(Dh, W, u, gettimesteps, gf, bs, s); break;
	case FLUX_HLL: launch_face<FLUX_HLL>(Dh, W, u, gettimesteps, gf, bs, s); break;
	default: launch_face<FLUX_HLLC>(Dh, W, u, gettimesteps, gf, bs, s); break;
	}
	return cudaGetLastError();
}

/* the residual's passes before the face kernel: primitive and ghost states,
 * gradients (+ Barth-Jespersen / Venkatakrishnan limiter values), WENO blend */
cudaError_t gradient_pass_launch(fv_disc_impl *Dh, const double *u, cudaStream_t s, const double *x,
                                 const double *pm, const ResidualWork *w)
{
	const DiscDev &D = Dh->d;
	const ResidualWork &W = w ? *w : Dh->w;
	const int B = Dh->batch;
	const int bp = Dh->bs[KBS_PREP], bg = Dh->bs[KBS_GRAD];
	int nk = 0;
	if (x) k_prep_mf<<<grid_of(D.nelem + D.nbface, bp, B), bp, 0, s>>>(D, u, x, pm, W);
	else k_prep<<<grid_of(D.nelem + D.nbface, bp, B), bp, 0, s>>>(D, u, W);
	nk++;
	if (D.gradscheme != GRAD_NONE) {
		const int lim = D.recon == REC_BARTHJESPERSEN || D.recon == REC_VENKATAKRISHNAN;
		k_grad<<<grid_of(D.nelem, bg, B), bg, 0, s>>>(D, W.prim, W.ghost_prim, W.grad, W.lgrad, lim);
		nk++;
		if (D.recon == REC_WENO) {
			k_weno<<<grid_of(D.nelem, bg, B), bg, 0, s>>>(D, W.grad, W.lgrad);
			nk++;
		}
	} else {
		// no gradients: every face value equals the cell value
		cudaMemsetAsync(W.grad, 0, sizeof(d4) * 2 * (size_t)D.nelem * B, s);
		if (recon_gradients(D.recon)) cudaMemsetAsync(W.lgrad, 0, sizeof(d4) * 2 * (size_t)D.nelem * B, s);
	}
	Dh->kernels_launched += nk;
	return cudaGetLastError();
}

cudaError_t residual_launch(fv_disc_impl *Dh, const double *u, double *r, int gettimesteps, double *dt, cudaStream_t s,
                            const ResidualWork *w)
{
	const DiscDev &D = Dh->d;
	const ResidualWork &W = w ? *w : Dh->w;
	if (D.order2) {
		const cudaError_t e = gradient_pass_launch(Dh, u, s, nullptr, nullptr, &W);
		if (e) return e;
	}
	face_launch(Dh, u, gettimesteps, s, &W);
	const int bc = Dh->bs[KBS_GATHER];
	k_gather<<<grid_of(D.nelem, bc, Dh->batch), bc, 0, s>>>(D, W, r, gettimesteps ? dt : nullptr);
	Dh->kernels_launched += 2;
	return cudaGetLastError();
}

/* y = dtm x + (R(u + pm x) - R(u)) / pm with r = -R(u): the residual's passes
 * at the perturbed state with the matrix-free finish fused into the gather.
 * Second order: the perturbed state is formed inside the first pass (the
 * later passes read only primitive and ghost states); first order: the face
 * kernel reads the state, so up = u + pm x must have been stored. */
cudaError_t residual_mf_launch(fv_disc_impl *Dh, const double *u, const double *up, const double *x,
                               const double *r, const double *dtm, const double *pm, double *y, cudaStream_t s)
{
	const DiscDev &D = Dh->d;
	if (D.order2) {
		const cudaError_t e = gradient_pass_launch(Dh, u, s, x, pm);
		if (e) return e;
	}
	face_launch(Dh, up, 0, s);
	const int bc = Dh->bs[KBS_GATHER];
	k_gather_mf<<<grid_of(D.nelem, bc, Dh->batch), bc, 0, s>>>(D, Dh->w, x, r, dtm, pm, y);
	Dh->kernels_launched += 2;
	return cudaGetLastError();
}

/* FlowFV_base::getGradients (flow_spatial.cpp:95-112) when conserved != 0:
 * gradients of the conserved variables with ghost states from cell values;
 * otherwise the primitive-variable gradients the residual uses. */
cudaError_t gradients_launch(fv_disc_impl *Dh, const double *u, double *grad, int conserved, cudaStream_t s)
{
	const DiscDev &D = Dh->d;
	const int B = Dh->batch;
	auto grid = [&](int n) { return grid_of(n, 128, B); };
	constexpr int BS = 128;
	k_prep<<<grid(D.nelem + D.nbface), BS, 0, s>>>(D, u, Dh->w);
	const d4 *q = conserved ? reinterpret_cast<const d4 *>(u) : Dh->w.prim;
	const d4 *qg = conserved ? Dh->w.ghost_cons : Dh->w.ghost_prim;
	if (D.gradscheme == GRAD_NONE) {
		cudaMemsetAsync(grad, 0, sizeof(double) * 8 * (size_t)D.nelem * B, s);
		Dh->kernels_launched += 1;
	} else {
		k_grad<<<grid(D.nelem), BS, 0, s>>>(D, q, qg, reinterpret_cast<d4 *>(grad), Dh->w.lgrad, 0);
		Dh->kernels_launched += 2;
	}
	return cudaGetLastError();
}

}  // namespace fvg

namespace fvg {

/* Launch-geometry autotuner of the residual kernels and of the Jacobian's
 * face kernel: each runs with 64, 128 and 256 threads per block at state u
 * (one warm-up, then three timed launches with CUDA events) and keeps the
 * fastest.  Every thread does the work of one cell or face whatever the block
 * size, so the choice changes timing, not results.  The Jacobian is timed into
 * a temporary FP32 matrix. */
cudaError_t residual_autotune(fv_disc_impl *Dh, const double *u, cudaStream_t s, int *chosen)
{
	const DiscDev &D = Dh->d;
	const int B = Dh->batch;
	const int cand[3] = {64, 128, 256};
	double *r = nullptr;
	cudaError_t e = cudaMalloc(&r, sizeof(double) * 4 * (size_t)D.nelem * B);
	if (!e) e = gradient_pass_launch(Dh, u, s);  // fill the scratch the later kernels read
	// temporary FP32 matrix for timing the Jacobian
	BlockMatrix J;
	J.nelem = D.nelem; J.batch = B; J.prec = 4;
	if (!e) e = cudaMalloc(&J.val, sizeof(float) * J.nval());
	if (!e) e = cudaMalloc(&J.bdiag, sizeof(double) * 16 * (size_t)B * (D.nbface > 0 ? D.nbface : 1));
	cudaEvent_t a, b;
	cudaEventCreate(&a);
	cudaEventCreate(&b);
	const int lim = D.recon == REC_BARTHJESPERSEN || D.recon == REC_VENKATAKRISHNAN;
	auto launch = [&](int kind, int bs) {
		switch (kind) {
		case KBS_PREP: k_prep<<<grid_of(D.nelem + D.nbface, bs, B), bs, 0, s>>>(D, u, Dh->w); break;
		case KBS_GRAD:
			if (D.order2) k_grad<<<grid_of(D.nelem, bs, B), bs, 0, s>>>(D, Dh->w.prim, Dh->w.ghost_prim, Dh->w.grad,
			                                                              Dh->w.lgrad, lim);
			break;
		case KBS_FACE: Dh->bs[KBS_FACE] = bs; face_launch(Dh, u, 1, s); break;
		case KBS_JAC: Dh->bs[KBS_JAC] = bs; return jacobian_launch(Dh, u, J, s);
		default: k_gather<<<grid_of(D.nelem, bs, B), bs, 0, s>>>(D, Dh->w, r, nullptr); break;
		}
		return cudaGetLastError();
	};
	for (int kind = 0; kind < KBS_COUNT && !e; kind++) {
		float best = 1e30f;
		int pick = Dh->bs[kind];
		for (int c = 0; c < 3 && !e; c++) {
			e = launch(kind, cand[c]);
			if (!e) e = cudaEventRecord(a, s);
			for (int k = 0; k < 3 && !e; k++) e = launch(kind, cand[c]);
			if (!e) e = cudaEventRecord(b, s);
			if (!e) e = cudaEventSynchronize(b);
			float ms = 0;
			if (!e) e = cudaEventElapsedTime(&ms, a, b);
			if (!e && ms < best) { best = ms; pick = cand[c]; }
		}
		Dh->bs[kind] = pick;
		if (chosen && kind < 4) chosen[kind] = pick;
	}
	Dh->kernels_launched += 4 * 3 * 4 + 2;  // the Jacobian's launches count themselves
	if (J.val) cudaFree(J.val);
	if (J.bdiag) cudaFree(J.bdiag);
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	if (r) cudaFree(r);
	return e;
}

}  // namespace fvg
