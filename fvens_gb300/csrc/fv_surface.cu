/*
 * Wall surface functionals: lift, pressure drag and skin-friction drag
 * coefficients over the faces of one boundary marker, FP64, for every member
 * of the batch (FlowFV_base::computeSurfaceData, flow_spatial.cpp:130-310 of
 * the reference), and its per-face output (x, y, Cp, Cf) for the surface files
 * of FlowOutput::exportSurfaceData (aoutput.cpp:181-238).
 *
 * Per wall face f with unit normal n, length len, tangent t = (n_y, -n_x),
 * cell-centred conserved state u of its interior cell and that cell's
 * conserved gradients (getGradients, flow_spatial.cpp:95-112):
 *   Cp   = 2 (p(u) - p_inf)
 *   Cf   = 2 mu(T(u)) ((grad v + grad v^T) n) . t,
 *          grad v_ij = (d_j(rho v_i) rho - rho v_i d_j rho) / rho^2
 *   Cl   = sum Cp (n . w_perp) len / sum len,   w = (cos aoa, sin aoa),
 *   CDp  = sum Cp (n . w) len / sum len,        w_perp = (-w_y, w_x)
 *   CDsf = sum Cf (t . w) len / sum len
 * The sums are a fixed-order tree reduction (one CTA per member), so results
 * are bitwise reproducible.
 *
 * Also the entropy error sqrt(sum_i ((s_i - s_inf)/s_inf)^2 A_i), s = p/rho^gamma
 * (FlowOutput::compute_entropy_cell, aoutput.cpp:28-62), the accuracy measure
 * of the reference's grid-convergence tests.
 */
#include <algorithm>
#include <cmath>
#include <vector>

#include <cuda_runtime.h>

#include "fv_abi_internal.hpp"

namespace fvg {
namespace {

constexpr int SBS = 256;

/* Cp and Cf of wall face f of member b from its interior cell's state and
 * conserved gradients (the per-face part of computeSurfaceData) */
__device__ __forceinline__ void wall_face(const DiscDev &D, const Phys &P, const double *__restrict__ u,
                                          const d4 *__restrict__ grad, int b, int f, double &cp, double &cf)
{
	const size_t N = D.nelem;
	const int le = D.flr[f].x;
	const d4 g4 = D.fgeo[f];
	const double nx = g4.x, ny = g4.y;
	const double tx = ny, ty = -nx;
	const d4 uc = reinterpret_cast<const d4 *>(u)[(size_t)b * N + le];
	const double rho = uc.x;
	const double p = P.gm1 * (uc.w - 0.5 * (uc.y * uc.y + uc.z * uc.z) / rho);
	cp = (p - P.pinf) * 2.0;
	const double Tt = P.tcoef * p / rho;
	const double mu = P.sutK / (Tt + P.sutC) * Tt * sqrt(Tt);
	// conserved gradients, 2x4 column-major: (d_x q0, d_y q0, d_x q1, d_y q1), (d_x q2, d_y q2, ...)
	const d4 g0 = grad[2 * ((size_t)b * N + le)], g1 = grad[2 * ((size_t)b * N + le) + 1];
	const double dr[2] = {g0.x, g0.y}, dmu[2] = {g0.z, g0.w}, dmv[2] = {g1.x, g1.y};
	const double mom[2] = {uc.y, uc.z};
	const double *dm[2] = {dmu, dmv};
	double gu[2][2];
	for (int i = 0; i < 2; i++)
		for (int j = 0; j < 2; j++) gu[i][j] = (dm[i][j] * rho - mom[i] * dr[j]) / (rho * rho);
	const double nn[2] = {nx, ny};
	double force[2];
	for (int i = 0; i < 2; i++) {
		force[i] = 0;
		for (int j = 0; j < 2; j++) force[i] += (gu[i][j] + gu[j][i]) * nn[j];
	}
	cf = 2.0 * mu * (force[0] * tx + force[1] * ty);
}

__global__ void __launch_bounds__(SBS) k_surface(DiscDev D, const double *__restrict__ u, const d4 *__restrict__ grad,
                                                  const int *__restrict__ btag, int marker, double *__restrict__ out)
{
	const int b = blockIdx.x;
	const Phys P = D.phys[b];
	const double wx = cos(P.aoa), wy = sin(P.aoa);
	const double fnx = -wy, fny = wx;
	double acc[4] = {0, 0, 0, 0};  // Cl, CDp, CDsf, total length
	for (int f = threadIdx.x; f < D.nbface; f += SBS) {
		if (btag[f] != marker) continue;
		const d4 g4 = D.fgeo[f];
		const double nx = g4.x, ny = g4.y, len = g4.z;
		const double tx = ny, ty = -nx;
		double cp, cf;
		wall_face(D, P, u, grad, b, f, cp, cf);
		acc[0] += cp * (nx * fnx + ny * fny) * len;
		acc[1] += cp * (nx * wx + ny * wy) * len;
		acc[2] += cf * (tx * wx + ty * wy) * len;
		acc[3] += len;
	}
	__shared__ double sh[4][SBS];
	for (int k = 0; k < 4; k++) sh[k][threadIdx.x] = acc[k];
	__syncthreads();
	for (int o = SBS / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o)
			for (int k = 0; k < 4; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x < 4) out[4 * b + threadIdx.x] = sh[threadIdx.x][0];
}

/* per-face rows (x, y, Cp, Cf) of the listed wall faces of member b: the
 * output array of computeSurfaceData (flow_spatial.cpp:168-237) */
__global__ void __launch_bounds__(SBS) k_surface_faces(DiscDev D, const double *__restrict__ u,
                                                        const d4 *__restrict__ grad, const int *__restrict__ faces,
                                                        int nw, int b, double *__restrict__ out)
{
	const int k = blockIdx.x * SBS + threadIdx.x;
	if (k >= nw) return;
	const int f = faces[k];
	double cp, cf;
	wall_face(D, D.phys[b], u, grad, b, f, cp, cf);
	const double2 c = D.fcen[f];
	out[4 * k] = c.x;
	out[4 * k + 1] = c.y;
	out[4 * k + 2] = cp;
	out[4 * k + 3] = cf;
}

/* entropy error partials: sum over cells of ((s - s_inf)/s_inf)^2 A, s = p / rho^gamma
 * (FlowOutput::compute_entropy_cell, aoutput.cpp:28-62) */
__global__ void __launch_bounds__(SBS) k_entropy_partial(DiscDev D, const double *__restrict__ u, int nblk,
                                                         double *__restrict__ part)
{
	const int b = blockIdx.y;
	const Phys P = D.phys[b];
	const double sinf = P.pinf_cons / pow(P.uinf[0], P.g);  // entropy of the freestream state
	double acc = 0;
	for (int i = blockIdx.x * SBS + threadIdx.x; i < D.nelem; i += nblk * SBS) {
		const d4 uc = reinterpret_cast<const d4 *>(u)[(size_t)b * D.nelem + i];
		const double p = P.gm1 * (uc.w - 0.5 * (uc.y * uc.y + uc.z * uc.z) / uc.x);
		const double e = (p / pow(uc.x, P.g) - sinf) / sinf;
		acc += e * e * D.area[i];
	}
	__shared__ double sh[SBS];
	sh[threadIdx.x] = acc;
	__syncthreads();
	for (int o = SBS / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0) part[(size_t)b * nblk + blockIdx.x] = sh[0];
}

}  // namespace
}  // namespace fvg

using namespace fvg;

extern "C" fv_status fv_entropy_error(fv_disc *D, const double *u, double *h_err)
{
	if (!D || !u || !h_err) { set_error("null argument"); return FV_ERR_INVALID; }
	const int B = D->batch;
	const int nblk = std::max(1, std::min(256, (D->d.nelem + SBS * 8 - 1) / (SBS * 8)));
	double *part = reinterpret_cast<double *>(D->w.fflux);  // residual scratch: >= 4 * naface doubles per member
	if ((size_t)nblk > 4 * (size_t)D->d.naface) { set_error("mesh too small for the entropy reduction"); return FV_ERR_INVALID; }
	k_entropy_partial<<<dim3(nblk, B), SBS, 0, D->stream>>>(D->d, u, nblk, part);
	count_launches(1);
	std::vector<double> h((size_t)nblk * B);
	cudaError_t e = cudaGetLastError();
	if (!e) e = cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, D->stream);
	if (!e) e = cudaStreamSynchronize(D->stream);
	if (e) return cuda_status(e, "entropy error");
	for (int b = 0; b < B; b++) {
		double s = 0;
		for (int k = 0; k < nblk; k++) s += h[(size_t)b * nblk + k];
		h_err[b] = sqrt(s);
	}
	return FV_OK;
}

extern "C" fv_status fv_surface_data(fv_disc *D, const double *u, int marker, double *h_out)
{
	if (!D || !u || !h_out) { set_error("null argument"); return FV_ERR_INVALID; }
	const int B = D->batch;
	bool found = false;
	for (int t : D->mesh->h.btag) found = found || t == marker;
	if (!found) { set_error("no boundary face has marker " + std::to_string(marker)); return FV_ERR_INVALID; }
	const int before = D->kernels_launched;
	// conserved gradients into the residual scratch (as FlowFV_base::getGradients)
	cudaError_t e = gradients_launch(D, u, reinterpret_cast<double *>(D->w.grad), 1, D->stream);
	if (!e) {
		k_surface<<<B, SBS, 0, D->stream>>>(D->d, u, D->w.grad, D->btag, marker, D->surf);
		D->kernels_launched++;
		e = cudaGetLastError();
	}
	count_launches(D->kernels_launched - before);
	std::vector<double> s(4 * (size_t)B);
	if (!e) e = cudaMemcpyAsync(s.data(), D->surf, sizeof(double) * 4 * B, cudaMemcpyDeviceToHost, D->stream);
	if (!e) e = cudaStreamSynchronize(D->stream);
	if (e) return cuda_status(e, "surface data");
	for (int b = 0; b < B; b++)
		for (int k = 0; k < 3; k++) h_out[3 * b + k] = s[4 * b + k] / s[4 * b + 3];
	return FV_OK;
}

/* per-face (x, y, Cp, Cf) of the faces of one wall marker for one member */
extern "C" fv_status fv_surface_distribution(fv_disc *D, const double *u, int marker, int member, double *h_out,
                                             int *nfaces)
{
	if (!D || !nfaces || (h_out && !u) || member < 0 || member >= D->batch) {
		set_error("invalid argument");
		return FV_ERR_INVALID;
	}
	std::vector<int> faces;
	const std::vector<int> &bt = D->mesh->h.btag;
	for (int f = 0; f < (int)bt.size(); f++)
		if (bt[f] == marker) faces.push_back(f);
	*nfaces = (int)faces.size();
	if (faces.empty()) { set_error("no boundary face has marker " + std::to_string(marker)); return FV_ERR_INVALID; }
	if (!h_out) return FV_OK;
	const int nw = (int)faces.size();
	int *df = nullptr;
	double *dout = nullptr;
	cudaError_t e = cudaMalloc(&df, sizeof(int) * nw);
	if (!e) e = cudaMalloc(&dout, sizeof(double) * 4 * nw);
	if (!e) e = cudaMemcpyAsync(df, faces.data(), sizeof(int) * nw, cudaMemcpyHostToDevice, D->stream);
	const int before = D->kernels_launched;
	if (!e) e = gradients_launch(D, u, reinterpret_cast<double *>(D->w.grad), 1, D->stream);
	if (!e) {
		k_surface_faces<<<(nw + SBS - 1) / SBS, SBS, 0, D->stream>>>(D->d, u, D->w.grad, df, nw, member, dout);
		D->kernels_launched++;
		e = cudaGetLastError();
	}
	count_launches(D->kernels_launched - before);
	if (!e) e = cudaMemcpyAsync(h_out, dout, sizeof(double) * 4 * nw, cudaMemcpyDeviceToHost, D->stream);
	if (!e) e = cudaStreamSynchronize(D->stream);
	if (df) cudaFree(df);
	if (dout) cudaFree(dout);
	return e ? cuda_status(e, "surface distribution") : FV_OK;
}
