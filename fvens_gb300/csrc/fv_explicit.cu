/*
 * Explicit time stepping on the GPU, batched over the conditions of a
 * discretisation:
 *   - SteadyForwardEulerSolver::solve (src/ode/aodesolver.cpp:136-282):
 *     u += cflinit dt_i / A_i r, r = -R(u), dt_i the local time steps; the
 *     CFL the reference ramps is never used by its update, so the step uses
 *     the initial CFL; the loop runs while the energy-residual norm (relative
 *     to the first step's, or absolute) exceeds the tolerance, and stopping at
 *     max_timesteps is a tolerance failure, as there.
 *   - TVDRKSolver::solve (:671-765, coefficients :45-67) as the reference
 *     has it: each stage evaluates the residual of the step's starting state,
 *     the step is dtmin * cfl with dtmin the smallest local time step of the
 *     first stage, and a stage sets ustage = c0 u + c1 ustage - c2 dtmin cfl
 *     / A r, until the elapsed time exceeds final_time - 1e-12.
 * Per-member step counters, norms, minima and flags live on the device; the
 * host polls the flags every few steps.
 */
#include <cmath>
#include <vector>

#include "fv_abi_internal.hpp"

namespace fvg {
namespace {

constexpr int EBS = 256;
constexpr int kPoll = 16;  // steps between host polls of the member flags

struct ExState {
	double *res, *res0, *time, *dtmin;  // [batch]
	int *step, *status, *active;        // [batch]
	double *part;                       // [batch][nblk]
	double *hist;                       // [maxiter][batch] residual norms (forward Euler)
};

__device__ __forceinline__ double block_reduce_sum(double s)
{
	__shared__ double sh[EBS];
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int o = EBS / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
		__syncthreads();
	}
	return sh[0];
}

/* forward Euler update u += cfl dt/A r and partial sums of r_3^2 A */
__global__ void __launch_bounds__(EBS) k_fe_update(int N, int nblk, double *__restrict__ u, const double *__restrict__ r,
                                                   const double *__restrict__ dt, const double *__restrict__ area,
                                                   double cfl, ExState S)
{
	const int b = blockIdx.y;
	if (!S.active[b]) return;
	double s = 0;
	for (int i = blockIdx.x * EBS + threadIdx.x; i < N; i += nblk * EBS) {
		const size_t k = (size_t)b * N + i;
		const double f = cfl * dt[k] * 1.0 / area[i];
		const double4 rv = reinterpret_cast<const double4 *>(r)[k];
		double4 uv = reinterpret_cast<double4 *>(u)[k];
		uv.x += f * rv.x; uv.y += f * rv.y; uv.z += f * rv.z; uv.w += f * rv.w;
		reinterpret_cast<double4 *>(u)[k] = uv;
		s += rv.w * rv.w * area[i];
	}
	s = block_reduce_sum(s);
	if (threadIdx.x == 0) S.part[(size_t)b * nblk + blockIdx.x] = s;
}

/* norm, NaN check, loop condition of the forward Euler solve */
__global__ void k_fe_norm(int B, int nblk, ExState S, double tol, int abs_tol, int maxiter)
{
	const int b = blockIdx.x * blockDim.x + threadIdx.x;
	if (b >= B || !S.active[b]) return;
	double s = 0;
	for (int k = 0; k < nblk; k++) s += S.part[(size_t)b * nblk + k];
	const double res = sqrt(s);
	const int step = S.step[b];
	if (step == 0) S.res0[b] = res;
	if (S.hist) S.hist[(size_t)step * B + b] = res;
	S.res[b] = res;
	S.step[b] = step + 1;
	if (!isfinite(res)) {
		S.status[b] = FV_ERR_NUMERICAL;
		S.active[b] = 0;
		return;
	}
	const bool more = (abs_tol ? res > tol : res / S.res0[b] > tol) && step + 1 < maxiter;
	if (!more) {
		S.active[b] = 0;
		S.status[b] = step + 1 >= maxiter ? FV_ERR_TOLERANCE : FV_OK;
	}
}

/* partial minima of the local time steps; a NaN anywhere makes the minimum
 * NaN (the reference's std::min_element sees a NaN only in the first cell) */
__device__ __forceinline__ double nan_min(double a, double c) { return (isnan(a) || isnan(c)) ? NAN : fmin(a, c); }

__global__ void __launch_bounds__(EBS) k_min_partial(int N, int nblk, const double *__restrict__ dt, ExState S)
{
	const int b = blockIdx.y;
	if (!S.active[b]) return;
	double m = INFINITY;
	for (int i = blockIdx.x * EBS + threadIdx.x; i < N; i += nblk * EBS) m = nan_min(m, dt[(size_t)b * N + i]);
	__shared__ double sh[EBS];
	sh[threadIdx.x] = m;
	__syncthreads();
	for (int o = EBS / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) sh[threadIdx.x] = nan_min(sh[threadIdx.x], sh[threadIdx.x + o]);
		__syncthreads();
	}
	if (threadIdx.x == 0) S.part[(size_t)b * nblk + blockIdx.x] = sh[0];
}

__global__ void k_rk_dtmin(int B, int nblk, ExState S)
{
	const int b = blockIdx.x * blockDim.x + threadIdx.x;
	if (b >= B || !S.active[b]) return;
	double m = INFINITY;
	for (int k = 0; k < nblk; k++) m = nan_min(m, S.part[(size_t)b * nblk + k]);
	S.dtmin[b] = m;
	if (!isfinite(m)) {
		S.status[b] = FV_ERR_NUMERICAL;
		S.active[b] = 0;
	}
}

/* ustage = c0 u + c1 ustage - c2 dtmin cfl / A r */
__global__ void __launch_bounds__(EBS) k_rk_stage(int N, const double *__restrict__ u, double *__restrict__ us,
                                                  const double *__restrict__ r, const double *__restrict__ area,
                                                  double cfl, double c0, double c1, double c2, ExState S)
{
	const int b = blockIdx.y;
	const int i = blockIdx.x * EBS + threadIdx.x;
	if (i >= N || !S.active[b]) return;
	const double f = c2 * S.dtmin[b] * cfl / area[i];
	const size_t k = (size_t)b * N + i;
	const double4 uv = reinterpret_cast<const double4 *>(u)[k], rv = reinterpret_cast<const double4 *>(r)[k];
	double4 sv = reinterpret_cast<double4 *>(us)[k];
	sv.x = c0 * uv.x + c1 * sv.x - f * rv.x;
	sv.y = c0 * uv.y + c1 * sv.y - f * rv.y;
	sv.z = c0 * uv.z + c1 * sv.z - f * rv.z;
	sv.w = c0 * uv.w + c1 * sv.w - f * rv.w;
	reinterpret_cast<double4 *>(us)[k] = sv;
}

__global__ void __launch_bounds__(EBS) k_rk_accept(int N, double *__restrict__ u, const double *__restrict__ us,
                                                   ExState S)
{
	const int b = blockIdx.y;
	const int i = blockIdx.x * EBS + threadIdx.x;
	if (i >= N || !S.active[b]) return;
	const size_t k = (size_t)b * N + i;
	reinterpret_cast<double4 *>(u)[k] = reinterpret_cast<const double4 *>(us)[k];
}

__global__ void k_rk_time(int B, ExState S, double cfl, double final_time, int max_steps)
{
	const int b = blockIdx.x * blockDim.x + threadIdx.x;
	if (b >= B || !S.active[b]) return;
	S.step[b] += 1;
	S.time[b] += S.dtmin[b] * cfl;
	if (!(S.time[b] <= final_time - 1e-12)) S.active[b] = 0;
	else if (S.step[b] >= max_steps) {
		S.active[b] = 0;
		S.status[b] = FV_ERR_TOLERANCE;
	}
}

__global__ void k_ex_init(int B, ExState S, int on)
{
	const int b = blockIdx.x * blockDim.x + threadIdx.x;
	if (b >= B) return;
	S.res[b] = 1.0; S.res0[b] = 1.0; S.time[b] = 0.0; S.dtmin[b] = 0.0;
	S.step[b] = 0; S.status[b] = FV_OK; S.active[b] = on;
}

struct ExBuffers {
	std::vector<void *> ptrs;
	cudaError_t e = cudaSuccess;
	template <class T>
	T *get(size_t n)
	{
		void *p = nullptr;
		if (!e) e = cudaMalloc(&p, n * sizeof(T) > 0 ? n * sizeof(T) : 1);
		if (!e) ptrs.push_back(p);
		return static_cast<T *>(p);
	}
	~ExBuffers()
	{
		for (void *p : ptrs) cudaFree(p);
	}
};

}  // namespace
}  // namespace fvg

using namespace fvg;

extern "C" fv_status fv_steady_fe_solve(fv_disc *D, const fv_solver_cfg *cfg, double *u, fv_solve_stats *stats)
{
	if (!D || !cfg || !u) { set_error("null argument"); return FV_ERR_INVALID; }
	if (cfg->max_timesteps <= 0) { set_error("SteadyForwardEulerSolver: solve(): No iterations to be done."); return FV_ERR_INVALID; }
	const int N = D->d.nelem, B = D->batch, maxit = cfg->max_timesteps;
	const int nblk = std::max(1, std::min(1024, (N + EBS * 4 - 1) / (EBS * 4)));
	cudaStream_t s = D->stream;
	ExBuffers buf;
	double *r = buf.get<double>(4 * (size_t)N * B), *dt = buf.get<double>((size_t)N * B);
	ExState S;
	S.res = buf.get<double>(B); S.res0 = buf.get<double>(B); S.time = buf.get<double>(B); S.dtmin = buf.get<double>(B);
	S.step = buf.get<int>(B); S.status = buf.get<int>(B); S.active = buf.get<int>(B);
	S.part = buf.get<double>((size_t)B * nblk);
	S.hist = nullptr;
	if (buf.e) return cuda_status(buf.e, "forward Euler buffers");
	cudaError_t e = cudaSuccess;
	k_ex_init<<<(B + 31) / 32, 32, 0, s>>>(B, S, 1);
	long long nk = 1;
	const int *saved = D->d.active;
	D->d.active = S.active;
	std::vector<int> act(B);
	for (int done = 0; done < maxit && !e;) {
		const int chunk = std::min(kPoll, maxit - done);
		for (int k = 0; k < chunk && !e; k++) {
			e = cudaMemsetAsync(r, 0, sizeof(double) * 4 * (size_t)N * B, s);
			const int before = D->kernels_launched;
			if (!e) e = residual_launch(D, u, r, 1, dt, s);
			nk += D->kernels_launched - before;
			D->kernels_launched = before;
			k_fe_update<<<dim3(nblk, B), EBS, 0, s>>>(N, nblk, u, r, dt, D->d.area, cfg->cfl_min, S);
			k_fe_norm<<<(B + 31) / 32, 32, 0, s>>>(B, nblk, S, cfg->tolerance, cfg->abs_tolerance, maxit);
			nk += 2;
			if (!e) e = cudaGetLastError();
		}
		done += chunk;
		if (!e) e = cudaMemcpyAsync(act.data(), S.active, sizeof(int) * B, cudaMemcpyDeviceToHost, s);
		if (!e) e = cudaStreamSynchronize(s);
		bool any = false;
		for (int b = 0; b < B; b++) any = any || act[b];
		if (!any) break;
	}
	D->d.active = saved;
	count_launches(nk);
	std::vector<double> res(B), res0(B);
	std::vector<int> step(B), status(B);
	if (!e) e = cudaMemcpy(res.data(), S.res, sizeof(double) * B, cudaMemcpyDeviceToHost);
	if (!e) e = cudaMemcpy(res0.data(), S.res0, sizeof(double) * B, cudaMemcpyDeviceToHost);
	if (!e) e = cudaMemcpy(step.data(), S.step, sizeof(int) * B, cudaMemcpyDeviceToHost);
	if (!e) e = cudaMemcpy(status.data(), S.status, sizeof(int) * B, cudaMemcpyDeviceToHost);
	if (e) return cuda_status(e, "forward Euler solve");
	fv_status worst = FV_OK;
	for (int b = 0; b < B; b++) {
		if (stats) {
			stats[b].steps = step[b]; stats[b].lin_iters = 0; stats[b].status = status[b];
			stats[b].res0 = res0[b]; stats[b].res = res[b]; stats[b].cfl = cfg->cfl_min;
		}
		if (status[b] == FV_ERR_NUMERICAL) worst = FV_ERR_NUMERICAL;
		else if (status[b] == FV_ERR_TOLERANCE && worst == FV_OK) worst = FV_ERR_TOLERANCE;
	}
	if (worst == FV_ERR_NUMERICAL) set_error("Steady forward Euler diverged - residual is Nan or inf!");
	else if (worst == FV_ERR_TOLERANCE) set_error("Steady forward Euler did not converge to specified tolerance!");
	return worst;
}

extern "C" fv_status fv_tvdrk_solve(fv_disc *D, int order, double cfl, double final_time, int max_steps, double *u,
                                    int *h_steps, double *h_time)
{
	if (!D || !u) { set_error("null argument"); return FV_ERR_INVALID; }
	if (order < 1 || order > 3) { set_error("! Temporal order not available!"); return FV_ERR_INVALID; }
	if (max_steps < 1) { set_error("max_steps must be positive"); return FV_ERR_INVALID; }
	double co[3][3] = {{1, 0, 1}, {0, 0, 0}, {0, 0, 0}};
	if (order == 2) { co[1][0] = 0.5; co[1][1] = 0.5; co[1][2] = 0.5; }
	if (order == 3) {
		co[1][0] = 0.75; co[1][1] = 0.25; co[1][2] = 0.25;
		co[2][0] = 0.3333333333333333; co[2][1] = 0.6666666666666667; co[2][2] = 0.6666666666666667;
	}
	const int N = D->d.nelem, B = D->batch;
	const int nblk = std::max(1, std::min(1024, (N + EBS * 4 - 1) / (EBS * 4)));
	cudaStream_t s = D->stream;
	ExBuffers buf;
	double *r = buf.get<double>(4 * (size_t)N * B), *dt = buf.get<double>((size_t)N * B);
	double *us = buf.get<double>(4 * (size_t)N * B);
	ExState S;
	S.res = buf.get<double>(B); S.res0 = buf.get<double>(B); S.time = buf.get<double>(B); S.dtmin = buf.get<double>(B);
	S.step = buf.get<int>(B); S.status = buf.get<int>(B); S.active = buf.get<int>(B);
	S.part = buf.get<double>((size_t)B * nblk);
	S.hist = nullptr;
	if (buf.e) return cuda_status(buf.e, "TVDRK buffers");
	cudaError_t e = cudaMemcpyAsync(us, u, sizeof(double) * 4 * (size_t)N * B, cudaMemcpyDeviceToDevice, s);
	k_ex_init<<<(B + 31) / 32, 32, 0, s>>>(B, S, final_time >= 1e-12 ? 1 : 0);
	long long nk = 1;
	const int *saved = D->d.active;
	D->d.active = S.active;
	const dim3 ge((N + EBS - 1) / EBS, B);
	std::vector<int> act(B, 1);
	for (int done = 0; done < max_steps && !e;) {
		const int chunk = std::min(kPoll, max_steps - done);
		for (int k = 0; k < chunk && !e; k++) {
			for (int st = 0; st < order && !e; st++) {
				e = cudaMemsetAsync(r, 0, sizeof(double) * 4 * (size_t)N * B, s);
				const int before = D->kernels_launched;
				if (!e) e = residual_launch(D, u, r, 1, dt, s);
				nk += D->kernels_launched - before;
				D->kernels_launched = before;
				if (st == 0) {
					k_min_partial<<<dim3(nblk, B), EBS, 0, s>>>(N, nblk, dt, S);
					k_rk_dtmin<<<(B + 31) / 32, 32, 0, s>>>(B, nblk, S);
					nk += 2;
				}
				k_rk_stage<<<ge, EBS, 0, s>>>(N, u, us, r, D->d.area, cfl, co[st][0], co[st][1], co[st][2], S);
				nk++;
			}
			k_rk_accept<<<ge, EBS, 0, s>>>(N, u, us, S);
			k_rk_time<<<(B + 31) / 32, 32, 0, s>>>(B, S, cfl, final_time, max_steps);
			nk += 2;
			if (!e) e = cudaGetLastError();
		}
		done += chunk;
		if (!e) e = cudaMemcpyAsync(act.data(), S.active, sizeof(int) * B, cudaMemcpyDeviceToHost, s);
		if (!e) e = cudaStreamSynchronize(s);
		bool any = false;
		for (int b = 0; b < B; b++) any = any || act[b];
		if (!any) break;
	}
	D->d.active = saved;
	count_launches(nk);
	std::vector<int> step(B), status(B);
	std::vector<double> tm(B);
	if (!e) e = cudaMemcpy(step.data(), S.step, sizeof(int) * B, cudaMemcpyDeviceToHost);
	if (!e) e = cudaMemcpy(status.data(), S.status, sizeof(int) * B, cudaMemcpyDeviceToHost);
	if (!e) e = cudaMemcpy(tm.data(), S.time, sizeof(double) * B, cudaMemcpyDeviceToHost);
	if (e) return cuda_status(e, "TVDRK solve");
	fv_status worst = FV_OK;
	for (int b = 0; b < B; b++) {
		if (h_steps) h_steps[b] = step[b];
		if (h_time) h_time[b] = tm[b];
		if (status[b] == FV_ERR_NUMERICAL) worst = FV_ERR_NUMERICAL;
		else if (status[b] == FV_ERR_TOLERANCE && worst == FV_OK) worst = FV_ERR_TOLERANCE;
	}
	if (worst == FV_ERR_NUMERICAL) set_error("TVDRK solver diverged - dtmin is Nan or inf!");
	else if (worst == FV_ERR_TOLERANCE) set_error("TVDRK solver: max_steps reached before final_time");
	return worst;
}
