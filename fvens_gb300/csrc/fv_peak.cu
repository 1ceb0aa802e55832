/*
 * FP64 throughput ceiling of the device: a measurement aid for the roofline
 * of the FP64-bound residual kernels (no counterpart in the reference).
 *
 * k_fp64_peak keeps eight independent fused multiply-add chains per thread
 * (x <- x a + b with |a| < 1, so the values stay bounded), unrolled so that
 * the loop overhead is a few percent of the issued instructions, on a full
 * machine of resident warps (8 CTAs of 256 threads per SM).  The sum of the
 * chains is compared against a value it never takes, so that the chains stay
 * live without a store in the timed loop.
 */
#include "fv_abi_internal.hpp"

namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 16;
constexpr int kThreads = 256;
constexpr int kCtasPerSm = 8;

__global__ void __launch_bounds__(kThreads) k_fp64_peak(double *sink, int iters, double a, double b)
{
	double x[kChains];
#pragma unroll
	for (int c = 0; c < kChains; c++) x[c] = 1e-3 * (double)(threadIdx.x + c);
	for (int i = 0; i < iters; i++) {
#pragma unroll
		for (int k = 0; k < kUnroll; k++) {
#pragma unroll
			for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
		}
	}
	double s = 0;
#pragma unroll
	for (int c = 0; c < kChains; c++) s += x[c];
	if (s == -1.0) sink[0] = s;  // never true for these inputs
}

}  // namespace

using namespace fvg;

extern "C" fv_status fv_fp64_peak(int reps, double *h_dfma_per_s, double *h_best_ms)
{
	if (!h_dfma_per_s || reps < 1) { set_error("null argument or reps < 1"); return FV_ERR_INVALID; }
	int dev = 0, nsm = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (!e) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
	if (e) return cuda_status(e, "fp64 peak: device query");
	double *sink = nullptr;
	e = cudaMalloc(&sink, sizeof(double));
	if (e) return cuda_status(e, "fp64 peak: allocation");
	cudaStream_t s = nullptr;
	cudaEvent_t t0 = nullptr, t1 = nullptr;
	e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
	if (!e) e = cudaEventCreate(&t0);
	if (!e) e = cudaEventCreate(&t1);
	const int iters = 256;
	const dim3 grid((unsigned)(nsm * kCtasPerSm));
	const double per_launch = (double)grid.x * kThreads * iters * kUnroll * kChains;
	float best = 1e30f;
	for (int r = -1; r < reps && !e; r++) {  // r = -1: untimed warm-up
		e = cudaEventRecord(t0, s);
		if (!e) k_fp64_peak<<<grid, kThreads, 0, s>>>(sink, iters, 0.9999999, 1e-7);
		if (!e) e = cudaGetLastError();
		if (!e) e = cudaEventRecord(t1, s);
		if (!e) e = cudaEventSynchronize(t1);
		float ms = 0;
		if (!e) e = cudaEventElapsedTime(&ms, t0, t1);
		if (!e && r >= 0 && ms < best) best = ms;
	}
	count_launches(reps + 1);
	if (t0) cudaEventDestroy(t0);
	if (t1) cudaEventDestroy(t1);
	if (s) cudaStreamDestroy(s);
	cudaFree(sink);
	if (e) return cuda_status(e, "fp64 peak");
	*h_dfma_per_s = per_launch / (best * 1e-3);
	if (h_best_ms) *h_best_ms = best;
	return FV_OK;
}
