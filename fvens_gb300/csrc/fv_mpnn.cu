/*
 * Learned warm start: a mesh message-passing network that predicts the
 * converged conserved state of a flow condition (M, AoA, Re) on a fixed mesh,
 * trained on states the steady solver itself converged.  No counterpart in
 * the reference; the solver then runs from the prediction (freestream stays
 * the fallback) and judges the result.
 *
 * Graph: cells are nodes, interior faces carry one message each way.
 *   node input  x_i = (cx, cy scaled by 1/(1+r), log10 area, log10 wall
 *                      distance, M, AoA, Re) (7, zero-padded to 16)
 *   encoder     h0 = relu(We x + be)                               64
 *   layer l     m_{s->d} = relu(Wm [h_s, h_d, e_sd] + bm)         131 -> 64
 *               a_d = sum of the messages into d
 *               h_{l+1} = h_l + relu(Wu [h_l, a] + bu)             128 -> 64
 *   decoder     y = Wd h + bd                                       64 -> 4
 *   e_sd = (nx, ny, log10 len) with the unit normal pointing from s to d.
 * y is the state's deviation from freestream, per variable over a scale the
 * caller sets (fv_mpnn_set_scale).
 *
 * Arithmetic: every contraction runs on the tensor cores as warp-level BF16
 * mma.sync (m16n8k16) with FP32 accumulation: GEMM operands (weights and
 * activations) are rounded to BF16 when they are staged in shared memory;
 * activations, biases, gradients and the Adam state stay FP32.  The GEMMs are
 * small (K <= 144, N = 64), far from the solver's hot path.
 * Reductions over rows (weight gradients, aggregation) run in fixed order.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "fv_abi_internal.hpp"

namespace fvg {
namespace {

constexpr int W = 64;        // width
constexpr int KENC = 16;     // encoder inputs, padded
constexpr int KMSG = 144;    // message inputs 64 + 64 + 3, padded
constexpr int KUPD = 128;    // update inputs
constexpr int NDEC = 8;      // decoder outputs 4, padded
constexpr int GT = 128;      // GEMM CTA threads (4 warps x 16 rows)
constexpr int GR = 64;       // GEMM rows per CTA

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi)
{
	const __nv_bfloat16 a = __float2bfloat16_rn(lo), b = __float2bfloat16_rn(hi);
	return (unsigned)__bfloat16_as_ushort(a) | ((unsigned)__bfloat16_as_ushort(b) << 16);
}

__device__ __forceinline__ void mma_bf16(float *c, const unsigned *a, const unsigned *b)
{
	asm volatile(
	    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
	    "{%0,%1,%2,%3};\n"
	    : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
	    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

/* One GEMM tile: out[r][n] = sum_k A[r][k] B[n][k] (+ bias[n]) for the 64 rows
 * of this CTA.  sA: [64][K] and sB: [N][K] bf16 in shared memory (row stride
 * K + 8 to spread banks); c: per warp 16 rows x N accumulators. */
template <int K, int N>
__device__ __forceinline__ void tile_mma(const __nv_bfloat16 *sA, const __nv_bfloat16 *sB, float (*c)[4])
{
	constexpr int LDA = K + 8;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int g = lane >> 2, t = lane & 3;
	const __nv_bfloat16 *a0 = sA + (warp * 16 + g) * LDA, *a1 = a0 + 8 * LDA;
	for (int nt = 0; nt < N / 8; nt++)
		for (int q = 0; q < 4; q++) c[nt][q] = 0.f;
	for (int k0 = 0; k0 < K; k0 += 16) {
		unsigned af[4];
		af[0] = *reinterpret_cast<const unsigned *>(a0 + k0 + 2 * t);
		af[1] = *reinterpret_cast<const unsigned *>(a1 + k0 + 2 * t);
		af[2] = *reinterpret_cast<const unsigned *>(a0 + k0 + 8 + 2 * t);
		af[3] = *reinterpret_cast<const unsigned *>(a1 + k0 + 8 + 2 * t);
		for (int nt = 0; nt < N / 8; nt++) {
			const __nv_bfloat16 *bp = sB + (nt * 8 + g) * LDA + k0 + 2 * t;
			unsigned bf[2];
			bf[0] = *reinterpret_cast<const unsigned *>(bp);
			bf[1] = *reinterpret_cast<const unsigned *>(bp + 8);
			mma_bf16(c[nt], af, bf);
		}
	}
}

/* stores the accumulators of a tile: rows r (< nrows), columns n < ncols */
template <int N>
__device__ __forceinline__ void tile_store(const float (*c)[4], int row0, int nrows, const float *bias, float *out,
                                           int ldo, int ncols, float *pre, int relu)
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int g = lane >> 2, t = lane & 3;
	for (int nt = 0; nt < N / 8; nt++)
		for (int h = 0; h < 2; h++) {
			const int r = row0 + warp * 16 + g + 8 * h;
			if (r >= nrows) continue;
			for (int j = 0; j < 2; j++) {
				const int n = nt * 8 + 2 * t + j;
				if (n >= ncols) continue;
				float v = c[nt][2 * h + j] + (bias ? bias[n] : 0.f);
				if (pre) pre[(size_t)r * ldo + n] = v;
				if (relu) v = fmaxf(v, 0.f);
				out[(size_t)r * ldo + n] = v;
			}
		}
}

/* stage B = W [N][K] (fp32, row stride ldw) as bf16 into shared memory */
template <int K, int N>
__device__ __forceinline__ void stage_w(const float *w, int ldw, int nvalid, int kvalid, __nv_bfloat16 *sB)
{
	constexpr int LDA = K + 8;
	for (int e = threadIdx.x; e < N * K; e += GT) {
		const int n = e / K, k = e - n * K;
		const float v = (n < nvalid && k < kvalid) ? w[(size_t)n * ldw + k] : 0.f;
		sB[n * LDA + k] = __float2bfloat16_rn(v);
	}
}

// --------------------------------- graph data --------------------------------

struct Graph {
	int nc = 0, nf = 0;          // cells, interior faces
	int2 *ef = nullptr;          // [nf] (L, R)
	float4 *ea = nullptr;        // [nf] (nx, ny, log10 len, 0), normal L -> R
	int *in_ptr = nullptr;       // [nc+1] CSR of messages into a cell (message id 2f+dir)
	int *in_idx = nullptr;
	int *out_ptr = nullptr;      // [nc+1] CSR of messages out of a cell
	int *out_idx = nullptr;
	float4 *xs = nullptr;        // [nc] static node features
};

/* message id 2f: L -> R, 2f+1: R -> L */
__device__ __forceinline__ void msg_ends(const Graph &G, int m, int &src, int &dst, float4 &e)
{
	const int f = m >> 1;
	const int2 lr = G.ef[f];
	e = G.ea[f];
	if (m & 1) { src = lr.y; dst = lr.x; e.x = -e.x; e.y = -e.y; }
	else { src = lr.x; dst = lr.y; }
}

// ------------------------------- forward kernels -------------------------------

/* h0 = relu(We x + be); x = static features + condition features */
__global__ void __launch_bounds__(GT) k_encode(Graph G, int B, const float *cond /*[B][3]*/, const float *We,
                                               const float *be, float *h, float *pre)
{
	__shared__ __align__(16) __nv_bfloat16 sA[GR * (KENC + 8)], sB[W * (KENC + 8)];
	const int rows = B * G.nc, row0 = blockIdx.x * GR;
	for (int e = threadIdx.x; e < GR * KENC; e += GT) {
		const int rr = e / KENC, k = e - rr * KENC, r = row0 + rr;
		float v = 0.f;
		if (r < rows && k < 7) {
			const int b = r / G.nc, i = r - b * G.nc;
			const float4 s = G.xs[i];
			v = k == 0 ? s.x : k == 1 ? s.y : k == 2 ? s.z : k == 3 ? s.w : cond[3 * b + (k - 4)];
		}
		sA[rr * (KENC + 8) + k] = __float2bfloat16_rn(v);
	}
	stage_w<KENC, W>(We, 7, W, 7, sB);
	__syncthreads();
	float c[W / 8][4];
	tile_mma<KENC, W>(sA, sB, c);
	tile_store<W>(c, row0, rows, be, h, W, W, pre, 1);
}

/* messages: Zm = Wm [h_src, h_dst, e] + bm, m = relu(Zm); rows = B * 2 nf */
__global__ void __launch_bounds__(GT) k_message(Graph G, int B, const float *h, const float *Wm, const float *bm,
                                                float *msg, float *pre)
{
	extern __shared__ __align__(16) unsigned char smem[];
	__nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smem);
	__nv_bfloat16 *sB = sA + GR * (KMSG + 8);
	const int per = 2 * G.nf, rows = B * per, row0 = blockIdx.x * GR;
	for (int e = threadIdx.x; e < GR * KMSG; e += GT) {
		const int rr = e / KMSG, k = e - rr * KMSG, r = row0 + rr;
		float v = 0.f;
		if (r < rows) {
			const int b = r / per, mid = r - b * per;
			int s, d;
			float4 ev;
			msg_ends(G, mid, s, d, ev);
			const float *hb = h + (size_t)b * G.nc * W;
			if (k < W) v = hb[(size_t)s * W + k];
			else if (k < 2 * W) v = hb[(size_t)d * W + (k - W)];
			else if (k == 2 * W) v = ev.x;
			else if (k == 2 * W + 1) v = ev.y;
			else if (k == 2 * W + 2) v = ev.z;
		}
		sA[rr * (KMSG + 8) + k] = __float2bfloat16_rn(v);
	}
	stage_w<KMSG, W>(Wm, 2 * W + 3, W, 2 * W + 3, sB);
	__syncthreads();
	float c[W / 8][4];
	tile_mma<KMSG, W>(sA, sB, c);
	tile_store<W>(c, row0, rows, bm, msg, W, W, pre, 1);
}

/* a_i = sum of the messages into cell i (fixed CSR order) */
__global__ void k_aggregate(Graph G, int B, const float *msg, float *agg)
{
	const int r = blockIdx.x, k = threadIdx.x;  // one block of 64 threads per (member, cell)
	const int b = r / G.nc, i = r - b * G.nc;
	const float *mb = msg + (size_t)b * 2 * G.nf * W;
	float s = 0.f;
	for (int q = G.in_ptr[i]; q < G.in_ptr[i + 1]; q++) s += mb[(size_t)G.in_idx[q] * W + k];
	agg[(size_t)r * W + k] = s;
}

/* hn = h + relu(Wu [h, a] + bu) */
__global__ void __launch_bounds__(GT) k_update(int rows, const float *h, const float *agg, const float *Wu,
                                               const float *bu, float *hn, float *pre)
{
	extern __shared__ __align__(16) unsigned char smem[];
	__nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smem);
	__nv_bfloat16 *sB = sA + GR * (KUPD + 8);
	const int row0 = blockIdx.x * GR;
	for (int e = threadIdx.x; e < GR * KUPD; e += GT) {
		const int rr = e / KUPD, k = e - rr * KUPD, r = row0 + rr;
		float v = 0.f;
		if (r < rows) v = k < W ? h[(size_t)r * W + k] : agg[(size_t)r * W + k - W];
		sA[rr * (KUPD + 8) + k] = __float2bfloat16_rn(v);
	}
	stage_w<KUPD, W>(Wu, KUPD, W, KUPD, sB);
	__syncthreads();
	float c[W / 8][4];
	tile_mma<KUPD, W>(sA, sB, c);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	for (int nt = 0; nt < W / 8; nt++)
		for (int hh = 0; hh < 2; hh++) {
			const int r = row0 + warp * 16 + g + 8 * hh;
			if (r >= rows) continue;
			for (int j = 0; j < 2; j++) {
				const int n = nt * 8 + 2 * t + j;
				const float z = c[nt][2 * hh + j] + bu[n];
				pre[(size_t)r * W + n] = z;
				hn[(size_t)r * W + n] = h[(size_t)r * W + n] + fmaxf(z, 0.f);
			}
		}
}

/* y = Wd h + bd (4 outputs) */
__global__ void __launch_bounds__(GT) k_decode(int rows, const float *h, const float *Wd, const float *bd, float *y)
{
	__shared__ __align__(16) __nv_bfloat16 sA[GR * (W + 8)], sB[NDEC * (W + 8)];
	const int row0 = blockIdx.x * GR;
	for (int e = threadIdx.x; e < GR * W; e += GT) {
		const int rr = e / W, k = e - rr * W, r = row0 + rr;
		sA[rr * (W + 8) + k] = __float2bfloat16_rn(r < rows ? h[(size_t)r * W + k] : 0.f);
	}
	stage_w<W, NDEC>(Wd, W, 4, W, sB);
	__syncthreads();
	float c[NDEC / 8][4];
	tile_mma<W, NDEC>(sA, sB, c);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	for (int hh = 0; hh < 2; hh++) {
		const int r = row0 + warp * 16 + g + 8 * hh;
		if (r >= rows) continue;
		for (int j = 0; j < 2; j++) {
			const int n = 2 * t + j;
			if (n < 4) y[(size_t)r * 4 + n] = c[0][2 * hh + j] + bd[n];
		}
	}
}

/* u = uinf + scale * y (double) */
__global__ void k_to_state(int nc, int B, const float *y, const float *uinf /*[B][4]*/, const float *scale,
                           double *u)
{
	const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= (size_t)B * nc * 4) return;
	const int v = (int)(e & 3);
	const int b = (int)(e / ((size_t)nc * 4));
	u[e] = (double)uinf[4 * b + v] + (double)scale[v] * (double)y[e];
}

/* loss pieces: dy = 2 (y - t) / count, partial sums of (y - t)^2 */
__global__ void k_loss(int n, const float *y, const double *target, const float *uinf, const float *scale, int nc,
                       float inv_count, float *dy, float *part)
{
	__shared__ float sh[256];
	float s = 0.f;
	for (int e = blockIdx.x * 256 + threadIdx.x; e < n; e += gridDim.x * 256) {
		const int v = e & 3, b = e / (nc * 4);
		const float t = (float)((target[e] - (double)uinf[4 * b + v]) / (double)scale[v]);
		const float d = y[e] - t;
		dy[e] = 2.f * d * inv_count;
		s += d * d;
	}
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int o = 128; o > 0; o >>= 1) {
		if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// ------------------------------- backward kernels -------------------------------

/* dZ = dY * (Z > 0) */
__global__ void k_relu_back(size_t n, const float *dy, const float *z, float *dz)
{
	const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (e < n) dz[e] = z[e] > 0.f ? dy[e] : 0.f;
}

/* dX[r][k] = sum_n dZ[r][n] W[n][k] for k < kout: a GEMM with B = W^T */
template <int K, int N>
__global__ void __launch_bounds__(GT) k_back_x(int rows, const float *dz, int ldz, int nz, const float *w, int ldw,
                                               int kout, float *dx, int ldx)
{
	extern __shared__ __align__(16) unsigned char smem[];
	__nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smem);  // [64][K] with K = nz padded
	__nv_bfloat16 *sB = sA + GR * (K + 8);                         // [N][K]: W^T
	const int row0 = blockIdx.x * GR;
	for (int e = threadIdx.x; e < GR * K; e += GT) {
		const int rr = e / K, k = e - rr * K, r = row0 + rr;
		sA[rr * (K + 8) + k] = __float2bfloat16_rn((r < rows && k < nz) ? dz[(size_t)r * ldz + k] : 0.f);
	}
	for (int e = threadIdx.x; e < N * K; e += GT) {
		const int n = e / K, k = e - n * K;
		sB[n * (K + 8) + k] = __float2bfloat16_rn((n < kout && k < nz) ? w[(size_t)k * ldw + n] : 0.f);
	}
	__syncthreads();
	float c[N / 8][4];
	tile_mma<K, N>(sA, sB, c);
	tile_store<N>(c, row0, rows, nullptr, dx, ldx, kout, nullptr, 0);
}

/* partial weight gradients of a 64-row chunk: P[chunk][n][k] = sum_r dZ[r][n] X[r][k]
 * (the rows of X come from a loader, as in the forward pass); db partials too */
template <int K, int N, class Loader>
__global__ void __launch_bounds__(GT) k_back_w(int rows, const float *dz, int ldz, int nz, Loader ld, float *part,
                                               float *bpart)
{
	extern __shared__ __align__(16) unsigned char smem[];
	// A = dZ^T [N rows][64 k], B = X^T [K rows][64 k]
	__nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smem);  // [N][64 + 8]
	__nv_bfloat16 *sB = sA + N * (GR + 8);                         // [K][64 + 8]
	const int row0 = blockIdx.x * GR;
	for (int e = threadIdx.x; e < N * GR; e += GT) {
		const int n = e / GR, rr = e - n * GR, r = row0 + rr;
		sA[n * (GR + 8) + rr] = __float2bfloat16_rn((r < rows && n < nz) ? dz[(size_t)r * ldz + n] : 0.f);
	}
	for (int e = threadIdx.x; e < K * GR; e += GT) {
		const int k = e / GR, rr = e - k * GR, r = row0 + rr;
		sB[k * (GR + 8) + rr] = __float2bfloat16_rn(r < rows ? ld(r, k) : 0.f);
	}
	__syncthreads();
	// each warp: 16 of the N rows (N = 64: 4 warps) x K columns
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	float c[K / 8][4];
	for (int nt = 0; nt < K / 8; nt++)
		for (int q = 0; q < 4; q++) c[nt][q] = 0.f;
	if (warp * 16 < N) {
		const __nv_bfloat16 *a0 = sA + (warp * 16 + g) * (GR + 8), *a1 = a0 + 8 * (GR + 8);
		for (int k0 = 0; k0 < GR; k0 += 16) {
			unsigned af[4];
			af[0] = *reinterpret_cast<const unsigned *>(a0 + k0 + 2 * t);
			af[1] = *reinterpret_cast<const unsigned *>(a1 + k0 + 2 * t);
			af[2] = *reinterpret_cast<const unsigned *>(a0 + k0 + 8 + 2 * t);
			af[3] = *reinterpret_cast<const unsigned *>(a1 + k0 + 8 + 2 * t);
			for (int nt = 0; nt < K / 8; nt++) {
				const __nv_bfloat16 *bp = sB + (nt * 8 + g) * (GR + 8) + k0 + 2 * t;
				unsigned bf[2];
				bf[0] = *reinterpret_cast<const unsigned *>(bp);
				bf[1] = *reinterpret_cast<const unsigned *>(bp + 8);
				mma_bf16(c[nt], af, bf);
			}
		}
		float *pc = part + (size_t)blockIdx.x * N * K;
		for (int nt = 0; nt < K / 8; nt++)
			for (int hh = 0; hh < 2; hh++)
				for (int j = 0; j < 2; j++) pc[(size_t)(warp * 16 + g + 8 * hh) * K + nt * 8 + 2 * t + j] = c[nt][2 * hh + j];
	}
	// bias partials (fp32, fixed order)
	for (int n = threadIdx.x; n < N; n += GT) {
		float s = 0.f;
		for (int rr = 0; rr < GR; rr++) {
			const int r = row0 + rr;
			if (r < rows && n < nz) s += dz[(size_t)r * ldz + n];
		}
		bpart[(size_t)blockIdx.x * N + n] = s;
	}
}

/* sum of the chunk partials into the gradient (fixed order); only the valid
 * [nv][kv] part of the padded [N][K] tiles, into g with row stride kv */
__global__ void k_reduce_parts(int nchunks, int N, int K, int nv, int kv, const float *part, const float *bpart,
                               float *gw, float *gb)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e < nv * kv) {
		const int n = e / kv, k = e - n * kv;
		float s = 0.f;
		for (int c = 0; c < nchunks; c++) s += part[((size_t)c * N + n) * K + k];
		gw[e] += s;
	}
	if (e < nv) {
		float s = 0.f;
		for (int c = 0; c < nchunks; c++) s += bpart[(size_t)c * N + e];
		gb[e] += s;
	}
}

/* dh of the message sources / destinations: per cell, the outgoing messages'
 * d[h_src] columns and the incoming messages' d[h_dst] columns */
__global__ void k_scatter_msg(Graph G, int B, const float *dxm /*[B*2nf][ld]*/, int ld, float *dh)
{
	const int r = blockIdx.x, k = threadIdx.x;
	const int b = r / G.nc, i = r - b * G.nc;
	const float *xb = dxm + (size_t)b * 2 * G.nf * ld;
	float s = 0.f;
	for (int q = G.out_ptr[i]; q < G.out_ptr[i + 1]; q++) s += xb[(size_t)G.out_idx[q] * ld + k];
	for (int q = G.in_ptr[i]; q < G.in_ptr[i + 1]; q++) s += xb[(size_t)G.in_idx[q] * ld + W + k];
	dh[(size_t)r * W + k] += s;
}

/* d(message) = d(aggregate) of its destination */
__global__ void k_gather_agg(Graph G, int B, const float *dagg /*[B*nc][ld]*/, int ld, float *dmsg)
{
	const int r = blockIdx.x, k = threadIdx.x;  // r over B * 2nf messages
	const int per = 2 * G.nf, b = r / per, mid = r - b * per;
	int s, d;
	float4 e;
	msg_ends(G, mid, s, d, e);
	dmsg[(size_t)r * W + k] = dagg[((size_t)b * G.nc + d) * ld + W + k];
}

/* dst[r][k] += src[r][k] for k < W (src row stride lds) */
__global__ void k_add_cols(size_t rows, const float *src, int lds, float *dst)
{
	const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= rows * W) return;
	const size_t r = e / W, k = e - r * W;
	dst[e] += src[r * lds + k];
}

/* Adam (Kingma & Ba 2015): m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2;
 * p -= lr mhat / (sqrt(vhat) + eps) */
__global__ void k_adam(int n, float *p, const float *g, float *m, float *v, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= n) return;
	const float gg = g[e];
	m[e] = b1 * m[e] + (1.f - b1) * gg;
	v[e] = b2 * v[e] + (1.f - b2) * gg * gg;
	p[e] -= lr * (m[e] / c1) / (sqrtf(v[e] / c2) + eps);
}

// ------------------------------------ loaders ------------------------------------

struct LoadEnc {
	Graph G;
	const float *cond;
	__device__ float operator()(int r, int k) const
	{
		if (k >= 7) return 0.f;
		const int b = r / G.nc, i = r - b * G.nc;
		const float4 s = G.xs[i];
		return k == 0 ? s.x : k == 1 ? s.y : k == 2 ? s.z : k == 3 ? s.w : cond[3 * b + (k - 4)];
	}
};
struct LoadMsg {
	Graph G;
	const float *h;
	__device__ float operator()(int r, int k) const
	{
		const int per = 2 * G.nf, b = r / per, mid = r - b * per;
		int s, d;
		float4 e;
		msg_ends(G, mid, s, d, e);
		const float *hb = h + (size_t)b * G.nc * W;
		if (k < W) return hb[(size_t)s * W + k];
		if (k < 2 * W) return hb[(size_t)d * W + k - W];
		return k == 2 * W ? e.x : k == 2 * W + 1 ? e.y : k == 2 * W + 2 ? e.z : 0.f;
	}
};
struct LoadUpd {
	const float *h, *agg;
	__device__ float operator()(int r, int k) const { return k < W ? h[(size_t)r * W + k] : agg[(size_t)r * W + k - W]; }
};
struct LoadRows {
	const float *x;
	int ld;
	__device__ float operator()(int r, int k) const { return x[(size_t)r * ld + k]; }
};

}  // namespace
}  // namespace fvg

using namespace fvg;

/* parameter layout in one flat FP32 array */
struct MpnnLayout {
	int layers = 4;
	size_t we, be, wm[8], bm[8], wu[8], bu[8], wd, bd, total;
	void build(int L)
	{
		layers = L;
		size_t o = 0;
		we = o; o += (size_t)W * 7;
		be = o; o += W;
		for (int l = 0; l < L; l++) {
			wm[l] = o; o += (size_t)W * (2 * W + 3);
			bm[l] = o; o += W;
			wu[l] = o; o += (size_t)W * KUPD;
			bu[l] = o; o += W;
		}
		wd = o; o += (size_t)4 * W;
		bd = o; o += 4;
		total = o;
	}
};

struct fv_mpnn {
	fv_mesh_impl *mesh = nullptr;
	Graph G;
	MpnnLayout lay;
	float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;  // params, grads, Adam moments
	int adam_t = 0;
	float scale_h[4] = {1.f, 1.f, 1.f, 1.f};
	float *scale = nullptr;
	// activations (sized for cap_b members)
	int cap_b = 0;
	float *h = nullptr, *zpre = nullptr, *msg = nullptr, *mpre = nullptr, *agg = nullptr, *upre = nullptr;
	float *y = nullptr, *dy = nullptr, *cond = nullptr, *uinf = nullptr, *t1 = nullptr, *t2 = nullptr, *dh = nullptr;
	float *dmsg = nullptr, *dxm = nullptr, *part = nullptr, *bpart = nullptr, *lpart = nullptr;
	std::vector<void *> owned;
};

namespace {

template <class T>
cudaError_t mall(fv_mpnn *N, T **p, size_t n)
{
	cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (n ? n : 1));
	if (!e) N->owned.push_back(*p);
	return e;
}

size_t smem_msg() { return sizeof(__nv_bfloat16) * (GR + W) * (KMSG + 8); }
size_t smem_upd() { return sizeof(__nv_bfloat16) * (GR + W) * (KUPD + 8); }

cudaError_t ensure_capacity(fv_mpnn *N, int B)
{
	if (B <= N->cap_b) return cudaSuccess;
	// activations are re-allocated for the larger batch
	for (void *q : {(void *)N->h, (void *)N->zpre, (void *)N->msg, (void *)N->mpre, (void *)N->agg, (void *)N->upre,
	                (void *)N->y, (void *)N->dy, (void *)N->cond, (void *)N->uinf, (void *)N->t1, (void *)N->t2, (void *)N->dh,
	                (void *)N->dmsg, (void *)N->dxm, (void *)N->part, (void *)N->bpart, (void *)N->lpart})
		if (q) {
			cudaFree(q);
			for (auto &o : N->owned)
				if (o == q) o = nullptr;
		}
	const size_t nc = N->G.nc, nm = 2 * (size_t)N->G.nf, L = N->lay.layers;
	const size_t rows_m = B * nm, rows_c = B * nc;
	cudaError_t e = cudaSuccess;
	auto al = [&](float **p, size_t n) { if (!e) e = mall(N, p, n); };
	al(&N->h, (L + 1) * rows_c * W);
	al(&N->zpre, rows_c * W);
	al(&N->msg, L * rows_m * W);
	al(&N->mpre, L * rows_m * W);
	al(&N->agg, L * rows_c * W);
	al(&N->upre, L * rows_c * W);
	al(&N->y, rows_c * 4);
	al(&N->dy, rows_c * 4);
	al(&N->cond, 3 * (size_t)B);
	al(&N->uinf, 4 * (size_t)B);
	al(&N->t1, rows_c * W);
	al(&N->t2, rows_c * KUPD);
	al(&N->dh, rows_c * W);
	al(&N->dmsg, rows_m * W);
	al(&N->dxm, rows_m * KMSG);
	const size_t chunks = (std::max(rows_m, rows_c) + GR - 1) / GR;
	al(&N->part, chunks * (size_t)W * KMSG);
	al(&N->bpart, chunks * (size_t)W);
	al(&N->lpart, 1024);
	if (!e) N->cap_b = B;
	return e;
}

void set_conditions(fv_mpnn *N, const fv_physics_cfg *phys, int B, std::vector<float> &cond, std::vector<float> &uinf)
{
	cond.resize(3 * (size_t)B);
	uinf.resize(4 * (size_t)B);
	for (int b = 0; b < B; b++) {
		const fv_physics_cfg &c = phys[b];
		cond[3 * b] = (float)((c.Minf - 0.5) / 0.2);
		cond[3 * b + 1] = (float)(c.aoa * 180.0 / M_PI / 4.0);
		cond[3 * b + 2] = (float)(c.viscous_sim ? std::log10(c.Reinf) - 4.0 : -1.0);
		const Phys P = make_phys(c);
		for (int k = 0; k < 4; k++) uinf[4 * b + k] = (float)P.uinf[k];
	}
}

unsigned nb(size_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

/* forward pass for B members; activations kept for the backward pass */
cudaError_t forward(fv_mpnn *N, int B, cudaStream_t s)
{
	const Graph &G = N->G;
	const MpnnLayout &Y = N->lay;
	const float *P = N->p;
	const size_t nc = G.nc, nm = 2 * (size_t)G.nf, rows_c = B * nc, rows_m = B * nm;
	k_encode<<<nb(rows_c, GR), GT, 0, s>>>(G, B, N->cond, P + Y.we, P + Y.be, N->h, N->zpre);
	for (int l = 0; l < Y.layers; l++) {
		const float *hl = N->h + l * rows_c * W;
		float *ml = N->msg + l * rows_m * W, *mp = N->mpre + l * rows_m * W;
		k_message<<<nb(rows_m, GR), GT, smem_msg(), s>>>(G, B, hl, P + Y.wm[l], P + Y.bm[l], ml, mp);
		float *al = N->agg + l * rows_c * W;
		k_aggregate<<<(unsigned)rows_c, W, 0, s>>>(G, B, ml, al);
		k_update<<<nb(rows_c, GR), GT, smem_upd(), s>>>((int)rows_c, hl, al, P + Y.wu[l], P + Y.bu[l],
		                                                N->h + (l + 1) * rows_c * W, N->upre + l * rows_c * W);
	}
	k_decode<<<nb(rows_c, GR), GT, 0, s>>>((int)rows_c, N->h + Y.layers * rows_c * W, P + Y.wd, P + Y.bd, N->y);
	count_launches(2 + 3 * Y.layers);
	return cudaGetLastError();
}

template <int K, int Nn, class Loader>
cudaError_t weight_grad(int rows, const float *dz, int ldz, int nz, Loader ld, float *part, float *bpart, int nv,
                        int kv, float *gw, float *gb, cudaStream_t s)
{
	const unsigned chunks = nb(rows, GR);
	const size_t sm = sizeof(__nv_bfloat16) * (Nn + K) * (GR + 8);
	k_back_w<K, Nn, Loader><<<chunks, GT, sm, s>>>(rows, dz, ldz, nz, ld, part, bpart);
	k_reduce_parts<<<nb((size_t)nv * kv, 256), 256, 0, s>>>((int)chunks, Nn, K, nv, kv, part, bpart, gw, gb);
	count_launches(2);
	return cudaGetLastError();
}

/* backward pass from N->dy; gradients accumulate into N->g */
cudaError_t backward(fv_mpnn *N, int B, cudaStream_t s)
{
	const Graph &G = N->G;
	const MpnnLayout &Y = N->lay;
	const float *P = N->p;
	float *Gr = N->g;
	const size_t nc = G.nc, nm = 2 * (size_t)G.nf, rows_c = B * nc, rows_m = B * nm;
	const float *hL = N->h + Y.layers * rows_c * W;
	// decoder: y = Wd h + bd
	weight_grad<W, 16>((int)rows_c, N->dy, 4, 4, LoadRows{hL, W}, N->part, N->bpart, 4, W, Gr + Y.wd, Gr + Y.bd, s);
	k_back_x<16, W><<<nb(rows_c, GR), GT, sizeof(__nv_bfloat16) * (GR + W) * (16 + 8), s>>>(
	    (int)rows_c, N->dy, 4, 4, P + Y.wd, W, W, N->dh, W);
	count_launches(1);
	for (int l = Y.layers - 1; l >= 0; l--) {
		const float *hl = N->h + l * rows_c * W;
		const float *al = N->agg + l * rows_c * W;
		// update: hn = h + relu(Zu), Zu = Wu [h, a] + bu
		k_relu_back<<<nb(rows_c * W, 256), 256, 0, s>>>(rows_c * W, N->dh, N->upre + l * rows_c * W, N->t1);
		weight_grad<KUPD, W>((int)rows_c, N->t1, W, W, LoadUpd{hl, al}, N->part, N->bpart, W, KUPD, Gr + Y.wu[l],
		                     Gr + Y.bu[l], s);
		k_back_x<W, KUPD><<<nb(rows_c, GR), GT, sizeof(__nv_bfloat16) * (GR + KUPD) * (W + 8), s>>>(
		    (int)rows_c, N->t1, W, W, P + Y.wu[l], KUPD, KUPD, N->t2, KUPD);
		// residual path and the update's d[h] columns
		k_add_cols<<<nb(rows_c * W, 256), 256, 0, s>>>(rows_c, N->t2, KUPD, N->dh);
		// messages: dm = d[a] of the destination, dZm = dm (Zm > 0)
		k_gather_agg<<<(unsigned)rows_m, W, 0, s>>>(G, B, N->t2, KUPD, N->dmsg);
		k_relu_back<<<nb(rows_m * W, 256), 256, 0, s>>>(rows_m * W, N->dmsg, N->mpre + l * rows_m * W, N->dmsg);
		weight_grad<KMSG, W>((int)rows_m, N->dmsg, W, W, LoadMsg{G, hl}, N->part, N->bpart, W, 2 * W + 3,
		                     Gr + Y.wm[l], Gr + Y.bm[l], s);
		k_back_x<W, KMSG><<<nb(rows_m, GR), GT, sizeof(__nv_bfloat16) * (GR + KMSG) * (W + 8), s>>>(
		    (int)rows_m, N->dmsg, W, W, P + Y.wm[l], 2 * W + 3, 2 * W, N->dxm, KMSG);
		k_scatter_msg<<<(unsigned)rows_c, W, 0, s>>>(G, B, N->dxm, KMSG, N->dh);
		count_launches(7);
	}
	// encoder: h0 = relu(We x + be)
	k_relu_back<<<nb(rows_c * W, 256), 256, 0, s>>>(rows_c * W, N->dh, N->zpre, N->t1);
	weight_grad<KENC, W>((int)rows_c, N->t1, W, W, LoadEnc{G, N->cond}, N->part, N->bpart, W, 7, Gr + Y.we,
	                     Gr + Y.be, s);
	count_launches(1);
	return cudaGetLastError();
}

cudaError_t loss_grad(fv_mpnn *N, int B, const double *target, float *h_loss, cudaStream_t s)
{
	const size_t n = (size_t)B * N->G.nc * 4;
	const int blocks = 256;
	k_loss<<<blocks, 256, 0, s>>>((int)n, N->y, target, N->uinf, N->scale, N->G.nc, 1.f / (float)n, N->dy, N->lpart);
	count_launches(1);
	cudaError_t e = cudaGetLastError();
	if (h_loss) {
		float hp[256];
		if (!e) e = cudaMemcpyAsync(hp, N->lpart, sizeof(hp), cudaMemcpyDeviceToHost, s);
		if (!e) e = cudaStreamSynchronize(s);
		double sum = 0;
		for (int k = 0; k < blocks; k++) sum += hp[k];
		*h_loss = (float)(sum / (double)n);
	}
	return e;
}

cudaError_t upload_conditions(fv_mpnn *N, const fv_physics_cfg *phys, int B, cudaStream_t s)
{
	std::vector<float> cond, uinf;
	set_conditions(N, phys, B, cond, uinf);
	cudaError_t e = cudaMemcpyAsync(N->cond, cond.data(), sizeof(float) * cond.size(), cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(N->uinf, uinf.data(), sizeof(float) * uinf.size(), cudaMemcpyHostToDevice, s);
	if (!e) e = cudaStreamSynchronize(s);  // host vectors go out of scope
	return e;
}

}  // namespace

extern "C" {

fv_status fv_mpnn_create(fv_mesh *m, int layers, const int *wall_markers, int nwall, unsigned long long seed,
                         fv_mpnn **out)
{
	if (!m || !out || layers < 1 || layers > 8 || (nwall > 0 && !wall_markers)) {
		set_error("invalid argument");
		return FV_ERR_INVALID;
	}
	const HostMesh &h = m->h;
	fv_mpnn *N = new fv_mpnn();
	N->mesh = m;
	N->lay.build(layers);
	Graph &G = N->G;
	G.nc = h.nelem;
	G.nf = h.naface - h.nbface;
	// graph and static node features
	std::vector<int2> ef(G.nf);
	std::vector<float4> ea(G.nf);
	std::vector<int> in_cnt(G.nc + 1, 0), out_cnt(G.nc + 1, 0);
	for (int f = 0; f < G.nf; f++) {
		const int F = h.nbface + f;
		ef[f] = make_int2(h.face_l[F], h.face_r[F]);
		ea[f] = make_float4((float)h.fnorm[3 * F], (float)h.fnorm[3 * F + 1], (float)std::log10(h.fnorm[3 * F + 2]), 0.f);
		out_cnt[h.face_l[F] + 1]++; in_cnt[h.face_r[F] + 1]++;   // message 2f: L -> R
		out_cnt[h.face_r[F] + 1]++; in_cnt[h.face_l[F] + 1]++;   // message 2f+1: R -> L
	}
	for (int i = 0; i < G.nc; i++) { in_cnt[i + 1] += in_cnt[i]; out_cnt[i + 1] += out_cnt[i]; }
	std::vector<int> in_idx(in_cnt[G.nc]), out_idx(out_cnt[G.nc]);
	{
		std::vector<int> ip(in_cnt.begin(), in_cnt.end() - 1), op(out_cnt.begin(), out_cnt.end() - 1);
		for (int f = 0; f < G.nf; f++) {
			const int F = h.nbface + f, L = h.face_l[F], R = h.face_r[F];
			out_idx[op[L]++] = 2 * f; in_idx[ip[R]++] = 2 * f;
			out_idx[op[R]++] = 2 * f + 1; in_idx[ip[L]++] = 2 * f + 1;
		}
	}
	// wall distance: to the nearest centre of a face of a wall marker
	std::vector<double> wc;
	for (int f = 0; f < h.nbface; f++)
		for (int k = 0; k < nwall; k++)
			if (h.btag[f] == wall_markers[k]) { wc.push_back(h.fc[2 * f]); wc.push_back(h.fc[2 * f + 1]); }
	std::vector<float4> xs(G.nc);
	for (int i = 0; i < G.nc; i++) {
		const double x = h.cc[2 * i], y = h.cc[2 * i + 1];
		const double r = std::sqrt((x - 0.5) * (x - 0.5) + y * y);
		double dw = 1e3;
		for (size_t q = 0; q < wc.size(); q += 2) dw = std::min(dw, std::hypot(x - wc[q], y - wc[q + 1]));
		xs[i] = make_float4((float)(x / (1.0 + r)), (float)(y / (1.0 + r)), (float)(std::log10(h.area[i]) / 4.0),
		                    (float)(std::log10(dw + 1e-6) / 3.0));
	}
	cudaError_t e = cudaSuccess;
	auto up = [&](auto **dst, const auto &v) {
		if (e) return;
		e = mall(N, dst, v.size());
		if (!e) e = cudaMemcpy(*dst, v.data(), sizeof(v[0]) * v.size(), cudaMemcpyHostToDevice);
	};
	up(&G.ef, ef); up(&G.ea, ea); up(&G.in_ptr, in_cnt); up(&G.in_idx, in_idx); up(&G.out_ptr, out_cnt);
	up(&G.out_idx, out_idx); up(&G.xs, xs);
	// parameters: uniform in +-sqrt(6 / fan_in) (He), decoder scaled down, biases 0
	const MpnnLayout &Y = N->lay;
	std::vector<float> p(Y.total, 0.f);
	std::mt19937_64 rng(seed);
	auto init = [&](size_t off, int rows, int fan_in, double gain) {
		std::uniform_real_distribution<double> U(-1.0, 1.0);
		const double a = gain * std::sqrt(6.0 / fan_in);
		for (size_t k = 0; k < (size_t)rows * fan_in; k++) p[off + k] = (float)(a * U(rng));
	};
	init(Y.we, W, 7, 1.0);
	for (int l = 0; l < layers; l++) {
		init(Y.wm[l], W, 2 * W + 3, 1.0);
		init(Y.wu[l], W, KUPD, 0.5);
	}
	init(Y.wd, 4, W, 0.1);
	up(&N->p, p);
	std::vector<float> z(Y.total, 0.f);
	up(&N->g, z); up(&N->m1, z); up(&N->m2, z);
	std::vector<float> sc(N->scale_h, N->scale_h + 4);
	up(&N->scale, sc);
	if (e) {
		fv_mpnn_destroy(N);
		return cuda_status(e, "mpnn allocation");
	}
	*out = N;
	return FV_OK;
}

void fv_mpnn_destroy(fv_mpnn *N)
{
	if (!N) return;
	for (void *q : N->owned)
		if (q) cudaFree(q);
	delete N;
}

fv_status fv_mpnn_set_scale(fv_mpnn *N, const float *scale4)
{
	if (!N || !scale4) { set_error("null argument"); return FV_ERR_INVALID; }
	for (int k = 0; k < 4; k++) N->scale_h[k] = scale4[k];
	return cuda_status(cudaMemcpy(N->scale, scale4, sizeof(float) * 4, cudaMemcpyHostToDevice), "mpnn scale");
}

fv_status fv_mpnn_params(fv_mpnn *N, float *h_out, const float *h_in, long long *count)
{
	if (!N) { set_error("null argument"); return FV_ERR_INVALID; }
	if (count) *count = (long long)N->lay.total;
	cudaError_t e = cudaSuccess;
	if (h_in) e = cudaMemcpy(N->p, h_in, sizeof(float) * N->lay.total, cudaMemcpyHostToDevice);
	if (!e && h_out) e = cudaMemcpy(h_out, N->p, sizeof(float) * N->lay.total, cudaMemcpyDeviceToHost);
	return cuda_status(e, "mpnn parameters");
}

fv_status fv_mpnn_graph(const fv_mpnn *N, float *xs, int *faces, float *eattr)
{
	if (!N) { set_error("null argument"); return FV_ERR_INVALID; }
	const Graph &G = N->G;
	cudaError_t e = cudaSuccess;
	if (xs) e = cudaMemcpy(xs, G.xs, sizeof(float4) * G.nc, cudaMemcpyDeviceToHost);
	if (!e && faces) e = cudaMemcpy(faces, G.ef, sizeof(int2) * G.nf, cudaMemcpyDeviceToHost);
	if (!e && eattr) {
		std::vector<float4> t(G.nf);
		e = cudaMemcpy(t.data(), G.ea, sizeof(float4) * G.nf, cudaMemcpyDeviceToHost);
		for (int f = 0; f < G.nf; f++) { eattr[3 * f] = t[f].x; eattr[3 * f + 1] = t[f].y; eattr[3 * f + 2] = t[f].z; }
	}
	return cuda_status(e, "mpnn graph");
}

fv_status fv_mpnn_predict(fv_mpnn *N, const fv_physics_cfg *phys, int batch, double *d_u)
{
	if (!N || !phys || batch < 1 || !d_u) { set_error("invalid argument"); return FV_ERR_INVALID; }
	cudaStream_t s = 0;
	cudaError_t e = ensure_capacity(N, batch);
	if (!e) e = upload_conditions(N, phys, batch, s);
	if (!e) e = forward(N, batch, s);
	if (!e) {
		const size_t n = (size_t)batch * N->G.nc * 4;
		k_to_state<<<nb(n, 256), 256, 0, s>>>(N->G.nc, batch, N->y, N->uinf, N->scale, d_u);
		count_launches(1);
		e = cudaGetLastError();
	}
	if (!e) e = cudaStreamSynchronize(s);
	return cuda_status(e, "mpnn predict");
}

/* gradients of the mean squared error of y against the target state (host
 * copies of gradient and loss), without an update */
fv_status fv_mpnn_gradients(fv_mpnn *N, const fv_physics_cfg *phys, int batch, const double *d_target, float *h_grad,
                            float *h_loss)
{
	if (!N || !phys || batch < 1 || !d_target) { set_error("invalid argument"); return FV_ERR_INVALID; }
	cudaStream_t s = 0;
	cudaError_t e = ensure_capacity(N, batch);
	if (!e) e = upload_conditions(N, phys, batch, s);
	if (!e) e = cudaMemsetAsync(N->g, 0, sizeof(float) * N->lay.total, s);
	if (!e) e = forward(N, batch, s);
	if (!e) e = loss_grad(N, batch, d_target, h_loss, s);
	if (!e) e = backward(N, batch, s);
	if (!e && h_grad) e = cudaMemcpy(h_grad, N->g, sizeof(float) * N->lay.total, cudaMemcpyDeviceToHost);
	if (!e) e = cudaStreamSynchronize(s);
	return cuda_status(e, "mpnn gradients");
}

/* one Adam step on the mean squared error of y against the target states */
fv_status fv_mpnn_train_step(fv_mpnn *N, const fv_physics_cfg *phys, int batch, const double *d_target, float lr,
                             float *h_loss)
{
	fv_status st = fv_mpnn_gradients(N, phys, batch, d_target, nullptr, h_loss);
	if (st) return st;
	N->adam_t++;
	const float b1 = 0.9f, b2 = 0.999f;
	const float c1 = 1.f - std::pow(b1, (float)N->adam_t), c2 = 1.f - std::pow(b2, (float)N->adam_t);
	const int n = (int)N->lay.total;
	k_adam<<<nb(n, 256), 256>>>(n, N->p, N->g, N->m1, N->m2, lr, b1, b2, 1e-8f, c1, c2);
	count_launches(1);
	return cuda_status(cudaDeviceSynchronize(), "mpnn adam");
}

}  // extern "C"
