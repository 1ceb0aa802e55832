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
 * The message MLP's first layer is linear in h_s and h_d, so it runs per
 * cell: pc = [W_s h, W_d h] (one GEMM over cells), and per message
 * Zm = pc_s[s] + pc_d[d] + W_e e_sd + bm (a gather, no GEMM over messages).
 * Its backward pass likewise sums dZm per cell over outgoing and incoming
 * messages (S_out, S_in) and forms the weight and input gradients with GEMMs
 * over cells; the edge weights' gradient and the bias sum over messages.
 *
 * Arithmetic: every contraction runs on the tensor cores as warp-level BF16
 * mma.sync (m16n8k16) with FP32 accumulation: GEMM operands (weights and
 * activations, S) are rounded to BF16 when they are staged in shared memory;
 * activations, biases, gradients and the Adam state stay FP32.  The GEMMs are
 * small (K <= 128, N <= 128), far from the solver's hot path.  Where a GEMM's
 * row operand is a contiguous block of FP32 rows, bulk copies (the TMA
 * engine) stage the CTA's next tiles while it multiplies the current one.
 * Reductions over rows (weight gradients, aggregation) run in fixed order.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "fv_abi_internal.hpp"
#include "fv_bulk.cuh"
#include "fv_tc05.cuh"

namespace fvg {
namespace {

constexpr int W = 64;        // width
constexpr int KENC = 16;     // encoder inputs, padded
constexpr int KUPD = 128;    // update inputs
constexpr int NDEC = 8;      // decoder outputs 4, padded
constexpr int GT = 128;      // GEMM CTA threads (4 warps x 16 rows)
constexpr int GR = 64;       // GEMM rows per CTA
constexpr int kWgradCtas = 608;  // weight-gradient CTAs (4 per SM of 152), each over many row chunks
constexpr int kReduceSlices = 16;  // slices of the CTA partials in the gradient reduction
constexpr int kMsgBackBlocks = 608;  // blocks of the message-layer backward (4 per SM of 152)

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

// --------------------------------- row operands ---------------------------------
/* Row operands of the GEMMs come from loaders: quad(r, ri, q) returns the
 * columns 4q..4q+3 of row r (FP32); prep(r, ri) fills per-row data that a
 * tile's loads share (message ends), once per row and tile. */
struct RowInfo {
	int src, dst;   // message source / destination rows (member offset included)
	float4 e;       // message edge features
};

struct LEnc {  // [xs (4), M, AoA, Re (3), 0...]: K = 16
	Graph G;
	const float *cond;
	__device__ void prep(int, RowInfo &) const {}
	__device__ float4 quad(int r, const RowInfo &, int q) const
	{
		const int b = r / G.nc, i = r - b * G.nc;
		if (q == 0) return G.xs[i];
		if (q == 1) return make_float4(cond[3 * b], cond[3 * b + 1], cond[3 * b + 2], 0.f);
		return make_float4(0.f, 0.f, 0.f, 0.f);
	}
};
struct LRows {  // plain rows x[r][0..nz) (row stride ld, both multiples of 4), zero beyond
	const float *x;
	int ld, nz;
	__device__ void prep(int, RowInfo &) const {}
	__device__ float4 quad(int r, const RowInfo &, int q) const
	{
		return 4 * q < nz ? reinterpret_cast<const float4 *>(x + (size_t)r * ld)[q] : make_float4(0.f, 0.f, 0.f, 0.f);
	}
};
struct LRelu {  // dZ = dY (Z > 0), rows of width 64
	const float *dy, *z;
	__device__ void prep(int, RowInfo &) const {}
	__device__ float4 quad(int r, const RowInfo &, int q) const
	{
		const float4 d = reinterpret_cast<const float4 *>(dy + (size_t)r * W)[q];
		const float4 zz = reinterpret_cast<const float4 *>(z + (size_t)r * W)[q];
		return make_float4(zz.x > 0.f ? d.x : 0.f, zz.y > 0.f ? d.y : 0.f, zz.z > 0.f ? d.z : 0.f,
		                   zz.w > 0.f ? d.w : 0.f);
	}
};
/* stages the rows of a 64-row tile as bf16 [64][K + 8] (8-byte stores) */
template <int K, class L>
__device__ __forceinline__ void stage_rows(const L &ld, int row0, int rows, RowInfo *ri, __nv_bfloat16 *sA)
{
	if (threadIdx.x < GR && row0 + (int)threadIdx.x < rows) ld.prep(row0 + threadIdx.x, ri[threadIdx.x]);
	__syncthreads();
	for (int e = threadIdx.x; e < GR * (K / 4); e += GT) {
		const int rr = e / (K / 4), q = e - rr * (K / 4), r = row0 + rr;
		const float4 v = r < rows ? ld.quad(r, ri[rr], q) : make_float4(0.f, 0.f, 0.f, 0.f);
		*reinterpret_cast<uint2 *>(sA + rr * (K + 8) + 4 * q) = make_uint2(pack_bf16(v.x, v.y), pack_bf16(v.z, v.w));
	}
}

// ----------------------------------- epilogues -----------------------------------
/* An epilogue gets columns n, n + 1 (n even) of output row r.  old(r, n) reads
 * what it adds to (or zeros): the kernels read it for all of a tile's
 * positions before the tile's MMAs, so those loads overlap the multiply
 * instead of waiting one by one between the stores. */
struct EStore {  // out = act(Z + bias) (pre = Z + bias when given), columns < ncols (even)
	const float *bias;
	float *out, *pre;
	int ldo, ncols, relu;
	__device__ float2 old(int, int) const { return make_float2(0.f, 0.f); }
	__device__ float4 old4(int, int) const { return make_float4(0.f, 0.f, 0.f, 0.f); }
	__device__ void put4(int r, int n, float4 z, float4) const  // columns n..n+3 (n % 4 == 0, n + 4 <= ncols)
	{
		const float4 v = bias ? make_float4(z.x + bias[n], z.y + bias[n + 1], z.z + bias[n + 2], z.w + bias[n + 3]) : z;
		if (pre) *reinterpret_cast<float4 *>(pre + (size_t)r * ldo + n) = v;
		*reinterpret_cast<float4 *>(out + (size_t)r * ldo + n) =
		    relu ? make_float4(fmaxf(v.x, 0.f), fmaxf(v.y, 0.f), fmaxf(v.z, 0.f), fmaxf(v.w, 0.f)) : v;
	}
	__device__ void operator()(int r, int n, float z0, float z1, float2) const
	{
		if (n >= ncols) return;
		const float2 v = make_float2(z0 + (bias ? bias[n] : 0.f), z1 + (bias ? bias[n + 1] : 0.f));
		if (pre) *reinterpret_cast<float2 *>(pre + (size_t)r * ldo + n) = v;
		*reinterpret_cast<float2 *>(out + (size_t)r * ldo + n) =
		    relu ? make_float2(fmaxf(v.x, 0.f), fmaxf(v.y, 0.f)) : v;
	}
};
struct EUpdate {  // hn = h + relu(Z + bu), pre = Z + bu
	const float *bias, *h;
	float *hn, *pre;
	__device__ float2 old(int r, int n) const { return *reinterpret_cast<const float2 *>(h + (size_t)r * W + n); }
	__device__ float4 old4(int r, int n) const { return *reinterpret_cast<const float4 *>(h + (size_t)r * W + n); }
	__device__ void put4(int r, int n, float4 z, float4 hh) const
	{
		const float4 v = make_float4(z.x + bias[n], z.y + bias[n + 1], z.z + bias[n + 2], z.w + bias[n + 3]);
		*reinterpret_cast<float4 *>(pre + (size_t)r * W + n) = v;
		*reinterpret_cast<float4 *>(hn + (size_t)r * W + n) = make_float4(
		    hh.x + fmaxf(v.x, 0.f), hh.y + fmaxf(v.y, 0.f), hh.z + fmaxf(v.z, 0.f), hh.w + fmaxf(v.w, 0.f));
	}
	__device__ void operator()(int r, int n, float z0, float z1, float2 hh) const
	{
		const float2 v = make_float2(z0 + bias[n], z1 + bias[n + 1]);
		*reinterpret_cast<float2 *>(pre + (size_t)r * W + n) = v;
		*reinterpret_cast<float2 *>(hn + (size_t)r * W + n) = make_float2(hh.x + fmaxf(v.x, 0.f), hh.y + fmaxf(v.y, 0.f));
	}
};

struct ESplit {  // input gradient of the node update [d h | d a]: dh += the first W columns, da stored
	float *dh, *da;   // da: row stride 2 W, columns W..2W-1 hold d a
	__device__ float2 old(int r, int n) const
	{
		return n < W ? *reinterpret_cast<const float2 *>(dh + (size_t)r * W + n) : make_float2(0.f, 0.f);
	}
	__device__ void operator()(int r, int n, float z0, float z1, float2 v) const
	{
		if (n < W) *reinterpret_cast<float2 *>(dh + (size_t)r * W + n) = make_float2(v.x + z0, v.y + z1);
		else *reinterpret_cast<float2 *>(da + (size_t)r * 2 * W + n) = make_float2(z0, z1);
	}
};
struct EAccum {  // out += Z (row stride ldo)
	float *out;
	int ldo;
	__device__ float2 old(int r, int n) const { return *reinterpret_cast<const float2 *>(out + (size_t)r * ldo + n); }
	__device__ void operator()(int r, int n, float z0, float z1, float2 v) const
	{
		*reinterpret_cast<float2 *>(out + (size_t)r * ldo + n) = make_float2(v.x + z0, v.y + z1);
	}
};

/* a tile's old values (epilogue inputs) for this thread's output positions */
template <int N, class E>
__device__ __forceinline__ void tile_old(const E &ep, int row0, int rows, float2 (*old)[2])
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	for (int nt = 0; nt < N / 8; nt++)
		for (int hh = 0; hh < 2; hh++) {
			const int r = row0 + warp * 16 + g + 8 * hh;
			old[nt][hh] = r < rows ? ep.old(r, nt * 8 + 2 * t) : make_float2(0.f, 0.f);
		}
}

template <int N, class E>
__device__ __forceinline__ void tile_epilogue(const E &ep, int row0, int rows, const float (*c)[4],
                                              const float2 (*old)[2])
{
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	for (int nt = 0; nt < N / 8; nt++)
		for (int hh = 0; hh < 2; hh++) {
			const int r = row0 + warp * 16 + g + 8 * hh;
			if (r < rows) ep(r, nt * 8 + 2 * t, c[nt][2 * hh], c[nt][2 * hh + 1], old[nt][hh]);
		}
}

// ------------------------------------ kernels ------------------------------------
/* Z = A W^T over persistent 64-row tiles: the CTA stages its weight operand once
 * (W [N][K], or with TRANS the transpose of W [K][N]: the input-gradient GEMM
 * dX = dZ W), then loops over tiles blockIdx.x, blockIdx.x + gridDim.x, ... */
template <int K, int N, bool TRANS, class L, class E>
__global__ void __launch_bounds__(GT) k_gemm(int rows, L ld, const float *w, int ldw, int nvalid, int kvalid, E ep)
{
	extern __shared__ __align__(16) unsigned char smem[];
	__nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(smem);  // [64][K + 8]
	__nv_bfloat16 *sB = sA + GR * (K + 8);                         // [N][K + 8]
	__shared__ RowInfo ri[GR];
	if (!TRANS) {
		stage_w<K, N>(w, ldw, nvalid, kvalid, sB);
	} else {
		for (int e = threadIdx.x; e < N * K; e += GT) {
			const int k = e / N, n = e - k * N;  // consecutive threads: consecutive columns of W's row k
			sB[n * (K + 8) + k] = __float2bfloat16_rn((n < nvalid && k < kvalid) ? w[(size_t)k * ldw + n] : 0.f);
		}
	}
	for (int row0 = blockIdx.x * GR; row0 < rows; row0 += gridDim.x * GR) {
		__syncthreads();  // the previous tile's operands are consumed
		stage_rows<K>(ld, row0, rows, ri, sA);
		__syncthreads();
		float2 old[N / 8][2];
		tile_old<N>(ep, row0, rows, old);
		float c[N / 8][4];
		tile_mma<K, N>(sA, sB, c);
		tile_epilogue<N>(ep, row0, rows, c, old);
	}
}

__device__ __forceinline__ void ldsm_x4_trans(unsigned *r, const __nv_bfloat16 *p)
{
	const unsigned a = (unsigned)__cvta_generic_to_shared(p);
	asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
	             : "r"(a));
}

/* Weight gradients dW[n][k] = sum_r dZ[r][n] X[r][k] and db[n] = sum_r dZ[r][n]:
 * the CTA accumulates its 64-row chunks blockIdx.x, blockIdx.x + gridDim.x, ...
 * in registers and writes one partial [N][K] (+ [N] for the bias).  Both
 * operands are staged row-major ([64][N + 8], [64][K + 8]); the MMA fragments
 * of their transposes come from ldmatrix.trans.  The chunk-to-CTA assignment
 * depends only on the row count and the grid, so the sums are reproducible;
 * the bias sums dZ in FP32. */
template <int K, int N, class XL, class ZL>
__global__ void __launch_bounds__(GT) k_wgrad(int rows, XL xl, ZL zl, float *part, float *bpart)
{
	static_assert(GT % (N / 4) == 0, "a thread stages the same column quad of dZ in every row");
	extern __shared__ __align__(16) unsigned char smem[];
	__nv_bfloat16 *sZ = reinterpret_cast<__nv_bfloat16 *>(smem);  // [64][N + 8]
	__nv_bfloat16 *sX = sZ + GR * (N + 8);                         // [64][K + 8]
	__shared__ RowInfo ri[GR];
	__shared__ float4 sbias[GT];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int nchunks = (rows + GR - 1) / GR;
	// warp w owns the output rows n in [16 w, 16 w + 16) (N = 64: 4 warps; N = 16: warp 0)
	float c[K / 8][4];
	for (int nt = 0; nt < K / 8; nt++)
		for (int q = 0; q < 4; q++) c[nt][q] = 0.f;
	float4 bsum = make_float4(0.f, 0.f, 0.f, 0.f);
	// ldmatrix row addresses: lane i -> matrix i / 8, row i % 8
	const int mi = lane >> 3, mr = lane & 7;
	for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
		const int row0 = ch * GR;
		__syncthreads();
		if (threadIdx.x < GR && row0 + (int)threadIdx.x < rows) {
			xl.prep(row0 + threadIdx.x, ri[threadIdx.x]);
		}
		__syncthreads();
		for (int e = threadIdx.x; e < GR * (K / 4); e += GT) {
			const int rr = e / (K / 4), q = e - rr * (K / 4), r = row0 + rr;
			const float4 v = r < rows ? xl.quad(r, ri[rr], q) : make_float4(0.f, 0.f, 0.f, 0.f);
			*reinterpret_cast<uint2 *>(sX + rr * (K + 8) + 4 * q) = make_uint2(pack_bf16(v.x, v.y), pack_bf16(v.z, v.w));
		}
		__syncthreads();  // zl.prep may overwrite ri (message ends of the same rows)
		if (threadIdx.x < GR && row0 + (int)threadIdx.x < rows) zl.prep(row0 + threadIdx.x, ri[threadIdx.x]);
		__syncthreads();
		for (int e = threadIdx.x; e < GR * (N / 4); e += GT) {
			const int rr = e / (N / 4), q = e - rr * (N / 4), r = row0 + rr;
			const float4 v = r < rows ? zl.quad(r, ri[rr], q) : make_float4(0.f, 0.f, 0.f, 0.f);
			bsum.x += v.x; bsum.y += v.y; bsum.z += v.z; bsum.w += v.w;
			*reinterpret_cast<uint2 *>(sZ + rr * (N + 8) + 4 * q) = make_uint2(pack_bf16(v.x, v.y), pack_bf16(v.z, v.w));
		}
		__syncthreads();
		if (warp * 16 < N) {
			for (int k0 = 0; k0 < GR; k0 += 16) {
				// A = dZ^T (16 x 16 at rows n0.., k = data rows k0..): matrices (k0, n0), (k0, n0+8), (k0+8, n0), (k0+8, n0+8)
				unsigned af[4];
				ldsm_x4_trans(af, sZ + (k0 + mr + ((mi & 2) ? 8 : 0)) * (N + 8) + warp * 16 + ((mi & 1) ? 8 : 0));
				for (int nt = 0; nt < K / 8; nt += 2) {
					// B = X (k = data rows): matrices (k0, f0), (k0+8, f0), (k0, f0+8), (k0+8, f0+8)
					unsigned bf[4];
					ldsm_x4_trans(bf, sX + (k0 + mr + ((mi & 1) ? 8 : 0)) * (K + 8) + nt * 8 + ((mi & 2) ? 8 : 0));
					mma_bf16(c[nt], af, bf);
					mma_bf16(c[nt + 1], af, bf + 2);
				}
			}
		}
	}
	const int g = lane >> 2, t = lane & 3;
	if (warp * 16 < N) {
		float *pc = part + (size_t)blockIdx.x * N * K;
		for (int nt = 0; nt < K / 8; nt++)
			for (int hh = 0; hh < 2; hh++)
				for (int j = 0; j < 2; j++) pc[(size_t)(warp * 16 + g + 8 * hh) * K + nt * 8 + 2 * t + j] = c[nt][2 * hh + j];
	}
	// bias: threads with the same column quad (threadIdx.x mod N/4) hold partials of different rows
	sbias[threadIdx.x] = bsum;
	__syncthreads();
	if (threadIdx.x < N / 4) {
		float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
		for (int j = threadIdx.x; j < GT; j += N / 4) {
			s.x += sbias[j].x; s.y += sbias[j].y; s.z += sbias[j].z; s.w += sbias[j].w;
		}
		reinterpret_cast<float4 *>(bpart + (size_t)blockIdx.x * N)[threadIdx.x] = s;
	}
}

/* ------------------------- GEMMs with bulk-copied operands -------------------------
 * Row operands that are whole contiguous FP32 row blocks are staged by bulk
 * copies (cp.async.bulk, the TMA engine) into a ring of NST tile buffers per
 * CTA: while the CTA converts one tile to BF16 and multiplies it, the copies
 * of its next tiles are in flight.  BRows<WA, WB, MODE>: rows of a (WA
 * columns) and, when WB > 0, rows of b (WB columns), both with row stride
 * equal to their width; MODE 0 gives the operand [a | b] (K = WA + WB), MODE 1
 * gives a where b > 0 (WB == WA, K = WA; the ReLU mask of a backward pass). */
constexpr int NST = 2;  // staged tiles per CTA

template <int WA, int WB, int MODE>
struct BRows {
	const float *a, *b;
	static constexpr int K = MODE == 0 ? WA + WB : WA;
	static constexpr int FLOATS = GR * (WA + WB);  // one staged tile
	static_assert(MODE == 0 || WA == WB, "a mask has the operand's width");
	__device__ unsigned bytes(int nr) const { return (unsigned)nr * (WA + WB) * 4u; }
	__device__ void copy(float *st, int row0, int nr, uint64_t *bar) const
	{
		bulk_g2s(st, a + (size_t)row0 * WA, (unsigned)nr * WA * 4u, bar);
		if (WB > 0) bulk_g2s(st + GR * WA, b + (size_t)row0 * WB, (unsigned)nr * WB * 4u, bar);
	}
	__device__ float4 quad(const float *st, int rr, int q) const
	{
		if (MODE == 1) {
			const float4 d = reinterpret_cast<const float4 *>(st + rr * WA)[q];
			const float4 z = reinterpret_cast<const float4 *>(st + GR * WA + rr * WA)[q];
			return make_float4(z.x > 0.f ? d.x : 0.f, z.y > 0.f ? d.y : 0.f, z.z > 0.f ? d.z : 0.f,
			                   z.w > 0.f ? d.w : 0.f);
		}
		if (WB == 0 || q < WA / 4) return reinterpret_cast<const float4 *>(st + rr * WA)[q];
		return reinterpret_cast<const float4 *>(st + GR * WA + rr * WB)[q - WA / 4];
	}
};

/* number of the CTA's tiles blockIdx.x + i gridDim.x below ntiles */
__device__ __forceinline__ int local_tiles(int ntiles)
{
	return (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
}

/* thread 0: the copies of the CTA's local tile i into ring slot i mod NST */
template <class X, class Z>
__device__ __forceinline__ void issue_tile(const X &x, const Z *z, int rows, int i, float *stg, uint64_t *bar,
                                           bool arm_only = false)
{
	const int s = i % NST, row0 = ((int)blockIdx.x + i * (int)gridDim.x) * GR, nr = min(GR, rows - row0);
	float *st = stg + (size_t)s * (X::FLOATS + (z ? Z::FLOATS : 0));
	mbar_arrive_expect_tx(&bar[s], x.bytes(nr) + (z ? z->bytes(nr) : 0u));
	if (arm_only) return;  // the wait-limit test: the bytes announced never come, no copy is in flight
	x.copy(st, row0, nr, &bar[s]);
	if (z) z->copy(st + X::FLOATS, row0, nr, &bar[s]);
}

/* after a wait ran out: thread 0 waits (bounded) for the copies still in
 * flight into the ring, from local tile i on, and records the error */
__device__ __forceinline__ void abort_ring(int i, int nloc, uint64_t *bar, int *err, long long limit)
{
	if (threadIdx.x != 0) return;
	for (int j = i; j < nloc && j < i + NST; j++) mbar_wait_bounded(&bar[j % NST], (j / NST) & 1, limit);
	atomicExch(err, 1);
}

/* k_gemm with the row operand staged by bulk copies (the weights as in k_gemm).
 * wait_test (the wait-limit test only): the CTA's first tile is announced on
 * its barrier but never copied, and waits give up after ~10 ms of SM clocks,
 * so every CTA takes the error path with no copy in flight for that slot. */
template <int K, int N, bool TRANS, class BL, class E>
__global__ void __launch_bounds__(GT) k_gemm_bulk(int rows, BL bl, const float *w, int ldw, int nvalid, int kvalid,
                                                   E ep, int *err, int wait_test)
{
	const long long limit = wait_test ? 20000000LL : 2000000000LL;
	static_assert(BL::K == K, "operand width");
	extern __shared__ __align__(16) unsigned char smem[];
	float *stg = reinterpret_cast<float *>(smem);                                   // [NST][BL::FLOATS]
	__nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(stg + NST * BL::FLOATS);  // [64][K + 8]
	__nv_bfloat16 *sB = sA + GR * (K + 8);                                          // [N][K + 8]
	__shared__ __align__(8) uint64_t bar[NST];
	__shared__ int abort_;
	const int nloc = local_tiles((rows + GR - 1) / GR);
	if (threadIdx.x == 0) {
		for (int s = 0; s < NST; s++) mbar_init(&bar[s], 1);
		abort_ = 0;
		mbar_init_fence();
	}
	__syncthreads();
	if (threadIdx.x == 0)
		for (int i = 0; i < NST && i < nloc; i++) issue_tile<BL, BL>(bl, nullptr, rows, i, stg, bar, wait_test && i == 0);
	if (!TRANS) {
		stage_w<K, N>(w, ldw, nvalid, kvalid, sB);
	} else {
		for (int e = threadIdx.x; e < N * K; e += GT) {
			const int k = e / N, n = e - k * N;
			sB[n * (K + 8) + k] = __float2bfloat16_rn((n < nvalid && k < kvalid) ? w[(size_t)k * ldw + n] : 0.f);
		}
	}
	for (int i = 0; i < nloc; i++) {
		const int s = i % NST, row0 = ((int)blockIdx.x + i * (int)gridDim.x) * GR, nr = min(GR, rows - row0);
		if (!mbar_wait_bounded(&bar[s], (i / NST) & 1, limit)) abort_ = 1;
		const float *st = stg + (size_t)s * BL::FLOATS;
		for (int e = threadIdx.x; e < GR * (K / 4); e += GT) {
			const int rr = e / (K / 4), q = e - rr * (K / 4);
			const float4 v = rr < nr ? bl.quad(st, rr, q) : make_float4(0.f, 0.f, 0.f, 0.f);
			*reinterpret_cast<uint2 *>(sA + rr * (K + 8) + 4 * q) = make_uint2(pack_bf16(v.x, v.y), pack_bf16(v.z, v.w));
		}
		fence_proxy_async_smem();  // this thread's reads of the slot before the copy that refills it
		__syncthreads();           // sA (and at i = 0 sB) ready; the slot is free
		if (abort_) { abort_ring(i, nloc, bar, err, limit / 10); return; }
		if (threadIdx.x == 0 && i + NST < nloc) issue_tile<BL, BL>(bl, nullptr, rows, i + NST, stg, bar);
		float2 old[N / 8][2];
		tile_old<N>(ep, row0, rows, old);
		float c[N / 8][4];
		tile_mma<K, N>(sA, sB, c);
		tile_epilogue<N>(ep, row0, rows, c, old);
		__syncthreads();  // sA consumed
	}
}

/* k_wgrad with both operands staged by bulk copies (one ring slot holds the
 * X and the dZ rows of a chunk) */
template <int K, int N, class XL, class ZL>
__global__ void __launch_bounds__(GT) k_wgrad_bulk(int rows, XL xl, ZL zl, float *part, float *bpart, int *err)
{
	static_assert(XL::K == K && ZL::K == N, "operand widths");
	static_assert(GT % (N / 4) == 0, "a thread stages the same column quad of dZ in every row");
	constexpr int SLOT = XL::FLOATS + ZL::FLOATS;
	extern __shared__ __align__(16) unsigned char smem[];
	float *stg = reinterpret_cast<float *>(smem);                                // [NST][SLOT]
	__nv_bfloat16 *sZ = reinterpret_cast<__nv_bfloat16 *>(stg + NST * SLOT);    // [64][N + 8]
	__nv_bfloat16 *sX = sZ + GR * (N + 8);                                       // [64][K + 8]
	__shared__ __align__(8) uint64_t bar[NST];
	__shared__ float4 sbias[GT];
	__shared__ int abort_;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int nloc = local_tiles((rows + GR - 1) / GR);
	if (threadIdx.x == 0) {
		for (int s = 0; s < NST; s++) mbar_init(&bar[s], 1);
		abort_ = 0;
		mbar_init_fence();
	}
	__syncthreads();
	if (threadIdx.x == 0)
		for (int i = 0; i < NST && i < nloc; i++) issue_tile(xl, &zl, rows, i, stg, bar);
	float c[K / 8][4];
	for (int nt = 0; nt < K / 8; nt++)
		for (int q = 0; q < 4; q++) c[nt][q] = 0.f;
	float4 bsum = make_float4(0.f, 0.f, 0.f, 0.f);
	const int mi = lane >> 3, mr = lane & 7;
	for (int i = 0; i < nloc; i++) {
		const int s = i % NST, row0 = ((int)blockIdx.x + i * (int)gridDim.x) * GR, nr = min(GR, rows - row0);
		if (!mbar_wait_bounded(&bar[s], (i / NST) & 1)) abort_ = 1;
		const float *st = stg + (size_t)s * SLOT;
		for (int e = threadIdx.x; e < GR * (K / 4); e += GT) {
			const int rr = e / (K / 4), q = e - rr * (K / 4);
			const float4 v = rr < nr ? xl.quad(st, rr, q) : make_float4(0.f, 0.f, 0.f, 0.f);
			*reinterpret_cast<uint2 *>(sX + rr * (K + 8) + 4 * q) = make_uint2(pack_bf16(v.x, v.y), pack_bf16(v.z, v.w));
		}
		for (int e = threadIdx.x; e < GR * (N / 4); e += GT) {
			const int rr = e / (N / 4), q = e - rr * (N / 4);
			const float4 v = rr < nr ? zl.quad(st + XL::FLOATS, rr, q) : make_float4(0.f, 0.f, 0.f, 0.f);
			bsum.x += v.x; bsum.y += v.y; bsum.z += v.z; bsum.w += v.w;
			*reinterpret_cast<uint2 *>(sZ + rr * (N + 8) + 4 * q) = make_uint2(pack_bf16(v.x, v.y), pack_bf16(v.z, v.w));
		}
		fence_proxy_async_smem();
		__syncthreads();
		if (abort_) { abort_ring(i, nloc, bar, err, 200000000LL); return; }
		if (threadIdx.x == 0 && i + NST < nloc) issue_tile(xl, &zl, rows, i + NST, stg, bar);
		if (warp * 16 < N) {
			for (int k0 = 0; k0 < GR; k0 += 16) {
				unsigned af[4];
				ldsm_x4_trans(af, sZ + (k0 + mr + ((mi & 2) ? 8 : 0)) * (N + 8) + warp * 16 + ((mi & 1) ? 8 : 0));
				for (int nt = 0; nt < K / 8; nt += 2) {
					unsigned bf[4];
					ldsm_x4_trans(bf, sX + (k0 + mr + ((mi & 1) ? 8 : 0)) * (K + 8) + nt * 8 + ((mi & 2) ? 8 : 0));
					mma_bf16(c[nt], af, bf);
					mma_bf16(c[nt + 1], af, bf + 2);
				}
			}
		}
		__syncthreads();  // sX, sZ consumed
	}
	const int g = lane >> 2, t = lane & 3;
	if (warp * 16 < N) {
		float *pc = part + (size_t)blockIdx.x * N * K;
		for (int nt = 0; nt < K / 8; nt++)
			for (int hh = 0; hh < 2; hh++)
				for (int j = 0; j < 2; j++) pc[(size_t)(warp * 16 + g + 8 * hh) * K + nt * 8 + 2 * t + j] = c[nt][2 * hh + j];
	}
	sbias[threadIdx.x] = bsum;
	__syncthreads();
	if (threadIdx.x < N / 4) {
		float4 sb = make_float4(0.f, 0.f, 0.f, 0.f);
		for (int j = threadIdx.x; j < GT; j += N / 4) {
			sb.x += sbias[j].x; sb.y += sbias[j].y; sb.z += sbias[j].z; sb.w += sbias[j].w;
		}
		reinterpret_cast<float4 *>(bpart + (size_t)blockIdx.x * N)[threadIdx.x] = sb;
	}
}

/* ------------------------ GEMMs on the fifth-generation tensor cores ------------------------
 * k_gemm_tc: Z = A W^T (+ epilogue) over 128-row tiles, one CTA of four warps
 * per tile at a time, persistent over its tiles.  The row operand arrives by
 * per-row bulk copies into a ring of NST padded FP32 tiles (row stride width + 4
 * floats: the conversion reads are free of bank conflicts); every thread
 * converts its own row to BF16 into the no-swizzle K-major core-matrix layout;
 * one thread issues the tile's K / 16 tcgen05.mma (M = 128) into a tensor-
 * memory accumulator of N FP32 columns and commits them to an mbarrier; each
 * thread then reads its row of the accumulator (tcgen05.ld 32x32b) and runs
 * the epilogue on it, four columns at a time.  The epilogue's inputs are
 * loaded while the MMAs run.  Every wait is bounded: one that runs out sets
 * the error word, and the CTA ends once its copies and MMAs are done and its
 * tensor memory is freed.
 * Measured on the 16 x 13,156-row node update: 129-148 us against 79 us for
 * k_gemm_bulk with mma.sync.  The GEMM moves rows (42 FLOP per FP32 byte) and
 * this kernel's 188 KB of shared memory leaves one CTA of four warps per SM,
 * each tile's steps in sequence; the mma.sync kernel runs two to three CTAs per
 * SM.  So mma.sync is the default path (fv_mpnn_set_gemm_path). */
constexpr int TM = 128;  // rows per tensor-core tile (one per thread)

/* [a | b] rows (WA, WB columns; b absent when WB == 0) copied row by row into
 * padded tile rows */
template <int WA, int WB>
struct PRows {
	const float *a, *b;
	static constexpr int K = WA + WB;
	static constexpr int PA = WA + 4, PB = WB > 0 ? WB + 4 : 0;  // padded row strides (floats)
	static constexpr int FLOATS = TM * (PA + PB);
	__device__ unsigned bytes(int nr) const { return (unsigned)nr * (WA + WB) * 4u; }
	/* warp-wide: lane l copies rows l, l + 32, ... of a, then of b */
	__device__ void copy_rows(float *st, int row0, int nr, uint64_t *bar, int lane) const
	{
		for (int j = lane; j < nr; j += 32) bulk_g2s(st + j * PA, a + (size_t)(row0 + j) * WA, WA * 4u, bar);
		if (WB > 0)
			for (int j = lane; j < nr; j += 32)
				bulk_g2s(st + TM * PA + j * PB, b + (size_t)(row0 + j) * WB, WB * 4u, bar);
	}
	/* columns 8 kc .. 8 kc + 7 of tile row m */
	__device__ void read8(const float *st, int m, int kc, float4 &lo, float4 &hi) const
	{
		const float *p = 8 * kc < WA ? st + m * PA + 8 * kc : st + TM * PA + m * PB + (8 * kc - WA);
		lo = reinterpret_cast<const float4 *>(p)[0];
		hi = reinterpret_cast<const float4 *>(p)[1];
	}
};

template <int K, int N, class PL, class E>
__global__ void __launch_bounds__(GT) k_gemm_tc(int rows, PL pl, const float *w, int ldw, int nvalid, int kvalid,
                                                 E ep, int *err)
{
	static_assert(PL::K == K && K % 16 == 0 && N % 16 == 0 && N >= 32 && N <= 256 && GT == TM, "tile shape");
	constexpr unsigned LBO_A = TM * 16, LBO_B = N * 16;  // bytes between K-chunks (8-row groups adjacent)
	constexpr uint32_t IDESC = tc_idesc_bf16(TM, N);
	extern __shared__ __align__(16) unsigned char smem[];
	unsigned char *sA = smem;                                           // [K / 8][TM][16 B]
	unsigned char *sB = sA + (size_t)TM * K * 2;                        // [K / 8][N][16 B]
	float *stg = reinterpret_cast<float *>(sB + (size_t)N * K * 2);     // [NST][PL::FLOATS]
	__shared__ __align__(8) uint64_t bar[NST];
	__shared__ __align__(8) uint64_t mma_bar;
	__shared__ uint32_t tmem_slot;
	// a copy wait that ran out (read after the conversion barrier), an MMA wait that ran out
	// (read after the tile's last barrier): two flags, so no write races with the other read
	__shared__ int abort_copy, abort_mma;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, m = threadIdx.x;
	const int ntiles = (rows + TM - 1) / TM;
	const int nloc = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
	if (warp == 0) tc_alloc(&tmem_slot, N);
	if (threadIdx.x == 0) {
		for (int s = 0; s < NST; s++) mbar_init(&bar[s], 1);
		mbar_init(&mma_bar, 1);
		abort_copy = 0;
		abort_mma = 0;
		mbar_init_fence();
	}
	tc_fence_before_sync();
	__syncthreads();
	tc_fence_after_sync();
	const uint32_t tmem = tmem_slot;
	auto issue = [&](int i) {  // warp 0: the copies of local tile i into ring slot i mod NST
		const int s = i % NST, row0 = ((int)blockIdx.x + i * (int)gridDim.x) * TM, nr = min(TM, rows - row0);
		if (lane == 0) mbar_arrive_expect_tx(&bar[s], pl.bytes(nr));
		__syncwarp();
		pl.copy_rows(stg + (size_t)s * PL::FLOATS, row0, nr, &bar[s], lane);
	};
	if (warp == 0)
		for (int i = 0; i < NST && i < nloc; i++) issue(i);
	// weights W [N][K] (row stride ldw) as BF16 core matrices, once per CTA
	for (int e = threadIdx.x; e < N * (K / 8); e += GT) {
		const int n = e % N, kc = e / N;
		unsigned q[4];
		for (int j = 0; j < 4; j++) {
			const int k = 8 * kc + 2 * j;
			const float x0 = (n < nvalid && k < kvalid) ? w[(size_t)n * ldw + k] : 0.f;
			const float x1 = (n < nvalid && k + 1 < kvalid) ? w[(size_t)n * ldw + k + 1] : 0.f;
			q[j] = pack_bf16(x0, x1);
		}
		*reinterpret_cast<uint4 *>(sB + (size_t)kc * LBO_B + n * 16) = make_uint4(q[0], q[1], q[2], q[3]);
	}
	const unsigned aaddr = smem_u32(sA), baddr = smem_u32(sB);
	int i = 0;
	for (; i < nloc; i++) {
		const int s = i % NST, row0 = ((int)blockIdx.x + i * (int)gridDim.x) * TM, nr = min(TM, rows - row0);
		if (!mbar_wait_bounded(&bar[s], (i / NST) & 1)) abort_copy = 1;
		const float *st = stg + (size_t)s * PL::FLOATS;
		for (int kc = 0; kc < K / 8; kc++) {
			float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
			if (m < nr) pl.read8(st, m, kc, lo, hi);
			*reinterpret_cast<uint4 *>(sA + (size_t)kc * LBO_A + m * 16) =
			    make_uint4(pack_bf16(lo.x, lo.y), pack_bf16(lo.z, lo.w), pack_bf16(hi.x, hi.y), pack_bf16(hi.z, hi.w));
		}
		fence_proxy_async_smem();  // the BF16 tile (and at i = 0 the weights) to the tensor cores; the slot's reads
		__syncthreads();
		if (abort_copy) break;
		if (warp == 0 && i + NST < nloc) issue(i + NST);
		if (threadIdx.x == 0) {
			tc_fence_after_sync();
			for (int kk = 0; kk < K / 16; kk++)
				tc_mma_bf16(tmem, tc_sdesc(aaddr + kk * 2 * LBO_A, LBO_A, 128), tc_sdesc(baddr + kk * 2 * LBO_B, LBO_B, 128),
				            IDESC, kk > 0);
			tc_commit(&mma_bar);
		}
		// The epilogue goes through shared memory (sA is free once the MMAs have completed):
		// each warp turns its 32 rows x 16 columns of the accumulator into pieces of 8 rows x
		// 64 bytes, so the epilogue's loads and stores are coalesced.  Its inputs are loaded
		// in the same pattern while the MMAs run.
		float *xp = reinterpret_cast<float *>(sA) + warp * 32 * 20;  // [32][20] per warp
		const int er = lane >> 2, ec = 4 * (lane & 3);               // row in an 8-row piece, column quad
		float4 old[N / 16][4];
		for (int cc = 0; cc < N / 16; cc++)
			for (int j = 0; j < 4; j++) {
				const int rr = warp * 32 + 8 * j + er;
				old[cc][j] = rr < nr ? ep.old4(row0 + rr, 16 * cc + ec) : make_float4(0.f, 0.f, 0.f, 0.f);
			}
		if (!mbar_wait_bounded(&mma_bar, i & 1)) abort_mma = 1;
		tc_fence_after_sync();
		for (int cc = 0; cc < N / 16; cc++) {
			float v[16];
			tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(16 * cc), v);
			for (int q = 0; q < 4; q++)
				reinterpret_cast<float4 *>(xp + lane * 20)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
			__syncwarp();
			for (int j = 0; j < 4; j++) {
				const int rr = warp * 32 + 8 * j + er;
				const float4 z = *reinterpret_cast<const float4 *>(xp + (8 * j + er) * 20 + ec);
				if (rr < nr) ep.put4(row0 + rr, 16 * cc + ec, z, old[cc][j]);
			}
			__syncwarp();
		}
		tc_fence_before_sync();
		__syncthreads();  // sA and the accumulator free for the next tile
		if (abort_mma) { i++; break; }
	}
	if ((abort_copy || abort_mma) && threadIdx.x == 0) {
		// copies still in flight into the ring (tiles from the one waited on), and the last MMAs
		for (int j = i; j < nloc && j < i + NST; j++) mbar_wait_bounded(&bar[j % NST], (j / NST) & 1, 200000000LL);
		mbar_wait_bounded(&mma_bar, (i - 1) & 1, 200000000LL);
		atomicExch(err, 1);
	}
	tc_fence_before_sync();
	__syncthreads();
	tc_fence_after_sync();
	if (warp == 0) tc_dealloc(tmem, N);
}

/* sum of the CTA partials of the valid [nv][kv] part of the padded [N][K]
 * tiles: S slices of the CTA list in blockIdx.y, each into tmp[slice][nv*kv + nv] */
__global__ void k_reduce_parts(int nparts, int N, int K, int nv, int kv, const float *part, const float *bpart,
                               float *tmp)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x, S = gridDim.y, sl = blockIdx.y;
	const int per = (nparts + S - 1) / S, c0 = sl * per, c1 = min(nparts, c0 + per);
	const int nw = nv * kv;
	if (e < nw) {
		const int n = e / kv, k = e - n * kv;
		float s = 0.f;
		for (int c = c0; c < c1; c++) s += part[((size_t)c * N + n) * K + k];
		tmp[(size_t)sl * (nw + nv) + e] = s;
	} else if (e < nw + nv) {
		float s = 0.f;
		for (int c = c0; c < c1; c++) s += bpart[(size_t)c * N + (e - nw)];
		tmp[(size_t)sl * (nw + nv) + e] = s;
	}
}

/* gw[e] += sum of the slices (fixed order); then the bias (gb may be null).
 * stacked: the partial is P[n][k] = sum_r h[r][n] [S_out, S_in][r][k] of a
 * message layer (nv = 64, kv = 128), added to the message weights' gradient
 * at row k mod 64, column (k / 64) * 64 + n (row stride ldg). */
__global__ void k_reduce_final(int S, int nw, int nv, int kv, const float *tmp, float *gw, float *gb, int stacked,
                               int ldg)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= nw + nv || (e >= nw && !gb)) return;
	float s = 0.f;
	for (int sl = 0; sl < S; sl++) s += tmp[(size_t)sl * (nw + nv) + e];
	if (e >= nw) gb[e - nw] += s;
	else if (!stacked) gw[e] += s;
	else {
		const int n = e / kv, k = e - n * kv;
		gw[(size_t)(k % W) * ldg + (k / W) * W + n] += s;
	}
}

__device__ __forceinline__ float4 relu4(float4 v)
{
	return make_float4(fmaxf(v.x, 0.f), fmaxf(v.y, 0.f), fmaxf(v.z, 0.f), fmaxf(v.w, 0.f));
}
__device__ __forceinline__ float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
/* v where z > 0, else 0 (per component) */
__device__ __forceinline__ float4 mask4(float4 z, float4 v)
{
	return make_float4(z.x > 0.f ? v.x : 0.f, z.y > 0.f ? v.y : 0.f, z.z > 0.f ? v.z : 0.f, z.w > 0.f ? v.w : 0.f);
}
__device__ __forceinline__ float bfr(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

/* The message-level kernels use 16 threads per row, 4 columns each (float4),
 * 256-thread blocks of 16 rows. */
constexpr int MROWS = 16;

/* a_i = sum of the messages relu(Zm) into cell i (fixed CSR order) */
__global__ void k_aggregate(Graph G, int B, const float *zm, float *agg)
{
	const int r = blockIdx.x * MROWS + (threadIdx.x >> 4), q4 = threadIdx.x & 15;
	if (r >= B * G.nc) return;
	const int b = r / G.nc, i = r - b * G.nc;
	const float4 *mb = reinterpret_cast<const float4 *>(zm + (size_t)b * 2 * G.nf * W);
	float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
	for (int q = G.in_ptr[i]; q < G.in_ptr[i + 1]; q++) s = add4(s, relu4(mb[(size_t)G.in_idx[q] * (W / 4) + q4]));
	reinterpret_cast<float4 *>(agg)[(size_t)r * (W / 4) + q4] = s;
}

/* Wst [128][64]: rows 0..63 the message weights' h_src block W_s, rows
 * 64..127 the h_dst block W_d (Wm row stride 2 W + 3) */
__global__ void k_stack_w(const float *wm, float *wst)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= 2 * W * W) return;
	const int n = e / W, k = e - n * W;
	wst[e] = wm[(size_t)(n % W) * (2 * W + 3) + (n / W) * W + k];
}

/* Zm = W_s h_src + W_d h_dst + W_e e + bm from the per-cell projections
 * pc = [W_s h, W_d h] (row stride 2 W); the edge term with BF16-rounded W_e and
 * e, as the GEMM operands. */
__global__ void k_msg_fwd(Graph G, int B, const float *pc, const float *wm, const float *bm, float *zm)
{
	__shared__ float swe[W][3];
	for (int e = threadIdx.x; e < 3 * W; e += blockDim.x) {
		const int n = e / 3, c = e - 3 * n;
		swe[n][c] = bfr(wm[(size_t)n * (2 * W + 3) + 2 * W + c]);
	}
	__syncthreads();
	const int r = blockIdx.x * MROWS + (threadIdx.x >> 4), q4 = threadIdx.x & 15;
	const int per = 2 * G.nf;
	if (r >= B * per) return;
	const int b = r / per;
	int src, dst;
	float4 e;
	msg_ends(G, r - b * per, src, dst, e);
	const float ex = bfr(e.x), ey = bfr(e.y), ez = bfr(e.z);
	const float4 ps = reinterpret_cast<const float4 *>(pc + ((size_t)b * G.nc + src) * 2 * W)[q4];
	const float4 pd = reinterpret_cast<const float4 *>(pc + ((size_t)b * G.nc + dst) * 2 * W + W)[q4];
	const float4 bb = reinterpret_cast<const float4 *>(bm)[q4];
	float z[4];
	const float a0[4] = {ps.x, ps.y, ps.z, ps.w}, a1[4] = {pd.x, pd.y, pd.z, pd.w}, a2[4] = {bb.x, bb.y, bb.z, bb.w};
	for (int j = 0; j < 4; j++) {
		const int n = 4 * q4 + j;
		z[j] = a0[j] + a1[j] + (ex * swe[n][0] + ey * swe[n][1] + ez * swe[n][2]) + a2[j];
	}
	reinterpret_cast<float4 *>(zm)[(size_t)r * (W / 4) + q4] = make_float4(z[0], z[1], z[2], z[3]);
}

/* Message-layer backward from da (the aggregate's gradient, columns off.. of
 * rows with stride lda): per cell the sums of dZm = da[dst] (Zm > 0) over its
 * outgoing and incoming messages, S = [S_out, S_in] (row stride 2 W); and the
 * edge-weight and bias gradients sum_m dZm e_m, sum_m dZm accumulated over
 * each cell's incoming messages (every message once), per thread in fixed
 * order over the cells it visits, then per block in fixed order into
 * epart[block][64][4].  Grid-stride over cells. */
__global__ void k_msg_back(Graph G, int B, const float *zm, const float *dagg, int lda, int off, float *S,
                           float *epart)
{
	const int q4 = threadIdx.x & 15, slot = threadIdx.x >> 4;
	const int rows = B * G.nc;
	const size_t per = 2 * (size_t)G.nf;
	float ae[4][4] = {};  // [column j][e0, e1, e2, bias]
	for (int r = blockIdx.x * MROWS + slot; r < rows; r += gridDim.x * MROWS) {
		const int b = r / G.nc, i = r - b * G.nc;
		const float4 *zb = reinterpret_cast<const float4 *>(zm + (size_t)b * per * W);
		const float4 di = reinterpret_cast<const float4 *>(dagg + (size_t)r * lda + off)[q4];
		float4 sin_ = make_float4(0.f, 0.f, 0.f, 0.f), sout = sin_;
		for (int q = G.in_ptr[i]; q < G.in_ptr[i + 1]; q++) {
			const int m = G.in_idx[q];
			const float4 dz = mask4(zb[(size_t)m * (W / 4) + q4], di);
			sin_ = add4(sin_, dz);
			int s0, d0;
			float4 e;
			msg_ends(G, m, s0, d0, e);
			const float ee[3] = {bfr(e.x), bfr(e.y), bfr(e.z)};
			const float dzs[4] = {dz.x, dz.y, dz.z, dz.w};
			for (int j = 0; j < 4; j++) {
				for (int c = 0; c < 3; c++) ae[j][c] += dzs[j] * ee[c];
				ae[j][3] += dzs[j];
			}
		}
		for (int q = G.out_ptr[i]; q < G.out_ptr[i + 1]; q++) {
			const int m = G.out_idx[q];
			int s0, d0;
			float4 e;
			msg_ends(G, m, s0, d0, e);
			const float4 dd = reinterpret_cast<const float4 *>(dagg + ((size_t)b * G.nc + d0) * lda + off)[q4];
			sout = add4(sout, mask4(zb[(size_t)m * (W / 4) + q4], dd));
		}
		reinterpret_cast<float4 *>(S + (size_t)r * 2 * W)[q4] = sout;
		reinterpret_cast<float4 *>(S + (size_t)r * 2 * W + W)[q4] = sin_;
	}
	__shared__ float sh[MROWS][W][4];
	for (int j = 0; j < 4; j++)
		for (int c = 0; c < 4; c++) sh[slot][4 * q4 + j][c] = ae[j][c];
	__syncthreads();
	{
		const int n = threadIdx.x >> 2, c = threadIdx.x & 3;  // 256 threads: 64 columns x 4
		float t = 0.f;
		for (int k = 0; k < MROWS; k++) t += sh[k][n][c];
		epart[((size_t)blockIdx.x * W + n) * 4 + c] = t;
	}
}

/* edge-weight columns and bias of a message layer's gradient: one block per
 * (column n, component c): the block partials summed in a fixed order (strided
 * per thread, then a shared-memory tree) */
__global__ void k_reduce_edge(int nblk, const float *epart, float *gwm, float *gbm)
{
	__shared__ float sh[128];
	const int n = blockIdx.x >> 2, c = blockIdx.x & 3;
	float t = 0.f;
	for (int k = threadIdx.x; k < nblk; k += 128) t += epart[((size_t)k * W + n) * 4 + c];
	sh[threadIdx.x] = t;
	__syncthreads();
	for (int o = 64; o > 0; o >>= 1) {
		if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		if (c < 3) gwm[(size_t)n * (2 * W + 3) + 2 * W + c] += sh[0];
		else gbm[n] += sh[0];
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
	float *h = nullptr, *zpre = nullptr, *mpre = nullptr, *agg = nullptr, *upre = nullptr;
	float *y = nullptr, *dy = nullptr, *cond = nullptr, *uinf = nullptr, *t2 = nullptr, *dh = nullptr;
	float *pc = nullptr, *sgrad = nullptr, *wst = nullptr, *epart = nullptr;
	float *part = nullptr, *bpart = nullptr, *rtmp = nullptr, *lpart = nullptr;
	int *err = nullptr;  // set by a kernel whose bulk-copy or MMA wait ran out of time
	int gemm_path = 1;   // forward cell GEMMs: 0 tcgen05, 1 mma.sync (faster here: see k_gemm_tc)
	int wait_test = 0;   // the wait-limit test (k_gemm_bulk)
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


cudaError_t ensure_capacity(fv_mpnn *N, int B)
{
	if (B <= N->cap_b) return cudaSuccess;
	// activations are re-allocated for the larger batch; until all of them
	// are, the network holds none (a failed allocation leaves no stale buffer)
	N->cap_b = 0;
	for (float **q : {&N->h, &N->zpre, &N->mpre, &N->agg, &N->upre, &N->y, &N->dy, &N->cond, &N->uinf, &N->t2,
	                  &N->dh, &N->pc, &N->sgrad, &N->wst, &N->epart, &N->part, &N->bpart, &N->rtmp, &N->lpart})
		if (*q) {
			cudaFree(*q);
			for (auto &o : N->owned)
				if (o == *q) o = nullptr;
			*q = nullptr;
		}
	const size_t nc = N->G.nc, nm = 2 * (size_t)N->G.nf, L = N->lay.layers;
	const size_t rows_m = B * nm, rows_c = B * nc;
	cudaError_t e = cudaSuccess;
	auto al = [&](float **p, size_t n) { if (!e) e = mall(N, p, n); };
	al(&N->h, (L + 1) * rows_c * W);
	al(&N->zpre, rows_c * W);
	al(&N->mpre, L * rows_m * W);
	al(&N->agg, L * rows_c * W);
	al(&N->upre, L * rows_c * W);
	al(&N->y, rows_c * 4);
	al(&N->dy, rows_c * 4);
	al(&N->cond, 3 * (size_t)B);
	al(&N->uinf, 4 * (size_t)B);
	al(&N->t2, rows_c * KUPD);
	al(&N->dh, rows_c * W);
	al(&N->pc, rows_c * 2 * W);
	al(&N->sgrad, rows_c * 2 * W);
	al(&N->wst, L * 2 * W * W);
	al(&N->epart, (size_t)kMsgBackBlocks * W * 4);
	al(&N->part, kWgradCtas * (size_t)W * 2 * W);
	al(&N->bpart, kWgradCtas * (size_t)W);
	al(&N->rtmp, kReduceSlices * ((size_t)W * 2 * W + W));
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
/* persistent GEMM grid: at most 4 CTAs per SM (152 SMs) over the 64-row tiles */
unsigned gemm_grid(size_t rows) { return std::min<unsigned>(nb(rows, GR), 4 * 152); }

/* Z = A W^T (or A W with TRANS) over rows, epilogue ep */
template <int K, int Nn, bool TRANS, class L, class E>
void gemm(size_t rows, L ld, const float *w, int ldw, int nvalid, int kvalid, E ep, cudaStream_t s)
{
	const size_t sm = sizeof(__nv_bfloat16) * (GR + Nn) * (K + 8);
	k_gemm<K, Nn, TRANS, L, E><<<gemm_grid(rows), GT, sm, s>>>((int)rows, ld, w, ldw, nvalid, kvalid, ep);
}

/* CTAs of kern resident at once on the current device (dynamic shared memory
 * smem), at most cap; raises the kernel's dynamic shared-memory limit first */
template <class F>
unsigned resident_grid(F *kern, size_t smem, size_t work, unsigned cap)
{
	int dev = 0, sms = 0, per = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, GT, smem);
	const size_t n = std::min<size_t>({work, (size_t)std::max(per, 1) * std::max(sms, 1), (size_t)cap});
	return (unsigned)std::max<size_t>(n, 1);
}

/* gemm on the fifth-generation tensor cores (k_gemm_tc; rows of PRows) */
template <int K, int Nn, class PL, class E>
void gemm_tc(fv_mpnn *N, size_t rows, PL pl, const float *w, int ldw, int nvalid, int kvalid, E ep, cudaStream_t s)
{
	const size_t sm = sizeof(__nv_bfloat16) * (size_t)(TM + Nn) * K + sizeof(float) * NST * PL::FLOATS;
	auto *kern = k_gemm_tc<K, Nn, PL, E>;
	const unsigned grid = resident_grid(kern, sm, nb(rows, TM), 4 * 152);
	kern<<<grid, GT, sm, s>>>((int)rows, pl, w, ldw, nvalid, kvalid, ep, N->err);
}

/* gemm with the row operand staged by bulk copies (BRows) */
template <int K, int Nn, bool TRANS, class BL, class E>
void gemm_bulk(fv_mpnn *N, size_t rows, BL bl, const float *w, int ldw, int nvalid, int kvalid, E ep, cudaStream_t s)
{
	const size_t sm = sizeof(float) * NST * BL::FLOATS + sizeof(__nv_bfloat16) * (GR + Nn) * (K + 8);
	auto *kern = k_gemm_bulk<K, Nn, TRANS, BL, E>;
	const unsigned grid = resident_grid(kern, sm, nb(rows, GR), 4 * 152);
	kern<<<grid, GT, sm, s>>>((int)rows, bl, w, ldw, nvalid, kvalid, ep, N->err, N->wait_test);
}

/* forward pass for B members; activations kept for the backward pass */
cudaError_t forward(fv_mpnn *N, int B, cudaStream_t s)
{
	const Graph &G = N->G;
	const MpnnLayout &Y = N->lay;
	const float *P = N->p;
	const size_t nc = G.nc, nm = 2 * (size_t)G.nf, rows_c = B * nc, rows_m = B * nm;
	gemm<KENC, W, false>(rows_c, LEnc{G, N->cond}, P + Y.we, 7, W, 7, EStore{P + Y.be, N->h, N->zpre, W, W, 1}, s);
	for (int l = 0; l < Y.layers; l++) {
		const float *hl = N->h + l * rows_c * W;
		float *mp = N->mpre + l * rows_m * W;  // Zm; the messages relu(Zm) are not stored
		// the message MLP's first layer per cell: pc = [W_s h, W_d h], then per message
		// Zm = pc_s[src] + pc_d[dst] + W_e e + bm
		float *wst = N->wst + (size_t)l * 2 * W * W;
		k_stack_w<<<nb(2 * W * W, 256), 256, 0, s>>>(P + Y.wm[l], wst);
		const EStore pc_ep{nullptr, N->pc, nullptr, 2 * W, 2 * W, 0};
		if (N->gemm_path == 0) gemm_tc<W, 2 * W>(N, rows_c, PRows<W, 0>{hl, nullptr}, wst, W, 2 * W, W, pc_ep, s);
		else gemm_bulk<W, 2 * W, false>(N, rows_c, BRows<W, 0, 0>{hl, nullptr}, wst, W, 2 * W, W, pc_ep, s);
		k_msg_fwd<<<nb(rows_m, MROWS), 256, 0, s>>>(G, B, N->pc, P + Y.wm[l], P + Y.bm[l], mp);
		float *al = N->agg + l * rows_c * W;
		k_aggregate<<<nb(rows_c, MROWS), 256, 0, s>>>(G, B, mp, al);
		const EUpdate up_ep{P + Y.bu[l], hl, N->h + (l + 1) * rows_c * W, N->upre + l * rows_c * W};
		if (N->gemm_path == 0) gemm_tc<KUPD, W>(N, rows_c, PRows<W, W>{hl, al}, P + Y.wu[l], KUPD, W, KUPD, up_ep, s);
		else gemm_bulk<KUPD, W, false>(N, rows_c, BRows<W, W, 0>{hl, al}, P + Y.wu[l], KUPD, W, KUPD, up_ep, s);
	}
	gemm_bulk<W, NDEC, false>(N, rows_c, BRows<W, 0, 0>{N->h + Y.layers * rows_c * W, nullptr}, P + Y.wd, W, 4, W,
	                          EStore{P + Y.bd, N->y, nullptr, 4, 4, 0}, s);
	count_launches(2 + 5 * Y.layers);
	return cudaGetLastError();
}

/* weight and bias gradients of one layer: CTA partials, then a sliced
 * fixed-order reduction into gw [nv][kv] and gb [nv] (accumulated) */
template <int K, int Nn, class XL, class ZL>
void wgrad(fv_mpnn *N, size_t rows, XL xl, ZL zl, int nv, int kv, float *gw, float *gb, cudaStream_t s,
           int stacked = 0)
{
	const unsigned ctas = std::min<unsigned>(nb(rows, GR), kWgradCtas);
	const size_t sm = sizeof(__nv_bfloat16) * GR * (Nn + 8 + K + 8);
	k_wgrad<K, Nn, XL, ZL><<<ctas, GT, sm, s>>>((int)rows, xl, zl, N->part, N->bpart);
	const int nw = nv * kv;
	k_reduce_parts<<<dim3(nb(nw + nv, 256), kReduceSlices), 256, 0, s>>>((int)ctas, Nn, K, nv, kv, N->part, N->bpart,
	                                                                   N->rtmp);
	k_reduce_final<<<nb(nw + nv, 256), 256, 0, s>>>(kReduceSlices, nw, nv, kv, N->rtmp, gw, gb, stacked, 2 * W + 3);
	count_launches(3);
}

/* wgrad with both operands staged by bulk copies (BRows) */
template <int K, int Nn, class XL, class ZL>
void wgrad_bulk(fv_mpnn *N, size_t rows, XL xl, ZL zl, int nv, int kv, float *gw, float *gb, cudaStream_t s,
                int stacked = 0)
{
	const size_t sm = sizeof(float) * NST * (XL::FLOATS + ZL::FLOATS) + sizeof(__nv_bfloat16) * GR * (Nn + 8 + K + 8);
	auto *kern = k_wgrad_bulk<K, Nn, XL, ZL>;
	const unsigned ctas = resident_grid(kern, sm, nb(rows, GR), kWgradCtas);
	kern<<<ctas, GT, sm, s>>>((int)rows, xl, zl, N->part, N->bpart, N->err);
	const int nw = nv * kv;
	k_reduce_parts<<<dim3(nb(nw + nv, 256), kReduceSlices), 256, 0, s>>>((int)ctas, Nn, K, nv, kv, N->part, N->bpart,
	                                                                   N->rtmp);
	k_reduce_final<<<nb(nw + nv, 256), 256, 0, s>>>(kReduceSlices, nw, nv, kv, N->rtmp, gw, gb, stacked, 2 * W + 3);
	count_launches(3);
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
	// decoder: y = Wd h + bd;  dh = dy Wd
	wgrad<W, 16>(N, rows_c, LRows{hL, W, W}, LRows{N->dy, 4, 4}, 4, W, Gr + Y.wd, Gr + Y.bd, s);
	gemm<16, W, true>(rows_c, LRows{N->dy, 4, 4}, P + Y.wd, W, W, 4, EStore{nullptr, N->dh, nullptr, W, W, 0}, s);
	count_launches(1);
	for (int l = Y.layers - 1; l >= 0; l--) {
		const float *hl = N->h + l * rows_c * W;
		const float *al = N->agg + l * rows_c * W;
		const float *up = N->upre + l * rows_c * W, *mp = N->mpre + l * rows_m * W;
		// update: hn = h + relu(Zu), Zu = Wu [h, a] + bu;  dZu = dh (Zu > 0)
		wgrad_bulk<KUPD, W>(N, rows_c, BRows<W, W, 0>{hl, al}, BRows<W, W, 1>{N->dh, up}, W, KUPD, Gr + Y.wu[l],
		                    Gr + Y.bu[l], s);
		// dh (residual path) += the update's d[h] columns; d[a] into t2 (columns W..2W-1).
		// Each CTA reads and then updates only its own rows of dh.
		gemm_bulk<W, KUPD, true>(N, rows_c, BRows<W, W, 1>{N->dh, up}, P + Y.wu[l], KUPD, KUPD, W,
		                         ESplit{N->dh, N->t2}, s);
		// messages: dZm = d[a] of the destination, masked by Zm > 0, summed per cell over
		// outgoing (S_out) and incoming (S_in) messages; the first layer's weight and input
		// gradients are cell-level GEMMs of S = [S_out, S_in]
		const unsigned mb = std::min<unsigned>(nb(rows_c, MROWS), kMsgBackBlocks);
		k_msg_back<<<mb, 256, 0, s>>>(G, B, mp, N->t2, KUPD, W, N->sgrad, N->epart);
		k_reduce_edge<<<4 * W, 128, 0, s>>>((int)mb, N->epart, Gr + Y.wm[l], Gr + Y.bm[l]);
		// (plain loads: one CTA per SM fits the bulk ring of this pair, which ran slower)
		wgrad<2 * W, W>(N, rows_c, LRows{N->sgrad, 2 * W, 2 * W}, LRows{hl, W, W}, W, 2 * W, Gr + Y.wm[l], nullptr, s,
		                1);
		const float *wst = N->wst + (size_t)l * 2 * W * W;
		gemm_bulk<2 * W, W, true>(N, rows_c, BRows<2 * W, 0, 0>{N->sgrad, nullptr}, wst, W, W, 2 * W, EAccum{N->dh, W},
		                          s);
		count_launches(4);
	}
	// encoder: h0 = relu(We x + be)
	wgrad<KENC, W>(N, rows_c, LEnc{G, N->cond}, LRelu{N->dh, N->zpre}, W, 7, Gr + Y.we, Gr + Y.be, s);
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

/* status of a synchronised call: a kernel whose bulk-copy wait ran out of
 * time left its error word set (cleared here) */
fv_status finish(fv_mpnn *N, cudaError_t e, const char *what)
{
	int timed_out = 0;
	if (!e) e = cudaMemcpy(&timed_out, N->err, sizeof(int), cudaMemcpyDeviceToHost);
	if (!e && timed_out) {
		cudaMemset(N->err, 0, sizeof(int));
		set_error(std::string(what) + ": a bulk-copy or MMA wait of a GEMM ran out of time");
		return FV_ERR_CUDA;
	}
	return cuda_status(e, what);
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
	up(&N->err, std::vector<int>(1, 0));
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

fv_status fv_mpnn_set_gemm_path(fv_mpnn *N, int path)
{
	if (!N || path < 0 || path > 1) { set_error("invalid argument"); return FV_ERR_INVALID; }
	N->gemm_path = path;
	return FV_OK;
}

fv_status fv_mpnn_test_wait_limit(fv_mpnn *N, int on)
{
	if (!N) { set_error("null argument"); return FV_ERR_INVALID; }
	N->wait_test = on ? 1 : 0;
	return FV_OK;
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
	return finish(N, e, "mpnn predict");
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
	return finish(N, e, "mpnn gradients");
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
