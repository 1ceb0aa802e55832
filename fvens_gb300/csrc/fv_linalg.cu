// Preconditioners, block SpMV and batched FGMRES; see fv_linalg.cuh.
#include <algorithm>
#include <cmath>
#include "fv_linalg.cuh"

namespace fvg {

namespace {

constexpr int BS = 128;
constexpr int RBS = 256;  // reduction block size

template <class R>
__device__ __forceinline__ void load_blk(const R *p, R *b)
{
	if (sizeof(R) == 4) {
		const float4 *q = reinterpret_cast<const float4 *>(p);
		for (int k = 0; k < 4; k++) {
			const float4 v = q[k];
			b[4 * k] = R(v.x); b[4 * k + 1] = R(v.y); b[4 * k + 2] = R(v.z); b[4 * k + 3] = R(v.w);
		}
	} else {
		const double2 *q = reinterpret_cast<const double2 *>(p);
		for (int k = 0; k < 8; k++) {
			const double2 v = q[k];
			b[2 * k] = R(v.x); b[2 * k + 1] = R(v.y);
		}
	}
}

template <class R>
__device__ __forceinline__ void store_blk(R *p, const R *b)
{
	if (sizeof(R) == 4) {
		float4 *q = reinterpret_cast<float4 *>(p);
		for (int k = 0; k < 4; k++) q[k] = make_float4(float(b[4 * k]), float(b[4 * k + 1]), float(b[4 * k + 2]), float(b[4 * k + 3]));
	} else {
		double2 *q = reinterpret_cast<double2 *>(p);
		for (int k = 0; k < 8; k++) q[k] = make_double2(double(b[2 * k]), double(b[2 * k + 1]));
	}
}

template <class R>
__device__ __forceinline__ void mv(const R *a, const R *x, R *y)
{
	for (int i = 0; i < 4; i++) y[i] = a[4 * i] * x[0] + a[4 * i + 1] * x[1] + a[4 * i + 2] * x[2] + a[4 * i + 3] * x[3];
}

template <class R>
__device__ __forceinline__ void mm(const R *a, const R *b, R *c)
{
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++)
			c[4 * i + j] = a[4 * i] * b[j] + a[4 * i + 1] * b[4 + j] + a[4 * i + 2] * b[8 + j] + a[4 * i + 3] * b[12 + j];
}

/* 4x4 inverse by Gauss-Jordan with partial pivoting; false if singular */
template <class R>
__device__ __forceinline__ bool inv4(const R *a, R *out)
{
	R m[4][8];
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++) {
			m[i][j] = a[4 * i + j];
			m[i][4 + j] = i == j ? R(1) : R(0);
		}
	for (int c = 0; c < 4; c++) {
		int p = c;
		R best = fabs(m[c][c]);
		for (int r = c + 1; r < 4; r++)
			if (fabs(m[r][c]) > best) { best = fabs(m[r][c]); p = r; }
		if (!(best > R(0))) return false;
		if (p != c)
			for (int j = 0; j < 8; j++) { const R t = m[p][j]; m[p][j] = m[c][j]; m[c][j] = t; }
		const R iv = R(1) / m[c][c];
		for (int j = 0; j < 8; j++) m[c][j] *= iv;
		for (int r = 0; r < 4; r++)
			if (r != c) {
				const R f = m[r][c];
				for (int j = 0; j < 8; j++) m[r][j] -= f * m[c][j];
			}
	}
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++) out[4 * i + j] = m[i][4 + j];
	return true;
}

__device__ __forceinline__ bool member_off(const int *active, int b) { return active && !active[b]; }

// ------------------------------ preconditioners -------------------------------

/* inverted diagonal blocks in colour order (Jacobi, SGS); SGS also copies the
 * matrix rows into colour order */
template <class R, class RA>
__global__ void __launch_bounds__(BS) k_diag_setup(int nelem, const RA *__restrict__ A, const int *__restrict__ pos_cell,
                                                   R *__restrict__ F, R *__restrict__ Dinv, int copy_rows,
                                                   int *err, const int *active)
{
	const int b = blockIdx.y;
	const int p = blockIdx.x * BS + threadIdx.x;
	if (p >= nelem || member_off(active, b)) return;
	const int i = pos_cell[p];
	const size_t N = nelem;
	const RA *Ab = A + (size_t)b * 5 * N * 16;
	R blk[16], inv[16];
	RA tmp[16];
	load_blk(Ab + (size_t)i * 16, tmp);
	for (int q = 0; q < 16; q++) blk[q] = R(tmp[q]);
	if (!inv4(blk, inv)) { atomicOr(err + b, 1); for (int q = 0; q < 16; q++) inv[q] = R(0); }
	store_blk(Dinv + ((size_t)b * N + p) * 16, inv);
	if (copy_rows) {
		R *Fb = F + (size_t)b * 5 * N * 16;
		for (int s = 0; s < 5; s++) {
			load_blk(Ab + ((size_t)s * N + i) * 16, tmp);
			for (int q = 0; q < 16; q++) blk[q] = R(tmp[q]);
			store_blk(Fb + ((size_t)s * N + p) * 16, blk);
		}
	}
}

/* block ILU(0) of the row at elimination position p (IKJ, no fill): every
 * lower neighbour's row must already be final */
template <class R, class RA>
__device__ __forceinline__ void ilu_row(int nelem, int p, int b, const RA *__restrict__ A,
                                        const int *__restrict__ pos_cell, const int4 *__restrict__ pnbr,
                                        const int4 *__restrict__ pnbrpos, R *__restrict__ F, R *__restrict__ Dinv,
                                        int *err)
{
	const size_t N = nelem;
	const int i = pos_cell[p];
	const RA *Ab = A + (size_t)b * 5 * N * 16;
	R *Fb = F + (size_t)b * 5 * N * 16;
	R *Db = Dinv + (size_t)b * N * 16;
	const int4 nb4 = pnbr[p], np4 = pnbrpos[p];
	const int nbc[4] = {nb4.x, nb4.y, nb4.z, nb4.w};
	const int nbp[4] = {np4.x, np4.y, np4.z, np4.w};
	R row[5][16];
	for (int s = 0; s < 5; s++) {
		RA tmp[16];
		load_blk(Ab + ((size_t)s * N + i) * 16, tmp);
		for (int q = 0; q < 16; q++) row[s][q] = R(tmp[q]);
	}
	// lower neighbours in ascending elimination position
	int ord[4], nl = 0;
	for (int j = 0; j < 4; j++)
		if (nbp[j] >= 0 && nbp[j] < p) ord[nl++] = j;
	for (int a = 1; a < nl; a++)
		for (int c = a; c > 0 && nbp[ord[c]] < nbp[ord[c - 1]]; c--) { const int t = ord[c]; ord[c] = ord[c - 1]; ord[c - 1] = t; }
	for (int a = 0; a < nl; a++) {
		const int jk = ord[a];
		const int pk = nbp[jk];
		R dk[16], L[16];
		load_blk(Db + (size_t)pk * 16, dk);
		mm(row[1 + jk], dk, L);
		for (int q = 0; q < 16; q++) row[1 + jk][q] = L[q];
		// row k's neighbours (cells) to locate U_kj
		const int4 kn4 = pnbr[pk];
		const int kn[4] = {kn4.x, kn4.y, kn4.z, kn4.w};
		// columns j of row i after k: the diagonal (j = i) and upper-position neighbours
		for (int s = 0; s < 5; s++) {
			int colcell, colpos;
			if (s == 0) { colcell = i; colpos = p; }
			else { colcell = nbc[s - 1]; colpos = nbp[s - 1]; }
			if (colpos < 0 || colpos <= pk) continue;
			int ks = -1;
			for (int t = 0; t < 4; t++)
				if (kn[t] == colcell) ks = t;
			if (ks < 0) continue;
			R ukj[16], prod[16];
			load_blk(Fb + ((size_t)(1 + ks) * N + pk) * 16, ukj);
			mm(L, ukj, prod);
			for (int q = 0; q < 16; q++) row[s][q] -= prod[q];
		}
	}
	R inv[16];
	if (!inv4(row[0], inv)) { atomicOr(err + b, 1); for (int q = 0; q < 16; q++) inv[q] = R(0); }
	store_blk(Db + (size_t)p * 16, inv);
	for (int s = 0; s < 5; s++) store_blk(Fb + ((size_t)s * N + p) * 16, row[s]);
}

/* rows of one point colour (no dependencies inside the launch) */
template <class R, class RA>
__global__ void __launch_bounds__(BS) k_ilu_colour(int nelem, int p0, int p1, const RA *__restrict__ A,
                                                   const int *__restrict__ pos_cell, const int4 *__restrict__ pnbr,
                                                   const int4 *__restrict__ pnbrpos, R *__restrict__ F,
                                                   R *__restrict__ Dinv, int *err, const int *active)
{
	const int b = blockIdx.y;
	const int p = p0 + blockIdx.x * BS + threadIdx.x;
	if (p >= p1 || member_off(active, b)) return;
	ilu_row<R, RA>(nelem, p, b, A, pos_cell, pnbr, pnbrpos, F, Dinv, err);
}

/* forward sweep of one colour: y_p = r_i - sum_{lower} L y  (ILU) or
 * Dinv (r_i - sum_{lower} A y) (SGS) */
template <class R>
__device__ __forceinline__ void fwd_row(int nelem, int p, int b, int sgs, const double *__restrict__ r,
                                        const int *__restrict__ pos_cell, const int4 *__restrict__ pnbrpos,
                                        const R *__restrict__ F, const R *__restrict__ Dinv, R *__restrict__ y)
{
	const size_t N = nelem;
	const int i = pos_cell[p];
	const double4 *rb = reinterpret_cast<const double4 *>(r + (size_t)b * N * 4);
	const double4 rv = rb[i];
	R s[4] = {R(rv.x), R(rv.y), R(rv.z), R(rv.w)};
	const int4 np4 = pnbrpos[p];
	const int nbp[4] = {np4.x, np4.y, np4.z, np4.w};
	const R *Fb = F + (size_t)b * 5 * N * 16;
	const R *yb = y + (size_t)b * N * 4;
	for (int j = 0; j < 4; j++) {
		if (nbp[j] < 0 || nbp[j] >= p) continue;
		R blk[16], t[4];
		load_blk(Fb + ((size_t)(1 + j) * N + p) * 16, blk);
		const R yy[4] = {yb[4 * (size_t)nbp[j]], yb[4 * (size_t)nbp[j] + 1], yb[4 * (size_t)nbp[j] + 2], yb[4 * (size_t)nbp[j] + 3]};
		mv(blk, yy, t);
		for (int q = 0; q < 4; q++) s[q] -= t[q];
	}
	R *yo = y + ((size_t)b * N + p) * 4;
	if (sgs) {
		R d[16], t[4];
		load_blk(Dinv + ((size_t)b * N + p) * 16, d);
		mv(d, s, t);
		for (int q = 0; q < 4; q++) yo[q] = t[q];
	} else {
		for (int q = 0; q < 4; q++) yo[q] = s[q];
	}
}

template <class R>
__global__ void __launch_bounds__(BS) k_fwd(int nelem, int p0, int p1, int sgs, const double *__restrict__ r,
                                            const int *__restrict__ pos_cell, const int4 *__restrict__ pnbrpos,
                                            const R *__restrict__ F, const R *__restrict__ Dinv, R *__restrict__ y,
                                            const int *active)
{
	const int b = blockIdx.y;
	const int p = p0 + blockIdx.x * BS + threadIdx.x;
	if (p >= p1 || member_off(active, b)) return;
	fwd_row<R>(nelem, p, b, sgs, r, pos_cell, pnbrpos, F, Dinv, y);
}

/* backward sweep of one colour: z_i = Dinv (y_p - sum_{upper} U z) (ILU) or
 * y_p - Dinv sum_{upper} A z (SGS) */
template <class R>
__device__ __forceinline__ void bwd_row(int nelem, int p, int b, int sgs, const int *__restrict__ pos_cell,
                                        const int4 *__restrict__ pnbr, const int4 *__restrict__ pnbrpos,
                                        const R *__restrict__ F, const R *__restrict__ Dinv, const R *__restrict__ y,
                                        double *__restrict__ z)
{
	const size_t N = nelem;
	const int i = pos_cell[p];
	const int4 nb4 = pnbr[p], np4 = pnbrpos[p];
	const int nbc[4] = {nb4.x, nb4.y, nb4.z, nb4.w};
	const int nbp[4] = {np4.x, np4.y, np4.z, np4.w};
	const R *Fb = F + (size_t)b * 5 * N * 16;
	double *zb = z + (size_t)b * N * 4;
	R t[4] = {R(0), R(0), R(0), R(0)};
	for (int j = 0; j < 4; j++) {
		if (nbp[j] < 0 || nbp[j] <= p) continue;
		R blk[16], u[4];
		load_blk(Fb + ((size_t)(1 + j) * N + p) * 16, blk);
		const double4 zz = reinterpret_cast<const double4 *>(zb)[nbc[j]];
		const R zv[4] = {R(zz.x), R(zz.y), R(zz.z), R(zz.w)};
		mv(blk, zv, u);
		for (int q = 0; q < 4; q++) t[q] += u[q];
	}
	const R *yp = y + ((size_t)b * N + p) * 4;
	R d[16], out[4];
	load_blk(Dinv + ((size_t)b * N + p) * 16, d);
	if (sgs) {
		R u[4];
		mv(d, t, u);
		for (int q = 0; q < 4; q++) out[q] = yp[q] - u[q];
	} else {
		const R v[4] = {yp[0] - t[0], yp[1] - t[1], yp[2] - t[2], yp[3] - t[3]};
		mv(d, v, out);
	}
	reinterpret_cast<double4 *>(zb)[i] = make_double4(double(out[0]), double(out[1]), double(out[2]), double(out[3]));
}

template <class R>
__global__ void __launch_bounds__(BS) k_bwd(int nelem, int p0, int p1, int sgs, const int *__restrict__ pos_cell,
                                            const int4 *__restrict__ pnbr, const int4 *__restrict__ pnbrpos,
                                            const R *__restrict__ F, const R *__restrict__ Dinv, const R *__restrict__ y,
                                            double *__restrict__ z, const int *active)
{
	const int b = blockIdx.y;
	const int p = p0 + blockIdx.x * BS + threadIdx.x;
	if (p >= p1 || member_off(active, b)) return;
	bwd_row<R>(nelem, p, b, sgs, pos_cell, pnbr, pnbrpos, F, Dinv, y, z);
}

/* ---- block-colour sweeps and factorisation: one CTA per part, the part staged in shared memory ----
 *
 * A part's cells occupy the contiguous elimination positions [p0, p1), sorted
 * by dependency level.  Every neighbour of a part cell outside the part lies
 * in another colour, so it is either finished by an earlier launch (it comes
 * before the whole part) or untouched until a later one.  Phase 1 (all PT
 * threads, one cell each) therefore does all the work that involves
 * neighbours outside the part -- in parallel, with the part's own blocks
 * copied to shared memory; phase 2 (all threads, four lanes per cell, one
 * block row each, a CTA barrier between levels) walks the part's dependency
 * levels reading shared memory only; phase 3 (all threads) writes the part
 * back.  The dependency chain of a part thus costs shared-memory latency and
 * one barrier per level. */
constexpr int PT = 128;  // threads per part CTA (32 cells x 4 block rows per pass of a level)

/* dynamic shared memory of the sweep kernels for parts of at most cap cells
 * with at most bcap in-part neighbour blocks on the sweep's side (lower for the
 * forward, upper for the backward sweep), with or without inverted diagonals:
 * only the blocks a part has are staged, so more parts fit on an SM */
template <class R>
size_t sweep_smem(int cap, int bcap, bool diag)
{
	return ((size_t)bcap * 16 + (diag ? (size_t)cap * 16 : 0) + (size_t)cap * 8) * sizeof(R) +
	       (size_t)cap * sizeof(int4);
}
/* Staging layout of a sweep launch.  A launch whose CTAs all fit on the machine
 * at four per SM (one condition: a colour's parts) is bound by each part's
 * dependency chain; it stages each cell's blocks at fixed slots (4 c + j), so a
 * level reads a block at an address that does not wait for the neighbour entry
 * (one condition's apply 0.126 ms; 0.152 ms with the slots of the compact
 * layout).  A larger launch (a batch) stages only the blocks a part has (slots
 * from pblk), so more CTAs fit on an SM and hide each other's latency (64
 * conditions: 3.40 -> 2.37 ms). */
bool sweep_compact(const Precond &P, int parts) { return (size_t)parts * P.batch > (size_t)4 * P.num_sms; }

/* a staged in-part neighbour: with compact staging its local index and block
 * slot in one int, else its local index (slot 4 c + j) (-1: none) */
__device__ __forceinline__ int pack_nb(int loc, int slot) { return loc | (slot << 16); }
template <bool COMPACT>
__device__ __forceinline__ int nb_loc(int v) { return COMPACT ? (v & 0xFFFF) : v; }
/* the staged block of cell c's neighbour j (entry v); with fixed slots its
 * address does not wait for the neighbour entry */
template <class R, bool COMPACT>
__device__ __forceinline__ const R *blk_at(const R *sF, int c, int j, int v)
{
	return COMPACT ? sF + (size_t)(v >> 16) * 16 : sF + ((size_t)c * 4 + j) * 16;
}
/* ... and of the factorisation */
template <class R>
size_t ilu_smem(int cap) { return (size_t)cap * (80 + 16) * sizeof(R); }

template <class R>
__device__ __forceinline__ R dot4(const R *a, const R *v) { return a[0] * v[0] + a[1] * v[1] + a[2] * v[2] + a[3] * v[3]; }

/* forward sweep of the parts of one colour: y_p = r_i - sum_{lower} L y (ILU)
 * or Dinv (r_i - sum_{lower} A y) (SGS) */
template <class R, bool COMPACT>
__global__ void __launch_bounds__(PT) k_fwd_parts(int nelem, int part0, int cap, int bcap,
                                                  const int *__restrict__ part_ptr,
                                                  const int *__restrict__ lev_ptr, const int *__restrict__ lev_pos,
                                                  int sgs, const double *__restrict__ r, const int *__restrict__ pos_cell,
                                                  const int4 *__restrict__ pnbrpos, const int2 *__restrict__ pblk,
                                                  const R *__restrict__ F, const R *__restrict__ Dinv,
                                                  R *__restrict__ y, const int *active)
{
	extern __shared__ __align__(16) unsigned char smem[];
	R *sF = reinterpret_cast<R *>(smem);            // [bcap][16]  in-part lower blocks (bcap = 4 cap unless compact)
	R *sD = sF + (size_t)bcap * 16;                  // [cap][16]   Dinv (SGS only)
	R *sv = sD + (sgs ? (size_t)cap * 16 : 0);       // [cap][4]    y of the part
	R *st = sv + (size_t)cap * 4;                    // [cap][4]    right-hand side
	int4 *snb = reinterpret_cast<int4 *>(st + (size_t)cap * 4);  // in-part lower neighbours (pack_nb), -1 none
	const int b = blockIdx.y;
	if (member_off(active, b)) return;
	const int part = part0 + blockIdx.x;
	const int p0 = part_ptr[part], p1 = part_ptr[part + 1], n = p1 - p0;
	const size_t N = nelem;
	const R *Fb = F + (size_t)b * 5 * N * 16;
	R *yb = y + (size_t)b * N * 4;
	const double4 *rb = reinterpret_cast<const double4 *>(r + (size_t)b * N * 4);
	for (int c = threadIdx.x; c < n; c += PT) {
		const int p = p0 + c;
		const double4 rv = rb[pos_cell[p]];
		R s[4] = {R(rv.x), R(rv.y), R(rv.z), R(rv.w)};
		const int4 np4 = pnbrpos[p];
		const int nbp[4] = {np4.x, np4.y, np4.z, np4.w};
		int loc[4], slot = COMPACT ? pblk[p].x : 0;
		for (int j = 0; j < 4; j++) {
			loc[j] = -1;
			const int q = nbp[j];
			if (q < 0 || q >= p) continue;
			R blk[16];
			load_blk(Fb + ((size_t)(1 + j) * N + p) * 16, blk);
			if (q >= p0) {
				if (COMPACT) {
					loc[j] = pack_nb(q - p0, slot);
					store_blk(sF + (size_t)slot * 16, blk);
					slot++;
				} else {
					loc[j] = q - p0;
					store_blk(sF + ((size_t)c * 4 + j) * 16, blk);
				}
			} else {
				const R yy[4] = {yb[4 * (size_t)q], yb[4 * (size_t)q + 1], yb[4 * (size_t)q + 2], yb[4 * (size_t)q + 3]};
				R t[4];
				mv(blk, yy, t);
				for (int k = 0; k < 4; k++) s[k] -= t[k];
			}
		}
		for (int k = 0; k < 4; k++) st[4 * c + k] = s[k];
		snb[c] = make_int4(loc[0], loc[1], loc[2], loc[3]);
		if (sgs) {
			R d[16];
			load_blk(Dinv + ((size_t)b * N + p) * 16, d);
			store_blk(sD + (size_t)c * 16, d);
		}
	}
	__syncthreads();
	{
		const int l0 = lev_ptr[part], l1 = lev_ptr[part + 1];
		const int g = threadIdx.x >> 2, row = threadIdx.x & 3;
		for (int l = l0; l < l1; l++) {
			const int ls = lev_pos[l] - p0, le = (l + 1 < l1 ? lev_pos[l + 1] : p1) - p0;
			for (int c0 = ls; c0 < le; c0 += PT / 4) {
				const int c = c0 + g;
				const bool on = c < le;
				R acc = R(0);
				if (on) {
					acc = st[4 * c + row];
					const int4 nb = snb[c];
					const int l4[4] = {nb.x, nb.y, nb.z, nb.w};
					for (int j = 0; j < 4; j++)
						if (l4[j] >= 0) acc -= dot4(blk_at<R, COMPACT>(sF, c, j, l4[j]) + 4 * row, sv + 4 * nb_loc<COMPACT>(l4[j]));
				}
				if (sgs) {
					if (on) st[4 * c + row] = acc;
					__syncwarp();
					if (on) acc = dot4(sD + (size_t)c * 16 + 4 * row, st + 4 * c);
				}
				if (on) sv[4 * c + row] = acc;
			}
			__syncthreads();  // the level's values are read by the next level
		}
	}
	for (int e = threadIdx.x; e < 4 * n; e += PT) yb[(size_t)p0 * 4 + e] = sv[e];
}

/* backward sweep of the parts of one colour (levels in reverse):
 * z_i = Dinv (y_p - sum_{upper} U z) (ILU) or y_p - Dinv sum_{upper} A z (SGS) */
template <class R, bool COMPACT>
__global__ void __launch_bounds__(PT) k_bwd_parts(int nelem, int part0, int cap, int bcap,
                                                  const int *__restrict__ part_ptr,
                                                  const int *__restrict__ lev_ptr, const int *__restrict__ lev_pos,
                                                  int sgs, const int *__restrict__ pos_cell, const int4 *__restrict__ pnbr,
                                                  const int4 *__restrict__ pnbrpos, const int2 *__restrict__ pblk,
                                                  const R *__restrict__ F, const R *__restrict__ Dinv,
                                                  const R *__restrict__ y, double *__restrict__ z, const int *active)
{
	extern __shared__ __align__(16) unsigned char smem[];
	R *sF = reinterpret_cast<R *>(smem);  // [bcap][16]   in-part upper blocks
	R *sD = sF + (size_t)bcap * 16;        // [cap][16]    Dinv
	R *sv = sD + (size_t)cap * 16;         // [cap][4]     z of the part
	R *st = sv + (size_t)cap * 4;          // [cap][4]     right-hand side (ILU) / outside sum (SGS)
	int4 *snb = reinterpret_cast<int4 *>(st + (size_t)cap * 4);
	const int b = blockIdx.y;
	if (member_off(active, b)) return;
	const int part = part0 + blockIdx.x;
	const int p0 = part_ptr[part], p1 = part_ptr[part + 1], n = p1 - p0;
	const size_t N = nelem;
	const R *Fb = F + (size_t)b * 5 * N * 16;
	const R *yb = y + (size_t)b * N * 4;
	double *zb = z + (size_t)b * N * 4;
	for (int c = threadIdx.x; c < n; c += PT) {
		const int p = p0 + c;
		const int4 nb4 = pnbr[p], np4 = pnbrpos[p];
		const int nbc[4] = {nb4.x, nb4.y, nb4.z, nb4.w};
		const int nbp[4] = {np4.x, np4.y, np4.z, np4.w};
		R s[4] = {R(0), R(0), R(0), R(0)};
		int loc[4], slot = COMPACT ? pblk[p].y : 0;
		for (int j = 0; j < 4; j++) {
			loc[j] = -1;
			const int q = nbp[j];
			if (q < 0 || q <= p) continue;
			R blk[16];
			load_blk(Fb + ((size_t)(1 + j) * N + p) * 16, blk);
			if (q < p1) {
				if (COMPACT) {
					loc[j] = pack_nb(q - p0, slot);
					store_blk(sF + (size_t)slot * 16, blk);
					slot++;
				} else {
					loc[j] = q - p0;
					store_blk(sF + ((size_t)c * 4 + j) * 16, blk);
				}
			} else {
				const double4 zz = reinterpret_cast<const double4 *>(zb)[nbc[j]];
				const R zv[4] = {R(zz.x), R(zz.y), R(zz.z), R(zz.w)};
				R t[4];
				mv(blk, zv, t);
				for (int k = 0; k < 4; k++) s[k] += t[k];
			}
		}
		const R *yp = yb + ((size_t)p) * 4;
		for (int k = 0; k < 4; k++) st[4 * c + k] = sgs ? s[k] : yp[k] - s[k];
		if (sgs)
			for (int k = 0; k < 4; k++) sv[4 * c + k] = yp[k];  // y kept beside the sum until the cell's level
		snb[c] = make_int4(loc[0], loc[1], loc[2], loc[3]);
		R d[16];
		load_blk(Dinv + ((size_t)b * N + p) * 16, d);
		store_blk(sD + (size_t)c * 16, d);
	}
	__syncthreads();
	{
		const int l0 = lev_ptr[part], l1 = lev_ptr[part + 1];
		const int g = threadIdx.x >> 2, row = threadIdx.x & 3;
		for (int l = l1 - 1; l >= l0; l--) {
			const int ls = lev_pos[l] - p0, le = (l + 1 < l1 ? lev_pos[l + 1] : p1) - p0;
			for (int c0 = ls; c0 < le; c0 += PT / 4) {
				const int c = c0 + g;
				const bool on = c < le;
				if (on) {
					const int4 nb = snb[c];
					const int l4[4] = {nb.x, nb.y, nb.z, nb.w};
					R acc = R(0);
					for (int j = 0; j < 4; j++)
						if (l4[j] >= 0) acc += dot4(blk_at<R, COMPACT>(sF, c, j, l4[j]) + 4 * row, sv + 4 * nb_loc<COMPACT>(l4[j]));
					// ILU: t = (y - outside) - inside;  SGS: t = outside + inside
					st[4 * c + row] = sgs ? st[4 * c + row] + acc : st[4 * c + row] - acc;
				}
				__syncwarp();
				if (on) {
					const R dz = dot4(sD + (size_t)c * 16 + 4 * row, st + 4 * c);
					sv[4 * c + row] = sgs ? sv[4 * c + row] - dz : dz;
				}
			}
			__syncthreads();  // the level's values are read by the next level
		}
	}
	for (int c = threadIdx.x; c < n; c += PT) {
		const R *v = sv + 4 * c;
		reinterpret_cast<double4 *>(zb)[pos_cell[p0 + c]] = make_double4(double(v[0]), double(v[1]), double(v[2]), double(v[3]));
	}
}

/* row i -= its elimination by lower neighbour k (IKJ, no fill): L_ik = A_ik Dinv_k
 * replaces A_ik, and every column j of row i after k (diagonal and neighbours
 * at positions > p_k) that row k also holds loses L_ik U_kj.  rw: row i's five
 * blocks (slot 0 diagonal, 1+j neighbour j); dk, uk: row k's inverted
 * diagonal and its blocks (slot 1+t for k's neighbour t); kn: k's neighbours. */
template <class R>
__device__ __forceinline__ void ilu_eliminate_row(R *rw, int jk, int pk, int icell, const int *nbc, const int *nbp,
                                                  int p, const R *dk, const R *uk, size_t ustride, const int *kn)
{
	R L[16];
	mm(rw + (1 + jk) * 16, dk, L);
	for (int q = 0; q < 16; q++) rw[(1 + jk) * 16 + q] = L[q];
	for (int s = 0; s < 5; s++) {
		const int colcell = s == 0 ? icell : nbc[s - 1];
		const int colpos = s == 0 ? p : nbp[s - 1];
		if (colpos < 0 || colpos <= pk) continue;
		int ks = -1;
		for (int t = 0; t < 4; t++)
			if (kn[t] == colcell) ks = t;
		if (ks < 0) continue;
		R ukj[16], prod[16];
		load_blk(uk + (size_t)(1 + ks) * ustride, ukj);
		mm(L, ukj, prod);
		for (int q = 0; q < 16; q++) rw[s * 16 + q] -= prod[q];
	}
}

/* block ILU(0) of the parts of one colour */
template <class R, class RA>
__global__ void __launch_bounds__(PT) k_ilu_parts(int nelem, int part0, int cap, const int *__restrict__ part_ptr,
                                                  const int *__restrict__ lev_ptr, const int *__restrict__ lev_pos,
                                                  const RA *__restrict__ A, const int *__restrict__ pos_cell,
                                                  const int4 *__restrict__ pnbr, const int4 *__restrict__ pnbrpos,
                                                  R *__restrict__ F, R *__restrict__ Dinv, int *err, const int *active)
{
	extern __shared__ __align__(16) unsigned char smem[];
	R *sRow = reinterpret_cast<R *>(smem);  // [cap][5][16]
	R *sD = sRow + (size_t)cap * 80;         // [cap][16] inverted factored diagonal
	const int b = blockIdx.y;
	if (member_off(active, b)) return;
	const int part = part0 + blockIdx.x;
	const int p0 = part_ptr[part], p1 = part_ptr[part + 1], n = p1 - p0;
	const size_t N = nelem;
	const RA *Ab = A + (size_t)b * 5 * N * 16;
	R *Fb = F + (size_t)b * 5 * N * 16;
	R *Db = Dinv + (size_t)b * N * 16;
	for (int e = threadIdx.x; e < n * 5; e += PT) {
		const int s = e / n, c = e - s * n;
		RA tmp[16];
		R blk[16];
		load_blk(Ab + ((size_t)s * N + pos_cell[p0 + c]) * 16, tmp);
		for (int q = 0; q < 16; q++) blk[q] = R(tmp[q]);
		store_blk(sRow + ((size_t)c * 5 + s) * 16, blk);
	}
	__syncthreads();
	// lower neighbours outside the part are final and precede every part cell
	for (int c = threadIdx.x; c < n; c += PT) {
		const int p = p0 + c;
		const int4 nb4 = pnbr[p], np4 = pnbrpos[p];
		const int nbc[4] = {nb4.x, nb4.y, nb4.z, nb4.w};
		const int nbp[4] = {np4.x, np4.y, np4.z, np4.w};
		int ord[4], nl = 0;
		for (int j = 0; j < 4; j++)
			if (nbp[j] >= 0 && nbp[j] < p0) ord[nl++] = j;
		for (int a = 1; a < nl; a++)
			for (int d = a; d > 0 && nbp[ord[d]] < nbp[ord[d - 1]]; d--) { const int t = ord[d]; ord[d] = ord[d - 1]; ord[d - 1] = t; }
		for (int a = 0; a < nl; a++) {
			const int jk = ord[a], pk = nbp[jk];
			R dk[16];
			load_blk(Db + (size_t)pk * 16, dk);
			const int4 kn4 = pnbr[pk];
			const int kn[4] = {kn4.x, kn4.y, kn4.z, kn4.w};
			ilu_eliminate_row(sRow + (size_t)c * 80, jk, pk, pos_cell[p], nbc, nbp, p, dk, Fb + (size_t)pk * 16,
			                  N * 16, kn);
		}
	}
	__syncthreads();
	{
		const int l0 = lev_ptr[part], l1 = lev_ptr[part + 1];
		const int g = threadIdx.x >> 2, row = threadIdx.x & 3;
		for (int l = l0; l < l1; l++) {
			const int ls = lev_pos[l] - p0, le = (l + 1 < l1 ? lev_pos[l + 1] : p1) - p0;
			for (int c0 = ls; c0 < le; c0 += PT / 4) {
				const int c = c0 + g;
				const bool on = c < le;
				if (on) {
					const int p = p0 + c;
					const int icell = pos_cell[p];
					R *rw = sRow + (size_t)c * 80;
					const int4 nb4 = pnbr[p], np4 = pnbrpos[p];
					const int nbc[4] = {nb4.x, nb4.y, nb4.z, nb4.w};
					const int nbp[4] = {np4.x, np4.y, np4.z, np4.w};
					int ord[4], nl = 0;
					for (int j = 0; j < 4; j++)
						if (nbp[j] >= p0 && nbp[j] < p) ord[nl++] = j;
					for (int a = 1; a < nl; a++)
						for (int d = a; d > 0 && nbp[ord[d]] < nbp[ord[d - 1]]; d--) { const int t = ord[d]; ord[d] = ord[d - 1]; ord[d - 1] = t; }
					for (int a = 0; a < nl; a++) {
						const int jk = ord[a], pk = nbp[jk];
						const R *dk = sD + (size_t)(pk - p0) * 16;
						// L_ik = A_ik Dinv_k : lane `row` computes block row `row`
						R Lr[4];
						R *aik = rw + (1 + jk) * 16 + 4 * row;
						for (int m = 0; m < 4; m++) Lr[m] = aik[0] * dk[m] + aik[1] * dk[4 + m] + aik[2] * dk[8 + m] + aik[3] * dk[12 + m];
						for (int m = 0; m < 4; m++) aik[m] = Lr[m];
						const int4 kn4 = pnbr[pk];
						const int kn[4] = {kn4.x, kn4.y, kn4.z, kn4.w};
						for (int s = 0; s < 5; s++) {
							const int colcell = s == 0 ? icell : nbc[s - 1];
							const int colpos = s == 0 ? p : nbp[s - 1];
							if (colpos < 0 || colpos <= pk) continue;
							int ks = -1;
							for (int t = 0; t < 4; t++)
								if (kn[t] == colcell) ks = t;
							if (ks < 0) continue;
							const R *ukj = sRow + ((size_t)(pk - p0) * 5 + 1 + ks) * 16;
							R *ais = rw + s * 16 + 4 * row;
							for (int m = 0; m < 4; m++) ais[m] -= Lr[0] * ukj[m] + Lr[1] * ukj[4 + m] + Lr[2] * ukj[8 + m] + Lr[3] * ukj[12 + m];
						}
					}
				}
				__syncwarp();
				if (on) {
					R dblk[16], inv[16];
					for (int q = 0; q < 16; q++) dblk[q] = sRow[(size_t)c * 80 + q];
					if (!inv4(dblk, inv)) {
						if (row == 0) atomicOr(err + b, 1);
						for (int q = 0; q < 16; q++) inv[q] = R(0);
					}
					for (int m = 0; m < 4; m++) sD[(size_t)c * 16 + 4 * row + m] = inv[4 * row + m];
				}
				__syncwarp();
			}
			__syncthreads();  // the level's rows and inverted diagonals are read by later levels
		}
	}
	__syncthreads();
	for (int e = threadIdx.x; e < n * 5; e += PT) {
		const int s = e / n, c = e - s * n;
		R blk[16];
		for (int q = 0; q < 16; q++) blk[q] = sRow[((size_t)c * 5 + s) * 16 + q];
		store_blk(Fb + ((size_t)s * N + p0 + c) * 16, blk);
	}
	for (int e = threadIdx.x; e < n; e += PT) {
		R blk[16];
		for (int q = 0; q < 16; q++) blk[q] = sD[(size_t)e * 16 + q];
		store_blk(Db + ((size_t)p0 + e) * 16, blk);
	}
}

template <class R>
__global__ void __launch_bounds__(BS) k_jacobi_apply(int nelem, const double *__restrict__ r, const int *__restrict__ cell_pos,
                                                     const R *__restrict__ Dinv, double *__restrict__ z, const int *active)
{
	const int b = blockIdx.y;
	const int i = blockIdx.x * BS + threadIdx.x;
	if (i >= nelem || member_off(active, b)) return;
	const size_t N = nelem;
	const double4 rv = reinterpret_cast<const double4 *>(r + (size_t)b * N * 4)[i];
	const R s[4] = {R(rv.x), R(rv.y), R(rv.z), R(rv.w)};
	R d[16], o[4];
	load_blk(Dinv + ((size_t)b * N + cell_pos[i]) * 16, d);
	mv(d, s, o);
	reinterpret_cast<double4 *>(z + (size_t)b * N * 4)[i] = make_double4(double(o[0]), double(o[1]), double(o[2]), double(o[3]));
}

__global__ void k_copy(size_t n, const double *__restrict__ a, double *__restrict__ b, const int *active, size_t per)
{
	const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n) return;
	if (active && !active[t / per]) return;
	b[t] = a[t];
}

// ---------------------------------- SpMV ---------------------------------------

template <class R>
__global__ void __launch_bounds__(BS) k_spmv(int nelem, const R *__restrict__ A, const int4 *__restrict__ cnbr,
                                             const double *__restrict__ x, double *__restrict__ y, const int *active)
{
	const int b = blockIdx.y;
	const int i = blockIdx.x * BS + threadIdx.x;
	if (i >= nelem || member_off(active, b)) return;
	const size_t N = nelem;
	const R *Ab = A + (size_t)b * 5 * N * 16;
	const double4 *xb = reinterpret_cast<const double4 *>(x + (size_t)b * N * 4);
	const int4 c4 = cnbr[i];
	const int cols[5] = {i, c4.x, c4.y, c4.z, c4.w};
	R acc[4] = {R(0), R(0), R(0), R(0)};
	for (int s = 0; s < 5; s++) {
		if (cols[s] < 0) continue;
		R blk[16], t[4];
		load_blk(Ab + ((size_t)s * N + i) * 16, blk);
		const double4 xv = xb[cols[s]];
		const R xx[4] = {R(xv.x), R(xv.y), R(xv.z), R(xv.w)};
		mv(blk, xx, t);
		for (int q = 0; q < 4; q++) acc[q] += t[q];
	}
	reinterpret_cast<double4 *>(y + (size_t)b * N * 4)[i] = make_double4(double(acc[0]), double(acc[1]), double(acc[2]), double(acc[3]));
}

// ------------------------------ Krylov kernels ---------------------------------

/* partial dot products: part[b][slot][blk] = sum over this block's share of a.b
 * (a = V_i when vbase != NULL: vector index i = blockIdx.z) */
__global__ void __launch_bounds__(RBS) k_dot_partial(int n, int nblk, const double *__restrict__ a, size_t astride,
                                                     size_t aistride, const double *__restrict__ w, size_t wstride,
                                                     double *__restrict__ part, int slot0, int pstride,
                                                     const int *active, const int *ilim)
{
	const int b = blockIdx.y, i = blockIdx.z;
	if (member_off(active, b) || (ilim && i > *ilim)) return;
	const double *av = a + (size_t)b * astride + (size_t)i * aistride;
	const double *wv = w + (size_t)b * wstride;
	double s = 0;
	for (int e = blockIdx.x * RBS + threadIdx.x; e < n; e += nblk * RBS) s += av[e] * wv[e];
	__shared__ double sh[RBS];
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int o = RBS / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0) part[((size_t)b * pstride + slot0 + i) * nblk + blockIdx.x] = sh[0];
}

__device__ __forceinline__ double block_sum(const double *p, int nblk)
{
	// deterministic fixed-order sum by one warp
	double s = 0;
	for (int k = threadIdx.x; k < nblk; k += 32) s += p[k];
	for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
	return __shfl_sync(0xffffffffu, s, 0);
}

/* init: bnorm, target, g, flags; x := 0 */
__global__ void k_gm_init(Krylov K, int nblk, double rtol, const int *member_active)
{
	const int b = blockIdx.x;
	const double bn = sqrt(block_sum(K.part + (size_t)b * (K.restart + 2) * nblk, nblk));
	if (threadIdx.x == 0) {
		double *sc = K.scal + 8 * b;
		sc[0] = bn;
		sc[1] = rtol * bn;
		sc[3] = bn > 0 ? 1.0 / bn : 0.0;
		const bool on = (!member_active || member_active[b]) && bn > 0;
		K.active[b] = on ? 1 : 0;
		K.iters[b] = 0;
		K.kdone[b] = 0;
		if (b == 0) *K.jcur = 0;
		double *g = K.g + (size_t)b * (K.restart + 1);
		for (int k = 0; k <= K.restart; k++) g[k] = 0;
		g[0] = bn;
	}
}

/* v0 = vcur = b / ||b|| for active members; x := 0 */
__global__ void k_first_basis(Krylov K, const double *__restrict__ bvec, double *__restrict__ x)
{
	const int b = blockIdx.y;
	const size_t n = K.n;
	const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= n) return;
	if (x) x[(size_t)b * n + e] = 0.0;
	if (!K.active[b]) return;
	const double v = K.scal[8 * b + 3] * bvec[(size_t)b * n + e];
	K.V[(size_t)b * n + e] = v;
	K.vcur[(size_t)b * n + e] = v;
}

/* v_{j+1} = vcur = w / h_{j+1,j} for members still iterating */
__global__ void k_next_basis(Krylov K)
{
	const int b = blockIdx.y;
	const size_t n = K.n;
	const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= n || !K.active[b]) return;
	const int j = *K.jcur;
	const double v = K.scal[8 * b + 2] * K.w[(size_t)b * n + e];
	K.V[((size_t)(j + 1) * K.batch + b) * n + e] = v;
	K.vcur[(size_t)b * n + e] = v;
}

/* end of an Arnoldi step: j += 1; with a graph loop, continue while any
 * member iterates and j < maxit */
__global__ void k_loop_ctrl(Krylov K, int maxit, cudaGraphConditionalHandle h, int set_cond)
{
	if (threadIdx.x != 0) return;
	const int j = *K.jcur + 1;
	*K.jcur = j;
	*K.loops += 1;
	bool any = false;
	for (int b = 0; b < K.batch; b++) any = any || K.active[b];
	if (set_cond) cudaGraphSetConditional(h, (any && j < maxit) ? 1u : 0u);
}

/* h_i (i <= j) from partials into H[:, j] */
__global__ void k_reduce_h(Krylov K, int nblk)
{
	const int b = blockIdx.x, i = blockIdx.y;  // one warp per (member, basis vector)
	if (!K.active[b]) return;
	const int j = *K.jcur;
	if (i > j) return;
	const double h = block_sum(K.part + ((size_t)b * (K.restart + 2) + i) * nblk, nblk);
	if (threadIdx.x == 0) K.H[(size_t)b * (K.restart + 1) * K.restart + (size_t)i * K.restart + j] = h;
}

/* w -= sum_{i<=j} h_i v_i; partial ||w||^2 into part slot restart+1; Z_j = zcur */
__global__ void __launch_bounds__(RBS) k_cgs_update(Krylov K, int nblk)
{
	const int b = blockIdx.y;
	if (!K.active[b]) return;
	const int j = *K.jcur;
	const int n = K.n;
	const size_t vstep = (size_t)K.batch * n;  // V layout [vector][member][n]
	const double *Vb = K.V + (size_t)b * n;
	const double *Hb = K.H + (size_t)b * (K.restart + 1) * K.restart;
	double *wb = K.w + (size_t)b * n;
	const double *zc = K.zcur + (size_t)b * n;
	double *zj = K.Z + (size_t)j * vstep + (size_t)b * n;
	double s = 0;
	for (int e = blockIdx.x * RBS + threadIdx.x; e < n; e += nblk * RBS) {
		zj[e] = zc[e];
		double x = wb[e];
		for (int i = 0; i <= j; i++) x -= Hb[(size_t)i * K.restart + j] * Vb[(size_t)i * vstep + e];
		wb[e] = x;
		s += x * x;
	}
	__shared__ double sh[RBS];
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int o = RBS / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
		__syncthreads();
	}
	if (threadIdx.x == 0) K.part[((size_t)b * (K.restart + 2) + K.restart + 1) * nblk + blockIdx.x] = sh[0];
}

/* Givens rotation of column j, residual estimate, convergence */
__global__ void k_givens(Krylov K, int nblk, int maxit)
{
	const int b = blockIdx.x;
	if (!K.active[b]) return;
	const int j = *K.jcur;
	const double hn = sqrt(block_sum(K.part + ((size_t)b * (K.restart + 2) + K.restart + 1) * nblk, nblk));
	const int m = K.restart;
	double *H = K.H + (size_t)b * (m + 1) * m;
	double *cs = K.cs + (size_t)b * (m + 1), *sn = K.sn + (size_t)b * (m + 1), *g = K.g + (size_t)b * (m + 1);
	double *sc = K.scal + 8 * b;
	// column j and the previous rotations staged in shared memory by the warp, so the
	// serial rotation chain below waits on shared memory, not on global loads
	extern __shared__ double gsh[];  // [3][m + 1]: column j, cs, sn
	double *hc = gsh, *cc = gsh + (m + 1), *ss = gsh + 2 * (m + 1);
	for (int i = threadIdx.x; i <= j; i += 32) {
		hc[i] = H[(size_t)i * m + j];
		cc[i] = cs[i];
		ss[i] = sn[i];
	}
	__syncwarp();
	if (threadIdx.x != 0) return;
	hc[j + 1] = hn;
	for (int i = 0; i < j; i++) {
		const double a = hc[i], c = hc[i + 1];
		hc[i] = cc[i] * a + ss[i] * c;
		hc[i + 1] = -ss[i] * a + cc[i] * c;
	}
	for (int i = 0; i < j; i++) H[(size_t)i * m + j] = hc[i];
	const double a = hc[j], c = hc[j + 1];
	const double den = sqrt(a * a + c * c);
	cs[j] = a / den;
	sn[j] = c / den;
	H[(size_t)j * m + j] = den;
	H[(size_t)(j + 1) * m + j] = 0.0;
	g[j + 1] = -sn[j] * g[j];
	g[j] = cs[j] * g[j];
	K.iters[b] = j + 1;
	K.kdone[b] = j + 1;
	sc[2] = hn > 0 ? 1.0 / hn : 0.0;
	sc[4] = fabs(g[j + 1]);
	if (fabs(g[j + 1]) <= sc[1] || hn == 0.0 || j + 1 >= maxit) K.active[b] = 0;
}

/* y = H^{-1} g (upper triangular kdone x kdone), stored in g */
__global__ void k_backsolve(Krylov K, const int *member_active)
{
	const int b = blockIdx.x * blockDim.x + threadIdx.x;
	if (b >= K.batch) return;
	if (member_active && !member_active[b]) return;
	const int m = K.restart, k = K.kdone[b];
	const double *H = K.H + (size_t)b * (m + 1) * m;
	double *g = K.g + (size_t)b * (m + 1);
	for (int i = k - 1; i >= 0; i--) {
		double s = g[i];
		for (int jj = i + 1; jj < k; jj++) s -= H[(size_t)i * m + jj] * g[jj];
		g[i] = s / H[(size_t)i * m + i];
	}
}

/* x += sum_i y_i z_i */
__global__ void k_update_x(Krylov K, double *__restrict__ x, const int *member_active)
{
	const int b = blockIdx.y;
	if (member_active && !member_active[b]) return;
	const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= (size_t)K.n) return;
	const int k = K.kdone[b];
	const double *g = K.g + (size_t)b * (K.restart + 1);
	const size_t zstep = (size_t)K.batch * K.n;  // Z layout [vector][member][n]
	const double *Zb = K.Z + (size_t)b * K.n;
	double s = x[(size_t)b * K.n + e];
	for (int i = 0; i < k; i++) s += g[i] * Zb[(size_t)i * zstep + e];
	x[(size_t)b * K.n + e] = s;
}

template <class R>
cudaError_t precond_setup_t(Precond &P, int *err, const int *active, cudaStream_t s, int *nk)
{
	const int N = P.nelem, B = P.batch;
	R *F = (R *)P.F, *D = (R *)P.Dinv;
	auto go = [&](const auto *A) {
		if (P.type == PC_JACOBI || P.type == PC_SGS) {
			k_diag_setup<R><<<dim3((N + BS - 1) / BS, B), BS, 0, s>>>(N, A, P.pos_cell, F, D, P.type == PC_SGS, err, active);
			(*nk)++;
		} else if (P.type == PC_ILU0 && P.ordering == 1) {
			for (int c = 0; c < P.ncolors; c++) {
				const int q0 = P.cpart[c], q1 = P.cpart[c + 1];
				if (q1 <= q0) continue;
				k_ilu_parts<R><<<dim3(q1 - q0, B), PT, ilu_smem<R>(P.part_cap), s>>>(
				    N, q0, P.part_cap, P.part_ptr, P.lev_ptr, P.lev_pos, A, P.pos_cell, P.pnbr, P.pnbrpos, F, D, err, active);
				(*nk)++;
			}
		} else if (P.type == PC_ILU0) {
			for (int c = 0; c < P.ncolors; c++) {
				const int p0 = P.cptr[c], p1 = P.cptr[c + 1];
				if (p1 <= p0) continue;
				k_ilu_colour<R><<<dim3((p1 - p0 + BS - 1) / BS, B), BS, 0, s>>>(N, p0, p1, A, P.pos_cell, P.pnbr,
				                                                              P.pnbrpos, F, D, err, active);
				(*nk)++;
			}
		}
	};
	if (P.A->prec == 4) go((const float *)P.A->val);
	else go((const double *)P.A->val);
	return cudaGetLastError();
}

template <class R>
cudaError_t precond_apply_t(const Precond &P, const double *r, double *z, const int *active, cudaStream_t s, int *nk)
{
	const int N = P.nelem, B = P.batch;
	const R *F = (const R *)P.F, *D = (const R *)P.Dinv;
	R *y = (R *)P.y;
	if (P.type == PC_NONE) {
		const size_t n = (size_t)B * N * 4;
		k_copy<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, r, z, active, (size_t)N * 4);
		(*nk)++;
	} else if (P.type == PC_JACOBI) {
		k_jacobi_apply<R><<<dim3((N + BS - 1) / BS, B), BS, 0, s>>>(N, r, P.cell_pos, D, z, active);
		(*nk)++;
	} else if (P.ordering == 1) {
		const int sgs = P.type == PC_SGS;
		for (int c = 0; c < P.ncolors; c++) {
			const int q0 = P.cpart[c], q1 = P.cpart[c + 1];
			if (q1 <= q0) continue;
			const bool cm = sweep_compact(P, q1 - q0);
			const int bcap = cm ? P.blk_cap_lo : 4 * P.part_cap;
			auto *kern = cm ? k_fwd_parts<R, true> : k_fwd_parts<R, false>;
			// (fixed slots: the staging size of the inverted diagonals too, as one part per
			// launch was measured with)
			kern<<<dim3(q1 - q0, B), PT, sweep_smem<R>(P.part_cap, bcap, cm ? (bool)sgs : true), s>>>(
			    N, q0, P.part_cap, bcap, P.part_ptr, P.lev_ptr, P.lev_pos, sgs, r, P.pos_cell, P.pnbrpos, P.pblk,
			    F, D, y, active);
			(*nk)++;
		}
		for (int c = P.ncolors - 1; c >= 0; c--) {
			const int q0 = P.cpart[c], q1 = P.cpart[c + 1];
			if (q1 <= q0) continue;
			const bool cm = sweep_compact(P, q1 - q0);
			const int bcap = cm ? P.blk_cap_up : 4 * P.part_cap;
			auto *kern = cm ? k_bwd_parts<R, true> : k_bwd_parts<R, false>;
			kern<<<dim3(q1 - q0, B), PT, sweep_smem<R>(P.part_cap, bcap, true), s>>>(
			    N, q0, P.part_cap, bcap, P.part_ptr, P.lev_ptr, P.lev_pos, sgs, P.pos_cell, P.pnbr, P.pnbrpos,
			    P.pblk, F, D, y, z, active);
			(*nk)++;
		}
	} else {
		const int sgs = P.type == PC_SGS;
		for (int c = 0; c < P.ncolors; c++) {
			const int p0 = P.cptr[c], p1 = P.cptr[c + 1];
			if (p1 <= p0) continue;
			k_fwd<R><<<dim3((p1 - p0 + BS - 1) / BS, B), BS, 0, s>>>(N, p0, p1, sgs, r, P.pos_cell, P.pnbrpos, F, D, y, active);
			(*nk)++;
		}
		for (int c = P.ncolors - 1; c >= 0; c--) {
			const int p0 = P.cptr[c], p1 = P.cptr[c + 1];
			if (p1 <= p0) continue;
			k_bwd<R><<<dim3((p1 - p0 + BS - 1) / BS, B), BS, 0, s>>>(N, p0, p1, sgs, P.pos_cell, P.pnbr, P.pnbrpos, F, D, y, z, active);
			(*nk)++;
		}
	}
	return cudaGetLastError();
}

}  // namespace

cudaError_t precond_alloc(Precond &P, fv_mesh_impl *m, int batch, int type, int prec, int ordering, int part_size)
{
	P.type = type;
	const int colouring = ordering == 2 ? 1 : 0;
	P.ordering = ordering ? 1 : 0;
	P.part_size = part_size;
	P.prec = prec;
	P.batch = batch;
	const HostMesh &h = m->h;
	const int N = h.nelem;
	P.nelem = N;
	std::vector<int> pos_cell, cell_pos(N);
	std::vector<int> part_ptr, lev_ptr, lev_pos;
	if (P.ordering == 1) {
		const BlockOrder bo = block_colour_order(h, P.part_size, colouring);
		P.ncolors = bo.ncolors;
		P.cpart = bo.cpart_ptr;
		pos_cell = bo.pos_cell;
		part_ptr = bo.part_ptr;
		lev_ptr = bo.lev_ptr;
		lev_pos = bo.lev_pos;
		P.nparts = bo.nparts;
		P.max_width = bo.max_width;
		for (size_t k = 0; k + 1 < part_ptr.size(); k++) P.part_cap = std::max(P.part_cap, part_ptr[k + 1] - part_ptr[k]);
	} else {
		P.ncolors = h.ncolors;
		P.cptr = h.color_ptr;
		pos_cell = h.color_cells;
	}
	for (int p = 0; p < N; p++) cell_pos[pos_cell[p]] = p;
	P.order_h = pos_cell;
	std::vector<int4> pn(N), pp(N);
	for (int p = 0; p < N; p++) {
		const int i = pos_cell[p];
		int a[4], c[4];
		for (int j = 0; j < 4; j++) {
			const int nb = j < h.nnode[i] ? h.esuel[4 * i + j] : NO_EDGE;
			a[j] = nb >= 0 ? nb : -1;
			c[j] = nb >= 0 ? cell_pos[nb] : -1;
		}
		pn[p] = make_int4(a[0], a[1], a[2], a[3]);
		pp[p] = make_int4(c[0], c[1], c[2], c[3]);
	}
	// block colours: each cell's first slot among its part's in-part lower and upper
	// neighbour blocks (the sweeps stage exactly these), and the fullest part's counts
	std::vector<int2> pb;
	if (P.ordering == 1) {
		pb.resize(N);
		for (size_t k = 0; k + 1 < part_ptr.size(); k++) {
			const int p0 = part_ptr[k], p1 = part_ptr[k + 1];
			int lo = 0, upc = 0;
			for (int p = p0; p < p1; p++) {
				pb[p] = make_int2(lo, upc);
				const int q4[4] = {pp[p].x, pp[p].y, pp[p].z, pp[p].w};
				for (int j = 0; j < 4; j++) {
					if (q4[j] >= p0 && q4[j] < p) lo++;
					if (q4[j] > p && q4[j] < p1) upc++;
				}
			}
			P.blk_cap_lo = std::max(P.blk_cap_lo, lo);
			P.blk_cap_up = std::max(P.blk_cap_up, upc);
		}
	}
	cudaError_t e = cudaSuccess;
	auto up = [&](void **d, const void *src, size_t bytes) {
		if (e) return;
		e = cudaMalloc(d, bytes);
		if (!e) e = cudaMemcpy(*d, src, bytes, cudaMemcpyHostToDevice);
	};
	up((void **)&P.pos_cell, pos_cell.data(), sizeof(int) * N);
	up((void **)&P.cell_pos, cell_pos.data(), sizeof(int) * N);
	up((void **)&P.pnbr, pn.data(), sizeof(int4) * N);
	up((void **)&P.pnbrpos, pp.data(), sizeof(int4) * N);
	if (P.ordering == 1) {
		up((void **)&P.pblk, pb.data(), sizeof(int2) * N);
		up((void **)&P.part_ptr, part_ptr.data(), sizeof(int) * part_ptr.size());
		up((void **)&P.lev_ptr, lev_ptr.data(), sizeof(int) * lev_ptr.size());
		up((void **)&P.lev_pos, lev_pos.data(), sizeof(int) * lev_pos.size());
	}
	if (!e) {
		int dev = 0;
		e = cudaGetDevice(&dev);
		if (!e) e = cudaDeviceGetAttribute(&P.num_sms, cudaDevAttrMultiProcessorCount, dev);
	}
	if (!e && P.ordering == 1) {
		// shared memory of the part kernels beyond the 48 KB default
		// (the sweeps' limit is set for the largest parts any preconditioner may have, since the
		// setting is per kernel, not per preconditioner; a launch's own size sets its occupancy)
		const int cap = std::max(P.part_cap, 1), big = kMaxPartSize;
		if (prec == 4) {
			const int lim = (int)sweep_smem<float>(big, 4 * big, true);
			for (const void *k : {(const void *)k_fwd_parts<float, false>, (const void *)k_fwd_parts<float, true>,
			                      (const void *)k_bwd_parts<float, false>, (const void *)k_bwd_parts<float, true>})
				if (!e) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
			if (!e) e = cudaFuncSetAttribute(k_ilu_parts<float, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ilu_smem<float>(cap));
			if (!e) e = cudaFuncSetAttribute(k_ilu_parts<float, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ilu_smem<float>(cap));
		} else {
			const int lim = (int)sweep_smem<double>(big, 4 * big, true);
			for (const void *k : {(const void *)k_fwd_parts<double, false>, (const void *)k_fwd_parts<double, true>,
			                      (const void *)k_bwd_parts<double, false>, (const void *)k_bwd_parts<double, true>})
				if (!e) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
			if (!e) e = cudaFuncSetAttribute(k_ilu_parts<double, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ilu_smem<double>(cap));
			if (!e) e = cudaFuncSetAttribute(k_ilu_parts<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ilu_smem<double>(cap));
		}
	}
	const size_t w = prec;
	if (!e && (type == PC_SGS || type == PC_ILU0)) e = cudaMalloc(&P.F, (size_t)batch * 5 * N * 16 * w);
	if (!e) e = cudaMalloc(&P.Dinv, (size_t)batch * N * 16 * w);
	if (!e) e = cudaMalloc(&P.y, (size_t)batch * N * 4 * w);
	return e;
}

void precond_free(Precond &P)
{
	void *ps[] = {P.pos_cell, P.cell_pos, P.pnbr, P.pnbrpos, P.pblk, P.F, P.Dinv, P.y, P.part_ptr, P.lev_ptr, P.lev_pos};
	for (void *p : ps)
		if (p) cudaFree(p);
	P.pos_cell = nullptr; P.cell_pos = nullptr; P.pnbr = nullptr; P.pnbrpos = nullptr; P.pblk = nullptr;
	P.F = nullptr; P.Dinv = nullptr; P.y = nullptr;
	P.part_ptr = nullptr; P.lev_ptr = nullptr; P.lev_pos = nullptr;
}

cudaError_t precond_setup(Precond &P, int *err, const int *active, cudaStream_t s, int *nk)
{
	if (P.type == PC_NONE) return cudaSuccess;
	return P.prec == 4 ? precond_setup_t<float>(P, err, active, s, nk) : precond_setup_t<double>(P, err, active, s, nk);
}

cudaError_t precond_apply(const Precond &P, const double *r, double *z, const int *active, cudaStream_t s, int *nk)
{
	return P.prec == 4 ? precond_apply_t<float>(P, r, z, active, s, nk) : precond_apply_t<double>(P, r, z, active, s, nk);
}

cudaError_t block_spmv(const BlockMatrix &A, const int4 *cnbr, const double *x, double *y, const int *active,
                       cudaStream_t s, int *nk)
{
	const dim3 g((A.nelem + BS - 1) / BS, A.batch);
	if (A.prec == 4) k_spmv<float><<<g, BS, 0, s>>>(A.nelem, (const float *)A.val, cnbr, x, y, active);
	else k_spmv<double><<<g, BS, 0, s>>>(A.nelem, (const double *)A.val, cnbr, x, y, active);
	(*nk)++;
	return cudaGetLastError();
}

cudaError_t krylov_alloc(Krylov &K, int n, int batch, int restart)
{
	K.n = n;
	K.batch = batch;
	K.restart = restart;
	K.nblk = std::max(1, std::min(1024, (n + RBS * 4 - 1) / (RBS * 4)));
	const size_t B = batch;
	cudaError_t e = cudaSuccess;
	auto al = [&](void **p, size_t bytes) {
		if (!e) e = cudaMalloc(p, bytes);
		if (!e) e = cudaMemset(*p, 0, bytes);
	};
	al((void **)&K.V, sizeof(double) * B * (restart + 1) * n);  // [vector][member][n]
	al((void **)&K.Z, sizeof(double) * B * restart * n);
	al((void **)&K.w, sizeof(double) * B * n);
	al((void **)&K.H, sizeof(double) * B * (restart + 1) * restart);
	al((void **)&K.cs, sizeof(double) * B * (restart + 1));
	al((void **)&K.sn, sizeof(double) * B * (restart + 1));
	al((void **)&K.g, sizeof(double) * B * (restart + 1));
	al((void **)&K.part, sizeof(double) * B * (restart + 2) * K.nblk);
	al((void **)&K.scal, sizeof(double) * B * 8);
	al((void **)&K.active, sizeof(int) * B);
	al((void **)&K.iters, sizeof(int) * B);
	al((void **)&K.kdone, sizeof(int) * B);
	al((void **)&K.vcur, sizeof(double) * B * n);
	al((void **)&K.zcur, sizeof(double) * B * n);
	al((void **)&K.jcur, sizeof(int));
	al((void **)&K.loops, sizeof(unsigned));
	if (!e) e = cudaStreamCreateWithFlags(&K.aux, cudaStreamNonBlocking);
	return e;
}

void krylov_free(Krylov &K)
{
	void *ps[] = {K.V, K.Z, K.w, K.H, K.cs, K.sn, K.g, K.part, K.scal, K.active, K.iters, K.kdone,
	              K.vcur, K.zcur, K.jcur, K.loops};
	for (void *p : ps)
		if (p) cudaFree(p);
	if (K.aux) cudaStreamDestroy(K.aux);
	K = Krylov();
}

/* one Arnoldi step on stream s (preconditioner, operator, classical
 * Gram-Schmidt, Givens rotation, next basis vector, loop control) */
static cudaError_t arnoldi_step(Krylov &K, LinOp &op, const Precond &P, int maxit, cudaStream_t s, int *nk,
                                cudaGraphConditionalHandle h, int set_cond)
{
	const int n = K.n, B = K.batch, m = K.restart, nb = K.nblk;
	const size_t vstep = (size_t)B * n;
	cudaError_t e;
	if ((e = precond_apply(P, K.vcur, K.zcur, K.active, s, nk)) != cudaSuccess) return e;
	if ((e = op.apply(K.zcur, K.w, K.active, s, nk)) != cudaSuccess) return e;
	k_dot_partial<<<dim3(nb, B, maxit), RBS, 0, s>>>(n, nb, K.V, n, vstep, K.w, n, K.part, 0, m + 2, K.active, K.jcur);
	k_reduce_h<<<dim3(B, maxit), 32, 0, s>>>(K, nb);
	k_cgs_update<<<dim3(nb, B), RBS, 0, s>>>(K, nb);
	k_givens<<<B, 32, sizeof(double) * 3 * (m + 1), s>>>(K, nb, maxit);
	k_next_basis<<<dim3((unsigned)((n + 255) / 256), B), 256, 0, s>>>(K);
	k_loop_ctrl<<<1, 32, 0, s>>>(K, maxit, h, set_cond);
	*nk += 6;
	return cudaGetLastError();
}

cudaError_t fgmres_solve(Krylov &K, LinOp &op, const Precond &P, const double *b, double *x, int maxit, double rtol,
                         const int *member_active, cudaStream_t s, int *nk_fixed, int *nk_iter)
{
	const int n = K.n, B = K.batch, m = K.restart, nb = K.nblk;
	if (maxit > m) maxit = m;  // one cycle (the reference configuration: restart = max_it = 30)
	const dim3 ge((unsigned)((n + 255) / 256), B);
	cudaError_t e;
	// ||b||, x = 0, v0 = b/||b||
	k_dot_partial<<<dim3(nb, B, 1), RBS, 0, s>>>(n, nb, b, n, 0, b, n, K.part, 0, m + 2, member_active, nullptr);
	k_gm_init<<<B, 32, 0, s>>>(K, nb, rtol, member_active);
	k_first_basis<<<ge, 256, 0, s>>>(K, b, x);
	*nk_fixed += 3;
	cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
	if ((e = cudaStreamIsCapturing(s, &cst)) != cudaSuccess) return e;
	*nk_iter = 0;
	if (cst == cudaStreamCaptureStatusActive) {
		// WHILE node in the graph being captured; its body is one Arnoldi step
		cudaGraph_t g;
		const cudaGraphNode_t *deps = nullptr;
		size_t nd = 0;
		if ((e = cudaStreamGetCaptureInfo(s, &cst, nullptr, &g, &deps, nullptr, &nd)) != cudaSuccess) return e;
		cudaGraphConditionalHandle h;
		if ((e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
		cudaGraphNodeParams cp = {};
		cp.type = cudaGraphNodeTypeConditional;
		cp.conditional.handle = h;
		cp.conditional.type = cudaGraphCondTypeWhile;
		cp.conditional.size = 1;
		cudaGraphNode_t node;
		if ((e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp)) != cudaSuccess) return e;
		if ((e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies)) != cudaSuccess)
			return e;
		cudaGraph_t body = cp.conditional.phGraph_out[0];
		if ((e = cudaStreamBeginCaptureToGraph(K.aux, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
			return e;
		cudaError_t e1 = arnoldi_step(K, op, P, maxit, K.aux, nk_iter, h, 1);
		cudaError_t e2 = cudaStreamEndCapture(K.aux, &body);
		if (e1 != cudaSuccess) return e1;
		if (e2 != cudaSuccess) return e2;
	} else {
		for (int j = 0; j < maxit; j++) {
			int nki = 0;
			if ((e = arnoldi_step(K, op, P, maxit, s, &nki, 0, 0)) != cudaSuccess) return e;
			*nk_iter = nki;
			*nk_fixed += nki;
		}
	}
	k_backsolve<<<(B + 31) / 32, 32, 0, s>>>(K, member_active);
	k_update_x<<<ge, 256, 0, s>>>(K, x, member_active);
	*nk_fixed += 2;
	return cudaGetLastError();
}

}  // namespace fvg
