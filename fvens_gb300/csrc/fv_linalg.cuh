// Block linear algebra of the implicit solve: preconditioners on the stored
// block Jacobian (point-block Jacobi, multicolour symmetric Gauss-Seidel,
// multicolour block ILU(0)), block SpMV and batched flexible GMRES.
//
// Replaces PETSc's -pc_type pbjacobi / sor / bjacobi+ilu on BAIJ(4) and
// KSPFGMRES (external to the reference; called from aodesolver.cpp:483).
// The elimination order of SGS and ILU(0) is either the block-colour order
// (default: compact parts of ~128 cells, parts coloured so that parts of one
// colour share no face; one launch per colour, one CTA per part sweeping the
// part's dependency levels with a barrier between levels) or the point-colour
// order (cells of one colour share no face; one fully parallel launch per
// colour).  The factor is stored in elimination order so each launch reads
// contiguous blocks.
#pragma once
#include "fv_core.cuh"

namespace fvg {

/* Preconditioner state; PR = float (FP32 sweeps) or double. */
struct Precond {
	int type = PC_NONE;
	int prec = 4;               // 4: FP32 factor, 8: FP64 factor
	int nelem = 0, batch = 1, ncolors = 0;
	int ordering = 1;           // 0: point colours, 1: block colours (parts of ~part_size cells)
	int part_size = 128;
	int nparts = 0, max_width = 0;
	int part_cap = 0;           // cells in the largest part (shared-memory staging size)
	std::vector<int> cptr;      // point colours: position range of each colour
	std::vector<int> cpart;     // block colours: part range of each colour
	int *part_ptr = nullptr;    // [nparts+1] position range of each part
	int *lev_ptr = nullptr;     // [nparts+1] range of each part's levels in lev_pos
	int *lev_pos = nullptr;     // level start positions
	std::vector<int> order_h;   // host copy of the elimination order (position -> cell)
	int *pos_cell = nullptr;    // [nelem] cell at colour-order position p
	int *cell_pos = nullptr;    // [nelem] position of cell i
	int4 *pnbr = nullptr;       // [nelem] neighbours (as cells) of the cell at position p, -1 none
	int4 *pnbrpos = nullptr;    // [nelem] their positions, -1 none
	int2 *pblk = nullptr;       // [nelem] block colours: first shared-memory slot of the cell's in-part
	                            // lower (x) and upper (y) neighbour blocks within its part
	int blk_cap_lo = 0, blk_cap_up = 0;  // in-part lower / upper blocks of the fullest part
	int num_sms = 1;            // SMs of the device (the sweeps' staging layout depends on the waves)
	void *F = nullptr;          // [batch][5][nelem][16] factor / copy in colour order
	void *Dinv = nullptr;       // [batch][nelem][16] inverted (factored) diagonal, colour order
	void *y = nullptr;          // [batch][nelem][4] intermediate sweep vector, colour order
	BlockMatrix *A = nullptr;   // source matrix (cell order)
};

/* ordering: 0 point colours, 1 block colours with parts of at most part_size
 * (parts coloured greedily), 2 block colours with the parts coloured by
 * DSatur and Kempe-chain interchanges (usually one colour fewer);
 * cells (1 <= part_size <= kMaxPartSize: a part is staged in shared memory) */
constexpr int kMaxPartSize = 256;
cudaError_t precond_alloc(Precond &P, fv_mesh_impl *m, int batch, int type, int prec, int ordering = 1,
                          int part_size = 128);
void precond_free(Precond &P);
/* factorisation / diagonal inversion from P.A; err_flag[b] (device ints, one
 * per batch member) is set non-zero when a diagonal block of member b is singular */
cudaError_t precond_setup(Precond &P, int *err_flag, const int *active, cudaStream_t s, int *nk);
/* z = M^{-1} r, FP64 vectors in cell order [batch][nelem][4] */
cudaError_t precond_apply(const Precond &P, const double *r, double *z, const int *active, cudaStream_t s, int *nk);
/* y = A x (FP64 vectors, cell order) plus optional diagonal shift diag[cell]*x */
cudaError_t block_spmv(const BlockMatrix &A, const int4 *cnbr, const double *x, double *y, const int *active,
                       cudaStream_t s, int *nk);

/* Batched FGMRES(m) workspace (classical Gram-Schmidt, Givens rotations, x0 = 0). */
struct Krylov {
	int n = 0;                  // unknowns per member (4 * nelem)
	int batch = 1, restart = 30;
	int nblk = 0;               // partial-sum blocks per member
	double *V = nullptr;        // [restart+1][batch][n]: each basis vector is a batched vector
	double *Z = nullptr;        // [restart][batch][n]
	double *w = nullptr;        // [batch][n]
	double *H = nullptr;        // [batch][(restart+1)*restart]
	double *cs = nullptr, *sn = nullptr, *g = nullptr;  // [batch][restart+1]
	double *part = nullptr;     // [batch][restart+2][nblk] partial sums
	double *scal = nullptr;     // [batch][8]: bnorm, target, hnorm, ...
	int *active = nullptr;      // [batch] member still iterating
	int *iters = nullptr;       // [batch] iterations done in this solve
	int *kdone = nullptr;       // [batch] Krylov dimension used
	double *vcur = nullptr;     // [batch][n] the basis vector being preconditioned (copy of V_j)
	double *zcur = nullptr;     // [batch][n] its preconditioned image (copied into Z_j)
	int *jcur = nullptr;        // iteration index j (device; all members share it)
	unsigned *loops = nullptr;  // Arnoldi iterations executed since the counter was last cleared
	cudaStream_t aux = nullptr; // stream the loop body is captured on
};

cudaError_t krylov_alloc(Krylov &K, int n, int batch, int restart);
void krylov_free(Krylov &K);

/* Operator callback: y = Op(x) for all active members. */
struct LinOp {
	virtual cudaError_t apply(const double *x, double *y, const int *active, cudaStream_t s, int *nk) = 0;
	virtual ~LinOp() {}
};

/* Solves Op x = b to ||b - Op x|| <= rtol ||b|| (or maxit iterations) for
 * every member whose member_active flag is set (NULL = all).  The iteration
 * count per member lands in K.iters.  The iteration index lives in device
 * memory, so one Arnoldi step is a fixed launch sequence.  Outside stream
 * capture the host issues maxit such steps (members that converged skip their
 * work); under stream capture the step becomes the body of a CUDA-graph WHILE
 * conditional node that the device stops once no member is iterating.
 * nk_fixed / nk_iter receive the launches outside / inside one step. */
cudaError_t fgmres_solve(Krylov &K, LinOp &op, const Precond &P, const double *b, double *x, int maxit, double rtol,
                         const int *member_active, cudaStream_t s, int *nk_fixed, int *nk_iter);

}  // namespace fvg
