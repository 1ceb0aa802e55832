// Internal device data structures of the GB300 hot path.
//
// HBM layout (all device arrays, batch-major where a batch dimension exists):
//   cells (RCM order): centroid double2, area, 1/area; per cell an int4 of
//     encoded faces ((face << 1) | side, side 1 = cell is the right cell,
//     -1 = no fourth edge) and an int4 of neighbours (cell index, or
//     -1 - ib for the ghost of boundary face ib, NO_EDGE none), both in local-edge
//     order so a warp reads its cells' stencils with 16-byte loads.
//   faces (boundary faces first): int2 (left, right | -1-ib), double4
//     (nx, ny, len, 0), face centre double2; per-face gradient weights.
//   states: u, r  [batch][cell][4] FP64 (the reference's row-major Vec);
//           prim  [batch][cell] (rho,u,v,p) FP64, grad [batch][cell][8]
//           (GradBlock_t order: (x,v0),(y,v0),(x,v1),...).
//   Jacobian: fixed-width block rows, 5 slots per cell (diagonal + local
//     edges), each slot a 4x4 row-major block; values [batch][slot][cell][16]
//     so consecutive cells of one slot are contiguous (coalesced).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include "fv_device.cuh"
#include "fv_mesh.hpp"

namespace fvg {

/* marker of the unused fourth edge of a triangle in per-cell neighbour lists
 * (distinct from every boundary-ghost code -1 - ib) */
constexpr int NO_EDGE = -2147483647 - 1;

struct __align__(32) d4 { double x, y, z, w; };
struct __align__(16) f4 { float x, y, z, w; };

enum { GRAD_NONE = 0, GRAD_GREENGAUSS = 1, GRAD_LEASTSQUARES = 2 };
enum { REC_NONE = 0, REC_VANALBADA = 1, REC_BARTHJESPERSEN = 2, REC_VENKATAKRISHNAN = 3, REC_WENO = 4 };
enum { PC_NONE = 0, PC_JACOBI = 1, PC_SGS = 2, PC_ILU0 = 3 };

/* Device mesh (owned by fv_mesh). */
struct DevMesh {
	int nelem = 0, nbface = 0, naface = 0, ncolors = 0;
	double2 *cc = nullptr;
	double *area = nullptr, *iarea = nullptr;
	int4 *cface = nullptr, *cnbr = nullptr;
	int4 *cslot_rev = nullptr;  // for cell i, edge j: the edge index of the same face in the neighbour
	int2 *flr = nullptr;
	int2 *fslot = nullptr;      // local edge of the face in its left / right cell
	d4 *fgeo = nullptr;
	double2 *fcen = nullptr;
	double2 *gcen = nullptr;
	int *color_cells = nullptr;
	std::vector<int> color_ptr;  // host copy
};

struct fv_mesh_impl {
	HostMesh h;
	DevMesh d;
	bool dev_ready = false;
};

/* Spatial discretisation state (owned by fv_disc). */
struct DiscDev {
	int nelem, nbface, naface, batch;
	// mesh views
	const double2 *cc; const double *area, *iarea;
	const int4 *cface, *cnbr;
	const int2 *flr; const d4 *fgeo; const double2 *fcen, *gcen;
	const int *bcid;                // per boundary face: index into bcs
	const BCDev *bcs;
	const Phys *phys;               // [batch]
	// precomputed gradient coefficients per cell and local edge j (the
	// gradient is linear in the cell's and its neighbours' values):
	//   Green-Gauss  grad_i = gself_i q_i + sum_j gcoef_ij q_nbr(j)
	//   least squares grad_i = sum_j gcoef_ij (q_nbr(j) - q_i)
	// gcoef[2 i] = (x, y of edge 0, x, y of edge 1), gcoef[2 i + 1] = edges 2, 3
	const d4 *gcoef;
	const double2 *gself;           // Green-Gauss self coefficient (x, y)
	const d4 *fvis;                 // viscous: unit (rc_R - rc_L), 1/|rc_R - rc_L|
	const double *veps2;            // Venkatakrishnan (K h)^3 per cell
	// configuration
	int flux, jflux, gradscheme, recon, order2, viscous, constvisc;
	double limparam;
	// batch members to skip (set by the steady solver once a member has
	// converged or failed); NULL = evaluate every member
	const int *active;
};

__device__ __forceinline__ bool skip_member(const DiscDev &D, int b) { return D.active && !D.active[b]; }

/* reconstructions whose face values use gradients of their own (ResidualWork::lgrad) */
inline bool recon_gradients(int recon) { return recon == 2 || recon == 3 || recon == 4; }

/* Scratch of one residual evaluation (per batch member slices). */
struct ResidualWork {
	d4 *prim = nullptr;        // [batch][nelem]
	d4 *ghost_prim = nullptr;  // [batch][nbface]  cell-centred ghost state, primitive
	d4 *ghost_cons = nullptr;  // [batch][nbface]  cell-centred ghost state, conserved
	d4 *grad = nullptr;        // [batch][nelem][2]
	d4 *lgrad = nullptr;       // [batch][nelem][2] reconstruction gradients: WENO-blended, or
	                           // scaled by the Barth-Jespersen / Venkatakrishnan limiter values
	d4 *fflux = nullptr;       // [batch][naface] integrated face fluxes
	double2 *spec = nullptr;   // [batch][naface] spectral radii (left, right)
};

enum { KBS_PREP = 0, KBS_GRAD = 1, KBS_FACE = 2, KBS_GATHER = 3, KBS_JAC = 4, KBS_COUNT = 5 };

struct fv_disc_impl {
	fv_mesh_impl *mesh = nullptr;
	DiscDev d;
	int batch = 1;
	std::vector<Phys> phys_h;
	std::vector<BCDev> bcs_h;
	std::vector<int> bctags;
	// owned device arrays
	std::vector<void *> owned;
	ResidualWork w;
	int bs[KBS_COUNT] = {128, 128, 128, 128, 128};  // block sizes of the residual and Jacobian kernels (KBS_*), fv_disc_autotune
	int *btag = nullptr;       // device: boundary marker of each boundary face
	double *surf = nullptr;    // device: surface-integral partials [batch][4]
	cudaStream_t stream = 0;
	int device = 0;            // CUDA device current when the handle was created
	int kernels_launched = 0;  // running count of this handle's kernel launches
};

// ------------------------------- kernels -------------------------------------
/* w: the scratch to evaluate into (NULL: the handle's own, D->w) */
cudaError_t residual_launch(fv_disc_impl *D, const double *u, double *r, int gettimesteps, double *dt,
                            cudaStream_t s, const ResidualWork *w = nullptr);
cudaError_t gradients_launch(fv_disc_impl *D, const double *u, double *grad, int conserved, cudaStream_t s);
/* the residual's passes before the face kernel (primitive/ghost states,
 * gradients, limiter values, WENO blend) into the handle's scratch */
/* the passes before the face kernel; with x, at the state u + pm x (per member pm) */
cudaError_t gradient_pass_launch(fv_disc_impl *D, const double *u, cudaStream_t s, const double *x = nullptr,
                                 const double *pm = nullptr, const ResidualWork *w = nullptr);
cudaError_t residual_mf_launch(fv_disc_impl *D, const double *u, const double *up, const double *x, const double *r,
                               const double *dtm, const double *pm, double *y, cudaStream_t s);
/* times the residual kernels at 64 / 128 / 256 threads per block at state u
 * and keeps the fastest per kernel in D->bs; chosen[4] (may be NULL) receives them */
cudaError_t residual_autotune(fv_disc_impl *D, const double *u, cudaStream_t s, int *chosen);
/* the face-flux launch alone (reads the prep/gradient/limiter results of the
 * last residual evaluation of the same state) */
cudaError_t face_launch(fv_disc_impl *D, const double *u, int gettimesteps, cudaStream_t s,
                        const ResidualWork *w = nullptr);

/* Block-row matrix: 5 slots per cell (0 = diagonal, 1+j = neighbour across
 * local edge j); values [batch][slot][cell][16], FP32 or FP64. */
struct BlockMatrix {
	int nelem = 0, batch = 1, prec = 4;
	void *val = nullptr;        // float or double
	double *bdiag = nullptr;    // scratch: boundary-face diagonal contributions [batch][nbface][16]
	size_t nval() const { return (size_t)batch * 5 * nelem * 16; }
};

cudaError_t jacobian_launch(fv_disc_impl *D, const double *u, BlockMatrix &A, cudaStream_t s);

}  // namespace fvg
