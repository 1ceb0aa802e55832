/*
 * fvens_gb300 — C ABI of the GB300 (sm_103a) steady implicit flow hot path.
 *
 * The entry points replace the reference's spatial-discretisation and
 * steady-solver interfaces (paths relative to the reference project):
 *   Spatial / FlowFV            src/spatial/aspatial.hpp:37-167,
 *                               src/spatial/flow_spatial.hpp:61-324
 *   FlowPhysicsConfig,
 *   FlowNumericsConfig          src/spatial/flow_spatial.hpp:33-55
 *   FlowBCConfig                src/spatial/abc.hpp:34-40
 *   UMesh construction          src/mesh/mesh.hpp, src/mesh/ameshutils.cpp:102-157
 *   SteadyBackwardEulerSolver   src/ode/aodesolver.hpp, aodesolver.cpp:363-638
 *   KSP/PC (PETSc, external)    FGMRES + bjacobi/ILU(0), SOR, point-block Jacobi
 *
 * Conventions
 *   - Plain C types only.  Device pointers (d_*) point to CUDA global memory;
 *     host pointers (h_*) to host memory.
 *   - State vectors are the reference's PETSc block layout: nelem x 4 doubles
 *     per flow condition (rho, rho*u, rho*v, rho*E), row-major; a batch of B
 *     conditions on one mesh is B such vectors back to back.
 *   - Calls on a handle are ordered on that handle's CUDA stream
 *     (fv_disc_set_stream); device-pointer calls return before the GPU work
 *     completes unless stated otherwise.  Host-pointer calls synchronise.
 *   - No exception crosses the ABI: every call returns an fv_status; the
 *     reference's Numerical_error / Tolerance_error map to FV_ERR_NUMERICAL /
 *     FV_ERR_TOLERANCE.  fv_last_error() describes the most recent failure of
 *     the calling thread.
 *   - Handles are not reentrant: one thread at a time per handle, as the
 *     reference's FlowFV::compute_residual (flow_spatial.hpp:190-198).
 */
#ifndef FVENS_GB300_H
#define FVENS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ABI version of this header.  A caller compiled against it checks
 * fv_abi_version() == FVENS_GB300_ABI_VERSION after loading the library.
 *   1  first release
 *   2  fv_mesh_line_ordering gained its `rcm` argument (before `order`)
 *   3  fv_solver_cfg gained stall_steps and stall_factor (at its end) */
#define FVENS_GB300_ABI_VERSION 3

typedef int fv_status;
#define FV_OK 0
#define FV_ERR_INVALID 1      /* bad argument or configuration */
#define FV_ERR_CUDA 2         /* CUDA runtime failure (no device, launch or memory error) */
#define FV_ERR_NUMERICAL 3    /* non-finite residual norm (reference: Numerical_error) */
#define FV_ERR_TOLERANCE 4    /* max steps reached (reference: Tolerance_error) */
#define FV_ERR_UNSUPPORTED 5  /* option the reference does not implement (e.g. VanLeer Jacobian) */
#define FV_ERR_MESH 6         /* mesh topology/geometry error */

/* FVENS_GB300_ABI_VERSION of the loaded library */
int fv_abi_version(void);

/* inviscid fluxes (afactory.cpp:31-92 names) */
#define FV_FLUX_LLF 0
#define FV_FLUX_VANLEER 1
#define FV_FLUX_AUSM 2
#define FV_FLUX_AUSMPLUS 3
#define FV_FLUX_ROE 4
#define FV_FLUX_HLL 5
#define FV_FLUX_HLLC 6
/* gradients (afactory.cpp:103-139) */
#define FV_GRAD_NONE 0
#define FV_GRAD_GREENGAUSS 1
#define FV_GRAD_LEASTSQUARES 2
/* reconstructions / limiters (afactory.cpp:168-227) */
#define FV_REC_NONE 0
#define FV_REC_VANALBADA 1
#define FV_REC_BARTHJESPERSEN 2
#define FV_REC_VENKATAKRISHNAN 3
#define FV_REC_WENO 4
/* boundary conditions: the reference's BCType numbering (abctypes.hpp) */
#define FV_BC_SLIPWALL 0
#define FV_BC_FARFIELD 1
#define FV_BC_INFLOW_OUTFLOW 2
#define FV_BC_SUBSONIC_INFLOW 3
#define FV_BC_EXTRAPOLATION 4
#define FV_BC_PERIODIC 5
#define FV_BC_ISOTHERMALWALL 6
#define FV_BC_ADIABATICWALL 7
/* preconditioners (PETSc -pc_type pbjacobi / sor / bjacobi+ilu) */
#define FV_PC_NONE 0
#define FV_PC_JACOBI 1
#define FV_PC_SGS 2
#define FV_PC_ILU0 3
/* synthetic meshes for fv_mesh_generate */
#define FV_MESH_CHANNEL_BUMP 1  /* params: nx, ny, split_fraction, seed */
#define FV_MESH_NACA_OGRID 2    /* params: nc, nr, rfar, nbl, h0, growth, tri_from_ring, seed */
#define FV_MESH_NACA_HYBRID 3   /* params: nc, nbl, h0, growth, rfar, beta: quad boundary layer, near-isotropic
                                   outer triangles marched out to rfar (beta in [0,1] bounds surface clustering) */

typedef struct fv_mesh fv_mesh;
typedef struct fv_disc fv_disc;
typedef struct fv_matrix fv_matrix;

/* ---- utilities ---- */
const char *fv_status_string(fv_status s);
const char *fv_last_error(void);
/* Number of CUDA kernels this library has launched in the process so far. */
long long fv_kernel_launch_count(void);

/* ---- mesh: UMesh + preprocessMesh (mesh.cpp, ameshutils.cpp:39-157) ---- */
typedef struct {
	int npoin, nelem, nbface;
	const double *coords; /* npoin x 2 */
	const int *nnode;     /* nelem, 3 or 4 */
	const int *inpoel;    /* nelem x 4, counter-clockwise, -1 padded */
	const int *bface;     /* nbface x 2 node indices */
	const int *btag;      /* nbface boundary markers */
} fv_mesh_desc;

/* reorder: 0 keep the input cell order, 1 reverse Cuthill-McKee (-mesh_reorder rcm). */
fv_status fv_mesh_create(const fv_mesh_desc *desc, int reorder, fv_mesh **out);
fv_status fv_mesh_generate(int kind, const double *params, int nparams, int reorder, fv_mesh **out);
/* Gmsh 2.2 ASCII (meshreaders.cpp:66-265) */
fv_status fv_mesh_read_gmsh(const char *path, int reorder, fv_mesh **out);
/* SU2 ASCII, 2-D, numeric marker tags (meshreaders.cpp:267-397) */
fv_status fv_mesh_read_su2(const char *path, int reorder, fv_mesh **out);
/* readMesh (meshreaders.cpp:33-50): .msh (Gmsh) or .su2 by extension */
fv_status fv_mesh_read(const char *path, int reorder, fv_mesh **out);
/* counts: nelem, nbface, ninface, naface, npoin, ncolors */
fv_status fv_mesh_counts(const fv_mesh *m, int counts[6]);
/* The mesh as built (cells in their final order, boundary faces oriented);
 * perm[k] = input index of cell k.  Any pointer may be NULL. */
fv_status fv_mesh_export(const fv_mesh *m, double *coords, int *nnode, int *inpoel, int *bface, int *btag, int *perm);
/* face_lr: naface x 2 (left, right; right = -1-ib on boundary face ib);
 * fnorm: naface x 3 (nx, ny, len); area: nelem; cc: nelem x 2; color: nelem */
fv_status fv_mesh_geometry(const fv_mesh *m, int *face_lr, double *fnorm, double *area, double *cc, int *color);
/* block-colour elimination order of the SGS / ILU(0) preconditioners
 * (compact parts of ~part_size cells, parts coloured): order[position] = cell */
fv_status fv_mesh_block_order(const fv_mesh *m, int part_size, int *order, int *nparts, int *ncolors);
/* fv_mesh_block_order with the parts coloured greedily (colouring 0, as
 * fv_mesh_block_order) or by DSatur with Kempe-chain interchanges (1: usually
 * one colour, so one launch per sweep, fewer); the orders of fv_solver_cfg
 * pc_ordering 1 and 2 */
fv_status fv_mesh_block_order_ex(const fv_mesh *m, int part_size, int colouring, int *order, int *nparts,
                                 int *ncolors);
/* Lines of strongly coupled cells (findLines, meshordering.cpp:131-262; the
 * reference's -mesh_reorder line -mesh_anisotropy_threshold): from the cell
 * of each boundary face, follow the neighbour of largest (1/distance) weight,
 * relative to the cell's smallest, while it exceeds threshold.  The mesh keeps
 * the lines: preconditioners created afterwards put whole lines into their
 * parts.  threshold <= 0 removes them.  *nlines, cell_line[nelem] (line index
 * or -1; either may be NULL) receive the result. */
fv_status fv_mesh_find_lines(fv_mesh *m, double threshold, int *nlines, int *cell_line);
/* getHybridLineOrdering (meshordering.cpp:69-141) on the lines found by
 * fv_mesh_find_lines: rcm = 0 ("natural") gives the cells of each line, line
 * by line, then the cells outside lines in index order; rcm = 1 first
 * reorders the graph of lines and remaining cells by reverse Cuthill-McKee
 * (PETSc's "rcm", SPARSEPACK GENRCM).  order[nelem] = cell at each position
 * (without lines: the identity, or the RCM order of the cells). */
fv_status fv_mesh_line_ordering(const fv_mesh *m, int rcm, int *order);
/* UMesh::compute_periodic_map (mesh.cpp:368-421): pairs the boundary faces of
 * `marker` whose centres agree (to 1e-8) along the axis other than `axis`
 * (0 = x, 1 = y); map[nbface] = partner boundary face or -1.  The flow
 * discretisation, as the reference's, has no periodic boundary condition
 * (FV_BC_PERIODIC is rejected). */
fv_status fv_mesh_periodic_map(const fv_mesh *m, int marker, int axis, int *map);
void fv_mesh_destroy(fv_mesh *m);

/* ---- spatial discretisation: FlowFV<freal,order2,constVisc> (afactory.cpp:252-276) ---- */
typedef struct {
	double gamma, Minf, Tinf, Reinf, Pr;
	double aoa;          /* radians */
	int viscous_sim, const_visc;
} fv_physics_cfg;
typedef struct {
	int conv_numflux, conv_numflux_jac, gradientscheme, reconstruction;
	double limiter_param;
	int order2;
} fv_numerics_cfg;
typedef struct {
	int bc_tag, bc_type;
	double bc_vals[2];
} fv_bc_cfg;

/* One discretisation of `batch` flow conditions on one mesh (phys[batch]). */
fv_status fv_disc_create(fv_mesh *m, const fv_physics_cfg *phys, int batch, const fv_numerics_cfg *num,
                         const fv_bc_cfg *bcs, int nbc, fv_disc **out);
void fv_disc_destroy(fv_disc *d);
/* cudaStream_t passed as void*; NULL = legacy default stream */
fv_status fv_disc_set_stream(fv_disc *d, void *stream);
fv_status fv_disc_synchronize(fv_disc *d);
/* Autotuner (no counterpart in the reference): times the residual kernels
 * (states, gradients/limiter, faces, gather) and the Jacobian's face kernel
 * with 64, 128 and 256 threads per block at device state d_u and keeps the
 * fastest for this handle; results do not depend on the choice.
 * h_block_sizes[4] (host, may be NULL) receives the residual kernels' choice
 * (fv_disc_block_sizes gives all).  Synchronises. */
fv_status fv_disc_autotune(fv_disc *d, const double *d_u, int *h_block_sizes);
/* The block sizes in use (no counterpart in the reference): up to n of
 * [states, gradients, faces, gather, Jacobian faces]; fv_disc_autotune also
 * tunes the last one. */
fv_status fv_disc_block_sizes(const fv_disc *d, int n, int *h_block_sizes);
/* freestream conserved states (IdealGasPhysics::compute_freestream_state), batch x 4 */
fv_status fv_disc_freestream(const fv_disc *d, double *h_uinf);

/* Spatial::compute_residual (aspatial.hpp:64): d_r += -R(d_u); when
 * gettimesteps, d_dt[nelem*batch] receives the local time steps. */
fv_status fv_compute_residual(fv_disc *d, const double *d_u, double *d_r, int gettimesteps, double *d_dt);
/* fv_compute_residual with its scratch in one static device array of the
 * library (64 MiB) instead of the handle's own buffers; no counterpart in the
 * reference.  For callers whose evaluation path must not allocate device
 * memory: neither the call nor its set-up allocates.  The first call on a
 * device (that device current) looks up the array's address -- make it
 * before any stream capture.  The handle's device must be current
 * (FV_ERR_INVALID otherwise).  Discretisations whose scratch (cells x batch)
 * exceeds the array are rejected with FV_ERR_INVALID.  All calls share the
 * array: calls whose GPU work overlaps race on it. */
fv_status fv_compute_residual_static(fv_disc *d, const double *d_u, double *d_r, int gettimesteps, double *d_dt);
/* FlowFV_base::getGradients (flow_spatial.cpp:95-112): conserved-variable
 * cell gradients, nelem x 8 per condition in GradBlock_t order
 * ((x,v0),(y,v0),(x,v1),...).  With primitive != 0: the primitive-variable
 * gradients the second-order residual uses. */
fv_status fv_get_gradients(fv_disc *d, const double *d_u, double *d_grad, int primitive);
/* FlowFV_base::computeSurfaceData (flow_spatial.cpp:130-310): lift, pressure
 * drag and skin-friction drag coefficients over the boundary faces of marker
 * wall_marker, from the cell-centred state and its conserved gradients, FP64.
 * h_out[3*batch] = (Cl, CDp, CDsf) per condition (host).  Synchronises. */
fv_status fv_surface_data(fv_disc *d, const double *d_u, int wall_marker, double *h_out);
/* The per-face output of computeSurfaceData (flow_spatial.cpp:168-237), the
 * rows of FlowOutput::exportSurfaceData's wall files (aoutput.cpp:181-238):
 * h_out[4*nfaces] = (x, y, Cp, Cf) of each boundary face of wall_marker in
 * boundary-face order, for batch member `member`.  *nfaces receives the face
 * count; h_out == NULL only counts.  Synchronises. */
fv_status fv_surface_distribution(fv_disc *d, const double *d_u, int wall_marker, int member, double *h_out,
                                  int *nfaces);
/* FlowOutput::compute_entropy_cell (aoutput.cpp:28-62): sqrt(sum_i
 * ((s_i - s_inf)/s_inf)^2 A_i), s = p / rho^gamma, per condition into
 * h_err[batch] (host).  Uses the residual scratch.  Synchronises. */
fv_status fv_entropy_error(fv_disc *d, const double *d_u, double *h_err);

/* ---- Jacobian: Spatial::assemble_jacobian (aspatial.cpp:242-340) ---- */
/* precision 4: FP32 blocks, 8: FP64 blocks */
fv_status fv_matrix_create(fv_disc *d, int precision, fv_matrix **out);
void fv_matrix_destroy(fv_matrix *A);
fv_status fv_assemble_jacobian(fv_disc *d, const double *d_u, fv_matrix *A);
/* Adds d_diag[cell] * I to the diagonal blocks (addPseudoTimeTerm, aodesolver.cpp:300-329). */
fv_status fv_matrix_add_diagonal(fv_disc *d, fv_matrix *A, const double *d_diag);
/* Block-CSR copy of condition `member` (columns sorted, diagonal included):
 * rowptr[nelem+1], col[nnzb], val[nnzb*16] (row-major 4x4).  Pass val == NULL
 * to get nnzb only.  Synchronises. */
fv_status fv_matrix_to_host(fv_disc *d, const fv_matrix *A, int member, int *nnzb, int *rowptr, int *col,
                            double *val);

/* ---- preconditioners and Krylov solve (PETSc PC / KSP equivalents) ---- */
typedef struct fv_precond fv_precond;
/* type: FV_PC_*; the factor has the matrix's precision.  SGS and ILU(0)
 * eliminate in a colour order (fv_precond_order): ordering 1 = block colours
 * (compact parts of ~part_size cells, natural order inside a part; the
 * default), 0 = point colours. */
fv_status fv_precond_create(fv_disc *d, fv_matrix *A, int type, int ordering, int part_size, fv_precond **out);
void fv_precond_destroy(fv_precond *p);
/* factorises / inverts from the matrix's current values; FV_ERR_NUMERICAL on a
 * singular diagonal block.  Synchronises. */
fv_status fv_precond_setup(fv_precond *p);
/* d_z = M^{-1} d_r (all conditions of the batch) */
fv_status fv_precond_apply(fv_precond *p, const double *d_r, double *d_z);
/* elimination order: cell at each position (nelem ints) */
fv_status fv_precond_order(const fv_precond *p, int *order);
/* d_y = A d_x */
fv_status fv_matvec(fv_disc *d, fv_matrix *A, const double *d_x, double *d_y);
/* FGMRES(restart) on A x = b with the preconditioner's matrix, x0 = 0, stops
 * when ||b - A x|| <= rtol ||b|| or after maxit iterations (maxit <= restart);
 * h_iters[batch] receives the iteration counts.  Synchronises. */
fv_status fv_ksp_solve(fv_precond *p, const double *d_b, double *d_x, int restart, int maxit, double rtol,
                       int *h_iters);

/* ---- steady implicit solver: SteadyBackwardEulerSolver (aodesolver.hpp, aodesolver.cpp:363-638) ---- */
typedef struct fv_solver fv_solver;
typedef struct {
	double cfl_min, cfl_max;   /* pseudotime.main.cfl_min / cfl_max */
	double tolerance;          /* pseudotime.main.tolerance */
	int max_timesteps;         /* pseudotime.main.max_timesteps */
	int abs_tolerance;         /* 1: ||R|| <= tolerance; 0: relative to step 0 (the reference) */
	int pc_type;               /* FV_PC_* */
	int ksp_restart, ksp_maxit;
	double ksp_rtol;
	int matrix_free;           /* -matrix_free_jacobian */
	double mf_eps;             /* -matrix_free_difference_step */
	int nl_update;             /* 0 full, 1 robust_flow (FlowSimpleUpdate), 2 robust_flow whose
	                              factor above the threshold is min_relax (1 - min_relax) / danger
	                              and is then halved until the updated density and pressure stay
	                              above min_relax times their old values (positivity; not in the
	                              reference) */
	double min_relax;          /* min_nonlinear_relaxation_factor */
	int precision;             /* stored Jacobian and preconditioner: 4 FP32, 8 FP64 */
	int check_every;           /* steps between host polls of the convergence flags */
	int use_graph;             /* replay each step as a captured CUDA graph */
	int pc_ordering;           /* 1 block colours (default), 2 block colours with fewer colours
	                              (fv_mesh_block_order_ex colouring 1), 0 point colours */
	int pc_part_size;          /* cells per part of the block-colour order (default 128, at most 256) */
	int stall_steps;           /* stagnation stop (not in the reference): 0 off (default); else a
	                              member whose residual has not fallen below stall_factor times
	                              its last reference value within stall_steps steps ends with
	                              FV_ERR_TOLERANCE before max_timesteps */
	double stall_factor;       /* default 0.5 */
} fv_solver_cfg;
typedef struct {
	int steps, lin_iters, status; /* status: FV_OK, FV_ERR_NUMERICAL, FV_ERR_TOLERANCE */
	double res0, res, cfl;        /* area-weighted energy-residual L2 norm at step 0 / last step; last CFL */
} fv_solve_stats;

void fv_solver_cfg_default(fv_solver_cfg *cfg);
fv_status fv_solver_create(fv_disc *d, const fv_solver_cfg *cfg, fv_solver **out);
void fv_solver_destroy(fv_solver *s);
/* Solves every condition of the batch in place (d_u device state); member_mask
 * (host, batch ints, NULL = all) selects conditions; stats[batch] per member.
 * Returns FV_ERR_NUMERICAL if any member diverged, else FV_ERR_TOLERANCE if any
 * member hit max_timesteps, else FV_OK.  Synchronises. */
fv_status fv_solver_solve(fv_solver *s, double *d_u, const int *member_mask, fv_solve_stats *stats);
/* The same with a host state: copies in, solves, copies out. */
fv_status fv_solver_solve_host(fv_solver *s, double *h_u, const int *member_mask, fv_solve_stats *stats);
/* convergence history of one member (aoutput.cpp:617-640 columns): residual
 * norm, CFL and linear iterations per step; *n = steps written */
fv_status fv_solver_history(const fv_solver *s, int member, int maxn, double *res, double *cfl, int *linits, int *n);
/* kernels launched by one pseudo-time step (all members) */
long long fv_solver_kernels_per_step(const fv_solver *s);
/* Times one hot-path launch sequence in isolation with CUDA events on the
 * handle's stream (3 warm-up launches, then reps timed ones, each after a
 * 256 MB write that evicts L2) at state d_u;
 * *avg_ms = mean duration, *bytes = compulsory (algorithmic) bytes of one
 * launch for the roofline.  Synchronises. */
#define FV_KERNEL_RESIDUAL 0        /* whole residual evaluation */
#define FV_KERNEL_FACE_FLUX 1       /* face reconstruction + flux kernel */
#define FV_KERNEL_JACOBIAN 2        /* Jacobian assembly */
#define FV_KERNEL_PRECOND_APPLY 3   /* one preconditioner application */
#define FV_KERNEL_SPMV 4            /* block SpMV */
#define FV_KERNEL_PRECOND_SETUP 5   /* factorisation */
#define FV_KERNEL_GRADIENTS 6       /* residual passes before the face kernel (states, gradients, limiter) */
fv_status fv_solver_time_kernel(fv_solver *s, const double *d_u, int which, int reps, double *avg_ms, double *bytes);
/* FP64 throughput ceiling of the current device (a measurement aid; no
 * counterpart in the reference): a kernel of independent FP64 fused
 * multiply-add chains on every SM, timed with CUDA events, best of reps
 * launches after one warm-up.  *h_dfma_per_s = FMA thread-instructions per
 * second (2 FLOP each); *h_best_ms (may be NULL) = the best launch's time.
 * Changes no clock or power setting.  Synchronises. */
fv_status fv_fp64_peak(int reps, double *h_dfma_per_s, double *h_best_ms);

/* ---- explicit time stepping ---- */
/* SteadyForwardEulerSolver::solve (aodesolver.cpp:136-282): d_u (device,
 * every member) += cfg->cfl_min dt/A r with local time steps dt, until the
 * energy-residual norm meets cfg->tolerance (relative to the first step's, or
 * absolute with cfg->abs_tolerance) or cfg->max_timesteps steps ran (then
 * FV_ERR_TOLERANCE, as the reference's Tolerance_error).  The reference ramps a
 * CFL it never applies; the update uses the initial CFL.  stats[batch].
 * Synchronises. */
fv_status fv_steady_fe_solve(fv_disc *d, const fv_solver_cfg *cfg, double *d_u, fv_solve_stats *stats);
/* TVDRKSolver::solve (aodesolver.cpp:671-765) of temporal order 1..3 with
 * physical CFL cfl up to final_time, as the reference has it: every stage
 * evaluates the residual of the step's starting state; the step is
 * cfl * min_i dt_i.  max_steps bounds the steps (FV_ERR_TOLERANCE when
 * reached first; the reference has no bound).  h_steps[batch], h_time[batch]
 * (host, may be NULL) receive the steps taken and the time reached.
 * Synchronises. */
fv_status fv_tvdrk_solve(fv_disc *d, int order, double cfl, double final_time, int max_steps, double *d_u,
                         int *h_steps, double *h_time);

/* ---- pointwise device evaluations (for validation against the reference) ---- */
/* n states: d_ul, d_ur n x 4, d_n n x 2 -> d_f n x 4 (condition 0's physics) */
fv_status fv_pointwise_flux(fv_disc *d, int kind, int n, const double *d_ul, const double *d_ur, const double *d_nrm,
                            double *d_f);
/* flux Jacobian blocks in the reference's convention: d_dfdl = -dF/dul, d_dfdr = dF/dur (n x 16) */
fv_status fv_pointwise_flux_jacobian(fv_disc *d, int kind, int n, const double *d_ul, const double *d_ur,
                                     const double *d_nrm, double *d_dfdl, double *d_dfdr);
/* ghost states and BC Jacobians for BC kind bc_type with values bc_vals */
fv_status fv_pointwise_bc(fv_disc *d, int bc_type, const double *bc_vals, int n, const double *d_in,
                          const double *d_nrm, double *d_ghost, double *d_jac_ghost, double *d_dgdu);

/* ---- learned warm start (no counterpart in the reference) ----
 * A message-passing network on the mesh's cell graph predicts the converged
 * state of flow conditions (Minf, aoa, Reinf of fv_physics_cfg); the steady
 * solver starts from the prediction instead of freestream.  Width 64, `layers`
 * message-passing layers, BF16 tensor-core GEMMs with FP32 accumulation,
 * trained with Adam on states the solver converged.  The output y is the
 * state's deviation from freestream over a per-variable scale:
 * u = uinf + scale * y. */
typedef struct fv_mpnn fv_mpnn;
/* wall_markers: boundary markers whose faces give the wall-distance feature */
fv_status fv_mpnn_create(fv_mesh *m, int layers, const int *wall_markers, int nwall, unsigned long long seed,
                         fv_mpnn **out);
void fv_mpnn_destroy(fv_mpnn *n);
fv_status fv_mpnn_set_scale(fv_mpnn *n, const float *h_scale4);
/* tensor-core path of the forward pass's cell GEMMs (node update, message
 * MLP's first layer): 0 tcgen05.mma with tensor-memory accumulators, 1
 * (default, the faster on GB300 for these row-bound GEMMs) warp-level
 * mma.sync; both take BF16 operands and accumulate in FP32 */
fv_status fv_mpnn_set_gemm_path(fv_mpnn *n, int path);
/* test of the bounded waits (on != 0): the bulk-copy GEMMs announce their first
 * tile on its mbarrier without copying it, so every wait for it runs out
 * (after ~10 ms) and calls return FV_ERR_CUDA with the context still usable */
fv_status fv_mpnn_test_wait_limit(fv_mpnn *n, int on);
/* copies the flat FP32 parameter vector in (h_in != NULL) and then out
 * (h_out != NULL); *count receives its length */
fv_status fv_mpnn_params(fv_mpnn *n, float *h_out, const float *h_in, long long *count);
/* graph inputs: cell features nelem x 4, interior faces (L, R) nf x 2, face
 * features nf x 3 (any may be NULL) */
fv_status fv_mpnn_graph(const fv_mpnn *n, float *h_xs, int *h_faces, float *h_eattr);
/* d_u: batch x nelem x 4 predicted conserved states.  Synchronises. */
fv_status fv_mpnn_predict(fv_mpnn *n, const fv_physics_cfg *phys, int batch, double *d_u);
/* gradient (h_grad, length of fv_mpnn_params) and value (h_loss) of the mean
 * squared error of y against the targets d_target (batch x nelem x 4 conserved
 * states); either output may be NULL.  Synchronises. */
fv_status fv_mpnn_gradients(fv_mpnn *n, const fv_physics_cfg *phys, int batch, const double *d_target,
                            float *h_grad, float *h_loss);
/* one Adam step (beta 0.9, 0.999, eps 1e-8) with learning rate lr */
fv_status fv_mpnn_train_step(fv_mpnn *n, const fv_physics_cfg *phys, int batch, const double *d_target, float lr,
                             float *h_loss);

#ifdef __cplusplus
}
#endif
#endif
