// Declarations shared by the C ABI translation units.
#pragma once
#include <string>
#include "../../include/fvens_gb300.h"
#include "fv_core.cuh"

struct fv_mesh : fvg::fv_mesh_impl {};
struct fv_disc : fvg::fv_disc_impl {};
struct fv_matrix {
	fvg::BlockMatrix A;
	fv_disc *owner = nullptr;
};

namespace fvg {
void set_error(const std::string &s);
void count_launches(long long n);
fv_status cuda_status(cudaError_t e, const char *what);
Phys make_phys(const fv_physics_cfg &c);

cudaError_t matrix_add_diag_launch(BlockMatrix &A, const double *diag, cudaStream_t s);
cudaError_t pointwise_flux_launch(fv_disc_impl *D, int kind, int n, const double *ul, const double *ur,
                                  const double *nrm, double *f, cudaStream_t s);
cudaError_t pointwise_flux_jac_launch(fv_disc_impl *D, int kind, int n, const double *ul, const double *ur,
                                      const double *nrm, double *dfdl, double *dfdr, cudaStream_t s);
cudaError_t pointwise_bc_launch(fv_disc_impl *D, BCDev bc, int n, const double *in, const double *nrm, double *ghost,
                                double *jac_ghost, double *dgdu, cudaStream_t s);
}  // namespace fvg
