/*
 * C++ host interface over the fvens_gb300 C ABI, shaped like the reference's
 * classes so that existing call sites keep their form:
 *
 *   reference (paths in the reference project)        here
 *   UMesh + preprocessMesh (src/mesh)                  fvg::Mesh
 *   FlowFV_base / FlowFV (src/spatial/flow_spatial.hpp) fvg::FlowFV
 *     compute_residual(u, r, gettimesteps, dt)           same name and meaning (r += -R(u))
 *     assemble_jacobian(u, A)                            same, into fvg::BlockJacobian
 *     getGradients(u, grads)                             getGradients
 *   SteadyBackwardEulerSolver::solve (src/ode)          fvg::SteadyBackwardEulerSolver::solve
 *
 * Errors become exceptions of the reference's kinds: Numerical_error,
 * Tolerance_error, std::invalid_argument / std::runtime_error.
 * Device buffers are raw CUDA pointers; the *_host overloads copy.
 */
#ifndef FVENS_GB300_HPP
#define FVENS_GB300_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "fvens_gb300.h"

namespace fvg {

struct Numerical_error : std::runtime_error {
	explicit Numerical_error(const std::string &s) : std::runtime_error(s) {}
};
struct Tolerance_error : std::runtime_error {
	explicit Tolerance_error(const std::string &s) : std::runtime_error(s) {}
};

inline void check(fv_status s)
{
	if (s == FV_OK) return;
	const std::string msg = std::string(fv_status_string(s)) + ": " + fv_last_error();
	if (s == FV_ERR_NUMERICAL) throw Numerical_error(msg);
	if (s == FV_ERR_TOLERANCE) throw Tolerance_error(msg);
	if (s == FV_ERR_INVALID) throw std::invalid_argument(msg);
	throw std::runtime_error(msg);
}

class Mesh {
public:
	explicit Mesh(const fv_mesh_desc &d, int reorder = 1) { check(fv_mesh_create(&d, reorder, &m_)); counts(); }
	static Mesh from_gmsh(const std::string &path, int reorder = 1)
	{
		fv_mesh *m = nullptr;
		check(fv_mesh_read_gmsh(path.c_str(), reorder, &m));
		return Mesh(m);
	}
	static Mesh generate(int kind, const std::vector<double> &params, int reorder = 1)
	{
		fv_mesh *m = nullptr;
		check(fv_mesh_generate(kind, params.data(), (int)params.size(), reorder, &m));
		return Mesh(m);
	}
	Mesh(Mesh &&o) noexcept : m_(o.m_) { o.m_ = nullptr; for (int k = 0; k < 6; k++) c_[k] = o.c_[k]; }
	Mesh(const Mesh &) = delete;
	Mesh &operator=(const Mesh &) = delete;
	~Mesh() { fv_mesh_destroy(m_); }
	int gnelem() const { return c_[0]; }
	int gnbface() const { return c_[1]; }
	int gnaface() const { return c_[3]; }
	fv_mesh *get() const { return m_; }

private:
	explicit Mesh(fv_mesh *m) : m_(m) { counts(); }
	void counts() { check(fv_mesh_counts(m_, c_)); }
	fv_mesh *m_ = nullptr;
	int c_[6] = {0, 0, 0, 0, 0, 0};
};

class BlockJacobian;

class FlowFV {
public:
	FlowFV(Mesh &m, const std::vector<fv_physics_cfg> &phys, const fv_numerics_cfg &num,
	       const std::vector<fv_bc_cfg> &bcs)
	    : mesh_(m), batch_((int)phys.size())
	{
		check(fv_disc_create(m.get(), phys.data(), batch_, &num, bcs.data(), (int)bcs.size(), &d_));
	}
	FlowFV(const FlowFV &) = delete;
	FlowFV &operator=(const FlowFV &) = delete;
	~FlowFV() { fv_disc_destroy(d_); }
	/* r += -R(u); dt receives local time steps when gettimesteps (device pointers) */
	void compute_residual(const double *u, double *r, bool gettimesteps, double *dt)
	{
		check(fv_compute_residual(d_, u, r, gettimesteps ? 1 : 0, dt));
	}
	void getGradients(const double *u, double *grads) { check(fv_get_gradients(d_, u, grads, 0)); }
	inline void assemble_jacobian(const double *u, BlockJacobian &A);
	std::vector<double> freestream() const
	{
		std::vector<double> u(4 * (size_t)batch_);
		check(fv_disc_freestream(d_, u.data()));
		return u;
	}
	void synchronize() { check(fv_disc_synchronize(d_)); }
	fv_disc *get() const { return d_; }
	int batch() const { return batch_; }
	const Mesh &mesh() const { return mesh_; }

private:
	Mesh &mesh_;
	int batch_;
	fv_disc *d_ = nullptr;
};

class BlockJacobian {
public:
	BlockJacobian(FlowFV &d, int precision) { check(fv_matrix_create(d.get(), precision, &a_)); }
	BlockJacobian(const BlockJacobian &) = delete;
	BlockJacobian &operator=(const BlockJacobian &) = delete;
	~BlockJacobian() { fv_matrix_destroy(a_); }
	fv_matrix *get() const { return a_; }

private:
	fv_matrix *a_ = nullptr;
};

inline void FlowFV::assemble_jacobian(const double *u, BlockJacobian &A) { check(fv_assemble_jacobian(d_, u, A.get())); }

class SteadyBackwardEulerSolver {
public:
	SteadyBackwardEulerSolver(FlowFV &d, const fv_solver_cfg &cfg) : batch_(d.batch())
	{
		check(fv_solver_create(d.get(), &cfg, &s_));
	}
	SteadyBackwardEulerSolver(const SteadyBackwardEulerSolver &) = delete;
	SteadyBackwardEulerSolver &operator=(const SteadyBackwardEulerSolver &) = delete;
	~SteadyBackwardEulerSolver() { fv_solver_destroy(s_); }
	/* device state, solved in place; throws Numerical_error / Tolerance_error like the reference */
	std::vector<fv_solve_stats> solve(double *d_u)
	{
		std::vector<fv_solve_stats> st(batch_);
		check(fv_solver_solve(s_, d_u, nullptr, st.data()));
		return st;
	}
	std::vector<fv_solve_stats> solve_host(std::vector<double> &u)
	{
		std::vector<fv_solve_stats> st(batch_);
		check(fv_solver_solve_host(s_, u.data(), nullptr, st.data()));
		return st;
	}
	fv_solver *get() const { return s_; }

private:
	int batch_;
	fv_solver *s_ = nullptr;
};

}  // namespace fvg

#endif
