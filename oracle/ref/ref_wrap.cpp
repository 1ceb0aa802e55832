/* Test-only C shim over the reference's own pointwise physics.
 *
 * This translation unit is compiled against the reference sources where they
 * lie (see build_ref.sh); it exists only so that tests can call the
 * reference's compiled numerical fluxes, flux Jacobians, ghost-state boundary
 * conditions and viscous fluxes on arbitrary states and compare them with the
 * oracle's restatement.  Nothing in the product links against it.
 *
 * Reference files compiled through this shim:
 *   src/physics/aphysics.cpp        (IdealGasPhysics)
 *   src/physics/viscousphysics.cpp  (getPrimitive2StatesAndGradients,
 *                                    computeViscousFlux, computeViscousFluxJacobian)
 *   src/spatial/anumericalflux.cpp  (LLF, VanLeer, AUSM, AUSM+, Roe, HLL, HLLC)
 *   src/spatial/abc.cpp             (ghost-state BCs and their Jacobians)
 */
#include <cstdio>
#include <cstring>
#include "physics/aphysics.cpp"
#include "physics/viscousphysics.cpp"
#include "spatial/anumericalflux.cpp"
#include "spatial/abc.cpp"

namespace fvens {
// The abstract bases are only instantiated implicitly by the reference's own
// library build; name them here so their destructors are emitted.
template class InviscidFlux<double, double>;
template class FlowBC<double, double>;
}

using namespace fvens;

namespace {
// phys = {gamma, Minf, Tinf, Reinf, Pr}
IdealGasPhysics<double> make_phys(const double *phys)
{
	return IdealGasPhysics<double>(phys[0], phys[1], phys[2], phys[3], phys[4]);
}

// Flux kinds, numbered as in the build's C ABI:
// 0 LLF, 1 VANLEER, 2 AUSM, 3 AUSMPLUS, 4 ROE, 5 HLL, 6 HLLC
InviscidFlux<double> *make_flux(int kind, const IdealGasPhysics<double> *p)
{
	switch (kind) {
	case 0: return new LocalLaxFriedrichsFlux<double>(p);
	case 1: return new VanLeerFlux<double>(p);
	case 2: return new AUSMFlux<double>(p);
	case 3: return new AUSMPlusFlux<double>(p);
	case 4: return new RoeFlux<double>(p);
	case 5: return new HLLFlux<double>(p);
	case 6: return new HLLCFlux<double>(p);
	default: return nullptr;
	}
}

// BC types use the reference's BCType numbering.
FlowBC<double> *make_bc(int type, const IdealGasPhysics<double> &p, const double *vals,
                        const std::array<double, NVARS> &uinf)
{
	switch (type) {
	case SLIP_WALL_BC: return new Slipwall<double>(0, p);
	case FARFIELD_BC: return new Farfield<double>(0, p, uinf);
	case INFLOW_OUTFLOW_BC: return new InOutFlow<double>(0, p, uinf);
	case SUBSONIC_INFLOW_BC: return new InFlow<double>(0, p, vals[0], vals[1]);
	case EXTRAPOLATION_BC: return new Extrapolation<double>(0, p);
	case ISOTHERMAL_WALL_BC: return new Isothermalwall2D<double>(0, p, vals[0], vals[1]);
	case ADIABATIC_WALL_BC: return new Adiabaticwall2D<double>(0, p, vals[0]);
	default: return nullptr;
	}
}
}  // namespace

extern "C" {

int ref_freestream(const double *phys, double aoa, double *uinf)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	const std::array<double, NVARS> u = p.compute_freestream_state(aoa);
	for (int i = 0; i < NVARS; i++) uinf[i] = u[i];
	return 0;
}

int ref_flux(int kind, const double *phys, const double *ul, const double *ur, const double *n,
             double *flux)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	InviscidFlux<double> *f = make_flux(kind, &p);
	if (!f) return 1;
	f->get_flux(ul, ur, n, flux);
	delete f;
	return 0;
}

/* Returns 0 on success, 2 when the reference does not implement the Jacobian
 * (VanLeer throws, AUSM+ prints a message and leaves the outputs untouched). */
int ref_flux_jacobian(int kind, const double *phys, const double *ul, const double *ur,
                      const double *n, double *dfdl, double *dfdr)
{
	if (kind == 1 || kind == 3) return 2;
	const IdealGasPhysics<double> p = make_phys(phys);
	InviscidFlux<double> *f = make_flux(kind, &p);
	if (!f) return 1;
	f->get_jacobian(ul, ur, n, dfdl, dfdr);
	delete f;
	return 0;
}

int ref_bc_ghost(int type, const double *phys, double aoa, const double *vals, const double *ins,
                 const double *n, double *gs)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	const std::array<double, NVARS> uinf = p.compute_freestream_state(aoa);
	FlowBC<double> *bc = make_bc(type, p, vals, uinf);
	if (!bc) return 1;
	bc->computeGhostState(ins, n, gs);
	delete bc;
	return 0;
}

/* Returns 2 for the subsonic-inflow BC, whose reference Jacobian exits the process. */
int ref_bc_ghost_jacobian(int type, const double *phys, double aoa, const double *vals,
                          const double *ins, const double *n, double *gs, double *dgs)
{
	if (type == SUBSONIC_INFLOW_BC) return 2;
	const IdealGasPhysics<double> p = make_phys(phys);
	const std::array<double, NVARS> uinf = p.compute_freestream_state(aoa);
	FlowBC<double> *bc = make_bc(type, p, vals, uinf);
	if (!bc) return 1;
	bc->computeGhostStateAndJacobian(ins, n, gs, dgs);
	delete bc;
	return 0;
}

/* Primitive-2 (rho,u,v,T) states and gradients from conserved cell states and
 * primitive (rho,u,v,p) gradients; grads are NDIM x NVARS row-major. */
int ref_prim2_states_gradients(int order2, const double *phys, const double *ucl,
                               const double *ucr, const double *gradl, const double *gradr,
                               double *uctl, double *uctr, double *gradtl, double *gradtr)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	if (order2)
		getPrimitive2StatesAndGradients<double, NDIM, true>(p, ucl, ucr, gradl, gradr, uctl, uctr,
		                                                    gradtl, gradtr);
	else
		getPrimitive2StatesAndGradients<double, NDIM, false>(p, ucl, ucr, gradl, gradr, uctl, uctr,
		                                                     gradtl, gradtr);
	return 0;
}

/* Viscous flux from a face gradient of primitive-2 variables (NDIM x NVARS). */
int ref_viscous_flux(int constvisc, const double *phys, const double *n, const double *grad,
                     const double *ul, const double *ur, double *vflux)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	double g[NDIM][NVARS];
	std::memcpy(g, grad, sizeof(g));
	if (constvisc)
		computeViscousFlux<double, NDIM, NVARS, true>(p, n, g, ul, ur, vflux);
	else
		computeViscousFlux<double, NDIM, NVARS, false>(p, n, g, ul, ur, vflux);
	return 0;
}

/* Viscous flux Jacobian given the face gradient and its Jacobians
 * (NDIM x NVARS x NVARS each); outputs are ADDED to dvfi/dvfj. */
int ref_viscous_flux_jacobian(int constvisc, const double *phys, const double *n,
                              const double *ul, const double *ur, const double *grad,
                              const double *dgradl, const double *dgradr, double *dvfi,
                              double *dvfj)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	double g[NDIM][NVARS], dgl[NDIM][NVARS][NVARS], dgr[NDIM][NVARS][NVARS];
	std::memcpy(g, grad, sizeof(g));
	std::memcpy(dgl, dgradl, sizeof(dgl));
	std::memcpy(dgr, dgradr, sizeof(dgr));
	if (constvisc)
		computeViscousFluxJacobian<double, NDIM, NVARS, true>(p, n, ul, ur, g, dgl, dgr, dvfi, dvfj);
	else
		computeViscousFluxJacobian<double, NDIM, NVARS, false>(p, n, ul, ur, g, dgl, dgr, dvfi,
		                                                       dvfj);
	return 0;
}

/* Primitive-2 Jacobian w.r.t. conserved (added to jac, row-major 4x4). */
int ref_prim2_jacobian(const double *phys, const double *uc, double *up2, double *jac)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	p.getPrimitive2FromConserved(uc, up2);
	p.getJacobianPrimitive2WrtConserved(uc, jac);
	return 0;
}

/* Pointwise conversions used by the residual driver. */
int ref_prim_from_cons(const double *phys, const double *uc, double *up)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	p.getPrimitiveFromConserved(uc, up);
	return 0;
}

int ref_cons_from_prim(const double *phys, const double *up, double *uc)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	p.getConservedFromPrimitive(up, uc);
	return 0;
}

double ref_delta_pressure(const double *phys, const double *u, const double *du)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	return p.getDeltaPressureFromConserved(u, du);
}

double ref_viscosity(const double *phys, const double *uc)
{
	const IdealGasPhysics<double> p = make_phys(phys);
	return p.getViscosityCoeffFromConserved(uc);
}

}  // extern "C"
