/* ORACLE (test infrastructure only): pointwise ideal-gas physics, inviscid
 * numerical fluxes, ghost-state boundary conditions and the viscous flux,
 * restated from the reference.  Every function is templated on the scalar so
 * the same restatement gives values (double) and Jacobians (Dual<8>).
 *
 * Restated from (reference paths):
 *   src/physics/aphysics_defs.hpp, src/physics/aphysics.cpp
 *   src/spatial/anumericalflux.hpp:175-189, src/spatial/anumericalflux.cpp
 *   src/spatial/abc.cpp
 *   src/physics/viscousphysics.cpp
 *   src/spatial/aspatial.cpp:172-240 (face gradients)
 */
#pragma once
#include <cmath>
#include "orc_dual.hpp"

namespace orc {

constexpr int NV = 4;

// Flux kinds (numbering shared with the product ABI)
enum { F_LLF = 0, F_VANLEER = 1, F_AUSM = 2, F_AUSMPLUS = 3, F_ROE = 4, F_HLL = 5, F_HLLC = 6 };
// BC kinds, reference BCType numbering (src/spatial/abctypes.hpp)
enum { BC_SLIPWALL = 0, BC_FARFIELD = 1, BC_INOUTFLOW = 2, BC_SUBSONIC_INFLOW = 3,
       BC_EXTRAPOLATION = 4, BC_PERIODIC = 5, BC_ISOTHERMALWALL = 6, BC_ADIABATICWALL = 7 };

/* IdealGasPhysics constants: aphysics.cpp:16-22 (Sutherland C = 110.5 K). */
struct Phys {
	double g, Minf, Tinf, Reinf, Pr;
	double sC = 110.5;
};

template <class T> inline T dot2(const T *a, const T *b) { return a[0] * b[0] + a[1] * b[1]; }
template <class T> inline T dot2n(const T *a, const double *n) { return a[0] * n[0] + a[1] * n[1]; }

// ---- aphysics_defs.hpp -------------------------------------------------

/* getVarsFromConserved, aphysics_defs.hpp:27-40 */
template <class T>
inline void vars_from_cons(const Phys &P, const T *uc, const double *n, T *v, T &vn, T &p, T &H)
{
	for (int j = 0; j < 2; j++) v[j] = uc[j + 1] / uc[0];
	vn = dot2n(v, n);
	const T vmag2 = dot2(v, v);
	p = (P.g - 1.0) * (uc[3] - 0.5 * uc[0] * vmag2);
	H = (uc[3] + p) / uc[0];
}

/* getPressureFromConserved, aphysics_defs.hpp:58-64 */
template <class T>
inline T pressure_from_cons(const Phys &P, const T *uc)
{
	return (P.g - 1.0) * (uc[3] - 0.5 * dot2(&uc[1], &uc[1]) / uc[0]);
}

/* getSoundSpeed, aphysics_defs.hpp:134-139 */
template <class T> inline T sound_speed(const Phys &P, const T &rho, const T &p) { return sqrt(P.g * p / rho); }

/* getTemperature, aphysics_defs.hpp:116-121 */
template <class T> inline T temperature(const Phys &P, const T &rho, const T &p) { return p / rho * P.g * P.Minf * P.Minf; }

/* getDirectionalFlux, aphysics_defs.hpp:15-24 */
template <class T>
inline void directional_flux(const T *uc, const double *n, const T &vn, const T &p, T *flux)
{
	flux[0] = vn * uc[0];
	for (int i = 1; i < 3; i++) flux[i] = vn * uc[i] + p * n[i - 1];
	flux[3] = vn * (uc[3] + p);
}

/* getDirectionalFluxFromConserved, aphysics.cpp:32-38 */
template <class T>
inline void directional_flux_from_cons(const Phys &P, const T *u, const double *n, T *flux)
{
	const T vn = dot2n(&u[1], n) / u[0];
	const T p = (P.g - 1.0) * (u[3] - 0.5 * dot2(&u[1], &u[1]) / u[0]);
	directional_flux(u, n, vn, p, flux);
}

/* getEnergyFromPressure, aphysics_defs.hpp:203-208 */
template <class T> inline T energy_from_pressure(const Phys &P, const T &p, const T &d, const T &vmag2)
{
	return p / (P.g - 1.0) + 0.5 * d * vmag2;
}

/* getEnergyFromTemperature, aphysics_defs.hpp:210-216 */
template <class T> inline T energy_from_temperature(const Phys &P, const T &Tt, const T &d, const T &vmag2)
{
	return d * (Tt / (P.g * (P.g - 1.0) * P.Minf * P.Minf) + 0.5 * vmag2);
}

/* getPrimitiveFromConserved, aphysics_defs.hpp:257-268 (in-place safe) */
template <class T>
inline void prim_from_cons(const Phys &P, const T *uc, T *up)
{
	const T rho = uc[0];
	const T p = pressure_from_cons(P, uc);
	const T vx = uc[1] / uc[0], vy = uc[2] / uc[0];
	up[0] = rho; up[1] = vx; up[2] = vy; up[3] = p;
}

/* getPrimitive2FromConserved, aphysics_defs.hpp:270-282 */
template <class T>
inline void prim2_from_cons(const Phys &P, const T *uc, T *up)
{
	const T rho = uc[0];
	const T p = pressure_from_cons(P, uc);
	const T vx = uc[1] / uc[0], vy = uc[2] / uc[0];
	up[0] = rho; up[1] = vx; up[2] = vy; up[3] = temperature(P, uc[0], p);
}

/* getConservedFromPrimitive, aphysics_defs.hpp:284-296 (in-place safe) */
template <class T>
inline void cons_from_prim(const Phys &P, const T *up, T *uc)
{
	const T rhoE = energy_from_pressure(P, up[3], up[0], dot2(&up[1], &up[1]));
	const T r = up[0], m1 = up[0] * up[1], m2 = up[0] * up[2];
	uc[0] = r; uc[1] = m1; uc[2] = m2; uc[3] = rhoE;
}

/* getDeltaPressureFromConserved, aphysics_defs.hpp:67-80 */
inline double delta_pressure(const Phys &P, const double *u, const double *du)
{
	double unew[4];
	for (int i = 0; i < 4; i++) unew[i] = u[i] + du[i];
	double dp = 0;
	for (int i = 2; i < 4; i++)
		dp -= ((u[i] + unew[i]) * (u[0] + unew[0]) / 2.0 * du[i] - (unew[i] * unew[i] + u[i] * u[i]) / 2.0 * du[0]);
	dp = (P.g - 1.0) * (du[3] - 1.0 / (2 * u[0] * unew[0]) * dp);
	return dp;
}

/* getGradTemperature, aphysics_defs.hpp:340-346 */
template <class T>
inline T grad_temperature(const Phys &P, const T &rho, const T &gradrho, const T &p, const T &gradp)
{
	return (gradp * rho - p * gradrho) / (rho * rho) * P.g * P.Minf * P.Minf;
}

/* Sutherland viscosity / Re: getViscosityCoeffFromTemperature, aphysics_defs.hpp:408-413 */
inline double sutherland(const Phys &P, double Tt)
{
	return (1.0 + P.sC / P.Tinf) / (Tt + P.sC / P.Tinf) * std::pow(Tt, 1.5) / P.Reinf;
}
/* For the Jacobian the reference differentiates with
 * d mu/dT = coef*(1.5*T^-1.5*(T+C') - T^1.5)/(T+C')^2
 * (getJacobianSutherlandViscosityWrtConserved, aphysics_defs.hpp:422-437). */
template <int N>
inline Dual<N> sutherland(const Phys &P, const Dual<N> &Tt)
{
	Dual<N> r;
	const double T = Tt.v, Cp = P.sC / P.Tinf;
	r.v = sutherland(P, T);
	const double coef = (1.0 + Cp) / P.Reinf;
	const double dmudT = coef * (1.5 * std::pow(T, -1.5) * (T + Cp) - std::pow(T, 1.5)) / ((T + Cp) * (T + Cp));
	for (int i = 0; i < N; i++) r.d[i] = dmudT * Tt.d[i];
	return r;
}

/* getThermalConductivityFromViscosity, aphysics_defs.hpp:445-448 */
template <class T> inline T conductivity(const Phys &P, const T &mu) { return mu / (P.Minf * P.Minf * (P.g - 1.0) * P.Pr); }

/* getStressTensor, aphysics_defs.hpp:471-488 */
template <class T>
inline void stress_tensor(const T &mu, const T grad[2][4], T stress[2][2])
{
	T ldiv = grad[0][1] + grad[1][2];
	ldiv = ldiv * (2.0 / 3.0 * mu);
	for (int i = 0; i < 2; i++) {
		for (int j = 0; j < 2; j++) stress[i][j] = mu * (grad[i][j + 1] + grad[j][i + 1]);
		stress[i][i] = stress[i][i] - ldiv;
	}
}

/* compute_freestream_state, aphysics.cpp:44-58 */
inline void freestream_state(const Phys &P, double aoa, double *uinf)
{
	uinf[0] = 1.0;
	uinf[1] = std::cos(aoa) * std::cos(0.0);
	uinf[2] = std::sin(aoa) * std::cos(0.0);
	const double pinf = 1.0 / (P.g * P.Minf * P.Minf);
	uinf[3] = pinf / (P.g - 1.0) + 0.5 * 1.0 * 1.0;
}

// ---- numerical fluxes: anumericalflux.cpp ----------------------------------

/* getRoeAverages, anumericalflux.hpp:175-189 */
template <class T>
inline void roe_averages(const Phys &P, const T *ul, const T *ur, const double *n, const T *vi, const T &Hi,
                         const T *vj, const T &Hj, T &Rij, T &rhoij, T *vij, T &vm2ij, T &vnij, T &Hij, T &cij)
{
	Rij = sqrt(ur[0] / ul[0]);
	rhoij = Rij * ul[0];
	for (int i = 0; i < 2; i++) vij[i] = (Rij * vj[i] + vi[i]) / (Rij + 1.0);
	Hij = (Rij * Hj + Hi) / (Rij + 1.0);
	vm2ij = dot2(vij, vij);
	vnij = dot2n(vij, n);
	cij = sqrt((P.g - 1.0) * (Hij - vm2ij * 0.5));
}

/* LLF flux anumericalflux.cpp:41-61; its Jacobian (:66-107) freezes the spectral radius. */
template <class T>
inline void flux_llf(const Phys &P, const T *ul, const T *ur, const double *n, T *flux)
{
	T vi[2], vj[2], vni, vnj, pi, pj, Hi, Hj;
	vars_from_cons(P, ul, n, vi, vni, pi, Hi);
	vars_from_cons(P, ur, n, vj, vnj, pj, Hj);
	const T ci = sound_speed(P, ul[0], pi), cj = sound_speed(P, ur[0], pj);
	const T a = fabs(vni) + ci, b = fabs(vnj) + cj;
	const T eig = frozen(a > b ? a : b);
	T fl[4], fr[4];
	directional_flux_from_cons(P, ul, n, fl);
	directional_flux_from_cons(P, ur, n, fr);
	for (int i = 0; i < 4; i++) flux[i] = 0.5 * (fl[i] + fr[i] - eig * (ur[i] - ul[i]));
}

/* Van Leer flux-vector splitting, anumericalflux.cpp:203-250 (no Jacobian in the reference). */
template <class T>
inline void flux_vanleer(const Phys &P, const T *ul, const T *ur, const double *n, T *flux)
{
	const double g = P.g;
	T fip[4], fjm[4];
	T vi[2], vj[2], vni, vnj, pi, pj, Hi, Hj;
	vars_from_cons(P, ul, n, vi, vni, pi, Hi);
	vars_from_cons(P, ur, n, vj, vnj, pj, Hj);
	const T ci = sound_speed(P, ul[0], pi), cj = sound_speed(P, ur[0], pj);
	const T Mni = vni / ci, Mnj = vnj / cj;
	if (Mni < -1.0) {
		for (int i = 0; i < 4; i++) fip[i] = 0;
	} else if (Mni > 1.0) {
		directional_flux(ul, n, vni, pi, fip);
	} else {
		const T vmags = pow(ul[1] / ul[0], 2.0) + pow(ul[2] / ul[0], 2.0);
		fip[0] = ul[0] * ci * pow(Mni + 1.0, 2.0) / 4.0;
		fip[1] = fip[0] * (ul[1] / ul[0] + n[0] * (2.0 * ci - vni) / g);
		fip[2] = fip[0] * (ul[2] / ul[0] + n[1] * (2.0 * ci - vni) / g);
		fip[3] = fip[0] * ((vmags - vni * vni) / 2.0 + pow((g - 1) * vni + 2.0 * ci, 2.0) / (2 * (g * g - 1)));
	}
	if (Mnj > 1.0) {
		for (int i = 0; i < 4; i++) fjm[i] = 0;
	} else if (Mnj < -1.0) {
		directional_flux(ur, n, vnj, pj, fjm);
	} else {
		const T vmags = pow(ur[1] / ur[0], 2.0) + pow(ur[2] / ur[0], 2.0);
		fjm[0] = -ur[0] * cj * pow(Mnj - 1.0, 2.0) / 4.0;
		fjm[1] = fjm[0] * (ur[1] / ur[0] + n[0] * (-2.0 * cj - vnj) / g);
		fjm[2] = fjm[0] * (ur[2] / ur[0] + n[1] * (-2.0 * cj - vnj) / g);
		fjm[3] = fjm[0] * ((vmags - vnj * vnj) / 2.0 + pow((g - 1) * vnj - 2.0 * cj, 2.0) / (2 * (g * g - 1)));
	}
	for (int i = 0; i < 4; i++) flux[i] = fip[i] + fjm[i];
}

/* Liou-Steffen AUSM, anumericalflux.cpp:265-315; Jacobian :318-472 is its exact derivative. */
template <class T>
inline void flux_ausm(const Phys &P, const T *ul, const T *ur, const double *n, T *flux)
{
	T ML, MR, pL, pR;
	T vi[2], vj[2], vni, vnj, pi, pj, Hi, Hj;
	vars_from_cons(P, ul, n, vi, vni, pi, Hi);
	vars_from_cons(P, ur, n, vj, vnj, pj, Hj);
	const T ci = sound_speed(P, ul[0], pi), cj = sound_speed(P, ur[0], pj);
	const T Mni = vni / ci, Mnj = vnj / cj;
	if (fabs(Mni) <= 1.0) {
		ML = 0.25 * (Mni + 1.0) * (Mni + 1.0);
		pL = ML * pi * (2.0 - Mni);
	} else if (Mni < -1.0) {
		ML = 0; pL = 0;
	} else {
		ML = Mni; pL = pi;
	}
	if (fabs(Mnj) <= 1.0) {
		MR = -0.25 * (Mnj - 1.0) * (Mnj - 1.0);
		pR = -MR * pj * (2.0 + Mnj);
	} else if (Mnj < -1.0) {
		MR = Mnj; pR = pj;
	} else {
		MR = 0; pR = 0;
	}
	const T Mh = ML + MR, ph = pL + pR;
	flux[0] = Mh / 2.0 * (ul[0] * ci + ur[0] * cj) - fabs(Mh) / 2.0 * (ur[0] * cj - ul[0] * ci);
	for (int j = 1; j < 3; j++)
		flux[j] = Mh / 2.0 * (ul[j] * ci + ur[j] * cj) - fabs(Mh) / 2.0 * (ur[j] * cj - ul[j] * ci) + ph * n[j - 1];
	flux[3] = Mh / 2.0 * (ci * (ul[3] + pi) + cj * (ur[3] + pj)) - fabs(Mh) / 2.0 * (cj * (ur[3] + pj) - ci * (ul[3] + pi));
}

/* Liou's AUSM+, anumericalflux.cpp:480-553 (no Jacobian in the reference). */
template <class T>
inline void flux_ausmplus(const Phys &P, const T *ul, const T *ur, const double *n, T *flux)
{
	const double g = P.g;
	T ML, MR, pL, pR;
	T vi[2], vj[2], vni, vnj, pi, pj, Hi, Hj;
	vars_from_cons(P, ul, n, vi, vni, pi, Hi);
	vars_from_cons(P, ur, n, vj, vnj, pj, Hj);
	const T ci = sound_speed(P, ul[0], pi), cj = sound_speed(P, ur[0], pj);
	const T vmag2i = dot2(vi, vi), vmag2j = dot2(vj, vj);
	T csi = sqrt((ci * ci / (g - 1.0) + 0.5 * vmag2i) * 2.0 * (g - 1.0) / (g + 1.0));
	T csj = sqrt((cj * cj / (g - 1.0) + 0.5 * vmag2j) * 2.0 * (g - 1.0) / (g + 1.0));
	const T corri = csi > vni ? csi : vni;
	const T corrj = csj > -vnj ? csj : -vnj;
	csi = csi * csi / corri;
	csj = csj * csj / corrj;
	const T chalf = csi < csj ? csi : csj;
	const T Mni = vni / chalf, Mnj = vnj / chalf;
	if (fabs(Mni) <= 1.0) {
		ML = 0.25 * (Mni + 1.0) * (Mni + 1.0) + 1.0 / 8.0 * (Mni * Mni - 1.0) * (Mni * Mni - 1.0);
		pL = pi * (0.25 * (Mni + 1.0) * (Mni + 1.0) * (2.0 - Mni) + 3.0 / 16 * Mni * (Mni * Mni - 1.0) * (Mni * Mni - 1.0));
	} else if (Mni < -1.0) {
		ML = 0; pL = 0;
	} else {
		ML = Mni; pL = pi;
	}
	if (fabs(Mnj) <= 1.0) {
		MR = -0.25 * (Mnj - 1.0) * (Mnj - 1.0) - 1.0 / 8.0 * (Mnj * Mnj - 1.0) * (Mnj * Mnj - 1.0);
		pR = pj * (0.25 * (Mnj - 1.0) * (Mnj - 1.0) * (2.0 + Mnj) - 3.0 / 16 * Mnj * (Mnj * Mnj - 1.0) * (Mnj * Mnj - 1.0));
	} else if (Mnj < -1.0) {
		MR = Mnj; pR = pj;
	} else {
		MR = 0; pR = 0;
	}
	const T Mh = ML + MR, ph = pL + pR;
	flux[0] = chalf * (Mh / 2.0 * (ul[0] + ur[0]) - fabs(Mh) / 2.0 * (ur[0] - ul[0]));
	for (int j = 1; j < 3; j++)
		flux[j] = chalf * (Mh / 2.0 * (ul[j] + ur[j]) - fabs(Mh) / 2.0 * (ur[j] - ul[j])) + ph * n[j - 1];
	flux[3] = chalf * (Mh / 2.0 * (ul[3] + pi + ur[3] + pj) - fabs(Mh) / 2.0 * ((ur[3] + pj) - (ul[3] + pi)));
}

/* Harten entropy fix as the Roe Jacobian evaluates it (anumericalflux.cpp:803-819):
 * the value is (l^2+d^2)/(2d); the derivative formula is evaluated with the
 * already-fixed eigenvalue in place of the unfixed one. */
inline double harten_fix(double l, double delta) { return (l * l + delta * delta) / (2.0 * delta); }
template <int N>
inline Dual<N> harten_fix(const Dual<N> &l, const Dual<N> &delta)
{
	Dual<N> r;
	r.v = (l.v * l.v + delta.v * delta.v) / (2.0 * delta.v);
	for (int k = 0; k < N; k++)
		r.d[k] = ((2.0 * (r.v * l.d[k] + delta.v * delta.d[k]) * 2.0 * delta.v) -
		          (r.v * r.v + delta.v * delta.v) * 2.0 * delta.d[k]) / (4.0 * delta.v * delta.v);
	return r;
}

/* Roe-Pike flux, anumericalflux.cpp:668-732 (Harten fix eps 1e-4, :664). */
template <class T>
inline void flux_roe(const Phys &P, const T *ul, const T *ur, const double *n, T *flux)
{
	const double fixeps = 1.0e-4;
	T vi[2], vj[2], vni, vnj, pi, pj, Hi, Hj;
	vars_from_cons(P, ul, n, vi, vni, pi, Hi);
	vars_from_cons(P, ur, n, vj, vnj, pj, Hj);
	T Rij, rhoij, vij[2], vm2ij, vnij, Hij, cij;
	roe_averages(P, ul, ur, n, vi, Hi, vj, Hj, Rij, rhoij, vij, vm2ij, vnij, Hij, cij);
	T l[4];
	l[0] = fabs(vnij - cij);
	l[1] = fabs(vnij);
	l[2] = fabs(vnij);
	l[3] = fabs(vnij + cij);
	const T delta = fixeps * cij;
	for (int iv = 0; iv < 4; iv++)
		if (l[iv] < delta) l[iv] = harten_fix(l[iv], delta);
	const T devn = vnj - vni, dep = pj - pi, derho = ur[0] - ul[0];
	T la[4];
	la[0] = l[0] * (dep - rhoij * cij * devn) / (2.0 * cij * cij);
	la[1] = l[1] * (derho - dep / (cij * cij));
	la[2] = l[1] * rhoij;
	la[3] = l[3] * (dep + rhoij * cij * devn) / (2.0 * cij * cij);
	T adu[4];
	adu[0] = la[0];
	adu[1] = la[0] * (vij[0] - cij * n[0]);
	adu[2] = la[0] * (vij[1] - cij * n[1]);
	adu[3] = la[0] * (Hij - cij * vnij);
	adu[0] += la[1];
	adu[1] += la[1] * vij[0] + la[2] * (vj[0] - vi[0] - devn * n[0]);
	adu[2] += la[1] * vij[1] + la[2] * (vj[1] - vi[1] - devn * n[1]);
	adu[3] += la[1] * vm2ij / 2.0 + la[2] * (vij[0] * (vj[0] - vi[0]) + vij[1] * (vj[1] - vi[1]) - vnij * devn);
	adu[0] += la[3];
	adu[1] += la[3] * (vij[0] + cij * n[0]);
	adu[2] += la[3] * (vij[1] + cij * n[1]);
	adu[3] += la[3] * (Hij + cij * vnij);
	T fi[4], fj[4];
	directional_flux(ul, n, vni, pi, fi);
	directional_flux(ur, n, vnj, pj, fj);
	for (int iv = 0; iv < 4; iv++) flux[iv] = 0.5 * (fi[iv] + fj[iv] - adu[iv]);
}

/* HLL with Einfeldt speeds, anumericalflux.cpp:974-1007; the Jacobian (:1013-1061)
 * freezes t1, t2, t3. */
template <class T>
inline void flux_hll(const Phys &P, const T *ul, const T *ur, const double *n, T *flux)
{
	T vi[2], vj[2], vni, vnj, pi, pj, Hi, Hj;
	vars_from_cons(P, ul, n, vi, vni, pi, Hi);
	vars_from_cons(P, ur, n, vj, vnj, pj, Hj);
	const T ci = sound_speed(P, ul[0], pi), cj = sound_speed(P, ur[0], pj);
	T Rij, rhoij, vij[2], vm2ij, vnij, Hij, cij;
	roe_averages(P, ul, ur, n, vi, Hi, vj, Hj, Rij, rhoij, vij, vm2ij, vnij, Hij, cij);
	T sl = vni - ci;
	if (sl > vnij - cij) sl = vnij - cij;
	T sr = vnj + cj;
	if (sr < vnij + cij) sr = vnij + cij;
	const T sr0 = sr > 0 ? T(0.0) : sr;
	const T sl0 = sl > 0 ? T(0.0) : sl;
	const T t1 = frozen((sr0 - sl0) / (sr - sl));
	const T t2 = frozen(1.0 - (sr0 - sl0) / (sr - sl));
	const T t3 = frozen(0.5 * (sr * fabs(sl) - sl * fabs(sr)) / (sr - sl));
	flux[0] = t1 * vnj * ur[0] + t2 * vni * ul[0] - t3 * (ur[0] - ul[0]);
	flux[1] = t1 * (vnj * ur[1] + pj * n[0]) + t2 * (vni * ul[1] + pi * n[0]) - t3 * (ur[1] - ul[1]);
	flux[2] = t1 * (vnj * ur[2] + pj * n[1]) + t2 * (vni * ul[2] + pi * n[1]) - t3 * (ur[2] - ul[2]);
	flux[3] = t1 * (vnj * ur[0] * Hj) + t2 * (vni * ul[0] * Hi) - t3 * (ur[3] - ul[3]);
}

/* HLLC star state, anumericalflux.cpp:1071-1081 */
template <class T>
inline void hllc_star(const T *u, const double *n, const T &vn, const T &p, const T &ss, const T &sm, T *us)
{
	const T pstar = u[0] * (vn - ss) * (vn - sm) + p;
	us[0] = u[0] * (ss - vn) / (ss - sm);
	us[1] = ((ss - vn) * u[1] + (pstar - p) * n[0]) / (ss - sm);
	us[2] = ((ss - vn) * u[2] + (pstar - p) * n[1]) / (ss - sm);
	us[3] = ((ss - vn) * u[3] - p * vn + pstar * sm) / (ss - sm);
}

/* HLLC flux, anumericalflux.cpp:1176-1228; Jacobian :1231-1397 is its exact derivative. */
template <class T>
inline void flux_hllc(const Phys &P, const T *ul, const T *ur, const double *n, T *flux)
{
	T vi[2], vj[2], vni, vnj, pi, pj, Hi, Hj;
	vars_from_cons(P, ul, n, vi, vni, pi, Hi);
	vars_from_cons(P, ur, n, vj, vnj, pj, Hj);
	const T ci = sound_speed(P, ul[0], pi), cj = sound_speed(P, ur[0], pj);
	T Rij, rhoij, vij[2], vm2ij, vnij, Hij, cij;
	roe_averages(P, ul, ur, n, vi, Hi, vj, Hj, Rij, rhoij, vij, vm2ij, vnij, Hij, cij);
	T sl = vni - ci;
	if (sl > vnij - cij) sl = vnij - cij;
	T sr = vnj + cj;
	if (sr < vnij + cij) sr = vnij + cij;
	const T sm = (ur[0] * vnj * (sr - vnj) - ul[0] * vni * (sl - vni) + pi - pj) / (ur[0] * (sr - vnj) - ul[0] * (sl - vni));
	if (sl > 0) {
		directional_flux(ul, n, vni, pi, flux);
	} else if (sl <= 0 && sm > 0) {
		directional_flux(ul, n, vni, pi, flux);
		T us[4];
		hllc_star(ul, n, vni, pi, sl, sm, us);
		for (int i = 0; i < 4; i++) flux[i] += sl * (us[i] - ul[i]);
	} else if (sm <= 0 && sr >= 0) {
		directional_flux(ur, n, vnj, pj, flux);
		T us[4];
		hllc_star(ur, n, vnj, pj, sr, sm, us);
		for (int i = 0; i < 4; i++) flux[i] += sr * (us[i] - ur[i]);
	} else {
		directional_flux(ur, n, vnj, pj, flux);
	}
}

template <class T>
inline int numerical_flux(int kind, const Phys &P, const T *ul, const T *ur, const double *n, T *flux)
{
	switch (kind) {
	case F_LLF: flux_llf(P, ul, ur, n, flux); return 0;
	case F_VANLEER: flux_vanleer(P, ul, ur, n, flux); return 0;
	case F_AUSM: flux_ausm(P, ul, ur, n, flux); return 0;
	case F_AUSMPLUS: flux_ausmplus(P, ul, ur, n, flux); return 0;
	case F_ROE: flux_roe(P, ul, ur, n, flux); return 0;
	case F_HLL: flux_hll(P, ul, ur, n, flux); return 0;
	case F_HLLC: flux_hllc(P, ul, ur, n, flux); return 0;
	}
	return 1;
}

// ---- boundary conditions: abc.cpp -----------------------------------------

struct BCSpec {
	int type;
	double vals[2];
};

/* computeGhostState of each BC class (abc.cpp:49,152,194,218,272,354,417).
 * jac_mode selects the branch rules of computeGhostStateAndJacobian, which
 * differ for the in/outflow BC (subsonic test "<= 1" and p_inf from u_inf). */
template <class T>
inline int ghost_state(const Phys &P, const BCSpec &bc, const double *uinf, const T *ins, const double *n, T *gs,
                       bool jac_mode = false)
{
	switch (bc.type) {
	case BC_INOUTFLOW: {
		const T vni = dot2n(&ins[1], n) / ins[0];
		const T ci = sound_speed(P, ins[0], pressure_from_cons(P, ins));
		const T Mni = vni / ci;
		const double pinf = jac_mode ? value(pressure_from_cons(P, uinf)) : 1.0 / (P.g * P.Minf * P.Minf);
		const bool subsonic = jac_mode ? (Mni <= 1.0) : (Mni < 1.0);
		if (Mni <= 0) {
			for (int i = 0; i < 4; i++) gs[i] = uinf[i];
		} else if (subsonic) {
			gs[0] = ins[0]; gs[1] = ins[1]; gs[2] = ins[2];
			gs[3] = energy_from_pressure(P, T(pinf), ins[0], dot2(&ins[1], &ins[1]) / (ins[0] * ins[0]));
		} else {
			for (int i = 0; i < 4; i++) gs[i] = ins[i];
		}
		return 0;
	}
	case BC_SUBSONIC_INFLOW: {
		const double g = P.g, ptotal = bc.vals[0], ttotal = bc.vals[1];
		const T ci = sound_speed(P, ins[0], pressure_from_cons(P, ins));
		const T Rminus = dot2n(&ins[1], n) / ins[0] - ci / (2 * g - 1.0);
		const T co2 = ci * ci + (g - 1.0) / 2.0 * dot2(&ins[1], &ins[1]) / (ins[0] * ins[0]);
		const T q = sqrt((g + 1) * co2 / ((g - 1) * Rminus * Rminus) - (g - 1) / 2.0);
		const T cg = -Rminus * (g - 1) / (g + 1) * (1.0 + q);
		const T tg = ttotal * cg * cg / co2;
		const T pg = ptotal * pow(tg / ttotal, g / (g - 1.0));
		gs[0] = g * P.Minf * P.Minf * pg / tg;
		const T vgmag = sqrt(2.0 / (g - 1.0) * (co2 - cg * cg));
		gs[1] = gs[0] * (vgmag * n[0]);
		gs[2] = gs[0] * (vgmag * n[1]);
		gs[3] = energy_from_pressure(P, pg, gs[0], vgmag * vgmag);
		return 0;
	}
	case BC_FARFIELD:
		for (int i = 0; i < 4; i++) gs[i] = uinf[i];
		return 0;
	case BC_SLIPWALL: {
		const T vni = dot2n(&ins[1], n) / ins[0];
		gs[0] = ins[0];
		for (int i = 1; i < 3; i++) gs[i] = ins[i] - 2.0 * vni * n[i - 1] * ins[0];
		gs[3] = ins[3];
		return 0;
	}
	case BC_ADIABATICWALL: {
		const double tv = bc.vals[0];
		const T tm = tv * ins[0];
		gs[0] = ins[0];
		gs[1] = 2.0 * tm * n[1] - ins[1];
		gs[2] = -2.0 * tm * n[0] - ins[2];
		gs[3] = ins[3];
		return 0;
	}
	case BC_ISOTHERMALWALL: {
		const double tv = bc.vals[0], twall = bc.vals[1];
		if (jac_mode) {
			/* computeGhostStateAndJacobian's ghost value, abc.cpp:360-378 */
			const T tm = tv * ins[0];
			gs[0] = ins[0];
			gs[1] = 2.0 * tm * n[1] - ins[1];
			gs[2] = -2.0 * tm * n[0] - ins[2];
			const T vmag2 = dot2(&gs[1], &gs[1]) / (ins[0] * ins[0]);
			gs[3] = energy_from_temperature(P, T(twall), ins[0], vmag2);
			return 0;
		}
		const T p = pressure_from_cons(P, ins);
		const T gtemp = 2.0 * twall - temperature(P, ins[0], p);
		gs[0] = ins[0];
		gs[1] = gs[0] * (2.0 * tv * n[1] - ins[1] / ins[0]);
		gs[2] = gs[0] * (-2.0 * tv * n[0] - ins[2] / ins[0]);
		const T vmag2 = dot2(&gs[1], &gs[1]) / (gs[0] * gs[0]);
		gs[3] = energy_from_temperature(P, gtemp, gs[0], vmag2);
		return 0;
	}
	case BC_EXTRAPOLATION:
		for (int k = 0; k < 4; k++) gs[k] = ins[k];
		return 0;
	}
	return 1;
}

/* computeGhostStateAndJacobian (row-major dgs = d ghost / d interior).
 * All but the isothermal wall are exact derivatives of the jac_mode ghost
 * state; the isothermal wall follows the reference's own formula
 * (abc.cpp:357-398, marked FIXME there).  The subsonic inflow BC has no
 * Jacobian in the reference (abc.cpp:179-185 exits); returns 2. */
inline int ghost_jacobian(const Phys &P, const BCSpec &bc, const double *uinf, const double *ins, const double *n,
                          double *gs, double *dgs)
{
	if (bc.type == BC_SUBSONIC_INFLOW) return 2;
	for (int k = 0; k < 16; k++) dgs[k] = 0;
	if (bc.type == BC_ISOTHERMALWALL) {
		ghost_state(P, bc, uinf, ins, n, gs, true);
		const double tv = bc.vals[0], twall = bc.vals[1];
		dgs[0] = 1.0;
		dgs[4 + 0] = 2.0 * tv * n[1]; dgs[4 + 1] = -1.0;
		dgs[8 + 0] = -2.0 * tv * n[0]; dgs[8 + 2] = -1.0;
		const double vmag2 = dot2(&gs[1], &gs[1]) / (ins[0] * ins[0]);
		double dvm[4];
		dvm[0] = -2.0 * dot2(&gs[1], &gs[1]) / (ins[0] * ins[0] * ins[0]);
		for (int i = 1; i < 3; i++) dvm[i] = 1.0 / (ins[0] * ins[0]) * gs[i] * (-1.0);
		dvm[3] = 0;
		/* getJacobianEnergyFromJacobiansTemperatureVmag2 with dT = 0 */
		const double coeff = 1.0 / (P.g * (P.g - 1.0) * P.Minf * P.Minf);
		dgs[12 + 0] += coeff * (twall + ins[0] * 0.0) + 0.5 * (vmag2 + ins[0] * dvm[0]);
		for (int i = 1; i < 4; i++) dgs[12 + i] += ins[0] * (coeff * 0.0 + 0.5 * dvm[i]);
		return 0;
	}
	Dual<4> di[4], dg[4];
	for (int i = 0; i < 4; i++) { di[i] = Dual<4>(ins[i]); di[i].d[i] = 1.0; }
	if (ghost_state(P, bc, uinf, di, n, dg, true)) return 1;
	for (int i = 0; i < 4; i++) {
		gs[i] = dg[i].v;
		for (int k = 0; k < 4; k++) dgs[i * 4 + k] = dg[i].d[k];
	}
	return 0;
}

// ---- viscous flux: viscousphysics.cpp, aspatial.cpp ---------------------------

/* getFaceGradient_modifiedAverage, aspatial.cpp:172-205 (grads NDIM x NVARS row-major) */
inline void face_gradient_modavg(const double *rcl, const double *rcr, const double *ucl, const double *ucr,
                                 const double *gradl, const double *gradr, double grad[2][4])
{
	double dr[2], dist = 0;
	for (int i = 0; i < 2; i++) { dr[i] = rcr[i] - rcl[i]; dist += dr[i] * dr[i]; }
	dist = std::sqrt(dist);
	for (int i = 0; i < 2; i++) dr[i] /= dist;
	for (int i = 0; i < 4; i++) {
		double davg[2];
		for (int j = 0; j < 2; j++) davg[j] = 0.5 * (gradl[j * 4 + i] + gradr[j * 4 + i]);
		const double corr = (ucr[i] - ucl[i]) / dist;
		const double ddr = davg[0] * dr[0] + davg[1] * dr[1];
		for (int j = 0; j < 2; j++) grad[j][i] = davg[j] - ddr * dr[j] + corr * dr[j];
	}
}

/* getPrimitive2StatesAndGradients, viscousphysics.cpp:15-63; in: conserved
 * states and primitive gradients (NDIM x NVARS); out: prim-2 states and grads. */
inline void prim2_states_grads(const Phys &P, bool order2, const double *ucl, const double *ucr, const double *gradl,
                               const double *gradr, double *uctl, double *uctr, double *gtl, double *gtr)
{
	if (order2) {
		prim_from_cons(P, ucl, uctl);
		prim_from_cons(P, ucr, uctr);
		for (int k = 0; k < 8; k++) { gtl[k] = gradl[k]; gtr[k] = gradr[k]; }
		for (int j = 0; j < 2; j++) {
			gtl[j * 4 + 3] = grad_temperature(P, uctl[0], gradl[j * 4], uctl[3], gradl[j * 4 + 3]);
			gtr[j * 4 + 3] = grad_temperature(P, uctr[0], gradr[j * 4], uctr[3], gradr[j * 4 + 3]);
		}
		uctl[3] = temperature(P, uctl[0], uctl[3]);
		uctr[3] = temperature(P, uctr[0], uctr[3]);
	} else {
		prim2_from_cons(P, ucl, uctl);
		prim2_from_cons(P, ucr, uctr);
	}
}

/* computeViscousFlux, viscousphysics.cpp:71-122 */
template <class T>
inline void viscous_flux(const Phys &P, bool constvisc, const double *n, const T grad[2][4], const T *ul, const T *ur,
                         T *vflux)
{
	T muRe;
	if (constvisc)
		muRe = T(1.0 / P.Reinf);
	else
		muRe = 0.5 * (sutherland(P, temperature(P, ul[0], pressure_from_cons(P, ul))) +
		              sutherland(P, temperature(P, ur[0], pressure_from_cons(P, ur))));
	const T kdiff = conductivity(P, muRe);
	T stress[2][2];
	stress_tensor(muRe, grad, stress);
	vflux[0] = 0;
	for (int i = 0; i < 2; i++) {
		vflux[i + 1] = 0;
		for (int j = 0; j < 2; j++) vflux[i + 1] -= stress[i][j] * n[j];
	}
	T vavg[2];
	for (int j = 0; j < 2; j++) vavg[j] = 0.5 * (ul[j + 1] / ul[0] + ur[j + 1] / ur[0]);
	vflux[3] = 0;
	for (int i = 0; i < 2; i++) {
		T comp = 0;
		for (int j = 0; j < 2; j++) comp += stress[i][j] * vavg[j];
		comp += kdiff * grad[i][3];
		vflux[3] -= comp * n[i];
	}
}

/* The viscous flux Jacobian of the reference (flow_spatial.cpp:397-446,
 * aspatial.cpp:207-240, viscousphysics.cpp:125-245) is the derivative of the
 * viscous flux evaluated with the thin-layer face gradient
 * (q_R - q_L)/d * t of primitive-2 variables of the cell-centred states. */
template <class T>
inline void viscous_flux_thinlayer(const Phys &P, bool constvisc, const double *n, const double *rcl,
                                   const double *rcr, const T *ul, const T *ur, T *vflux)
{
	T upl[4], upr[4];
	prim2_from_cons(P, ul, upl);
	prim2_from_cons(P, ur, upr);
	double dr[2], dist = 0;
	for (int i = 0; i < 2; i++) { dr[i] = rcr[i] - rcl[i]; dist += dr[i] * dr[i]; }
	dist = std::sqrt(dist);
	for (int i = 0; i < 2; i++) dr[i] /= dist;
	T grad[2][4];
	for (int i = 0; i < 4; i++) {
		const T corr = (upr[i] - upl[i]) / dist;
		for (int j = 0; j < 2; j++) grad[j][i] = corr * dr[j];
	}
	viscous_flux(P, constvisc, n, grad, ul, ur, vflux);
}

}  // namespace orc
