// Device-side pointwise physics for the GB300 hot path: ideal-gas relations,
// the seven inviscid numerical fluxes, ghost-state boundary conditions and the
// modified-average / thin-layer viscous fluxes.
//
// Everything is templated on the arithmetic type T so one definition serves
//   * the FP64 residual (T = double),
//   * Jacobian blocks by forward-mode differentiation (T = Dual<float|double, 8>).
// The formulas follow the reference's pointwise physics
// (src/physics/aphysics_defs.hpp, src/spatial/anumericalflux.cpp,
//  src/spatial/abc.cpp, src/physics/viscousphysics.cpp) but are arranged for
// a GPU with slow FP64: face states carry primitive and conserved forms
// together so velocities are never re-derived by division, and each state's
// reciprocal density is computed once.
//
// Reference Jacobian conventions reproduced here:
//   * LLF linearises with a frozen spectral radius (anumericalflux.cpp:66-107);
//   * HLL freezes t1, t2, t3 (anumericalflux.cpp:1013-1061);
//   * Roe's entropy-fix derivative is evaluated with the already-fixed
//     eigenvalue (anumericalflux.cpp:803-819);
//   * the Sutherland derivative in the viscous Jacobian uses T^-1.5 where the
//     exact derivative has T^0.5 (aphysics_defs.hpp:422-437);
//   * d|x|/dx = +1 at x = 0.
#pragma once
#include <cuda_runtime.h>

namespace fvg {

// numbering shared with the C ABI (include/fvens_gb300.h)
enum { FLUX_LLF = 0, FLUX_VANLEER = 1, FLUX_AUSM = 2, FLUX_AUSMPLUS = 3, FLUX_ROE = 4, FLUX_HLL = 5, FLUX_HLLC = 6 };
enum { BC_SLIPWALL = 0, BC_FARFIELD = 1, BC_INOUTFLOW = 2, BC_SUBSONIC_INFLOW = 3, BC_EXTRAPOLATION = 4,
       BC_PERIODIC = 5, BC_ISOTHERMALWALL = 6, BC_ADIABATICWALL = 7 };

#define FV_HD __host__ __device__ __forceinline__

// ---------------------------------------------------------------------------
// forward-mode dual numbers
template <class R, int N>
struct Dual {
	R v;
	R d[N];
};

template <class R, int N> FV_HD Dual<R, N> dconst(R x) { Dual<R, N> r; r.v = x; for (int i = 0; i < N; i++) r.d[i] = 0; return r; }
template <class R, int N> FV_HD Dual<R, N> operator+(const Dual<R, N> &a, const Dual<R, N> &b) { Dual<R, N> r; r.v = a.v + b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] + b.d[i]; return r; }
template <class R, int N> FV_HD Dual<R, N> operator-(const Dual<R, N> &a, const Dual<R, N> &b) { Dual<R, N> r; r.v = a.v - b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] - b.d[i]; return r; }
template <class R, int N> FV_HD Dual<R, N> operator-(const Dual<R, N> &a) { Dual<R, N> r; r.v = -a.v; for (int i = 0; i < N; i++) r.d[i] = -a.d[i]; return r; }
template <class R, int N> FV_HD Dual<R, N> operator*(const Dual<R, N> &a, const Dual<R, N> &b) { Dual<R, N> r; r.v = a.v * b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <class R, int N> FV_HD Dual<R, N> operator/(const Dual<R, N> &a, const Dual<R, N> &b)
{
	Dual<R, N> r; const R ib = R(1) / b.v; r.v = a.v * ib;
	for (int i = 0; i < N; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
	return r;
}
template <class R, int N> FV_HD Dual<R, N> operator+(const Dual<R, N> &a, R b) { Dual<R, N> r = a; r.v += b; return r; }
template <class R, int N> FV_HD Dual<R, N> operator+(R b, const Dual<R, N> &a) { Dual<R, N> r = a; r.v += b; return r; }
template <class R, int N> FV_HD Dual<R, N> operator-(const Dual<R, N> &a, R b) { Dual<R, N> r = a; r.v -= b; return r; }
template <class R, int N> FV_HD Dual<R, N> operator-(R b, const Dual<R, N> &a) { Dual<R, N> r = -a; r.v += b; return r; }
template <class R, int N> FV_HD Dual<R, N> operator*(const Dual<R, N> &a, R b) { Dual<R, N> r; r.v = a.v * b; for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b; return r; }
template <class R, int N> FV_HD Dual<R, N> operator*(R b, const Dual<R, N> &a) { return a * b; }
template <class R, int N> FV_HD Dual<R, N> operator/(const Dual<R, N> &a, R b) { return a * (R(1) / b); }
template <class R, int N> FV_HD Dual<R, N> operator/(R a, const Dual<R, N> &b)
{
	Dual<R, N> r; const R ib = R(1) / b.v; r.v = a * ib;
	for (int i = 0; i < N; i++) r.d[i] = -r.v * b.d[i] * ib;
	return r;
}
template <class R, int N> FV_HD bool operator<(const Dual<R, N> &a, const Dual<R, N> &b) { return a.v < b.v; }
template <class R, int N> FV_HD bool operator>(const Dual<R, N> &a, const Dual<R, N> &b) { return a.v > b.v; }
template <class R, int N> FV_HD bool operator<=(const Dual<R, N> &a, const Dual<R, N> &b) { return a.v <= b.v; }
template <class R, int N> FV_HD bool operator>=(const Dual<R, N> &a, const Dual<R, N> &b) { return a.v >= b.v; }
template <class R, int N> FV_HD bool operator<(const Dual<R, N> &a, R b) { return a.v < b; }
template <class R, int N> FV_HD bool operator>(const Dual<R, N> &a, R b) { return a.v > b; }
template <class R, int N> FV_HD bool operator<=(const Dual<R, N> &a, R b) { return a.v <= b; }
template <class R, int N> FV_HD bool operator>=(const Dual<R, N> &a, R b) { return a.v >= b; }

// scalar traits ---------------------------------------------------------------
template <class T> struct Real { typedef T type; };
template <class R, int N> struct Real<Dual<R, N>> { typedef R type; };

FV_HD double vsqrt(double x) { return sqrt(x); }
FV_HD float vsqrt(float x) { return sqrtf(x); }
template <class R, int N> FV_HD Dual<R, N> vsqrt(const Dual<R, N> &a)
{
	Dual<R, N> r; r.v = vsqrt(a.v); const R h = R(0.5) / r.v;
	for (int i = 0; i < N; i++) r.d[i] = a.d[i] * h;
	return r;
}
FV_HD double vabs(double x) { return fabs(x); }
FV_HD float vabs(float x) { return fabsf(x); }
template <class R, int N> FV_HD Dual<R, N> vabs(const Dual<R, N> &a) { return a.v >= R(0) ? a : -a; }
FV_HD double vpow(double x, double e) { return pow(x, e); }
FV_HD float vpow(float x, float e) { return powf(x, e); }
template <class R, int N> FV_HD Dual<R, N> vpow(const Dual<R, N> &a, R e)
{
	Dual<R, N> r; r.v = vpow(a.v, e); const R dr = e * vpow(a.v, e - R(1));
	for (int i = 0; i < N; i++) r.d[i] = a.d[i] * dr;
	return r;
}
FV_HD double value(double x) { return x; }
FV_HD float value(float x) { return x; }
template <class R, int N> FV_HD R value(const Dual<R, N> &x) { return x.v; }
/* stop-gradient: value with zero derivative */
FV_HD double frozen(double x) { return x; }
FV_HD float frozen(float x) { return x; }
template <class R, int N> FV_HD Dual<R, N> frozen(const Dual<R, N> &x) { return dconst<R, N>(x.v); }
template <class T> FV_HD T tmax(const T &a, const T &b) { return a > b ? a : b; }
template <class T> FV_HD T tmin(const T &a, const T &b) { return a < b ? a : b; }
template <class T> struct Lift;
template <> struct Lift<double> { static FV_HD double f(double x) { return x; } };
template <> struct Lift<float> { static FV_HD float f(float x) { return x; } };
template <class R, int N> struct Lift<Dual<R, N>> { static FV_HD Dual<R, N> f(R x) { return dconst<R, N>(x); } };
#define TL(x) Lift<T>::f((typename Real<T>::type)(x))

// ---------------------------------------------------------------------------
/* Per-condition physical parameters (IdealGasPhysics, aphysics.hpp; freestream
 * from compute_freestream_state, aphysics.cpp:44-58). */
struct Phys {
	double g, gm1, igm1;     // gamma, gamma-1, 1/(gamma-1)
	double Minf, Tinf, Reinf, Pr;
	double tcoef;            // gamma*Minf^2 : T = tcoef p / rho
	double pinf;             // 1/(gamma Minf^2)
	double sutC;             // Sutherland constant / Tinf
	double sutK;             // (1 + sutC)/Reinf
	double kcoef;            // 1/(Minf^2 (gamma-1) Pr): k = mu * kcoef
	double ivisc;            // 1/Reinf (constant viscosity)
	double uinf[4];
	double aoa;
	double pinf_cons;        // p from the conserved freestream (BC Jacobian branch)
};

/* A thermodynamic state carried in primitive and conserved form:
 * r density, u,v velocity, p pressure, E total energy per volume, ir = 1/r. */
template <class T>
struct St {
	T r, u, v, p, E, ir;
};

template <class T, class PP>
FV_HD St<T> st_from_cons(const PP &P, const T *uc)
{
	typedef typename Real<T>::type R;
	St<T> s;
	s.r = uc[0];
	s.ir = R(1) / uc[0];
	s.u = uc[1] * s.ir;
	s.v = uc[2] * s.ir;
	s.E = uc[3];
	s.p = R(P.gm1) * (uc[3] - R(0.5) * (uc[1] * s.u + uc[2] * s.v));
	return s;
}

template <class T, class PP>
FV_HD St<T> st_from_prim(const PP &P, const T *up)
{
	typedef typename Real<T>::type R;
	St<T> s;
	s.r = up[0]; s.u = up[1]; s.v = up[2]; s.p = up[3];
	s.ir = R(1) / up[0];
	s.E = s.p * R(P.igm1) + R(0.5) * s.r * (s.u * s.u + s.v * s.v);
	return s;
}

/* st_from_prim of two states with one division: 1/r_a and 1/r_b from
 * 1/(r_a r_b) (densities are positive and far from over- or underflow). */
template <class T, class PP>
FV_HD void st_pair_from_prim(const PP &P, const T *ua, const T *ub, St<T> &a, St<T> &b)
{
	typedef typename Real<T>::type R;
	const T t = R(1) / (ua[0] * ub[0]);
	a.r = ua[0]; a.u = ua[1]; a.v = ua[2]; a.p = ua[3];
	b.r = ub[0]; b.u = ub[1]; b.v = ub[2]; b.p = ub[3];
	a.ir = ub[0] * t;
	b.ir = ua[0] * t;
	a.E = a.p * R(P.igm1) + R(0.5) * a.r * (a.u * a.u + a.v * a.v);
	b.E = b.p * R(P.igm1) + R(0.5) * b.r * (b.u * b.u + b.v * b.v);
}

template <class T> FV_HD void st_cons(const St<T> &s, T *uc) { uc[0] = s.r; uc[1] = s.r * s.u; uc[2] = s.r * s.v; uc[3] = s.E; }

template <class T, class PP> FV_HD T sound_speed(const PP &P, const St<T> &s)
{
	typedef typename Real<T>::type R;
	return vsqrt(R(P.g) * s.p * s.ir);
}

/* directional flux of a state (aphysics_defs.hpp:15-24) */
template <class T> FV_HD void dir_flux(const St<T> &s, const T &vn, const double *n, T *f)
{
	typedef typename Real<T>::type R;
	const T mn = s.r * vn;
	f[0] = mn;
	f[1] = mn * s.u + s.p * R(n[0]);
	f[2] = mn * s.v + s.p * R(n[1]);
	f[3] = vn * (s.E + s.p);
}

// ------------------------------- fluxes --------------------------------------

template <class T, class PP>
FV_HD void flux_llf(const PP &P, const St<T> &L, const St<T> &Rr, const double *n, T *f)
{
	typedef typename Real<T>::type R;
	const T vnl = L.u * R(n[0]) + L.v * R(n[1]), vnr = Rr.u * R(n[0]) + Rr.v * R(n[1]);
	const T cl = sound_speed(P, L), cr = sound_speed(P, Rr);
	const T a = vabs(vnl) + cl, b = vabs(vnr) + cr;
	const T eig = frozen(a > b ? a : b);
	T fl[4], fr[4], ul[4], ur[4];
	dir_flux(L, vnl, n, fl);
	dir_flux(Rr, vnr, n, fr);
	st_cons(L, ul);
	st_cons(Rr, ur);
	for (int i = 0; i < 4; i++) f[i] = R(0.5) * (fl[i] + fr[i] - eig * (ur[i] - ul[i]));
}

template <class T, class PP>
FV_HD void flux_vanleer(const PP &P, const St<T> &L, const St<T> &Rr, const double *n, T *f)
{
	typedef typename Real<T>::type R;
	const R g = R(P.g);
	const T vni = L.u * R(n[0]) + L.v * R(n[1]), vnj = Rr.u * R(n[0]) + Rr.v * R(n[1]);
	const T ci = sound_speed(P, L), cj = sound_speed(P, Rr);
	const T Mni = vni / ci, Mnj = vnj / cj;
	T fp[4], fm[4];
	if (Mni < R(-1)) {
		for (int i = 0; i < 4; i++) fp[i] = TL(0);
	} else if (Mni > R(1)) {
		dir_flux(L, vni, n, fp);
	} else {
		const T vm = L.u * L.u + L.v * L.v;
		const T mp1 = Mni + R(1);
		fp[0] = L.r * ci * mp1 * mp1 * R(0.25);
		fp[1] = fp[0] * (L.u + R(n[0]) * (R(2) * ci - vni) / g);
		fp[2] = fp[0] * (L.v + R(n[1]) * (R(2) * ci - vni) / g);
		const T q = (g - R(1)) * vni + R(2) * ci;
		fp[3] = fp[0] * ((vm - vni * vni) * R(0.5) + q * q / (R(2) * (g * g - R(1))));
	}
	if (Mnj > R(1)) {
		for (int i = 0; i < 4; i++) fm[i] = TL(0);
	} else if (Mnj < R(-1)) {
		dir_flux(Rr, vnj, n, fm);
	} else {
		const T vm = Rr.u * Rr.u + Rr.v * Rr.v;
		const T mm1 = Mnj - R(1);
		fm[0] = -Rr.r * cj * mm1 * mm1 * R(0.25);
		fm[1] = fm[0] * (Rr.u + R(n[0]) * (R(-2) * cj - vnj) / g);
		fm[2] = fm[0] * (Rr.v + R(n[1]) * (R(-2) * cj - vnj) / g);
		const T q = (g - R(1)) * vnj - R(2) * cj;
		fm[3] = fm[0] * ((vm - vnj * vnj) * R(0.5) + q * q / (R(2) * (g * g - R(1))));
	}
	for (int i = 0; i < 4; i++) f[i] = fp[i] + fm[i];
}

template <class T, class PP>
FV_HD void flux_ausm(const PP &P, const St<T> &L, const St<T> &Rr, const double *n, T *f)
{
	typedef typename Real<T>::type R;
	const T vni = L.u * R(n[0]) + L.v * R(n[1]), vnj = Rr.u * R(n[0]) + Rr.v * R(n[1]);
	const T ci = sound_speed(P, L), cj = sound_speed(P, Rr);
	const T Mni = vni / ci, Mnj = vnj / cj;
	T ML, MR, pL, pR;
	if (vabs(Mni) <= R(1)) {
		ML = R(0.25) * (Mni + R(1)) * (Mni + R(1));
		pL = ML * L.p * (R(2) - Mni);
	} else if (Mni < R(-1)) {
		ML = TL(0); pL = TL(0);
	} else {
		ML = Mni; pL = L.p;
	}
	if (vabs(Mnj) <= R(1)) {
		MR = R(-0.25) * (Mnj - R(1)) * (Mnj - R(1));
		pR = -MR * Rr.p * (R(2) + Mnj);
	} else if (Mnj < R(-1)) {
		MR = Mnj; pR = Rr.p;
	} else {
		MR = TL(0); pR = TL(0);
	}
	const T Mh = ML + MR, ph = pL + pR;
	const T hp = R(0.5) * Mh, ha = R(0.5) * vabs(Mh);
	T ul[4], ur[4];
	st_cons(L, ul);
	st_cons(Rr, ur);
	for (int j = 0; j < 3; j++) f[j] = hp * (ul[j] * ci + ur[j] * cj) - ha * (ur[j] * cj - ul[j] * ci);
	f[1] = f[1] + ph * R(n[0]);
	f[2] = f[2] + ph * R(n[1]);
	const T hl = ci * (L.E + L.p), hr = cj * (Rr.E + Rr.p);
	f[3] = hp * (hl + hr) - ha * (hr - hl);
}

template <class T, class PP>
FV_HD void flux_ausmplus(const PP &P, const St<T> &L, const St<T> &Rr, const double *n, T *f)
{
	typedef typename Real<T>::type R;
	const R g = R(P.g);
	const T vni = L.u * R(n[0]) + L.v * R(n[1]), vnj = Rr.u * R(n[0]) + Rr.v * R(n[1]);
	const T ci = sound_speed(P, L), cj = sound_speed(P, Rr);
	const T vmi = L.u * L.u + L.v * L.v, vmj = Rr.u * Rr.u + Rr.v * Rr.v;
	const R cf = R(2) * (g - R(1)) / (g + R(1));
	T csi = vsqrt((ci * ci / (g - R(1)) + R(0.5) * vmi) * cf);
	T csj = vsqrt((cj * cj / (g - R(1)) + R(0.5) * vmj) * cf);
	const T corri = csi > vni ? csi : vni;
	const T corrj = csj > -vnj ? csj : -vnj;
	csi = csi * csi / corri;
	csj = csj * csj / corrj;
	const T ch = csi < csj ? csi : csj;
	const T Mni = vni / ch, Mnj = vnj / ch;
	T ML, MR, pL, pR;
	if (vabs(Mni) <= R(1)) {
		const T a = Mni + R(1), b = Mni * Mni - R(1);
		ML = R(0.25) * a * a + R(0.125) * b * b;
		pL = L.p * (R(0.25) * a * a * (R(2) - Mni) + R(3.0 / 16) * Mni * b * b);
	} else if (Mni < R(-1)) {
		ML = TL(0); pL = TL(0);
	} else {
		ML = Mni; pL = L.p;
	}
	if (vabs(Mnj) <= R(1)) {
		const T a = Mnj - R(1), b = Mnj * Mnj - R(1);
		MR = R(-0.25) * a * a - R(0.125) * b * b;
		pR = Rr.p * (R(0.25) * a * a * (R(2) + Mnj) - R(3.0 / 16) * Mnj * b * b);
	} else if (Mnj < R(-1)) {
		MR = Mnj; pR = Rr.p;
	} else {
		MR = TL(0); pR = TL(0);
	}
	const T Mh = ML + MR, ph = pL + pR;
	const T hp = R(0.5) * Mh, ha = R(0.5) * vabs(Mh);
	T ul[4], ur[4];
	st_cons(L, ul);
	st_cons(Rr, ur);
	for (int j = 0; j < 3; j++) f[j] = ch * (hp * (ul[j] + ur[j]) - ha * (ur[j] - ul[j]));
	f[1] = f[1] + ph * R(n[0]);
	f[2] = f[2] + ph * R(n[1]);
	f[3] = ch * (hp * (L.E + L.p + Rr.E + Rr.p) - ha * ((Rr.E + Rr.p) - (L.E + L.p)));
}

/* Roe averages (anumericalflux.hpp:175-189) */
template <class T, class PP>
FV_HD void roe_avg(const PP &P, const St<T> &L, const St<T> &Rr, const T &Hl, const T &Hr, const double *n, T &Rij,
                   T &rij, T &uij, T &vij, T &vm2, T &vnij, T &Hij, T &cij)
{
	typedef typename Real<T>::type R;
	Rij = vsqrt(Rr.r * L.ir);
	rij = Rij * L.r;
	const T iR1 = R(1) / (Rij + R(1));
	uij = (Rij * Rr.u + L.u) * iR1;
	vij = (Rij * Rr.v + L.v) * iR1;
	Hij = (Rij * Hr + Hl) * iR1;
	vm2 = uij * uij + vij * vij;
	vnij = uij * R(n[0]) + vij * R(n[1]);
	cij = vsqrt(R(P.gm1) * (Hij - R(0.5) * vm2));
}

/* Harten fix as differentiated by the reference Roe Jacobian */
FV_HD double harten(double l, double d) { return (l * l + d * d) / (2.0 * d); }
FV_HD float harten(float l, float d) { return (l * l + d * d) / (2.0f * d); }
template <class R, int N>
FV_HD Dual<R, N> harten(const Dual<R, N> &l, const Dual<R, N> &d)
{
	Dual<R, N> r;
	r.v = (l.v * l.v + d.v * d.v) / (R(2) * d.v);
	const R i4 = R(1) / (R(4) * d.v * d.v);
	for (int k = 0; k < N; k++)
		r.d[k] = ((R(2) * (r.v * l.d[k] + d.v * d.d[k]) * R(2) * d.v) - (r.v * r.v + d.v * d.v) * R(2) * d.d[k]) * i4;
	return r;
}

template <class T, class PP>
FV_HD void flux_roe(const PP &P, const St<T> &L, const St<T> &Rr, const double *n, T *f)
{
	typedef typename Real<T>::type R;
	const R n0 = R(n[0]), n1 = R(n[1]);
	const T vni = L.u * n0 + L.v * n1, vnj = Rr.u * n0 + Rr.v * n1;
	const T Hi = (L.E + L.p) * L.ir, Hj = (Rr.E + Rr.p) * Rr.ir;
	T Rij, rij, uij, vij, vm2, vnij, Hij, cij;
	roe_avg(P, L, Rr, Hi, Hj, n, Rij, rij, uij, vij, vm2, vnij, Hij, cij);
	T l0 = vabs(vnij - cij), l1 = vabs(vnij), l3 = vabs(vnij + cij);
	const T delta = R(1.0e-4) * cij;
	if (l0 < delta) l0 = harten(l0, delta);
	if (l1 < delta) l1 = harten(l1, delta);
	if (l3 < delta) l3 = harten(l3, delta);
	const T devn = vnj - vni, dep = Rr.p - L.p, derho = Rr.r - L.r;
	const T ic2 = R(1) / (cij * cij);
	const T rcd = rij * cij * devn;
	const T la0 = l0 * (dep - rcd) * (R(0.5) * ic2);
	const T la1 = l1 * (derho - dep * ic2);
	const T la2 = l1 * rij;
	const T la3 = l3 * (dep + rcd) * (R(0.5) * ic2);
	const T du = Rr.u - L.u, dv = Rr.v - L.v;
	T adu[4];
	adu[0] = la0 + la1 + la3;
	adu[1] = la0 * (uij - cij * n0) + la1 * uij + la2 * (du - devn * n0) + la3 * (uij + cij * n0);
	adu[2] = la0 * (vij - cij * n1) + la1 * vij + la2 * (dv - devn * n1) + la3 * (vij + cij * n1);
	adu[3] = la0 * (Hij - cij * vnij) + la1 * vm2 * R(0.5) + la2 * (uij * du + vij * dv - vnij * devn) +
	         la3 * (Hij + cij * vnij);
	T fi[4], fj[4];
	dir_flux(L, vni, n, fi);
	dir_flux(Rr, vnj, n, fj);
	for (int i = 0; i < 4; i++) f[i] = R(0.5) * (fi[i] + fj[i] - adu[i]);
}

template <class T, class PP>
FV_HD void einfeldt(const PP &P, const St<T> &L, const St<T> &Rr, const double *n, T &vni, T &vnj, T &sl, T &sr)
{
	typedef typename Real<T>::type R;
	vni = L.u * R(n[0]) + L.v * R(n[1]);
	vnj = Rr.u * R(n[0]) + Rr.v * R(n[1]);
	const T ci = sound_speed(P, L), cj = sound_speed(P, Rr);
	const T Hi = (L.E + L.p) * L.ir, Hj = (Rr.E + Rr.p) * Rr.ir;
	T Rij, rij, uij, vij, vm2, vnij, Hij, cij;
	roe_avg(P, L, Rr, Hi, Hj, n, Rij, rij, uij, vij, vm2, vnij, Hij, cij);
	sl = vni - ci;
	if (sl > vnij - cij) sl = vnij - cij;
	sr = vnj + cj;
	if (sr < vnij + cij) sr = vnij + cij;
}

template <class T, class PP>
FV_HD void flux_hll(const PP &P, const St<T> &L, const St<T> &Rr, const double *n, T *f)
{
	typedef typename Real<T>::type R;
	T vni, vnj, sl, sr;
	einfeldt(P, L, Rr, n, vni, vnj, sl, sr);
	const T sr0 = sr > R(0) ? TL(0) : sr;
	const T sl0 = sl > R(0) ? TL(0) : sl;
	const T idn = R(1) / (sr - sl);
	const T t1 = frozen((sr0 - sl0) * idn);
	const T t2 = frozen(R(1) - (sr0 - sl0) * idn);
	const T t3 = frozen(R(0.5) * (sr * vabs(sl) - sl * vabs(sr)) * idn);
	T fi[4], fj[4], ul[4], ur[4];
	dir_flux(L, vni, n, fi);
	dir_flux(Rr, vnj, n, fj);
	st_cons(L, ul);
	st_cons(Rr, ur);
	for (int i = 0; i < 4; i++) f[i] = t1 * fj[i] + t2 * fi[i] - t3 * (ur[i] - ul[i]);
}

/* HLLC (anumericalflux.cpp:1040-1110).  Of its four cases (supersonic left,
 * left star state, right star state, supersonic right) the left two use the
 * left state and speed, the right two the right ones, with the same formulas:
 * the side is picked by selection and one flux (plus, inside the fan, its
 * star-state correction) is evaluated, so faces on either side of the
 * contact take one path through the FP64 pipe instead of two. */
template <class T, class PP>
FV_HD void flux_hllc(const PP &P, const St<T> &L, const St<T> &Rr, const double *n, T *f)
{
	typedef typename Real<T>::type R;
	T vni, vnj, sl, sr;
	einfeldt(P, L, Rr, n, vni, vnj, sl, sr);
	// contact speed sm = num / den; den > 0 (both of its terms are: sr > vnj, sl < vni)
	const T num = Rr.r * vnj * (sr - vnj) - L.r * vni * (sl - vni) + L.p - Rr.p;
	const T den = Rr.r * (sr - vnj) - L.r * (sl - vni);
	const bool left = sl > R(0) || num > R(0);
	const bool star = left ? !(sl > R(0)) : (sr >= R(0));
	const St<T> &S = left ? L : Rr;
	const T vn = left ? vni : vnj;
	const T sk = left ? sl : sr;
	dir_flux(S, vn, n, f);
	if (star) {
		// F_K + s_K (U*_K - U_K), star state anumericalflux.cpp:1071-1081;
		// sm and 1/(s_K - sm) from one division: e = den (s_K - sm)
		const T e = sk * den - num, t = R(1) / (den * e);
		const T sm = num * e * t, is = den * den * t;
		const T a = sk - vn;
		const T dps = S.r * (vn - sk) * (vn - sm);  // p* - p
		T uk[4];
		st_cons(S, uk);
		const T us0 = S.r * a * is;
		const T us1 = (a * uk[1] + dps * R(n[0])) * is;
		const T us2 = (a * uk[2] + dps * R(n[1])) * is;
		const T us3 = (a * S.E - S.p * vn + (dps + S.p) * sm) * is;
		f[0] = f[0] + sk * (us0 - uk[0]);
		f[1] = f[1] + sk * (us1 - uk[1]);
		f[2] = f[2] + sk * (us2 - uk[2]);
		f[3] = f[3] + sk * (us3 - uk[3]);
	}
}

template <int FLUX, class T, class PP>
FV_HD void numflux(const PP &P, const St<T> &L, const St<T> &Rr, const double *n, T *f)
{
	if (FLUX == FLUX_LLF) flux_llf(P, L, Rr, n, f);
	else if (FLUX == FLUX_VANLEER) flux_vanleer(P, L, Rr, n, f);
	else if (FLUX == FLUX_AUSM) flux_ausm(P, L, Rr, n, f);
	else if (FLUX == FLUX_AUSMPLUS) flux_ausmplus(P, L, Rr, n, f);
	else if (FLUX == FLUX_ROE) flux_roe(P, L, Rr, n, f);
	else if (FLUX == FLUX_HLL) flux_hll(P, L, Rr, n, f);
	else flux_hllc(P, L, Rr, n, f);
}

// ------------------------------ boundary conditions ---------------------------

struct BCDev {
	int type;
	double v0, v1;  // boundary values (tangential velocity / total p, T)
};

/* Ghost state from the interior conserved state (abc.cpp); jac selects the
 * branch rules of computeGhostStateAndJacobian (in/outflow: subsonic test
 * "<= 1", p_inf of the conserved freestream; isothermal wall: wall
 * temperature in the ghost energy). */
template <class T, class PP>
FV_HD void ghost_cons(const PP &P, const BCDev &bc, const T *in, const double *n, T *gs, bool jac)
{
	typedef typename Real<T>::type R;
	const R n0 = R(n[0]), n1 = R(n[1]);
	switch (bc.type) {
	case BC_SLIPWALL: {
		const T vn = (in[1] * n0 + in[2] * n1) / in[0];
		gs[0] = in[0];
		gs[1] = in[1] - R(2) * vn * n0 * in[0];
		gs[2] = in[2] - R(2) * vn * n1 * in[0];
		gs[3] = in[3];
		return;
	}
	case BC_FARFIELD:
		for (int i = 0; i < 4; i++) gs[i] = TL(P.uinf[i]);
		return;
	case BC_INOUTFLOW: {
		const T ir = R(1) / in[0];
		const T vn = (in[1] * n0 + in[2] * n1) * ir;
		const T m2 = in[1] * in[1] + in[2] * in[2];
		const T p = R(P.gm1) * (in[3] - R(0.5) * m2 * ir);
		const T c = vsqrt(R(P.g) * p * ir);
		const T Mn = vn / c;
		const bool sub = jac ? (Mn <= R(1)) : (Mn < R(1));
		if (Mn <= R(0)) {
			for (int i = 0; i < 4; i++) gs[i] = TL(P.uinf[i]);
		} else if (sub) {
			gs[0] = in[0]; gs[1] = in[1]; gs[2] = in[2];
			const R pb = R(jac ? P.pinf_cons : P.pinf);
			gs[3] = pb * R(P.igm1) + R(0.5) * m2 * ir;
		} else {
			for (int i = 0; i < 4; i++) gs[i] = in[i];
		}
		return;
	}
	case BC_SUBSONIC_INFLOW: {
		const R g = R(P.g), pt = R(bc.v0), tt = R(bc.v1);
		const T ir = R(1) / in[0];
		const T m2 = in[1] * in[1] + in[2] * in[2];
		const T p = R(P.gm1) * (in[3] - R(0.5) * m2 * ir);
		const T ci = vsqrt(g * p * ir);
		const T Rm = (in[1] * n0 + in[2] * n1) * ir - ci / (R(2) * g - R(1));
		const T co2 = ci * ci + (g - R(1)) * R(0.5) * m2 * ir * ir;
		const T q = vsqrt((g + R(1)) * co2 / ((g - R(1)) * Rm * Rm) - (g - R(1)) * R(0.5));
		const T cg = -Rm * (g - R(1)) / (g + R(1)) * (R(1) + q);
		const T tg = tt * cg * cg / co2;
		const T pg = pt * vpow(tg / tt, g / (g - R(1)));
		gs[0] = R(P.tcoef) * pg / tg;
		const T vg = vsqrt(R(2) / (g - R(1)) * (co2 - cg * cg));
		gs[1] = gs[0] * (vg * n0);
		gs[2] = gs[0] * (vg * n1);
		gs[3] = pg * R(P.igm1) + R(0.5) * gs[0] * vg * vg;
		return;
	}
	case BC_ADIABATICWALL: {
		const T tm = R(bc.v0) * in[0];
		gs[0] = in[0];
		gs[1] = R(2) * tm * n1 - in[1];
		gs[2] = R(-2) * tm * n0 - in[2];
		gs[3] = in[3];
		return;
	}
	case BC_ISOTHERMALWALL: {
		const R tv = R(bc.v0), tw = R(bc.v1);
		const R ec = R(1) / (R(P.g) * R(P.gm1) * R(P.Minf) * R(P.Minf));
		if (jac) {
			const T tm = tv * in[0];
			gs[0] = in[0];
			gs[1] = R(2) * tm * n1 - in[1];
			gs[2] = R(-2) * tm * n0 - in[2];
			const T vm2 = (gs[1] * gs[1] + gs[2] * gs[2]) / (in[0] * in[0]);
			gs[3] = in[0] * (tw * ec + R(0.5) * vm2);
			return;
		}
		const T ir = R(1) / in[0];
		const T p = R(P.gm1) * (in[3] - R(0.5) * (in[1] * in[1] + in[2] * in[2]) * ir);
		const T gt = R(2) * tw - R(P.tcoef) * p * ir;
		gs[0] = in[0];
		gs[1] = in[0] * (R(2) * tv * n1 - in[1] * ir);
		gs[2] = in[0] * (R(-2) * tv * n0 - in[2] * ir);
		const T vm2 = (gs[1] * gs[1] + gs[2] * gs[2]) * ir * ir;
		gs[3] = in[0] * (gt * ec + R(0.5) * vm2);
		return;
	}
	default:  // extrapolation
		for (int i = 0; i < 4; i++) gs[i] = in[i];
		return;
	}
}

/* d(ghost)/d(interior) row-major 4x4 and the jac-mode ghost value.  The
 * isothermal wall reproduces the reference's own formula (abc.cpp:357-398);
 * the others are exact derivatives.  The subsonic inflow BC, which has no
 * Jacobian in the reference (abc.cpp:179-185 exits), is differentiated
 * exactly here. */
template <class R, class PP>
FV_HD void ghost_jacobian(const PP &P, const BCDev &bc, const R *in, const double *n, R *gs, R *G)
{
	if (bc.type == BC_ISOTHERMALWALL) {
		ghost_cons<R>(P, bc, in, n, gs, true);
		const R tv = R(bc.v0), tw = R(bc.v1);
		for (int k = 0; k < 16; k++) G[k] = R(0);
		G[0] = R(1);
		G[4] = R(2) * tv * R(n[1]); G[5] = R(-1);
		G[8] = R(-2) * tv * R(n[0]); G[10] = R(-1);
		const R i2 = R(1) / (in[0] * in[0]);
		const R vm2 = (gs[1] * gs[1] + gs[2] * gs[2]) * i2;
		const R d0 = R(-2) * (gs[1] * gs[1] + gs[2] * gs[2]) * i2 / in[0];
		const R d1 = -i2 * gs[1], d2 = -i2 * gs[2];
		const R coeff = R(1) / (R(P.g) * R(P.gm1) * R(P.Minf) * R(P.Minf));
		G[12] = coeff * tw + R(0.5) * (vm2 + in[0] * d0);
		G[13] = in[0] * R(0.5) * d1;
		G[14] = in[0] * R(0.5) * d2;
		G[15] = R(0);
		return;
	}
	typedef Dual<R, 4> D4;
	D4 a[4], b[4];
	for (int i = 0; i < 4; i++) {
		a[i] = dconst<R, 4>(in[i]);
		a[i].d[i] = R(1);
	}
	ghost_cons<D4>(P, bc, a, n, b, true);
	for (int i = 0; i < 4; i++) {
		gs[i] = b[i].v;
		for (int k = 0; k < 4; k++) G[4 * i + k] = b[i].d[k];
	}
}

// ------------------------------ viscous ----------------------------------------

/* Sutherland viscosity / Re from temperature; the Dual overload carries the
 * reference Jacobian's derivative rule. */
FV_HD double sutherland(const Phys &P, double Tt) { return P.sutK / (Tt + P.sutC) * Tt * sqrt(Tt); }
FV_HD float sutherland(const Phys &P, float Tt) { return float(P.sutK) / (Tt + float(P.sutC)) * Tt * sqrtf(Tt); }
template <class R, int N>
FV_HD Dual<R, N> sutherland(const Phys &P, const Dual<R, N> &Tt)
{
	Dual<R, N> r;
	const R T = Tt.v, C = R(P.sutC), K = R(P.sutK);
	const R sq = vsqrt(T);
	r.v = K / (T + C) * T * sq;
	const R dmu = K * (R(1.5) / (T * sq) * (T + C) - T * sq) / ((T + C) * (T + C));
	for (int i = 0; i < N; i++) r.d[i] = dmu * Tt.d[i];
	return r;
}

/* Viscous flux given the face gradient of primitive-2 variables (rho,u,v,T),
 * grad[dim][var]; mu from the two face states (viscousphysics.cpp:71-122). */
template <class T>
FV_HD void viscous_flux(const Phys &P, bool constvisc, const double *n, const T grad[2][4], const St<T> &L,
                        const St<T> &Rr, T *vf)
{
	typedef typename Real<T>::type R;
	T mu;
	if (constvisc) mu = TL(P.ivisc);
	else mu = R(0.5) * (sutherland(P, R(P.tcoef) * L.p * L.ir) + sutherland(P, R(P.tcoef) * Rr.p * Rr.ir));
	const T kd = mu * R(P.kcoef);
	const T ld = (grad[0][1] + grad[1][2]) * (R(2.0 / 3.0) * mu);
	const T s00 = mu * (grad[0][1] + grad[0][1]) - ld;
	const T s01 = mu * (grad[0][2] + grad[1][1]);
	const T s11 = mu * (grad[1][2] + grad[1][2]) - ld;
	const R n0 = R(n[0]), n1 = R(n[1]);
	vf[0] = TL(0);
	vf[1] = -(s00 * n0 + s01 * n1);
	vf[2] = -(s01 * n0 + s11 * n1);
	const T va = R(0.5) * (L.u + Rr.u), vb = R(0.5) * (L.v + Rr.v);
	const T cx = s00 * va + s01 * vb + kd * grad[0][3];
	const T cy = s01 * va + s11 * vb + kd * grad[1][3];
	vf[3] = -(cx * n0 + cy * n1);
}

}  // namespace fvg
