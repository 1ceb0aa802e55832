/* ORACLE (test infrastructure only): forward-mode dual numbers.
 *
 * The oracle restates the reference's analytic flux/BC/viscous Jacobians as
 * exact derivatives of the restated functions, evaluated by forward-mode
 * differentiation.  Where the reference's hand-derived Jacobian is not the
 * exact derivative (frozen wave speeds, the Harten entropy fix, the
 * Sutherland derivative) the restated functions carry explicit rules that
 * reproduce the reference's formula; the tests check every flux and BC
 * Jacobian against the reference's compiled code.
 */
#pragma once
#include <cmath>

namespace orc {

template <int N>
struct Dual {
	double v;
	double d[N];
	Dual() : v(0) { for (int i = 0; i < N; i++) d[i] = 0; }
	Dual(double x) : v(x) { for (int i = 0; i < N; i++) d[i] = 0; }
	Dual &operator+=(const Dual &b) { v += b.v; for (int i = 0; i < N; i++) d[i] += b.d[i]; return *this; }
	Dual &operator-=(const Dual &b) { v -= b.v; for (int i = 0; i < N; i++) d[i] -= b.d[i]; return *this; }
	Dual &operator*=(const Dual &b) { *this = *this * b; return *this; }
	Dual &operator/=(const Dual &b) { *this = *this / b; return *this; }
	friend Dual operator+(const Dual &a, const Dual &b) { Dual r; r.v = a.v + b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] + b.d[i]; return r; }
	friend Dual operator-(const Dual &a, const Dual &b) { Dual r; r.v = a.v - b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] - b.d[i]; return r; }
	friend Dual operator-(const Dual &a) { Dual r; r.v = -a.v; for (int i = 0; i < N; i++) r.d[i] = -a.d[i]; return r; }
	friend Dual operator*(const Dual &a, const Dual &b) { Dual r; r.v = a.v * b.v; for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
	friend Dual operator/(const Dual &a, const Dual &b) {
		Dual r; r.v = a.v / b.v;
		for (int i = 0; i < N; i++) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v);
		return r;
	}
	friend Dual operator+(const Dual &a, double b) { Dual r = a; r.v += b; return r; }
	friend Dual operator+(double b, const Dual &a) { Dual r = a; r.v += b; return r; }
	friend Dual operator-(const Dual &a, double b) { Dual r = a; r.v -= b; return r; }
	friend Dual operator-(double b, const Dual &a) { Dual r = -a; r.v += b; return r; }
	friend Dual operator*(const Dual &a, double b) { Dual r; r.v = a.v * b; for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b; return r; }
	friend Dual operator*(double b, const Dual &a) { return a * b; }
	friend Dual operator/(const Dual &a, double b) { Dual r; r.v = a.v / b; for (int i = 0; i < N; i++) r.d[i] = a.d[i] / b; return r; }
	friend Dual operator/(double a, const Dual &b) {
		Dual r; r.v = a / b.v;
		for (int i = 0; i < N; i++) r.d[i] = -a * b.d[i] / (b.v * b.v);
		return r;
	}
	friend bool operator<(const Dual &a, const Dual &b) { return a.v < b.v; }
	friend bool operator>(const Dual &a, const Dual &b) { return a.v > b.v; }
	friend bool operator<=(const Dual &a, const Dual &b) { return a.v <= b.v; }
	friend bool operator>=(const Dual &a, const Dual &b) { return a.v >= b.v; }
	friend bool operator<(const Dual &a, double b) { return a.v < b; }
	friend bool operator>(const Dual &a, double b) { return a.v > b; }
	friend bool operator<=(const Dual &a, double b) { return a.v <= b; }
	friend bool operator>=(const Dual &a, double b) { return a.v >= b; }
	friend bool operator<(double a, const Dual &b) { return a < b.v; }
	friend bool operator>(double a, const Dual &b) { return a > b.v; }
	friend bool operator<=(double a, const Dual &b) { return a <= b.v; }
	friend bool operator>=(double a, const Dual &b) { return a >= b.v; }
};

template <int N>
inline Dual<N> sqrt(const Dual<N> &a)
{
	Dual<N> r; r.v = std::sqrt(a.v);
	for (int i = 0; i < N; i++) r.d[i] = 0.5 * a.d[i] / r.v;
	return r;
}

/* |x| with d|x|/dx = +1 for x >= 0 and -1 otherwise, the sign convention the
 * reference's hand-derived Jacobians use (e.g. anumericalflux.cpp:792-800). */
template <int N>
inline Dual<N> fabs(const Dual<N> &a)
{
	if (a.v >= 0) return a;
	return -a;
}

template <int N>
inline Dual<N> pow(const Dual<N> &a, double e)
{
	Dual<N> r; r.v = std::pow(a.v, e);
	const double dr = e * std::pow(a.v, e - 1.0);
	for (int i = 0; i < N; i++) r.d[i] = dr * a.d[i];
	return r;
}

inline double value(double x) { return x; }
template <int N> inline double value(const Dual<N> &x) { return x.v; }

/* Stop-gradient: the value with zero derivative.  Used where the reference
 * linearises with "frozen" quantities (LLF spectral radius, HLL wave speeds). */
inline double frozen(double x) { return x; }
template <int N> inline Dual<N> frozen(const Dual<N> &x) { return Dual<N>(x.v); }

using std::sqrt;
using std::fabs;
using std::pow;

}  // namespace orc
