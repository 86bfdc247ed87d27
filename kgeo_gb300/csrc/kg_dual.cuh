// Forward-mode dual numbers for the image adjoint: a value with N tangent components,
// the elementary functions on it, and the special functions the equatorial source radius
// needs (F(phi|m), K(m), sn/cn/dn(u|m)) with their derivatives in closed form.
//
// Derivatives of the elliptic functions with respect to the parameter m (DLMF 19.4.1-2,
// 22.13, rewritten without the 1/m factor):
//   dF(phi|m)/dm = (F - D) / (2 (1 - m)) - sin(phi) cos(phi) / (2 (1 - m) Delta),
//   D(phi|m) = int_0^phi sin^2 / Delta = sin^3(phi) R_D(cos^2 phi, Delta^2, 1) / 3,
//   Delta = sqrt(1 - m sin^2 phi); dK/dm = (K - D(pi/2|m)) / (2 (1 - m));
//   d am(u|m)/dm at fixed u = (sn cn - dn (u - D(am u|m))) / (2 (1 - m)),
// so that no form divides by m and the m -> 0 limit needs no special case.
#pragma once

#include "kg_common.cuh"
#include "kg_elliptic.cuh"

namespace kg {

KG_HD double val(double x) { return x; }

// The dual type and its overloads live in a nested namespace: code in namespace kg calls
// sqrt, log, ... unqualified and gets the global double functions by ordinary lookup and
// these by argument-dependent lookup, so one template serves both scalar types.
namespace ad {

template <int N>
struct Dual {
  double v;
  double d[N];
};

template <int N>
KG_HD Dual<N> dconst(double x) {
  Dual<N> r;
  r.v = x;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}

// Independent variable number `slot` with value x.
template <int N>
KG_HD Dual<N> dvar(double x, int slot) {
  Dual<N> r = dconst<N>(x);
  r.d[slot] = 1.0;
  return r;
}

// f(x) with f'(x) = df: the chain rule on every tangent component.
template <int N>
KG_HD Dual<N> dchain(const Dual<N>& x, double f, double df) {
  Dual<N> r;
  r.v = f;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = df * x.d[i];
  return r;
}

template <int N>
KG_HD double val(const Dual<N>& x) { return x.v; }

template <int N>
KG_HD Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
KG_HD Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
KG_HD Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
KG_HD Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N>
KG_HD Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N>
KG_HD Dual<N> operator+(const Dual<N>& a, double b) {
  Dual<N> r = a;
  r.v += b;
  return r;
}
template <int N>
KG_HD Dual<N> operator+(double b, const Dual<N>& a) { return a + b; }
template <int N>
KG_HD Dual<N> operator-(const Dual<N>& a, double b) {
  Dual<N> r = a;
  r.v -= b;
  return r;
}
template <int N>
KG_HD Dual<N> operator-(double b, const Dual<N>& a) {
  Dual<N> r = -a;
  r.v += b;
  return r;
}
template <int N>
KG_HD Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N>
KG_HD Dual<N> operator*(double b, const Dual<N>& a) { return a * b; }
template <int N>
KG_HD Dual<N> operator/(const Dual<N>& a, double b) { return a * (1.0 / b); }
template <int N>
KG_HD Dual<N> operator/(double a, const Dual<N>& b) {
  const double v = a / b.v;
  return dchain(b, v, -v / b.v);
}

template <int N>
KG_HD Dual<N> sqrt(const Dual<N>& x) {
  const double s = ::sqrt(x.v);
  return dchain(x, s, 0.5 / s);
}
template <int N>
KG_HD Dual<N> cbrt(const Dual<N>& x) {
  const double c = ::cbrt(x.v);
  return dchain(x, c, 1.0 / (3.0 * c * c));
}
template <int N>
KG_HD Dual<N> log(const Dual<N>& x) { return dchain(x, ::log(x.v), 1.0 / x.v); }
template <int N>
KG_HD Dual<N> exp(const Dual<N>& x) {
  const double e = ::exp(x.v);
  return dchain(x, e, e);
}
template <int N>
KG_HD Dual<N> sin(const Dual<N>& x) { return dchain(x, ::sin(x.v), ::cos(x.v)); }
template <int N>
KG_HD Dual<N> cos(const Dual<N>& x) { return dchain(x, ::cos(x.v), -::sin(x.v)); }
template <int N>
KG_HD Dual<N> atan(const Dual<N>& x) { return dchain(x, ::atan(x.v), 1.0 / (1.0 + x.v * x.v)); }
template <int N>
KG_HD Dual<N> asin(const Dual<N>& x) { return dchain(x, ::asin(x.v), 1.0 / ::sqrt(1.0 - x.v * x.v)); }
template <int N>
KG_HD Dual<N> acos(const Dual<N>& x) { return dchain(x, ::acos(x.v), -1.0 / ::sqrt(1.0 - x.v * x.v)); }
template <int N>
KG_HD Dual<N> asinh(const Dual<N>& x) { return dchain(x, ::asinh(x.v), 1.0 / ::sqrt(1.0 + x.v * x.v)); }
// x**p for a constant exponent, x > 0
template <int N>
KG_HD Dual<N> pow(const Dual<N>& x, double p) {
  const double y = ::pow(x.v, p);
  return dchain(x, y, p * y / x.v);
}

}  // namespace ad

using ad::Dual;
using ad::dconst;
using ad::dvar;
using ad::dchain;

// A constant of scalar type T (double, or a dual with zero tangents).
template <class T>
struct Lift;
template <>
struct Lift<double> {
  static KG_HD double c(double x) { return x; }
};
template <int N>
struct Lift<Dual<N>> {
  static KG_HD Dual<N> c(double x) { return dconst<N>(x); }
};

// D(phi|m) = int_0^phi sin^2 t / sqrt(1 - m sin^2 t) dt for |phi| <= pi/2.
KG_HD double ellip_d_red(double s, double c, double m) {
  return (s * s * s / 3.0) * carlson_rd(c * c, 1.0 - m * s * s, 1.0);
}

// F(phi|m) with both arguments dual; the value is ellip_f's.
template <int N>
KG_HD Dual<N> dual_ellip_f(const Dual<N>& phi, const Dual<N>& m) {
  const double n = rint(phi.v / PI);
  const double p0 = phi.v - n * PI;
  const double s = ::sin(p0), c = ::cos(p0);
  const double mv = m.v;
  const double F = ellip_f(phi.v, mv);
  double D = ellip_d_red(s, c, mv);
  if (n != 0.0) D += 2.0 * n * (carlson_rd(0.0, 1.0 - mv, 1.0) / 3.0);
  const double del = ::sqrt(1.0 - mv * s * s);
  const double dphi = 1.0 / del;
  const double dm = (F - D) / (2.0 * (1.0 - mv)) - s * c / (2.0 * (1.0 - mv) * del);
  Dual<N> r;
  r.v = F;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = dphi * phi.d[i] + dm * m.d[i];
  return r;
}

template <int N>
KG_HD Dual<N> dual_ellip_k(const Dual<N>& m) {
  const double K = ellip_k(m.v);
  const double Dc = carlson_rd(0.0, 1.0 - m.v, 1.0) / 3.0;
  return dchain(m, K, (K - Dc) / (2.0 * (1.0 - m.v)));
}

// sn, cn, dn(u|m) for |u| <= K(m) (the caller reduces by the half period), 0 <= m < 1.
template <int N>
KG_HD void dual_jacobi(const Dual<N>& u, const Dual<N>& m, Dual<N>* sn, Dual<N>* cn, Dual<N>* dn) {
  const double mv = m.v;
  Jacobi J = jacobi_landen(u.v, mv);
  const double D = ellip_d_red(J.sn, J.cn, mv);
  // amplitude derivatives: d am/du = dn, d am/dm (fixed u)
  const double am_m = (J.sn * J.cn - J.dn * (u.v - D)) / (2.0 * (1.0 - mv));
  sn->v = J.sn;
  cn->v = J.cn;
  dn->v = J.dn;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const double dam = J.dn * u.d[i] + am_m * m.d[i];
    sn->d[i] = J.cn * dam;
    cn->d[i] = -J.sn * dam;
    dn->d[i] = -(J.sn * J.sn * m.d[i] + 2.0 * mv * J.sn * J.cn * dam) / (2.0 * J.dn);
  }
}

}  // namespace kg
