// Equatorial lensing per pixel: crossing counts, the source radius r_s of the m-th
// equatorial crossing, and the critical-curve side of a pixel, FP64.
//
// kgeo/equatorial_lensing.py:85-196 (r_equatorial), kgeo/kerr_raytracing_utils.py:551-684
// (n_poloidal_orbits, n_equatorial_crossings) and :794-826 (is_outside_crit). Compiled in
// the no-FMA translation unit with the per-ray setup: the crossing counts are floor()s of
// ratios of elliptic integrals and must round like numpy's to stay bit-exact.
#pragma once

#include "kg_ray.cuh"

namespace kg {

// r(tau) only (kgeo/kerr_raytracing_ana.py:404-595 with do_phi_and_t=False).
KG_HD double radial_r_at(const Observer& o, const Roots& R, double tau) {
  const double rplus = o.rplus, r_o = o.r_o;
  double r = 0.0;
  bool c4 = R.r1.im != 0;
  bool c3 = (R.r3.im != 0) && !c4;
  bool c2 = (R.r3.im == 0.) && !c3;
  if (c4) {
    double a1 = R.r4.im, b1 = R.r4.re, a2i = R.r2.im, b2 = R.r2.re;
    double CC = sqrt((a1 - a2i) * (a1 - a2i) + (b1 - b2) * (b1 - b2));
    double DD = sqrt((a1 + a2i) * (a1 + a2i) + (b1 - b2) * (b1 - b2));
    double k4 = (4 * CC * DD) / ((CC + DD) * (CC + DD));
    double x4ro = o.r_o_inf ? kg_inf() : (r_o + b1) / a2i;
    double g0 = sqrt((4 * (a2i * a2i) - (CC - DD) * (CC - DD)) / ((CC + DD) * (CC + DD) - 4 * (a2i * a2i)));
    double aux = atan(x4ro) + atan(g0);
    double pref = 2. / (CC + DD);
    double Ir_o = pref * ellip_f(aux, k4);
    double X4 = (1. / pref) * (-tau + Ir_o);
    double v, K2 = 2.0 * ellip_k(k4);
    double nr = reduce_half_period(X4, K2, &v);
    Jacobi J = jacobi_landen(v, k4);
    double odd = fmod(fabs(nr), 2.0) == 1.0 ? -1.0 : 1.0;
    double sc = (odd * J.sn) / (odd * J.cn);
    r = -a2i * (g0 - sc) / (1 + g0 * sc) - b1;
  }
  if (c3) {
    double a1 = R.r4.im, b1 = R.r4.re, rr1 = R.r1.re, rr2 = R.r2.re;
    double rr21 = rr2 - rr1;
    double AA = sqrt(a1 * a1 + (b1 - rr2) * (b1 - rr2));
    double BB = sqrt(a1 * a1 + (b1 - rr1) * (b1 - rr1));
    double k3 = ((AA + BB) * (AA + BB) - rr21 * rr21) / (4 * AA * BB);
    double x3ro;
    if (o.r_o_inf) x3ro = (AA - BB) / (AA + BB);
    else x3ro = (AA * (r_o - rr1) - BB * (r_o - rr2)) / (AA * (r_o - rr1) + BB * (r_o - rr2));
    double aux = acos(x3ro);
    double pref = (1. / sqrt(AA * BB));
    double Ir_o = pref * ellip_f(aux, k3);
    double X3 = (1. / pref) * (-tau + Ir_o);
    double v, K2 = 2.0 * ellip_k(k3);
    double nr = reduce_half_period(X3, K2, &v);
    Jacobi J = jacobi_landen(v, k3);
    double cn = (fmod(fabs(nr), 2.0) == 1.0 ? -1.0 : 1.0) * J.cn;
    r = ((BB * rr2 - AA * rr1) + (BB * rr2 + AA * rr1) * cn) / ((BB - AA) + (BB + AA) * cn);
  }
  if (c2) {
    double rr1 = R.r1.re, rr2 = R.r2.re, rr3 = R.r3.re, rr4 = R.r4.re;
    double rr31 = rr3 - rr1, rr32 = rr3 - rr2, rr41 = rr4 - rr1, rr42 = rr4 - rr2;
    double k2 = (rr32 * rr41) / (rr31 * rr42);
    double x2ro = o.r_o_inf ? sqrt(rr31 / rr41) : sqrt((rr31 * (r_o - rr4)) / (rr41 * (r_o - rr3)));
    double aux = asin(x2ro);
    double Ir_o = 2 * ellip_f(aux, k2) / sqrt(rr31 * rr42);
    double X2 = 0.5 * sqrt(rr31 * rr42) * (-tau + Ir_o);
    double v, K2 = 2.0 * ellip_k(k2);
    reduce_half_period(X2, K2, &v);
    Jacobi J = jacobi_landen(v, k2);
    double sn2 = J.sn * J.sn;
    r = (rr4 * rr31 - rr3 * rr41 * sn2) / (rr31 - rr41 * sn2);
  }
  (void)rplus;
  return r;
}

// Ray constants shared by the crossing counts (kgeo/equatorial_lensing.py:133-147).
struct EqConsts {
  bool vort;      // eta <= 0
  double sqa;     // sqrt(-a^2 u_-)
  double F0;      // F(asin(cos th_o / sqrt(u_+)) | u_+/u_-)
  double K;       // F(pi/2 | u_+/u_-)
  double a2um;
  double ratio;
};

KG_HD EqConsts eq_consts(const Observer& o, double lam, double eta) {
  EqConsts c;
  c.vort = eta <= 0;
  c.sqa = c.F0 = c.K = c.a2um = c.ratio = 0.0;
  if (c.vort) return c;
  Turning U = u_turning(o, lam, eta);
  u_ratio(o, lam, eta, U, &c.ratio, &c.a2um);
  c.F0 = ellip_f(asin(o.cos_th / sqrt(U.up)), c.ratio);
  c.K = ellip_f(0.5 * PI, c.ratio);
  c.sqa = sqrt(-c.a2um);
  return c;
}

// n_equatorial_crossings at Mino time tau (kgeo/kerr_raytracing_utils.py:660-677).
KG_HD double n_eq_at(const Observer& o, const EqConsts& c, double beta, double tau) {
  if (c.vort) return -2;
  if (o.th_o < (PI / 2.)) {
    if (beta <= 0) return floor((tau * c.sqa - c.F0) / (2 * c.K));
    return floor((tau * c.sqa + c.F0) / (2 * c.K)) - 1;
  }
  if (beta >= 0) return floor((tau * c.sqa + c.F0) / (2 * c.K));
  return floor((tau * c.sqa - c.F0) / (2 * c.K)) - 1;
}

// n_poloidal_orbits at Mino time tau (kgeo/kerr_raytracing_utils.py:591-595).
KG_HD double n_pol_at(const EqConsts& c, double Kc, double tau) {
  if (c.vort) return -2;
  // real(sqrt(complex(-a^2 u_-)) * tau) / (4 K): zero when -a^2 u_- < 0
  if (!(-c.a2um >= 0)) return 0.0 * tau / (4 * Kc);
  return (sqrt(-c.a2um) * tau) / (4 * Kc);
}

// Constants of n_angular_turnings (kgeo/kerr_raytracing_utils.py:686-792): ordinary rays
// (eta > 0) as the crossing counts; vortical rays (eta <= 0) through the vortical amplitude
// Nu = asin(sqrt((cos^2 th_o - u_-) / (u_+ - u_-))) and parameter 1 - u_+/u_- (GL19b Eqs 56,
// 60), as the reference evaluates them.
struct TurnConsts {
  bool vort;
  double sq, F0, K;
};

KG_HD TurnConsts turn_consts(const Observer& o, double lam, double eta) {
  TurnConsts c;
  c.vort = eta <= 0;
  Turning U = u_turning(o, lam, eta);
  double ratio, a2um;
  u_ratio(o, lam, eta, U, &ratio, &a2um);
  if (!c.vort) {
    c.F0 = ellip_f(asin(o.cos_th / sqrt(U.up)), ratio);
    c.K = ellip_f(0.5 * PI, ratio);
    c.sq = sqrt(-a2um);
  } else {
    const double nu = asin(sqrt((o.cos2 - U.um) / (U.up - U.um)));
    c.F0 = ellip_f(nu, 1 - ratio);
    c.K = ellip_f(0.5 * PI, 1 - ratio);
    c.sq = sqrt(a2um);
  }
  return c;
}

// Fractional number of angular turnings at Mino time tau (kgeo/kerr_raytracing_utils.py:
// 742-787, including its vortical rule: beta <= 0 counts above 1/2 gain another 1/2).
KG_HD double n_turn_at(const TurnConsts& c, double beta, double tau) {
  if (beta <= 0) {
    double n = (tau * c.sq - c.F0) / (2 * c.K) + 0.5;
    if (c.vort && n > 0.5) n += 0.5;
    return n;
  }
  return (tau * c.sq + c.F0) / (2 * c.K) + 0.5;
}

// is_outside_crit (kgeo/kerr_raytracing_utils.py:816-826): real r4 > r_h and eta >= 0.
KG_HD double outside_crit(const Observer& o, double lam, double eta) {
  Roots R = radial_roots(o, lam, eta);
  bool out = (R.r4.im == 0) && (R.r4.re > o.rplus) && !(eta < 0);
  return out ? 1.0 : 0.0;
}

struct EqResult {
  double Imax, Nmax;
};

// r_equatorial for orders mbar_lo .. mbar_lo + nord - 1 (kgeo/equatorial_lensing.py:108-196).
KG_HD EqResult r_equatorial_px(const Observer& o, double alpha, double beta, int mbar_lo, int nord,
                               double* r_s, double* Ir, int64_t stride) {
  double lam = -alpha * o.sin_th;
  double eta = (alpha * alpha - o.a2) * o.cos2 + beta * beta;
  EqResult res;
  if (eta <= 0) {
    for (int j = 0; j < nord; ++j) {
      r_s[j * stride] = -1;
      Ir[j * stride] = -1;
    }
    res.Imax = -1;
    res.Nmax = -2;
    return res;
  }
  EqConsts c = eq_consts(o, lam, eta);
  Roots R = radial_roots(o, lam, eta);
  double imax = mino_total(o, R);
  double nmax;
  bool north = o.th_o < (PI / 2.);
  if (north) {
    if (beta <= 0) nmax = floor((imax * c.sqa - c.F0) / (2 * c.K));
    else nmax = floor((imax * c.sqa + c.F0) / (2 * c.K)) - 1;
  } else {
    if (beta >= 0) nmax = floor((imax * c.sqa + c.F0) / (2 * c.K));
    else nmax = floor((imax * c.sqa - c.F0) / (2 * c.K)) - 1;
  }
  for (int j = 0; j < nord; ++j) {
    double mbar = (double)(mbar_lo + j);
    double ir;
    if (north) {
      double m = mbar + (beta > 0 ? 1.0 : 0.0);  // np.heaviside(beta, 0)
      if (beta <= 0) ir = (2 * m * c.K + c.F0) / c.sqa;
      else ir = (2 * m * c.K - c.F0) / c.sqa;
    } else {
      double m = mbar + (-beta > 0 ? 1.0 : 0.0);
      if (beta >= 0) ir = (2 * m * c.K - c.F0) / c.sqa;
      else ir = (2 * m * c.K + c.F0) / c.sqa;
    }
    double rs = radial_r_at(o, R, ir);
    if (nmax < mbar) rs = 0;
    r_s[j * stride] = rs;
    Ir[j * stride] = ir;
  }
  res.Imax = imax;
  res.Nmax = nmax;
  return res;
}

}  // namespace kg
