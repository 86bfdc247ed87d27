// Lensed curves of constant equatorial radius (rho(varphi) such that the m-th equatorial
// crossing of the ray at image-plane polar coordinates (rho, varphi) is at r_eq) and the
// closed-form critical curve.
//
// kgeo/equatorial_lensing.py:198-258 (r_equatorial2, objfunc, rho_of_req,
// rho_of_req_single: scipy.optimize.brentq per angle on a fixed bracket) and :260-289
// (critical_curve). Here every (curve, angle) pair is one thread running Brent's method on
// the same objective; a whole library of curves (spins x inclinations x orders x angles) is
// one launch.
#pragma once

#include "kg_equatorial.cuh"

namespace kg {

constexpr double CURVE_INF = 1.e50;  // equatorial_lensing.INF

// One curve of the batch: observer constants (r_o = inf), target radius, order, bracket.
struct CurveSpec {
  Observer obs;
  double r_target, rho_min, rho_max;
  int mbar;
};

// objfunc / r_equatorial2 (kgeo/equatorial_lensing.py:198-221): r_s of order mbar at
// (rho cos varphi, rho sin varphi), with r_s <= 0 replaced by INF outside the critical
// curve and by 1 inside, minus the target radius.
KG_HD double curve_objective(const CurveSpec& c, double cphi, double sphi, double rho) {
  const double alpha = cphi * rho;
  const double beta = sphi * rho;
  double rs, ir;
  r_equatorial_px(c.obs, alpha, beta, c.mbar, 1, &rs, &ir, 1);
  if (rs <= 0) {
    const double lam = -alpha * c.obs.sin_th;
    const double eta = (alpha * alpha - c.obs.a2) * c.obs.cos2 + beta * beta;
    rs = outside_crit(c.obs, lam, eta) == 1.0 ? CURVE_INF : 1.0;
  }
  return rs - c.r_target;
}

enum : int { CURVE_OK = 0, CURVE_SIGN = 1, CURVE_MAXITER = 2 };

// Root of f on [x0, x1] by Brent's method (R. P. Brent, Algorithms for Minimization without
// Derivatives, 1973, ch. 4): inverse quadratic interpolation or secant steps, kept inside the
// bracket and replaced by bisection when they do not shrink it fast enough. Converged when the
// bracket half-width is below (xtol + rtol |x|) / 2 or f(x) == 0 (the criterion of
// scipy.optimize.brentq). status: CURVE_SIGN when f(x0), f(x1) have the same sign,
// CURVE_MAXITER after maxiter steps.
template <class F>
KG_HD double brent_root(F f, double x0, double x1, double xtol, double rtol, int maxiter, int* status) {
  double a = x0, b = x1;
  double fa = f(a), fb = f(b);
  *status = CURVE_OK;
  if (fa * fb > 0) {
    *status = CURVE_SIGN;
    return kg_nan();
  }
  if (fa == 0) return a;
  if (fb == 0) return b;
  // c: the point that brackets the root with b; b: the best estimate
  double c = a, fc = fa;
  double d = b - a, e = d;
  for (int it = 0; it < maxiter; ++it) {
    if (fb * fc > 0) {  // re-bracket
      c = a;
      fc = fa;
      d = e = b - a;
    }
    if (fabs(fc) < fabs(fb)) {
      a = b;
      b = c;
      c = a;
      fa = fb;
      fb = fc;
      fc = fa;
    }
    const double tol = 0.5 * (xtol + rtol * fabs(b));
    const double m = 0.5 * (c - b);
    if (fb == 0 || fabs(m) < tol) return b;
    if (fabs(e) >= tol && fabs(fa) > fabs(fb)) {
      double p, q;
      const double s = fb / fa;
      if (a == c) {  // secant
        p = 2.0 * m * s;
        q = 1.0 - s;
      } else {  // inverse quadratic interpolation through (a, fa), (b, fb), (c, fc)
        const double qq = fa / fc, r = fb / fc;
        p = s * (2.0 * m * qq * (qq - r) - (b - a) * (r - 1.0));
        q = (qq - 1.0) * (r - 1.0) * (s - 1.0);
      }
      if (p > 0) q = -q;
      else p = -p;
      if (2.0 * p < fmin(3.0 * m * q - fabs(tol * q), fabs(e * q))) {
        e = d;
        d = p / q;
      } else {
        d = m;
        e = m;
      }
    } else {
      d = m;
      e = m;
    }
    a = b;
    fa = fb;
    b += fabs(d) > tol ? d : (m > 0 ? tol : -tol);
    fb = f(b);
  }
  *status = CURVE_MAXITER;
  return b;
}

// rho at one angle of one curve.
KG_HD double curve_rho(const CurveSpec& c, double varphi, double xtol, double rtol, int maxiter, int* status) {
  const double cphi = cos(varphi), sphi = sin(varphi);
  auto f = [&](double rho) { return curve_objective(c, cphi, sphi, rho); };
  return brent_root(f, c.rho_min, c.rho_max, xtol, rtol, maxiter, status);
}

// critical_curve (kgeo/equatorial_lensing.py:260-289): point i of r = linspace(r_-, r_+, n)
// on the spherical photon orbits, lambda and eta there (GL19 Eqs 38-40) and the screen
// coordinates; NaN where the reference's mask drops the point.
KG_HD void critical_point(double a, double sin_th, double cos_th, double tan_th, double rminus, double rplus,
                          int64_t n, int64_t i, double* alpha, double* beta) {
  // numpy.linspace: start + i * step, the last point set to stop; one point is start
  const double r = n == 1 ? rminus : (i == n - 1 ? rplus : rminus + (double)i * ((rplus - rminus) / (double)(n - 1)));
  const double a2 = a * a;
  const double r2 = r * r;
  const double lam = -(pow(r, 3.0) + a2 + r * a2 - 3.0 * r2) / (a * r - a);
  const double eta = r2 * (3.0 * r2 + a2 - lam * lam) / (r2 - a2);
  const double ac = a * cos_th;
  const double lt = lam / tan_th;
  *alpha = -lam / sin_th;
  *beta = sqrt(eta + ac * ac - lt * lt);
}

}  // namespace kg
