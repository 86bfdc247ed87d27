// Crossings of null geodesics with a jet field line psi(r, theta) = psi_target (the
// off-equatorial emission model's solver).
//
// kgeo/solver.py:14-207: the stream functions (psi_BZ_para, psi_BZ_mono, psi_power), the
// Mino-time bound of the search (get_maxtau_forwardjet), the guesses from the sign changes of
// psi - psi_target along a sampled geodesic (getguesses), the secant iteration of
// scipy.optimize.newton on the coordinates at a Mino time (findroot), the momentum signs and
// the equatorial-crossing count before the crossing (getneq). Here one thread scans one
// pixel's samples for guesses, and one thread iterates one (guess, pixel) pair to its root
// with the direct theta / r evaluators of the tracer.
#pragma once

#include "kg_equatorial.cuh"

namespace kg {

enum : int { JET_PARA = 0, JET_MONO = 1, JET_POWER = 2, JET_NONE = 3 };
constexpr double JET_MAXTAUFRAC = 1. - 1.e-10;  // kgeo/solver.py:12

struct JetField {
  int model;
  double psitarget, pval;
  double rp;  // outer horizon of the spin
};

// psifunc (kgeo/solver.py:14-38)
KG_HD double jet_psi(const JetField& J, double r, double th) {
  const double abscth = fabs(cos(th));
  switch (J.model) {
    case JET_PARA:
      return r * (1 - abscth) + J.rp * (1 + abscth) * (1 - log(1 + abscth)) - 2 * J.rp * (1 - log(2.0));
    case JET_MONO: return 1 - abscth;
    case JET_POWER: return pow(r, J.pval) * (1 - abscth);
    default: return 0.0;
  }
}

// get_maxtau_forwardjet (kgeo/solver.py:57-87): MAXTAUFRAC tau_tot, or the Mino time of the
// neqmax-th equatorial crossing when that is earlier (neqmax <= 0: no limit). numpy's min
// propagates NaN.
KG_HD double jet_taumax(const Observer& o, double alpha, double beta, int neqmax) {
  const double lam = -alpha * o.sin_th;
  const double eta = (alpha * alpha - o.a2) * o.cos2 + beta * beta;
  const Roots R = radial_roots(o, lam, eta);
  const double tt = mino_total(o, R) * JET_MAXTAUFRAC;
  if (neqmax <= 0 || eta <= 0) return tt;
  const Turning U = u_turning(o, lam, eta);
  double ratio, a2um;
  u_ratio(o, lam, eta, U, &ratio, &a2um);
  const double F0 = ellip_f(asin(o.cos_th / sqrt(U.up)), ratio);
  const double K = ellip_f(0.5 * PI, ratio);
  const double mmax = (double)(neqmax - 1) + (beta > 0 ? 1.0 : 0.0);
  const double sb = beta > 0 ? 1.0 : (beta < 0 ? -1.0 : 0.0);
  const double tm = (2 * mmax * K - sb * F0) / sqrt(-U.um * o.a2);
  if (tm != tm || tt != tt) return kg_nan();
  return tm < tt ? tm : tt;
}

// getneq (kgeo/solver.py:40-55) at Mino time tau with findroot's conserved quantities
// (eta < 0 lifted to EP below MINSPIN): ceil(nan_to_num(m - heaviside(beta, 0))).
KG_HD double jet_neq(const Observer& o, double alpha, double beta, double tau) {
  const double lam = -alpha * o.sin_th;
  double eta = (alpha * alpha - o.a2) * o.cos2 + beta * beta;
  if (o.minspin && eta < 0) eta = EP;
  const Turning U = u_turning(o, lam, eta);
  const double ratio = U.up / U.um;
  const double F0 = ellip_f(asin(o.cos_th / sqrt(U.up)), ratio);
  const double K = ellip_f(0.5 * PI, ratio);
  const double sb = beta > 0 ? 1.0 : (beta < 0 ? -1.0 : 0.0);
  double m = (sqrt(-U.um * o.a2) * tau + sb * F0) / (2 * K) - (beta > 0 ? 1.0 : 0.0);
  if (m != m) m = 0.0;
  else if (m == kg_inf()) m = 1.7976931348623157e308;
  else if (m == -kg_inf()) m = -1.7976931348623157e308;
  return ceil(m);
}

// The guesses of one pixel (getguesses, kgeo/solver.py:97-134): with out == NULL, their
// number (1 when there is none: the -1 placeholder); otherwise written to out[k * stride].
// r, th, mino: the pixel's ngeo samples (stride npix).
KG_HD int jet_pixel_guesses(const Observer& o, const JetField& J, double alpha, double beta, const double* r,
                            const double* th, const double* mino, int64_t ngeo, int64_t stride, int neqmax,
                            double* out, int64_t ostride) {
  const double b = sqrt(alpha * alpha + beta * beta);
  if (fabs(o.sin_th) < .1 && b > 100 && ((J.model == JET_POWER && J.pval > 0) || J.model == JET_PARA)) {
    double rparam;
    if (J.model == JET_POWER) rparam = pow(b * b / (2 * J.psitarget), 1 / (2 - J.pval));
    else rparam = (b * b + J.psitarget * J.psitarget) / (2 * J.psitarget);
    if (out) {
      out[0] = 1 / rparam;
      out[ostride] = 2 / b - 1 / rparam;
    }
    return 2;
  }
  const double tmax = jet_taumax(o, alpha, beta, neqmax);
  // argmin |mino - taumax| (first minimum; a NaN distance is the minimum, as numpy's argmin)
  int64_t indmax = 0;
  double best = kg_inf();
  for (int64_t j = 0; j < ngeo; ++j) {
    const double d = fabs(mino[j * stride] - tmax);
    if (d != d) {
      indmax = j;
      break;
    }
    if (d < best) {
      best = d;
      indmax = j;
    }
  }
  const int64_t L = indmax + 1 < ngeo ? indmax + 1 : ngeo;
  int n = 0;
  if (L >= 4) {
    double p0 = jet_psi(J, r[stride], th[stride]) - J.psitarget;
    for (int64_t j = 1; j <= L - 3; ++j) {
      const double p1 = jet_psi(J, r[(j + 1) * stride], th[(j + 1) * stride]) - J.psitarget;
      if (p1 * p0 < 0) {
        if (out) out[n * ostride] = (mino[j * stride] + mino[(j + 1) * stride]) / 2;
        ++n;
      }
      p0 = p1;
    }
  }
  if (n == 0) {
    if (out) out[0] = -1.0;
    return 1;
  }
  return n;
}

struct JetRoot {
  double tau, r, th, signpr, signpth, neq;
  int status;  // 0 converged, 1 maxiter
};

// findroot for one (guess, pixel) (kgeo/solver.py:136-207): the secant form of
// scipy.optimize.newton (start p1 = p (1 + eps^0.33) -+ eps^0.33, step p1 - q1 (p1 - p) /
// (q1 - q0), converged when |step| < tol; a flat pair q1 == q0 ends at (p + p1) / 2), then up to
// three further steps (the reference iterates every guess until all have converged), the
// coordinates at the root and at root (1 + 1e-5) for the momentum signs, and getneq. A -1
// guess (no crossing) is solved on a zero function and reported as zeros, its neq kept.
template <class FV>
KG_HD JetRoot jet_solve(const Observer& o, const JetField& J, const FV& f, int code, bool ordinary_active,
                        double alpha, double beta, double guess, double tol, int maxiter) {
  const bool none = guess == -1.0;
  auto psi_at = [&](double tau) {
    if (none) return 0.0;
    const ThetaOut T = sample_theta(f, code, tau, ordinary_active);
    const RadialOut R = sample_radial(f, code, tau, false);
    return jet_psi(J, R.r, T.th) - J.psitarget;
  };
  const double dx = 6.055454452393343e-06;  // numpy.finfo(float).eps ** 0.33
  double p = guess;
  double p1 = p * (1 + dx) + (p >= 0 ? dx : -dx);
  double q0 = psi_at(p), q1 = psi_at(p1);
  JetRoot out;
  out.status = 1;
  int extra = -1;  // steps left after convergence
  for (int it = 0; it < maxiter; ++it) {
    if (q1 == q0) {
      p = (p1 + p) / 2.0;
      out.status = 0;
      break;
    }
    const double dp = q1 * (p1 - p) / (q1 - q0);
    const double pn = p1 - dp;
    if (extra < 0 && fabs(dp) < tol) extra = 3;
    if (extra >= 0) {
      out.status = 0;
      if (extra == 0 || dp == 0.0) {
        p = pn;
        break;
      }
      --extra;
    }
    p = p1;
    p1 = pn;
    q0 = q1;
    q1 = psi_at(p1);
  }
  out.neq = jet_neq(o, alpha, beta, p);
  if (none) {
    out.tau = out.r = out.th = out.signpr = out.signpth = 0.0;
    return out;
  }
  const ThetaOut T0 = sample_theta(f, code, p, ordinary_active);
  const RadialOut R0 = sample_radial(f, code, p, false);
  const double p2 = p * (1 + 1e-5);
  const ThetaOut T1 = sample_theta(f, code, p2, ordinary_active);
  const RadialOut R1 = sample_radial(f, code, p2, false);
  auto sgn = [](double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : (x == 0 ? 0.0 : x)); };
  out.tau = p;
  out.r = R0.r;
  out.th = T0.th;
  out.signpr = sgn(R0.r - R1.r);
  out.signpth = sgn(T0.th - T1.th);
  return out;
}

}  // namespace kg
