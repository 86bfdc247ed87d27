// Emission of the off-equatorial jet crossings (the monopole field-line model of the
// reference's getstokes): at each crossing of a geodesic with the field line, the
// continuity-equation density, the drift-frame velocity of the force-free field, the
// redshift, the polarisation and the observed Stokes I, Q, U.
//
// kgeo/off_eq.py:15-119 (Iobs_off) and :124-233 (getstokes); kgeo/densityfuncs.py:32-78
// (eta_mono, density_mono_all); kgeo/velocities.py:487-623 (u_driftframe, numeric parallel
// boost, no Lorentz-factor cap); kgeo/bfields.py:544-593, 667-697 (the BZ monopole and the p = 0
// power field, general theta); kgeo/equatorial_images.py:307-334, 336-487, 524-544 (redshift,
// calc_polquantities, calc_evpa) at general theta with u^theta != 0.
#pragma once

#include "kg_polar.cuh"

namespace kg {

// The reference evaluates the BZ f(r) by linear interpolation of a table on
// linspace(1, 100, 100000) (kgeo/bfields.py:23-31); the table's node values are filled on the
// device from the closed form (bz_f) and interpolated the same way.
constexpr int BZ_TABLE_N = 100000;
constexpr double BZ_TABLE_STEP = 99.0 / (BZ_TABLE_N - 1);

KG_HD double bz_node(int64_t k) { return k == BZ_TABLE_N - 1 ? 100.0 : 1.0 + (double)k * BZ_TABLE_STEP; }

KG_HD void bz_f_table(const double* tab, double r, double* f, double* fp) {
  if (r > 100.0) {
    *f = 1.0 / (4.0 * r);
    *fp = -1.0 / (4.0 * r * r);
    return;
  }
  double kf = floor((r - 1.0) / BZ_TABLE_STEP);
  int64_t k = 0;  // r below 1 or NaN: the first interval
  if (kf >= 0) k = kf > BZ_TABLE_N - 2 ? BZ_TABLE_N - 2 : (int64_t)kf;
  const double r0 = bz_node(k), r1 = bz_node(k + 1);
  const double slope = (tab[k + 1] - tab[k]) / (r1 - r0);
  *f = tab[k] + (r - r0) * slope;
  *fp = slope;
}

enum : int { JETF_MONO = 0, JETF_POWER0 = 1 };

struct Trig {
  double cth, sth, cth2, sth2, c2th;
};

KG_HD Trig trig_of(double th) {
  Trig t;
  t.cth = cos(th);
  t.sth = sin(th);
  t.cth2 = t.cth * t.cth;
  t.sth2 = t.sth * t.sth;
  t.c2th = cos(2 * th);
  return t;
}

// B^i and Omega_F of the BZ monopole (C = 1) or of the p = 0 power field at (r, theta).
KG_HD BLab jet_field(int field, const double* tab, double a, double r, const Trig& T, double* omega) {
  const double a2 = a * a, r2 = r * r;
  const double Delta = r2 - 2 * r + a2;
  const double Sigma = r2 + a2 * T.cth2;
  const double gdet = T.sth * Sigma;
  BLab B;
  if (field == JETF_MONO) {
    double fr, frp;
    bz_f_table(tab, r, &fr, &frp);
    const double f2 = (6 * PI * PI - 49.) / 72.;
    const double omega2 = 1. / 32. - T.sth2 * (4 * f2 - 1) / 64.;
    const double dphidtheta = T.sth * (1 + 0.5 * a2 * fr * (1 + 3 * T.c2th));
    const double dphidr = a2 * T.sth2 * T.cth * frp;
    const double I = -1 * 2 * PI * T.sth2 * (a / 8. + (a2 * a) * (omega2 + 0.25 * fr * T.cth2));
    B.b1 = dphidtheta / gdet;
    B.b2 = -dphidr / gdet;
    B.b3 = I / (2 * PI * Delta * T.sth2);
    const double spin = fabs(a);
    double om = spin / 8. + spin * spin * spin * omega2;
    *omega = a < 0 ? -om : om;
  } else {
    // psi = 1 - |cos theta|, Omega = a / 8, I = -2 pi psi (2 - psi) Omega sign(cos theta)
    const double sc = T.cth > 0 ? 1.0 : (T.cth < 0 ? -1.0 : 0.0);
    const double psi = 1 - fabs(T.cth);
    const double Om = a / 8;
    const double I = -2 * PI * psi * (2 - psi) * Om * sc;
    B.b1 = (sc * T.sth * 1.0) / gdet;
    B.b2 = -(0.0 * psi / r) / gdet;
    B.b3 = I / (2 * PI * Delta * T.sth2);
    *omega = Om;
  }
  return B;
}

struct U4 {
  double u0, u1, u2, u3;
};

// u_driftframe (kgeo/velocities.py:541-623) for a numeric parallel boost nu.
KG_HD U4 jet_drift(int field, const double* tab, double a, double r, const Trig& T, double nu, BLab* Bout) {
  const double a2 = a * a, r2 = r * r;
  const double Delta = r2 - 2 * r + a2;
  const double Sigma = r2 + a2 * T.cth2;
  const double Xi = (r2 + a2) * (r2 + a2) - Delta * a2 * T.sth2;
  const double omegaz = 2 * a * r / Xi;
  const double gdet = Sigma * T.sth;
  const double g11 = Sigma / Delta, g22 = Sigma, g33 = Xi * T.sth2 / Sigma;
  const double alpha = sqrt(Delta * Sigma / Xi);
  const double eta3 = 2 * a * r / sqrt(Delta * Sigma * Xi);
  double omegaf;
  const BLab B = jet_field(field, tab, a, r, T, &omegaf);
  if (Bout) *Bout = B;
  const double E1 = (omegaf - omegaz) * Xi * T.sth * B.b2 / Sigma;
  const double E2 = -(omegaf - omegaz) * Xi * T.sth * B.b1 / (Sigma * Delta);
  const double Bsq = g11 * B.b1 * B.b1 + g22 * B.b2 * B.b2 + g33 * B.b3 * B.b3;
  const double Esq = g11 * E1 * E1 + g22 * E2 * E2;
  const double B1c = g11 * B.b1, B2c = g22 * B.b2, B3c = g33 * B.b3;
  const double E1c = g11 * E1, E2c = g22 * E2;
  const double f = alpha / (Bsq * gdet);
  const double vperp1 = f * (E2c * B3c - B2c * 0.0);
  const double vperp2 = f * (0.0 * B1c - B3c * E1c);
  const double vperp3 = f * (E1c * B2c - B1c * E2c);
  const double vpar_max = sqrt(1 - Esq / Bsq);
  const double sB = sqrt(Bsq);
  const double v1 = vperp1 + nu * vpar_max * B.b1 / sB;
  const double v2 = vperp2 + nu * vpar_max * B.b2 / sB;
  const double v3 = vperp3 + nu * vpar_max * B.b3 / sB;
  const double vsq = g11 * v1 * v1 + g22 * v2 * v2 + g33 * v3 * v3;
  const double gamma = 1. / sqrt(1 - vsq);
  return U4{gamma / alpha, gamma * (v1 + 0), gamma * (v2 + 0), gamma * (v3 + eta3)};
}

// eta_mono (kgeo/densityfuncs.py:32-44): the Gaussian source integrated from the stagnation radius.
KG_HD double eta_mono(double r, double cth, double r0, double spin, double sigma) {
  if (sigma == 0) return r > r0 ? 1.0 : (r < r0 ? -1.0 : (r == r0 ? 0.0 : r - r0));
  const double e = exp(-(r - r0) * (r - r0) / (2 * sigma * sigma));
  const double t1 = 2 * sigma * (2 * r0 - (r + r0) * e);
  const double s2p = sqrt(2 * PI);
  const double t2 = s2p * erf((r - r0) / (sqrt(2.0) * sigma)) * (r0 * r0 + sigma * sigma + spin * spin * cth * cth);
  const double den = 4 * r0 * sigma + s2p * sigma * sigma + s2p * (r0 * r0 + spin * spin * cth * cth);
  return (t1 + t2) / den;
}

KG_HD double nan_to_num(double x) {
  if (x != x) return 0.0;
  if (x == kg_inf()) return 1.7976931348623157e308;
  if (x == -kg_inf()) return -1.7976931348623157e308;
  return x;
}

struct Stokes {
  double I, Q, U;
};

// calc_polquantities at (r, theta) for u = (u0, u1, u2, u3), the lab-frame field B and the
// momentum signs (kgeo/equatorial_images.py:336-487): sin(theta_B), kappa, the path length
// across the field surface and the comoving b^2.
KG_HD void pol_general(double a, double r, const Trig& T, double lam, double eta, double kr, double kth, const U4& u,
                       const BLab& Bl, double* sinthb, double* k1, double* k2, double* plen, double* bsq) {
  const double a2 = a * a, r2 = r * r;
  const double Delta = r2 - 2 * r + a2;
  const double Sigma = r2 + a2 * T.cth2;
  const double gdet = Sigma * sqrt(T.sth2);
  const double g00 = -(1 - 2 * r / Sigma);
  const double g11 = Sigma / Delta, g22 = Sigma;
  const double g33 = (r2 + a2 + 2 * r * a2 * T.sth2 / Sigma) * T.sth2;
  const double g03 = -2 * r * a * T.sth2 / Sigma;
  const double g00_up = -(r2 + a2 + 2 * r * a2 * T.sth2 / Sigma) / Delta;
  const double g11_up = Delta / Sigma, g22_up = 1. / Sigma;
  const double g33_up = (Delta - a2 * T.sth2) / (Sigma * Delta * T.sth2);
  const double g03_up = -(2 * a * r) / (Sigma * Delta);
  const double u0_l = g00 * u.u0 + g03 * u.u3, u1_l = g11 * u.u1, u2_l = g22 * u.u2;
  const double u3_l = g33 * u.u3 + g03 * u.u0;
  const double uu = u0_l * u.u0 + u3_l * u.u3;
  const double Nr = sqrt(-g11 * uu * (1 + u2_l * u.u2));
  const double Nth = sqrt(g22 * (1 + u2_l * u.u2));
  const double Nph = sqrt(-Delta * T.sth2 * uu);
  const double e0x = u1_l * u.u0 / Nr, e1x = -uu / Nr, e3x = u1_l * u.u3 / Nr;
  const double e0y = u2_l * u.u0 / Nth, e1y = u2_l * u.u1 / Nth, e2y = (1 + u2_l * u.u2) / Nth,
               e3y = u2_l * u.u3 / Nth;
  const double e0z = u3_l / Nph, e3z = -u0_l / Nph;
  const double b0 = Bl.b1 * u1_l + Bl.b2 * u2_l + Bl.b3 * u3_l;
  const double b1 = (Bl.b1 + b0 * u.u1) / u.u0;
  const double b2 = (Bl.b2 + b0 * u.u2) / u.u0;
  const double b3 = (Bl.b3 + b0 * u.u3) / u.u0;
  const double b0_l = g00 * b0 + g03 * b3, b1_l = g11 * b1, b2_l = g22 * b2, b3_l = g33 * b3 + g03 * b0;
  const double Bx = e0x * b0_l + e1x * b1_l + e3x * b3_l;
  const double By = e0y * b0_l + e1y * b1_l + e2y * b2_l + e3y * b3_l;
  const double Bz = e0z * b0_l + e3z * b3_l;
  const double Bmag = sqrt(Bx * Bx + By * By + Bz * Bz);
  const double n1 = -Bl.b2 * gdet, n2 = Bl.b1 * gdet;
  const double nx = e1x * n1, ny = e1y * n1 + e2y * n2, nz = 0.0 * n1;
  const double nmag = sqrt(nx * nx + ny * ny + nz * nz);
  const double q = r2 + a2 - a * lam;
  const double lma = lam - a;
  const double R = q * q - Delta * (eta + lma * lma);
  const double TH = eta + a2 * T.cth2 - lam * lam * T.cth2 / T.sth2;
  const double kk1 = kr * sqrt(R) / Delta, kk2 = kth * sqrt(TH), kk3 = lam;
  const double K0 = g00_up * -1.0 + g03_up * kk3, K1 = g11_up * kk1, K2 = g22_up * kk2;
  const double K3 = g33_up * kk3 + g03_up * -1.0;
  const double kx = -e0x + e1x * kk1 + e3x * kk3;
  const double ky = -e0y + e1y * kk1 + e2y * kk2 + e3y * kk3;
  const double kz = -e0z + e3z * kk3;
  const double kmag = sqrt(kx * kx + ky * ky + kz * kz);
  const double kdn = kx * (nx / nmag) + ky * (ny / nmag) + kz * (nz / nmag);
  *plen = fabs(kmag / kdn);
  const double fx = (ky * Bz - kz * By) / kmag, fy = (kz * Bx - kx * Bz) / kmag, fz = (kx * By - ky * Bx) / kmag;
  *sinthb = sqrt(fx * fx + fy * fy + fz * fz) / Bmag;
  *bsq = Bmag * Bmag;
  const double f0 = e0x * fx + e0y * fy + e0z * fz, f1 = e1x * fx + e1y * fy, f2 = e2y * fy;
  const double f3 = e3x * fx + e3y * fy + e3z * fz;
  const double A = K0 * f1 - K1 * f0 + a * T.sth2 * (K1 * f3 - K3 * f1);
  const double Bk = ((r2 + a2) * (K3 * f2 - K2 * f3) - a * (K0 * f2 - K2 * f0)) * T.sth;
  const double ac = a * T.cth;
  *k1 = r * A - ac * Bk;
  *k2 = -(r * Bk) - ac * A;
}

// ---------------------------------------------------------------------------
// Stagnation radius of the monopole outflow (kgeo/ff_boost.py:7-18): numpy's sorted root 4 of
// the quintic c0 + c1 x + c2 x^2 + c3 x^3 + c5 x^5, i.e. the largest real part over the five
// roots. The roots come from the Aberth-Ehrlich simultaneous iteration (Aberth 1973) started on
// a circle of the Fujiwara bound's radius, and the chosen one is polished by Newton steps.

struct Cplx {
  double re, im;
};
KG_HD Cplx c_sub(Cplx x, Cplx y) { return Cplx{x.re - y.re, x.im - y.im}; }
KG_HD Cplx c_mul(Cplx x, Cplx y) { return Cplx{x.re * y.re - x.im * y.im, x.re * y.im + x.im * y.re}; }
KG_HD Cplx c_div(Cplx x, Cplx y) {
  const double d = 1.0 / (y.re * y.re + y.im * y.im);
  return Cplx{(x.re * y.re + x.im * y.im) * d, (x.im * y.re - x.re * y.im) * d};
}
KG_HD double c_abs(Cplx x) { return hypot(x.re, x.im); }
KG_HD bool kg_finite(double x) { return x - x == 0.0; }

// p(z) and p'(z) of the degree-5 polynomial with coefficients c[0..5] (Horner).
KG_HD void poly5(const double* c, Cplx z, Cplx* p, Cplx* dp) {
  Cplx v{c[5], 0.0}, d{0.0, 0.0};
  for (int k = 4; k >= 0; --k) {
    d = c_mul(d, z);
    d.re += v.re;
    d.im += v.im;
    v = c_mul(v, z);
    v.re += c[k];
  }
  *p = v;
  *dp = d;
}

// Aberth-Ehrlich correction of root i from the current roots z (the simultaneous form: every
// root's correction uses the previous iterate of the others, so the five can run in parallel).
KG_HD Cplx aberth_correction(const double* c, const Cplx* z, int i) {
  Cplx p, dp;
  poly5(c, z[i], &p, &dp);
  if (p.re == 0.0 && p.im == 0.0) return Cplx{0.0, 0.0};
  const Cplx ratio = c_div(p, dp);
  Cplx sum{0.0, 0.0};
  for (int j = 0; j < 5; ++j) {
    if (j == i) continue;
    const Cplx inv = c_div(Cplx{1.0, 0.0}, c_sub(z[i], z[j]));
    sum.re += inv.re;
    sum.im += inv.im;
  }
  const Cplx rs = c_mul(ratio, sum);
  const Cplx w = c_div(ratio, Cplx{1.0 - rs.re, -rs.im});
  if (!kg_finite(w.re) || !kg_finite(w.im)) return Cplx{0.0, 0.0};
  return w;
}

// Start of the iteration: five points on a circle of radius 2 max_k |c_k / c_5|^(1 / (5 - k)),
// the Fujiwara bound (>= every root's modulus); 0 when the start is unusable.
KG_HD double aberth_radius(const double* c) {
  double rad = 0.0;
  for (int k = 0; k < 5; ++k) rad = fmax(rad, pow(fabs(c[k] / c[5]), 1.0 / (5 - k)));
  rad = 2.0 * rad;
  return (rad > 0.0 && kg_finite(rad)) ? rad : 0.0;
}

KG_HD Cplx aberth_start(double rad, int k) {
  const double ang = 2.0 * PI * k / 5.0 + 0.4;
  return Cplx{rad * cos(ang), rad * sin(ang)};
}

constexpr int ABERTH_MAXITER = 200;
constexpr double ABERTH_TOL = 1e-15;  // largest relative correction of the last iteration

// The largest real part of the converged roots, after three Newton steps on that root.
KG_HD int aberth_finish(const double* c, const Cplx* z, double* out) {
  int best = 0;
  for (int k = 1; k < 5; ++k)
    if (z[k].re > z[best].re) best = k;
  Cplx zb = z[best];
  for (int it = 0; it < 3; ++it) {
    Cplx p, dp;
    poly5(c, zb, &p, &dp);
    const Cplx w = c_div(p, dp);
    if (!kg_finite(w.re) || !kg_finite(w.im)) break;
    zb = c_sub(zb, w);
  }
  if (!kg_finite(zb.re)) return 3;
  *out = zb.re;
  return 0;
}

// Largest real part of the roots of c[0] + ... + c[5] z^5 (serial form of the iteration that
// jet_stagnation_kernel runs on five lanes); 0 when found, 2 when c[5] == 0 (numpy trims the
// leading zero and the reference's root 4 does not exist), 3 without a usable start.
KG_HD int quintic_max_real_root(const double* c, double* out) {
  if (!(c[5] != 0.0) || !kg_finite(c[5])) return 2;
  const double rad = aberth_radius(c);
  if (rad == 0.0) return 3;
  Cplx z[5], w[5];
  for (int k = 0; k < 5; ++k) z[k] = aberth_start(rad, k);
  for (int it = 0; it < ABERTH_MAXITER; ++it) {
    double corr = 0.0;
    for (int i = 0; i < 5; ++i) w[i] = aberth_correction(c, z, i);
    for (int i = 0; i < 5; ++i) {
      z[i] = c_sub(z[i], w[i]);
      corr = fmax(corr, c_abs(w[i]) / fmax(c_abs(z[i]), 1e-300));
    }
    if (corr < ABERTH_TOL) break;
  }
  return aberth_finish(c, z, out);
}

// Coefficients of the stagnation quintic and Omega_F of the field line through theta
// (kgeo/ff_boost.py:7-18 with M = 1; kgeo/bfields.py:590-593 at the reflected angle).
KG_HD void stagnation_quintic(double a, double th, double* c, double* omega) {
  const double thn = acos(fabs(cos(th)));
  const Trig T = trig_of(thn);
  const double f2 = (6 * PI * PI - 49.) / 72.;
  const double omega2 = 1. / 32. - T.sth2 * (4 * f2 - 1) / 64.;
  const double spin = fabs(a);
  double om = spin / 8. + spin * spin * spin * omega2;
  om = a < 0 ? -om : om;
  *omega = om;
  const double k = 2 - a * om + a * om * T.c2th;
  const double s2t = sin(2 * thn);
  c[0] = -(a * a) / 2 * 1.0 * T.cth2 * (k * k);
  c[1] = -2 * pow(a, 4.0) * (om * om) * pow(T.cth, 4.0) * T.sth2;
  c[2] = 1.0 / 2 * (k * k);
  c[3] = -(a * a) * (om * om) * (s2t * s2t);
  c[4] = 0.0;
  c[5] = -2 * (om * om) * T.sth2;
}

// r0 and Omega_F of the field line through the crossing (r, th): the BZ monopole's Omega at
// the reflected angle and the quintic's root (kgeo/densityfuncs.py:47-60, kgeo/ff_boost.py).
KG_HD int jet_stagnation(double a, double th, double* r0, double* omega) {
  double c[6];
  stagnation_quintic(a, th, c, omega);
  return quintic_max_real_root(c, r0);
}

struct JetImgParams {
  int field;         // JETF_*
  double nu, sigma, r0, specind;
};

// One crossing: (I, Q, U) after the zeroing and nan_to_num of getstokes (kgeo/off_eq.py:197-213).
KG_HD Stokes jet_stokes(const JetImgParams& P, const double* tab, const Observer& o, double alpha, double beta,
                        double r, double th, double kr, double kth) {
  Stokes S{0.0, 0.0, 0.0};
  if (r == 0.0 || r <= o.rplus) return S;
  const double a = o.a;
  // density at the crossing reflected into the northern hemisphere, on the BZ monopole
  const double thn = acos(fabs(cos(th)));
  const Trig Tn = trig_of(thn);
  BLab Bn;
  const U4 un = jet_drift(JETF_MONO, tab, a, r, Tn, P.nu, &Bn);
  const double dens = nan_to_num(eta_mono(r, Tn.cth, P.r0, a, P.sigma) * Bn.b1 / un.u1);
  // emission at the crossing itself
  const Trig T = trig_of(th);
  BLab B;
  const U4 u = jet_drift(P.field, tab, a, r, T, P.nu, &B);
  const double lam = -alpha * o.sin_th;
  const double eta = (alpha * alpha - o.a2) * o.cos2 + beta * beta;
  const double TH = eta + o.a2 * T.cth2 - lam * lam * T.cth2 / T.sth2;
  const double R = (r * r + o.a2 - a * lam) * (r * r + o.a2 - a * lam) - (r * r - 2 * r + o.a2) * (eta + (lam - a) * (lam - a));
  const double skr = kr > 0 ? 1.0 : (kr < 0 ? -1.0 : 0.0), skth = kth > 0 ? 1.0 : (kth < 0 ? -1.0 : 0.0);
  const double g = 1 / (1 * u.u0 - lam * u.u3 - skth * u.u2 * sqrt(TH) - skr * u.u1 * sqrt(R) / (r * r - 2 * r + o.a2));
  double sinthb, k1, k2, plen, bsq;
  pol_general(a, r, T, lam, eta, kr, kth, u, B, &sinthb, &k1, &k2, &plen, &bsq);
  double c2, s2;
  evpa(a, o.sin_th, alpha, beta, PolResult{sinthb, k1, k2}, &c2, &s2);
  double Iemis = 1.0 * dens;
  Iemis = Iemis * pow(bsq, (1 + P.specind) / 2);
  const double I = pow(g, 3.0) * pow(g, P.specind) * plen * Iemis * pow(sinthb, 1 + P.specind);
  S.I = nan_to_num(I);
  S.Q = nan_to_num(c2 * I);
  S.U = nan_to_num(s2 * I);
  return S;
}

}  // namespace kg
