// Polarised equatorial image: lab-frame magnetic field models, the comoving-frame emission
// angle sin(theta_B), the Penrose-Walker constant and the observed EVPA, and the rest-frame
// path length through the disk.
//
// kgeo/equatorial_images.py:336-487 (calc_polquantities), :489-522
// (calc_pathlength_equatorial), :524-544 (calc_evpa); kgeo/velocities.py:124-176 (tetrades);
// kgeo/bfields.py:93-131 (Bfield.bfield_lab) with the model functions :429-736. Everything
// is evaluated at th = pi/2 as the reference evaluates it: with the double nearest pi/2,
// cos(th) = COS_EQ, cos(th)^2 = COS2_EQ, sin(th) = sin(th)^2 = 1 and cos(2 th) = -1 exactly.
// All supported velocities have u^theta = 0, which removes the terms that multiply it.
#pragma once

#include "kg_image.cuh"

namespace kg {

// values of kgeo_bfield's enum
enum : int {
  BF_SIMPLE = 0,
  BF_SIMPLE_RM1 = 1,
  BF_MONOPOLE_A = 2,
  BF_BZ_GUESS = 3,
  BF_BZ_MONOPOLE = 4,
  BF_BZ_PARA = 5,
  BF_POWER = 6,
  BF_GEN_POWER = 7,
};

constexpr double COS_EQ = 6.123233995736766e-17;  // cos of the double nearest pi/2
constexpr double INV_E = 0.36787944117144233;     // 1/e
constexpr double LN2 = 0.6931471805599453;
constexpr double PI2_6 = 1.6449340668482264;      // pi^2 / 6

struct BLab {
  double b1, b2, b3;
};

// Real dilogarithm Li2(y) for -1 <= y <= 1/2 by the Bernoulli-number series in
// u = -ln(1 - y): Li2 = sum_n B_n u^(n+1) / (n+1)! ('t Hooft and Veltman 1979). |u| <= ln 2
// here, so the terms fall like (u / 2 pi)^(2k) and B_16 ends the sum below 1e-17.
KG_HD double li2_series(double y) {
  const double u = -log1p(-y);
  const double u2 = u * u;
  // B_2k / (2k + 1)!, k = 1..8
  const double c[8] = {1.0 / 36.0,
                       -1.0 / 3600.0,
                       1.0 / 211680.0,
                       -1.0 / 10886400.0,
                       1.0 / 526901760.0,
                       -4.0647616451442255e-11,
                       8.9216910204564526e-13,
                       -1.9939295860721076e-14};
  double s = c[7];
  for (int k = 6; k >= 0; --k) s = s * u2 + c[k];
  return u - 0.25 * u2 + u * u2 * s;
}

// Re Li2(x) for 0 < x <= 2 (x = 2/r, r >= 1): Euler's reflection
// Li2(x) + Li2(1 - x) = pi^2/6 - ln(x) ln(1 - x), real part for x > 1.
KG_HD double re_li2(double x) {
  if (x <= 0.5) return li2_series(x);
  if (x == 1.0) return PI2_6;
  return PI2_6 - log(x) * log(fabs(1.0 - x)) - li2_series(1.0 - x);
}

// BZ monopole radial function f(r) and f'(r) in closed form (kgeo/bfields.py:7-13):
// f = Re[Li2(2/r) - ln(1 - 2/r) ln(r/2)] r^2 (2r - 3) / 8 + (1 + 3r - 6r^2) ln(r/2) / 12
//     + 11/72 + 1/(3r) + r/2 - r^2/2,
// with d/dr [Li2(2/r) - ln(1 - 2/r) ln(r/2)] = -2 ln(r/2) / (r (r - 2)). Beyond r = 100 the
// reference uses 1/(4r) and -1/(4r^2) (kgeo/bfields.py:540-543); so does this. (The reference
// reads f on [1, 100] from a linearly interpolated table.)
KG_HD void bz_f(double r, double* f, double* fp) {
  if (r > 100.0) {
    *f = 1.0 / (4.0 * r);
    *fp = -1.0 / (4.0 * r * r);
    return;
  }
  const double x = 2.0 / r;
  const double lr = log(r / 2.0);
  const double P = re_li2(x) - (r == 2.0 ? 0.0 : log(fabs(1.0 - x)) * lr);
  const double Q = r * r * (2.0 * r - 3.0) / 8.0;
  double ff = P * Q + (1.0 + 3.0 * r - 6.0 * r * r) * lr / 12.0;
  ff += 11.0 / 72.0 + 1.0 / (3.0 * r) + r / 2.0 - r * r / 2.0;
  const double q = (r == 2.0) ? 0.5 : log1p((r - 2.0) / 2.0) / (r - 2.0);
  const double dP = -2.0 * q / r;
  double d = dP * Q + P * 3.0 * r * (r - 1.0) / 4.0;
  d += (3.0 - 12.0 * r) * lr / 12.0 + (1.0 + 3.0 * r - 6.0 * r * r) / (12.0 * r);
  d += -1.0 / (3.0 * r * r) + 0.5 - r;
  *f = ff;
  *fp = d;
}

// Principal branch W0(z) of the Lambert W function for z >= -1/e by Halley's iteration
// (Corless, Gonnet, Hare, Jeffrey and Knuth 1996), started from the branch-point series
// near -1/e and from ln(1 + z) elsewhere.
KG_HD double lambert_w0(double z) {
  if (z == 0.0) return 0.0;
  double w;
  const double q = z + INV_E;
  if (q < 0.25) {
    const double p = sqrt(fmax(2.0 * 2.718281828459045 * q, 0.0));
    w = -1.0 + p * (1.0 + p * (-1.0 / 3.0 + p * (11.0 / 72.0)));
  } else {
    w = log1p(z);
    if (z > 3.0) w -= log(w);
  }
  for (int it = 0; it < 12; ++it) {
    const double ew = exp(w);
    const double fw = w * ew - z;
    const double wp1 = w + 1.0;
    if (wp1 == 0.0) break;
    const double dw = fw / (ew * wp1 - (w + 2.0) * fw / (2.0 * wp1));
    w -= dw;
    if (fabs(dw) <= 1e-16 * (1.0 + fabs(w))) break;
  }
  return w;
}

struct FieldModel {
  int field, flag;
  double c[3];
};

// Lab-frame B^i = *F^{i0} at (r, pi/2) (kgeo/bfields.py:93-131). rp: outer horizon.
KG_HD BLab bfield_lab(const FieldModel& F, double a, double r, double rp) {
  const double a2 = a * a;
  const double r2 = r * r;
  const double Delta = r2 - 2.0 * r + a2;
  const double Sigma = r2 + a2 * COS2_EQ;
  const double gdet = Sigma;  // sin(th) Sigma
  BLab B;
  switch (F.field) {
    case BF_SIMPLE:
    case BF_SIMPLE_RM1: {  // kgeo/bfields.py:429-476
      const double arad = F.c[0], avert = F.c[1], ator = F.c[2];
      const double rad = (F.field == BF_SIMPLE_RM1) ? r / gdet : 1.0 / gdet;
      B.b1 = arad * rad + avert * (r * COS_EQ / gdet);
      B.b2 = avert * (-1.0 / gdet);
      B.b3 = ator * (1.0 / gdet);
      break;
    }
    case BF_MONOPOLE_A: {  // :479-499
      const double C = F.c[0];
      const double omegah = a / (2.0 * rp);
      const double phih = 4.0 * PI * C;
      const double omegaf = F.c[1] * omegah;
      const double I = phih * rp * (omegaf - omegah) / (rp * rp + a2 * COS2_EQ);
      B.b1 = (phih / (4.0 * PI)) / Sigma;
      B.b2 = 0.0;
      B.b3 = I / (2.0 * PI * Delta);
      break;
    }
    case BF_BZ_GUESS: {  // :502-541
      const double C = F.c[0];
      const double Pi = (r2 + a2) * (r2 + a2) - a2 * Delta;
      const double OmegaH = a / (2.0 * rp);
      const double spin = fabs(a);
      const double f2 = (6.0 * PI * PI - 49.0) / 72.0;
      const double omega2 = 1.0 / 32.0 - (4.0 * f2 - 1.0) / 64.0;
      double OmegaBZ = spin * (1.0 / 8.0) + (spin * spin * spin) * omega2;
      if (a < 0) OmegaBZ = -OmegaBZ;
      const double Br = C / r2;
      B.b1 = Br;
      B.b2 = 0.0;
      B.b3 = (-1.0 * (OmegaH - OmegaBZ) * sqrt(Pi) / Delta) * Br;
      break;
    }
    case BF_BZ_MONOPOLE: {  // :544-589
      const double C = F.c[0];
      double fr, frp;
      bz_f(r, &fr, &frp);
      const double f2 = (6.0 * PI * PI - 49.0) / 72.0;
      const double omega2 = 1.0 / 32.0 - (4.0 * f2 - 1.0) / 64.0;
      if (F.flag) {  // secondorder_only
        const double d = r2 - 2.0 * r;
        B.b1 = C / r2 + C * a2 * (-COS2_EQ / (r2 * r2) + fr * (0.5 - 1.5) / r2);
        B.b2 = -C * a2 * frp * COS_EQ / r2;
        B.b3 = -C * 0.125 * a / d + C * (a2 * a) * (0.125 / (d * d) - (omega2 + 0.25 * COS2_EQ * fr) / d);
      } else {
        const double dphidtheta = C * (1.0 + 0.5 * a2 * fr * (1.0 - 3.0));
        const double dphidr = C * a2 * COS_EQ * frp;
        const double I = -1.0 * C * 2.0 * PI * (a / 8.0 + (a2 * a) * (omega2 + 0.25 * fr * COS2_EQ));
        B.b1 = dphidtheta / gdet;
        B.b2 = -dphidr / gdet;
        B.b3 = I / (2.0 * PI * Delta);
      }
      break;
    }
    case BF_BZ_PARA: {  // :618-663 with omega_BZpara :600-606
      // 1 -+ |cos th| and 1 + |cos th| round to 1 at th = pi/2, and ln(1) = 0
      const double C = F.c[0];
      const double psi = r + rp - 2.0 * rp * (1.0 - LN2);
      const double argv = -psi / rp + 2.0 * LN2;
      double Omega = 0.0;
      if (argv >= -INV_E) {
        const double w = lambert_w0(argv);
        const double x = exp(w);
        const double y = 1.0 + psi / (1.0 + w) / (x * (2.0 - x));
        Omega = C * (a / 4.0 / y);
      }
      const double I = -4.0 * PI * psi * Omega;
      B.b1 = C * r / gdet;
      B.b2 = -C * 1.0 / gdet;
      B.b3 = I / (2.0 * PI * Delta);
      break;
    }
    case BF_POWER: {  // :667-697 with omega_BZpower :609-615
      const double C = F.c[0], p = F.c[1];
      const double rpow = pow(r, p);
      const double psi = rpow;  // r^p (1 - |cos th|)
      const double dpsidr = p * psi / r;
      double Omega;
      if (F.flag || p == 0.0) {
        Omega = a / 8.0;
      } else {
        const double cthh = 1.0 - psi * pow(rp, -p);
        Omega = a / (4.0 + 8.0 / (1.0 + cthh));
      }
      const double I = (p > 0.0) ? -4.0 * PI * psi * Omega : -2.0 * PI * psi * (2.0 - psi) * Omega;
      B.b1 = C * rpow / gdet;
      B.b2 = -C * dpsidr / gdet;
      B.b3 = I / (2.0 * PI * Delta);
      break;
    }
    default: {  // BF_GEN_POWER, :700-732
      const double n_I = F.c[0], p_val = F.c[1];
      double I_0 = (a * PI) / (rp * rp + a2 * COS2_EQ);
      double dpsidtheta = pow(r / rp, p_val);
      if (!F.flag) {  // isAbove == False
        I_0 = -I_0;
        dpsidtheta = -dpsidtheta;
      }
      const double I = I_0 * pow(r / rp, -n_I);
      const double dpsidr = (p_val * pow(r, p_val - 1.0)) / pow(rp, p_val);
      B.b1 = dpsidtheta / gdet;
      B.b2 = -1.0 * (dpsidr / gdet);
      B.b3 = I / (2.0 * PI * Delta);
      break;
    }
  }
  return B;
}

struct PolResult {
  double sinthb;
  double kappa1, kappa2;  // Penrose-Walker constant
};

// calc_polquantities for a lab-frame field at (r, pi/2): tetrads of the fluid frame
// (kgeo/velocities.py:145-168), the fluid-frame field with e^mu = 0, the photon momentum,
// the polarisation vector f = k x B / |k| and kappa = (r - i a cos th)(A - i B).
KG_HD PolResult pol_quantities(double a, double r, double lam, double eta, double kr, double kth,
                               const Ucon<double>& u, const BLab& Bl) {
  const double a2 = a * a;
  const double r2 = r * r;
  const double Delta = r2 - 2.0 * r + a2;
  const double Sigma = r2 + a2 * COS2_EQ;
  const double g00 = -(1.0 - 2.0 * r / Sigma);
  const double g11 = Sigma / Delta;
  const double g22 = Sigma;
  const double g33 = r2 + a2 + 2.0 * r * a2 / Sigma;
  const double g03 = -2.0 * r * a / Sigma;
  const double g00_up = -(r2 + a2 + 2.0 * r * a2 / Sigma) / Delta;
  const double g11_up = Delta / Sigma;
  const double g22_up = 1.0 / Sigma;
  const double g33_up = (Delta - a2) / (Sigma * Delta);
  const double g03_up = -(2.0 * a * r) / (Sigma * Delta);
  const double u0 = u.u0, u1 = u.u1, u3 = u.u3;
  const double u0_l = g00 * u0 + g03 * u3;
  const double u1_l = g11 * u1;
  const double u3_l = g33 * u3 + g03 * u0;
  // tetrads (u^theta = 0)
  const double uu = u0_l * u0 + u3_l * u3;
  const double Nr = sqrt(-g11 * uu);
  const double Nth = sqrt(g22);
  const double Nph = sqrt(-Delta * uu);
  const double e0x = u1_l * u0 / Nr, e1x = -uu / Nr, e3x = u1_l * u3 / Nr;
  const double e2y = 1.0 / Nth;
  const double e0z = u3_l / Nph, e3z = -u0_l / Nph;
  // fluid-frame field b^mu, lowered
  const double b0 = Bl.b1 * u1_l + Bl.b3 * u3_l;
  const double b1 = (Bl.b1 + b0 * u1) / u0;
  const double b2 = Bl.b2 / u0;
  const double b3 = (Bl.b3 + b0 * u3) / u0;
  const double b0_l = g00 * b0 + g03 * b3;
  const double b1_l = g11 * b1;
  const double b2_l = g22 * b2;
  const double b3_l = g33 * b3 + g03 * b0;
  const double Bx = e0x * b0_l + e1x * b1_l + e3x * b3_l;
  const double By = e2y * b2_l;
  const double Bz = e0z * b0_l + e3z * b3_l;
  const double Bmag = sqrt(Bx * Bx + By * By + Bz * Bz);
  // photon momentum
  const double q = r2 + a2 - a * lam;
  const double lma = lam - a;
  const double R = q * q - Delta * (eta + lma * lma);
  const double TH = eta + a2 * COS2_EQ - lam * lam * COS2_EQ;
  const double k1_l = kr * sqrt(R) / Delta;
  const double k2_l = kth * sqrt(TH);
  const double k3_l = lam;
  const double k0 = g00_up * -1.0 + g03_up * k3_l;
  const double k1 = g11_up * k1_l;
  const double k2 = g22_up * k2_l;
  const double k3 = g33_up * k3_l + g03_up * -1.0;
  const double kx = -e0x + e1x * k1_l + e3x * k3_l;
  const double ky = e2y * k2_l;
  const double kz = -e0z + e3z * k3_l;
  const double kmag = sqrt(kx * kx + ky * ky + kz * kz);
  // polarisation vector and emission angle
  const double fx = (ky * Bz - kz * By) / kmag;
  const double fy = (kz * Bx - kx * Bz) / kmag;
  const double fz = (kx * By - ky * Bx) / kmag;
  PolResult P;
  P.sinthb = sqrt(fx * fx + fy * fy + fz * fz) / Bmag;
  const double f0 = e0x * fx + e0z * fz;
  const double f1 = e1x * fx;
  const double f2 = e2y * fy;
  const double f3 = e3x * fx + e3z * fz;
  const double A = k0 * f1 - k1 * f0 + a * (k1 * f3 - k3 * f1);
  const double Bk = (r2 + a2) * (k3 * f2 - k2 * f3) - a * (k0 * f2 - k2 * f0);
  const double ac = a * COS_EQ;
  P.kappa1 = r * A - ac * Bk;
  P.kappa2 = -(r * Bk) - ac * A;
  return P;
}

// (cos 2 chi, sin 2 chi) of the observed EVPA (kgeo/equatorial_images.py:524-544).
KG_HD void evpa(double a, double sin_th_o, double alpha, double beta, const PolResult& P, double* c2, double* s2) {
  const double mu = -(alpha + a * sin_th_o);
  const double x = beta * P.kappa1 + mu * P.kappa2;
  const double y = mu * P.kappa1 - beta * P.kappa2;
  const double den = (beta * beta + mu * mu) * (P.kappa1 * P.kappa1 + P.kappa2 * P.kappa2);
  *c2 = (x * x - y * y) / den;
  *s2 = (2.0 * x * y) / den;
}

// Rest-frame path length (Narayan et al. 2021 eq 13; kgeo/equatorial_images.py:489-522):
// disk height diskangle * r times k^t / k^y in the fluid frame, k^t = 1/g, k^y = -k_theta / r.
KG_HD double pathlength_eq(double a, double r, double lam, double eta, double kth, double g, double diskangle) {
  const double TH = eta + a * a * COS2_EQ - lam * lam * COS2_EQ;
  const double kyhat = -(kth * sqrt(TH)) / r;
  return (diskangle * r) * ((1.0 / g) / kyhat);
}

// make_image options beyond the emission model (values of kgeo_image_options).
struct ImageOptions {
  int polarization, pathlength;
  double diskangle;
  FieldModel field;
};

struct PixelOut {
  double I, Q, U, g, sinthb, lp, Ie;
};

// One unmasked order of a pixel with the options (Iobs, kgeo/equatorial_images.py:185-259):
// sin(theta_B) and the EVPA from the field when polarised, one more power of g and |l_p| with
// the path length.
KG_HD void emission_px_opts(const EmissionModel& M, const ImageOptions& P, const Observer& o, const PixelGeo& p,
                            int j, double alpha, double beta, PixelOut* out) {
  const double rs = p.r_s[j];
  const double kr = kr_sign(p, j);
  Ucon<double> u = velocity_t<double>(M, o.a, rs, M.vel_p);
  const double gg = redshift_t<double>(o.a, rs, p.lam, p.eta, kr, u);
  double em = emissivity_t<double>(M, o.a, rs, M.emis_p);
  em = em * pow(gg, M.specind);
  double c2 = 0.0, s2 = 0.0, sb;
  if (P.polarization) {
    const BLab B = bfield_lab(P.field, o.a, rs, o.rplus);
    const PolResult pr = pol_quantities(o.a, rs, p.lam, p.eta, kr, kth_sign(o.th_o, p.m_lo + j), u, B);
    evpa(o.a, o.sin_th, alpha, beta, pr, &c2, &s2);
    sb = pr.sinthb;
    em = em * pow(sb, 1.0 + M.specind);
  } else {
    sb = M.sinthb;
    em = em * M.sinthb_pow;
  }
  double I;
  out->lp = 0.0;
  out->Ie = 0.0;
  if (P.pathlength) {
    const double lp = pathlength_eq(o.a, rs, p.lam, p.eta, kth_sign(o.th_o, p.m_lo + j), gg, P.diskangle);
    em = em * fabs(lp);
    I = pow(gg, 3.0) * em;
    out->lp = lp;
    out->Ie = em;
  } else {
    I = (gg * gg) * em;
  }
  out->I = I;
  out->Q = c2 * I;
  out->U = s2 * I;
  out->g = gg;
  out->sinthb = sb;
}

}  // namespace kg
