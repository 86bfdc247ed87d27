// Unpolarised equatorial image (one ray per pixel, every image order m <= mbar_max) and
// its adjoint with respect to spin, inclination and the emission-model parameters.
//
// Forward: kgeo/equatorial_images.py:124-264 (Iobs with polarization=False and
// pathlength=False) for every order of make_image (:23-122): r_s, Ir, Imax, Nmax from
// r_equatorial, the zero mask (:170-178), the momentum signs (:266-305), the lab-frame
// velocity (kgeo/velocities.py:180-470), the redshift (:307-334) and the emissivity
// (kgeo/emissivities.py:83-160), I = g^2 j g^specind sin(theta_B)^(1 + specind).
//
// Adjoint: the same chain in forward-mode dual numbers. r_s depends on (a, theta_o)
// through the conserved quantities, the angular turning points, the crossing Mino time
// Ir = (2 m K -+ F_o) / sqrt(-a^2 u_-) and the radial inversion r(Ir); the radial roots
// are differentiated implicitly (dr_i = -dR(r_i) / R'(r_i), R' = prod_{j != i} (r_i - r_j))
// and the elliptic functions by the closed forms of kg_dual.cuh. The emission chain then
// carries seven tangents: (a, theta_o, the two emissivity and the three velocity
// parameters).
#pragma once

#include "kg_dual.cuh"
#include "kg_equatorial.cuh"

namespace kg {

// Models (values of kgeo_emission's enums).
enum : int { EMIS_BPL = 0, EMIS_CONSTANT = 1, EMIS_GLM = 2, EMIS_RING = 3 };
enum : int { VEL_ZAMO = 0, VEL_INFALL = 1, VEL_KEP = 2, VEL_SUBKEP = 3, VEL_GENERAL = 4 };

// Orders are processed in groups of ORDER_GROUP per pass over a pixel (any mbar_max).
constexpr int ORDER_GROUP = 4;
constexpr int NQ = 7;  // adjoint tangents: a, theta_o, emis_p[0..1], vel_p[0..2]

// cos(pi/2)**2 and sin(pi/2)**2 of the double nearest pi/2, as the reference's th = pi/2
// evaluates them.
constexpr double COS2_EQ = 3.749399456654644e-33;

struct EmissionModel {
  int emis, vel, retrograde;
  double emis_p[2];  // bpl: p1, p2; glm / ring: gamma_off, sigma
  double mu_ring;    // ring radius (0: glm's 1 - sqrt(1 - a^2))
  double vel_p[3];   // subkep: fac_subkep; general: fac_subkep, beta_phi, beta_r
  double emiscut_in, emiscut_out;
  double specind;
  double sinthb;     // sin(theta_B)
  double sinthb_pow; // sin(theta_B) ** (1 + specind), host-evaluated
};

template <class T>
KG_HD T sign_val(const T& x) {
  return Lift<T>::c(val(x) > 0 ? 1.0 : (val(x) < 0 ? -1.0 : 0.0));
}

// ISCO radius (kgeo/velocities.py:300-302).
template <class T>
KG_HD T r_isco_t(const T& a, double s) {
  T z1 = 1.0 + cbrt(1.0 - a * a) * (cbrt(1.0 + a) + cbrt(1.0 - a));
  T z2 = sqrt(3.0 * (a * a) + z1 * z1);
  return 3.0 + z2 - s * sqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2));
}

template <class T>
struct Ucon {
  T u0, u1, u3;  // u2 = 0 for every supported model
};

// kgeo/velocities.py:180-206 at th = pi/2
template <class T>
KG_HD Ucon<T> u_zamo_t(const T& a, const T& r) {
  T Delta = r * r - 2.0 * r + a * a;
  T Sigma = r * r + (a * a) * COS2_EQ;
  T g00 = -(1.0 - 2.0 * r / Sigma);
  T g11 = Sigma / Delta;
  (void)g11;
  T g33 = (r * r + a * a + 2.0 * r * (a * a) / Sigma);
  T g03 = -2.0 * r * a / Sigma;
  T v3 = -g03 / g33;
  T u0 = sqrt(-1.0 / (g00 + 2.0 * g03 * v3 + g33 * v3 * v3));
  return Ucon<T>{u0, Lift<T>::c(0.0), u0 * v3};
}

// kgeo/velocities.py:211-226
template <class T>
KG_HD Ucon<T> u_infall_t(const T& a, const T& r) {
  T Delta = r * r + a * a - 2.0 * r;
  T ra = r * r + a * a;
  T Xi = ra * ra - Delta * (a * a);
  T u0 = Xi / ((r * r) * Delta);
  T u1 = -sqrt(2.0 * r * (r * r + a * a)) / (r * r);
  T u3 = 2.0 * a / (r * Delta);
  return Ucon<T>{u0, u1, u3};
}

// kgeo/velocities.py:229-281 (Cunningham: Keplerian outside the ISCO, plunging inside)
template <class T>
KG_HD Ucon<T> u_kep_t(const T& a, const T& r, bool retro) {
  const double s = retro ? -1.0 : 1.0;
  T ri = r_isco_t(a, s);
  T spin = sign_val(a) * a;
  T asign = sign_val(a);
  if (val(r) >= val(ri)) {
    T r15 = pow(r, 1.5);
    T Omega = asign * s / (r15 + s * spin);
    T u0 = (r15 + s * spin) / sqrt(r * r * r - 3.0 * (r * r) + 2.0 * s * spin * r15);
    return Ucon<T>{u0, Lift<T>::c(0.0), Omega * u0};
  }
  T Delta = r * r - 2.0 * r + a * a;
  T ell_i = s * asign * (ri * ri + a * a - s * 2.0 * spin * sqrt(ri)) / (pow(ri, 1.5) - 2.0 * sqrt(ri) + s * spin);
  T gam_i = sqrt(1.0 - 2.0 / (3.0 * ri));
  T H = (2.0 * r - a * ell_i) / Delta;
  T u0 = gam_i * (1.0 + (2.0 / r) * (1.0 + H));
  T u1 = -sqrt(2.0 / (3.0 * ri)) * pow(ri / r - 1.0, 1.5);
  T u3 = gam_i * (ell_i + a * H) / (r * r);
  return Ucon<T>{u0, u1, u3};
}

// kgeo/velocities.py:284-359
template <class T>
KG_HD Ucon<T> u_subkep_t(const T& a, const T& r, const T& fac, bool retro) {
  const double s = retro ? -1.0 : 1.0;
  T ri = r_isco_t(a, s);
  T spin = sign_val(a) * a;
  T asign = sign_val(a);
  T Delta = r * r - 2.0 * r + a * a;
  T ra = r * r + a * a;
  T Xi = ra * ra - Delta * (a * a);
  if (val(r) >= val(ri)) {
    T ell = asign * s * (r * r + spin * spin - s * 2.0 * spin * sqrt(r)) / (pow(r, 1.5) - 2.0 * sqrt(r) + s * spin);
    ell = ell * fac;
    T gam = sqrt(Delta / (Xi / (r * r) - 4.0 * a * ell / r - (1.0 - 2.0 / r) * (ell * ell)));
    T H = (2.0 * r - a * ell) / Delta;
    T chi = 1.0 / (1.0 + (2.0 / r) * (1.0 + H));
    T Omega = (chi / (r * r)) * (ell + a * H);
    return Ucon<T>{gam / chi, Lift<T>::c(0.0), (gam / chi) * Omega};
  }
  T Delta_i = ri * ri - 2.0 * ri + a * a;
  T rai = ri * ri + a * a;
  T Xi_i = rai * rai - Delta_i * (a * a);
  T ell_i = asign * s * (ri * ri + spin * spin - s * 2.0 * spin * sqrt(ri)) / (pow(ri, 1.5) - 2.0 * sqrt(ri) + s * spin);
  ell_i = ell_i * fac;
  T gam_i = sqrt(Delta_i / (Xi_i / (ri * ri) - 4.0 * a * ell_i / ri - (1.0 - 2.0 / ri) * (ell_i * ell_i)));
  T H = (2.0 * r - a * ell_i) / Delta;
  T chi = 1.0 / (1.0 + (2.0 / r) * (1.0 + H));
  T Omega = (chi / (r * r)) * (ell_i + a * H);
  T nu = (r / Delta) * sqrt(Xi / (r * r) - 4.0 * a * ell_i / r - (1.0 - 2.0 / r) * (ell_i * ell_i) - Delta / (gam_i * gam_i));
  return Ucon<T>{gam_i / chi, -gam_i * (Delta / (r * r)) * nu, (gam_i / chi) * Omega};
}

// kgeo/velocities.py:442-470
template <class T>
KG_HD Ucon<T> u_general_t(const T& a, const T& r, const T& fac, const T& beta_phi, const T& beta_r, bool retro) {
  T Delta = r * r + a * a - 2.0 * r;
  Ucon<T> ui = u_infall_t(a, r);
  T Om_i = ui.u3 / ui.u0;
  Ucon<T> us = u_subkep_t(a, r, fac, retro);
  T Om_s = us.u3 / us.u0;
  T u1 = us.u1 + (1.0 - beta_r) * (ui.u1 - us.u1);
  T Omega = Om_s + (1.0 - beta_phi) * (Om_i - Om_s);
  T u0 = sqrt(1.0 + (r * r) * (u1 * u1) / Delta);
  T oma = 1.0 - a * Omega;
  u0 = u0 / sqrt(1.0 - (r * r + a * a) * (Omega * Omega) - (2.0 / r) * (oma * oma));
  return Ucon<T>{u0, u1, u0 * Omega};
}

template <class T>
KG_HD Ucon<T> velocity_t(const EmissionModel& M, const T& a, const T& r, const T* vp) {
  switch (M.vel) {
    case VEL_ZAMO: return u_zamo_t(a, r);
    case VEL_INFALL: return u_infall_t(a, r);
    case VEL_KEP: return u_kep_t(a, r, M.retrograde != 0);
    case VEL_SUBKEP: return u_subkep_t(a, r, vp[0], M.retrograde != 0);
    default: return u_general_t(a, r, vp[0], vp[1], vp[2], M.retrograde != 0);
  }
}

// Rest-frame emissivity before the spectral factors (kgeo/emissivities.py:121-139).
template <class T>
KG_HD T emissivity_t(const EmissionModel& M, const T& a, const T& r, const T* ep) {
  switch (M.emis) {
    case EMIS_CONSTANT: return Lift<T>::c(1.0);
    case EMIS_GLM:
    case EMIS_RING: {
      T mu = (M.emis == EMIS_RING && M.mu_ring != 0.0) ? Lift<T>::c(M.mu_ring) : 1.0 - sqrt(1.0 - a * a);
      T x = r - mu;
      T q = ep[0] + asinh(x / ep[1]);
      return exp(-0.5 * (q * q)) / sqrt(x * x + ep[1] * ep[1]);
    }
    default: {
      T rh = 1.0 + sqrt(1.0 - a * a);
      T l = log(r / rh);
      return exp(ep[0] * l + ep[1] * (l * l));
    }
  }
}

// Redshift factor (kgeo/equatorial_images.py:307-334) at th = pi/2 with u2 = 0; the
// theta-momentum term 0 * sqrt(Theta) only contributes a NaN where Theta < 0.
template <class T>
KG_HD T redshift_t(const T& a, const T& r, const T& lam, const T& eta, double kr, const Ucon<T>& u) {
  T a2 = a * a;
  T Delta = r * r - 2.0 * r + a2;
  T q = r * r + a2 - a * lam;
  T lma = lam - a;
  T R = q * q - Delta * (eta + lma * lma);
  double TH = val(eta) + val(a2) * COS2_EQ - val(lam) * val(lam) * COS2_EQ / 1.0;
  T den = u.u0 - lam * u.u3 - kr * u.u1 * sqrt(R) / Delta;
  T g = 1.0 / den;
  if (!(TH >= 0)) g = g + kg_nan();
  return g;
}

KG_HD double kth_sign(double th_o, int m) {
  double p = (m % 2) ? -1.0 : 1.0;
  return th_o < 0.5 * PI ? -p : p;
}

// Per pixel: every order's r_s, Ir and the masks, in double, as the forward pass and the
// adjoint both need them.
struct PixelGeo {
  double lam, eta;
  int m_lo;  // order of r_s[0]
  double r_s[ORDER_GROUP], Ir[ORDER_GROUP];
  double Imax, Nmax;
  double outside;  // is_outside_crit
  double npol;     // nmax_poloidal
  Roots R;
};

// Orders m_lo .. m_lo + n - 1 (n <= ORDER_GROUP).
KG_HD void pixel_geo(const Observer& o, double alpha, double beta, int m_lo, int n, PixelGeo* p) {
  p->lam = -alpha * o.sin_th;
  p->eta = (alpha * alpha - o.a2) * o.cos2 + beta * beta;
  p->m_lo = m_lo;
  EqResult er = r_equatorial_px(o, alpha, beta, m_lo, n, p->r_s, p->Ir, 1);
  p->Imax = er.Imax;
  p->Nmax = er.Nmax;
  p->R = radial_roots(o, p->lam, p->eta);
  p->outside = ((p->R.r4.im == 0) && (p->R.r4.re > o.rplus) && !(p->eta < 0)) ? 1.0 : 0.0;
  if (p->eta <= 0) {
    p->npol = -2;
  } else {
    EqConsts c = eq_consts(o, p->lam, p->eta);
    p->npol = n_pol_at(c, ellip_k(c.ratio), er.Imax);
  }
}

// j: index within the group (order p.m_lo + j)
KG_HD bool image_zero(const EmissionModel& M, const Observer& o, const PixelGeo& p, int j) {
  const int m = p.m_lo + j;
  double rs = p.r_s[j];
  bool z = (p.Nmax < m) || (p.Nmax == -1) || (rs <= o.rplus);
  if (M.emiscut_in > 0) z = z || (rs < M.emiscut_in);
  if (M.emiscut_out > 0) z = z || (rs > M.emiscut_out);
  return z;
}

KG_HD double kr_sign(const PixelGeo& p, int j) {
  return (p.outside == 0.0 || p.Ir[j] <= 0.5 * p.Imax) ? 1.0 : -1.0;
}

// I, g of one unmasked order in double.
KG_HD void emission_px(const EmissionModel& M, const Observer& o, const PixelGeo& p, int j, double* I, double* g) {
  const double rs = p.r_s[j];
  Ucon<double> u = velocity_t<double>(M, o.a, rs, M.vel_p);
  double gg = redshift_t<double>(o.a, rs, p.lam, p.eta, kr_sign(p, j), u);
  double em = emissivity_t<double>(M, o.a, rs, M.emis_p);
  em = em * pow(gg, M.specind);
  em = em * M.sinthb_pow;
  *g = gg;
  *I = (gg * gg) * em;
}

// ---------------------------------------------------------------------------
// adjoint: d r_s / d(a, theta_o)
// ---------------------------------------------------------------------------

using D2 = Dual<2>;

// Radial roots with their tangents, from the double roots by implicit differentiation of
// R(r) = r^4 + A r^2 + B r + C (kgeo/kerr_raytracing_utils.py:342-345).
struct DRoots {
  D2 re[4], im[4];
};

KG_HD DRoots droots(const Roots& R, const D2& a2, const D2& lam, const D2& eta, const D2& a) {
  D2 A = a2 - eta - lam * lam;
  D2 lma = lam - a;
  D2 B = 2.0 * (eta + lma * lma);
  D2 C = -(a2 * eta);
  const cplx r[4] = {R.r1, R.r2, R.r3, R.r4};
  DRoots out;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    cplx dR = cx_real(1.0);
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (j != i) dR = dR * (r[i] - r[j]);
    cplx r2 = r[i] * r[i];
    out.re[i] = dconst<2>(r[i].re);
    out.im[i] = dconst<2>(r[i].im);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      cplx num = cx_real(A.d[k]) * r2 + cx_real(B.d[k]) * r[i] + cx_real(C.d[k]);
      cplx dr = -(num / dR);
      out.re[i].d[k] = dr.re;
      out.im[i].d[k] = dr.im;
    }
  }
  return out;
}

// sn, cn of X (any real X) through the half-period reduction, as radial_r_at does it.
KG_HD void dual_jacobi_reduced(const D2& X, const D2& m, D2* sn, D2* cn) {
  D2 K2 = 2.0 * dual_ellip_k(m);
  double nr = rint(X.v / K2.v);
  D2 v = X - nr * K2;
  D2 dn;
  dual_jacobi(v, m, sn, cn, &dn);
  if (fmod(fabs(nr), 2.0) == 1.0) {
    *sn = -(*sn);
    *cn = -(*cn);
  }
}

// r(tau) of radial_r_at in dual numbers.
KG_HD D2 radial_r_dual(const Observer& o, const Roots& R, const DRoots& D, const D2& tau) {
  const double r_o = o.r_o;
  bool c4 = R.r1.im != 0;
  bool c3 = (R.r3.im != 0) && !c4;
  if (c4) {
    D2 a1 = D.im[3], b1 = D.re[3], a2i = D.im[1], b2 = D.re[1];
    D2 CC = sqrt((a1 - a2i) * (a1 - a2i) + (b1 - b2) * (b1 - b2));
    D2 DD = sqrt((a1 + a2i) * (a1 + a2i) + (b1 - b2) * (b1 - b2));
    D2 k4 = (4.0 * CC * DD) / ((CC + DD) * (CC + DD));
    D2 g0 = sqrt((4.0 * (a2i * a2i) - (CC - DD) * (CC - DD)) / ((CC + DD) * (CC + DD) - 4.0 * (a2i * a2i)));
    D2 at_o = o.r_o_inf ? dconst<2>(HALFPI) : atan((r_o + b1) / a2i);
    D2 aux = at_o + atan(g0);
    D2 pref = 2.0 / (CC + DD);
    D2 Ir_o = pref * dual_ellip_f(aux, k4);
    D2 X4 = (1.0 / pref) * (Ir_o - tau);
    D2 sn, cn;
    dual_jacobi_reduced(X4, k4, &sn, &cn);
    D2 sc = sn / cn;
    return -a2i * (g0 - sc) / (1.0 + g0 * sc) - b1;
  }
  if (c3) {
    D2 a1 = D.im[3], b1 = D.re[3], rr1 = D.re[0], rr2 = D.re[1];
    D2 rr21 = rr2 - rr1;
    D2 AA = sqrt(a1 * a1 + (b1 - rr2) * (b1 - rr2));
    D2 BB = sqrt(a1 * a1 + (b1 - rr1) * (b1 - rr1));
    D2 k3 = ((AA + BB) * (AA + BB) - rr21 * rr21) / (4.0 * AA * BB);
    D2 x3ro = o.r_o_inf ? (AA - BB) / (AA + BB)
                        : (AA * (r_o - rr1) - BB * (r_o - rr2)) / (AA * (r_o - rr1) + BB * (r_o - rr2));
    D2 aux = acos(x3ro);
    D2 pref = 1.0 / sqrt(AA * BB);
    D2 Ir_o = pref * dual_ellip_f(aux, k3);
    D2 X3 = (1.0 / pref) * (Ir_o - tau);
    D2 sn, cn;
    dual_jacobi_reduced(X3, k3, &sn, &cn);
    return ((BB * rr2 - AA * rr1) + (BB * rr2 + AA * rr1) * cn) / ((BB - AA) + (BB + AA) * cn);
  }
  D2 rr1 = D.re[0], rr2 = D.re[1], rr3 = D.re[2], rr4 = D.re[3];
  D2 rr31 = rr3 - rr1, rr32 = rr3 - rr2, rr41 = rr4 - rr1, rr42 = rr4 - rr2;
  D2 k2 = (rr32 * rr41) / (rr31 * rr42);
  D2 x2ro = o.r_o_inf ? sqrt(rr31 / rr41) : sqrt((rr31 * (r_o - rr4)) / (rr41 * (r_o - rr3)));
  D2 aux = asin(x2ro);
  D2 s3142 = sqrt(rr31 * rr42);
  D2 Ir_o = 2.0 * dual_ellip_f(aux, k2) / s3142;
  D2 X2 = 0.5 * s3142 * (Ir_o - tau);
  D2 sn, cn;
  dual_jacobi_reduced(X2, k2, &sn, &cn);
  D2 sn2 = sn * sn;
  return (rr4 * rr31 - rr3 * rr41 * sn2) / (rr31 - rr41 * sn2);
}

// d r_s / d(a, theta_o) for the n orders of the group of a pixel with eta > 0 (value
// slots are the dual path's own evaluation; the caller keeps the forward values).
KG_HD void rs_tangents(const Observer& o, double alpha, double beta, const PixelGeo& p, int n, D2* rs) {
  D2 a = dvar<2>(o.a, 0);
  D2 sin_t, cos_t;
  sin_t.v = o.sin_th; sin_t.d[0] = 0.0; sin_t.d[1] = o.cos_th;
  cos_t.v = o.cos_th; cos_t.d[0] = 0.0; cos_t.d[1] = -o.sin_th;
  D2 cos2 = cos_t * cos_t;
  D2 a2 = a * a;
  D2 lam = -alpha * sin_t;
  D2 eta = (alpha * alpha - a2) * cos2 + beta * beta;
  // u_+-, clamps of u_turning (eta > 0 here)
  D2 up, um, ratio, a2um;
  if (o.minspin) {
    up = eta / (eta + lam * lam);
    if ((o.cos2 - up.v) > 0) up = cos2;
    if (up.v * up.v > 1) up = dconst<2>(1.0);
    if (up.v == 0) up = dconst<2>(-EP);
    um = up;
    ratio = dconst<2>(0.0);
    a2um = -(eta + lam * lam);
  } else {
    D2 half = 0.5 * (1.0 - (eta + lam * lam) / a2);
    D2 root = sqrt(half * half + eta / a2);
    up = half + root;
    um = half - root;
    if ((o.cos2 - up.v) > 0) up = cos2;
    if (up.v * up.v > 1) up = dconst<2>(1.0);
    if (um.v == 0) um = dconst<2>(-EP);
    ratio = up / um;
    a2um = a2 * um;
  }
  D2 F0 = dual_ellip_f(asin(cos_t / sqrt(up)), ratio);
  D2 K = dual_ellip_f(dconst<2>(0.5 * PI), ratio);
  D2 sqa = sqrt(-a2um);
  DRoots DR = droots(p.R, a2, lam, eta, a);
  const bool north = o.th_o < (PI / 2.);
  for (int j = 0; j < n; ++j) {
    double mbar = (double)(p.m_lo + j);
    D2 ir;
    if (north) {
      double m = mbar + (beta > 0 ? 1.0 : 0.0);
      ir = beta <= 0 ? (2.0 * m * K + F0) / sqa : (2.0 * m * K - F0) / sqa;
    } else {
      double m = mbar + (-beta > 0 ? 1.0 : 0.0);
      ir = beta >= 0 ? (2.0 * m * K - F0) / sqa : (2.0 * m * K + F0) / sqa;
    }
    rs[j] = radial_r_dual(o, p.R, DR, ir);
  }
}

// dI/dq for one unmasked order: the emission chain in Dual<NQ> from r_s with tangents.
KG_HD Dual<NQ> emission_dual(const EmissionModel& M, const Observer& o, const PixelGeo& p, int j, double alpha,
                             double beta, const D2& rs2) {
  using DQ = Dual<NQ>;
  DQ a = dvar<NQ>(o.a, 0);
  DQ sin_t = dconst<NQ>(o.sin_th), cos_t = dconst<NQ>(o.cos_th);
  sin_t.d[1] = o.cos_th;
  cos_t.d[1] = -o.sin_th;
  DQ lam = -alpha * sin_t;
  DQ eta = (alpha * alpha - a * a) * (cos_t * cos_t) + beta * beta;
  DQ rs = dconst<NQ>(p.r_s[j]);
  rs.d[0] = rs2.d[0];
  rs.d[1] = rs2.d[1];
  DQ ep[2] = {dvar<NQ>(M.emis_p[0], 2), dvar<NQ>(M.emis_p[1], 3)};
  DQ vp[3] = {dvar<NQ>(M.vel_p[0], 4), dvar<NQ>(M.vel_p[1], 5), dvar<NQ>(M.vel_p[2], 6)};
  Ucon<DQ> u = velocity_t<DQ>(M, a, rs, vp);
  DQ g = redshift_t<DQ>(a, rs, lam, eta, kr_sign(p, j), u);
  DQ em = emissivity_t<DQ>(M, a, rs, ep);
  em = em * pow(g, M.specind);
  em = em * M.sinthb_pow;
  return (g * g) * em;
}

}  // namespace kg
