/*
 * kgeo_gb300 C ABI: the analytic Kerr null-geodesic tracer on one GB300 (sm_103a).
 *
 * Every entry point is stream-ordered and takes device pointers (CUDA global
 * memory) sized as documented; nothing is copied to or from the host except
 * where a function says so. Arrays of samples are (n_samples, npix) row-major,
 * the layout of the reference's numpy output. Any output pointer may be NULL,
 * in which case that output is not written. Return values are kgeo_status codes;
 * conditions only known on the device (see KGEO_FLAG_*) are reported in the
 * caller-visible flags word after the stream has run.
 *
 * The reference (achael/kgeo) is a Python library with no FFI; each declaration
 * below names the Python call it replaces (file:line in the reference).
 */
#ifndef KGEO_GB300_H
#define KGEO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KGEO_ABI_VERSION 2

/* Return codes. The argument errors correspond one-to-one to the reference's
 * exceptions (kgeo/kerr_raytracing_ana.py:59-71, kgeo/equatorial_lensing.py:100-101). */
typedef enum {
  KGEO_OK = 0,
  KGEO_ERR_SPIN = 1,        /* "|a| should be a float in range [0,1)" */
  KGEO_ERR_R_O = 2,         /* "r_o should be a float > 100" */
  KGEO_ERR_TH_O = 3,        /* "th_o should be a float in range (0,pi/2) or (pi/2,pi)" */
  KGEO_ERR_LENGTHS = 4,     /* "alpha, beta are different lengths!" / bad npix */
  KGEO_ERR_NGEO = 5,        /* negative sample count */
  KGEO_ERR_MBAR = 6,        /* "mbar should be an integer >=0!" */
  KGEO_ERR_WORKSPACE = 7,   /* workspace too small */
  KGEO_ERR_NULL = 8,        /* a required pointer is NULL */
  KGEO_ERR_CUDA = 9,        /* a CUDA runtime call failed */
  KGEO_ERR_MODEL = 10,      /* unknown / out-of-range emissivity, velocity or B-field model parameter, or image option */
  KGEO_ERR_NOALLOC_SIZE = 11, /* npix above KGEO_NOALLOC_MAX_PIXELS for kgeo_raytrace_noalloc */
  KGEO_ERR_SOLVER = 12      /* root-solver arguments: xtol <= 0, rtol < 4 eps, maxiter < 0 (scipy brentq's checks) */
} kgeo_status;

/* Arithmetic of the sample kernels. FP64: every output within the FP64 parity bars.
 * MIXED: the recurrence on the FP32 pipe — Jacobi states, integral accumulators, r and the
 * sums into t, phi, sigma in float-float (two FP32 words, ~48 bits), the Pi / E increments as a
 * float-float leading term plus an FP32 correction, theta from an FP32 atan2; FP64 at chunk
 * starts, next to an elliptic-Pi pole and at the final horizon-adjacent sample. Measured against
 * the FP64 oracle on 2048^2 images: r <= 5e-9, theta <= 2e-7, t and sigma <= 1.3e-8 of r_o, phi
 * within max(1e-6, 1e-12 / rho) where rho is the distance to the nearest elliptic-Pi pole. */
#define KGEO_PRECISION_FP64 0
#define KGEO_PRECISION_MIXED 1

/* Bits of the device flags word written by the tracing entry points. */
#define KGEO_FLAG_ANY_ETA_POS 1u
#define KGEO_FLAG_ANY_ETA_NONPOS 2u
#define KGEO_FLAG_ANY_STEP_ZERO 4u
/* |a| < 1e-4 and some pixel has eta == 0: the reference raises
 * "below MINSPIN but there are eta<0 points in th_integrate!" (kgeo/kerr_raytracing_ana.py:301-302) */
#define KGEO_FLAG_MINSPIN_VORTICAL 8u
/* An iterative loop of the elliptic arithmetic (Carlson duplication, descending Landen
 * transformation) stopped at its iteration cap without meeting its convergence test; the
 * affected samples may be inaccurate. The reference surfaces such failures as NaN or as an
 * exception (kgeo/gsl_ellip_binding.py:92-136); the caps are far above FP64 convergence, so
 * on finite inputs this bit is not expected. */
#define KGEO_FLAG_LOOP_CAP 16u

/* Observer: spin a (|a| < 1), radius r_o (>= 100, may be +inf), inclination th_o in (0, pi) minus pi/2. */
typedef struct {
  double a;
  double r_o;
  double th_o;
} kgeo_observer;

/* Outputs of a trace. Sample arrays are (n_samples, npix); per-pixel arrays are (npix). */
typedef struct {
  double* t;          /* Boyer-Lindquist t */
  double* r;          /* r */
  double* th;         /* theta */
  double* ph;         /* phi */
  double* sig;        /* affine parameter sigma (Geodesics.affine_times) */
  double* mino;       /* Mino time tau of each sample (Geodesics.mino_times) */
  double* tau_tot;    /* total Mino time per pixel (before maxtaufrac) */
  int32_t* rclass;    /* radial class 1..4 (kgeo/kerr_raytracing_utils.py:365-378) */
  int32_t* thclass;   /* angular class 1..3 (kgeo/kerr_raytracing_utils.py:265-272) */
  uint32_t* flags;    /* one device word, KGEO_FLAG_* bits (cleared by the call) */
} kgeo_geodesics;

/* Bytes of device scratch that kgeo_raytrace / kgeo_coords_at_tau need for npix pixels. */
size_t kgeo_workspace_size(int64_t npix);

/* raytrace_ana(a, observer_coords, image_coords, ngeo, maxtaufrac)
 * (kgeo/kerr_raytracing_ana.py:46-122): ngeo samples per pixel, evenly spaced in Mino
 * time from 0 to maxtaufrac * tau_tot (numpy.linspace arithmetic).
 * alpha, beta: (npix) device arrays. workspace: device scratch of at least
 * kgeo_workspace_size(npix) bytes, or NULL to let the call allocate (and free) it
 * stream-ordered. stream: a cudaStream_t (NULL = default stream). */
int kgeo_raytrace(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                  int32_t ngeo, double maxtaufrac, kgeo_geodesics* out, void* workspace,
                  size_t workspace_bytes, void* stream);

/* kgeo_raytrace with the mixed-precision sample kernel (KGEO_PRECISION_MIXED); same
 * arguments and outputs. */
int kgeo_raytrace_mixed(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                        int32_t ngeo, double maxtaufrac, kgeo_geodesics* out, void* workspace,
                        size_t workspace_bytes, void* stream);

/* raytrace_ana with HOST buffers end to end (kgeo/kerr_raytracing_ana.py:46-122, the call a
 * numpy caller makes): alpha, beta (npix) and every non-NULL output of `out` (t, r, th, ph,
 * sig, mino (ngeo, npix) row-major; tau_tot, rclass, thclass (npix); flags, one word) are
 * host pointers. Results equal kgeo_raytrace / kgeo_raytrace_mixed (precision =
 * KGEO_PRECISION_FP64 / _MIXED). When every sample output is page-locked host memory that the
 * device can address (cudaHostAlloc, cudaHostRegister: cudaPointerGetAttributes reports a device
 * pointer for it), the sample kernel stores into the host outputs directly (48 B per sample over
 * the host link, no staging, no copy engine). Otherwise the samples are computed in windows of
 * whole recurrence chunks into a ring of device buffers, and each window is copied to the host
 * on a second stream while the next one computes; pageable outputs work but serialise. On GB300
 * the direct stores keep the call at the kernels' own time, where the copy engine's rate varies
 * several-fold while FP64 kernels run beside it. workspace: device scratch of
 * kgeo_raytrace_host_workspace_size(npix, ngeo, precision) bytes, or NULL (allocated and freed
 * stream-ordered). The call returns once the work is queued on `stream`; the host outputs are
 * complete when that stream has synchronised. */
size_t kgeo_raytrace_host_workspace_size(int64_t npix, int32_t ngeo, int32_t precision);
int kgeo_raytrace_host(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                       int32_t ngeo, double maxtaufrac, int32_t precision, kgeo_geodesics* out, void* workspace,
                       size_t workspace_bytes, void* stream);

/* coords_at_tau(a, observer_coords, image_coords, tau, do_phi_and_t)
 * (kgeo/kerr_raytracing_ana.py:126-193): coordinates at caller-given Mino times
 * tau (ntau, npix). With do_phi_and_t == 0 only r and theta are meaningful
 * (t, ph, sig are written as the reference leaves them: zero-based partial sums). */
int kgeo_coords_at_tau(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                       const double* tau, int32_t ntau, int32_t do_phi_and_t, kgeo_geodesics* out,
                       void* workspace, size_t workspace_bytes, void* stream);

/* The two halves of kgeo_raytrace, for callers that sample the same rays repeatedly
 * (e.g. at new Mino times inside an iterative solver):
 * kgeo_ray_setup evaluates every per-ray quantity (conserved quantities, turning points,
 * radial roots and class, Mino totals, antiderivative constants: the per-pixel part of
 * kgeo/kerr_raytracing_ana.py:76-94 and 151-167 and of kgeo/kerr_raytracing_utils.py:242-548)
 * into the caller's workspace; per_ray may carry tau_tot / rclass / thclass outputs (the
 * sample pointers are ignored). ngeo is the linspace length the samples will use (0 if
 * tau is given later).
 * kgeo_ray_samples evaluates t, r, theta, phi, sigma (and the Mino times) of those rays:
 * at tau (nsamp, npix) when tau is non-NULL, else at the ngeo-point linspace of the setup
 * (the sample loop of kgeo/kerr_raytracing_ana.py:169-188). The workspace must not be
 * modified between the two calls. chunk selects the evaluation of the even grid: 0 evaluates
 * every sample independently (Landen + Carlson per sample); k > 0 gives each thread k
 * consecutive samples, the first (and the grid's last) evaluated directly and the rest by
 * the addition theorems of sn/cn/dn, E and Pi from the previous sample (k is capped at 64,
 * 256 for KGEO_PRECISION_MIXED);
 * < 0 picks the library default. Caller-given tau always uses independent evaluation.
 * precision: KGEO_PRECISION_FP64 or KGEO_PRECISION_MIXED (the latter for the recurrence). */
int kgeo_ray_setup(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix, int32_t ngeo,
                   double maxtaufrac, void* workspace, size_t workspace_bytes, kgeo_geodesics* per_ray,
                   void* stream);
int kgeo_ray_samples(const kgeo_observer* obs, const void* workspace, size_t workspace_bytes, int64_t npix,
                     const double* tau, int32_t nsamp, int32_t do_phi_and_t, int32_t chunk, int32_t precision,
                     kgeo_geodesics* out, void* stream);

/* r_equatorial(a, r_o, th_o, mbar, alpha, beta) (kgeo/equatorial_lensing.py:85-196) for the
 * orders mbar = mbar_lo .. mbar_lo + n_orders - 1 in one pass: r_s and Ir are (n_orders, npix),
 * Imax and Nmax (npix) are order-independent (either may be NULL). Vortical pixels
 * (eta <= 0) get r_s = Ir = Imax = -1, Nmax = -2; r_s = 0 where Nmax < mbar. */
int kgeo_r_equatorial(const kgeo_observer* obs, int32_t mbar_lo, int32_t n_orders, const double* alpha,
                      const double* beta, int64_t npix, double* r_s, double* Ir, double* Imax, double* Nmax,
                      void* stream);

/* Per-pixel crossing counts at Mino times tau (ntau, npix):
 * n_eq  = n_equatorial_crossings (kgeo/kerr_raytracing_utils.py:605-684; Geodesics.nmax_eq),
 * n_pol = n_poloidal_orbits (kgeo/kerr_raytracing_utils.py:551-603; Geodesics.n_poloidal),
 * and outside_crit (npix) = is_outside_crit (kgeo/kerr_raytracing_utils.py:794-826).
 * Any of the three outputs may be NULL; tau is only read when n_eq or n_pol is requested. */
int kgeo_equatorial_crossings(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                              const double* tau, int32_t ntau, double* n_eq, double* n_pol,
                              double* outside_crit, void* stream);

/* n_angular_turnings (kgeo/kerr_raytracing_utils.py:686-792): the fractional number of
 * angular turning points passed by Mino time tau (ntau, npix), n_turn (ntau, npix), including
 * the reference's provisional rule for vortical rays. Its check: 0 <= th_o <= pi/2
 * (KGEO_ERR_TH_O otherwise; r_o is not used). */
int kgeo_angular_turnings(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                          const double* tau, int32_t ntau, double* n_turn, void* stream);

/* Emission model of an unpolarised equatorial image: Emissivity(emistype, **kwargs)
 * (kgeo/emissivities.py:38-72) and Velocity(veltype, **kwargs) (kgeo/velocities.py:23-67)
 * restricted to the models below, plus Iobs' specind and sin(theta_B)
 * (kgeo/equatorial_images.py:17-20). */
#define KGEO_EMIS_BPL 0        /* emisBPL: exp(p1 ln(r/r_h) + p2 ln^2(r/r_h)) */
#define KGEO_EMIS_CONSTANT 1   /* 1 */
#define KGEO_EMIS_GLM 2        /* emisGLM with mu = 1 - sqrt(1 - a^2) */
#define KGEO_EMIS_RING 3       /* emisGLM with mu = mu_ring (0: as GLM) */
#define KGEO_VEL_ZAMO 0
#define KGEO_VEL_INFALL 1
#define KGEO_VEL_KEP 2         /* 'kep' / 'cunningham' */
#define KGEO_VEL_SUBKEP 3      /* 'subkep' / 'cunningham_subkep' */
#define KGEO_VEL_GENERAL 4
typedef struct {
  int32_t emissivity;   /* KGEO_EMIS_* */
  int32_t velocity;     /* KGEO_VEL_* */
  int32_t retrograde;   /* kep / subkep / general */
  int32_t reserved;
  double emis_p[2];     /* bpl: (p1, p2); glm / ring: (gamma_off, sigma) */
  double mu_ring;       /* ring: r_ring */
  double vel_p[3];      /* subkep: (fac_subkep); general: (fac_subkep, beta_phi, beta_r), each in [0, 1] */
  double emiscut_in;    /* pixels with r_s < emiscut_in are dark when emiscut_in > 0 */
  double emiscut_out;   /* pixels with r_s > emiscut_out are dark when emiscut_out > 0 */
  double specind;       /* spectral index (1 in make_image) */
  double sinthb;        /* sin(theta_B) of the unpolarised image (pi/4 in the reference) */
} kgeo_emission;

/* Outputs of kgeo_image. Per-order arrays are (npix, n_orders) row-major, the layout of
 * make_image's outarr_*; I is required, every other pointer may be NULL. */
typedef struct {
  double* I;        /* observed intensity g^2 j g^specind sin(theta_B)^(1 + specind), 0 where masked */
  double* g;        /* redshift factor, 0 where masked */
  double* r_s;      /* emission radius (r_equatorial's r_s) */
  double* Ir;       /* Mino time of the crossing (make_image's outarr_t) */
  double* sinthb;   /* sin(theta_B) where lit, else 0 */
  double* imax;     /* (npix) Imax, the total Mino time (Iobs' Imax) */
  double* nmax;     /* (npix) Nmax, make_image's outarr_n */
  double* npol;     /* (npix) nmax_poloidal, make_image's outarr_np */
  double* Q;        /* kgeo_image_ex with polarization: cos(2 chi) I (make_image's outarr_Q) */
  double* U;        /* kgeo_image_ex with polarization: sin(2 chi) I (outarr_U) */
  double* lp;       /* kgeo_image_ex with pathlength: rest-frame path length (outarr_lp) */
  double* Ie;       /* kgeo_image_ex with pathlength: emission before g^3 (outarr_Ie) */
} kgeo_image_out;

/* make_image(a, r_o, th_o, mbar_max, ...) with polarization=False, pathlength=False
 * (kgeo/equatorial_images.py:23-122; per order Iobs, :124-264) on the caller's pixels
 * (alpha, beta), for the orders mbar = mbar_lo .. mbar_lo + n_orders - 1 in one pass over the
 * pixels (make_image: mbar_lo = 0, n_orders = mbar_max + 1; Iobs: one order). Q and U of the
 * reference are zero in this mode and are not produced. The threads take the pixels in
 * radial-class order (a deterministic counting sort into about 8 B per pixel of stream-ordered
 * scratch, cudaMallocAsync / cudaFreeAsync on the stream); every output stays at its pixel. */
int kgeo_image(const kgeo_observer* obs, int32_t mbar_lo, int32_t n_orders, const double* alpha, const double* beta,
               int64_t npix, const kgeo_emission* model, kgeo_image_out* out, void* stream);

/* Lab-frame magnetic field of a polarised image: Bfield(fieldtype, **kwargs).bfield_lab
 * (kgeo/bfields.py:33-131; model functions :429-736) in the equatorial plane. Only the
 * lab-frame B^i enter the image (calc_polquantities, kgeo/equatorial_images.py:336-487). */
#define KGEO_BFIELD_SIMPLE 0       /* 'simple', 'rad' (1,0,0), 'vert' (0,1,0), 'tor' (0,0,1): c = (Cr, Cvert, Cph) */
#define KGEO_BFIELD_SIMPLE_RM1 1   /* 'simple_rm1': c = (Cr, Cvert, Cph) */
#define KGEO_BFIELD_MONOPOLE_A 2   /* 'monopoleA': c = (C, omegafac) */
#define KGEO_BFIELD_BZ_GUESS 3     /* 'bz_guess': c = (C) */
#define KGEO_BFIELD_BZ_MONOPOLE 4  /* 'bz_monopole': c = (C); flag = secondorder_only. f(r) in closed form */
#define KGEO_BFIELD_BZ_PARA 5      /* 'bz_para': c = (C) */
#define KGEO_BFIELD_POWER 6        /* 'power': c = (C, p); flag = usemono */
#define KGEO_BFIELD_GEN_POWER 7    /* 'gen_power': c = (n_I, p_val); flag = isAbove */
typedef struct {
  int32_t field;  /* KGEO_BFIELD_* */
  int32_t flag;
  double c[3];
} kgeo_bfield;

/* make_image / Iobs options beyond the emission model (kgeo/equatorial_images.py:23-32). */
typedef struct {
  int32_t polarization;  /* sin(theta_B) and the EVPA from the field: calc_polquantities + calc_evpa (:524-544) */
  int32_t pathlength;    /* I = g^3 j |l_p|, l_p from calc_pathlength_equatorial (:489-522) */
  double diskangle;      /* full opening angle h/r of the disk for the path length (0.1 in the reference) */
  kgeo_bfield bfield;    /* read when polarization != 0 */
} kgeo_image_options;

/* kgeo_image with options: make_image(..., bfield, polarization, pathlength, diskangle)
 * (kgeo/equatorial_images.py:23-122, Iobs :124-264). options == NULL is kgeo_image. With
 * polarization, sinthb is the computed sin(theta_B) and Q, U are written when non-NULL;
 * with pathlength, lp and Ie are written when non-NULL. The reference's make_image raises
 * for 'bz_para' with polarization=True (its complex-typed Omega reaches an in-place float
 * multiply); here the field's real value is used. */
int kgeo_image_ex(const kgeo_observer* obs, int32_t mbar_lo, int32_t n_orders, const double* alpha,
                  const double* beta, int64_t npix, const kgeo_emission* model, const kgeo_image_options* options,
                  kgeo_image_out* out, void* stream);

/* Adjoint of kgeo_image's I (no counterpart in the reference): given grad_I = dL/dI
 * (npix, n_orders) for the orders mbar_lo .. mbar_lo + n_orders - 1, writes grad[7] = dL/dq for q = (a, th_o, emis_p[0], emis_p[1],
 * vel_p[0], vel_p[1], vel_p[2]) to device memory. Masks, the momentum signs and Nmax are
 * held fixed (they are piecewise constant); the geodesic is recomputed, not stored.
 * workspace: device scratch of kgeo_image_adjoint_workspace_size(npix) bytes (per-block partial
 * sums, then the radial-class pixel order of kgeo_image). Deterministic: the pixel order comes
 * from a counting sort without atomics in its ranks, and the per-block partial sums are added
 * in a fixed order. */
size_t kgeo_image_adjoint_workspace_size(int64_t npix);
int kgeo_image_adjoint(const kgeo_observer* obs, int32_t mbar_lo, int32_t n_orders, const double* alpha,
                       const double* beta, int64_t npix, const kgeo_emission* model, const double* grad_I, double* grad,
                       void* workspace, size_t workspace_bytes, void* stream);

/* Lensed curves of constant equatorial radius: rho_of_req / rho_of_req_single
 * (kgeo/equatorial_lensing.py:223-258) for many curves at once. Curve c is the image-plane
 * curve rho(varphi) on which the mbar-th equatorial crossing of the ray at
 * (alpha, beta) = rho (cos varphi, sin varphi) lies at r_eq, for an observer at r_o = inf
 * (equatorial_lensing.R0): at every angle, the root of objfunc (r_s of r_equatorial with the
 * reference's fill-ins INF / 1 where there is no crossing, minus r_eq; :198-221) on
 * [rho_min, rho_max] by Brent's method with scipy.optimize.brentq's convergence test
 * (xtol, rtol; its defaults are 2e-12, 4 eps, 100). curves: host array; varphi (nphi), rho and
 * status (ncurves, nphi) row-major: device arrays. status (may be NULL):
 * KGEO_CURVE_SIGN where f(rho_min), f(rho_max) have the same sign (rho = NaN; brentq raises),
 * KGEO_CURVE_MAXITER where maxiter steps did not converge (brentq raises). One launch over all
 * (curve, angle) pairs: a whole curve library (make_curves2 / generate_library, :327-423) is one
 * call. */
#define KGEO_CURVE_OK 0
#define KGEO_CURVE_SIGN 1
#define KGEO_CURVE_MAXITER 2
typedef struct {
  double a, th_o;           /* spin and inclination (the kgeo_observer rules; r_o = inf) */
  double r_eq;              /* equatorial radius of the curve */
  double rho_min, rho_max;  /* bracket (rho_of_req: mbar 0: (0, r_eq + 5); 1: (0, 100); else (1, 10)) */
  int32_t mbar;             /* image order >= 0 */
  int32_t reserved;
} kgeo_curve;
int kgeo_rho_of_req(const kgeo_curve* curves, int32_t ncurves, const double* varphi, int32_t nphi, double xtol,
                    double rtol, int32_t maxiter, double* rho, int32_t* status, void* stream);

/* critical_curve(a, th0, n) (kgeo/equatorial_lensing.py:260-289) before its mask: the n
 * points of r = linspace(r_-, r_+, n) over the prograde / retrograde spherical photon orbit
 * radii, mapped to the screen (alpha, beta >= 0); a point the reference drops has alpha or beta
 * NaN. alpha, beta: (n) device arrays. */
int kgeo_critical_curve(double a, double th_o, int64_t n, double* alpha, double* beta, void* stream);

/* Crossings of the geodesics with a jet field line psi(r, theta) = psi_target
 * (kgeo/solver.py:14-207; the solver of the off-equatorial model, kgeo/off_eq.py:124-172).
 * Field lines: KGEO_JET_PARA psi_BZ_para (the BZ paraboloid), KGEO_JET_MONO psi_BZ_mono,
 * KGEO_JET_POWER r^p (1 - |cos theta|). */
#define KGEO_JET_PARA 0
#define KGEO_JET_MONO 1
#define KGEO_JET_POWER 2
typedef struct {
  int32_t model;     /* KGEO_JET_* */
  int32_t reserved;
  double psitarget;  /* psi of the field line */
  double pval;       /* power: p */
} kgeo_jet_field;

/* getguesses (kgeo/solver.py:97-134) on a sampled geodesic set: r, th, mino (ngeo, npix)
 * device arrays (kgeo_raytrace's outputs) and the pixels alpha, beta. count (npix, may be
 * NULL): the number of Mino-time guesses of each pixel (the sign changes of psi - psi_target
 * before the search bound of get_maxtau_forwardjet, endpoints excluded; 2 for the flat-space
 * guesses of a nearly face-on view at impact parameter > 100; 1 (the guess -1) when there is
 * none). guesses (nguess, npix, may be NULL): the guesses padded with -1 (pixels with more than
 * nguess are all -1: size nguess from max(count)). taumax (npix, may be NULL): the bound
 * (get_maxtau_forwardjet, :57-87); with r == NULL only taumax is computed. neqmax <= 0: no
 * bound but the total Mino time. */
int kgeo_jet_guesses(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                     const double* r, const double* th, const double* mino, int32_t ngeo,
                     const kgeo_jet_field* field, int32_t neqmax, double* taumax, int32_t* count, double* guesses,
                     int32_t nguess, void* stream);

/* findroot (kgeo/solver.py:136-207): from each guess (nguess, npix), the Mino time tau of the
 * crossing by the secant iteration of scipy.optimize.newton (tol on the step, maxiter steps),
 * the coordinates r, th there, the signs of p_r and p_theta (from the coordinates at
 * tau (1 + 1e-5)) and neq, the equatorial crossings before tau (getneq, :40-55). Entries of a
 * -1 guess are 0 but neq. Every output is (nguess, npix), device memory; any but tau may be
 * NULL; status (may be NULL): 0 converged, 1 not within maxiter (scipy warns). workspace: device
 * scratch of kgeo_workspace_size(npix) bytes or NULL. */
int kgeo_jet_findroot(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                      const double* guesses, int32_t nguess, const kgeo_jet_field* field, double tol, int32_t maxiter,
                      void* workspace, size_t workspace_bytes, double* tau, double* r, double* th, double* signpr,
                      double* signpth, double* neq, int32_t* status, void* stream);

/* getstokes (kgeo/off_eq.py:124-233) after findroot, for the monopole field-line model:
 * the Stokes I, Q, U of every crossing (Iobs_off, :15-119: constant emissivity times the
 * continuity-equation density of kgeo/densityfuncs.py:47-78, the force-free drift-frame
 * velocity of kgeo/velocities.py:487-623 with a numeric parallel boost, the polarisation of
 * calc_polquantities with its path length and comoving b^2), summed over the guess rows into
 * the images of neq = 0 .. neqmax - 1 and their total (sort_image, kgeo/geometry.py:38-61), and
 * the EVPA 0.5 atan2(U, Q) of each. The density's stagnation radius comes from the first
 * crossing of the first guess row (kgeo/densityfuncs.py:47-60, kgeo/ff_boost.py:7-18).
 * r, th, signpr, signpth, neq: (nguess, npix) device arrays, kgeo_jet_findroot's outputs.
 * I, Q, U, evpa: (neqmax + 1, npix) device outputs (evpa may be NULL); I_c, Q_c, U_c (may be
 * NULL): (nguess, npix) per crossing; stagnation (may be NULL): device (2) r0, Omega_F;
 * status (may be NULL): device (1), 0 ok, 1 no crossing in the first row, 2 or 3 no stagnation
 * root (a = 0 or a crossing on the axis; the reference fails on both), with all images 0.
 * The BZ f(r) is the linear interpolant of its values on linspace(1, 100, 100000) as the
 * reference evaluates it (kgeo/bfields.py:16-31); the first call on a device builds that table
 * (one synchronous kernel). */
typedef struct {
  int32_t model;       /* KGEO_JET_MONO, or KGEO_JET_POWER with pval == 0 */
  int32_t neqmax;      /* >= 1 */
  double pval;
  double nu_parallel;  /* in [-1, 1] */
  double sigma;        /* width of the mass-loading Gaussian (0: a step at r0) */
  double specind;      /* spectral index */
} kgeo_jet_emission;
int kgeo_jet_stokes(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                    const double* r, const double* th, const double* signpr, const double* signpth,
                    const double* neq, int32_t nguess, const kgeo_jet_emission* emission, double* I, double* Q,
                    double* U, double* evpa, double* I_c, double* Q_c, double* U_c, double* stagnation,
                    int32_t* status, void* stream);

/* Batched tracing: many images of different size, spin, inclination and ngeo traced as one
 * job (no counterpart in the reference, whose raytrace_ana takes one image per call:
 * kgeo/kerr_raytracing_ana.py:46). A plan describes the images; kgeo_batch_bind attaches the
 * device buffers: alpha, beta are every image's pixels concatenated (image i owns rays
 * [sum_{j<i} npix_j, ... + npix_i)); per-ray outputs (tau_tot, rclass, thclass) follow the
 * same concatenation; each sample output (t, r, th, ph, sig, mino) holds image i's
 * (ngeo_i, npix_i) row-major block at offset sum_{j<i} ngeo_j npix_j. A run is one setup pass
 * over all rays (per-image class sort) and one persistent sample kernel whose blocks pull
 * tiles of work items from a device counter. Results equal kgeo_raytrace of each image with the
 * same chunk length to rounding (the kernels may contract different multiply-adds; Mino times and
 * classes are identical). A plan and its bound buffers are used by one stream at a time.
 *
 * kgeo_batch_autotune times the sample kernel's launch shapes (block size, CTAs per SM, samples
 * per work item; tiles of one item per thread) on a subset of the bound batch's tiles within
 * about budget_ms and keeps the fastest; results are cached per device, precision and image sizes (the cache
 * and the BZ f(r) tables of kgeo_jet_stokes are the library's only global state, both
 * mutex-guarded), so a new plan for the same batch shape
 * starts tuned. kgeo_batch_graph_launch captures the whole run into a CUDA graph on first use
 * (and again after a bind or a configuration change) and replays it on `stream`. */
#define KGEO_BATCH_MAX_IMAGES 4096
typedef struct {
  double a, r_o, th_o;    /* observer of this image (the kgeo_observer rules apply) */
  int64_t npix;
  int32_t ngeo;
  int32_t reserved;
  double maxtaufrac;
} kgeo_batch_image;
typedef struct {
  int32_t block;          /* threads per block of the sample kernel: 128 or 256 */
  int32_t ctas_per_sm;    /* resident blocks per SM of the persistent grid (1..4) */
  int32_t tile;           /* work items per tile taken from the counter (multiple of block) */
  int32_t chunk;          /* samples per work item (<= 64 FP64, <= 256 mixed) */
} kgeo_batch_config;
typedef struct kgeo_batch_plan kgeo_batch_plan;
int kgeo_batch_create(const kgeo_batch_image* images, int32_t nimg, int32_t precision, kgeo_batch_plan** plan);
void kgeo_batch_destroy(kgeo_batch_plan* plan);
int kgeo_batch_sizes(const kgeo_batch_plan* plan, int64_t* n_rays, int64_t* n_samples, size_t* workspace_bytes);
/* kgeo_batch_bind: out->flags, when not NULL, receives nimg words after each run (image i's
 * KGEO_FLAG_* bits). */
int kgeo_batch_bind(kgeo_batch_plan* plan, const double* alpha, const double* beta, kgeo_geodesics* out,
                    void* workspace, size_t workspace_bytes);
int kgeo_batch_get_config(const kgeo_batch_plan* plan, kgeo_batch_config* cfg, int32_t* tuned);
int kgeo_batch_set_config(kgeo_batch_plan* plan, const kgeo_batch_config* cfg);
int kgeo_batch_autotune(kgeo_batch_plan* plan, int32_t budget_ms, void* stream, kgeo_batch_config* best);
int kgeo_batch_run(kgeo_batch_plan* plan, void* stream);
int kgeo_batch_graph_launch(kgeo_batch_plan* plan, void* stream);

/* Allocation-free kgeo_raytrace. No counterpart in the reference: it exists for callers
 * that may not allocate device memory when they call in — an application that owns all
 * device memory under a fixed budget, a latency-critical loop that cannot afford an
 * allocator call, or a host that offers no allocator. Same arguments, outputs and status
 * codes as kgeo_raytrace minus the workspace: the per-ray scratch lives in a fixed array
 * inside the library (room for KGEO_NOALLOC_MAX_PIXELS rays, about 15.9 MB of device memory
 * that every GPU loading the library keeps until the process exits). Larger npix is
 * refused with KGEO_ERR_NOALLOC_SIZE before any work. The call allocates and frees nothing.
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress)
 * once for that device and keeps it for the life of the process; make that first call before
 * any stream capture, and do not call this entry point on a device after a cudaDeviceReset of
 * it (the kept address would be stale). Every call on a
 * device shares the one array and it keeps the last call's contents, so calls whose work
 * overlaps on the GPU (different streams, or different host threads) race: order them on one
 * stream or serialise them. */
#define KGEO_NOALLOC_MAX_PIXELS 16384
int kgeo_raytrace_noalloc(const kgeo_observer* obs, const double* alpha, const double* beta, int64_t npix,
                          int32_t ngeo, double maxtaufrac, kgeo_geodesics* out, void* stream);

/* ellip_pi_arr(n, phi, m) (kgeo/scipy_ellip_binding.py:87-237): the incomplete elliptic
 * integral of the third kind Pi(n; phi | m) in Abramowitz & Stegun's convention, with the
 * reference adapter's special cases (phi ~ 0, m < -1e14, 1 - m sin^2 < 0, |phi| > pi/2 with
 * m >= 1 or n = 1, 1 - n sin^2 = 0, n = inf) and its periodic continuation, evaluated on the
 * device exactly as the kernels evaluate it: `form` 0 = the per-ray setup's arithmetic
 * (FMA contraction off), 1 = the direct sample evaluators' (contraction on), 2 = the
 * standalone adapter kg::ellip_pi_ref. n, phi, m, out: N doubles (device memory); the
 * caller broadcasts. Stream-ordered, allocates nothing. */
int kgeo_ellip_pi(const double* n, const double* phi, const double* m, int64_t N, int32_t form, double* out,
                  void* stream);

/* Measurement helper (no counterpart in the reference): runs a fixed FP64 fused
 * multiply-add loop on every SM and returns the achieved FP64 rate in TFLOP/s (an FMA
 * counts as 2 FLOP). Used as the FP64 roofline denominator; blocks until done. */
int kgeo_measure_fp64_peak(double* tflops, void* stream);

/* Human-readable text of a kgeo_status code (the reference's exception message where one exists). */
const char* kgeo_status_string(int status);

/* ABI version (KGEO_ABI_VERSION of the library that was built). */
int kgeo_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* KGEO_GB300_H */
