// Per-ray setup kernel. Compiled with FMA contraction off (-fmad=false) so that the
// classification arithmetic rounds one operation at a time, as numpy does.
#include "kg_launch.h"

namespace kg {

__global__ void __launch_bounds__(128) ray_setup_kernel(SetupArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned fl = 0;
  if (i < a.npix) {
    RayRec R;
    int rc = 0, tc = 0;
    fl = ray_setup(a.obs, a.alpha[i], a.beta[i], a.maxtaufrac, &R, &rc, &tc);
#pragma unroll
    for (int k = 0; k < NUM_FIELDS; ++k) a.rec[(int64_t)k * a.npix + i] = R.f[k];
    a.code[i] = R.code;
    if (a.rclass) a.rclass[i] = rc;
    if (a.thclass) a.thclass[i] = tc;
    if (a.tau_tot) a.tau_tot[i] = R.f[F_TAUTOT];
    if (a.ngeo > 1 && R.f[F_TAUMAX] / (double)(a.ngeo - 1) == 0.0) fl |= FLAG_ANY_STEP_ZERO;
  }
  fl = __reduce_or_sync(0xffffffffu, fl);
  if ((threadIdx.x & 31) == 0 && fl) atomicOr(a.flags, fl);
}

cudaError_t launch_ray_setup(const SetupArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const int block = 128;
  const int64_t grid = (a.npix + block - 1) / block;
  ray_setup_kernel<<<(unsigned)grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(128) equatorial_kernel(EquatorialArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.npix) return;
  EqResult r = r_equatorial_px(a.obs, a.alpha[i], a.beta[i], a.mbar_lo, a.nord, a.r_s + i, a.Ir + i, a.npix);
  if (a.Imax) a.Imax[i] = r.Imax;
  if (a.Nmax) a.Nmax[i] = r.Nmax;
}

cudaError_t launch_equatorial(const EquatorialArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const int block = 128;
  equatorial_kernel<<<(unsigned)((a.npix + block - 1) / block), block, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(128) crossings_kernel(CrossingArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.npix) return;
  const Observer& o = a.obs;
  double alpha = a.alpha[i], beta = a.beta[i];
  double lam = -alpha * o.sin_th;
  double eta = (alpha * alpha - o.a2) * o.cos2 + beta * beta;
  if (a.outside) a.outside[i] = outside_crit(o, lam, eta);
  if (a.ntau <= 0 || (!a.n_eq && !a.n_pol)) return;
  EqConsts c = eq_consts(o, lam, eta);
  double Kc = c.vort ? 0.0 : ellip_k(c.ratio);
  for (int64_t g = 0; g < a.ntau; ++g) {
    double tau = a.tau[g * a.npix + i];
    if (a.n_eq) a.n_eq[g * a.npix + i] = n_eq_at(o, c, beta, tau);
    if (a.n_pol) a.n_pol[g * a.npix + i] = n_pol_at(c, Kc, tau);
  }
}

cudaError_t launch_crossings(const CrossingArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const int block = 128;
  crossings_kernel<<<(unsigned)((a.npix + block - 1) / block), block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace kg
