// Curve-library kernels: Brent root per (curve, angle) and the critical curve. Compiled with
// FMA contraction off (-fmad=false) like the other r_equatorial kernels, so the objective's
// crossing counts round as numpy's do.
#include "kg_curves.cuh"
#include "kg_launch.h"

namespace kg {

__global__ void __launch_bounds__(128) curve_kernel(CurveArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.ncurves * a.nphi) return;
  const int64_t c = i / a.nphi;
  const int64_t j = i - c * a.nphi;
  int st = CURVE_OK;
  const double rho = curve_rho(a.curves[c], a.varphi[j], a.xtol, a.rtol, a.maxiter, &st);
  a.rho[i] = rho;
  if (a.status) a.status[i] = st;
}

cudaError_t launch_curves(const CurveArgs& a, cudaStream_t s) {
  const int64_t n = a.ncurves * a.nphi;
  if (n <= 0) return cudaSuccess;
  const int block = 128;
  curve_kernel<<<(unsigned)((n + block - 1) / block), block, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(256) critical_kernel(CriticalArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  critical_point(a.a, a.sin_th, a.cos_th, a.tan_th, a.rminus, a.rplus, a.n, i, a.alpha + i, a.beta + i);
}

cudaError_t launch_critical(const CriticalArgs& a, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  critical_kernel<<<(unsigned)((a.n + 255) / 256), 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace kg
