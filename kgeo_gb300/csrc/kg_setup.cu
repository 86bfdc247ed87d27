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

}  // namespace kg
