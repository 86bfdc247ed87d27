// Equatorial image kernels (unpolarised, and polarised / with path length). Compiled with
// FMA contraction off (-fmad=false), like the per-ray setup: the crossing count Nmax that
// masks each image order is a floor() of elliptic-integral ratios and must round as numpy's
// does. The adjoint is in kg_image_adj.cu (a separate translation unit, compiled in parallel).
#include "kg_launch.h"

namespace kg {

// OPTS: polarisation and / or path length requested (kg_polar.cuh); the plain image keeps
// the shorter kernel.
template <bool OPTS>
__global__ void __launch_bounds__(IMAGE_BLOCK, 1) image_kernel(ImageArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.npix) return;
  const Observer& o = a.obs;
  const double alpha = a.alpha[i], beta = a.beta[i];
  PixelGeo p;
  for (int m0 = 0; m0 < a.nord; m0 += ORDER_GROUP) {
    const int n = min(ORDER_GROUP, a.nord - m0);
    pixel_geo(o, alpha, beta, a.mbar_lo + m0, n, &p);
    for (int j = 0; j < n; ++j) {
      const int64_t k = i * a.nord + m0 + j;
      PixelOut px{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      if (!image_zero(a.model, o, p, j)) {
        if (OPTS) {
          emission_px_opts(a.model, a.opts, o, p, j, alpha, beta, &px);
        } else {
          emission_px(a.model, o, p, j, &px.I, &px.g);
          px.sinthb = a.model.sinthb;
        }
      }
      a.I[k] = px.I;
      if (a.g) a.g[k] = px.g;
      if (a.r_s) a.r_s[k] = p.r_s[j];
      if (a.Ir) a.Ir[k] = p.Ir[j];
      if (a.sinthb) a.sinthb[k] = px.sinthb;
      if (OPTS) {
        if (a.Q) a.Q[k] = px.Q;
        if (a.U) a.U[k] = px.U;
        if (a.lp) a.lp[k] = px.lp;
        if (a.Ie) a.Ie[k] = px.Ie;
      }
    }
  }
  if (a.imax) a.imax[i] = p.Imax;
  if (a.nmax) a.nmax[i] = p.Nmax;
  if (a.npol) a.npol[i] = p.npol;
}

cudaError_t launch_image(const ImageArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const unsigned nb = (unsigned)image_adjoint_blocks(a.npix);
  if (a.opts.polarization || a.opts.pathlength)
    image_kernel<true><<<nb, IMAGE_BLOCK, 0, s>>>(a);
  else
    image_kernel<false><<<nb, IMAGE_BLOCK, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace kg
