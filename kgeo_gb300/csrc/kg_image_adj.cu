// Image-adjoint kernels (forward-mode dual numbers through the image chain, kg_image.cuh).
// Compiled with FMA contraction off (-fmad=false), like the forward image in kg_image.cu.
#include "kg_launch.h"

namespace kg {

// Block sum of NQ values per thread into partial[block * NQ + q] (fixed order: warp
// shuffles, then warp 0 over the warp sums), so the result does not depend on scheduling.
__device__ void block_sum_nq(double* v, double* out) {
  __shared__ double warp_sums[IMAGE_BLOCK / 32][NQ];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    double x = v[q];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    if (lane == 0) warp_sums[w][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < NQ) {
    double x = 0.0;
#pragma unroll
    for (int k = 0; k < IMAGE_BLOCK / 32; ++k) x += warp_sums[k][threadIdx.x];
    out[threadIdx.x] = x;
  }
}

__global__ void __launch_bounds__(IMAGE_BLOCK, 1) image_adjoint_kernel(ImageAdjointArgs a) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double acc[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
  if (t < a.npix) {
    const int64_t i = a.perm ? (int64_t)a.perm[t] : t;
    const Observer& o = a.obs;
    const double alpha = a.alpha[i], beta = a.beta[i];
    PixelGeo p;
    for (int m0 = 0; m0 < a.nord; m0 += ORDER_GROUP) {
      const int n = min(ORDER_GROUP, a.nord - m0);
      pixel_geo(o, alpha, beta, a.mbar_lo + m0, n, &p);
      bool any = false;
      for (int j = 0; j < n; ++j) any = any || (!image_zero(a.model, o, p, j) && a.grad_I[i * a.nord + m0 + j] != 0.0);
      if (!any) continue;
      D2 rs[ORDER_GROUP];
      rs_tangents(o, alpha, beta, p, n, rs);
      for (int j = 0; j < n; ++j) {
        if (image_zero(a.model, o, p, j)) continue;
        const double gI = a.grad_I[i * a.nord + m0 + j];
        if (gI == 0.0) continue;
        Dual<NQ> I = emission_dual(a.model, o, p, j, alpha, beta, rs[j]);
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] += gI * I.d[q];
      }
    }
  }
  block_sum_nq(acc, a.partial + (int64_t)blockIdx.x * NQ);
}

// One block sums the per-block partials in a fixed order.
__global__ void __launch_bounds__(256) adjoint_reduce_kernel(const double* partial, int64_t nblocks, double* grad) {
  __shared__ double sh[256][NQ];
  double acc[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) acc[q] = 0.0;
  for (int64_t b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] += partial[b * NQ + q];
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) sh[threadIdx.x][q] = acc[q];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) sh[threadIdx.x][q] += sh[threadIdx.x + s][q];
    }
    __syncthreads();
  }
  if (threadIdx.x < NQ) grad[threadIdx.x] = sh[0][threadIdx.x];
}

cudaError_t launch_image_adjoint(const ImageAdjointArgs& a, cudaStream_t s) {
  if (a.npix <= 0) return cudaMemsetAsync(a.grad, 0, NQ * sizeof(double), s);
  const int64_t nb = image_adjoint_blocks(a.npix);
  image_adjoint_kernel<<<(unsigned)nb, IMAGE_BLOCK, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  adjoint_reduce_kernel<<<1, 256, 0, s>>>(a.partial, nb, a.grad);
  return cudaGetLastError();
}

}  // namespace kg
