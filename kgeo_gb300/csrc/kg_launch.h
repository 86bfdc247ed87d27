// Internal launch interface between the C ABI and the kernel translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "kg_polar.cuh"
#include "kg_curves.cuh"
#include "kg_jet.cuh"
#include "kg_jetimg.cuh"

namespace kg {

// Device scratch layout for npix pixels: the per-ray record (NUM_FIELDS doubles per ray,
// structure of arrays), the per-ray code word, the class-sorted ray permutation, the
// class-bucket counters and cursors, and one flags word.
constexpr int NBUCKET = 32;

KG_HD constexpr size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

KG_HD constexpr size_t workspace_bytes_n(size_t n) {
  return align_up(sizeof(double) * NUM_FIELDS * n, 256) + 2 * align_up(sizeof(int) * n, 256) +
         align_up(sizeof(uint32_t) * (2 * NBUCKET + 1), 256);
}

inline size_t workspace_bytes(int64_t npix) { return workspace_bytes_n((size_t)(npix > 0 ? npix : 1)); }

struct Workspace {
  double* rec;
  int* code;
  int* perm;          // rays ordered by class bucket
  uint32_t* counts;   // NBUCKET ray counts, then NBUCKET cursors
  uint32_t* flags;    // launch flags (follows the counters: one memset clears both)
};

inline Workspace carve_workspace(void* base, int64_t npix) {
  size_t n = (size_t)(npix > 0 ? npix : 1);
  char* p = static_cast<char*>(base);
  Workspace w;
  w.rec = reinterpret_cast<double*>(p);
  p += align_up(sizeof(double) * NUM_FIELDS * n, 256);
  w.code = reinterpret_cast<int*>(p);
  p += align_up(sizeof(int) * n, 256);
  w.perm = reinterpret_cast<int*>(p);
  p += align_up(sizeof(int) * n, 256);
  w.counts = reinterpret_cast<uint32_t*>(p);
  w.flags = w.counts + 2 * NBUCKET;
  return w;
}

// Class bucket of a ray: recurrence flag, radial case, theta branch, ordered so that the
// costliest work comes first in the sorted order (rays without the recurrence, evaluated
// directly at every sample; then radial cases 4, 3, 2): the kernels take items in that order,
// so the last blocks of a launch hold the cheapest rays and the launch ends without a long
// tail (5 % on 512x512 x 400 samples, 5 % on the 5.2 M-ray mixed launch, measured on GB300).
KG_HD int ray_bucket(int code) {
  return (code_step(code) ? 16 : 0) + (4 - code_rcase(code)) * 3 + code_th(code);
}

struct SetupArgs {
  Observer obs;
  const double* alpha;
  const double* beta;
  int64_t npix;
  int64_t ngeo;  // for the linspace zero-step test; 0 when tau is given
  double maxtaufrac;
  double* rec;
  int* code;
  int32_t* rclass;
  int32_t* thclass;
  double* tau_tot;
  uint32_t* flags;      // launch flags (workspace)
  uint32_t* counts;     // class-bucket counters (workspace)
  int* perm;            // class-sorted permutation (workspace)
};

struct SampleArgs {
  Observer obs;
  const double* rec;
  const int* code;
  int64_t npix;
  int64_t nsamp;
  const double* tau;    // (nsamp, npix) or NULL for the linspace grid
  int do_phi_t;
  int chunk;            // > 0: even grid by the addition-theorem recurrence, chunk samples per thread
  const int* perm;      // class-sorted rays for the recurrence kernel
  int mixed;            // 1: mixed-precision recurrence (kg_mixed.cuh)
  int64_t c_begin;      // recurrence kernel: chunks [c_begin, c_end) only (c_end < 0: to the last)
  int64_t c_end;
  int64_t row0;         // sample g is stored in row g - row0 of the outputs
  uint32_t* flags;      // launch flags: read at start; FLAG_LOOP_CAP is OR-ed in
  double* t;
  double* r;
  double* th;
  double* ph;
  double* sig;
  double* mino;
};

struct EquatorialArgs {
  Observer obs;
  const double* alpha;
  const double* beta;
  int64_t npix;
  int mbar_lo;
  int nord;
  double* r_s;   // (nord, npix)
  double* Ir;    // (nord, npix)
  double* Imax;  // (npix)
  double* Nmax;  // (npix)
};

struct CrossingArgs {
  Observer obs;
  const double* alpha;
  const double* beta;
  int64_t npix;
  const double* tau;  // (ntau, npix)
  int64_t ntau;
  double* n_eq;       // (ntau, npix)
  double* n_pol;      // (ntau, npix)
  double* outside;    // (npix) is_outside_crit
  double* n_turn;     // (ntau, npix) n_angular_turnings
};

// Default and largest samples per thread of the stepped kernel (longer recurrence chains
// accumulate more rounding: 64 keeps every output within the FP64 parity bars, max error over
// bar 0.62 on 12 seeded 48x48x400 draws; the chunk-start direct evaluation is amortised over
// the whole chunk).
constexpr int DEFAULT_CHUNK = 64;
constexpr int MAX_CHUNK = 64;
// The mixed recurrence accumulates FP32 increments into FP64 sums, so its chains may be
// longer: the chunk-start evaluation is amortised over more samples.
constexpr int DEFAULT_CHUNK_MIXED = 256;
constexpr int MAX_CHUNK_MIXED = 256;

// Equatorial image of orders mbar_lo .. mbar_lo + nord - 1 (kg_image.cuh); outputs are
// (npix, nord) row-major.
struct ImageArgs {
  Observer obs;
  EmissionModel model;
  const double* alpha;
  const double* beta;
  int64_t npix;
  int mbar_lo;
  int nord;
  double* I;
  double* g;
  double* r_s;
  double* Ir;
  double* sinthb;
  double* imax;   // (npix)
  double* nmax;   // (npix)
  double* npol;   // (npix)
  ImageOptions opts;
  double* Q;      // polarised: cos(2 chi) I
  double* U;      // polarised: sin(2 chi) I
  double* lp;     // path length (pathlength)
  double* Ie;     // emission before g^3 (pathlength)
  const int* perm;  // (npix) pixel order of the threads (launch_pixel_sort), or NULL for 0..npix-1
};

// Adjoint of the image: sum over pixels and orders of grad_I * dI/dq for the NQ parameters.
struct ImageAdjointArgs {
  Observer obs;
  EmissionModel model;
  const double* alpha;
  const double* beta;
  int64_t npix;
  int mbar_lo;
  int nord;
  const double* grad_I;  // (npix, nord)
  double* partial;       // (blocks, NQ) per-block sums
  double* grad;          // (NQ)
  const int* perm;       // (npix) pixel order of the threads, or NULL
};

// ---------------------------------------------------------------------------
// batched images (kg_batch.cu): many images of different size, spin, inclination and ngeo in
// one setup pass and one persistent sample kernel. Rays of all images are concatenated
// (image i owns rays [pix_off, pix_off + npix)); the per-ray records are one
// structure-of-arrays buffer with stride ntot; image i's samples are the (ngeo, npix)
// row-major block at out_off of each output.
struct BatchImage {
  Observer obs;
  int64_t pix_off, npix, ngeo, out_off;
  double maxtaufrac;
};

struct BatchArgs {
  const BatchImage* img;   // (nimg)
  const int64_t* pix_off;  // (nimg + 1) ray offsets, for the image lookup
  int64_t* item_off;       // (nimg + 1) work-item offsets of the sample kernel (chunk dependent)
  int nimg;
  int64_t ntot;
  const double* alpha;     // (ntot)
  const double* beta;      // (ntot)
  double* rec;             // NUM_FIELDS x ntot
  int* code;               // (ntot)
  int* perm;               // (ntot) rays of each image sorted by class bucket (global ray indices)
  uint32_t* counts;        // (nimg * NBUCKET) bucket counts, then (nimg * NBUCKET) cursors
  uint32_t* flags;         // (nimg) launch flags per image
  unsigned long long* work;  // work counter of the persistent kernel
  int32_t* rclass;         // per-ray outputs (ntot), may be NULL
  int32_t* thclass;
  double* tau_tot;
  double *t, *r, *th, *ph, *sig, *mino;  // concatenated sample outputs
  int chunk;               // samples per work item
  int tile;                // work items per tile (multiple of the block size)
  int tile_skip;           // 1: every tile; S > 1: every S-th tile (autotuner timing runs)
  int mixed;
};

constexpr int BATCH_MAX_IMAGES = 4096;

// Image containing global index x of a prefix-offset table off (nimg + 1 entries).
KG_HD int batch_find(const int64_t* off, int nimg, int64_t x) {
  int lo = 0, hi = nimg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

cudaError_t launch_batch_setup(const BatchArgs& a, cudaStream_t s);
cudaError_t launch_batch_step(const BatchArgs& a, cudaStream_t s);

#if defined(__CUDACC__)
// End of a batch setup block: a capped loop in it is charged to the images of the block's first
// and last rays (every thread of the block calls it; it synchronises).
__device__ __forceinline__ void batch_loop_cap_end(const BatchArgs& a) {
  __syncthreads();
  if (threadIdx.x == 0 && kg_loop_cap_word && a.ntot > 0) {
    const int64_t r0 = (int64_t)blockIdx.x * blockDim.x;
    const int64_t r1 = r0 + blockDim.x - 1 < a.ntot ? r0 + blockDim.x - 1 : a.ntot - 1;
    const int i0 = batch_find(a.pix_off, a.nimg, r0), i1 = batch_find(a.pix_off, a.nimg, r1);
    for (int j = i0; j <= i1; ++j) atomicOr(a.flags + j, kg_loop_cap_word);
  }
}
#endif
cudaError_t launch_batch_samples(const BatchArgs& a, int block, int grid, cudaStream_t s);
cudaError_t prepare_batch_kernels();

constexpr int IMAGE_BLOCK = 128;
KG_HD constexpr int64_t image_adjoint_blocks(int64_t npix) { return (npix + IMAGE_BLOCK - 1) / IMAGE_BLOCK; }

// Pixel order of the image kernels (kg_image.cu): pixels sorted by radial class (eta <= 0
// first, then rclass 1..4) with a deterministic counting sort, so that the lanes of a warp take
// the same radial case; each pixel's values do not depend on the order, and the adjoint's block
// sums stay in a fixed order. Scratch: key and permutation (int32 per pixel) and the
// per-(class, block) counts.
constexpr int PIX_SORT_BLOCK = 256;
constexpr int PIX_BUCKETS = 8;
KG_HD constexpr int64_t pixel_sort_blocks(int64_t npix) { return (npix + PIX_SORT_BLOCK - 1) / PIX_SORT_BLOCK; }
KG_HD constexpr size_t pixel_sort_bytes(int64_t npix) {
  return npix > 0 ? 2 * align_up(sizeof(int) * (size_t)npix, 256) +
                        align_up(sizeof(uint32_t) * PIX_BUCKETS * (size_t)pixel_sort_blocks(npix), 256)
                  : 0;
}
// Sorts the pixels into scratch (pixel_sort_bytes(npix) bytes); *perm points into it.
cudaError_t launch_pixel_sort(const Observer& o, const double* alpha, const double* beta, int64_t npix, void* scratch,
                              const int** perm, cudaStream_t s);

cudaError_t launch_ray_setup(const SetupArgs& a, cudaStream_t s);
cudaError_t launch_ray_step(const SetupArgs& a, cudaStream_t s);
// curve library (kg_curves.cu)
struct CurveArgs {
  const CurveSpec* curves;  // (ncurves) device table
  int64_t ncurves;
  const double* varphi;     // (nphi) angles shared by every curve
  int64_t nphi;
  double xtol, rtol;
  int maxiter;
  double* rho;              // (ncurves, nphi)
  int32_t* status;          // (ncurves, nphi) CURVE_* or NULL
};

struct CriticalArgs {
  double a, sin_th, cos_th, tan_th, rminus, rplus;
  int64_t n;
  double* alpha;
  double* beta;
};

// jet field-line crossings (kg_jet.cu)
struct JetGuessArgs {
  Observer obs;
  JetField field;
  const double* alpha;
  const double* beta;
  int64_t npix;
  const double* r;      // (ngeo, npix) samples, or NULL: taumax only
  const double* th;
  const double* mino;
  int64_t ngeo;
  int neqmax;           // <= 0: no limit
  double* taumax;       // (npix) or NULL
  int32_t* count;       // (npix) or NULL
  double* guesses;      // (nguess, npix) or NULL
  int64_t nguess;
};

struct JetSolveArgs {
  Observer obs;
  JetField field;
  const double* rec;
  const int* code;
  const uint32_t* flags;
  const double* alpha;
  const double* beta;
  int64_t npix;
  const double* guesses;  // (nguess, npix)
  int64_t nguess;
  double tol;
  int maxiter;
  double* tau;
  double* r;
  double* th;
  double* signpr;
  double* signpth;
  double* neq;
  int32_t* status;
};

// Stokes images of the off-equatorial crossings (kg_jetimg.cu).
struct JetStokesArgs {
  Observer obs;
  JetImgParams p;          // r0 is found on the device from the first crossing row
  const double* tab;       // BZ f(r) node values (BZ_TABLE_N)
  const double* alpha;     // (npix)
  const double* beta;
  int64_t npix;
  const double* r;         // (nguess, npix) crossings
  const double* th;
  const double* signpr;
  const double* signpth;
  const double* neq;
  int64_t nguess;
  int neqmax;
  double* par;             // device scratch: r0, Omega, status
  double* I;               // (neqmax + 1, npix) per-subring images, then the total
  double* Q;
  double* U;
  double* evpa;
  double* Ic;              // (nguess, npix) per crossing, or NULL
  double* Qc;
  double* Uc;
  double* stagnation;      // (2) r0, Omega, or NULL
  int32_t* status;         // (1) or NULL
};

// Device table of BZ f(r) node values, built once per device on first use (synchronously).
cudaError_t jet_bz_table(const double** tab);
cudaError_t launch_jet_stokes(const JetStokesArgs& a, cudaStream_t s);

cudaError_t launch_jet_guesses(const JetGuessArgs& a, cudaStream_t s);
cudaError_t launch_jet_solve(const JetSolveArgs& a, cudaStream_t s);
cudaError_t launch_curves(const CurveArgs& a, cudaStream_t s);
cudaError_t launch_critical(const CriticalArgs& a, cudaStream_t s);
cudaError_t launch_image(const ImageArgs& a, cudaStream_t s);
cudaError_t launch_image_adjoint(const ImageAdjointArgs& a, cudaStream_t s);
cudaError_t launch_equatorial(const EquatorialArgs& a, cudaStream_t s);
cudaError_t launch_crossings(const CrossingArgs& a, cudaStream_t s);
cudaError_t launch_samples(const SampleArgs& a, cudaStream_t s);
cudaError_t launch_ellip_pi_setup(const double* n, const double* phi, const double* m, int64_t N, double* out,
                                  cudaStream_t s);
cudaError_t launch_ellip_pi_samples(const double* n, const double* phi, const double* m, int64_t N, int form,
                                    double* out, cudaStream_t s);

}  // namespace kg
