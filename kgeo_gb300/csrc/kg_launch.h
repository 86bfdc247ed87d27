// Internal launch interface between the C ABI and the kernel translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "kg_equatorial.cuh"

namespace kg {

// Device scratch layout for npix pixels: the per-ray record (NUM_FIELDS doubles per ray,
// structure of arrays), the per-ray code word, and one flags word.
struct Workspace {
  double* rec;
  int* code;
  uint32_t* flags;
};

KG_HD size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

inline size_t workspace_bytes(int64_t npix) {
  size_t n = (size_t)(npix > 0 ? npix : 1);
  return align_up(sizeof(double) * NUM_FIELDS * n, 256) + align_up(sizeof(int) * n, 256) + 256;
}

inline Workspace carve_workspace(void* base, int64_t npix) {
  size_t n = (size_t)(npix > 0 ? npix : 1);
  char* p = static_cast<char*>(base);
  Workspace w;
  w.rec = reinterpret_cast<double*>(p);
  p += align_up(sizeof(double) * NUM_FIELDS * n, 256);
  w.code = reinterpret_cast<int*>(p);
  p += align_up(sizeof(int) * n, 256);
  w.flags = reinterpret_cast<uint32_t*>(p);
  return w;
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
};

struct SampleArgs {
  Observer obs;
  const double* rec;
  const int* code;
  int64_t npix;
  int64_t nsamp;
  const double* tau;    // (nsamp, npix) or NULL for the linspace grid
  int do_phi_t;
  const uint32_t* flags;
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
};

cudaError_t launch_ray_setup(const SetupArgs& a, cudaStream_t s);
cudaError_t launch_equatorial(const EquatorialArgs& a, cudaStream_t s);
cudaError_t launch_crossings(const CrossingArgs& a, cudaStream_t s);
cudaError_t launch_samples(const SampleArgs& a, cudaStream_t s);

}  // namespace kg
