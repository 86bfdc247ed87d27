// kgeo_raytrace_noalloc: the same trace as kgeo_raytrace, with its scratch in a fixed
// device array that ships inside this library instead of memory the call allocates.
//
// Who needs it: some hosts of this library may not allocate device memory at all at call
// time — an application that owns every byte of device memory under a fixed budget and
// forbids stray allocations, a latency-critical loop that cannot afford an allocator call
// (cudaMalloc can synchronise the device), or a plugin environment that exposes no
// allocator. kgeo_raytrace needs per-ray scratch (the ray records the sample kernel reads)
// and either takes it from the caller or allocates it; this entry point does neither.
//
// The cost: the array below (KGEO_NOALLOC_MAX_PIXELS rays' records and sort keys, about 15.9 MB) is part of
// the library's device image, so every GPU that loads the library holds it until the
// process exits, whether or not this entry point is called.
#include <cstring>
#include <mutex>

#include "../../include/kgeo_gb300.h"
#include "kg_launch.h"

using namespace kg;

namespace {

constexpr int64_t kMaxPixels = KGEO_NOALLOC_MAX_PIXELS;

// Scratch for kMaxPixels rays, sized by the same rule as kgeo_workspace_size.
constexpr size_t kScratchBytes = workspace_bytes_n((size_t)kMaxPixels);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch, looked up once per device and kept for the process. In
// host code the array's name only stands in for the symbol; the address a kernel can use comes
// from the runtime. A cudaDeviceReset unloads the module and would leave the kept address
// stale: the entry point is documented as not to be called on a device after its reset.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};

int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return KGEO_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return KGEO_ERR_CUDA;
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return KGEO_OK;
}

}  // namespace

extern "C" int kgeo_raytrace_noalloc(const kgeo_observer* obs, const double* alpha, const double* beta,
                                     int64_t npix, int32_t ngeo, double maxtaufrac, kgeo_geodesics* out,
                                     void* stream) {
  if (npix > kMaxPixels) return KGEO_ERR_NOALLOC_SIZE;
  if (npix < 0) return KGEO_ERR_LENGTHS;
  void* scratch = nullptr;
  int st = scratch_address(&scratch);
  if (st) return st;
  // kgeo_raytrace with caller workspace: it allocates nothing when given one, and clears the
  // flags word of the workspace on the stream before the setup kernel runs.
  return kgeo_raytrace(obs, alpha, beta, npix, ngeo, maxtaufrac, out, scratch, kScratchBytes, stream);
}
