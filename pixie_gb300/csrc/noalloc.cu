// pxg_image_blur_noalloc: the gaussian blur of pxg_image_blur for callers
// that cannot allocate GPU memory.
//
// Some host programs own every byte of device memory through their own pool
// and forbid other code from calling cudaMalloc/cudaFree; others run on
// latency-critical paths where an allocation (which may block, or
// synchronise the device) is not acceptable.  This entry point works on the
// caller's image buffer and stream and takes its work space from a
// fixed-size array in the library's own device image instead of allocating:
//   - the blur's intermediate image and the gaussian weights live in
//     g_noalloc_scratch below (the weights are passed by value to a small
//     kernel that stores them there, so the call never copies from host
//     memory), a file-scope static __device__ array of
//     kWeightsBytes + 4 * kNoAllocMaxPixels bytes (8 MiB + 16 KiB).  Every GPU
//     that loads the library holds it until the process exits;
//   - images larger than kNoAllocMaxPixels pixels, or radii above
//     kNoAllocMaxRadius, are rejected with an error;
//   - every call shares the array and leaves its contents behind; nothing in
//     it has to start at zero (the weights and the intermediate are fully
//     rewritten by each call), but calls whose GPU work overlaps (on
//     different streams, or from different threads) race on it;
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) and sets the blur kernels' shared-memory limits;
//     make that first call before any stream capture.
//   - the blur runs the CUDA-core passes (k_blurf_x/k_blurf_y below radius 8,
//     the register-blocked k_blurb passes from radius 8), not the default
//     small-radius or tensor-core passes of pxg_image_blur; the bytes are the
//     same.
// No cudaMalloc, cudaFree or other allocating routine is called, on the GPU
// or on the host (errors go to fixed per-thread buffers).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "../../include/pxg.h"
#include "host_geom.h"

namespace pxg {
void record_error(const char* msg);
void launch_blur(uint32_t* img, uint32_t* tmp, long long W, long long H, int r,
                 const uint16_t* kern, uint32_t oob, int nsm, size_t maxSmem, cudaStream_t st);
void* blurb_kernel(bool x);
__global__ void k_blur_x(const uint32_t*, uint32_t*, long long, long long, int, const uint16_t*, uint32_t);
__global__ void k_blur_y(const uint32_t*, uint32_t*, long long, long long, int, const uint16_t*, uint32_t);
__global__ void k_blurf_x(const uint32_t*, uint32_t*, long long, long long, int, const uint16_t*, uint32_t);
__global__ void k_blurf_y(const uint32_t*, uint32_t*, long long, long long, int, const uint16_t*, uint32_t);
}  // namespace pxg

namespace {

constexpr int64_t kNoAllocMaxPixels = 2 * 1024 * 1024;  // 8 MiB of RGBX intermediate
constexpr int64_t kNoAllocMaxRadius = 2048;
constexpr size_t kWeightsBytes = 16 * 1024;             // >= (2 * 2048 + 1) * 2 bytes
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kWeightsBytes + kNoAllocMaxPixels * 4];

// Gaussian weights passed by value: (2 * 2048 + 1) uint16 = 8194 bytes, inside
// the 32764-byte kernel-parameter limit of sm_70 and later.
struct WeightsParam {
  uint16_t w[2 * kNoAllocMaxRadius + 2];
  int n;
};
static_assert(sizeof(WeightsParam) <= 32764, "kernel parameter too large");

__global__ void k_store_weights(const WeightsParam p, uint16_t* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < p.n) dst[i] = p.w[i];
}

struct DeviceSetup {
  bool ready;
  unsigned char* scratch;  // device address of g_noalloc_scratch on this device
  int nsm;
  size_t maxSmem;
};
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

int fail(const char* msg) {
  pxg::record_error(msg);
  return 1;
}

// Once per device, with that device current.
int setup_device(int dev, DeviceSetup& out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (g_setup[dev].ready) {
    out = g_setup[dev];
    return 0;
  }
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
    return fail("pxg_image_blur_noalloc: cannot resolve the scratch array on this device");
  int nsm = 0, optin = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return fail("pxg_image_blur_noalloc: cannot query the device");
  const void* kernels[] = {pxg::blurb_kernel(true), pxg::blurb_kernel(false), (const void*)pxg::k_blurf_x,
                           (const void*)pxg::k_blurf_y, (const void*)pxg::k_blur_x,
                           (const void*)pxg::k_blur_y};
  size_t maxSmem = (size_t)optin;
  for (const void* k : kernels) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, k) != cudaSuccess)
      return fail("pxg_image_blur_noalloc: cannot query the blur kernels");
    size_t dyn = (size_t)optin > fa.sharedSizeBytes ? (size_t)optin - fa.sharedSizeBytes : 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) != cudaSuccess)
      return fail("pxg_image_blur_noalloc: cannot set the blur kernels' shared memory");
    if (dyn < maxSmem) maxSmem = dyn;
  }
  g_setup[dev] = DeviceSetup{true, (unsigned char*)p, nsm, maxSmem};
  out = g_setup[dev];
  return 0;
}

}  // namespace

extern "C" int pxg_image_blur_noalloc(void* rgbx, int64_t width, int64_t height, float radius,
                                      const float out_of_bounds[4], void* cuda_stream) {
  if (!rgbx || ((uintptr_t)rgbx & 15)) return fail("Device pointer must be non-null and 16-byte aligned");
  if (width <= 0 || height <= 0) return fail("Image width and height must be > 0");
  if (width > kNoAllocMaxPixels || height > kNoAllocMaxPixels || width * height > kNoAllocMaxPixels)
    return fail("pxg_image_blur_noalloc: image larger than 2097152 pixels (use pxg_image_blur)");
  // radius = round(radius).int  (images.nim:308-312)
  const float rf = roundf(radius);
  if (!(rf >= -9223372036854775808.0f && rf < 9223372036854775808.0f)) return fail("Cannot apply negative blur");
  const int64_t r = (int64_t)rf;
  if (r == 0) return 0;
  if (r < 0) return fail("Cannot apply negative blur");
  if (r > kNoAllocMaxRadius) return fail("pxg_image_blur_noalloc: radius above 2048 (use pxg_image_blur)");

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail("pxg_image_blur_noalloc: no usable current device");
  DeviceSetup s;
  if (setup_device(dev, s) != 0) return 1;

  // The weights travel by value, as a kernel parameter, and one small kernel
  // writes them into the head of the scratch array: no host buffer has to
  // outlive the call and the stream never waits for a pageable copy.
  WeightsParam wp;
  float work[2 * kNoAllocMaxRadius + 1];
  pxg::gaussian_kernel_into(r, work, wp.w);
  wp.n = (int)(2 * r + 1);
  cudaStream_t st = (cudaStream_t)cuda_stream;
  k_store_weights<<<(wp.n + 255) / 256, 256, 0, st>>>(wp, (uint16_t*)s.scratch);
  static const float zero[4] = {0, 0, 0, 0};
  const uint32_t oob = pxg::color_to_rgbx(out_of_bounds ? out_of_bounds : zero);
  pxg::launch_blur((uint32_t*)rgbx, (uint32_t*)(s.scratch + kWeightsBytes), width, height, (int)r,
                   (const uint16_t*)s.scratch, oob, s.nsm, s.maxSmem, st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(cudaGetErrorString(e));
  return 0;
}
