// render_noalloc.cu -- nes_render_view_noalloc: the plain FP32 render of one
// view that allocates no device memory.
//
// Who needs it: a caller whose device memory is owned by someone else and
// who may not call cudaMalloc/cudaFree itself -- e.g. a host application
// that hands a plugin a fixed pool carved out at start-up and forbids further
// allocation, or a frame loop that cannot afford the implicit device-wide
// synchronisation cudaMalloc/cudaFree may cause.  Such a caller supplies the
// scene arrays and the output buffers; the only other device memory the
// render needs (the compacted ray list and its counters) is the file-scope
// array below, part of the library's static device data.
//
// Limits and sharing:
//  - at most NES_NOALLOC_MAX_PIXELS (262,144) pixels per call: the array
//    holds one 32-byte ray record per pixel plus the counters, 8 MiB + 256 B;
//    larger views are rejected with NES_EINVAL before anything is launched;
//  - the array is device memory of the library's module, so every GPU on
//    which that module is loaded holds it until the process exits;
//  - every call on a device shares the one array and it keeps the last
//    call's contents: each call clears the counters on its stream before use,
//    and calls whose work overlaps on the GPU (different streams, or other
//    host threads, without ordering between them) race on the array.
//  - the first call on a device (per process) looks up the array's device
//    address with cudaGetSymbolAddress, with that device current; make that
//    first call before any stream capture on that device.  The address is
//    kept for the life of the process: a cudaDeviceReset of the device after
//    that first call (which unloads the module and its array) is not
//    supported.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "ctx_internal.h"
#include "kernels.h"
#include "nes_gb300.h"

namespace nes {
namespace {

constexpr uint32_t kNoAllocMaxRays = NES_NOALLOC_MAX_PIXELS;
constexpr size_t kRayDtBytes = sizeof(float4) * kNoAllocMaxRays;    // 4 MiB
constexpr size_t kRayMetaBytes = sizeof(RayMeta) * kNoAllocMaxRays; // 4 MiB
constexpr size_t kCounterBytes = 256;
constexpr size_t kScratchBytes = kRayDtBytes + kRayMetaBytes + kCounterBytes;
static_assert(kCounterBytes >= kCtrWords * sizeof(uint32_t), "counter block too small");

// The scratch.  In host code this name is only a host-side stand-in for the
// symbol; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_dev[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};

// Set-up, once per device, with that device current.
int scratch_for_current_device(unsigned char** base, int* sms) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return NES_ENODEV;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return NES_EIO;
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return NES_EIO;
    g_scratch_dev[dev] = p;
    g_num_sms[dev] = n;
  }
  *base = static_cast<unsigned char*>(g_scratch_dev[dev]);
  *sms = g_num_sms[dev];
  return NES_OK;
}

}  // namespace
}  // namespace nes

extern "C" int nes_render_view_noalloc(const float* table_dev, uint32_t log2_table_size, const float* weights_dev,
                                       const uint32_t* occupancy_dev, const nes_view* view, float* rgb_dev,
                                       float* depth_dev, void* stream) {
  using namespace nes;
  if (!table_dev || !weights_dev || !occupancy_dev || !view || (!rgb_dev && !depth_dev)) return NES_EINVAL;
  if (log2_table_size < 10 || log2_table_size > 24) return NES_EINVAL;
  if (!view_ok(*view)) return NES_EINVAL;  // the renderer's own view check
  const uint64_t px = (uint64_t)view->width * view->height;
  if (px > kNoAllocMaxRays) return NES_EINVAL;  // beyond the static scratch

  unsigned char* base = nullptr;
  int sms = 0;
  const int rc = scratch_for_current_device(&base, &sms);
  if (rc != NES_OK) return rc;
  DevScratch s;
  s.ray_dt = reinterpret_cast<float4*>(base);
  s.ray_meta = reinterpret_cast<RayMeta*>(base + kRayDtBytes);
  s.counters = reinterpret_cast<uint32_t*>(base + kRayDtBytes + kRayMetaBytes);
  s.max_rays = kNoAllocMaxRays;

  DevScene sc;
  sc.table32 = reinterpret_cast<const float2*>(table_dev);
  sc.weights = weights_dev;
  sc.occ = occupancy_dev;
  sc.T = 1u << log2_table_size;
  sc.dense_mask = dense_level_mask(sc.T);

  ViewBatch vb;
  std::memset(&vb, 0, sizeof(vb));
  vb.n = 1;
  vb.total_pixels = view_threads((int)view->width, (int)view->height);
  std::memcpy(vb.v[0].M, view->matrix, sizeof(vb.v[0].M));
  vb.v[0].W = (int)view->width;
  vb.v[0].H = (int)view->height;
  vb.v[0].focal = view->focal_px;
  vb.v[0].pix_offset = 0;
  vb.v[0].rgb = rgb_dev;
  vb.v[0].depth = depth_dev;

  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // The array keeps the previous call's counters: clear them first.
  if (cudaMemsetAsync(s.counters, 0, kCounterBytes, st) != cudaSuccess) return NES_EIO;
  if (launch_raygen(vb, s, st) != cudaSuccess) return NES_EIO;
  if (launch_march_fp32(vb, sc, s, sms, st) != cudaSuccess) return NES_EIO;
  return NES_OK;
}
