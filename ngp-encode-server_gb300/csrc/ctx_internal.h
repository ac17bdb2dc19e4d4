// ctx_internal.h -- the rendering context behind nes_ctx and the batch
// helpers shared by the synchronous C ABI (nes_api.cu) and the serving loop
// (serve.cu).
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "kernels.h"
#include "nes_gb300.h"

struct nes_ctx {
  nes_config cfg{};
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  std::mutex mu;

  float2* d_table32 = nullptr;
  __half2* d_table16 = nullptr;
  uint4* d_rec16 = nullptr;
  float* d_weights = nullptr;
  uint8_t* d_tc_weights = nullptr;
  uint32_t* d_occ = nullptr;
  nes::DevScene scene;

  nes::DevScratch scratch;
  float* d_rgb = nullptr;         // max_pixels * 3
  float* d_depth = nullptr;       // max_pixels
  uint8_t* d_rgb8 = nullptr;      // max_pixels * 3
  uint8_t* d_gray = nullptr;      // max_pixels
  uint8_t* d_yuv = nullptr;       // yuv_capacity
  size_t yuv_capacity = 0;
  uint16_t* d_depth16 = nullptr;  // max_pixels

  uint64_t last_samples = 0;
  bool samples_pending = false;

  bool profiling = false;
  bool timings_pending = false;
  cudaEvent_t ev_t[3] = {nullptr, nullptr, nullptr};
};

namespace nes {

// A view the renderer accepts: 1..16384 pixels on each side, a finite
// positive focal length and a finite pose matrix.
bool view_ok(const nes_view& v);

// Validates views and fills the kernel-side batch descriptor.  *pixels
// receives the batch's real pixel count.  NES_EINVAL on a bad view, more
// than kMaxViews views, or more than max_pixels pixels.
int fill_view_batch(const nes_view* views, int n, float* const* rgb, float* const* depth, uint64_t max_pixels,
                    ViewBatch* vb, uint64_t* pixels);

// Queues the render of a batch on `stream`: counter reset, ray generation
// with compaction, and the march of the given precision.
cudaError_t enqueue_march(const ViewBatch& vb, const DevScene& scene, const DevScratch& s, int precision, int num_sms,
                          cudaStream_t stream);

}  // namespace nes
