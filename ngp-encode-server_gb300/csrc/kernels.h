// kernels.h -- host-side launchers of the CUDA kernels (one declaration per
// kernel family).  All launchers are asynchronous on `stream` and return the
// launch's cudaError_t.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "render_common.cuh"

namespace nes {

// Device-resident scene handles used by every render kernel.
struct DevScene {
  const float2* table32 = nullptr;  // [16][T] float2
  const __half2* table16 = nullptr; // [16][T] half2 (tensor-core path)
  const uint4* rec16 = nullptr;     // per-cell corner records of levels 0..rec_levels-1 (2 x uint4 each)
  const float* weights = nullptr;   // kWeightFloats FP32 blob
  const uint8_t* tc_weights = nullptr; // FP16 weights in the MMA operand layout
  const uint32_t* occ = nullptr;    // kOccWords
  uint32_t T = 0;
  uint32_t dense_mask = 0;
  uint32_t rec_levels = 0;          // levels with records (kRecLevelsDefault or kRecLevelsSmall)
};

// Per-call scratch shared by the render kernels.
struct DevScratch {
  float4* ray_dt = nullptr;   // compacted rays: direction + t_start
  RayMeta* ray_meta = nullptr;
  uint32_t* counters = nullptr;  // [0] rays, [1] work cursor, [2..3] samples (u64)
  uint32_t max_rays = 0;
};

// Counter slots inside DevScratch::counters.
constexpr int kCtrRays = 0;
constexpr int kCtrCursor = 1;
constexpr int kCtrSamples = 2;  // 64-bit, occupies words 2 and 3
constexpr int kCtrError = 4;    // nonzero: a bounded device wait ran out
constexpr int kCtrWords = 8;

// Ray generation + unit-cube clip + warp-ballot compaction of hits; writes
// zero colour/depth for pixels whose ray misses.  counters must be zeroed.
cudaError_t launch_raygen(const ViewBatch& views, const DevScratch& s, cudaStream_t stream);
// The same with the batch descriptor read from device memory at run time (a
// fixed grid sized for max_pixels, so a captured graph serves any batch).
cudaError_t launch_raygen(const ViewBatch* views_dev, uint32_t max_pixels, int num_sms, const DevScratch& s,
                          cudaStream_t stream);

// Plain FP32 march: persistent CTAs pull compacted rays, evaluate the FP32
// table + FP32 MLP on CUDA cores and composite.
cudaError_t launch_march_fp32(const ViewBatch& views, const DevScene& scene, const DevScratch& s,
                              int num_sms, cudaStream_t stream);
cudaError_t launch_march_fp32(const ViewBatch* views_dev, const DevScene& scene, const DevScratch& s, int num_sms,
                              cudaStream_t stream);

// FP16 tensor-core march (tcgen05 MLP).  Needs scene.table16 and
// scene.tc_weights (the FP16 operand image from launch_pack_tc_weights).
cudaError_t launch_march_tc(const ViewBatch& views, const DevScene& scene, const DevScratch& s,
                            int num_sms, cudaStream_t stream);
cudaError_t launch_march_tc(const ViewBatch* views_dev, const DevScene& scene, const DevScratch& s, int num_sms,
                            cudaStream_t stream);

// Bytes of the per-cell corner records and their construction from the FP16
// table (tensor-core path).
size_t tc_record_bytes(int rec_levels);
cudaError_t launch_build_records(const __half2* table16, uint32_t T, uint32_t dense_mask, int rec_levels, uint4* rec,
                                 cudaStream_t stream);

// Bytes of the FP16 MLP weight image and its packing from the FP32 blob.
size_t tc_weight_bytes();
cudaError_t launch_pack_tc_weights(const float* w32, uint8_t* out, cudaStream_t stream);

// 128^3 occupancy bitfield from the FP32 density at cell centres.
cudaError_t launch_occupancy(const DevScene& scene, float threshold, uint32_t* occ_out,
                             cudaStream_t stream);

// Frame glue.
cudaError_t launch_rgb24_to_yuv420p(const uint8_t* rgb, int w, int h, int rgb_ls, uint8_t* y,
                                    uint8_t* u, uint8_t* v, const int ls[3], cudaStream_t stream);
cudaError_t launch_gray8_to_yuv420p(const uint8_t* g, int w, int h, int g_ls, uint8_t* y, uint8_t* u,
                                    uint8_t* v, const int ls[3], cudaStream_t stream);
cudaError_t launch_depth_pack_u16mm(const float* d, size_t n, uint16_t* out, cudaStream_t stream);
cudaError_t launch_depth_to_gray8(const float* d, size_t n, float dmax, uint8_t* out,
                                  cudaStream_t stream);
cudaError_t launch_rgb_to_rgb24(const float* rgb, size_t n, uint8_t* out, cudaStream_t stream);

// Fused frame output of a rendered batch: per view, FP32 RGB -> RGB24
// quantisation -> YUV420P and FP32 depth -> uint16 mm in one pass, the
// same bytes as launch_rgb_to_rgb24 + launch_rgb24_to_yuv420p +
// launch_depth_pack_u16mm.  Descriptor by value (grid sized to the batch) or
// in device memory (fixed grid of num_sms x 8 blocks, grid-stride).
cudaError_t launch_frame_out(const FrameBatch& fb, cudaStream_t stream);
cudaError_t launch_frame_out(const FrameBatch* fb_dev, int num_sms, cudaStream_t stream);
// Fills fb->f[i].first_block and fb->total_blocks from the views' sizes.
void frame_batch_index(FrameBatch* fb);

// Batched frame glue: up to kMaxBatchFrames frames of one geometry per
// launch, per-frame device pointers passed by value.
constexpr int kMaxBatchFrames = 64;
struct FrameSet {
  const uint8_t* src[kMaxBatchFrames];
  uint8_t* y[kMaxBatchFrames];
  uint8_t* u[kMaxBatchFrames];
  uint8_t* v[kMaxBatchFrames];
};
struct DepthSet {
  const float* src[kMaxBatchFrames];
  uint16_t* dst[kMaxBatchFrames];
};
cudaError_t launch_yuv420p_batch(bool gray, const FrameSet& fs, int nframes, int w, int h, int src_ls,
                                 const int ls[3], cudaStream_t stream);
cudaError_t launch_depth_pack_u16mm_batch(const DepthSet& ds, int nframes, size_t n, cudaStream_t stream);

// Self-test of the bounded device waits: one CTA waits (at most poll_limit
// polls, 1..2^24) on an mbarrier nothing arrives at (arrive = 0) or that it
// completed itself (arrive = 1), and sets counters[kCtrError] when the wait
// ran out.
cudaError_t launch_bounded_wait_probe(uint32_t poll_limit, int arrive, uint32_t* counters, cudaStream_t stream);

// Gather ceilings of the tensor-core march (probe.cu).  gather_probe:
// `threads` threads (a multiple of 256) each make loads_per_thread uniformly
// random loads of load_bytes (4, 16, or 32 as two 16-byte loads) over
// table_bytes (table_bytes / load_bytes a power of two), XOR-folded into
// sink[thread].  gather_replay: the march's own load stream over the rays
// already generated in s (num_sms CTAs of `threads` = 256 or 512 threads;
// sink holds num_sms * threads words).
cudaError_t launch_gather_probe(const void* table, uint64_t table_bytes, int load_bytes, uint32_t loads_per_thread,
                                uint32_t* sink, uint32_t threads, cudaStream_t stream);
cudaError_t launch_gather_replay(const ViewBatch& views, const DevScene& scene, const DevScratch& s, int num_sms,
                                 int threads, uint32_t* sink, cudaStream_t stream);

// FP32 -> FP16 table conversion (level-major, same indexing).
cudaError_t launch_table_to_fp16(const float2* src, __half2* dst, size_t n, cudaStream_t stream);

}  // namespace nes
