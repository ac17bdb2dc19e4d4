// render_fp32.cu -- ray generation + compaction, the plain FP32 march
// (CUDA cores only), the occupancy-grid build and the FP16 table copy.
//
// These kernels stand in for the external instant-ngp-renderer that
// neserver reaches over TCP (src/server.cpp:161-194): a FrameRequest's
// camera becomes one ray per pixel, rays that miss the unit cube are dropped
// by a warp-ballot prefix sum, and the survivors are marched through the
// hash-grid field and composited into RGB and expected depth.
#include <cuda_fp16.h>

#include "kernels.h"
#include "mlp32.cuh"

namespace nes {

namespace {

constexpr int kRaygenThreads = 256;
constexpr int kMarchThreads = 128;

// Grid-stride over the batch's ray-generation threads (the loop bound is
// uniform per block, and every view's thread count is a multiple of 32, so
// each warp's ballot sees whole warps).
template <class Src>
__global__ void __launch_bounds__(kRaygenThreads)
raygen_kernel(const __grid_constant__ Src src, float4* __restrict__ ray_dt, RayMeta* __restrict__ ray_meta,
              uint32_t* __restrict__ counters, uint32_t max_rays) {
  const ViewBatch& vb = src.get();
  const uint32_t total = vb.total_pixels;
  for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
    const uint32_t gid = base + threadIdx.x;
    const bool valid = gid < total;
    int v = 0;
    if (valid)
      while (v + 1 < vb.n && gid >= vb.v[v + 1].pix_offset) ++v;
    int n = 0, pix = 0;
    float3 o, d;
    float ts = 0.0f;
    if (valid) {
      const DevView& V = vb.v[v];
      const uint32_t local = gid - V.pix_offset;
      const uint32_t tile = local / (kTileW * kTileH), in = local % (kTileW * kTileH);
      const uint32_t tiles_x = (uint32_t)(V.W + kTileW - 1) / kTileW;
      const int px = (int)((tile % tiles_x) * kTileW + in % kTileW);
      const int py = (int)((tile / tiles_x) * kTileH + in / kTileW);
      if (px < V.W && py < V.H) {  // tile padding beyond the frame edge does nothing
        pix = py * V.W + px;
        n = ray_setup(V.M, V.W, V.H, V.focal, px, py, o, d, ts);
        if (n == 0) {  // miss: nothing to march, the pixel is black at depth 0
          if (V.rgb) {
            V.rgb[(size_t)pix * 3 + 0] = 0.0f;
            V.rgb[(size_t)pix * 3 + 1] = 0.0f;
            V.rgb[(size_t)pix * 3 + 2] = 0.0f;
          }
          if (V.depth) V.depth[pix] = 0.0f;
        }
      }
    }
    const unsigned lane = threadIdx.x & 31u;
    const unsigned mask = __ballot_sync(0xffffffffu, n > 0);
    if (mask == 0) continue;
    const int leader = __ffs(mask) - 1;
    uint32_t first = 0;
    if ((int)lane == leader) first = atomicAdd(counters + kCtrRays, (uint32_t)__popc(mask));
    first = __shfl_sync(0xffffffffu, first, leader);
    if (n > 0) {
      const uint32_t slot = first + (uint32_t)__popc(mask & ((1u << lane) - 1u));
      if (slot < max_rays) {
        ray_dt[slot] = make_float4(d.x, d.y, d.z, ts);
        ray_meta[slot] = RayMeta{v, pix, n, 0};
      }
    }
  }
}

template <class Src>
__global__ void __launch_bounds__(kMarchThreads)
march_fp32_kernel(const __grid_constant__ Src src, const DevScene sc, const DevScratch s) {
  const ViewBatch& vb = src.get();
  extern __shared__ float4 smem_raw[];
  SmemWeights32& W = *reinterpret_cast<SmemWeights32*>(smem_raw);
  load_weights32(W, sc.weights);
  __syncthreads();

  const uint32_t nrays = min(s.counters[kCtrRays], s.max_rays);
  const unsigned lane = threadIdx.x & 31u;
  unsigned long long my_samples = 0;
  for (;;) {
    const uint32_t base = warp_claim(s.counters + kCtrCursor, 32);
    if (base >= nrays) break;
    const uint32_t r = base + lane;
    if (r < nrays) {
    const float4 rd = s.ray_dt[r];
    const RayMeta m = s.ray_meta[r];
    const DevView& V = vb.v[m.view];
    const float3 o = make_float3(V.M[3], V.M[7], V.M[11]);
    const float3 d = make_float3(rd.x, rd.y, rd.z);
    float sh[16];
    sh16(d, sh);
    float T = 1.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f, dep = 0.0f;
    for (int i = 0; i < m.n; ++i) {
      const float t = fmaf((float)i + 0.5f, kDt, rd.w);
      const float3 x = sample_pos(o, d, t);
      if (!occupied(sc.occ, x)) continue;
      float enc[kEnc];
      encode_fp32(sc.table32, sc.T, sc.dense_mask, x, enc);
      float dout[kDOut];
      density_mlp32(W, enc, dout);
      const float sigma = expf(dout[0] - 1.0f);
      const float3 c = colour_mlp32(W, sh, dout);
      ++my_samples;
      const float alpha = -expm1f(-sigma * kDt);
      const float w = T * alpha;
      cr = fmaf(w, c.x, cr);
      cg = fmaf(w, c.y, cg);
      cb = fmaf(w, c.z, cb);
      dep = fmaf(w, t, dep);
      T -= w;
      if (T < kTStop) break;
    }
    if (V.rgb) {
      V.rgb[(size_t)m.pixel * 3 + 0] = cr;
      V.rgb[(size_t)m.pixel * 3 + 1] = cg;
      V.rgb[(size_t)m.pixel * 3 + 2] = cb;
    }
    if (V.depth) V.depth[m.pixel] = dep;
    }
  }
  // One 64-bit atomic per warp for the sample count.
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) my_samples += __shfl_down_sync(0xffffffffu, my_samples, off);
  if (lane == 0 && my_samples)
    atomicAdd(reinterpret_cast<unsigned long long*>(s.counters + kCtrSamples), my_samples);
}

constexpr int kOccThreads = 128;

__global__ void __launch_bounds__(kOccThreads)
occupancy_kernel(const DevScene sc, float threshold, uint32_t* __restrict__ occ) {
  extern __shared__ float4 smem_raw[];
  SmemWeights32& W = *reinterpret_cast<SmemWeights32*>(smem_raw);
  load_weights32(W, sc.weights);
  __syncthreads();
  const uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x;  // grid covers 128^3 exactly
  const uint32_t cx = cell % kOccRes, cy = (cell / kOccRes) % kOccRes, cz = cell / (kOccRes * kOccRes);
  const float3 x = make_float3(((float)cx + 0.5f) / kOccRes, ((float)cy + 0.5f) / kOccRes,
                               ((float)cz + 0.5f) / kOccRes);
  float enc[kEnc];
  encode_fp32(sc.table32, sc.T, sc.dense_mask, x, enc);
  float dout[kDOut];
  density_mlp32(W, enc, dout);
  const float sigma = expf(dout[0] - 1.0f);
  const unsigned bits = __ballot_sync(0xffffffffu, sigma > threshold);
  if ((threadIdx.x & 31u) == 0) occ[cell >> 5] = bits;
}

__global__ void table_to_fp16_kernel(const float2* __restrict__ src, __half2* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = __float22half2_rn(src[i]);
}

}  // namespace

cudaError_t launch_raygen(const ViewBatch& views, const DevScratch& s, cudaStream_t stream) {
  if (views.total_pixels == 0) return cudaSuccess;
  const unsigned blocks = (views.total_pixels + kRaygenThreads - 1) / kRaygenThreads;
  raygen_kernel<<<blocks, kRaygenThreads, 0, stream>>>(InParam<ViewBatch>{views}, s.ray_dt, s.ray_meta, s.counters,
                                                       s.max_rays);
  return cudaGetLastError();
}

cudaError_t launch_raygen(const ViewBatch* views_dev, uint32_t max_pixels, int num_sms, const DevScratch& s,
                          cudaStream_t stream) {
  // Enough blocks for max_pixels in one pass, at most 8 per SM (grid-stride).
  const unsigned need = (max_pixels + kRaygenThreads - 1) / kRaygenThreads;
  const unsigned cap = (unsigned)num_sms * 8u;
  const unsigned blocks = need < cap ? (need ? need : 1u) : cap;
  raygen_kernel<<<blocks, kRaygenThreads, 0, stream>>>(InMemory<ViewBatch>{views_dev}, s.ray_dt, s.ray_meta,
                                                       s.counters, s.max_rays);
  return cudaGetLastError();
}

namespace {

template <class Src>
cudaError_t launch_march_fp32_src(const Src& src, const DevScene& scene, const DevScratch& s, int num_sms,
                                  cudaStream_t stream) {
  const int smem = (int)sizeof(SmemWeights32);
  static bool attr_set = false;  // idempotent; harmless if two threads race on it
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(march_fp32_kernel<Src>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  int per_sm = 0;
  cudaError_t e =
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_fp32_kernel<Src>, kMarchThreads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  march_fp32_kernel<Src><<<num_sms * per_sm, kMarchThreads, smem, stream>>>(src, scene, s);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_march_fp32(const ViewBatch& views, const DevScene& scene, const DevScratch& s,
                              int num_sms, cudaStream_t stream) {
  return launch_march_fp32_src(InParam<ViewBatch>{views}, scene, s, num_sms, stream);
}

cudaError_t launch_march_fp32(const ViewBatch* views_dev, const DevScene& scene, const DevScratch& s, int num_sms,
                              cudaStream_t stream) {
  return launch_march_fp32_src(InMemory<ViewBatch>{views_dev}, scene, s, num_sms, stream);
}

cudaError_t launch_occupancy(const DevScene& scene, float threshold, uint32_t* occ_out, cudaStream_t stream) {
  const int smem = (int)sizeof(SmemWeights32);
  cudaError_t e = cudaFuncSetAttribute(occupancy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const unsigned cells = kOccRes * kOccRes * kOccRes;
  occupancy_kernel<<<cells / kOccThreads, kOccThreads, smem, stream>>>(scene, threshold, occ_out);
  return cudaGetLastError();
}

cudaError_t launch_table_to_fp16(const float2* src, __half2* dst, size_t n, cudaStream_t stream) {
  table_to_fp16_kernel<<<1024, 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError();
}

}  // namespace nes
