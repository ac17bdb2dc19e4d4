// glue.cu -- frame glue kernels: RGB24/GRAY8 -> YUV420P, depth packing and
// quantisation.  They replace RenderedFrame::convert_frame, which runs
// libswscale on the CPU once per eye and frame
// (include/base/video/rendered_frame.h:24-33,
// src/base/video/type_managers.cc:241-251), writing the YUV420P plane layout
// that AVCodecContextManager::send_frame consumes (src/encode.cpp:136-137).
//
// Conversion: ITU-R BT.601 studio range in fixed point (coefficients in
// nes_spec.h).  Luma per pixel with 16 fractional bits; chroma from the sum
// of each 2x2 block (18 fractional bits = block average), with the last row
// and column replicated when a dimension is odd.  All integer, so the result
// is bit-exact against the CPU restatement.  Every kernel is HBM-bound.
#include "kernels.h"

namespace nes {

namespace {

constexpr int kGlueThreads = 256;

__device__ __forceinline__ uint8_t clamp8(int32_t v) { return (uint8_t)min(max(v, 0), 255); }

__device__ __forceinline__ uint8_t luma(int r, int g, int b) {
  return clamp8((kYR * r + kYG * g + kYB * b + (16 << 16) + (1 << 15)) >> 16);
}

// One thread per 2x2 block: 4 luma samples and one Cb/Cr pair.
__global__ void __launch_bounds__(kGlueThreads)
rgb24_to_yuv420p_kernel(const uint8_t* __restrict__ rgb, int w, int h, int rgb_ls, uint8_t* __restrict__ Y,
                        uint8_t* __restrict__ U, uint8_t* __restrict__ V, int ls0, int ls1, int ls2) {
  const int cw = (w + 1) >> 1, ch = (h + 1) >> 1;
  const int cx = blockIdx.x * blockDim.x + threadIdx.x;
  const int cy = blockIdx.y;
  if (cx >= cw || cy >= ch) return;
  int sr = 0, sg = 0, sb = 0;
#pragma unroll
  for (int dy = 0; dy < 2; ++dy) {
    const int yy = 2 * cy + dy;
    const int ry = min(yy, h - 1);
    const uint8_t* row = rgb + (size_t)ry * rgb_ls;
#pragma unroll
    for (int dx = 0; dx < 2; ++dx) {
      const int xx = 2 * cx + dx;
      const int rx = min(xx, w - 1);
      const int r = row[3 * rx], g = row[3 * rx + 1], b = row[3 * rx + 2];
      sr += r;
      sg += g;
      sb += b;
      if (yy < h && xx < w) Y[(size_t)yy * ls0 + xx] = luma(r, g, b);
    }
  }
  U[(size_t)cy * ls1 + cx] = clamp8((kUR * sr + kUG * sg + kUB * sb + (128 << 18) + (1 << 17)) >> 18);
  V[(size_t)cy * ls2 + cx] = clamp8((kVR * sr + kVG * sg + kVB * sb + (128 << 18) + (1 << 17)) >> 18);
}

__global__ void __launch_bounds__(kGlueThreads)
gray8_to_yuv420p_kernel(const uint8_t* __restrict__ g, int w, int h, int g_ls, uint8_t* __restrict__ Y,
                        uint8_t* __restrict__ U, uint8_t* __restrict__ V, int ls0, int ls1, int ls2) {
  const int cw = (w + 1) >> 1, ch = (h + 1) >> 1;
  const int cx = blockIdx.x * blockDim.x + threadIdx.x;
  const int cy = blockIdx.y;
  if (cx >= cw || cy >= ch) return;
  constexpr int32_t ys = kYR + kYG + kYB;
#pragma unroll
  for (int dy = 0; dy < 2; ++dy) {
    const int yy = 2 * cy + dy;
    if (yy >= h) break;
#pragma unroll
    for (int dx = 0; dx < 2; ++dx) {
      const int xx = 2 * cx + dx;
      if (xx < w) Y[(size_t)yy * ls0 + xx] = clamp8((ys * g[(size_t)yy * g_ls + xx] + (16 << 16) + (1 << 15)) >> 16);
    }
  }
  U[(size_t)cy * ls1 + cx] = 128;
  V[(size_t)cy * ls2 + cx] = 128;
}

// round-half-up of d * 1000 in FP32; NaN/negative -> 0; saturate at 65535.
__global__ void depth_pack_u16mm_kernel(const float* __restrict__ d, size_t n, uint16_t* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float mm = __fmul_rn(d[i], 1000.0f);
    uint16_t q;
    if (!(mm >= 0.0f))
      q = 0;
    else if (mm >= 65535.0f)
      q = 65535;
    else
      q = (uint16_t)__float2uint_rz(__fadd_rn(mm, 0.5f));
    out[i] = q;
  }
}

__global__ void depth_to_gray8_kernel(const float* __restrict__ d, size_t n, float dmax, uint8_t* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float q = __fdiv_rn(d[i], dmax);
    const float c = q > 0.0f ? (q < 1.0f ? q : 1.0f) : 0.0f;
    out[i] = (uint8_t)__float2uint_rz(__fadd_rn(__fmul_rn(c, 255.0f), 0.5f));
  }
}

__global__ void rgb_to_rgb24_kernel(const float* __restrict__ rgb, size_t n, uint8_t* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float x = rgb[i];
    const float c = x > 0.0f ? (x < 1.0f ? x : 1.0f) : 0.0f;
    out[i] = (uint8_t)__float2uint_rz(__fadd_rn(__fmul_rn(c, 255.0f), 0.5f));
  }
}

unsigned grid_for(size_t n) {
  size_t b = (n + kGlueThreads - 1) / kGlueThreads;
  if (b > 152 * 32) b = 152 * 32;  // grid-stride beyond 32 resident blocks per SM
  return (unsigned)(b ? b : 1);
}

}  // namespace

cudaError_t launch_rgb24_to_yuv420p(const uint8_t* rgb, int w, int h, int rgb_ls, uint8_t* y, uint8_t* u,
                                    uint8_t* v, const int ls[3], cudaStream_t stream) {
  const int cw = (w + 1) / 2, ch = (h + 1) / 2;
  dim3 grid((cw + kGlueThreads - 1) / kGlueThreads, ch);
  rgb24_to_yuv420p_kernel<<<grid, kGlueThreads, 0, stream>>>(rgb, w, h, rgb_ls, y, u, v, ls[0], ls[1], ls[2]);
  return cudaGetLastError();
}

cudaError_t launch_gray8_to_yuv420p(const uint8_t* g, int w, int h, int g_ls, uint8_t* y, uint8_t* u, uint8_t* v,
                                    const int ls[3], cudaStream_t stream) {
  const int cw = (w + 1) / 2, ch = (h + 1) / 2;
  dim3 grid((cw + kGlueThreads - 1) / kGlueThreads, ch);
  gray8_to_yuv420p_kernel<<<grid, kGlueThreads, 0, stream>>>(g, w, h, g_ls, y, u, v, ls[0], ls[1], ls[2]);
  return cudaGetLastError();
}

cudaError_t launch_depth_pack_u16mm(const float* d, size_t n, uint16_t* out, cudaStream_t stream) {
  depth_pack_u16mm_kernel<<<grid_for(n), kGlueThreads, 0, stream>>>(d, n, out);
  return cudaGetLastError();
}

cudaError_t launch_depth_to_gray8(const float* d, size_t n, float dmax, uint8_t* out, cudaStream_t stream) {
  depth_to_gray8_kernel<<<grid_for(n), kGlueThreads, 0, stream>>>(d, n, dmax, out);
  return cudaGetLastError();
}

cudaError_t launch_rgb_to_rgb24(const float* rgb, size_t n, uint8_t* out, cudaStream_t stream) {
  rgb_to_rgb24_kernel<<<grid_for(n), kGlueThreads, 0, stream>>>(rgb, n, out);
  return cudaGetLastError();
}

}  // namespace nes
