// glue.cu -- frame glue kernels: RGB24/GRAY8 -> YUV420P, depth packing and
// quantisation.  They replace RenderedFrame::convert_frame, which runs
// libswscale on the CPU once per eye and frame
// (include/base/video/rendered_frame.h:24-33,
// src/base/video/type_managers.cc:143-153), writing the YUV420P plane layout
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

// Vector form of the two YUV kernels: one thread per 8x2 pixel block (four
// chroma samples), 8-byte row loads and stores, 4-byte chroma stores.  Used
// when every base pointer and linesize is aligned (RGB/GRAY/Y to 8 bytes,
// U/V to 4); blocks that reach past the right or bottom edge take the
// per-sample path of the kernels above, so results are identical.
__device__ __forceinline__ void rgb_block_scalar(const uint8_t* __restrict__ rgb, int w, int h, int rgb_ls,
                                                 uint8_t* __restrict__ Y, uint8_t* __restrict__ U,
                                                 uint8_t* __restrict__ V, int ls0, int ls1, int ls2, int cx,
                                                 int cy) {
  int sr = 0, sg = 0, sb = 0;
#pragma unroll
  for (int dy = 0; dy < 2; ++dy) {
    const int yy = 2 * cy + dy;
    const uint8_t* row = rgb + (size_t)min(yy, h - 1) * rgb_ls;
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

__device__ __forceinline__ void rgb24_to_yuv420p_v8(const uint8_t* __restrict__ rgb, int w, int h, int rgb_ls,
                                                    uint8_t* __restrict__ Y, uint8_t* __restrict__ U,
                                                    uint8_t* __restrict__ V, int ls0, int ls1, int ls2) {
  const int cw = (w + 1) >> 1, ch = (h + 1) >> 1;
  const int cx0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int cy = blockIdx.y;
  if (cx0 >= cw || cy >= ch) return;
  const int x0 = 2 * cx0;
  if (x0 + 8 > w || 2 * cy + 1 >= h) {
    for (int cx = cx0; cx < min(cx0 + 4, cw); ++cx) rgb_block_scalar(rgb, w, h, rgb_ls, Y, U, V, ls0, ls1, ls2, cx, cy);
    return;
  }
  uint32_t px[2][6];  // two rows of 8 RGB pixels (24 bytes each)
#pragma unroll
  for (int dy = 0; dy < 2; ++dy) {
    const uint2* p = reinterpret_cast<const uint2*>(rgb + (size_t)(2 * cy + dy) * rgb_ls + 3 * x0);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const uint2 v = __ldg(p + k);
      px[dy][2 * k] = v.x;
      px[dy][2 * k + 1] = v.y;
    }
  }
  int sr[4] = {0, 0, 0, 0}, sg[4] = {0, 0, 0, 0}, sb[4] = {0, 0, 0, 0};
#pragma unroll
  for (int dy = 0; dy < 2; ++dy) {
    uint32_t yw[2] = {0u, 0u};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = (px[dy][(3 * i) >> 2] >> (8 * ((3 * i) & 3))) & 0xff;
      const int g = (px[dy][(3 * i + 1) >> 2] >> (8 * ((3 * i + 1) & 3))) & 0xff;
      const int b = (px[dy][(3 * i + 2) >> 2] >> (8 * ((3 * i + 2) & 3))) & 0xff;
      yw[i >> 2] |= (uint32_t)luma(r, g, b) << (8 * (i & 3));
      sr[i >> 1] += r;
      sg[i >> 1] += g;
      sb[i >> 1] += b;
    }
    *reinterpret_cast<uint2*>(Y + (size_t)(2 * cy + dy) * ls0 + x0) = make_uint2(yw[0], yw[1]);
  }
  uint32_t uw = 0u, vw = 0u;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    uw |= (uint32_t)clamp8((kUR * sr[c] + kUG * sg[c] + kUB * sb[c] + (128 << 18) + (1 << 17)) >> 18) << (8 * c);
    vw |= (uint32_t)clamp8((kVR * sr[c] + kVG * sg[c] + kVB * sb[c] + (128 << 18) + (1 << 17)) >> 18) << (8 * c);
  }
  *reinterpret_cast<uint32_t*>(U + (size_t)cy * ls1 + cx0) = uw;
  *reinterpret_cast<uint32_t*>(V + (size_t)cy * ls2 + cx0) = vw;
}

__device__ __forceinline__ void gray8_to_yuv420p_v8(const uint8_t* __restrict__ g, int w, int h, int g_ls,
                                                    uint8_t* __restrict__ Y, uint8_t* __restrict__ U,
                                                    uint8_t* __restrict__ V, int ls0, int ls1, int ls2) {
  const int cw = (w + 1) >> 1, ch = (h + 1) >> 1;
  const int cx0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int cy = blockIdx.y;
  if (cx0 >= cw || cy >= ch) return;
  constexpr int32_t ys = kYR + kYG + kYB;
  const int x0 = 2 * cx0;
  if (x0 + 8 > w || 2 * cy + 1 >= h) {
    for (int dy = 0; dy < 2; ++dy) {
      const int yy = 2 * cy + dy;
      if (yy >= h) break;
      for (int xx = x0; xx < min(x0 + 8, w); ++xx)
        Y[(size_t)yy * ls0 + xx] = clamp8((ys * g[(size_t)yy * g_ls + xx] + (16 << 16) + (1 << 15)) >> 16);
    }
    for (int cx = cx0; cx < min(cx0 + 4, cw); ++cx) {
      U[(size_t)cy * ls1 + cx] = 128;
      V[(size_t)cy * ls2 + cx] = 128;
    }
    return;
  }
#pragma unroll
  for (int dy = 0; dy < 2; ++dy) {
    const uint2 v = __ldg(reinterpret_cast<const uint2*>(g + (size_t)(2 * cy + dy) * g_ls + x0));
    const uint32_t in[2] = {v.x, v.y};
    uint32_t yw[2] = {0u, 0u};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int gv = (in[i >> 2] >> (8 * (i & 3))) & 0xff;
      yw[i >> 2] |= (uint32_t)clamp8((ys * gv + (16 << 16) + (1 << 15)) >> 16) << (8 * (i & 3));
    }
    *reinterpret_cast<uint2*>(Y + (size_t)(2 * cy + dy) * ls0 + x0) = make_uint2(yw[0], yw[1]);
  }
  *reinterpret_cast<uint32_t*>(U + (size_t)cy * ls1 + cx0) = 0x80808080u;
  *reinterpret_cast<uint32_t*>(V + (size_t)cy * ls2 + cx0) = 0x80808080u;
}

__global__ void __launch_bounds__(kGlueThreads)
rgb24_to_yuv420p_v8_kernel(const uint8_t* __restrict__ rgb, int w, int h, int rgb_ls, uint8_t* __restrict__ Y,
                           uint8_t* __restrict__ U, uint8_t* __restrict__ V, int ls0, int ls1, int ls2) {
  rgb24_to_yuv420p_v8(rgb, w, h, rgb_ls, Y, U, V, ls0, ls1, ls2);
}

__global__ void __launch_bounds__(kGlueThreads)
gray8_to_yuv420p_v8_kernel(const uint8_t* __restrict__ g, int w, int h, int g_ls, uint8_t* __restrict__ Y,
                           uint8_t* __restrict__ U, uint8_t* __restrict__ V, int ls0, int ls1, int ls2) {
  gray8_to_yuv420p_v8(g, w, h, g_ls, Y, U, V, ls0, ls1, ls2);
}

// Batched forms: frame f = blockIdx.z of one launch, same geometry and
// linesizes for every frame, per-frame plane pointers in the parameter table.
__global__ void __launch_bounds__(kGlueThreads)
rgb24_to_yuv420p_batch_kernel(const FrameSet fs, int w, int h, int src_ls, int ls0, int ls1, int ls2, int vec) {
  const int f = blockIdx.z;
  if (vec) {
    rgb24_to_yuv420p_v8(fs.src[f], w, h, src_ls, fs.y[f], fs.u[f], fs.v[f], ls0, ls1, ls2);
  } else {
    const int cx = blockIdx.x * blockDim.x + threadIdx.x, cy = blockIdx.y;
    if (cx < (w + 1) >> 1 && cy < (h + 1) >> 1)
      rgb_block_scalar(fs.src[f], w, h, src_ls, fs.y[f], fs.u[f], fs.v[f], ls0, ls1, ls2, cx, cy);
  }
}

__global__ void __launch_bounds__(kGlueThreads)
gray8_to_yuv420p_batch_kernel(const FrameSet fs, int w, int h, int src_ls, int ls0, int ls1, int ls2, int vec) {
  const int f = blockIdx.z;
  if (vec) {
    gray8_to_yuv420p_v8(fs.src[f], w, h, src_ls, fs.y[f], fs.u[f], fs.v[f], ls0, ls1, ls2);
    return;
  }
  const int cx = blockIdx.x * blockDim.x + threadIdx.x, cy = blockIdx.y;
  if (cx >= (w + 1) >> 1 || cy >= (h + 1) >> 1) return;
  constexpr int32_t ys = kYR + kYG + kYB;
  const uint8_t* g = fs.src[f];
  for (int dy = 0; dy < 2; ++dy) {
    const int yy = 2 * cy + dy;
    if (yy >= h) break;
    for (int dx = 0; dx < 2; ++dx) {
      const int xx = 2 * cx + dx;
      if (xx < w) fs.y[f][(size_t)yy * ls0 + xx] = clamp8((ys * g[(size_t)yy * src_ls + xx] + (16 << 16) + (1 << 15)) >> 16);
    }
  }
  fs.u[f][(size_t)cy * ls1 + cx] = 128;
  fs.v[f][(size_t)cy * ls2 + cx] = 128;
}

// round-half-up of d * 1000 in FP32; NaN/negative -> 0; saturate at 65535.
__device__ __forceinline__ uint16_t pack_mm(float d) {
  const float mm = __fmul_rn(d, 1000.0f);
  if (!(mm >= 0.0f)) return 0;
  if (mm >= 65535.0f) return 65535;
  return (uint16_t)__float2uint_rz(__fadd_rn(mm, 0.5f));
}

__device__ __forceinline__ uint8_t gray_q(float d, float dmax) {
  const float q = __fdiv_rn(d, dmax);
  const float c = q > 0.0f ? (q < 1.0f ? q : 1.0f) : 0.0f;
  return (uint8_t)__float2uint_rz(__fadd_rn(__fmul_rn(c, 255.0f), 0.5f));
}

__device__ __forceinline__ uint8_t unit_q(float x) {
  const float c = x > 0.0f ? (x < 1.0f ? x : 1.0f) : 0.0f;
  return (uint8_t)__float2uint_rz(__fadd_rn(__fmul_rn(c, 255.0f), 0.5f));
}

// Elementwise kernels: four elements per step with a float4 load when the
// input is 16-byte aligned and the output aligned to its 4-element store
// (the host checks), elements past the last whole group scalar.
__global__ void depth_pack_u16mm_kernel(const float* __restrict__ d, size_t n, uint16_t* __restrict__ out, int vec) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  size_t done = 0;
  if (vec) {
    const size_t n4 = n / 4;
    for (size_t i = i0; i < n4; i += stride) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(d) + i);
      reinterpret_cast<uint2*>(out)[i] =
          make_uint2((uint32_t)pack_mm(v.x) | ((uint32_t)pack_mm(v.y) << 16),
                     (uint32_t)pack_mm(v.z) | ((uint32_t)pack_mm(v.w) << 16));
    }
    done = n4 * 4;
  }
  for (size_t i = done + i0; i < n; i += stride) out[i] = pack_mm(d[i]);
}

// Batched depth packing: frame f = blockIdx.y, n elements per frame.
__global__ void depth_pack_u16mm_batch_kernel(const DepthSet ds, size_t n, int vec) {
  const int f = blockIdx.y;
  const float* __restrict__ d = ds.src[f];
  uint16_t* __restrict__ out = ds.dst[f];
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t i0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  size_t done = 0;
  if (vec) {
    const size_t n4 = n / 4;
    for (size_t i = i0; i < n4; i += stride) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(d) + i);
      reinterpret_cast<uint2*>(out)[i] =
          make_uint2((uint32_t)pack_mm(v.x) | ((uint32_t)pack_mm(v.y) << 16),
                     (uint32_t)pack_mm(v.z) | ((uint32_t)pack_mm(v.w) << 16));
    }
    done = n4 * 4;
  }
  for (size_t i = done + i0; i < n; i += stride) out[i] = pack_mm(d[i]);
}

__global__ void depth_to_gray8_kernel(const float* __restrict__ d, size_t n, float dmax, uint8_t* __restrict__ out,
                                      int vec) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  size_t done = 0;
  if (vec) {
    const size_t n4 = n / 4;
    for (size_t i = i0; i < n4; i += stride) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(d) + i);
      reinterpret_cast<uint32_t*>(out)[i] = (uint32_t)gray_q(v.x, dmax) | ((uint32_t)gray_q(v.y, dmax) << 8) |
                                            ((uint32_t)gray_q(v.z, dmax) << 16) | ((uint32_t)gray_q(v.w, dmax) << 24);
    }
    done = n4 * 4;
  }
  for (size_t i = done + i0; i < n; i += stride) out[i] = gray_q(d[i], dmax);
}

__global__ void rgb_to_rgb24_kernel(const float* __restrict__ rgb, size_t n, uint8_t* __restrict__ out, int vec) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  size_t done = 0;
  if (vec) {
    const size_t n4 = n / 4;
    for (size_t i = i0; i < n4; i += stride) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(rgb) + i);
      reinterpret_cast<uint32_t*>(out)[i] = (uint32_t)unit_q(v.x) | ((uint32_t)unit_q(v.y) << 8) |
                                            ((uint32_t)unit_q(v.z) << 16) | ((uint32_t)unit_q(v.w) << 24);
    }
    done = n4 * 4;
  }
  for (size_t i = done + i0; i < n; i += stride) out[i] = unit_q(rgb[i]);
}

// Fused frame output: one thread per 2x2 pixel block of a view of the
// batch.  Each pixel's FP32 colour is quantised to RGB24 (unit_q), its luma
// written, the block's chroma computed from the quantised 2x2 sum (edge
// pixels replicated for odd sizes, as rgb24_to_yuv420p does) and its depth
// packed to uint16 mm: byte for byte the three-kernel sequence, without the
// RGB24 intermediate in memory.
template <class Src>
__global__ void __launch_bounds__(kGlueThreads) frame_out_kernel(const __grid_constant__ Src src) {
  const FrameBatch& fb = src.get();
  const uint32_t total = fb.total_blocks;
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < total; b += gridDim.x * blockDim.x) {
    int vi = 0;
    while (vi + 1 < fb.n && b >= fb.f[vi + 1].first_block) ++vi;
    const FrameOut& F = fb.f[vi];
    const uint32_t local = b - F.first_block;
    const uint32_t cw = (uint32_t)(F.w + 1) >> 1;
    const int cx = (int)(local % cw), cy = (int)(local / cw);
    int sr = 0, sg = 0, sb = 0;
#pragma unroll
    for (int dy = 0; dy < 2; ++dy) {
      const int yy = 2 * cy + dy;
      const size_t row = (size_t)min(yy, F.h - 1) * (size_t)F.w;
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const int xx = 2 * cx + dx;
        const size_t p = row + (size_t)min(xx, F.w - 1);
        const int r = unit_q(__ldg(F.rgb + 3 * p)), g = unit_q(__ldg(F.rgb + 3 * p + 1)),
                  bl = unit_q(__ldg(F.rgb + 3 * p + 2));
        sr += r;
        sg += g;
        sb += bl;
        if (yy < F.h && xx < F.w) {
          F.y[(size_t)yy * F.ls0 + xx] = luma(r, g, bl);
          if (F.depth_mm) F.depth_mm[p] = pack_mm(__ldg(F.depth + p));
        }
      }
    }
    F.u[(size_t)cy * F.ls1 + cx] = clamp8((kUR * sr + kUG * sg + kUB * sb + (128 << 18) + (1 << 17)) >> 18);
    F.v[(size_t)cy * F.ls2 + cx] = clamp8((kVR * sr + kVG * sg + kVB * sb + (128 << 18) + (1 << 17)) >> 18);
    if (cx == (int)cw - 1) {
      // The row padding up to each linesize is zeroed, so no plane carries
      // bytes of an earlier frame (serving reuses its output arena).
      for (int dy = 0; dy < 2; ++dy) {
        const int yy = 2 * cy + dy;
        if (yy < F.h)
          for (int xx = F.w; xx < F.ls0; ++xx) F.y[(size_t)yy * F.ls0 + xx] = 0;
      }
      for (int xx = (int)cw; xx < F.ls1; ++xx) F.u[(size_t)cy * F.ls1 + xx] = 0;
      for (int xx = (int)cw; xx < F.ls2; ++xx) F.v[(size_t)cy * F.ls2 + xx] = 0;
    }
  }
}

unsigned grid_for(size_t n) {
  size_t b = (n + 4 * kGlueThreads - 1) / (4 * kGlueThreads);
  if (b > 152 * 8) b = 152 * 8;  // grid-stride beyond 8 resident blocks per SM
  return (unsigned)(b ? b : 1);
}

bool aligned(const void* p, size_t a) { return ((uintptr_t)p % a) == 0; }

}  // namespace

namespace {

bool yuv_vec_ok(const uint8_t* src, int src_ls, const uint8_t* y, const uint8_t* u, const uint8_t* v,
                const int ls[3]) {
  return aligned(src, 8) && src_ls % 8 == 0 && aligned(y, 8) && ls[0] % 8 == 0 && aligned(u, 4) && ls[1] % 4 == 0 &&
         aligned(v, 4) && ls[2] % 4 == 0;
}

}  // namespace

cudaError_t launch_rgb24_to_yuv420p(const uint8_t* rgb, int w, int h, int rgb_ls, uint8_t* y, uint8_t* u,
                                    uint8_t* v, const int ls[3], cudaStream_t stream) {
  const int cw = (w + 1) / 2, ch = (h + 1) / 2;
  if (yuv_vec_ok(rgb, rgb_ls, y, u, v, ls)) {
    const int groups = (cw + 3) / 4;
    dim3 grid((groups + kGlueThreads - 1) / kGlueThreads, ch);
    rgb24_to_yuv420p_v8_kernel<<<grid, kGlueThreads, 0, stream>>>(rgb, w, h, rgb_ls, y, u, v, ls[0], ls[1], ls[2]);
  } else {
    dim3 grid((cw + kGlueThreads - 1) / kGlueThreads, ch);
    rgb24_to_yuv420p_kernel<<<grid, kGlueThreads, 0, stream>>>(rgb, w, h, rgb_ls, y, u, v, ls[0], ls[1], ls[2]);
  }
  return cudaGetLastError();
}

cudaError_t launch_gray8_to_yuv420p(const uint8_t* g, int w, int h, int g_ls, uint8_t* y, uint8_t* u, uint8_t* v,
                                    const int ls[3], cudaStream_t stream) {
  const int cw = (w + 1) / 2, ch = (h + 1) / 2;
  if (yuv_vec_ok(g, g_ls, y, u, v, ls)) {
    const int groups = (cw + 3) / 4;
    dim3 grid((groups + kGlueThreads - 1) / kGlueThreads, ch);
    gray8_to_yuv420p_v8_kernel<<<grid, kGlueThreads, 0, stream>>>(g, w, h, g_ls, y, u, v, ls[0], ls[1], ls[2]);
  } else {
    dim3 grid((cw + kGlueThreads - 1) / kGlueThreads, ch);
    gray8_to_yuv420p_kernel<<<grid, kGlueThreads, 0, stream>>>(g, w, h, g_ls, y, u, v, ls[0], ls[1], ls[2]);
  }
  return cudaGetLastError();
}

cudaError_t launch_depth_pack_u16mm(const float* d, size_t n, uint16_t* out, cudaStream_t stream) {
  depth_pack_u16mm_kernel<<<grid_for(n), kGlueThreads, 0, stream>>>(d, n, out, aligned(d, 16) && aligned(out, 8));
  return cudaGetLastError();
}

cudaError_t launch_depth_to_gray8(const float* d, size_t n, float dmax, uint8_t* out, cudaStream_t stream) {
  depth_to_gray8_kernel<<<grid_for(n), kGlueThreads, 0, stream>>>(d, n, dmax, out, aligned(d, 16) && aligned(out, 4));
  return cudaGetLastError();
}

cudaError_t launch_rgb_to_rgb24(const float* rgb, size_t n, uint8_t* out, cudaStream_t stream) {
  rgb_to_rgb24_kernel<<<grid_for(n), kGlueThreads, 0, stream>>>(rgb, n, out, aligned(rgb, 16) && aligned(out, 4));
  return cudaGetLastError();
}

cudaError_t launch_yuv420p_batch(bool gray, const FrameSet& fs, int nframes, int w, int h, int src_ls,
                                 const int ls[3], cudaStream_t stream) {
  if (nframes < 1 || nframes > kMaxBatchFrames) return cudaErrorInvalidValue;
  bool vec = true;
  for (int f = 0; f < nframes; ++f) vec = vec && yuv_vec_ok(fs.src[f], src_ls, fs.y[f], fs.u[f], fs.v[f], ls);
  const int cw = (w + 1) / 2, ch = (h + 1) / 2;
  const int xs = vec ? (cw + 3) / 4 : cw;
  dim3 grid((xs + kGlueThreads - 1) / kGlueThreads, ch, nframes);
  if (gray)
    gray8_to_yuv420p_batch_kernel<<<grid, kGlueThreads, 0, stream>>>(fs, w, h, src_ls, ls[0], ls[1], ls[2], vec);
  else
    rgb24_to_yuv420p_batch_kernel<<<grid, kGlueThreads, 0, stream>>>(fs, w, h, src_ls, ls[0], ls[1], ls[2], vec);
  return cudaGetLastError();
}

cudaError_t launch_depth_pack_u16mm_batch(const DepthSet& ds, int nframes, size_t n, cudaStream_t stream) {
  if (nframes < 1 || nframes > kMaxBatchFrames) return cudaErrorInvalidValue;
  bool vec = true;
  for (int f = 0; f < nframes; ++f) vec = vec && aligned(ds.src[f], 16) && aligned(ds.dst[f], 8);
  unsigned gx = grid_for(n * (size_t)nframes) / (unsigned)nframes;
  dim3 grid(gx ? gx : 1, nframes);
  depth_pack_u16mm_batch_kernel<<<grid, kGlueThreads, 0, stream>>>(ds, n, vec);
  return cudaGetLastError();
}

void frame_batch_index(FrameBatch* fb) {
  uint32_t blocks = 0;
  for (int i = 0; i < fb->n; ++i) {
    fb->f[i].first_block = blocks;
    blocks += (uint32_t)((fb->f[i].w + 1) / 2) * (uint32_t)((fb->f[i].h + 1) / 2);
  }
  fb->total_blocks = blocks;
}

cudaError_t launch_frame_out(const FrameBatch& fb, cudaStream_t stream) {
  if (fb.total_blocks == 0) return cudaSuccess;
  frame_out_kernel<<<(fb.total_blocks + kGlueThreads - 1) / kGlueThreads, kGlueThreads, 0, stream>>>(
      InParam<FrameBatch>{fb});
  return cudaGetLastError();
}

cudaError_t launch_frame_out(const FrameBatch* fb_dev, int num_sms, cudaStream_t stream) {
  frame_out_kernel<<<(unsigned)num_sms * 8u, kGlueThreads, 0, stream>>>(InMemory<FrameBatch>{fb_dev});
  return cudaGetLastError();
}

}  // namespace nes
