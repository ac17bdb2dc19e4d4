// render_common.cuh -- device pieces shared by every render kernel: ray
// set-up, occupancy lookup, hash-grid addressing, spherical harmonics.
// The math is that of the renderer neserver calls over TCP
// (src/server.cpp:161-194), fixed by nes_spec.h.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "nes_spec.h"

namespace nes {

constexpr int kMaxViews = 64;

struct DevView {
  float M[12];          // 3x4 row-major pose
  int W, H;
  float focal;
  uint32_t pix_offset;  // first ray-generation thread of this view
  float* rgb;           // W*H*3 (may be null)
  float* depth;         // W*H (may be null)
};

// Ray generation walks each view in 4x8-pixel tiles, one tile per warp, so
// the 32 rays a warp marches together cover a compact patch (better L1
// reuse of the hash-table gathers than a 32x1 row strip).
constexpr int kTileW = 4, kTileH = 8;

__host__ __device__ inline uint32_t view_threads(int W, int H) {
  return (uint32_t)((W + kTileW - 1) / kTileW) * (uint32_t)((H + kTileH - 1) / kTileH) * (kTileW * kTileH);
}

struct ViewBatch {
  int n;
  uint32_t total_pixels;  // ray-generation threads (tile-padded pixel count)
  DevView v[kMaxViews];
};

// Per-view frame output of a batch: the FP32 render (HWC RGB, depth) in, the
// YUV420P planes (caller linesizes) and uint16 millimetre depth out.
struct FrameOut {
  const float* rgb;
  const float* depth;
  uint8_t *y, *u, *v;
  uint16_t* depth_mm;  // may be null
  int w, h;
  int ls0, ls1, ls2;
  uint32_t first_block;  // first 2x2 pixel block of this view in the batch
};

struct FrameBatch {
  int n;
  uint32_t total_blocks;  // sum over views of ceil(w/2) * ceil(h/2)
  FrameOut f[kMaxViews];
};

// Where a kernel finds its batch descriptor: in its own parameters (one
// launch per batch), or in device memory, so that one instantiated CUDA
// graph serves every batch -- the host rewrites the descriptor before each
// replay and the graph's nodes never change.
template <class T>
struct InParam {
  T d;
  __device__ __forceinline__ const T& get() const { return d; }
};
template <class T>
struct InMemory {
  const T* p;
  __device__ __forceinline__ const T& get() const { return *p; }
};

// Compacted ray record: direction + start distance, and (view, pixel, n).
struct RayMeta {
  int view;
  int pixel;
  int n;
  int pad;
};

// Ray set-up in FP32 with explicit round-to-nearest operations (no FMA
// contraction) so the integer sample count matches the CPU restatement bit
// for bit.  Returns the number of samples (0: the ray misses the unit cube).
__device__ __forceinline__ int ray_setup(const float* M, int W, int H, float focal, int px, int py,
                                         float3& o, float3& d, float& t_start) {
  const float u = __fdiv_rn(__fsub_rn(__fadd_rn((float)px, 0.5f), __fmul_rn(0.5f, (float)W)), focal);
  const float v = __fdiv_rn(__fsub_rn(__fadd_rn((float)py, 0.5f), __fmul_rn(0.5f, (float)H)), focal);
  float dv[3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
    dv[a] = __fadd_rn(__fadd_rn(__fmul_rn(M[a * 4 + 0], u), __fmul_rn(M[a * 4 + 1], v)), M[a * 4 + 2]);
  const float n2 = __fadd_rn(__fadd_rn(__fmul_rn(dv[0], dv[0]), __fmul_rn(dv[1], dv[1])),
                             __fmul_rn(dv[2], dv[2]));
  const float nrm = __fsqrt_rn(n2);
  const float dd[3] = {__fdiv_rn(dv[0], nrm), __fdiv_rn(dv[1], nrm), __fdiv_rn(dv[2], nrm)};
  const float oo[3] = {M[3], M[7], M[11]};
  float tn = -INFINITY, tf = INFINITY;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float inv = __fdiv_rn(1.0f, dd[a]);
    const float t0 = __fmul_rn(__fsub_rn(0.0f, oo[a]), inv);
    const float t1 = __fmul_rn(__fsub_rn(1.0f, oo[a]), inv);
    tn = fmaxf(tn, fminf(t0, t1));
    tf = fminf(tf, fmaxf(t0, t1));
  }
  o = make_float3(oo[0], oo[1], oo[2]);
  d = make_float3(dd[0], dd[1], dd[2]);
  const float ts = fmaxf(tn, 0.0f);
  t_start = ts;
  if (!(tf > ts)) return 0;
  const float q = __fdiv_rn(__fsub_rn(tf, ts), kDt);
  const float fl = floorf(q);
  return fl >= (float)kMaxSteps ? kMaxSteps : (int)fl;
}

__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// Sample position t_i = t_start + (i + 1/2) dt, clamped to the unit cube.
__device__ __forceinline__ float3 sample_pos(const float3& o, const float3& d, float t) {
  return make_float3(clamp01(fmaf(t, d.x, o.x)), clamp01(fmaf(t, d.y, o.y)), clamp01(fmaf(t, d.z, o.z)));
}

__device__ __forceinline__ bool occupied(const uint32_t* __restrict__ occ, const float3& x) {
  const int cx = min(max((int)floorf(x.x * kOccRes), 0), kOccRes - 1);
  const int cy = min(max((int)floorf(x.y * kOccRes), 0), kOccRes - 1);
  const int cz = min(max((int)floorf(x.z * kOccRes), 0), kOccRes - 1);
  const uint32_t i = (uint32_t)cx + kOccRes * ((uint32_t)cy + kOccRes * (uint32_t)cz);
  return (__ldg(occ + (i >> 5)) >> (i & 31)) & 1u;
}

// Per-level cell and trilinear fractions: i0 = clamp(floor(x*N), 0, N-1).
struct LevelCell {
  uint32_t ix, iy, iz;
  float fx, fy, fz;
};

__device__ __forceinline__ LevelCell level_cell(const float3& x, int N) {
  const float fN = (float)N;
  const float px = x.x * fN, py = x.y * fN, pz = x.z * fN;
  const float lx = fminf(fmaxf(floorf(px), 0.0f), fN - 1.0f);
  const float ly = fminf(fmaxf(floorf(py), 0.0f), fN - 1.0f);
  const float lz = fminf(fmaxf(floorf(pz), 0.0f), fN - 1.0f);
  LevelCell c;
  c.ix = (uint32_t)lx;
  c.iy = (uint32_t)ly;
  c.iz = (uint32_t)lz;
  c.fx = px - lx;
  c.fy = py - ly;
  c.fz = pz - lz;
  return c;
}

// Table indices of the 8 corners (corner c = dx | dy<<1 | dz<<2).
__device__ __forceinline__ void corner_indices(const LevelCell& c, int N, bool dense, uint32_t T,
                                               uint32_t idx[8]) {
  if (dense) {
    const uint32_t s = (uint32_t)N + 1u;
    const uint32_t base = c.ix + s * (c.iy + s * c.iz);
#pragma unroll
    for (int k = 0; k < 8; ++k)
      idx[k] = base + (k & 1) + ((k >> 1) & 1) * s + ((k >> 2) & 1) * s * s;
  } else {
    const uint32_t m = T - 1u;
    const uint32_t hy0 = c.iy * kPrime1, hy1 = hy0 + kPrime1;
    const uint32_t hz0 = c.iz * kPrime2, hz1 = hz0 + kPrime2;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      idx[k] = ((c.ix + (k & 1)) ^ ((k & 2) ? hy1 : hy0) ^ ((k & 4) ? hz1 : hz0)) & m;
  }
}

__device__ __forceinline__ void corner_weights(const LevelCell& c, float w[8]) {
  const float gx = 1.0f - c.fx, gy = 1.0f - c.fy, gz = 1.0f - c.fz;
  const float xy0 = gx * gy, xy1 = c.fx * gy, xy2 = gx * c.fy, xy3 = c.fx * c.fy;
  w[0] = xy0 * gz;
  w[1] = xy1 * gz;
  w[2] = xy2 * gz;
  w[3] = xy3 * gz;
  w[4] = xy0 * c.fz;
  w[5] = xy1 * c.fz;
  w[6] = xy2 * c.fz;
  w[7] = xy3 * c.fz;
}

// Level l of the FP32 table (level-major float2 entries) at x -> its two
// features.
__device__ __forceinline__ void encode_level_fp32(const float2* __restrict__ table, uint32_t T, uint32_t dense_mask,
                                                  const float3& x, int l, float& f0, float& f1) {
  const int N = level_res(l);
  const LevelCell c = level_cell(x, N);
  uint32_t idx[8];
  corner_indices(c, N, (dense_mask >> l) & 1u, T, idx);
  float w[8];
  corner_weights(c, w);
  const float2* tab = table + (size_t)l * T;
  float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float2 e = __ldg(tab + idx[k]);
    a0 = fmaf(w[k], e.x, a0);
    a1 = fmaf(w[k], e.y, a1);
  }
  f0 = a0;
  f1 = a1;
}

// All levels of the FP32 table at x.
__device__ __forceinline__ void encode_fp32(const float2* __restrict__ table, uint32_t T,
                                            uint32_t dense_mask, const float3& x, float feat[kEnc]) {
#pragma unroll
  for (int l = 0; l < kLevels; ++l) encode_level_fp32(table, T, dense_mask, x, l, feat[2 * l], feat[2 * l + 1]);
}

// Real spherical harmonics, bands 0..3, orthonormal on the sphere.
__device__ __forceinline__ void sh16(const float3& d, float sh[16]) {
  const float PI = 3.14159265358979323846f;
  const float x = d.x, y = d.y, z = d.z;
  const float c0 = 0.5f * sqrtf(1.0f / PI), c1 = sqrtf(3.0f / (4.0f * PI));
  const float c2a = 0.5f * sqrtf(15.0f / PI), c2b = 0.25f * sqrtf(5.0f / PI), c2c = 0.25f * sqrtf(15.0f / PI);
  const float c3a = 0.25f * sqrtf(35.0f / (2.0f * PI)), c3b = 0.5f * sqrtf(105.0f / PI);
  const float c3c = 0.25f * sqrtf(21.0f / (2.0f * PI)), c3d = 0.25f * sqrtf(7.0f / PI);
  const float c3e = 0.25f * sqrtf(105.0f / PI);
  sh[0] = c0;
  sh[1] = c1 * y;
  sh[2] = c1 * z;
  sh[3] = c1 * x;
  sh[4] = c2a * x * y;
  sh[5] = c2a * y * z;
  sh[6] = c2b * (3.0f * z * z - 1.0f);
  sh[7] = c2a * x * z;
  sh[8] = c2c * (x * x - y * y);
  sh[9] = c3a * y * (3.0f * x * x - y * y);
  sh[10] = c3b * x * y * z;
  sh[11] = c3c * y * (5.0f * z * z - 1.0f);
  sh[12] = c3d * z * (5.0f * z * z - 3.0f);
  sh[13] = c3c * x * (5.0f * z * z - 1.0f);
  sh[14] = c3e * z * (x * x - y * y);
  sh[15] = c3a * x * (x * x - 3.0f * y * y);
}

__device__ __forceinline__ float sigmoidf(float a) { return 1.0f / (1.0f + expf(-a)); }

// Warp-aggregated claim of `want` consecutive items from a global counter.
__device__ __forceinline__ uint32_t warp_claim(uint32_t* counter, uint32_t want) {
  uint32_t base = 0;
  if ((threadIdx.x & 31) == 0) base = atomicAdd(counter, want);
  return __shfl_sync(0xffffffffu, base, 0);
}

}  // namespace nes
