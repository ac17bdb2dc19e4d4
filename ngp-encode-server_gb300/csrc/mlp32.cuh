// mlp32.cuh -- FP32 density and colour MLPs evaluated per thread with the
// weights broadcast from shared memory (the plain CUDA-core path, the
// occupancy build and the training kernels).
#pragma once
#include "render_common.cuh"

namespace nes {

// FP32 weights in shared memory, laid out for broadcast float4 reads.
struct SmemWeights32 {
  float dw1[kHid * kEnc];    // [j][k]
  float dw2t[kHid * kDOut];  // [j][m] (transposed)
  float cw1[kHid * kCIn];    // [j][k]
  float cw2[kHid * kHid];    // [j][k]
  float cw3t[kHid * 4];      // [j][c], c = 3 padded
};

__device__ inline void load_weights32(SmemWeights32& W, const float* __restrict__ g) {
  for (int i = threadIdx.x; i < kHid * kEnc; i += blockDim.x) W.dw1[i] = g[kOffDW1 + i];
  for (int i = threadIdx.x; i < kHid * kDOut; i += blockDim.x) {
    const int j = i / kDOut, m = i % kDOut;
    W.dw2t[i] = g[kOffDW2 + m * kHid + j];
  }
  for (int i = threadIdx.x; i < kHid * kCIn; i += blockDim.x) W.cw1[i] = g[kOffCW1 + i];
  for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) W.cw2[i] = g[kOffCW2 + i];
  for (int i = threadIdx.x; i < kHid * 4; i += blockDim.x) {
    const int j = i / 4, c = i % 4;
    W.cw3t[i] = c < 3 ? g[kOffCW3 + c * kHid + j] : 0.0f;
  }
}

__device__ __forceinline__ float dot32(const float* __restrict__ w, const float in[32]) {
  const float4* w4 = reinterpret_cast<const float4*>(w);
  float a = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float4 q = w4[k];
    a = fmaf(q.x, in[4 * k + 0], a);
    a = fmaf(q.y, in[4 * k + 1], a);
    a = fmaf(q.z, in[4 * k + 2], a);
    a = fmaf(q.w, in[4 * k + 3], a);
  }
  return a;
}

// Density MLP 32->64->16 (ReLU hidden), FP32.
__device__ __forceinline__ void density_mlp32(const SmemWeights32& W, const float enc[32], float out[16]) {
#pragma unroll
  for (int m = 0; m < kDOut; ++m) out[m] = 0.0f;
#pragma unroll 4
  for (int j = 0; j < kHid; ++j) {
    const float a = fmaxf(dot32(W.dw1 + j * kEnc, enc), 0.0f);
    const float4* w2 = reinterpret_cast<const float4*>(W.dw2t + j * kDOut);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float4 q = w2[k];
      out[4 * k + 0] = fmaf(q.x, a, out[4 * k + 0]);
      out[4 * k + 1] = fmaf(q.y, a, out[4 * k + 1]);
      out[4 * k + 2] = fmaf(q.z, a, out[4 * k + 2]);
      out[4 * k + 3] = fmaf(q.w, a, out[4 * k + 3]);
    }
  }
}

// Colour MLP [SH16 | out[1..15] | 0] 32->64->64->3, FP32.
__device__ __forceinline__ float3 colour_mlp32(const SmemWeights32& W, const float sh[16],
                                               const float dout[16]) {
  float cin[32];
#pragma unroll
  for (int k = 0; k < 16; ++k) cin[k] = sh[k];
#pragma unroll
  for (int k = 0; k < 15; ++k) cin[16 + k] = dout[1 + k];
  cin[31] = 0.0f;
  float g1[kHid];
#pragma unroll
  for (int j = 0; j < kHid; ++j) g1[j] = fmaxf(dot32(W.cw1 + j * kCIn, cin), 0.0f);
  float r = 0.0f, g = 0.0f, b = 0.0f;
#pragma unroll 2
  for (int j = 0; j < kHid; ++j) {
    const float4* w4 = reinterpret_cast<const float4*>(W.cw2 + j * kHid);
    float a = 0.0f;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const float4 q = w4[k];
      a = fmaf(q.x, g1[4 * k + 0], a);
      a = fmaf(q.y, g1[4 * k + 1], a);
      a = fmaf(q.z, g1[4 * k + 2], a);
      a = fmaf(q.w, g1[4 * k + 3], a);
    }
    a = fmaxf(a, 0.0f);
    const float4 c3 = *reinterpret_cast<const float4*>(W.cw3t + j * 4);
    r = fmaf(c3.x, a, r);
    g = fmaf(c3.y, a, g);
    b = fmaf(c3.z, a, b);
  }
  return make_float3(sigmoidf(r), sigmoidf(g), sigmoidf(b));
}

}  // namespace nes
