// march_tc.cu -- FP16 tensor-core march: the renderer's density and colour
// MLPs (the external instant-ngp-renderer neserver calls over TCP,
// src/server.cpp:161-194) evaluated with tcgen05 MMAs.
//
// Structure (one persistent CTA of 128 threads, up to 4 CTAs per SM):
//  - each thread owns one ray slot; per iteration every active slot
//    contributes its next occupied sample, so one iteration is one
//    128-sample tile (M = 128);
//  - the thread encodes its sample from the FP16 hash table (FP32
//    interpolation) and writes the 32 features as one FP16 row of the A tile
//    in shared memory (K-major canonical layout, no swizzle);
//  - one elected thread issues the five layers as tcgen05.mma kind::f16
//    (32->64, 64->16, 32->64, 64->64, 64->16 [3 used]) with FP32
//    accumulators in TMEM (128 columns per CTA); after each layer every
//    thread loads its own TMEM lane (= its sample), applies ReLU / exp /
//    sigmoid in FP32 and writes the next FP16 operand row;
//  - the weights (FP16, already in operand layout, 20 KiB) are staged once
//    per CTA with one bulk TMA copy;
//  - transmittance, compositing and depth stay in FP32 per thread.
// TMEM safety: 128 columns x at most 4 resident CTAs = 512 columns per SM;
// the dynamic shared-memory request (50 KiB) makes a fifth CTA impossible,
// so tcgen05.alloc never waits on a CTA that will not exit.
#include <cuda_fp16.h>

#include "kernels.h"
#include "tc_ptx.cuh"

namespace nes {

namespace {

constexpr int kTcThreads = 128;
constexpr uint32_t kTmemCols = 128;

// Weight image (bytes) in operand layout: [N][K] K-major, core matrices 8x16B.
constexpr int kWoffDW1 = 0;      // N=64, K=32
constexpr int kWoffDW2 = 4096;   // N=16, K=64
constexpr int kWoffCW1 = 6144;   // N=64, K=32
constexpr int kWoffCW2 = 10240;  // N=64, K=64
constexpr int kWoffCW3 = 18432;  // N=16 (rows 3..15 zero), K=64
constexpr int kWBytes = 20480;

// Shared-memory map (bytes from a 1024-aligned base).
constexpr int kOffW = 0;
constexpr int kOffA = kOffW + kWBytes;  // 128 x 32 FP16 = 8 KiB
constexpr int kOffH = kOffA + 8192;     // 128 x 64 FP16 = 16 KiB
constexpr int kOffBar = kOffH + 16384;  // two mbarriers
constexpr int kOffSlot = kOffBar + 16;  // TMEM address
constexpr int kSmemUsed = kOffSlot + 16;
constexpr int kSmemRequest = 50 * 1024 + 1024;  // 5 x (this + 1 KiB reserved) > 228 KiB per SM
static_assert(kSmemUsed + 1024 <= kSmemRequest, "shared memory map exceeds the request");
static_assert(5 * (kSmemRequest + 1024) > 228 * 1024, "a fifth CTA per SM would fit: TMEM oversubscribed");

// Byte offset of 16-byte chunk c (K elements 8c..8c+7) of row m in a
// K-major operand with K columns: core matrices 8 rows x 16 B, K-chunks
// adjacent (LBO = 128 B), 8-row groups K*16 B apart (SBO).
__host__ __device__ constexpr int op_chunk(int m, int c, int K) { return (m >> 3) * (K * 16) + c * 128 + (m & 7) * 16; }

__device__ __forceinline__ uint32_t h2u(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }

__device__ __forceinline__ void store_row_chunks(uint8_t* tile, int row, int K, int c0, const uint32_t* w, int nchunks) {
#pragma unroll
  for (int q = 0; q < nchunks; ++q)
    *reinterpret_cast<uint4*>(tile + op_chunk(row, c0 + q, K)) = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
}

// 32 FP32 TMEM columns -> ReLU -> FP16 -> 4 chunks of an H row (K = 64).
__device__ __forceinline__ void relu_to_h(uint32_t taddr, uint8_t* H, int row, int c0) {
  float v[32];
  tc::tmem_ld32(taddr, v);
  uint32_t w[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) w[k] = h2u(__floats2half2_rn(fmaxf(v[2 * k], 0.0f), fmaxf(v[2 * k + 1], 0.0f)));
  store_row_chunks(H, row, 64, c0, w, 4);
}

// FP16 table, FP32 interpolation.
__device__ __forceinline__ void encode_fp16(const __half2* __restrict__ table, uint32_t T, uint32_t dense_mask,
                                            const float3& x, float feat[kEnc]) {
#pragma unroll
  for (int l = 0; l < kLevels; ++l) {
    const int N = level_res(l);
    const LevelCell c = level_cell(x, N);
    uint32_t idx[8];
    corner_indices(c, N, (dense_mask >> l) & 1u, T, idx);
    float w[8];
    corner_weights(c, w);
    const __half2* tab = table + (size_t)l * T;
    float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const float2 e = __half22float2(__ldg(tab + idx[k]));
      a0 = fmaf(w[k], e.x, a0);
      a1 = fmaf(w[k], e.y, a1);
    }
    feat[2 * l] = a0;
    feat[2 * l + 1] = a1;
  }
}

// Issues one layer: D[128 x N] = A[128 x K] * B[N x K]^T, K in steps of 16.
__device__ __forceinline__ void mma_layer(uint32_t d_tmem, uint32_t a, int a_K, uint32_t b, int b_K, int K,
                                          uint32_t idesc) {
  for (int j = 0; j < K / 16; ++j)
    tc::mma_f16(d_tmem, tc::sdesc(a + j * 256, 128, a_K * 16), tc::sdesc(b + j * 256, 128, b_K * 16), idesc,
                j > 0 ? 1u : 0u);
}

struct RaySlot {
  bool active = false;
  int view = 0, pixel = 0, n = 0, i = 0;
  float3 o, d;
  float ts = 0.0f, T = 1.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f, dep = 0.0f;
  uint32_t sh[8];  // SH16(d) as FP16 pairs
};

__device__ __forceinline__ void write_ray(const ViewBatch& vb, const RaySlot& r) {
  const DevView& V = vb.v[r.view];
  if (V.rgb) {
    V.rgb[(size_t)r.pixel * 3 + 0] = r.cr;
    V.rgb[(size_t)r.pixel * 3 + 1] = r.cg;
    V.rgb[(size_t)r.pixel * 3 + 2] = r.cb;
  }
  if (V.depth) V.depth[r.pixel] = r.dep;
}

// Advances r.i to the next occupied sample (or r.n).
__device__ __forceinline__ void skip_empty(const DevScene& sc, RaySlot& r) {
  while (r.i < r.n && !occupied(sc.occ, sample_pos(r.o, r.d, fmaf((float)r.i + 0.5f, kDt, r.ts)))) ++r.i;
}

__device__ __forceinline__ void start_ray(const ViewBatch& vb, const DevScene& sc, const DevScratch& s, uint32_t id,
                                          RaySlot& r) {
  const float4 rd = s.ray_dt[id];
  const RayMeta m = s.ray_meta[id];
  r.view = m.view;
  r.pixel = m.pixel;
  r.n = m.n;
  r.i = 0;
  r.ts = rd.w;
  r.d = make_float3(rd.x, rd.y, rd.z);
  const DevView& V = vb.v[m.view];
  r.o = make_float3(V.M[3], V.M[7], V.M[11]);
  r.T = 1.0f;
  r.cr = r.cg = r.cb = r.dep = 0.0f;
  float sh[16];
  sh16(r.d, sh);
#pragma unroll
  for (int k = 0; k < 8; ++k) r.sh[k] = h2u(__floats2half2_rn(sh[2 * k], sh[2 * k + 1]));
  skip_empty(sc, r);
  r.active = r.i < r.n;
  if (!r.active) write_ray(vb, r);
}

__global__ void __launch_bounds__(kTcThreads, 4)
march_tc_kernel(const ViewBatch vb, const DevScene sc, const DevScratch s) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  // Align the working base to 1024 B (the request leaves room for it).
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint64_t* bar_w = reinterpret_cast<uint64_t*>(smem + kOffBar);
  uint64_t* bar_mma = bar_w + 1;
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + kOffSlot);
  uint8_t* A = smem + kOffA;
  uint8_t* Hs = smem + kOffH;

  if (tid == 0) {
    tc::mbar_init(bar_w, 1);
    tc::mbar_init(bar_mma, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(slot, kTmemCols);
    tc::tmem_relinquish();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *slot;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(bar_w, kWBytes);
    tc::bulk_g2s(smem + kOffW, sc.tc_weights, kWBytes, bar_w);
  }
  bool fail = !tc::mbar_wait(bar_w, 0);
  uint32_t phase = 0;

  const uint32_t sW = tc::smem_addr(smem + kOffW), sA = tc::smem_addr(A), sH = tc::smem_addr(Hs);
  const uint32_t t_row = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's TMEM lane quarter
  constexpr uint32_t id64 = tc::idesc_f16_f32(128, 64), id16 = tc::idesc_f16_f32(128, 16);
  const uint32_t nrays = min(s.counters[kCtrRays], s.max_rays);

  RaySlot r;
  uint32_t chunk_next = 0, chunk_end = 0;
  bool exhausted = false;
  unsigned long long my_samples = 0;

  for (;;) {
    // Refill idle slots from a per-warp chunk of 32 ray ids (one atomic per
    // 32 rays).  Warp-uniform loop.
    for (;;) {
      const unsigned need = __ballot_sync(0xffffffffu, !r.active);
      if (need == 0 || exhausted) break;
      const uint32_t avail = chunk_end - chunk_next;
      const uint32_t rank = (uint32_t)__popc(need & ((1u << lane) - 1u));
      if (!r.active && rank < avail) start_ray(vb, sc, s, chunk_next + rank, r);
      const uint32_t cnt = (uint32_t)__popc(need);
      if (cnt <= avail) {
        chunk_next += cnt;
      } else {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(s.counters + kCtrCursor, 32u);
        b = __shfl_sync(0xffffffffu, b, 0);
        if (b >= nrays) {
          exhausted = true;
        } else {
          chunk_next = b;
          chunk_end = min(b + 32u, nrays);
        }
      }
    }
    const bool has = r.active;
    if (!__syncthreads_or(has)) break;  // every slot idle and every warp's queue empty

    // ---- encode this slot's sample into row `tid` of A (K = 32) ----
    float t = 0.0f;
    {
      uint32_t w[16];
      if (has) {
        t = fmaf((float)r.i + 0.5f, kDt, r.ts);
        float feat[kEnc];
        encode_fp16(sc.table16, sc.T, sc.dense_mask, sample_pos(r.o, r.d, t), feat);
#pragma unroll
        for (int k = 0; k < 16; ++k) w[k] = h2u(__floats2half2_rn(feat[2 * k], feat[2 * k + 1]));
      } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) w[k] = 0u;
      }
      store_row_chunks(A, tid, 32, 0, w, 4);
    }

    // ---- layer 1: density 32 -> 64, D at TMEM columns 0..63 ----
    tc::fence_async_smem();
    tc::fence_before();
    if (__syncthreads_or(fail)) break;
    if (tid == 0) {
      tc::fence_after();
      mma_layer(tmem + 0, sA, 32, sW + kWoffDW1, 32, 32, id64);
      tc::mma_commit(bar_mma);
    }
    fail |= !tc::mbar_wait(bar_mma, phase);
    phase ^= 1u;
    tc::fence_after();
    relu_to_h(t_row + 0, Hs, tid, 0);
    relu_to_h(t_row + 32, Hs, tid, 4);

    // ---- layer 2: density 64 -> 16, D at columns 64..79 ----
    tc::fence_async_smem();
    tc::fence_before();
    if (__syncthreads_or(fail)) break;
    if (tid == 0) {
      tc::fence_after();
      mma_layer(tmem + 64, sH, 64, sW + kWoffDW2, 64, 64, id16);
      tc::mma_commit(bar_mma);
    }
    fail |= !tc::mbar_wait(bar_mma, phase);
    phase ^= 1u;
    tc::fence_after();
    float sigma;
    {
      float v[16];
      tc::tmem_ld16(t_row + 64, v);
      sigma = expf(v[0] - 1.0f);
      uint32_t w[16];
#pragma unroll
      for (int k = 0; k < 8; ++k) w[k] = r.sh[k];
#pragma unroll
      for (int k = 0; k < 7; ++k) w[8 + k] = h2u(__floats2half2_rn(v[1 + 2 * k], v[2 + 2 * k]));
      w[15] = h2u(__floats2half2_rn(v[15], 0.0f));
      store_row_chunks(A, tid, 32, 0, w, 4);
    }

    // ---- layer 3: colour 32 -> 64, D at columns 0..63 ----
    tc::fence_async_smem();
    tc::fence_before();
    if (__syncthreads_or(fail)) break;
    if (tid == 0) {
      tc::fence_after();
      mma_layer(tmem + 0, sA, 32, sW + kWoffCW1, 32, 32, id64);
      tc::mma_commit(bar_mma);
    }
    fail |= !tc::mbar_wait(bar_mma, phase);
    phase ^= 1u;
    tc::fence_after();
    relu_to_h(t_row + 0, Hs, tid, 0);
    relu_to_h(t_row + 32, Hs, tid, 4);

    // ---- layer 4: colour 64 -> 64, D at columns 64..127 ----
    tc::fence_async_smem();
    tc::fence_before();
    if (__syncthreads_or(fail)) break;
    if (tid == 0) {
      tc::fence_after();
      mma_layer(tmem + 64, sH, 64, sW + kWoffCW2, 64, 64, id64);
      tc::mma_commit(bar_mma);
    }
    fail |= !tc::mbar_wait(bar_mma, phase);
    phase ^= 1u;
    tc::fence_after();
    relu_to_h(t_row + 64, Hs, tid, 0);
    relu_to_h(t_row + 96, Hs, tid, 4);

    // ---- layer 5: colour 64 -> 3 (N = 16), D at columns 0..15 ----
    tc::fence_async_smem();
    tc::fence_before();
    if (__syncthreads_or(fail)) break;
    if (tid == 0) {
      tc::fence_after();
      mma_layer(tmem + 0, sH, 64, sW + kWoffCW3, 64, 64, id16);
      tc::mma_commit(bar_mma);
    }
    fail |= !tc::mbar_wait(bar_mma, phase);
    phase ^= 1u;
    tc::fence_after();
    float v5[16];
    tc::tmem_ld16(t_row + 0, v5);
    tc::fence_before();

    // ---- composite in FP32 ----
    if (has) {
      ++my_samples;
      const float alpha = -expm1f(-sigma * kDt);
      const float wgt = r.T * alpha;
      r.cr = fmaf(wgt, sigmoidf(v5[0]), r.cr);
      r.cg = fmaf(wgt, sigmoidf(v5[1]), r.cg);
      r.cb = fmaf(wgt, sigmoidf(v5[2]), r.cb);
      r.dep = fmaf(wgt, t, r.dep);
      r.T -= wgt;
      ++r.i;
      if (r.T >= kTStop) skip_empty(sc, r);
      if (r.T < kTStop || r.i >= r.n) {
        write_ray(vb, r);
        r.active = false;
      }
    }
  }

  // Teardown: on a failed wait give an outstanding MMA one more bounded wait
  // before the columns are released; then free TMEM and report.
  if (fail && tid == 0) {
    tc::mbar_wait(bar_mma, phase);
    atomicExch(s.counters + kCtrError, 1u);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, kTmemCols);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) my_samples += __shfl_down_sync(0xffffffffu, my_samples, off);
  if (lane == 0 && my_samples)
    atomicAdd(reinterpret_cast<unsigned long long*>(s.counters + kCtrSamples), my_samples);
}

// FP32 weight blob -> FP16 operand image (see the kWoff* map).
__global__ void pack_tc_weights_kernel(const float* __restrict__ w, uint8_t* __restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;  // FP16 element of the image
  if (e >= kWBytes / 2) return;
  int base, K, local, src_off, src_rows;
  if (e < 2048) {
    base = kWoffDW1; K = 32; local = e; src_off = kOffDW1; src_rows = 64;
  } else if (e < 3072) {
    base = kWoffDW2; K = 64; local = e - 2048; src_off = kOffDW2; src_rows = 16;
  } else if (e < 5120) {
    base = kWoffCW1; K = 32; local = e - 3072; src_off = kOffCW1; src_rows = 64;
  } else if (e < 9216) {
    base = kWoffCW2; K = 64; local = e - 5120; src_off = kOffCW2; src_rows = 64;
  } else {
    base = kWoffCW3; K = 64; local = e - 9216; src_off = kOffCW3; src_rows = 3;
  }
  const int n = local / K, k = local % K;
  const float v = n < src_rows ? w[src_off + n * K + k] : 0.0f;
  *reinterpret_cast<__half*>(out + base + op_chunk(n, k >> 3, K) + (k & 7) * 2) = __float2half_rn(v);
}

}  // namespace

size_t tc_weight_bytes() { return kWBytes; }

cudaError_t launch_pack_tc_weights(const float* w32, uint8_t* out, cudaStream_t stream) {
  pack_tc_weights_kernel<<<(kWBytes / 2 + 255) / 256, 256, 0, stream>>>(w32, out);
  return cudaGetLastError();
}

cudaError_t launch_march_tc(const ViewBatch& views, const DevScene& scene, const DevScratch& s, int num_sms,
                            cudaStream_t stream) {
  if (!scene.table16 || !scene.tc_weights) return cudaErrorInvalidValue;
  static bool attr_set = false;  // idempotent; a race only repeats the call
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(march_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemRequest);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_tc_kernel, kTcThreads, kSmemRequest);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if (per_sm > 4) per_sm = 4;
  march_tc_kernel<<<num_sms * per_sm, kTcThreads, kSmemRequest, stream>>>(views, scene, s);
  return cudaGetLastError();
}

}  // namespace nes
