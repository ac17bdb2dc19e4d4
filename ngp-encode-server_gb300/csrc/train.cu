// train.cu -- differentiation of the renderer and the Adam refit
// (nes_trainer_* in include/nes_gb300.h).  neserver itself only renders;
// this is the training form of the same field (refit configuration: teacher
// scene seed 1, student seed 2, 2^18 rays per step, L2 on RGB + 0.1 L2 on
// depth, Adam lr 1e-2, betas (0.9, 0.99), eps 1e-15).
//
// Per step:
//  1. rays: (view, pixel) pairs (drawn from the step seed or given) -> the
//     FP32 ray set-up of rendering, with the target colour and depth;
//  2. forward: the rays' occupied steps listed (thread per ray), the field
//     evaluated at every listed sample (by default the MLP products on the
//     tensor cores as 3xTF32, FP32-level; exact_weight_grads = 1: FP32 on the
//     CUDA cores), then each ray composited with early termination (thread
//     per ray), keeping each
//     evaluated sample's t, alpha, transmittance and colour in the ray's
//     scratch row; loss; then walk the samples backwards carrying
//     A = dL/dT_k for each one's compositing adjoint
//        g_w = g_C . c_k + g_D t_k,   dL/dc_k = g_C w_k,
//        dL/dsigma_k = dt T_{k+1} (g_w - A_{k+1}),
//        A_k = g_w alpha_k + A_{k+1} (1 - alpha_k),   A_K = 0,
//     with g_C = 2 (C - C*)/B and g_D = 2 lambda (D - D*)/B, written as a
//     compact 32-byte record (position, ray, dsigma, dc).  The backward
//     sweep keeps every term proportional to T_{k+1}; the equivalent
//     forward form with suffix sums (C - prefix) cancels in FP32 late in
//     the ray;
//  3. backward (thread per record, in chunks): recompute the encoding and
//     both MLPs, backpropagate, scatter-add the encoding gradient into the
//     FP32 gradient table with float2 atomics, and stage every layer's input
//     activations and output deltas.  By default the ten layer products of
//     the recompute and the backpropagation run on the tensor cores
//     (backward_tc_kernel, tcgen05 kind::tf32) and the staging is BF16;
//     exact_weight_grads = 1 keeps them in FP32 on the CUDA cores
//     (backward_kernel) with FP32 staging;
//  4. weight gradients: per layer dW[out][in] += sum_s delta[s][out] act[s][in]
//     over the chunk (by default dw_tc_kernel, tcgen05 kind::f16 with BF16
//     operands; exact: dw_kernel, register-tiled split-K reduction);
//  5. Adam on the table and the weights (bias-corrected); gradients zeroed.
// An FP64 variant of the loss evaluates the same function with one parameter
// perturbed, for central finite differences.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "ctx_internal.h"
#include "kernels.h"
#include "mlp32.cuh"
#include "nes_gb300.h"
#include "tc_ptx.cuh"

using namespace nes;

namespace {

struct TrainView {
  float M[12];
  int W, H;
  float focal;
  int pad;
  uint64_t offset;  // first pixel of this view in the concatenated targets
};

struct TrainRay {
  float ox, oy, oz, ts;
  float dx, dy, dz;
  int n;                 // march steps (0: the ray misses the cube)
  float tr, tg, tb, td;  // target colour and depth
};

struct ScratchSample {  // pass-1 state of one evaluated sample
  float t, alpha, T, cr, cg, cb, pad0, pad1;  // T: transmittance before the sample
};

struct SampleRec {  // compacted sample with its compositing adjoint
  float x, y, z;
  uint32_t ray;
  float dsigma, dcr, dcg, dcb;
};

// Per-sample staging of the weight-gradient reductions, in 32-sample
// tiles (FP32 layout of the strict mode; the tensor-core mode stages BF16,
// see stage8).  Each tile of an F-wide array (F a multiple of 8) is one
// contiguous block of F x 32 floats in the canonical K-major layout of the
// tensor core's shared-memory operands, no swizzle, K = sample: 8-feature x
// 4-sample core matrices of 128 bytes, the 8 core matrices of a feature
// group along K at 128-byte steps, feature groups at 1,024-byte steps.
// Feature f of sample k of a tile sits at float
//   (f / 8) * 256 + (k / 4) * 32 + (f % 8) * 4 + k % 4,
// so one bulk copy per array and tile lands a ready MMA operand, and a
// thread's features sit at immediate offsets from one base.
constexpr int kStageFloats = kEnc + kHid + kCIn + kHid + kHid  // activations: enc, h1, cin, g1, g2
                             + kHid + kDOut + kHid + kHid + 8;  // deltas: dh1, dout, dg1, dg2, dlogit(3)+zeros
struct Staging {
  float *enc, *h1, *cin, *g1, *g2;       // F = 32, 64, 32, 64, 64
  float *dh1, *dout, *dg1, *dg2, *dlog;  // F = 64, 16, 64, 64, 8 (features 3..7 zero)
};
constexpr int kFDlog = 8;

__device__ __forceinline__ float* stage_row(float* a, int F, uint32_t s) {
  const uint32_t k = s & 31u;
  return a + (size_t)(s >> 5) * F * 32 + (k >> 2) * 32 + (k & 3);
}
__host__ __device__ constexpr int soff(int f) { return (f >> 3) * 256 + (f & 7) * 4; }

// FP32 forward evaluation: 128-thread blocks, three resident per SM at its 167 registers.
// Backward: 256-thread blocks capped at 128 registers, two resident per SM
// (16 warps) with one shared copy of the weights per block, which leaves
// L1 for the table gathers.
constexpr int kFwdThreads = 128;
constexpr int kBwdThreads = 256;
constexpr uint32_t kErrBadRay = 2u, kErrOverflow = 3u;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Draw i of the step: view = low word mod nviews, pixel = high word mod W*H.
__global__ void sample_pairs_kernel(uint64_t seed, int n, const TrainView* __restrict__ views, int nviews,
                                    int2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t u = mix64(mix64(seed * 256ull + 7ull) + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull);
  const int v = (int)((u & 0xffffffffull) % (uint64_t)nviews);
  const uint64_t px = (uint64_t)views[v].W * views[v].H;
  out[i] = make_int2(v, (int)((u >> 32) % px));
}

__global__ void make_rays_kernel(const int2* __restrict__ pairs, int n, const TrainView* __restrict__ views, int nviews,
                                 const float* __restrict__ trgb, const float* __restrict__ tdep,
                                 TrainRay* __restrict__ rays, uint32_t* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int2 p = pairs[i];
  TrainRay r{};
  if (p.x < 0 || p.x >= nviews || p.y < 0 || (uint64_t)p.y >= (uint64_t)views[p.x].W * views[p.x].H) {
    atomicExch(err, kErrBadRay);
    rays[i] = r;
    return;
  }
  const TrainView& V = views[p.x];
  float3 o, d;
  float ts;
  r.n = ray_setup(V.M, V.W, V.H, V.focal, p.y % V.W, p.y / V.W, o, d, ts);
  r.ox = o.x; r.oy = o.y; r.oz = o.z; r.ts = ts;
  r.dx = d.x; r.dy = d.y; r.dz = d.z;
  const uint64_t q = V.offset + (uint64_t)p.y;
  r.tr = trgb[q * 3 + 0];
  r.tg = trgb[q * 3 + 1];
  r.tb = trgb[q * 3 + 2];
  r.td = tdep[q];
  rays[i] = r;
}

struct RayOut {  // composited result of one training ray
  float C0, C1, C2, D;
  int K;           // evaluated samples up to early termination, in the ray's scratch row
  uint32_t first;  // the ray's occupied steps in the sample list: [first, first + count)
  uint32_t count;
  int pad;
};

// Forward, in three passes, so that the per-sample MLP runs with every lane
// of a warp busy (marched one ray per thread, the lanes whose ray is at an
// empty step would idle while the others evaluate) or on the tensor cores in
// 128-sample tiles:
//  1. enumerate_kernel, thread per ray: the ray's occupied steps in order --
//     the march's sample set before early termination -- listed contiguously
//     as (ray, k | step << 16), k the sample's index along the ray;
//  2. eval_kernel (FP32, thread per listed sample) or eval_tc_kernel (the
//     MLP products on tcgen05 as 3xTF32, thread = TMEM lane per sample): the
//     encoding and MLPs at that sample, its t, alpha and colour written to the
//     ray's scratch row k (a warp's samples are consecutive samples of one or
//     two rays: coherent gathers);
//  3. composite_kernel, thread per ray: the ray's rows in order, composited
//     and stopped at T < kTStop exactly as a one-pass march composites, with
//     each row's transmittance and the ray's RayOut filled in.
// With eval_kernel the per-sample arithmetic is the one-pass FP32 march's;
// only the samples after an early termination are evaluated and then left
// unused.
constexpr uint32_t kListStepShift = 16;
static_assert(kMaxSteps <= (1 << kListStepShift), "k and step share one word");

__global__ void __launch_bounds__(256)
enumerate_kernel(const TrainRay* __restrict__ rays, int n, const DevScene sc, uint2* __restrict__ list,
                 uint32_t capacity, RayOut* __restrict__ rout, uint32_t* __restrict__ cursor,
                 uint32_t* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned lane = threadIdx.x & 31u;
  TrainRay r{};
  if (i < n) r = rays[i];
  const float3 o = make_float3(r.ox, r.oy, r.oz), d = make_float3(r.dx, r.dy, r.dz);
  int cnt = 0;
  for (int st = 0; st < r.n; ++st)
    if (occupied(sc.occ, sample_pos(o, d, fmaf((float)st + 0.5f, kDt, r.ts)))) ++cnt;
  int incl = cnt;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, off);
    if ((int)lane >= off) incl += v;
  }
  uint32_t base = 0;
  if (lane == 31 && incl > 0) base = atomicAdd(cursor, (uint32_t)incl);
  base = __shfl_sync(0xffffffffu, base, 31) + (uint32_t)(incl - cnt);
  if (i >= n) return;
  RayOut ro{};
  ro.first = base;
  if (cnt > 0 && (base > capacity || (uint32_t)cnt > capacity - base)) {
    atomicExch(err, kErrOverflow);
  } else if (cnt > 0) {
    ro.count = (uint32_t)cnt;
    uint32_t k = 0;
    for (int st = 0; st < r.n; ++st)
      if (occupied(sc.occ, sample_pos(o, d, fmaf((float)st + 0.5f, kDt, r.ts)))) {
        list[base + k] = make_uint2((uint32_t)i, k | ((uint32_t)st << kListStepShift));
        ++k;
      }
  }
  rout[i] = ro;
}

// Persistent grid-stride over the list; its length is the enumeration's
// cursor (read on the device: no host round trip between the passes).
__global__ void __launch_bounds__(kFwdThreads)
eval_kernel(const uint2* __restrict__ list, const uint32_t* __restrict__ total, uint32_t capacity,
            const TrainRay* __restrict__ rays, int n, const DevScene sc, ScratchSample* __restrict__ scratch) {
  extern __shared__ float4 smem_raw[];
  SmemWeights32& W = *reinterpret_cast<SmemWeights32*>(smem_raw);
  load_weights32(W, sc.weights);
  __syncthreads();
  const uint32_t m = min(*total, capacity);
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
    const uint2 e = list[j];
    const uint32_t k = e.y & ((1u << kListStepShift) - 1u), st = e.y >> kListStepShift;
    if (e.x >= (uint32_t)n || k >= (uint32_t)kMaxSteps) continue;  // only after an overflow (flagged)
    const TrainRay& r = rays[e.x];
    const float3 o = make_float3(r.ox, r.oy, r.oz), d = make_float3(r.dx, r.dy, r.dz);
    const float t = fmaf((float)st + 0.5f, kDt, r.ts);
    const float3 x = sample_pos(o, d, t);
    float enc[kEnc];
    encode_fp32(sc.table32, sc.T, sc.dense_mask, x, enc);
    float dout[kDOut];
    density_mlp32(W, enc, dout);
    const float sigma = expf(dout[0] - 1.0f);
    float sh[16];
    sh16(d, sh);
    const float3 c = colour_mlp32(W, sh, dout);
    const float alpha = -expm1f(-sigma * kDt);
    scratch[(size_t)e.x * kMaxSteps + k] = ScratchSample{t, alpha, 0.0f, c.x, c.y, c.z, 0.0f, 0.0f};
  }
}

__global__ void __launch_bounds__(256)
composite_kernel(int n, ScratchSample* __restrict__ scratch, RayOut* __restrict__ rout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  RayOut ro = rout[i];
  ScratchSample* row = scratch + (size_t)i * kMaxSteps;
  float T = 1.0f, C0 = 0.0f, C1 = 0.0f, C2 = 0.0f, D = 0.0f;
  int K = 0;
  bool stop = false;
  // Rows in batches of kBatch, all loaded before the first is used: the
  // stop test of one sample no longer holds back the next sample's load.
  constexpr uint32_t kBatch = 8;
  for (uint32_t k0 = 0; k0 < ro.count && !stop; k0 += kBatch) {
    ScratchSample q[kBatch];
#pragma unroll
    for (uint32_t u = 0; u < kBatch; ++u)
      if (k0 + u < ro.count) q[u] = row[k0 + u];
#pragma unroll
    for (uint32_t u = 0; u < kBatch; ++u) {
      if (stop || k0 + u >= ro.count) break;
      const float w = T * q[u].alpha;
      row[k0 + u].T = T;
      ++K;
      C0 = fmaf(w, q[u].cr, C0);
      C1 = fmaf(w, q[u].cg, C1);
      C2 = fmaf(w, q[u].cb, C2);
      D = fmaf(w, q[u].t, D);
      T -= w;
      stop = T < kTStop;
    }
  }
  ro.C0 = C0;
  ro.C1 = C1;
  ro.C2 = C2;
  ro.D = D;
  ro.K = K;
  rout[i] = ro;
}

// Loss and compositing adjoint, thread per ray: the ray's samples are walked
// backwards carrying A = dL/dT (see the file comment) and written as compact
// records; one record-range atomic per warp (warp prefix sum of K).
__global__ void __launch_bounds__(256)
adjoint_kernel(const TrainRay* __restrict__ rays, const RayOut* __restrict__ rout, int n,
               const ScratchSample* __restrict__ scratch, SampleRec* __restrict__ recs, uint32_t capacity,
               uint32_t* __restrict__ cursor, uint32_t* __restrict__ err, double* __restrict__ loss_sum,
               float depth_w, float inv_n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned lane = threadIdx.x & 31u;
  TrainRay r{};
  RayOut ro{};
  if (i < n) {
    r = rays[i];
    ro = rout[i];
  }
  const int K = i < n ? ro.K : 0;
  int incl = K;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, off);
    if ((int)lane >= off) incl += v;
  }
  uint32_t base = 0;
  if (lane == 31 && incl > 0) base = atomicAdd(cursor, (uint32_t)incl);
  base = __shfl_sync(0xffffffffu, base, 31) + (uint32_t)(incl - K);
  float my_loss = 0.0f;
  if (i < n) {
    const float ec0 = ro.C0 - r.tr, ec1 = ro.C1 - r.tg, ec2 = ro.C2 - r.tb, ed = ro.D - r.td;
    my_loss = (ec0 * ec0 + ec1 * ec1 + ec2 * ec2 + depth_w * ed * ed) * inv_n;
    if (K > 0 && base + (uint32_t)K > capacity) {
      atomicExch(err, kErrOverflow);
    } else if (K > 0) {
      const float gC0 = 2.0f * ec0 * inv_n, gC1 = 2.0f * ec1 * inv_n, gC2 = 2.0f * ec2 * inv_n;
      const float gD = 2.0f * depth_w * ed * inv_n;
      const float3 o = make_float3(r.ox, r.oy, r.oz), d = make_float3(r.dx, r.dy, r.dz);
      const ScratchSample* row = scratch + (size_t)i * kMaxSteps;
      float A = 0.0f;
      // Rows in batches of kBatch from the back, all loaded before the
      // first is used (the loads do not wait on the sweep's arithmetic).
      constexpr int kBatch = 8;
      for (int k1 = K - 1; k1 >= 0; k1 -= kBatch) {
        ScratchSample qb[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u)
          if (k1 - u >= 0) qb[u] = row[k1 - u];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
          const int k = k1 - u;
          if (k < 0) break;
          const ScratchSample& q = qb[u];
          const float w = q.T * q.alpha;
          const float T1 = q.T - w;
          const float gw = fmaf(gC0, q.cr, fmaf(gC1, q.cg, fmaf(gC2, q.cb, gD * q.t)));
          const float dsig = kDt * T1 * (gw - A);
          const float3 x = sample_pos(o, d, q.t);
          recs[base + k] = SampleRec{x.x, x.y, x.z, (uint32_t)i, dsig, gC0 * w, gC1 * w, gC2 * w};
          A = fmaf(gw, q.alpha, A * (1.0f - q.alpha));
        }
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) my_loss += __shfl_down_sync(0xffffffffu, my_loss, off);
  if (lane == 0 && my_loss != 0.0f) atomicAdd(loss_sum, (double)my_loss);
}

// Backward, thread per record of the chunk [first, first + count).
// Activations stay in registers (ReLU masks as 64-bit words); every staged
// value is written once, feature f of the sample at row[soff(f)].
__device__ __forceinline__ float dot64(const float* __restrict__ w, const float in[64]) {
  const float4* w4 = reinterpret_cast<const float4*>(w);
  float a = 0.0f;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const float4 q = w4[k];
    a = fmaf(q.x, in[4 * k + 0], a);
    a = fmaf(q.y, in[4 * k + 1], a);
    a = fmaf(q.z, in[4 * k + 2], a);
    a = fmaf(q.w, in[4 * k + 3], a);
  }
  return a;
}

// Shared memory of the backward: the FP32 weights plus colour W1's
// geometry-feature columns (16..30) transposed, for the dout pass.
struct SmemBackward {
  SmemWeights32 w;
  float cw1g[16 * kHid];  // [m][j] = cw1[j][16 + m], m < 15; row 15 zero
};

__global__ void __launch_bounds__(kBwdThreads, 2)
backward_kernel(const SampleRec* __restrict__ recs, uint32_t first, uint32_t count, const TrainRay* __restrict__ rays,
                const DevScene sc, Staging st, float2* __restrict__ gtable) {
  extern __shared__ float4 smem_raw[];
  SmemBackward& S = *reinterpret_cast<SmemBackward*>(smem_raw);
  SmemWeights32& W = S.w;
  load_weights32(W, sc.weights);
  for (int i = threadIdx.x; i < 16 * kHid; i += blockDim.x) {
    const int m = i / kHid, j = i % kHid;
    S.cw1g[i] = m < 15 ? sc.weights[kOffCW1 + j * kCIn + 16 + m] : 0.0f;
  }
  __syncthreads();
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ((count + 31u) & ~31u)) return;
  if (s >= count) {  // rows of the last tile past the chunk's samples: zeros for the reductions
    float* const arr[10] = {st.enc, st.h1, st.cin, st.g1, st.g2, st.dh1, st.dout, st.dg1, st.dg2, st.dlog};
    const int F[10] = {kEnc, kHid, kCIn, kHid, kHid, kHid, kDOut, kHid, kHid, 8};
    for (int a = 0; a < 10; ++a) {
      float* r = stage_row(arr[a], F[a], s);
      for (int f = 0; f < F[a]; ++f) r[soff(f)] = 0.0f;
    }
    return;
  }
  const SampleRec q = recs[first + s];
  const float3 x = make_float3(q.x, q.y, q.z);
  float* const r_enc = stage_row(st.enc, kEnc, s);
  float* const r_h1 = stage_row(st.h1, kHid, s);
  float* const r_cin = stage_row(st.cin, kCIn, s);
  float* const r_g1 = stage_row(st.g1, kHid, s);
  float* const r_g2 = stage_row(st.g2, kHid, s);
  float* const r_dh1 = stage_row(st.dh1, kHid, s);
  float* const r_dout = stage_row(st.dout, kDOut, s);
  float* const r_dg1 = stage_row(st.dg1, kHid, s);
  float* const r_dg2 = stage_row(st.dg2, kHid, s);
  float* const r_dlog = stage_row(st.dlog, 8, s);
  // ---- forward recompute ----
  float enc[kEnc];
  encode_fp32(sc.table32, sc.T, sc.dense_mask, x, enc);
#pragma unroll
  for (int k = 0; k < kEnc; ++k) r_enc[soff(k)] = enc[k];
  float out[kDOut];
#pragma unroll
  for (int m = 0; m < kDOut; ++m) out[m] = 0.0f;
  uint64_t m_h1 = 0;
#pragma unroll 1
  for (int j = 0; j < kHid; ++j) {
    const float a = fmaxf(dot32(W.dw1 + j * kEnc, enc), 0.0f);
    r_h1[soff(j)] = a;
    m_h1 |= (uint64_t)(a > 0.0f) << j;
    const float4* w2 = reinterpret_cast<const float4*>(W.dw2t + j * kDOut);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float4 w = w2[k];
      out[4 * k + 0] = fmaf(w.x, a, out[4 * k + 0]);
      out[4 * k + 1] = fmaf(w.y, a, out[4 * k + 1]);
      out[4 * k + 2] = fmaf(w.z, a, out[4 * k + 2]);
      out[4 * k + 3] = fmaf(w.w, a, out[4 * k + 3]);
    }
  }
  const float sigma = expf(out[0] - 1.0f);
  float cin[kCIn];
  {
    const TrainRay& r = rays[q.ray];
    sh16(make_float3(r.dx, r.dy, r.dz), cin);
  }
#pragma unroll
  for (int k = 0; k < 15; ++k) cin[16 + k] = out[1 + k];
  cin[31] = 0.0f;
#pragma unroll
  for (int k = 0; k < kCIn; ++k) r_cin[soff(k)] = cin[k];
  float g[kHid];  // g1, then its gradient
#pragma unroll
  for (int j = 0; j < kHid; ++j) {
    g[j] = fmaxf(dot32(W.cw1 + j * kCIn, cin), 0.0f);
    r_g1[soff(j)] = g[j];
  }
  uint64_t m_g1 = 0;
#pragma unroll
  for (int j = 0; j < kHid; ++j) m_g1 |= (uint64_t)(g[j] > 0.0f) << j;
  float lg0 = 0.0f, lg1 = 0.0f, lg2 = 0.0f;
  uint64_t m_g2 = 0;
#pragma unroll 1
  for (int j = 0; j < kHid; ++j) {
    const float a = fmaxf(dot64(W.cw2 + j * kHid, g), 0.0f);
    r_g2[soff(j)] = a;
    m_g2 |= (uint64_t)(a > 0.0f) << j;
    const float4 c3 = *reinterpret_cast<const float4*>(W.cw3t + j * 4);
    lg0 = fmaf(c3.x, a, lg0);
    lg1 = fmaf(c3.y, a, lg1);
    lg2 = fmaf(c3.z, a, lg2);
  }
  // ---- backward ----
  const float c0 = sigmoidf(lg0), c1 = sigmoidf(lg1), c2 = sigmoidf(lg2);
  const float dl0 = q.dcr * c0 * (1.0f - c0), dl1 = q.dcg * c1 * (1.0f - c1), dl2 = q.dcb * c2 * (1.0f - c2);
  r_dlog[soff(0)] = dl0;
  r_dlog[soff(1)] = dl1;
  r_dlog[soff(2)] = dl2;
#pragma unroll
  for (int f = 3; f < 8; ++f) r_dlog[soff(f)] = 0.0f;
#pragma unroll
  for (int k = 0; k < kHid; ++k) g[k] = 0.0f;
#pragma unroll 1
  for (int j = 0; j < kHid; ++j) {  // dg2_j, and dg1 += cw2[j][:] dg2_j
    const float4 c3 = *reinterpret_cast<const float4*>(W.cw3t + j * 4);
    const float d2 = ((m_g2 >> j) & 1) ? fmaf(c3.x, dl0, fmaf(c3.y, dl1, c3.z * dl2)) : 0.0f;
    r_dg2[soff(j)] = d2;
    const float4* w4 = reinterpret_cast<const float4*>(W.cw2 + j * kHid);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const float4 w = w4[k];
      g[4 * k + 0] = fmaf(w.x, d2, g[4 * k + 0]);
      g[4 * k + 1] = fmaf(w.y, d2, g[4 * k + 1]);
      g[4 * k + 2] = fmaf(w.z, d2, g[4 * k + 2]);
      g[4 * k + 3] = fmaf(w.w, d2, g[4 * k + 3]);
    }
  }
#pragma unroll
  for (int k = 0; k < kHid; ++k) {
    g[k] = ((m_g1 >> k) & 1) ? g[k] : 0.0f;
    r_dg1[soff(k)] = g[k];
  }
  float dout[kDOut];
  dout[0] = q.dsigma * sigma;
#pragma unroll
  for (int m = 0; m < 15; ++m) dout[1 + m] = dot64(S.cw1g + m * kHid, g);
#pragma unroll
  for (int m = 0; m < kDOut; ++m) r_dout[soff(m)] = dout[m];
  float denc[kEnc];
#pragma unroll
  for (int k = 0; k < kEnc; ++k) denc[k] = 0.0f;
#pragma unroll 1
  for (int j = 0; j < kHid; ++j) {  // dh1_j, and denc += dw1[j][:] dh1_j
    const float4* w2 = reinterpret_cast<const float4*>(W.dw2t + j * kDOut);
    float a = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float4 w = w2[k];
      a = fmaf(w.x, dout[4 * k + 0], a);
      a = fmaf(w.y, dout[4 * k + 1], a);
      a = fmaf(w.z, dout[4 * k + 2], a);
      a = fmaf(w.w, dout[4 * k + 3], a);
    }
    const float dh = ((m_h1 >> j) & 1) ? a : 0.0f;
    r_dh1[soff(j)] = dh;
    const float4* w1 = reinterpret_cast<const float4*>(W.dw1 + j * kEnc);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const float4 w = w1[k];
      denc[4 * k + 0] = fmaf(w.x, dh, denc[4 * k + 0]);
      denc[4 * k + 1] = fmaf(w.y, dh, denc[4 * k + 1]);
      denc[4 * k + 2] = fmaf(w.z, dh, denc[4 * k + 2]);
      denc[4 * k + 3] = fmaf(w.w, dh, denc[4 * k + 3]);
    }
  }
  // ---- hash-grid scatter-add: dtable[level][corner] += w_corner * denc[level] ----
#pragma unroll 1
  for (int l = 0; l < kLevels; ++l) {
    const int N = level_res(l);
    const LevelCell c = level_cell(x, N);
    uint32_t idx[8];
    corner_indices(c, N, (sc.dense_mask >> l) & 1u, sc.T, idx);
    float w[8];
    corner_weights(c, w);
    float2* gt = gtable + (size_t)l * sc.T;
    float d0 = 0.0f, d1 = 0.0f;
#pragma unroll
    for (int k = 0; k < kLevels; ++k)
      if (k == l) {
        d0 = denc[2 * k];
        d1 = denc[2 * k + 1];
      }
#pragma unroll
    for (int k = 0; k < 8; ++k) atomicAdd(gt + idx[k], make_float2(w[k] * d0, w[k] * d1));
  }
}

// dW[o][i] += sum_s delta[s][o] * act[s][i] over S samples of tiled staging
// (IN activation features, LDD-wide delta tiles of which OUT are real).  Every thread owns a 4x4 tile of dW; when the
// tiles number fewer than the block's threads, the thread groups split
// each 32-sample smem tile between them.  Each block reduces a contiguous
// range of samples and adds its partial dW with one atomic per element.
constexpr int kDwThreads = 256;
constexpr int kDwTile = 32;

template <int IN, int OUT, int LDD>
__global__ void __launch_bounds__(kDwThreads)
dw_kernel(const float* __restrict__ act, const float* __restrict__ delta, uint32_t S, float* __restrict__ dw) {
  static_assert(IN % 4 == 0 && LDD % 4 == 0 && OUT <= LDD, "tile shape");
  constexpr int TI = IN / 4, TO = LDD / 4, TILES = TI * TO;
  static_assert(TILES <= kDwThreads && kDwThreads % TILES == 0, "tile count");
  constexpr int G = kDwThreads / TILES;  // sample groups
  // Rows padded by 4 floats: the transposing stores (sample-fastest) hit 8
  // banks instead of 1, the float4 reads stay aligned.
  __shared__ __align__(16) float sa[kDwTile][IN + 4];
  __shared__ __align__(16) float sd[kDwTile][LDD + 4];
  const int tid = threadIdx.x;
  const int ti = tid % TI, to = (tid / TI) % TO, grp = tid / TILES;
  float acc[4][4] = {};
  const uint32_t per = ((S + gridDim.x - 1) / gridDim.x + kDwTile - 1) / kDwTile * kDwTile;
  const uint32_t lo = blockIdx.x * per, hi = min(S, lo + per);
  for (uint32_t base = lo; base < hi; base += kDwTile) {
    const uint32_t rows = min((uint32_t)kDwTile, hi - base);
    // The tile is one contiguous block: each float4 holds 4 samples of one
    // feature (core-matrix layout), stored transposed.
    const float4* ta = reinterpret_cast<const float4*>(act + (size_t)(base / kDwTile) * IN * kDwTile);
    const float4* td = reinterpret_cast<const float4*>(delta + (size_t)(base / kDwTile) * LDD * kDwTile);
    for (int e = tid; e < kDwTile * IN / 4; e += kDwThreads) {
      const int f = (e >> 6) * 8 + (e & 7), r = ((e >> 3) & 7) * 4;
      const float4 v = ta[e];
      sa[r + 0][f] = (uint32_t)(r + 0) < rows ? v.x : 0.0f;
      sa[r + 1][f] = (uint32_t)(r + 1) < rows ? v.y : 0.0f;
      sa[r + 2][f] = (uint32_t)(r + 2) < rows ? v.z : 0.0f;
      sa[r + 3][f] = (uint32_t)(r + 3) < rows ? v.w : 0.0f;
    }
    for (int e = tid; e < kDwTile * LDD / 4; e += kDwThreads) {
      const int f = (e >> 6) * 8 + (e & 7), r = ((e >> 3) & 7) * 4;
      const float4 v = f < OUT ? td[e] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      sd[r + 0][f] = (uint32_t)(r + 0) < rows ? v.x : 0.0f;
      sd[r + 1][f] = (uint32_t)(r + 1) < rows ? v.y : 0.0f;
      sd[r + 2][f] = (uint32_t)(r + 2) < rows ? v.z : 0.0f;
      sd[r + 3][f] = (uint32_t)(r + 3) < rows ? v.w : 0.0f;
    }
    __syncthreads();
#pragma unroll 4
    for (int r = grp; r < kDwTile; r += G) {
      const float4 a = *reinterpret_cast<const float4*>(&sa[r][ti * 4]);
      const float4 d = *reinterpret_cast<const float4*>(&sd[r][to * 4]);
      const float av[4] = {a.x, a.y, a.z, a.w}, dv[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[p][c] = fmaf(dv[p], av[c], acc[p][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int o = to * 4 + p;
    if (o < OUT)
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (acc[p][c] != 0.0f) atomicAdd(dw + o * IN + ti * 4 + c, acc[p][c]);
  }
}

// ---------------- weight gradients on the tensor cores (kind::f16, BF16 operands) ----------------
// The tensor-core backward stages its activations and deltas as BF16 (FP32's
// exponent range, 8-bit mantissa; FP16's range cannot hold the deltas) in the
// 16-bit operand layout of stage8: half the bytes of FP32 staging written by
// the backward and read back here, the round trip that bounds both kernels.
// Per 32-sample tile, two MMA groups, M = 128, K = 32 as two K = 16 steps:
//   D1[128 x 144] += [enc | cin | h1] (rows = features) x [dh1 | dg1 | dout]^T
//   D2[128 x  80] += [g1 | g2] x [dg2 | dlog | 0]^T
// whose diagonal blocks are the five dW^T (D1[enc][dh1] = DW1^T, D1[cin][dg1]
// = CW1^T, D1[h1][dout] = DW2^T, D2[g1][dg2] = CW2^T, D2[g2][dlog] = CW3^T);
// the off-diagonal products are discarded.  D stays in TMEM across all of a
// CTA's tiles and is added to dW once at the end.  One CTA per SM: warp 0
// lane 0 streams tiles into a 3-stage ring with bulk copies (one per array,
// the staging is already in the operand layout), warp 1 lane 0 issues the
// MMAs and releases stages by tcgen05.commit, all four warps read D back.
// The kernel is bound by reading the staging (30,208 B per tile).
constexpr int kTcStages = 3;
// Operand tiles of 32 records, BF16 (64 bytes per feature row).
constexpr uint32_t kA1Bytes = 128 * 64, kB1Bytes = 144 * 64, kA2Bytes = 128 * 64, kB2Bytes = 80 * 64;
constexpr uint32_t kStageBytes = kA1Bytes + kB1Bytes + kA2Bytes + kB2Bytes;
constexpr uint32_t kTileTx = (kEnc + kCIn + kHid + kHid + kHid + kDOut + kHid + kHid + kHid + kFDlog) * 64;
constexpr uint32_t kD1Col = 0, kD2Col = 144, kTmemCols = 256;
constexpr int kDwTcThreads = 128;
constexpr uint32_t kErrTimeout = 4u;

struct DwTcSmem {
  uint8_t stage[kTcStages][kStageBytes];
  uint64_t full[kTcStages], empty[kTcStages], done;
  uint32_t tmem_base;
};

__global__ void __launch_bounds__(kDwTcThreads, 1)
dw_tc_kernel(Staging st, uint32_t ntiles, float* __restrict__ dw, uint32_t* __restrict__ err) {
  extern __shared__ __align__(128) uint8_t smem_dw[];
  DwTcSmem& S = *reinterpret_cast<DwTcSmem*>(smem_dw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t per = (ntiles + gridDim.x - 1) / gridDim.x;
  const uint32_t t0 = blockIdx.x * per, t1 = min(ntiles, t0 + per);
  if (t1 <= t0) return;  // uniform over the CTA, before any barrier or TMEM use
  const uint32_t my = t1 - t0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kTcStages; ++i) {
      tc::mbar_init(&S.full[i], 1);
      tc::mbar_init(&S.empty[i], 1);
    }
    tc::mbar_init(&S.done, 1);
    tc::fence_mbar_init();
  }
  // B2 rows 72..79 are never copied: zero in every stage.
  for (int i = threadIdx.x; i < kTcStages * 128; i += blockDim.x)
    reinterpret_cast<float*>(S.stage[i / 128] + kA1Bytes + kB1Bytes + kA2Bytes + 72 * 64)[i % 128] = 0.0f;
  tc::fence_async_smem();
  if (warp == 1) {
    tc::tmem_alloc(&S.tmem_base, kTmemCols);
    tc::tmem_relinquish();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = S.tmem_base;
  if (warp == 0 && lane == 0) {  // producer
    uint32_t issued = 0;
    bool ok = true;
    for (uint32_t i = 0; i < my; ++i) {
      const int sidx = (int)(i % kTcStages);
      if (i >= (uint32_t)kTcStages && !tc::mbar_wait_sleep(&S.empty[sidx], ((i / kTcStages) & 1u) ^ 1u)) {
        ok = false;
        break;
      }
      uint8_t* a1 = S.stage[sidx];
      uint8_t* b1 = a1 + kA1Bytes;
      uint8_t* a2 = b1 + kB1Bytes;
      uint8_t* b2 = a2 + kA2Bytes;
      const size_t t = t0 + i;
      uint64_t* bar = &S.full[sidx];
      tc::mbar_arrive_expect_tx(bar, kTileTx);
      // Tile t of an F-wide BF16 array: F x 64 bytes at byte t x F x 64.
      auto tile = [&](const float* arr, int F) { return reinterpret_cast<const uint8_t*>(arr) + t * F * 64; };
      tc::bulk_g2s(a1, tile(st.enc, kEnc), kEnc * 64, bar);
      tc::bulk_g2s(a1 + kEnc * 64, tile(st.cin, kCIn), kCIn * 64, bar);
      tc::bulk_g2s(a1 + (kEnc + kCIn) * 64, tile(st.h1, kHid), kHid * 64, bar);
      tc::bulk_g2s(b1, tile(st.dh1, kHid), kHid * 64, bar);
      tc::bulk_g2s(b1 + kHid * 64, tile(st.dg1, kHid), kHid * 64, bar);
      tc::bulk_g2s(b1 + 2 * kHid * 64, tile(st.dout, kDOut), kDOut * 64, bar);
      tc::bulk_g2s(a2, tile(st.g1, kHid), kHid * 64, bar);
      tc::bulk_g2s(a2 + kHid * 64, tile(st.g2, kHid), kHid * 64, bar);
      tc::bulk_g2s(b2, tile(st.dg2, kHid), kHid * 64, bar);
      tc::bulk_g2s(b2 + kHid * 64, tile(st.dlog, kFDlog), kFDlog * 64, bar);
      ++issued;
    }
    if (!ok) atomicExch(err, kErrTimeout);
    // Copies still in flight land before the CTA may exit: wait (bounded)
    // for the last issued tile of every stage.
    for (uint32_t k = 0; k < (uint32_t)kTcStages && k < issued; ++k) {
      const uint32_t i = issued - 1 - k;
      if (!tc::mbar_wait_sleep(&S.full[i % kTcStages], (i / kTcStages) & 1u)) atomicExch(err, kErrTimeout);
    }
  } else if (warp == 1 && lane == 0) {  // MMA issuer
    constexpr uint32_t id1 = tc::idesc_bf16_f32(128, 144), id2 = tc::idesc_bf16_f32(128, 80);
    for (uint32_t i = 0; i < my; ++i) {
      const int sidx = (int)(i % kTcStages);
      if (!tc::mbar_wait_sleep(&S.full[sidx], (i / kTcStages) & 1u)) {
        atomicExch(err, kErrTimeout);
        break;
      }
      tc::fence_after();
      const uint32_t a1 = tc::smem_addr(S.stage[sidx]), b1 = a1 + kA1Bytes, a2 = b1 + kB1Bytes, b2 = a2 + kA2Bytes;
#pragma unroll
      for (uint32_t kk = 0; kk < 2; ++kk) {  // K = 32 records as two K = 16 steps
        const uint32_t acc = (i > 0 || kk > 0) ? 1u : 0u;
        tc::mma_f16(tmem + kD1Col, tc::sdesc(a1 + kk * 256, 128, 512), tc::sdesc(b1 + kk * 256, 128, 512), id1, acc);
        tc::mma_f16(tmem + kD2Col, tc::sdesc(a2 + kk * 256, 128, 512), tc::sdesc(b2 + kk * 256, 128, 512), id2, acc);
      }
      tc::mma_commit(&S.empty[sidx]);
    }
    tc::mma_commit(&S.done);
  }
  __syncwarp();
  // Epilogue: warp w owns TMEM lanes 32w..32w+31 (rows of D1 and D2).
  const bool done = tc::mbar_wait_sleep(&S.done, 0);
  tc::fence_after();
  if (!done) {
    if (lane == 0) atomicExch(err, kErrTimeout);
  } else {
    const uint32_t lanes = tmem + ((uint32_t)(warp * 32) << 16);
    const int row = warp * 32 + lane;
    float v[32];
    if (warp == 0) {  // D1 rows 0..31: enc feature `row` x dh1 j -> DW1[j][row]
      for (int c = 0; c < 2; ++c) {
        tc::tmem_ld32(lanes + kD1Col + 32 * c, v);
        for (int j = 0; j < 32; ++j) atomicAdd(dw + kOffDW1 + (32 * c + j) * kEnc + row, v[j]);
      }
    } else if (warp == 1) {  // D1 rows 32..63: cin feature row-32 x dg1 j -> CW1[j][row-32]
      for (int c = 0; c < 2; ++c) {
        tc::tmem_ld32(lanes + kD1Col + 64 + 32 * c, v);
        for (int j = 0; j < 32; ++j) atomicAdd(dw + kOffCW1 + (32 * c + j) * kCIn + (row - 32), v[j]);
      }
    } else {  // D1 rows 64..127: h1 feature row-64 x dout m -> DW2[m][row-64]
      float u[16];
      tc::tmem_ld16(lanes + kD1Col + 128, u);
      for (int m = 0; m < kDOut; ++m) atomicAdd(dw + kOffDW2 + m * kHid + (row - 64), u[m]);
    }
    if (warp < 2) {  // D2 rows 0..63: g1 feature `row` x dg2 j -> CW2[j][row]
      for (int c = 0; c < 2; ++c) {
        tc::tmem_ld32(lanes + kD2Col + 32 * c, v);
        for (int j = 0; j < 32; ++j) atomicAdd(dw + kOffCW2 + (32 * c + j) * kHid + row, v[j]);
      }
    } else {  // D2 rows 64..127: g2 feature row-64 x dlog c -> CW3[c][row-64]
      float u[16];
      tc::tmem_ld16(lanes + kD2Col + 64, u);
      for (int c = 0; c < 3; ++c) atomicAdd(dw + kOffCW3 + c * kHid + (row - 64), u[c]);
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 1) tc::tmem_dealloc(tmem, kTmemCols);
}

// ---------------- per-sample MLP recompute and backward on the tensor cores (kind::tf32) ----------------
// One CTA per SM, four independent groups of 4 warps; a group takes 128
// records at a time (thread = record = TMEM lane) and runs the 10 layer
// products of the recompute and the backward as tcgen05.mma kind::tf32 with
// the A operand (this layer's input, one FP32 element per TMEM column) in
// TMEM and B (a weight image, below) in shared memory, the FP32 product in
// TMEM.  Between products each thread reads its row back, applies the
// elementwise step (ReLU and its mask, exp, SH, sigmoid and their
// derivatives), stages activations and deltas for the weight-gradient GEMMs
// (same layout as backward_kernel) and writes the next A.  TF32 operands
// (10-bit mantissa, FP32 accumulation) put ~1e-3 relative error on the
// per-sample activations and deltas; backward_kernel is the FP32 form.
//   forward:  h1 = relu(enc dW1^T)  out = h1 dW2^T  g1 = relu(cin cW1^T)
//             g2 = relu(g1 cW2^T)   logit = g2 cW3^T
//   backward: dg2 = (dlog cW3) m2   dg1 = (dg2 cW2) m1   dgeo = dg1 cW1[:,16:32]
//             dh1 = (dout dW2) mh   denc = dh1 dW1
constexpr int kBtGroups = 4;
constexpr int kBtThreads = 128 * kBtGroups;
constexpr uint32_t kBtColsPerGroup = 128;  // A: 64 columns, D: 64 columns

// Hash-grid scatter-add of one record's encoding gradient,
// dtable[l][corner] += w_corner * denc[2l..2l+1].  Every lane of the warp
// calls it (valid = false for a lane without a record).  A warp's records
// are consecutive samples of one or two rays, so at the coarse levels runs
// of neighbouring lanes share a cell: levels 0..kAggLevels-1 sum each run's
// corner gradients with shuffles and add them with one atomic per run.
constexpr int kAggLevels = 13;  // levels whose scatter-add is warp-aggregated (N <= 776)
static_assert(level_res(kAggLevels - 1) < 1024, "cell key packs 10 bits per coordinate");

__device__ __forceinline__ void scatter_add_levels(float2* __restrict__ gtable, const DevScene& sc, float3 x,
                                                   const float (&denc)[kEnc], bool valid, uint32_t lane) {
#pragma unroll 1
  for (int l = 0; l < kLevels; ++l) {
    const int N = level_res(l);
    const LevelCell c = level_cell(x, N);
    uint32_t idx[8];
    corner_indices(c, N, (sc.dense_mask >> l) & 1u, sc.T, idx);
    float w[8];
    corner_weights(c, w);
    float2* gt = gtable + (size_t)l * sc.T;
    float d0 = 0.0f, d1 = 0.0f;
#pragma unroll
    for (int k = 0; k < kLevels; ++k)
      if (k == l) {
        d0 = denc[2 * k];
        d1 = denc[2 * k + 1];
      }
    if (l >= kAggLevels) {
      if (valid && !((sc.dense_mask >> l) & 1u) && (c.ix & 1u) == 0u) {
        // Hashed level, even x: the x prime is 1, so corners k and k + 1
        // are the aligned entry pair {i, i ^ 1}; one 16-byte atomic each.
#pragma unroll
        for (int k = 0; k < 8; k += 2) {
          const uint32_t i = idx[k];
          const float4 v = (i & 1u) ? make_float4(w[k + 1] * d0, w[k + 1] * d1, w[k] * d0, w[k] * d1)
                                    : make_float4(w[k] * d0, w[k] * d1, w[k + 1] * d0, w[k + 1] * d1);
          atomicAdd(reinterpret_cast<float4*>(gt + (i & ~1u)), v);
        }
      } else if (valid) {
#pragma unroll
        for (int k = 0; k < 8; ++k) atomicAdd(gt + idx[k], make_float2(w[k] * d0, w[k] * d1));
      }
      continue;
    }
    // Runs of lanes with the same cell (invalid lanes form runs of their
    // own and add nothing).  N <= 776 here: 10 bits per coordinate.
    const uint32_t key = valid ? (c.ix | (c.iy << 10) | (c.iz << 20)) : (0x80000000u | lane);
    const uint32_t kprev = __shfl_up_sync(0xffffffffu, key, 1);
    const uint32_t heads = __ballot_sync(0xffffffffu, lane == 0 || kprev != key);
    if (heads == 0xffffffffu) {  // no lane shares its cell
      if (valid)
#pragma unroll
        for (int k = 0; k < 8; ++k) atomicAdd(gt + idx[k], make_float2(w[k] * d0, w[k] * d1));
      continue;
    }
    // Step o adds the partial sum of lane + o when no run starts in
    // (lane, lane + o]; afterwards each run's first lane holds its total.
    uint32_t take = 0;
#pragma unroll
    for (int o = 1, b = 0; o < 32; o <<= 1, ++b) {
      const uint32_t span = (uint32_t)(((1ull << o) - 1ull) << (lane + 1));  // lanes lane+1 .. lane+o
      if (lane + o < 32u && (heads & span) == 0u) take |= 1u << b;
    }
    const bool head = (heads >> lane) & 1u;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      float a0 = w[k] * d0, a1 = w[k] * d1;
#pragma unroll
      for (int o = 1, b = 0; o < 32; o <<= 1, ++b) {
        const float p0 = __shfl_down_sync(0xffffffffu, a0, o), p1 = __shfl_down_sync(0xffffffffu, a1, o);
        if ((take >> b) & 1u) {
          a0 += p0;
          a1 += p1;
        }
      }
      if (valid && head) atomicAdd(gt + idx[k], make_float2(a0, a1));
    }
  }
}

// Weight images, [N][K] K-major, no swizzle, FP32 bits read as TF32: core
// matrices of 8 rows x 4 elements (16 B rows, 128 B each), K-adjacent at
// 128 B (LBO), 8-row groups K/4 x 128 B apart (SBO).
__host__ __device__ constexpr uint32_t tf32_off(int n, int k, int K) {
  return (uint32_t)((n >> 3) * (K * 32) + (k >> 2) * 128 + (n & 7) * 16 + (k & 3) * 4);
}
struct BtImage {
  uint32_t off, N, K;
};
constexpr int kBtImages = 10;
// dW1, dW2, cW1, cW2, cW3 (rows 3..15 zero), cW3^T (k 3..15 zero), cW2^T,
// cW1 geometry columns transposed ([n][j] = cW1[j][16 + n], row 15 zero),
// dW2^T, dW1^T.
__host__ __device__ constexpr BtImage bt_image(int i) {
  return i == 0   ? BtImage{0, 64, 32}
         : i == 1 ? BtImage{8192, 16, 64}
         : i == 2 ? BtImage{12288, 64, 32}
         : i == 3 ? BtImage{20480, 64, 64}
         : i == 4 ? BtImage{36864, 16, 64}
         : i == 5 ? BtImage{40960, 64, 16}
         : i == 6 ? BtImage{45056, 64, 64}
         : i == 7 ? BtImage{61440, 16, 64}
         : i == 8 ? BtImage{65536, 64, 16}
                  : BtImage{69632, 32, 64};
}
constexpr uint32_t kBtImageBytes = 77824;
static_assert(bt_image(9).off + bt_image(9).N * bt_image(9).K * 4 == kBtImageBytes, "image table");

// Value of element (n, k) of image i from the FP32 weight blob.
__device__ __forceinline__ float bt_value(const float* __restrict__ w, int i, int n, int k) {
  switch (i) {
    case 0: return w[kOffDW1 + n * kEnc + k];
    case 1: return w[kOffDW2 + n * kHid + k];
    case 2: return w[kOffCW1 + n * kCIn + k];
    case 3: return w[kOffCW2 + n * kHid + k];
    case 4: return n < 3 ? w[kOffCW3 + n * kHid + k] : 0.0f;
    case 5: return k < 3 ? w[kOffCW3 + k * kHid + n] : 0.0f;
    case 6: return w[kOffCW2 + k * kHid + n];
    case 7: return n < 15 ? w[kOffCW1 + k * kCIn + 16 + n] : 0.0f;
    case 8: return w[kOffDW2 + k * kHid + n];
    default: return w[kOffDW1 + k * kEnc + n];
  }
}

__global__ void pack_bt_images_kernel(const float* __restrict__ w, uint8_t* __restrict__ img) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;  // element of the concatenated images
  if (e >= kBtImageBytes / 4) return;
  int i = 0;
  while (i + 1 < kBtImages && e >= bt_image(i + 1).off / 4) ++i;
  const BtImage b = bt_image(i);
  const uint32_t local = e - b.off / 4;
  const int n = (int)(local / b.K), k = (int)(local % b.K);
  *reinterpret_cast<float*>(img + b.off + tf32_off(n, k, (int)b.K)) = bt_value(w, i, n, k);
}

__device__ __forceinline__ uint32_t f2u(float v) { return __float_as_uint(v); }

// Staging of features f..f+7 (f % 8 == 0) of this thread's record as BF16,
// in the canonical K-major layout of a 16-bit tensor-core operand with
// K = record: 8 features x 8 records per 128-byte core matrix (16-byte rows,
// one feature each), record groups of 8 at 128 B, feature groups of 8 at
// 512 B; an F-wide array's 32-record tile is F x 64 contiguous bytes.  The
// eight lanes of an octet hold eight consecutive records; an 8x8 transpose of
// 16-bit values inside the octet -- packed halves exchanged with the
// neighbouring lane, then a 4x4 transpose of 32-bit words across lanes 2 and
// 4 apart, six shuffles -- leaves lane r with feature f + r of all eight
// records: one 16-byte row.  A warp's 32 records are one tile, so each call
// writes one contiguous 512-byte block.  Every lane of the warp must call it.
// Two FP32 values -> packed BF16 (round to nearest even), lo in the low half.
__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}
__device__ __forceinline__ void stage8(float* arr, int F, uint32_t s, int f, float a0, float a1, float a2, float a3,
                                       float a4, float a5, float a6, float a7, bool stage) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t w[4] = {bf16x2(a0, a1), bf16x2(a2, a3), bf16x2(a4, a5), bf16x2(a6, a7)};  // low half: even feature
  // Records 2p and 2p + 1 (lanes r and r ^ 1): the even lane keeps the even
  // features of both, the odd lane the odd ones.
  const bool even = (lane & 1u) == 0u;
  const uint32_t give = even ? 0x7632u : 0x5410u;  // the halves the neighbour keeps
  const uint32_t r0 = __shfl_xor_sync(0xffffffffu, __byte_perm(w[0], w[1], give), 1);
  const uint32_t r1 = __shfl_xor_sync(0xffffffffu, __byte_perm(w[2], w[3], give), 1);
  uint32_t z0, z1, z2, z3;  // z_j: feature 2j + (lane & 1) of records 2p, 2p + 1
  if (even) {
    z0 = __byte_perm(w[0], r0, 0x5410u);
    z1 = __byte_perm(w[1], r0, 0x7610u);
    z2 = __byte_perm(w[2], r1, 0x5410u);
    z3 = __byte_perm(w[3], r1, 0x7610u);
  } else {
    z0 = __byte_perm(r0, w[0], 0x7610u);
    z1 = __byte_perm(r0, w[1], 0x7632u);
    z2 = __byte_perm(r1, w[2], 0x7610u);
    z3 = __byte_perm(r1, w[3], 0x7632u);
  }
  // 4x4 transpose over (record pair p = lane bits 1-2, j).
  const bool odd = (lane >> 1) & 1u, hi = (lane >> 2) & 1u;
  uint32_t t = __shfl_xor_sync(0xffffffffu, odd ? z0 : z1, 2);
  if (odd) z0 = t; else z1 = t;
  t = __shfl_xor_sync(0xffffffffu, odd ? z2 : z3, 2);
  if (odd) z2 = t; else z3 = t;
  t = __shfl_xor_sync(0xffffffffu, hi ? z0 : z2, 4);
  if (hi) z0 = t; else z2 = t;
  t = __shfl_xor_sync(0xffffffffu, hi ? z1 : z3, 4);
  if (hi) z1 = t; else z3 = t;
  if (stage) {
    uint8_t* tile = reinterpret_cast<uint8_t*>(arr) + (size_t)(s >> 5) * (size_t)F * 64u;
    *reinterpret_cast<uint4*>(tile + (f >> 3) * 512 + (lane >> 3) * 128 + (lane & 7u) * 16) = make_uint4(z0, z1, z2, z3);
  }
}

__global__ void __launch_bounds__(kBtThreads, 1)
backward_tc_kernel(const SampleRec* __restrict__ recs, uint32_t first, uint32_t count,
                   const TrainRay* __restrict__ rays, const DevScene sc, const uint8_t* __restrict__ images,
                   Staging st, float2* __restrict__ gtable, uint32_t* __restrict__ err) {
  extern __shared__ __align__(128) uint8_t smem_bt[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_bt + kBtImageBytes);  // [group] mma, [kBtGroups] weights
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + kBtGroups + 1);
  const int tid = threadIdx.x, warp = tid >> 5, g = tid >> 7, row = tid & 127;
  if (tid == 0) {
    for (int k = 0; k <= kBtGroups; ++k) tc::mbar_init(bars + k, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, kBtColsPerGroup * kBtGroups);
    tc::tmem_relinquish();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tslot;
  bool fail = false;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(bars + kBtGroups, kBtImageBytes);
    tc::bulk_g2s(smem_bt, images, kBtImageBytes, bars + kBtGroups);
    fail = !tc::mbar_wait(bars + kBtGroups, 0);
  }
  fail = __syncthreads_or(fail);
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
  const uint32_t a_col = tmem + g * kBtColsPerGroup, d_col = a_col + 64;
  const uint32_t a_row = a_col + lane_off, d_row = d_col + lane_off;
  const uint32_t sB = tc::smem_addr(smem_bt);
  const uint32_t gbar = 1 + g;
  uint64_t* mbar = bars + g;
  uint32_t pm = 0;
  bool ok = true;
  // D[:, :N] = A[:, :K] B_i^T.  Every thread publishes its TMEM writes; the
  // group learns of any failed wait here and stops as a whole.
  auto mma = [&](int i) -> bool {
    tc::tmem_wait_st();
    tc::fence_before();
    if (tc::named_sync_or(gbar, 128, !ok)) return false;
    const BtImage b = bt_image(i);
    if (row == 0) {
      tc::fence_after();
      const uint32_t idesc = tc::idesc_tf32_f32(128, (int)b.N);
      for (uint32_t j = 0; j < b.K / 8; ++j)
        tc::mma_tf32_at(d_col, a_col + 8 * j, tc::sdesc(sB + b.off + 256 * j, 128, b.K * 32), idesc, j > 0 ? 1u : 0u);
      tc::mma_commit(mbar);
    }
    ok = tc::mbar_wait(mbar, pm) && ok;
    pm ^= 1u;
    tc::fence_after();
    return true;
  };

  const uint32_t ntiles = (count + 127u) / 128u;
  const uint32_t staged = (count + 31u) & ~31u;  // rows the weight-gradient GEMMs read
  if (!fail) {
    for (uint32_t tile = blockIdx.x * kBtGroups + g; tile < ntiles; tile += gridDim.x * kBtGroups) {
      const uint32_t s = tile * 128u + (uint32_t)row;
      const bool valid = s < count, stage = s < staged;
      SampleRec q;
      if (valid) {
        q = recs[first + s];
      } else {
        q.x = q.y = q.z = 0.0f;
        q.ray = 0;
        q.dsigma = q.dcr = q.dcg = q.dcb = 0.0f;
      }
      const float3 x = make_float3(q.x, q.y, q.z);
      uint32_t u[32];
      float v[32];
      // ---- forward recompute ----
      {
        float enc[kEnc];
        if (valid) {
          encode_fp32(sc.table32, sc.T, sc.dense_mask, x, enc);
        } else {
#pragma unroll
          for (int k = 0; k < kEnc; ++k) enc[k] = 0.0f;
        }
#pragma unroll
        for (int k = 0; k < kEnc; ++k) u[k] = f2u(enc[k]);
        tc::tmem_st32_nowait(a_row, u);
#pragma unroll
        for (int k = 0; k < kEnc; k += 8) stage8(st.enc, kEnc, s, k, enc[k + 0], enc[k + 1], enc[k + 2], enc[k + 3], enc[k + 4], enc[k + 5], enc[k + 6], enc[k + 7], stage);
      }
      if (!mma(0)) break;
      uint64_t m_h1 = 0, m_g1 = 0, m_g2 = 0;
      // ReLU of D[:, :64] -> staging, mask, next A.
      auto relu64 = [&](float* act, uint64_t& m) {
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          tc::tmem_ld32(d_row + 32 * c, v);
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            v[j] = valid ? fmaxf(v[j], 0.0f) : 0.0f;
            m |= (uint64_t)(v[j] > 0.0f) << (32 * c + j);
            u[j] = f2u(v[j]);
          }
          tc::tmem_st32_nowait(a_row + 32 * c, u);
#pragma unroll
          for (int j = 0; j < 32; j += 8) stage8(act, kHid, s, 32 * c + j, v[j + 0], v[j + 1], v[j + 2], v[j + 3], v[j + 4], v[j + 5], v[j + 6], v[j + 7], stage);
        }
      };
      relu64(st.h1, m_h1);
      if (!mma(1)) break;
      float sigma;
      {
        float out[16];
        tc::tmem_ld16(d_row, reinterpret_cast<float(&)[16]>(out));
        sigma = expf(out[0] - 1.0f);
        float cin[kCIn];
        const TrainRay& r = rays[q.ray];
        sh16(make_float3(r.dx, r.dy, r.dz), cin);
#pragma unroll
        for (int k = 0; k < 15; ++k) cin[16 + k] = out[1 + k];
        cin[31] = 0.0f;
#pragma unroll
        for (int k = 0; k < kCIn; ++k) {
          cin[k] = valid ? cin[k] : 0.0f;
          u[k] = f2u(cin[k]);
        }
        tc::tmem_st32_nowait(a_row, u);
#pragma unroll
        for (int k = 0; k < kCIn; k += 8) stage8(st.cin, kCIn, s, k, cin[k + 0], cin[k + 1], cin[k + 2], cin[k + 3], cin[k + 4], cin[k + 5], cin[k + 6], cin[k + 7], stage);
      }
      if (!mma(2)) break;
      relu64(st.g1, m_g1);
      if (!mma(3)) break;
      relu64(st.g2, m_g2);
      if (!mma(4)) break;
      // ---- backward ----
      {
        float lg[16];
        tc::tmem_ld16(d_row, reinterpret_cast<float(&)[16]>(lg));
        const float c0 = sigmoidf(lg[0]), c1 = sigmoidf(lg[1]), c2 = sigmoidf(lg[2]);
        const float dl[3] = {q.dcr * c0 * (1.0f - c0), q.dcg * c1 * (1.0f - c1), q.dcb * c2 * (1.0f - c2)};
        uint32_t w16[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) w16[k] = k < 3 ? f2u(dl[k]) : 0u;
        tc::tmem_st16_nowait(a_row, w16);
        stage8(st.dlog, kFDlog, s, 0, dl[0], dl[1], dl[2], 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, stage);
      }
      // Masked D[:, :64] -> staging, next A.
      auto mask64 = [&](float* delta, uint64_t m) {
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          tc::tmem_ld32(d_row + 32 * c, v);
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            v[j] = ((m >> (32 * c + j)) & 1u) ? v[j] : 0.0f;
            u[j] = f2u(v[j]);
          }
          tc::tmem_st32_nowait(a_row + 32 * c, u);
#pragma unroll
          for (int j = 0; j < 32; j += 8) stage8(delta, kHid, s, 32 * c + j, v[j + 0], v[j + 1], v[j + 2], v[j + 3], v[j + 4], v[j + 5], v[j + 6], v[j + 7], stage);
        }
      };
      if (!mma(5)) break;
      mask64(st.dg2, m_g2);
      if (!mma(6)) break;
      mask64(st.dg1, m_g1);
      if (!mma(7)) break;
      {
        float geo[16];
        tc::tmem_ld16(d_row, reinterpret_cast<float(&)[16]>(geo));
        uint32_t w16[16];
        float dout[16];
        dout[0] = q.dsigma * sigma;
#pragma unroll
        for (int m = 0; m < 15; ++m) dout[1 + m] = geo[m];
#pragma unroll
        for (int m = 0; m < 16; ++m) w16[m] = f2u(dout[m]);
        tc::tmem_st16_nowait(a_row, w16);
#pragma unroll
        for (int m = 0; m < kDOut; m += 8) stage8(st.dout, kDOut, s, m, dout[m + 0], dout[m + 1], dout[m + 2], dout[m + 3], dout[m + 4], dout[m + 5], dout[m + 6], dout[m + 7], stage);
      }
      if (!mma(8)) break;
      mask64(st.dh1, m_h1);
      if (!mma(9)) break;
      tc::tmem_ld32(d_row, v);  // denc
      // The next tile's first product overwrites D: its sync follows these reads.
      scatter_add_levels(gtable, sc, x, v, valid, (uint32_t)(tid & 31));
    }
  }
  if (fail || !ok) atomicExch(err, kErrTimeout);
  tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, kBtColsPerGroup * kBtGroups);
  }
}
constexpr int kBtSmem = (int)kBtImageBytes + 8 * (kBtGroups + 1) + 16;

// ---------------- the forward's field evaluation on the tensor cores, 3xTF32 ----------------
// eval_kernel's work as tcgen05 kind::tf32 products at FP32-level accuracy:
// every operand is split into its TF32 rounding (hi) and the FP32 remainder
// (lo), and each layer accumulates A_hi B_hi + A_lo B_hi + A_hi B_lo in FP32.
// The dropped A_lo B_lo term and the remainders' own TF32 truncation are
// below 2^-21 of each product, so the loss keeps the FP32 evaluation's value
// (plain TF32 products would move it by ~1e-3 relative: a refit whose
// rendered colour sits within 1e-2 of the target then sees a few per cent of
// error in its loss and adjoints).  One CTA per SM, two independent groups of
// 4 warps; a group takes 128 listed samples at a time (thread = sample = TMEM
// lane), writes each layer's input as A_hi and A_lo into TMEM, one thread
// issues the three K-chains against the weight images' high and low parts in
// shared memory, and every thread reads its row of D back for the
// elementwise step (ReLU, exp, SH, sigmoid) and the next layer's input.  The
// table gathers of the group's next tile run while the MMAs of layers 1-4 of
// the current one do (four levels per layer), into TMEM columns of their own
// that layer 0 of the next tile reads: only two tiles' worth of warps per SM
// fit the TMEM, so the gathers' latency is hidden behind the layer chain.
constexpr int kEtGroups = 2;
constexpr int kEtThreads = 128 * kEtGroups;
// A_hi: 0..63, A_lo: 64..127, D: 128..191, next tile's encoding E_hi:
// 192..223, E_lo: 224..255.
constexpr uint32_t kEtColsPerGroup = 256;
constexpr uint32_t kFwdImageBytes = 40960;  // bt_image 0..4: dW1, dW2, cW1, cW2, cW3
static_assert(bt_image(5).off == kFwdImageBytes, "forward images first");
constexpr uint32_t kEtImageBytes = 2 * kFwdImageBytes;  // high parts, then low parts
constexpr int kEtSmem = (int)kEtImageBytes + 8 * (kEtGroups + 1) + 16;

__device__ __forceinline__ float tf32_hi(float v) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return __uint_as_float(r);
}

// The forward images' high and low parts from the FP32 weights.
__global__ void pack_et_images_kernel(const float* __restrict__ w, uint8_t* __restrict__ img) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kFwdImageBytes / 4) return;
  int i = 0;
  while (i + 1 < 5 && e >= bt_image(i + 1).off / 4) ++i;
  const BtImage b = bt_image(i);
  const uint32_t local = e - b.off / 4;
  const int n = (int)(local / b.K), k = (int)(local % b.K);
  const float v = bt_value(w, i, n, k), hi = tf32_hi(v);
  const uint32_t o = b.off + tf32_off(n, k, (int)b.K);
  *reinterpret_cast<float*>(img + o) = hi;
  *reinterpret_cast<float*>(img + kFwdImageBytes + o) = v - hi;
}

// One listed sample's inputs.
struct EtSample {
  uint32_t ray, k;
  float t;
  float3 o, d;
  bool valid;
};

__device__ __forceinline__ EtSample et_sample(const uint2* __restrict__ list, uint32_t j, uint32_t m,
                                              const TrainRay* __restrict__ rays, int n) {
  EtSample q;
  const uint2 e = j < m ? list[j] : make_uint2(0xFFFFFFFFu, 0u);
  q.ray = e.x;
  q.k = e.y & ((1u << kListStepShift) - 1u);
  // (an out-of-range entry exists only after an overflow, which is flagged)
  q.valid = j < m && q.ray < (uint32_t)n && q.k < (uint32_t)kMaxSteps;
  q.t = 0.0f;
  q.o = make_float3(0.0f, 0.0f, 0.0f);
  q.d = make_float3(0.0f, 0.0f, 1.0f);
  if (q.valid) {
    const TrainRay& r = rays[q.ray];
    q.t = fmaf((float)(e.y >> kListStepShift) + 0.5f, kDt, r.ts);
    q.o = make_float3(r.ox, r.oy, r.oz);
    q.d = make_float3(r.dx, r.dy, r.dz);
  }
  return q;
}

// Levels L0..L0+3 of a sample's encoding -> E_hi / E_lo columns 2 L0 ..
// 2 L0 + 7 of this thread's lane (no wait).  Every lane of the warp calls it.
template <int L0>
__device__ __forceinline__ void et_encode4(const DevScene& sc, const EtSample& q, uint32_t ehi_row,
                                           uint32_t elo_row) {
  float f[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) f[j] = 0.0f;
  if (q.valid) {
    const float3 x = sample_pos(q.o, q.d, q.t);
#pragma unroll
    for (int j = 0; j < 4; ++j) encode_level_fp32(sc.table32, sc.T, sc.dense_mask, x, L0 + j, f[2 * j], f[2 * j + 1]);
  }
  uint32_t h[8], l[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float hi = tf32_hi(f[j]);
    h[j] = __float_as_uint(hi);
    l[j] = __float_as_uint(f[j] - hi);
  }
  tc::tmem_st4(ehi_row + 2 * L0, h[0], h[1], h[2], h[3]);
  tc::tmem_st4(ehi_row + 2 * L0 + 4, h[4], h[5], h[6], h[7]);
  tc::tmem_st4(elo_row + 2 * L0, l[0], l[1], l[2], l[3]);
  tc::tmem_st4(elo_row + 2 * L0 + 4, l[4], l[5], l[6], l[7]);
}

__global__ void __launch_bounds__(kEtThreads, 1)
eval_tc_kernel(const uint2* __restrict__ list, const uint32_t* __restrict__ total, uint32_t capacity,
               const TrainRay* __restrict__ rays, int n, const DevScene sc, const uint8_t* __restrict__ images,
               ScratchSample* __restrict__ scratch, uint32_t* __restrict__ err) {
  extern __shared__ __align__(128) uint8_t smem_et[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_et + kEtImageBytes);  // [group] mma, [kEtGroups] images
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + kEtGroups + 1);
  const int tid = threadIdx.x, warp = tid >> 5, g = tid >> 7, row = tid & 127;
  if (tid == 0) {
    for (int k = 0; k <= kEtGroups; ++k) tc::mbar_init(bars + k, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, kEtColsPerGroup * kEtGroups);
    tc::tmem_relinquish();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *tslot;
  bool fail = false;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(bars + kEtGroups, kEtImageBytes);
    tc::bulk_g2s(smem_et, images, kEtImageBytes, bars + kEtGroups);
    fail = !tc::mbar_wait(bars + kEtGroups, 0);
  }
  fail = __syncthreads_or(fail);
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
  const uint32_t hi_col = tmem + g * kEtColsPerGroup, lo_col = hi_col + 64, d_col = hi_col + 128;
  const uint32_t ehi_col = hi_col + 192, elo_col = hi_col + 224;
  const uint32_t hi_row = hi_col + lane_off, lo_row = lo_col + lane_off, d_row = d_col + lane_off;
  const uint32_t ehi_row = ehi_col + lane_off, elo_row = elo_col + lane_off;
  const uint32_t sB = tc::smem_addr(smem_et);
  const uint32_t gbar = 1 + g;
  uint64_t* mbar = bars + g;
  uint32_t pm = 0;
  bool ok = true;
  // The layer input x[0..K) -> A_hi, A_lo (no wait: the next issue waits).
  auto put = [&](const float* x, int K) {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      if (c * 32 >= K) break;
      uint32_t uh[32], ul[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const float h = tf32_hi(x[32 * c + j]);
        uh[j] = __float_as_uint(h);
        ul[j] = __float_as_uint(x[32 * c + j] - h);
      }
      tc::tmem_st32_nowait(hi_row + 32 * c, uh);
      tc::tmem_st32_nowait(lo_row + 32 * c, ul);
    }
  };
  // D[:, :N] = A B_i^T at 3xTF32, A from columns (a_hi, a_lo): every thread
  // publishes its TMEM writes, one thread issues; the group learns of any
  // failed wait here and stops as a whole.
  auto issue = [&](int i, uint32_t a_hi, uint32_t a_lo) -> bool {
    tc::tmem_wait_st();
    tc::fence_before();
    if (tc::named_sync_or(gbar, 128, !ok)) return false;
    const BtImage b = bt_image(i);
    if (row == 0) {
      tc::fence_after();
      const uint32_t idesc = tc::idesc_tf32_f32(128, (int)b.N);
      const uint32_t steps = b.K / 8;
      for (uint32_t j = 0; j < steps; ++j)
        tc::mma_tf32_at(d_col, a_hi + 8 * j, tc::sdesc(sB + b.off + 256 * j, 128, b.K * 32), idesc, j > 0 ? 1u : 0u);
      for (uint32_t j = 0; j < steps; ++j)
        tc::mma_tf32_at(d_col, a_lo + 8 * j, tc::sdesc(sB + b.off + 256 * j, 128, b.K * 32), idesc, 1u);
      for (uint32_t j = 0; j < steps; ++j)
        tc::mma_tf32_at(d_col, a_hi + 8 * j, tc::sdesc(sB + kFwdImageBytes + b.off + 256 * j, 128, b.K * 32),
                        idesc, 1u);
      tc::mma_commit(mbar);
    }
    return true;
  };
  auto wait = [&]() {
    ok = tc::mbar_wait(mbar, pm) && ok;
    pm ^= 1u;
    tc::fence_after();
  };
  // ReLU of D[:, :64] -> x.
  auto relu64 = [&](float (&x)[64]) {
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      float v[32];
      tc::tmem_ld32(d_row + 32 * c, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) x[32 * c + j] = fmaxf(v[j], 0.0f);
    }
  };

  const uint32_t m = min(*total, capacity);
  const uint32_t ntiles = (m + 127u) / 128u;
  const uint32_t stride = gridDim.x * kEtGroups;
  uint32_t tile = blockIdx.x * kEtGroups + g;
  if (!fail && tile < ntiles) {
    // The first tile's encoding; later tiles' are gathered during the
    // previous tile's layers.
    EtSample cur = et_sample(list, tile * 128u + (uint32_t)row, m, rays, n);
    et_encode4<0>(sc, cur, ehi_row, elo_row);
    et_encode4<4>(sc, cur, ehi_row, elo_row);
    et_encode4<8>(sc, cur, ehi_row, elo_row);
    et_encode4<12>(sc, cur, ehi_row, elo_row);
    for (; tile < ntiles; tile += stride) {
      const bool more = tile + stride < ntiles;
      const EtSample nxt = et_sample(list, (tile + stride) * 128u + (uint32_t)row, more ? m : 0u, rays, n);
      float x[64];
      if (!issue(0, ehi_col, elo_col)) break;  // h1 = relu(enc dW1^T)
      wait();
      relu64(x);
      put(x, kHid);
      if (!issue(1, hi_col, lo_col)) break;  // out = h1 dW2^T
      et_encode4<0>(sc, nxt, ehi_row, elo_row);
      wait();
      float sigma;
      {
        float out[16];
        tc::tmem_ld16(d_row, out);
        sigma = expf(out[0] - 1.0f);
        float sh[16];
        sh16(cur.d, sh);
#pragma unroll
        for (int q = 0; q < 16; ++q) x[q] = sh[q];
#pragma unroll
        for (int q = 0; q < 15; ++q) x[16 + q] = out[1 + q];
        x[31] = 0.0f;
      }
      put(x, kCIn);
      if (!issue(2, hi_col, lo_col)) break;  // g1 = relu(cin cW1^T)
      et_encode4<4>(sc, nxt, ehi_row, elo_row);
      wait();
      relu64(x);
      put(x, kHid);
      if (!issue(3, hi_col, lo_col)) break;  // g2 = relu(g1 cW2^T)
      et_encode4<8>(sc, nxt, ehi_row, elo_row);
      wait();
      relu64(x);
      put(x, kHid);
      if (!issue(4, hi_col, lo_col)) break;  // logit = g2 cW3^T
      et_encode4<12>(sc, nxt, ehi_row, elo_row);
      wait();
      float lg[16];
      tc::tmem_ld16(d_row, lg);
      // The next tile's first product overwrites D: its sync follows these reads.
      if (cur.valid) {
        const float alpha = -expm1f(-sigma * kDt);
        scratch[(size_t)cur.ray * kMaxSteps + cur.k] =
            ScratchSample{cur.t, alpha, 0.0f, sigmoidf(lg[0]), sigmoidf(lg[1]), sigmoidf(lg[2]), 0.0f, 0.0f};
      }
      cur = nxt;
    }
  }
  if (fail || !ok) atomicExch(err, kErrTimeout);
  tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, kEtColsPerGroup * kEtGroups);
  }
}

__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                            size_t n, float lr, float b1, float b2, float eps, float bc1, float bc2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    g[i] = 0.0f;
  }
}

// ---------------- FP64 loss (finite differences) ----------------

struct ParamsF64 {
  const float* table;  // FP32 table, read as double
  const float* w;      // FP32 weight blob
  int which;           // perturbed array: 0 table, 1 weights
  uint64_t index;
  double delta;
};

__device__ __forceinline__ double tab(const ParamsF64& P, uint64_t i) {
  return (double)P.table[i] + ((P.which == 0 && i == P.index) ? P.delta : 0.0);
}
__device__ __forceinline__ double wt(const ParamsF64& P, int i) {
  return (double)P.w[i] + ((P.which == 1 && (uint64_t)i == P.index) ? P.delta : 0.0);
}

// Field query in FP64: same cells and hash indices as encode_fp32 (the cell
// is chosen from the FP32 position), FP64 weights and MLPs.
__device__ void query_f64(const ParamsF64& P, const DevScene& sc, const float3 xf, const float3 d, double& sigma,
                          double rgb[3]) {
  double enc[kEnc];
  const double x[3] = {xf.x, xf.y, xf.z};
  for (int l = 0; l < kLevels; ++l) {
    const int N = level_res(l);
    const LevelCell c = level_cell(xf, N);
    uint32_t idx[8];
    corner_indices(c, N, (sc.dense_mask >> l) & 1u, sc.T, idx);
    const double f[3] = {x[0] * N - (double)c.ix, x[1] * N - (double)c.iy, x[2] * N - (double)c.iz};
    double a0 = 0, a1 = 0;
    for (int k = 0; k < 8; ++k) {
      const double w = ((k & 1) ? f[0] : 1 - f[0]) * ((k & 2) ? f[1] : 1 - f[1]) * ((k & 4) ? f[2] : 1 - f[2]);
      const uint64_t e = ((uint64_t)l * sc.T + idx[k]) * 2;
      a0 += w * tab(P, e);
      a1 += w * tab(P, e + 1);
    }
    enc[2 * l] = a0;
    enc[2 * l + 1] = a1;
  }
  double h1[kHid], out[kDOut];
  for (int j = 0; j < kHid; ++j) {
    double a = 0;
    for (int k = 0; k < kEnc; ++k) a += wt(P, kOffDW1 + j * kEnc + k) * enc[k];
    h1[j] = a > 0 ? a : 0;
  }
  for (int m = 0; m < kDOut; ++m) {
    double a = 0;
    for (int j = 0; j < kHid; ++j) a += wt(P, kOffDW2 + m * kHid + j) * h1[j];
    out[m] = a;
  }
  sigma = exp(out[0] - 1);
  float sh[16];
  sh16(d, sh);  // the direction basis as rendered (FP32): it holds no parameter
  double cin[kCIn];
  for (int k = 0; k < 16; ++k) cin[k] = sh[k];
  for (int k = 0; k < 15; ++k) cin[16 + k] = out[1 + k];
  cin[31] = 0;
  double g1[kHid];
  for (int j = 0; j < kHid; ++j) {
    double a = 0;
    for (int k = 0; k < kCIn; ++k) a += wt(P, kOffCW1 + j * kCIn + k) * cin[k];
    g1[j] = a > 0 ? a : 0;
  }
  double lg[3] = {0, 0, 0};
  for (int j = 0; j < kHid; ++j) {
    double a = 0;
    for (int k = 0; k < kHid; ++k) a += wt(P, kOffCW2 + j * kHid + k) * g1[k];
    a = a > 0 ? a : 0;
    for (int c = 0; c < 3; ++c) lg[c] += wt(P, kOffCW3 + c * kHid + j) * a;
  }
  for (int c = 0; c < 3; ++c) rgb[c] = 1 / (1 + exp(-lg[c]));
}

// The FP32 forward's sample set (same t, positions and occupancy decisions),
// everything downstream in FP64.
__global__ void loss_f64_kernel(const TrainRay* __restrict__ rays, int n, const DevScene sc, ParamsF64 P,
                                double* __restrict__ loss_sum, double depth_w, double inv_n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const TrainRay r = rays[i];
  double C[3] = {0, 0, 0}, D = 0, T = 1;
  const float3 o = make_float3(r.ox, r.oy, r.oz), d = make_float3(r.dx, r.dy, r.dz);
  for (int s = 0; s < r.n; ++s) {
    const float t = fmaf((float)s + 0.5f, kDt, r.ts);
    const float3 x = sample_pos(o, d, t);
    if (!occupied(sc.occ, x)) continue;
    double sigma, c[3];
    query_f64(P, sc, x, d, sigma, c);
    const double alpha = -expm1(-sigma * (double)kDt);
    const double w = T * alpha;
    for (int a = 0; a < 3; ++a) C[a] += w * c[a];
    D += w * (double)t;
    T -= w;
    if (T < (double)kTStop) break;
  }
  const double e0 = C[0] - r.tr, e1 = C[1] - r.tg, e2 = C[2] - r.tb, ed = D - r.td;
  atomicAdd(loss_sum, (e0 * e0 + e1 * e1 + e2 * e2 + depth_w * ed * ed) * inv_n);
}

// The same loss for m perturbations at once (blockIdx.y = perturbation):
// a central-difference check of many parameters in one launch instead of one
// launch per evaluation (each evaluation alone fills one or two SMs).
struct PerturbF64 {
  int which;
  uint64_t index;
  double delta;
};

__global__ void loss_f64_batch_kernel(const TrainRay* __restrict__ rays, int n, const DevScene sc, const float* table,
                                      const float* w, const PerturbF64* __restrict__ pert,
                                      double* __restrict__ loss_sums, double depth_w, double inv_n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PerturbF64 q = pert[blockIdx.y];
  ParamsF64 P;
  P.table = table;
  P.w = w;
  P.which = q.which;
  P.index = q.index;
  P.delta = q.delta;
  const TrainRay r = rays[i];
  double C[3] = {0, 0, 0}, D = 0, T = 1;
  const float3 o = make_float3(r.ox, r.oy, r.oz), d = make_float3(r.dx, r.dy, r.dz);
  for (int s = 0; s < r.n; ++s) {
    const float t = fmaf((float)s + 0.5f, kDt, r.ts);
    const float3 x = sample_pos(o, d, t);
    if (!occupied(sc.occ, x)) continue;
    double sigma, c[3];
    query_f64(P, sc, x, d, sigma, c);
    const double alpha = -expm1(-sigma * (double)kDt);
    const double wgt = T * alpha;
    for (int a = 0; a < 3; ++a) C[a] += wgt * c[a];
    D += wgt * (double)t;
    T -= wgt;
    if (T < (double)kTStop) break;
  }
  const double e0 = C[0] - r.tr, e1 = C[1] - r.tg, e2 = C[2] - r.tb, ed = D - r.td;
  atomicAdd(loss_sums + blockIdx.y, (e0 * e0 + e1 * e1 + e2 * e2 + depth_w * ed * ed) * inv_n);
}

}  // namespace

struct nes_trainer {
  nes_ctx* ctx = nullptr;
  nes_train_config cfg{};
  cudaStream_t st = nullptr;
  TrainView* d_views = nullptr;
  int nviews = 0;
  const float* trgb = nullptr;
  const float* tdep = nullptr;
  uint32_t max_rays = 0;
  int2* d_pairs = nullptr;
  TrainRay* d_rays = nullptr;
  ScratchSample* d_scratch = nullptr;  // max_rays * kMaxSteps
  SampleRec* d_recs = nullptr;
  uint32_t rec_capacity = 0;
  uint32_t* d_ctr = nullptr;  // [0] record cursor, [1] error word, [2] sample-list cursor
  RayOut* d_rout = nullptr;
  double* d_loss = nullptr;
  float2* d_gtable = nullptr;
  float* d_gw = nullptr;
  float *d_mt = nullptr, *d_vt = nullptr, *d_mw = nullptr, *d_vw = nullptr;
  float* d_stage = nullptr;
  uint8_t* d_bimg = nullptr;  // TF32 weight images of backward_tc_kernel
  uint8_t* d_eimg = nullptr;  // high/low TF32 forward images of eval_tc_kernel
  uint32_t chunk = 0;
  int fwd_blocks = 0;  // persistent eval_kernel grid: SMs x resident blocks
  uint64_t steps = 0;
  uint64_t last_samples = 0;
  // Phase events on the trainer's stream: 0 forward start, 1 forward end,
  // 2 backward + weight-gradient end, 3 Adam start, 4 Adam end.
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  float phase_ms[3] = {0.0f, 0.0f, 0.0f};
};

namespace {

#define TR_CUDA(call)                      \
  do {                                     \
    cudaError_t e_ = (call);               \
    if (e_ != cudaSuccess) return NES_EIO; \
  } while (0)

constexpr int kSmemW = (int)sizeof(SmemWeights32);
constexpr int kSmemB = (int)sizeof(SmemBackward);

Staging staging(const nes_trainer* t) {
  Staging s;
  float* p = t->d_stage;
  const size_t S = t->chunk;
  s.enc = p; p += S * kEnc;
  s.h1 = p; p += S * kHid;
  s.cin = p; p += S * kCIn;
  s.g1 = p; p += S * kHid;
  s.g2 = p; p += S * kHid;
  s.dh1 = p; p += S * kHid;
  s.dout = p; p += S * kDOut;
  s.dg1 = p; p += S * kHid;
  s.dg2 = p; p += S * kHid;
  s.dlog = p;
  return s;
}

template <int IN, int OUT, int LDD>
cudaError_t launch_dw(const float* act, const float* delta, uint32_t S, float* dw, int num_sms, cudaStream_t st) {
  const uint32_t tiles = (S + kDwTile - 1) / kDwTile;
  const uint32_t want = 8u * (uint32_t)num_sms;  // 8 resident 256-thread blocks per SM
  dw_kernel<IN, OUT, LDD><<<tiles < want ? tiles : want, kDwThreads, 0, st>>>(act, delta, S, dw);
  return cudaGetLastError();
}

// Loss and gradients (accumulated into d_gtable / d_gw) for the n rays in d_rays.
int loss_and_grad(nes_trainer* t, int n, double* loss) {
  nes_ctx* c = t->ctx;
  TR_CUDA(cudaMemsetAsync(t->d_loss, 0, sizeof(double), t->st));
  TR_CUDA(cudaMemsetAsync(t->d_ctr, 0, sizeof(uint32_t), t->st));  // the error word is cleared by the caller
  TR_CUDA(cudaMemsetAsync(t->d_ctr + 2, 0, sizeof(uint32_t), t->st));
  TR_CUDA(cudaEventRecord(t->ev[0], t->st));
  // The sample list lives in the records' buffer until the adjoint (after
  // the composite) writes the records there.
  uint2* list = reinterpret_cast<uint2*>(t->d_recs);
  const uint32_t list_capacity = t->rec_capacity;  // SampleRec slots hold at least as many uint2
  enumerate_kernel<<<(n + 255) / 256, 256, 0, t->st>>>(t->d_rays, n, c->scene, list, list_capacity, t->d_rout,
                                                       t->d_ctr + 2, t->d_ctr + 1);
  TR_CUDA(cudaGetLastError());
  if (t->cfg.exact_weight_grads) {
    eval_kernel<<<t->fwd_blocks, kFwdThreads, kSmemW, t->st>>>(list, t->d_ctr + 2, list_capacity, t->d_rays, n,
                                                            c->scene, t->d_scratch);
  } else {  // this step's weights as high/low TF32 operand images
    pack_et_images_kernel<<<(kFwdImageBytes / 4 + 255) / 256, 256, 0, t->st>>>(c->d_weights, t->d_eimg);
    TR_CUDA(cudaGetLastError());
    eval_tc_kernel<<<c->num_sms, kEtThreads, kEtSmem, t->st>>>(list, t->d_ctr + 2, list_capacity, t->d_rays, n,
                                                             c->scene, t->d_eimg, t->d_scratch, t->d_ctr + 1);
  }
  TR_CUDA(cudaGetLastError());
  composite_kernel<<<(n + 255) / 256, 256, 0, t->st>>>(n, t->d_scratch, t->d_rout);
  TR_CUDA(cudaGetLastError());
  adjoint_kernel<<<(n + 255) / 256, 256, 0, t->st>>>(t->d_rays, t->d_rout, n, t->d_scratch, t->d_recs,
                                                     t->rec_capacity, t->d_ctr, t->d_ctr + 1, t->d_loss,
                                                     t->cfg.depth_weight, 1.0f / (float)n);
  TR_CUDA(cudaGetLastError());
  TR_CUDA(cudaEventRecord(t->ev[1], t->st));
  uint32_t h[2] = {0, 0};
  TR_CUDA(cudaMemcpyAsync(h, t->d_ctr, sizeof(h), cudaMemcpyDeviceToHost, t->st));
  TR_CUDA(cudaMemcpyAsync(loss, t->d_loss, sizeof(double), cudaMemcpyDeviceToHost, t->st));
  TR_CUDA(cudaStreamSynchronize(t->st));
  if (h[1] == kErrOverflow) return NES_ENOMEM;
  if (h[1] == kErrTimeout) return NES_ETIMEDOUT;
  if (h[1]) return NES_EINVAL;
  const uint32_t total = h[0];
  t->last_samples = total;
  const Staging sg = staging(t);
  float* gw = t->d_gw;
  const int sms = c->num_sms;
  if (!t->cfg.exact_weight_grads) {  // this step's weights as TF32 operand images
    pack_bt_images_kernel<<<(kBtImageBytes / 4 + 255) / 256, 256, 0, t->st>>>(c->d_weights, t->d_bimg);
    TR_CUDA(cudaGetLastError());
  }
  // BF16 staging (tensor-core mode) holds twice the records in the same bytes.
  const uint32_t chunk = t->cfg.exact_weight_grads ? t->chunk : 2u * t->chunk;
  for (uint32_t first = 0; first < total; first += chunk) {
    const uint32_t cnt = total - first < chunk ? total - first : chunk;
    if (t->cfg.exact_weight_grads) {
      backward_kernel<<<(cnt + kBwdThreads - 1) / kBwdThreads, kBwdThreads, kSmemB, t->st>>>(
          t->d_recs, first, cnt, t->d_rays, c->scene, sg, t->d_gtable);
    } else {
      const uint32_t groups = (cnt + 127u) / 128u;
      const uint32_t want = (groups + kBtGroups - 1) / kBtGroups;
      backward_tc_kernel<<<want < (uint32_t)sms ? want : (uint32_t)sms, kBtThreads, kBtSmem, t->st>>>(
          t->d_recs, first, cnt, t->d_rays, c->scene, t->d_bimg, sg, t->d_gtable, t->d_ctr + 1);
    }
    TR_CUDA(cudaGetLastError());
    if (t->cfg.exact_weight_grads) {
      TR_CUDA((launch_dw<kEnc, kHid, kHid>(sg.enc, sg.dh1, cnt, gw + kOffDW1, sms, t->st)));
      TR_CUDA((launch_dw<kHid, kDOut, kDOut>(sg.h1, sg.dout, cnt, gw + kOffDW2, sms, t->st)));
      TR_CUDA((launch_dw<kCIn, kHid, kHid>(sg.cin, sg.dg1, cnt, gw + kOffCW1, sms, t->st)));
      TR_CUDA((launch_dw<kHid, kHid, kHid>(sg.g1, sg.dg2, cnt, gw + kOffCW2, sms, t->st)));
      TR_CUDA((launch_dw<kHid, 3, kFDlog>(sg.g2, sg.dlog, cnt, gw + kOffCW3, sms, t->st)));
    } else {
      const uint32_t tiles = (cnt + 31) / 32;
      const uint32_t grid = tiles < (uint32_t)sms ? tiles : (uint32_t)sms;
      dw_tc_kernel<<<grid, kDwTcThreads, sizeof(DwTcSmem), t->st>>>(sg, tiles, gw, t->d_ctr + 1);
      TR_CUDA(cudaGetLastError());
    }
  }
  {  // a tensor-core wait that ran out reports through the error word
    uint32_t e = 0;
    TR_CUDA(cudaMemcpyAsync(&e, t->d_ctr + 1, sizeof(e), cudaMemcpyDeviceToHost, t->st));
    TR_CUDA(cudaStreamSynchronize(t->st));
    if (e == kErrTimeout) return NES_ETIMEDOUT;
    if (e) return NES_EINVAL;
  }
  TR_CUDA(cudaEventRecord(t->ev[2], t->st));
  return NES_OK;
}

int upload_rays(nes_trainer* t, const int32_t* rays, int n) {
  if (!rays || n < 1 || (uint32_t)n > t->max_rays || t->nviews == 0) return NES_EINVAL;
  TR_CUDA(cudaMemsetAsync(t->d_ctr + 1, 0, sizeof(uint32_t), t->st));
  TR_CUDA(cudaMemcpyAsync(t->d_pairs, rays, (size_t)n * sizeof(int2), cudaMemcpyHostToDevice, t->st));
  make_rays_kernel<<<(n + 255) / 256, 256, 0, t->st>>>(t->d_pairs, n, t->d_views, t->nviews, t->trgb, t->tdep,
                                                       t->d_rays, t->d_ctr + 1);
  TR_CUDA(cudaGetLastError());
  return NES_OK;
}

int adam(nes_trainer* t) {
  nes_ctx* c = t->ctx;
  t->steps++;
  const float b1 = t->cfg.beta1, b2 = t->cfg.beta2;
  const float bc1 = (float)(1.0 - std::pow((double)b1, (double)t->steps));
  const float bc2 = (float)(1.0 - std::pow((double)b2, (double)t->steps));
  const size_t nt = (size_t)kLevels * c->scene.T * 2;
  TR_CUDA(cudaEventRecord(t->ev[3], t->st));
  adam_kernel<<<4 * c->num_sms, 256, 0, t->st>>>(reinterpret_cast<float*>(c->d_table32),
                                                 reinterpret_cast<float*>(t->d_gtable), t->d_mt, t->d_vt, nt,
                                                 t->cfg.lr, b1, b2, t->cfg.eps, bc1, bc2);
  TR_CUDA(cudaGetLastError());
  adam_kernel<<<(kWeightFloats + 255) / 256, 256, 0, t->st>>>(c->d_weights, t->d_gw, t->d_mw, t->d_vw,
                                                              (size_t)kWeightFloats, t->cfg.lr, b1, b2, t->cfg.eps,
                                                              bc1, bc2);
  TR_CUDA(cudaGetLastError());
  TR_CUDA(cudaEventRecord(t->ev[4], t->st));
  TR_CUDA(cudaStreamSynchronize(t->st));
  TR_CUDA(cudaEventElapsedTime(&t->phase_ms[0], t->ev[0], t->ev[1]));
  TR_CUDA(cudaEventElapsedTime(&t->phase_ms[1], t->ev[1], t->ev[2]));
  TR_CUDA(cudaEventElapsedTime(&t->phase_ms[2], t->ev[3], t->ev[4]));
  return NES_OK;
}

void free_trainer(nes_trainer* t) {
  cudaFree(t->d_views);
  cudaFree(t->d_pairs);
  cudaFree(t->d_rays);
  cudaFree(t->d_scratch);
  cudaFree(t->d_recs);
  cudaFree(t->d_rout);
  cudaFree(t->d_ctr);
  cudaFree(t->d_loss);
  cudaFree(t->d_gtable);
  cudaFree(t->d_gw);
  cudaFree(t->d_mt);
  cudaFree(t->d_vt);
  cudaFree(t->d_mw);
  cudaFree(t->d_vw);
  cudaFree(t->d_stage);
  cudaFree(t->d_bimg);
  cudaFree(t->d_eimg);
  for (cudaEvent_t e : t->ev)
    if (e) cudaEventDestroy(e);
  if (t->st) cudaStreamDestroy(t->st);
  delete t;
}

}  // namespace

extern "C" {

void nes_train_config_default(nes_train_config* cfg) {
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->batch_rays = 1u << 18;
  cfg->lr = 1e-2f;
  cfg->beta1 = 0.9f;
  cfg->beta2 = 0.99f;
  cfg->eps = 1e-15f;
  cfg->depth_weight = 0.1f;
  cfg->exact_weight_grads = 0;
}

int nes_trainer_create(nes_ctx* ctx, const nes_train_config* cfg, nes_trainer** out) {
  if (!ctx || !cfg || !out) return NES_EINVAL;
  *out = nullptr;
  if (ctx->cfg.precision != NES_PREC_FP32) return NES_EINVAL;
  if (cfg->batch_rays == 0 || cfg->batch_rays > (1u << 20) || !(cfg->lr > 0.0f) || !(cfg->beta1 >= 0.0f) ||
      !(cfg->beta1 < 1.0f) || !(cfg->beta2 >= 0.0f) || !(cfg->beta2 < 1.0f) || !(cfg->eps >= 0.0f) ||
      !(cfg->depth_weight >= 0.0f))
    return NES_EINVAL;
  if (cudaSetDevice(ctx->cfg.device) != cudaSuccess) return NES_ENODEV;
  nes_trainer* t = new (std::nothrow) nes_trainer;
  if (!t) return NES_ENOMEM;
  t->ctx = ctx;
  t->cfg = *cfg;
  t->max_rays = cfg->batch_rays;
  auto fail = [&](int code) {
    free_trainer(t);
    return code;
  };
  if (cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking) != cudaSuccess) return fail(NES_EIO);
  for (cudaEvent_t& e : t->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(NES_EIO);
  const size_t nt = (size_t)kLevels * ctx->scene.T * 2;
  const size_t max_samples = (size_t)t->max_rays * kMaxSteps;  // every step of every ray: never overflows
  t->rec_capacity = (uint32_t)max_samples;
  t->chunk = 1u << 21;
  if (cudaMalloc(&t->d_pairs, (size_t)t->max_rays * sizeof(int2)) != cudaSuccess ||
      cudaMalloc(&t->d_rays, (size_t)t->max_rays * sizeof(TrainRay)) != cudaSuccess ||
      cudaMalloc(&t->d_scratch, max_samples * sizeof(ScratchSample)) != cudaSuccess ||
      cudaMalloc(&t->d_recs, max_samples * sizeof(SampleRec)) != cudaSuccess ||
      cudaMalloc(&t->d_rout, (size_t)t->max_rays * sizeof(RayOut)) != cudaSuccess ||
      cudaMalloc(&t->d_ctr, 4 * sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc(&t->d_loss, sizeof(double)) != cudaSuccess ||
      cudaMalloc(&t->d_gtable, nt * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&t->d_gw, kWeightFloats * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&t->d_mt, nt * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&t->d_vt, nt * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&t->d_mw, kWeightFloats * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&t->d_vw, kWeightFloats * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&t->d_stage, (size_t)t->chunk * kStageFloats * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&t->d_bimg, kBtImageBytes) != cudaSuccess ||
      cudaMalloc(&t->d_eimg, kEtImageBytes) != cudaSuccess)
    return fail(NES_ENOMEM);
  if (cudaMemset(t->d_gtable, 0, nt * sizeof(float)) != cudaSuccess ||
      cudaMemset(t->d_gw, 0, kWeightFloats * sizeof(float)) != cudaSuccess ||
      cudaMemset(t->d_mt, 0, nt * sizeof(float)) != cudaSuccess ||
      cudaMemset(t->d_vt, 0, nt * sizeof(float)) != cudaSuccess ||
      cudaMemset(t->d_mw, 0, kWeightFloats * sizeof(float)) != cudaSuccess ||
      cudaMemset(t->d_vw, 0, kWeightFloats * sizeof(float)) != cudaSuccess ||
      cudaMemset(t->d_ctr, 0, 4 * sizeof(uint32_t)) != cudaSuccess)
    return fail(NES_EIO);
  if (cudaFuncSetAttribute(eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemW) != cudaSuccess ||
      cudaFuncSetAttribute(backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemB) != cudaSuccess ||
      cudaFuncSetAttribute(dw_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(DwTcSmem)) !=
          cudaSuccess ||
      cudaFuncSetAttribute(backward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kBtSmem) != cudaSuccess ||
      cudaFuncSetAttribute(eval_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kEtSmem) != cudaSuccess)
    return fail(NES_EIO);
  {
    // backward_tc_kernel allocates all 512 TMEM columns: one CTA per SM,
    // which its register footprint (512 threads x > 64) guarantees.
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, backward_tc_kernel) != cudaSuccess || fa.numRegs <= 64) return fail(NES_EIO);
    // eval_tc_kernel too: two of its 256-thread CTAs must not fit an SM's
    // 65,536 registers.
    if (cudaFuncGetAttributes(&fa, eval_tc_kernel) != cudaSuccess || fa.numRegs * kEtThreads * 2 <= 65536)
      return fail(NES_EIO);
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, eval_kernel, kFwdThreads, kSmemW) != cudaSuccess)
    return fail(NES_EIO);
  t->fwd_blocks = ctx->num_sms * (per_sm < 1 ? 1 : per_sm);
  *out = t;
  return NES_OK;
}

void nes_trainer_destroy(nes_trainer* t) {
  if (!t) return;
  cudaSetDevice(t->ctx->cfg.device);
  cudaStreamSynchronize(t->st);
  free_trainer(t);
}

int nes_trainer_set_targets(nes_trainer* t, const nes_view* views, int nviews, const float* rgb_dev,
                            const float* depth_dev) {
  if (!t || !views || nviews < 1 || nviews > 1024 || !rgb_dev || !depth_dev) return NES_EINVAL;
  std::lock_guard<std::mutex> lk(t->ctx->mu);  // no render of the context meanwhile
  TR_CUDA(cudaSetDevice(t->ctx->cfg.device));
  std::vector<TrainView> hv(nviews);
  uint64_t off = 0;
  for (int i = 0; i < nviews; ++i) {
    const uint64_t px = (uint64_t)views[i].width * views[i].height;
    if (!view_ok(views[i])) return NES_EINVAL;  // the renderer's own view check
    std::memcpy(hv[i].M, views[i].matrix, sizeof(hv[i].M));
    hv[i].W = (int)views[i].width;
    hv[i].H = (int)views[i].height;
    hv[i].focal = views[i].focal_px;
    hv[i].pad = 0;
    hv[i].offset = off;
    off += px;
  }
  TrainView* dv = nullptr;
  TR_CUDA(cudaMalloc(&dv, nviews * sizeof(TrainView)));
  if (cudaMemcpy(dv, hv.data(), nviews * sizeof(TrainView), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(dv);
    return NES_EIO;
  }
  cudaFree(t->d_views);
  t->d_views = dv;
  t->nviews = nviews;
  t->trgb = rgb_dev;
  t->tdep = depth_dev;
  return NES_OK;
}

int nes_trainer_step(nes_trainer* t, uint64_t seed, double* loss) {
  if (!t || !loss || t->nviews == 0) return NES_EINVAL;
  std::lock_guard<std::mutex> lk(t->ctx->mu);  // no render of the context meanwhile
  TR_CUDA(cudaSetDevice(t->ctx->cfg.device));
  const int n = (int)t->cfg.batch_rays;
  TR_CUDA(cudaMemsetAsync(t->d_ctr + 1, 0, sizeof(uint32_t), t->st));
  sample_pairs_kernel<<<(n + 255) / 256, 256, 0, t->st>>>(seed, n, t->d_views, t->nviews, t->d_pairs);
  TR_CUDA(cudaGetLastError());
  make_rays_kernel<<<(n + 255) / 256, 256, 0, t->st>>>(t->d_pairs, n, t->d_views, t->nviews, t->trgb, t->tdep,
                                                       t->d_rays, t->d_ctr + 1);
  TR_CUDA(cudaGetLastError());
  const int rc = loss_and_grad(t, n, loss);
  if (rc != NES_OK) return rc;
  return adam(t);
}

int nes_trainer_step_rays(nes_trainer* t, const int32_t* rays, int n, double* loss) {
  if (!t || !loss) return NES_EINVAL;
  std::lock_guard<std::mutex> lk(t->ctx->mu);  // no render of the context meanwhile
  TR_CUDA(cudaSetDevice(t->ctx->cfg.device));
  int rc = upload_rays(t, rays, n);
  if (rc != NES_OK) return rc;
  if ((rc = loss_and_grad(t, n, loss)) != NES_OK) return rc;
  return adam(t);
}

int nes_trainer_grad(nes_trainer* t, const int32_t* rays, int n, double* loss, float* grad_table,
                     float* grad_weights) {
  if (!t || !loss) return NES_EINVAL;
  std::lock_guard<std::mutex> lk(t->ctx->mu);  // no render of the context meanwhile
  TR_CUDA(cudaSetDevice(t->ctx->cfg.device));
  int rc = upload_rays(t, rays, n);
  if (rc == NES_OK) rc = loss_and_grad(t, n, loss);
  const size_t nt = (size_t)kLevels * t->ctx->scene.T * 2;
  if (rc == NES_OK && grad_table)
    TR_CUDA(cudaMemcpyAsync(grad_table, t->d_gtable, nt * sizeof(float), cudaMemcpyDeviceToHost, t->st));
  if (rc == NES_OK && grad_weights)
    TR_CUDA(cudaMemcpyAsync(grad_weights, t->d_gw, kWeightFloats * sizeof(float), cudaMemcpyDeviceToHost, t->st));
  TR_CUDA(cudaMemsetAsync(t->d_gtable, 0, nt * sizeof(float), t->st));
  TR_CUDA(cudaMemsetAsync(t->d_gw, 0, kWeightFloats * sizeof(float), t->st));
  TR_CUDA(cudaStreamSynchronize(t->st));
  return rc;
}

int nes_trainer_loss_fp64(nes_trainer* t, const int32_t* rays, int n, int which, uint64_t index, double delta,
                          double* loss) {
  if (!t || !loss || (which != 0 && which != 1)) return NES_EINVAL;
  const uint64_t limit = which == 0 ? (uint64_t)kLevels * t->ctx->scene.T * 2 : (uint64_t)kWeightFloats;
  if (index >= limit) return NES_EINVAL;
  std::lock_guard<std::mutex> lk(t->ctx->mu);  // no render of the context meanwhile
  TR_CUDA(cudaSetDevice(t->ctx->cfg.device));
  int rc = upload_rays(t, rays, n);
  if (rc != NES_OK) return rc;
  ParamsF64 P;
  P.table = reinterpret_cast<const float*>(t->ctx->d_table32);
  P.w = t->ctx->d_weights;
  P.which = which;
  P.index = index;
  P.delta = delta;
  TR_CUDA(cudaMemsetAsync(t->d_loss, 0, sizeof(double), t->st));
  loss_f64_kernel<<<(n + 63) / 64, 64, 0, t->st>>>(t->d_rays, n, t->ctx->scene, P, t->d_loss,
                                                   (double)t->cfg.depth_weight, 1.0 / (double)n);
  TR_CUDA(cudaGetLastError());
  uint32_t err = 0;
  TR_CUDA(cudaMemcpyAsync(&err, t->d_ctr + 1, sizeof(err), cudaMemcpyDeviceToHost, t->st));
  TR_CUDA(cudaMemcpyAsync(loss, t->d_loss, sizeof(double), cudaMemcpyDeviceToHost, t->st));
  TR_CUDA(cudaStreamSynchronize(t->st));
  return err ? NES_EINVAL : NES_OK;
}

int nes_trainer_loss_fp64_batch(nes_trainer* t, const int32_t* rays, int n, int m, const int32_t* which,
                                const uint64_t* index, const double* delta, double* losses) {
  if (!t || !which || !index || !delta || !losses || m < 1 || m > 65535) return NES_EINVAL;
  const uint64_t limits[2] = {(uint64_t)kLevels * t->ctx->scene.T * 2, (uint64_t)kWeightFloats};
  std::vector<PerturbF64> host((size_t)m);
  for (int j = 0; j < m; ++j) {
    if (which[j] != 0 && which[j] != 1) return NES_EINVAL;
    if (index[j] >= limits[which[j]]) return NES_EINVAL;
    host[j] = PerturbF64{which[j], index[j], delta[j]};
  }
  std::lock_guard<std::mutex> lk(t->ctx->mu);  // no render of the context meanwhile
  TR_CUDA(cudaSetDevice(t->ctx->cfg.device));
  int rc = upload_rays(t, rays, n);
  if (rc != NES_OK) return rc;
  PerturbF64* d_pert = nullptr;
  double* d_loss = nullptr;
  if (cudaMalloc(&d_pert, sizeof(PerturbF64) * (size_t)m) != cudaSuccess) return NES_ENOMEM;
  if (cudaMalloc(&d_loss, sizeof(double) * (size_t)m) != cudaSuccess) {
    cudaFree(d_pert);
    return NES_ENOMEM;
  }
  cudaError_t e = cudaMemcpyAsync(d_pert, host.data(), sizeof(PerturbF64) * (size_t)m, cudaMemcpyHostToDevice, t->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_loss, 0, sizeof(double) * (size_t)m, t->st);
  if (e == cudaSuccess) {
    loss_f64_batch_kernel<<<dim3((n + 63) / 64, m), 64, 0, t->st>>>(
        t->d_rays, n, t->ctx->scene, reinterpret_cast<const float*>(t->ctx->d_table32), t->ctx->d_weights, d_pert,
        d_loss, (double)t->cfg.depth_weight, 1.0 / (double)n);
    e = cudaGetLastError();
  }
  uint32_t err = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, t->d_ctr + 1, sizeof(err), cudaMemcpyDeviceToHost, t->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(losses, d_loss, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost, t->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(t->st);
  cudaFree(d_pert);
  cudaFree(d_loss);
  if (e != cudaSuccess) return NES_EIO;
  return err ? NES_EINVAL : NES_OK;
}

uint64_t nes_trainer_last_samples(const nes_trainer* t) { return t ? t->last_samples : 0; }

int nes_trainer_last_timings(const nes_trainer* t, float* forward_ms, float* backward_ms, float* adam_ms) {
  if (!t || !forward_ms || !backward_ms || !adam_ms) return NES_EINVAL;
  if (t->steps == 0) return NES_EAGAIN;
  *forward_ms = t->phase_ms[0];
  *backward_ms = t->phase_ms[1];
  *adam_ms = t->phase_ms[2];
  return NES_OK;
}

}  // extern "C"
