// march_tc.cu -- FP16 tensor-core march: the renderer's density and colour
// MLPs (the external instant-ngp-renderer neserver calls over TCP,
// src/server.cpp:161-194) evaluated with tcgen05 MMAs whose activations never
// leave tensor memory, overlapped with the hash-grid gathers by warp
// specialisation.
//
// Why this shape: the march is bound by its hash-table gathers through the
// L1 data pipe (per sample 16 levels x 8 corners: the recorded levels as one
// 32-byte per-cell record, the others as eight scattered 4-byte gathers), and
// their speed depends on the L1 cache (a 28 KiB L1 made them ~2.5x slower
// than a 192 KiB one).  So shared memory holds only
// the MLP weights (the B operands, 20 KiB) and small per-row hand-off arrays,
// within the 32 KiB configuration; every A operand (encoded features, hidden
// layers, colour input) lives in TMEM and feeds tcgen05.mma directly.
//
// One CTA per SM: 4 groups x (4 ENCODER warps + 4 MLP warps) = 1024 threads.
//  - ENCODER thread = one ray slot.  Per tile it claims rays (a warp-wide
//    chunk of 32 at a time), encodes its slot's next occupied sample from the
//    FP16 table, writes the 32 FP16 features as its TMEM lane of the tile (16
//    columns), hands the row's ray id, flags and t over in shared memory and
//    marks the tile full.  It never waits for results: only for
//    its tile buffer to be free again (two buffers), which the MLP side
//    releases once its first layer is done and every row's hand-off has been
//    read.  Encoder warps run independently.
//  - MLP thread = TMEM lane = tile row.  One thread issues each layer
//    (32->64, 64->16, 32->64, 64->64, 64->16 [3 used]) as tcgen05.mma
//    kind::f16 with A from TMEM and B from shared memory, FP32 accumulators in
//    TMEM; between layers every thread loads its lane, applies ReLU / exp and
//    stores the next FP16 A operand back to TMEM.  The same thread then
//    composites its row's sample into the row's ray (FP32 transmittance,
//    colour, depth): a row's samples arrive in order, so each ray is
//    composited by one thread with one state.
//  - Early termination (T < 1e-4) is noticed by the MLP thread, which writes
//    the ray and tells the row's encoder to move on; samples the encoder
//    produced meanwhile are dropped.
// TMEM (512 columns): group g encoder tiles at 32g (+16 for the second
// buffer), MLP hidden activations at 128+96g (32 columns of packed FP16;
// also the colour input), accumulator after them (64 FP32 columns).  Two CTAs
// cannot share an SM: 1024 threads x >32 registers fill the register file,
// and the launcher checks it.
#include <cuda_fp16.h>

#include "kernels.h"
#include "tc_ptx.cuh"

namespace nes {

namespace {

constexpr int kGroups = 4;
constexpr int kRoleThreads = 128;  // encoder threads = MLP threads = tile rows
constexpr int kGroupThreads = 2 * kRoleThreads;
constexpr int kTcThreads = kGroups * kGroupThreads;  // 1024
constexpr uint32_t kLaunchRegs = 64, kEncRegs = 80, kMlpRegs = 48;
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kEncColsPerGroup = 32;  // two 16-column tile buffers
constexpr uint32_t kMlpBase = kGroups * kEncColsPerGroup;
constexpr uint32_t kMlpColsPerGroup = 96;  // 64 accumulator + 32 hidden activations
static_assert(kMlpBase + kGroups * kMlpColsPerGroup <= kTmemCols, "TMEM column budget");

// Weight image (bytes) in operand layout: [N][K] K-major, core matrices 8x16B.
constexpr int kWoffDW1 = 0;      // N=64, K=32
constexpr int kWoffDW2 = 4096;   // N=16, K=64
constexpr int kWoffCW1 = 6144;   // N=64, K=32
constexpr int kWoffCW2 = 10240;  // N=64, K=64
constexpr int kWoffCW3 = 18432;  // N=16 (rows 3..15 zero), K=64
constexpr int kWBytes = 20480;

// Per-group shared memory: the per-row hand-off of both tile buffers (ray id
// with the flags in its top bits, and t), per-warp "out of rays" flags,
// early-termination notices, the group's stop flag and mbarriers.  The whole
// CTA stays within the 32 KiB shared-memory configuration, which leaves the
// rest of the SM's 256 KiB as L1 for the hash-table gathers.
constexpr int kGOffHand = 0;                          // [2][128] uint2 (id | flags << 28, t)
constexpr int kGOffFin = kGOffHand + 2 * 128 * 8;     // [2][4] uint32
constexpr int kGOffTerm = kGOffFin + 32;              // [128] uint32
constexpr int kGOffDone = kGOffTerm + 128 * 4;        // uint32
constexpr int kGOffBar = (kGOffDone + 4 + 7) / 8 * 8; // full0, full1, free0, free1, mma
constexpr int kGroupBytes = (kGOffBar + 5 * 8 + 127) / 128 * 128;

constexpr int kOffW = 0;
constexpr int kOffGroups = kOffW + kWBytes;
constexpr int kOffBarW = kOffGroups + kGroups * kGroupBytes;
constexpr int kOffSlot = kOffBarW + 8;
constexpr int kSmemUsed = kOffSlot + 8;
constexpr int kSmemAlign = 128;  // operand images need 16 B, mbarriers 8 B
constexpr int kSmemRequest = kSmemUsed + kSmemAlign;
// 1 KiB of each CTA's shared memory is reserved by the system.
static_assert(kSmemRequest + 1024 <= 32 * 1024, "shared memory above the 32 KiB configuration");
constexpr uint32_t kIdMask = (1u << 28) - 1u;  // ray ids < 2^27 (max_pixels bound)

// Byte offset of 16-byte chunk c (K elements 8c..8c+7) of row n in a
// K-major shared-memory operand with K columns (core matrices 8 rows x 16 B,
// K-chunks adjacent: LBO = 128 B, 8-row groups K*16 B apart: SBO).
__host__ __device__ constexpr int op_chunk(int n, int c, int K) { return (n >> 3) * (K * 16) + c * 128 + (n & 7) * 16; }

__device__ __forceinline__ uint32_t h2u(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }
__device__ __forceinline__ uint32_t pk(float a, float b) { return h2u(__floats2half2_rn(a, b)); }
// max(a, 0), max(b, 0) -> packed FP16 (a in the low half), one instruction.
__device__ __forceinline__ uint32_t pk_relu(float a, float b) {
  uint32_t r;
  asm("cvt.rn.relu.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
  return r;
}

// Trilinear interpolation of 8 FP16 corner entries (corner c = dx + 2 dy +
// 4 dz) as three rounds of packed FP16 lerps, a + f (b - a): four along x,
// two along y, one along z, both features at once (HSUB2 + HFMA2 per lerp,
// 14 instructions).  The fractions are rounded to FP16 and every step rounds
// to FP16 (|values| <= 0.5: ~2.4e-4 per rounding, the size of the table's
// own FP16 rounding); measured against the FP64 oracle the render's PSNR is
// unchanged (114.6 dB) and the march 7 % faster than the weighted-sum form.
__device__ __forceinline__ uint32_t interp_lerp(const __half2 (&e)[8], float fx, float fy, float fz) {
  const __half2 hx = __float2half2_rn(fx), hy = __float2half2_rn(fy), hz = __float2half2_rn(fz);
  const __half2 a0 = __hfma2(hx, __hsub2(e[1], e[0]), e[0]);
  const __half2 a1 = __hfma2(hx, __hsub2(e[3], e[2]), e[2]);
  const __half2 a2 = __hfma2(hx, __hsub2(e[5], e[4]), e[4]);
  const __half2 a3 = __hfma2(hx, __hsub2(e[7], e[6]), e[6]);
  const __half2 b0 = __hfma2(hy, __hsub2(a1, a0), a0);
  const __half2 b1 = __hfma2(hy, __hsub2(a3, a2), a2);
  return h2u(__hfma2(hz, __hsub2(b1, b0), b0));
}

// Level L of the FP16 table at x -> its two features packed as FP16.
// Instruction-lean form of the trilinear interpolation (the march is
// issue-bound here): integer floor/clamp for the cell, hash terms masked
// once so each corner index is one 3-input XOR, and the interpolation as
// packed FP16 lerps (interp_lerp).
// The recorded levels (0..kRec-1) also exist as per-cell records: the 8 corner
// entries of every cell (c = dx + 2 dy + 4 dz) in 32 contiguous bytes, so a
// sample's level costs two 16-byte loads instead of eight scattered 4-byte
// gathers (the encoder is bound by L1 wavefronts).  The records are copies of
// table entries (built by build_records_kernel), so the result is the same.
// Records of levels kEvictFirstFrom and up are read once per sample and come
// from HBM (cells smaller than a sample step): they are loaded with an L2
// evict-first policy so that they do not displace the table and the coarser
// records, which are reused (1080p march 24.2 -> 23.6 ms; from level 7 up: no
// gain, those records are still reused).
constexpr int kEvictFirstFrom = 10;

__device__ __forceinline__ uint4 ldg_evict_first(const uint4* p, uint64_t policy) {
  uint4 r;
  asm("ld.global.nc.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
      : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
      : "l"(p), "l"(policy));
  return r;
}

template <int L>
__device__ __forceinline__ uint32_t encode_level_rec(const uint4* __restrict__ rec, const float3& x) {
  constexpr int N = level_res(L);
  const float px = x.x * (float)N, py = x.y * (float)N, pz = x.z * (float)N;
  const int ix = min(__float2int_rd(px), N - 1), iy = min(__float2int_rd(py), N - 1),
            iz = min(__float2int_rd(pz), N - 1);
  const float fx = px - (float)ix, fy = py - (float)iy, fz = pz - (float)iz;
  const uint32_t cell = rec_cell_offset(L) + (uint32_t)ix + (uint32_t)N * ((uint32_t)iy + (uint32_t)N * (uint32_t)iz);
  uint4 a, b;
  if constexpr (L >= kEvictFirstFrom) {
    uint64_t policy;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
    a = ldg_evict_first(rec + 2 * cell, policy);
    b = ldg_evict_first(rec + 2 * cell + 1, policy);
  } else {
    a = __ldg(rec + 2 * cell);
    b = __ldg(rec + 2 * cell + 1);
  }
  __half2 e[8];
  e[0] = *reinterpret_cast<const __half2*>(&a.x);
  e[1] = *reinterpret_cast<const __half2*>(&a.y);
  e[2] = *reinterpret_cast<const __half2*>(&a.z);
  e[3] = *reinterpret_cast<const __half2*>(&a.w);
  e[4] = *reinterpret_cast<const __half2*>(&b.x);
  e[5] = *reinterpret_cast<const __half2*>(&b.y);
  e[6] = *reinterpret_cast<const __half2*>(&b.z);
  e[7] = *reinterpret_cast<const __half2*>(&b.w);
  return interp_lerp(e, fx, fy, fz);
}

template <int L>
__device__ __forceinline__ uint32_t encode_level(const __half2* __restrict__ table, uint32_t T, uint32_t dense_mask,
                                                 const float3& x) {
  constexpr int N = level_res(L);
  const float px = x.x * (float)N, py = x.y * (float)N, pz = x.z * (float)N;
  const int ix = min(__float2int_rd(px), N - 1), iy = min(__float2int_rd(py), N - 1),
            iz = min(__float2int_rd(pz), N - 1);  // x >= 0, so the floor is >= 0
  const float fx = px - (float)ix, fy = py - (float)iy, fz = pz - (float)iz;
  uint32_t idx[8];
  if ((dense_mask >> L) & 1u) {
    constexpr uint32_t s = (uint32_t)N + 1u;
    const uint32_t b = (uint32_t)ix + s * ((uint32_t)iy + s * (uint32_t)iz);
#pragma unroll
    for (int k = 0; k < 8; ++k) idx[k] = b + (k & 1) + ((k >> 1) & 1) * s + ((k >> 2) & 1) * s * s;
  } else {
    const uint32_t m = T - 1u;
    const uint32_t x0 = (uint32_t)ix & m, x1 = (uint32_t)(ix + 1) & m;
    const uint32_t y0 = ((uint32_t)iy * kPrime1) & m, y1 = ((uint32_t)iy * kPrime1 + kPrime1) & m;
    const uint32_t z0 = ((uint32_t)iz * kPrime2) & m, z1 = ((uint32_t)iz * kPrime2 + kPrime2) & m;
#pragma unroll
    for (int k = 0; k < 8; ++k) idx[k] = ((k & 1) ? x1 : x0) ^ ((k & 2) ? y1 : y0) ^ ((k & 4) ? z1 : z0);
  }
  const __half2* tab = table + (size_t)L * T;
  __half2 e[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) e[k] = __ldg(tab + idx[k]);
  return interp_lerp(e, fx, fy, fz);
}

// All 16 levels -> TMEM columns 0..15 of this lane (no wait).  Every level
// is computed before the first TMEM store: the stores are compiler
// barriers, so storing per 4 levels would serialise four rounds of
// gathers per sample.
template <int L, int kRec>
__device__ __forceinline__ uint32_t encode_level_any(const __half2* __restrict__ table, const uint4* __restrict__ rec,
                                                     uint32_t T, uint32_t dense_mask, const float3& x) {
  if constexpr (L < kRec) return encode_level_rec<L>(rec, x);
  else return encode_level<L>(table, T, dense_mask, x);
}

template <int kRec>
__device__ __forceinline__ void encode_all(const __half2* __restrict__ table, const uint4* __restrict__ rec,
                                           uint32_t T, uint32_t dense_mask, const float3& x, bool has,
                                           uint32_t taddr) {
  static_assert(kRec >= 10 && kRec <= 13, "records cover levels 0..9 at least, 0..12 at most");
  uint32_t f[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) f[k] = 0u;
  if (has) {
    f[0] = encode_level_any<0, kRec>(table, rec, T, dense_mask, x);
    f[1] = encode_level_any<1, kRec>(table, rec, T, dense_mask, x);
    f[2] = encode_level_any<2, kRec>(table, rec, T, dense_mask, x);
    f[3] = encode_level_any<3, kRec>(table, rec, T, dense_mask, x);
    f[4] = encode_level_any<4, kRec>(table, rec, T, dense_mask, x);
    f[5] = encode_level_any<5, kRec>(table, rec, T, dense_mask, x);
    f[6] = encode_level_any<6, kRec>(table, rec, T, dense_mask, x);
    f[7] = encode_level_any<7, kRec>(table, rec, T, dense_mask, x);
    f[8] = encode_level_any<8, kRec>(table, rec, T, dense_mask, x);
    f[9] = encode_level_any<9, kRec>(table, rec, T, dense_mask, x);
    f[10] = encode_level_any<10, kRec>(table, rec, T, dense_mask, x);
    f[11] = encode_level_any<11, kRec>(table, rec, T, dense_mask, x);
    f[12] = encode_level_any<12, kRec>(table, rec, T, dense_mask, x);
    f[13] = encode_level_any<13, kRec>(table, rec, T, dense_mask, x);
    f[14] = encode_level_any<14, kRec>(table, rec, T, dense_mask, x);
    f[15] = encode_level_any<15, kRec>(table, rec, T, dense_mask, x);
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) tc::tmem_st4(taddr + 4 * c, f[4 * c], f[4 * c + 1], f[4 * c + 2], f[4 * c + 3]);
}

// D[128 x N] = A[128 x K] (TMEM) * B[N x K]^T (shared), K in steps of 16
// (8 TMEM columns of packed FP16 per step).
__device__ __forceinline__ void mma_layer(uint32_t d_tmem, uint32_t a_tmem, uint32_t b, int K, uint32_t idesc) {
  for (int j = 0; j < K / 16; ++j)
    tc::mma_f16_at(d_tmem, a_tmem + j * 8, tc::sdesc(b + j * 256, 128, K * 16), idesc, j > 0 ? 1u : 0u);
}

// 64 accumulator columns -> ReLU -> FP16 -> 32 hidden-activation columns in
// two 32-column rounds; the stores are not waited for here (the caller's
// sync waits once for all of them).
__device__ __forceinline__ void relu_to_h(uint32_t d_row, uint32_t h_row) {
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float v[32];
    tc::tmem_ld32(d_row + 32 * half, v);
    uint32_t w[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) w[k] = pk_relu(v[2 * k], v[2 * k + 1]);
    tc::tmem_st16_nowait(h_row + 16 * half, w);
  }
}

__device__ __forceinline__ void write_ray(const ViewBatch& vb, const DevScratch& s, uint32_t id, float cr, float cg,
                                          float cb, float dep) {
  const RayMeta m = s.ray_meta[id];
  const DevView& V = vb.v[m.view];
  if (V.rgb) {
    V.rgb[(size_t)m.pixel * 3 + 0] = cr;
    V.rgb[(size_t)m.pixel * 3 + 1] = cg;
    V.rgb[(size_t)m.pixel * 3 + 2] = cb;
  }
  if (V.depth) V.depth[m.pixel] = dep;
}

// Per-row hand-off flags of a tile (with the ray id, encoder -> MLP).
constexpr uint32_t kTagSample = 1u, kTagFirst = 2u, kTagLast = 4u;

// Encoder-side state of one ray slot.
struct Slot {
  bool live = false;
  bool first = false;
  float3 o, d;
  float ts = 0.0f;
  int n = 0, ei = 0;
  uint32_t id = 0;
};

__device__ __forceinline__ void skip_empty(const DevScene& sc, Slot& q) {
  while (q.ei < q.n && !occupied(sc.occ, sample_pos(q.o, q.d, fmaf((float)q.ei + 0.5f, kDt, q.ts)))) ++q.ei;
}

template <class Src, int kRec>
__global__ void __launch_bounds__(kTcThreads, 1)
march_tc_kernel(const __grid_constant__ Src src, const DevScene sc, const DevScratch s) {
  const ViewBatch& vb = src.get();
  extern __shared__ __align__(128) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + kSmemAlign - 1) &
                                             ~uintptr_t(kSmemAlign - 1));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = tid / kGroupThreads;
  const bool is_mlp = (tid % kGroupThreads) >= kRoleThreads;
  const int row = tid % kRoleThreads;  // tile row = TMEM lane
  uint8_t* G = smem + kOffGroups + g * kGroupBytes;
  uint64_t* bar = reinterpret_cast<uint64_t*>(G + kGOffBar);  // full0, full1, free0, free1, mma
  uint2* hand = reinterpret_cast<uint2*>(G + kGOffHand);      // [2][128] (id | flags << 28, t)
  uint32_t* wfin = reinterpret_cast<uint32_t*>(G + kGOffFin); // [2][4] encoder warp finished
  uint32_t* term = reinterpret_cast<uint32_t*>(G + kGOffTerm);  // [128] early-terminated ray id + 1
  volatile uint32_t* gdone = reinterpret_cast<volatile uint32_t*>(G + kGOffDone);
  uint64_t* bar_w = reinterpret_cast<uint64_t*>(smem + kOffBarW);
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + kOffSlot);
  const uint32_t mlp_bar = 1 + g;

  if (tid == 0) {
    tc::mbar_init(bar_w, 1);
    for (int k = 0; k < kGroups; ++k) {
      uint8_t* Gk = smem + kOffGroups + k * kGroupBytes;
      uint64_t* b = reinterpret_cast<uint64_t*>(Gk + kGOffBar);
      tc::mbar_init(b + 0, kRoleThreads);  // full: every encoder thread arrives
      tc::mbar_init(b + 1, kRoleThreads);
      tc::mbar_init(b + 2, 1);             // free: MLP row 0 arrives after layer 1 (or at the stop)
      tc::mbar_init(b + 3, 1);
      tc::mbar_init(b + 4, 1);             // mma: commit of each layer
      *reinterpret_cast<uint32_t*>(Gk + kGOffDone) = 0u;
    }
    tc::fence_mbar_init();
  }
  if (!is_mlp) term[row] = 0u;
  if (warp == 0) {
    tc::tmem_alloc(slot, kTmemCols);
    tc::tmem_relinquish();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = *slot;
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;  // this warp's TMEM lane quarter
  const uint32_t enc_cols = tmem + g * kEncColsPerGroup;        // + 16 * buffer
  bool fail = false;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(bar_w, kWBytes);
    tc::bulk_g2s(smem + kOffW, sc.tc_weights, kWBytes, bar_w);
    fail = !tc::mbar_wait(bar_w, 0);
  }
  fail = __syncthreads_or(fail);

  // Registers move from the MLP warpgroups to the gather-bound encoders:
  // 512 x kEncRegs + 512 x kMlpRegs = 1024 x 64, the launch allocation
  // (the launcher checks the kernel was built with exactly 64).
  static_assert(kGroups * kRoleThreads * (kEncRegs + kMlpRegs) == kTcThreads * kLaunchRegs, "register split");

  unsigned long long my_samples = 0;
  if (!fail && is_mlp) {
    // ======================= MLP warps =======================
    // One thread per tile row: it evaluates the row's sample through the
    // five layers and composites it into the row's current ray, so a ray's
    // samples are composited in order by one thread with one state.
    tc::regs_dec<kMlpRegs>();
    const uint32_t sW = tc::smem_addr(smem + kOffW);
    const uint32_t h_col = tmem + kMlpBase + g * kMlpColsPerGroup;  // hidden activations (lane 0)
    const uint32_t d_col = h_col + 32;                              // accumulator (lane 0)
    const uint32_t d_row = d_col + lane_off, h_row = h_col + lane_off;
    constexpr uint32_t id64 = tc::idesc_f16_f32(128, 64), id16 = tc::idesc_f16_f32(128, 16);
    uint32_t pm = 0;
    uint32_t cur = 0xFFFFFFFFu;  // ray being composited in this row (none)
    float T = 1.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f, cz = 0.0f;
    float dx = 0.0f, dy = 0.0f, dz = 1.0f;  // direction of the row's current ray

    // Issues one layer (one thread) and waits for it (every thread); the
    // free barrier of the tile's buffer, if given, is released by the same
    // completion.  A failed wait is reported at the next sync().
    bool ok = true;
    auto layer = [&](uint32_t a_tmem, uint32_t b_off, int K, uint32_t idesc, uint64_t* also) {
      if (row == 0) {
        tc::fence_after();
        mma_layer(d_col, a_tmem, sW + b_off, K, idesc);
        tc::mma_commit(bar + 4);
        if (also) tc::mma_commit(also);
      }
      ok = tc::mbar_wait(bar + 4, pm) && ok;
      pm ^= 1u;
      tc::fence_after();
    };
    // This thread's TMEM writes -> visible to the next MMA; true when any
    // MLP thread of the group saw a wait fail (all of them then stop
    // together, so no thread is left at a named barrier).
    auto sync_bad = [&]() -> bool {
      tc::tmem_wait_st();
      tc::fence_before();
      return tc::named_sync_or(mlp_bar, kRoleThreads, !ok);
    };

    for (uint32_t k = 0;; ++k) {
      const int b = (int)(k & 1u);
      // Only row 0 waits for the tile; the barrier hands its outcome to the
      // others.  (Were every thread to poll, one that fell two phases behind
      // would wait for a phase that had already come round.)
      if (row == 0) ok = tc::mbar_wait_sleep(bar + b, (k >> 1) & 1u);
      if (sync_bad()) { fail = true; break; }
      tc::fence_after();
      if (wfin[b * 4 + 0] & wfin[b * 4 + 1] & wfin[b * 4 + 2] & wfin[b * 4 + 3]) {
        // Every encoder warp of the group is out of rays: release the
        // encoders that wait for this buffer and stop.
        if (row == 0) {
          *gdone = 1u;
          tc::mbar_arrive(bar + 2 + b);
        }
        break;
      }
      const uint2 hd = hand[b * 128 + row];
      const uint32_t rid = hd.x & kIdMask, flags = hd.x >> 28;
      const float t = __uint_as_float(hd.y);
      if (flags & kTagFirst) {  // a new ray in this row: its direction, for the colour MLP
        const float4 rd = s.ray_dt[rid];
        dx = rd.x;
        dy = rd.y;
        dz = rd.z;
      }
      const uint32_t a_col = enc_cols + 16 * b;  // encoded features of this tile
      // density 32 -> 64 -> 16 (the first layer is the features' last reader)
      layer(a_col, kWoffDW1, 32, id64, nullptr);
      relu_to_h(d_row, h_row);
      if (sync_bad()) { fail = true; break; }
      // The tile buffer goes back to the encoders once its features have
      // been read (the first layer is complete) and every row's hand-off
      // entry has been read (the barrier above).
      if (row == 0) tc::mbar_arrive(bar + 2 + b);
      layer(h_col, kWoffDW2, 64, id16, nullptr);
      float sigma;
      {
        // colour input [SH16(d) | density outputs 1..15 | 0] -> h (layer 2
        // is done with h)
        float v[16];
        tc::tmem_ld16(d_row, v);
        sigma = expf(v[0] - 1.0f);
        uint32_t w[8];
#pragma unroll
        for (int j = 0; j < 7; ++j) w[j] = pk(v[1 + 2 * j], v[2 + 2 * j]);
        w[7] = pk(v[15], 0.0f);
        tc::tmem_st8_nowait(h_row + 8, w);
        float sh[16];
        sh16(make_float3(dx, dy, dz), sh);
#pragma unroll
        for (int j = 0; j < 8; ++j) w[j] = pk(sh[2 * j], sh[2 * j + 1]);
        tc::tmem_st8_nowait(h_row, w);
      }
      if (sync_bad()) { fail = true; break; }
      // colour 32 -> 64 -> 64 -> 3
      layer(h_col, kWoffCW1, 32, id64, nullptr);
      relu_to_h(d_row, h_row);
      if (sync_bad()) { fail = true; break; }
      layer(h_col, kWoffCW2, 64, id64, nullptr);
      relu_to_h(d_row, h_row);
      if (sync_bad()) { fail = true; break; }
      layer(h_col, kWoffCW3, 64, id16, nullptr);
      float v5[16];
      tc::tmem_ld16(d_row, v5);
      // Compositing (FP32, every operation rounded explicitly).
      if (flags & kTagSample) {
        if (flags & kTagFirst) {
          cur = rid;
          T = 1.0f;
          cr = cg = cb = cz = 0.0f;
        }
        if (cur == rid) {  // samples of a ray that already terminated are dropped
          ++my_samples;
          const float alpha = -expm1f(__fmul_rn(-sigma, kDt));
          const float wgt = __fmul_rn(T, alpha);
          cr = __fmaf_rn(wgt, sigmoidf(v5[0]), cr);
          cg = __fmaf_rn(wgt, sigmoidf(v5[1]), cg);
          cb = __fmaf_rn(wgt, sigmoidf(v5[2]), cb);
          cz = __fmaf_rn(wgt, t, cz);
          T = __fsub_rn(T, wgt);
          const bool stop_early = T < kTStop;
          if (stop_early || (flags & kTagLast)) {
            write_ray(vb, s, cur, cr, cg, cb, cz);
            if (stop_early && !(flags & kTagLast)) term[row] = cur + 1u;  // tells the encoder to move on
            cur = 0xFFFFFFFFu;
          }
        }
      }
      // The next tile's first layer overwrites the accumulator this thread
      // has just read: the wait at the top of the loop is a barrier.
    }
  } else if (!fail) {
    // ======================= encoder warps =======================
    // Each warp runs on its own: it waits only for its tile buffer to be
    // free (the MLP's first layer has read it), never for results.
    tc::regs_inc<kEncRegs>();
    const uint32_t nrays = min(s.counters[kCtrRays], s.max_rays);
    const int wq = warp & 3;
    Slot q;
    bool exhausted = false;
    for (uint32_t k = 0;; ++k) {
      const int b = (int)(k & 1u);
      if (k >= 2) {
        // Lane 0 waits and reads the group's stop flag; the warp learns both
        // from it, so every lane takes the same exit.
        int st = 0;
        if (lane == 0) st = !tc::mbar_wait_sleep(bar + 2 + b, ((k >> 1) - 1u) & 1u) ? 1 : (*gdone ? 2 : 0);
        st = __shfl_sync(0xffffffffu, st, 0);
        if (st == 1) { fail = true; break; }
        if (st == 2) break;
      }
      // A ray the MLP terminated early (T < 1e-4) is encoded no further.
      if (q.live && term[row] == q.id + 1u) q.live = false;
      // Refill a whole warp at once: the warp claims 32 consecutive rays (one
      // 4x8 pixel tile) only when all its lanes are done, so its 32 samples
      // stay neighbours in space and each warp-wide gather stays coherent.
      for (;;) {
        if (__ballot_sync(0xffffffffu, q.live) != 0u || exhausted) break;
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(s.counters + kCtrCursor, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= nrays) {
          exhausted = true;
          break;
        }
        const uint32_t id = base + lane;
        if (id < nrays) {
          const float4 rd = s.ray_dt[id];
          const RayMeta m = s.ray_meta[id];
          const DevView& V = vb.v[m.view];
          q.o = make_float3(V.M[3], V.M[7], V.M[11]);
          q.d = make_float3(rd.x, rd.y, rd.z);
          q.ts = rd.w;
          q.n = m.n;
          q.ei = 0;
          q.id = id;
          skip_empty(sc, q);
          if (q.ei < q.n) {
            q.live = true;
            q.first = true;
          } else {
            write_ray(vb, s, id, 0.0f, 0.0f, 0.0f, 0.0f);  // no occupied sample
          }
        }
      }
      const bool has = q.live;
      uint32_t tag = 0;
      const float t = has ? fmaf((float)q.ei + 0.5f, kDt, q.ts) : 0.0f;
      const float3 x = sample_pos(q.o, q.d, t);
      encode_all<kRec>(sc.table16, sc.rec16, sc.T, sc.dense_mask, x, has, enc_cols + 16 * b + lane_off);
      if (has) {
        tag = kTagSample | (q.first ? kTagFirst : 0u);
        q.first = false;
        ++q.ei;
        skip_empty(sc, q);
        if (q.ei >= q.n) {
          tag |= kTagLast;
          q.live = false;
        }
      }
      hand[b * 128 + row] = make_uint2(q.id | (tag << 28), __float_as_uint(t));
      const bool fin = exhausted && __ballot_sync(0xffffffffu, has) == 0u;
      if (lane == 0) wfin[b * 4 + wq] = fin ? 1u : 0u;
      tc::tmem_wait_st();
      tc::fence_before();
      tc::mbar_arrive(bar + b);
    }
  }

  if (fail) atomicExch(s.counters + kCtrError, 1u);
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

// One thread per cell of the record levels: copies the cell's 8 corner
// entries (same index rule as encode_level) into its 32-byte record.
__global__ void build_records_kernel(const __half2* __restrict__ table, uint32_t T, uint32_t dense_mask,
                                     int rec_levels, uint4* __restrict__ rec) {
  const uint32_t cells = rec_cell_offset(rec_levels);
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += gridDim.x * blockDim.x) {
    int L = 0;
    while (L + 1 < rec_levels && c >= rec_cell_offset(L + 1)) ++L;
    const uint32_t N = (uint32_t)level_res(L), local = c - rec_cell_offset(L);
    const uint32_t ix = local % N, iy = (local / N) % N, iz = local / (N * N);
    uint32_t e[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint32_t x = ix + (k & 1), y = iy + ((k >> 1) & 1), z = iz + ((k >> 2) & 1);
      uint32_t idx;
      if ((dense_mask >> L) & 1u) {
        const uint32_t s = N + 1u;
        idx = x + s * (y + s * z);
      } else {
        idx = (x ^ (y * kPrime1) ^ (z * kPrime2)) & (T - 1u);
      }
      const __half2 v = table[(size_t)L * T + idx];
      e[k] = *reinterpret_cast<const uint32_t*>(&v);
    }
    rec[2 * (size_t)c] = make_uint4(e[0], e[1], e[2], e[3]);
    rec[2 * (size_t)c + 1] = make_uint4(e[4], e[5], e[6], e[7]);
  }
}

}  // namespace

size_t tc_record_bytes(int rec_levels) { return (size_t)rec_cell_offset(rec_levels) * 32; }

cudaError_t launch_build_records(const __half2* table16, uint32_t T, uint32_t dense_mask, int rec_levels, uint4* rec,
                                 cudaStream_t stream) {
  if (rec_levels != kRecLevelsDefault && rec_levels != kRecLevelsSmall) return cudaErrorInvalidValue;
  build_records_kernel<<<2048, 256, 0, stream>>>(table16, T, dense_mask, rec_levels, rec);
  return cudaGetLastError();
}

size_t tc_weight_bytes() { return kWBytes; }

cudaError_t launch_pack_tc_weights(const float* w32, uint8_t* out, cudaStream_t stream) {
  pack_tc_weights_kernel<<<(kWBytes / 2 + 255) / 256, 256, 0, stream>>>(w32, out);
  return cudaGetLastError();
}

namespace {

template <class Src, int kRec>
cudaError_t launch_march_tc_rec(const Src& src, const DevScene& scene, const DevScratch& s, int num_sms,
                                cudaStream_t stream) {
  if (!scene.table16 || !scene.rec16 || !scene.tc_weights) return cudaErrorInvalidValue;
  if (s.max_rays > kIdMask) return cudaErrorInvalidValue;  // ray ids share a word with the flags
  static bool attr_set = false;  // idempotent; a race only repeats the calls
  if (!attr_set) {
    cudaError_t e =
        cudaFuncSetAttribute(march_tc_kernel<Src, kRec>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemRequest);
    if (e != cudaSuccess) return e;
    // 14 % of 228 KiB selects the 32 KiB configuration, which holds the
    // request: the rest of the SM's 256 KiB stays L1 for the table gathers.
    e = cudaFuncSetAttribute(march_tc_kernel<Src, kRec>, cudaFuncAttributePreferredSharedMemoryCarveout, 14);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  // One CTA per SM is what makes the 512-column TMEM allocation safe: two
  // 1024-thread CTAs fit on an SM only at <= 32 registers per thread.
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, march_tc_kernel<Src, kRec>);
  if (e != cudaSuccess) return e;
  // The setmaxnreg split hands out exactly 1024 x kLaunchRegs registers: a
  // build with a smaller launch allocation would stall the encoders' increase.
  if (fa.numRegs != (int)kLaunchRegs) return cudaErrorInvalidConfiguration;
  march_tc_kernel<Src, kRec><<<num_sms, kTcThreads, kSmemRequest, stream>>>(src, scene, s);
  return cudaGetLastError();
}

template <class Src>
cudaError_t launch_march_tc_src(const Src& src, const DevScene& scene, const DevScratch& s, int num_sms,
                                cudaStream_t stream) {
  if (scene.rec_levels == kRecLevelsDefault)
    return launch_march_tc_rec<Src, kRecLevelsDefault>(src, scene, s, num_sms, stream);
  if (scene.rec_levels == kRecLevelsSmall)
    return launch_march_tc_rec<Src, kRecLevelsSmall>(src, scene, s, num_sms, stream);
  return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_march_tc(const ViewBatch& views, const DevScene& scene, const DevScratch& s, int num_sms,
                            cudaStream_t stream) {
  return launch_march_tc_src(InParam<ViewBatch>{views}, scene, s, num_sms, stream);
}

cudaError_t launch_march_tc(const ViewBatch* views_dev, const DevScene& scene, const DevScratch& s, int num_sms,
                            cudaStream_t stream) {
  return launch_march_tc_src(InMemory<ViewBatch>{views_dev}, scene, s, num_sms, stream);
}

}  // namespace nes
