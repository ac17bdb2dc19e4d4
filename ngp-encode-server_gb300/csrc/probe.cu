// probe.cu -- measured ceilings for the tensor-core march's gather stream.
//
// The march's MLP contraction has a tensor-core roofline (the measured bf16
// peak); its other term is the hash-table gather stream: per sample one
// per-cell corner record for each of the recorded levels (32 bytes,
// read as two 16-byte loads) and 8 scattered 4-byte table entries for each
// level above: the 512 bytes of algorithmic gathers.  No library figure exists for such a
// stream, so these kernels measure it on the device itself:
//
//  - gather_probe_kernel: uniformly random loads of 4, 16 or 32 bytes over a
//    table of a given size (e.g. the 32 MiB FP16 table, L2-resident): the
//    hardware's random-gather rate with no locality to exploit;
//  - replay_kernel: the march's own load stream -- the same compacted rays,
//    the same warp-wide 32-ray refills, the same sample positions and the same
//    record and table addresses -- with no interpolation, no MLP and no
//    compositing: the floor the gathers alone put under the march.
#include <cuda_fp16.h>

#include "kernels.h"

namespace nes {

namespace {

constexpr int kProbeThreads = 256;

// xorshift32: a cheap per-thread index stream.
__device__ __forceinline__ uint32_t xs32(uint32_t& s) {
  s ^= s << 13;
  s ^= s >> 17;
  s ^= s << 5;
  return s;
}

template <int kBytes>
__global__ void __launch_bounds__(kProbeThreads)
gather_probe_kernel(const uint8_t* __restrict__ table, uint32_t mask, uint32_t loads, uint32_t* __restrict__ sink) {
  const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t s = gid * 2654435761u + 12345u;
  s = s ? s : 1u;
  uint32_t acc = 0;
  for (uint32_t i = 0; i < loads; ++i) {
    const uint32_t e = xs32(s) & mask;  // element index, kBytes each
    if (kBytes == 4) {
      acc ^= __ldg(reinterpret_cast<const uint32_t*>(table) + e);
    } else if (kBytes == 16) {
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(table) + e);
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    } else {  // a 32-byte record as two 16-byte loads, like the march
      const uint4 a = __ldg(reinterpret_cast<const uint4*>(table) + 2 * (size_t)e);
      const uint4 b = __ldg(reinterpret_cast<const uint4*>(table) + 2 * (size_t)e + 1);
      acc ^= a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w;
    }
  }
  sink[gid] = acc;
}

template <int L>
__device__ __forceinline__ uint32_t replay_level_rec(const uint4* __restrict__ rec, const float3& x) {
  constexpr int N = level_res(L);
  const int ix = min(__float2int_rd(x.x * (float)N), N - 1), iy = min(__float2int_rd(x.y * (float)N), N - 1),
            iz = min(__float2int_rd(x.z * (float)N), N - 1);
  const uint32_t cell = rec_cell_offset(L) + (uint32_t)ix + (uint32_t)N * ((uint32_t)iy + (uint32_t)N * (uint32_t)iz);
  const uint4 a = __ldg(rec + 2 * cell), b = __ldg(rec + 2 * cell + 1);
  return a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w;
}

template <int L>
__device__ __forceinline__ uint32_t replay_level_tab(const uint32_t* __restrict__ table, uint32_t T,
                                                     uint32_t dense_mask, const float3& x) {
  constexpr int N = level_res(L);
  const int ix = min(__float2int_rd(x.x * (float)N), N - 1), iy = min(__float2int_rd(x.y * (float)N), N - 1),
            iz = min(__float2int_rd(x.z * (float)N), N - 1);
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
  const uint32_t* tab = table + (size_t)L * T;
  uint32_t acc = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) acc ^= __ldg(tab + idx[k]);
  return acc;
}

// Level L as the march reads it: a per-cell record if the level is recorded, else
// eight table entries.
template <int L>
__device__ __forceinline__ uint32_t replay_level(const DevScene& sc, const uint32_t* __restrict__ table,
                                                 const float3& x) {
  if ((uint32_t)L < sc.rec_levels) return replay_level_rec<L>(sc.rec16, x);
  return replay_level_tab<L>(table, sc.T, sc.dense_mask, x);
}

// One thread per ray slot, warps refilled 32 rays at a time (one 4x8 pixel
// tile) once all their lanes are done, every occupied sample's records and
// table entries loaded in order, the occupancy bit of every sample read as
// the march reads it; one CTA per SM of 512 threads (as many slots as the
// march's encoder threads) or 256.  Like the march's encoder groups, each
// group of 128 slots advances one sample per step together (a named-barrier
// step per sample, the march's tile), so rays that are neighbours on screen
// stay neighbours in t and share the lines they load.
__global__ void __launch_bounds__(512, 1)
replay_kernel(const __grid_constant__ InParam<ViewBatch> src, const DevScene sc, const DevScratch s,
              uint32_t* __restrict__ sink) {
  const ViewBatch& vb = src.get();
  const uint32_t nrays = min(s.counters[kCtrRays], s.max_rays);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t group_bar = 1u + (threadIdx.x >> 7);  // 128 threads per group
  const uint32_t* table = reinterpret_cast<const uint32_t*>(sc.table16);
  uint32_t acc = 0;
  bool live = false, exhausted = false;
  float3 o = make_float3(0.f, 0.f, 0.f), d = o;
  float ts = 0.0f;
  int n = 0, ei = 0;
  auto occ_at = [&](int i) { return occupied(sc.occ, sample_pos(o, d, fmaf((float)i + 0.5f, kDt, ts))); };
  for (;;) {
    for (;;) {  // whole-warp refill, as the march's encoders
      if (__ballot_sync(0xffffffffu, live) != 0u || exhausted) break;
      const uint32_t base = warp_claim(s.counters + kCtrCursor, 32);
      if (base >= nrays) {
        exhausted = true;
        break;
      }
      const uint32_t id = base + lane;
      if (id < nrays) {
        const float4 rd = s.ray_dt[id];
        const RayMeta m = s.ray_meta[id];
        const DevView& V = vb.v[m.view];
        o = make_float3(V.M[3], V.M[7], V.M[11]);
        d = make_float3(rd.x, rd.y, rd.z);
        ts = rd.w;
        n = m.n;
        ei = 0;
        while (ei < n && !occ_at(ei)) ++ei;
        live = ei < n;
      }
    }
    if (live) {
      const float3 x = sample_pos(o, d, fmaf((float)ei + 0.5f, kDt, ts));
      acc ^= replay_level<0>(sc, table, x) ^ replay_level<1>(sc, table, x) ^ replay_level<2>(sc, table, x) ^
             replay_level<3>(sc, table, x) ^ replay_level<4>(sc, table, x) ^ replay_level<5>(sc, table, x) ^
             replay_level<6>(sc, table, x) ^ replay_level<7>(sc, table, x) ^ replay_level<8>(sc, table, x) ^
             replay_level<9>(sc, table, x) ^ replay_level<10>(sc, table, x) ^ replay_level<11>(sc, table, x) ^
             replay_level<12>(sc, table, x) ^ replay_level<13>(sc, table, x) ^ replay_level<14>(sc, table, x) ^
             replay_level<15>(sc, table, x);
      ++ei;
      while (ei < n && !occ_at(ei)) ++ei;
      live = ei < n;
    }
    // One step per sample for the whole group; it ends when no warp of the
    // group has a ray left (every thread takes the same number of steps).
    const bool warp_busy = !exhausted || __ballot_sync(0xffffffffu, live) != 0u;
    uint32_t more;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(more)
        : "r"((uint32_t)warp_busy), "r"(group_bar)
        : "memory");
    if (!more) break;
  }
  sink[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

}  // namespace

cudaError_t launch_gather_probe(const void* table, uint64_t table_bytes, int load_bytes, uint32_t loads_per_thread,
                                uint32_t* sink, uint32_t threads, cudaStream_t stream) {
  if (load_bytes != 4 && load_bytes != 16 && load_bytes != 32) return cudaErrorInvalidValue;
  const uint64_t elems = table_bytes / (uint64_t)load_bytes;
  if (elems < 2 || (elems & (elems - 1)) || elems > (1ull << 32)) return cudaErrorInvalidValue;
  if (threads == 0 || threads % kProbeThreads) return cudaErrorInvalidValue;
  const uint32_t mask = (uint32_t)(elems - 1);
  const unsigned blocks = threads / kProbeThreads;
  const uint8_t* t = static_cast<const uint8_t*>(table);
  if (load_bytes == 4)
    gather_probe_kernel<4><<<blocks, kProbeThreads, 0, stream>>>(t, mask, loads_per_thread, sink);
  else if (load_bytes == 16)
    gather_probe_kernel<16><<<blocks, kProbeThreads, 0, stream>>>(t, mask, loads_per_thread, sink);
  else
    gather_probe_kernel<32><<<blocks, kProbeThreads, 0, stream>>>(t, mask, loads_per_thread, sink);
  return cudaGetLastError();
}

cudaError_t launch_gather_replay(const ViewBatch& views, const DevScene& scene, const DevScratch& s, int num_sms,
                                 int threads, uint32_t* sink, cudaStream_t stream) {
  if (threads != 256 && threads != 512) return cudaErrorInvalidValue;
  if (!scene.table16 || !scene.rec16) return cudaErrorInvalidValue;
  // The march's L1 / shared-memory split (32 KiB shared, the rest L1): the
  // gathers' speed depends on it.
  cudaError_t e = cudaFuncSetAttribute(replay_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 14);
  if (e != cudaSuccess) return e;
  replay_kernel<<<num_sms, threads, 0, stream>>>(InParam<ViewBatch>{views}, scene, s, sink);
  return cudaGetLastError();
}

}  // namespace nes
