// nes_spec.h -- the scene specification shared by every kernel and the host
// generator.  The renderer these constants describe is the one neserver
// reaches over TCP (src/server.cpp:161-194); its math follows the published
// Instant-NGP method, with every free choice fixed here.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define NES_HD __host__ __device__
#else
#define NES_HD
#endif

namespace nes {

constexpr int kLevels = 16;      // hash-grid levels
constexpr int kFeats = 2;        // features per level
constexpr int kEnc = 32;         // encoded width = levels * features
constexpr int kHid = 64;         // hidden width of both MLPs
constexpr int kDOut = 16;        // density MLP output (logit + 15 geometry features)
constexpr int kCIn = 32;         // colour input: 16 SH + 15 geometry + 1 zero pad
constexpr int kOccRes = 128;     // occupancy grid cells per axis
constexpr int kOccWords = kOccRes * kOccRes * kOccRes / 32;
constexpr int kMaxSteps = 1024;  // march steps per ray
constexpr float kOccThreshold = 0.01f;
constexpr float kTStop = 1e-4f;  // stop once transmittance falls below this
// sqrt(3)/1024 rounded once to FP32.
constexpr float kDt = 0x1.bb67aep-10f;

// N_l = floor(16 * b^l), b = (2048/16)^(1/15), fixed as integers.
NES_HD constexpr int level_res(int l) {
  return l == 0 ? 16 : l == 1 ? 22 : l == 2 ? 30 : l == 3 ? 42 : l == 4 ? 58 : l == 5 ? 80
       : l == 6 ? 111 : l == 7 ? 153 : l == 8 ? 212 : l == 9 ? 294 : l == 10 ? 406
       : l == 11 ? 561 : l == 12 ? 776 : l == 13 ? 1072 : l == 14 ? 1482 : 2048;
}

// The tensor-core march also stores its coarse levels as per-cell records
// of their 8 corner entries: each record replaces eight scattered table
// gathers by one 32-byte read.  Cells of level l start at rec_cell_offset(l)
// (N_0^3 + ... + N_{l-1}^3).  A context records levels 0..12 by default
// (751,482,937 cells, 24.0 GB) or, to save device memory, levels 0..9
// (40,712,464 cells, 1.30 GB).
constexpr int kRecLevelsDefault = 13;
constexpr int kRecLevelsSmall = 10;
NES_HD constexpr uint32_t rec_cell_offset(int l) {
  uint32_t o = 0;
  for (int j = 0; j < l; ++j) o += (uint32_t)level_res(j) * (uint32_t)level_res(j) * (uint32_t)level_res(j);
  return o;
}
static_assert(rec_cell_offset(kRecLevelsDefault) == 751482937u, "record cells of levels 0..12");
static_assert(rec_cell_offset(kRecLevelsSmall) == 40712464u, "record cells of levels 0..9");

// Spatial-hash primes (Instant-NGP paper, Sec. 3).
constexpr uint32_t kPrime1 = 2654435761u;
constexpr uint32_t kPrime2 = 805459861u;

// Bit l set when level l is indexed densely: (N_l + 1)^3 <= T.
inline uint32_t dense_level_mask(uint32_t T) {
  uint32_t m = 0;
  for (int l = 0; l < kLevels; ++l) {
    uint64_t s = (uint64_t)level_res(l) + 1;
    if (s * s * s <= (uint64_t)T) m |= 1u << l;
  }
  return m;
}

// BT.601 studio-range coefficients with 16 fractional bits (luma) and 18
// (chroma from the 2x2 sum).  Luma row sums to round(219/255 * 2^16); each
// chroma row sums to zero so grey maps to 128.
constexpr int32_t kYR = 16829, kYG = 33039, kYB = 6416;
constexpr int32_t kUR = -9714, kUG = -19071, kUB = 28785;
constexpr int32_t kVR = 28784, kVG = -24103, kVB = -4681;

// Scene parameter blob (FP32, row-major [out][in]) offsets in floats.
constexpr int kOffDW1 = 0;                       // [64][32]
constexpr int kOffDW2 = kOffDW1 + kHid * kEnc;   // [16][64]
constexpr int kOffCW1 = kOffDW2 + kDOut * kHid;  // [64][32], column 31 = 0
constexpr int kOffCW2 = kOffCW1 + kHid * kCIn;   // [64][64]
constexpr int kOffCW3 = kOffCW2 + kHid * kHid;   // [3][64]
constexpr int kWeightFloats = kOffCW3 + 3 * kHid;  // 9408

}  // namespace nes
