// scene.cpp -- seeded scene generator; the rules are written out in scene.h.
#include "scene.h"

#include <cmath>
#include <thread>

#include "nes_spec.h"

namespace nes {

namespace {
constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;

inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

inline uint32_t top24(uint64_t key, uint64_t i) { return (uint32_t)(splitmix_draw(key, i) >> 40); }

float xavier(uint64_t key, uint64_t i, int fan_in, int fan_out) {
  const double a = std::sqrt(6.0 / (double)(fan_in + fan_out));
  const double u = (double)top24(key, i) * 0x1p-23 - 1.0;  // exact, in [-1, 1)
  return (float)(u * a);
}

void fill_matrix(float* w, int rows, int cols, int fan_in, int fan_out, uint64_t key) {
  for (int r = 0; r < rows; ++r)
    for (int c = 0; c < cols; ++c) w[r * cols + c] = xavier(key, (uint64_t)r * cols + c, fan_in, fan_out);
}
}  // namespace

uint64_t splitmix_key(uint64_t seed, uint32_t stream) { return mix64(seed * 256ull + stream); }
uint64_t splitmix_draw(uint64_t key, uint64_t i) { return mix64(key + (i + 1ull) * kGamma); }

bool generate_scene(uint64_t seed, uint32_t log2T, SceneHost* out) {
  if (log2T < 10 || log2T > 24) return false;
  out->log2T = log2T;
  out->T = 1u << log2T;
  const size_t n = (size_t)kLevels * out->T * kFeats;
  out->table.resize(n);
  const uint64_t kt = splitmix_key(seed, 0);
  // The table draw is embarrassingly parallel (counter-based generator).
  unsigned nth = std::thread::hardware_concurrency();
  if (nth == 0) nth = 1;
  if (nth > 16) nth = 16;
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nth; ++t) {
    pool.emplace_back([&, t] {
      const size_t b = n * t / nth, e = n * (t + 1) / nth;
      float* tab = out->table.data();
      for (size_t i = b; i < e; ++i) tab[i] = (float)((int32_t)top24(kt, i) - (1 << 23)) * 0x1p-24f;
    });
  }
  for (auto& th : pool) th.join();

  out->weights.assign(kWeightFloats, 0.0f);
  float* w = out->weights.data();
  fill_matrix(w + kOffDW1, kHid, kEnc, kEnc, kHid, splitmix_key(seed, 1));
  fill_matrix(w + kOffDW2, kDOut, kHid, kHid, kDOut, splitmix_key(seed, 2));
  {
    const uint64_t k = splitmix_key(seed, 3);
    for (int r = 0; r < kHid; ++r) {
      for (int c = 0; c < 31; ++c) w[kOffCW1 + r * kCIn + c] = xavier(k, (uint64_t)r * 31 + c, 31, kHid);
      w[kOffCW1 + r * kCIn + 31] = 0.0f;
    }
  }
  fill_matrix(w + kOffCW2, kHid, kHid, kHid, kHid, splitmix_key(seed, 4));
  fill_matrix(w + kOffCW3, 3, kHid, kHid, 3, splitmix_key(seed, 5));
  return true;
}

}  // namespace nes
