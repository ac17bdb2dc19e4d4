// scene.h -- seeded scene generator (host side).
//
// The reference has no scene: neserver receives finished frames from an
// external instant-ngp-renderer (README.md:3-5).  The GB300 build generates
// the hash-grid NeRF itself from a seed so every request is reproducible:
//  - SplitMix64 (Steele, Lea, Flood, OOPSLA 2014) in counter form:
//    draw i of stream s = mix(key + (i+1) * 0x9E3779B97F4A7C15),
//    key = mix(seed * 256 + s);
//  - table entries U(-0.5, 0.5) from the top 24 bits (exact in FP32),
//    stream 0, index (level * T + entry) * 2 + feature;
//  - Xavier-uniform weights U(-a, a), a = sqrt(6 / (fan_in + fan_out)),
//    streams 1..5 for density W1, W2 and colour W1, W2, W3; colour W1 draws
//    31 columns per row (fan_in 31) and its padding column 31 is zero.
#pragma once
#include <cstdint>
#include <vector>

namespace nes {

struct SceneHost {
  uint32_t log2T = 19;
  uint32_t T = 1u << 19;
  std::vector<float> table;    // [16][T][2], level-major
  std::vector<float> weights;  // kWeightFloats, offsets in nes_spec.h
};

uint64_t splitmix_key(uint64_t seed, uint32_t stream);
uint64_t splitmix_draw(uint64_t key, uint64_t i);

// Generates the scene for seed and 2^log2T entries per level.
bool generate_scene(uint64_t seed, uint32_t log2T, SceneHost* out);

}  // namespace nes
