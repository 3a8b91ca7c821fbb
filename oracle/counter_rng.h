/*
 * Counter-based sampler keys shared by the oracle and the reference harness
 * (test infrastructure only).  The GPU library carries its own copy of the
 * same three functions; tests check that all three agree.
 *
 * One uniform float per (seed, pixel, sample, dimension): the SplitMix64
 * finaliser (Steele, Lea, Flood, "Fast splittable pseudorandom number
 * generators", OOPSLA 2014) keyed by (seed, pixel, sample), offset by the
 * dimension, converted to float the way PCG32::NextFloat does
 * (ajisai/core/random.h:46-53: 23 mantissa bits in [0, 1)).
 */
#pragma once
#include <stdint.h>
#include <string.h>

static inline uint64_t ajg_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline uint64_t ajg_path_key(uint64_t seed, uint32_t pixel,
                                    uint32_t sample) {
  return ajg_mix64(seed * 0x9E3779B97F4A7C15ull +
                   (((uint64_t)pixel << 32) | (uint64_t)sample));
}
static inline float ajg_key_float(uint64_t key, uint32_t dim) {
  uint32_t u = (uint32_t)(ajg_mix64(key + (uint64_t)(dim + 1) *
                                              0x9E3779B97F4A7C15ull) >> 32);
  uint32_t b = (u >> 9) | 0x3f800000u;
  float f;
  memcpy(&f, &b, 4);
  return f - 1.0f;
}

/* SPPM photon streams: photon i of iteration k draws from
 * ajg_path_key(ajg_photon_seed(seed), i, k). */
static inline uint64_t ajg_photon_seed(uint64_t seed) {
  return ajg_mix64(seed ^ 0x50484F544F4E5321ull);
}
