// Seeded synthetic texts: a counter-based splitmix64 stream (value i depends
// only on the seed and i, so host and device produce identical texts) mapped
// through inverse-CDF threshold tables of 53-bit integers.
#pragma once

#include <cstdint>

namespace pwmgpu {

__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// First index with u53 < thr[idx]; thr[nthr-1] == 2^53.
__host__ __device__ inline uint32_t search_thresholds(const uint64_t* thr, uint32_t nthr, uint64_t u53) {
  uint32_t lo = 0, hi = nthr - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (u53 < thr[mid]) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// Symbol i of distribution `dist` (PWMGPU_GEN_* in pwmgpu.h); key = mix64(seed).
__host__ __device__ inline uint64_t gen_value(int dist, uint64_t key, uint64_t param, uint64_t i, const uint64_t* thr,
                                              uint32_t nthr, const uint32_t* perm) {
  const uint64_t r = mix64(key + i);
  switch (dist) {
    case 0: return param ? (r >> 11) % param : 0;                   // uniform [0, param)
    case 1: return search_thresholds(thr, nthr, r >> 11);           // DNA4
    case 2: return perm[search_thresholds(thr, nthr, r >> 11)];     // Zipf(1.0) over 256, permuted
    default:                                                         // MIX16
      return (r & 1) ? ((r >> 16) & 0xFFFF) : search_thresholds(thr, nthr, mix64(r) >> 11);
  }
}

}  // namespace pwmgpu
