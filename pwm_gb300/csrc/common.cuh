// Shared device/host helpers of the GB300 wavelet construction engine.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pwmgpu {

// Device status word bits (set by kernels, read by the host after a sync).
constexpr uint32_t kErrSymbol = 1u;   // a symbol >= 2^levels was seen
constexpr uint32_t kErrTimeout = 2u;  // a bounded spin-wait gave up
constexpr uint32_t kErrBounds = 4u;   // a kernel-side bounds check tripped

// Default upper bound on the polls of one decoupled look-back wait (each poll
// sleeps ~64-100 ns), ~1.5 s in total; after that the kernel records
// kErrTimeout and carries on with a zero prefix so that it always terminates.
// The tile engine takes its bound per launch (pwmgpu_ctx_set_spin_limit).
constexpr uint32_t kSpinLimit = 1u << 24;

__host__ __device__ inline uint64_t words_for(uint64_t bits) { return (bits + 63) >> 6; }
// Words of one level in pwm's flat layout: padded to 16 words (128 bytes).
__host__ __device__ inline uint64_t padded_words(uint64_t bits) { return (words_for(bits) + 15) & ~uint64_t(15); }

// Reverse the low `bits` bits of v (bits <= 32).
__host__ __device__ inline uint32_t reverse_low_bits(uint32_t v, uint32_t bits) {
#ifdef __CUDA_ARCH__
  return bits == 0 ? 0u : (__brev(v) >> (32 - bits));
#else
  uint32_t r = 0;
  for (uint32_t i = 0; i < bits; ++i) { r = (r << 1) | (v & 1u); v >>= 1; }
  return r;
#endif
}

// A pwm level seen as u32 chunks: chunk q holds positions 32q..32q+31 with
// position 32q at bit 31.  In little-endian memory the first 32 positions of
// a u64 word are its high half, so chunk q lives at u32 index q ^ 1.
__host__ __device__ inline uint64_t chunk_u32_index(uint64_t q) { return q ^ 1ull; }

// Mask of the chunk bits for chunk positions [lo, hi) (0 <= lo <= hi <= 32),
// position p at bit 31-p.
__device__ inline uint32_t chunk_mask(uint32_t lo, uint32_t hi) {
  uint32_t a = lo >= 32 ? 0u : (0xFFFFFFFFu >> lo);
  uint32_t b = hi >= 32 ? 0xFFFFFFFFu : (hi == 0 ? 0u : ~(0xFFFFFFFFu >> hi));
  return a & b;
}

// Decoupled look-back state word: flag in bits 62-63, count in bits 0-61.
constexpr uint64_t kFlagAggregate = 1ull << 62;
constexpr uint64_t kFlagPrefix = 2ull << 62;
constexpr uint64_t kCountMask = (1ull << 62) - 1;

__device__ inline uint64_t ld_volatile(const unsigned long long* p) {
  return *reinterpret_cast<const volatile unsigned long long*>(p);
}
__device__ inline void st_volatile(unsigned long long* p, uint64_t v) {
  *reinterpret_cast<volatile unsigned long long*>(p) = v;
}

// Wait (bounded) for the look-back word of a predecessor tile and return it;
// on timeout records kErrTimeout in *status and returns a zero prefix.
__device__ inline uint64_t lookback_wait(const unsigned long long* word, uint32_t* status) {
  uint64_t s = ld_volatile(word);
  uint32_t spins = 0;
  while ((s >> 62) == 0) {
    if (++spins > kSpinLimit) {
      atomicOr(status, kErrTimeout);
      return kFlagPrefix;
    }
    __nanosleep(100);
    s = ld_volatile(word);
  }
  return s;
}

// Select the bit position (counted from the most significant bit) of the
// bit with the given 1-based rank inside a word: the published branch-free
// method from Sean Eron Anderson's "Bit Twiddling Hacks", the same method
// pwm uses (include/queries/bin_select_popcnt.hpp:123-164), so that ranks
// outside 1..popcount give the same value as pwm.
__host__ __device__ inline uint32_t word_select1(uint64_t v, uint32_t rank) {
  const uint64_t m1 = ~0ull / 3, m2 = ~0ull / 5, m4 = ~0ull / 0x11, m8 = ~0ull / 0x101;
  uint32_t r = rank;
  uint64_t a = v - ((v >> 1) & m1);
  uint64_t b = (a & m2) + ((a >> 2) & m2);
  uint64_t c = (b + (b >> 4)) & m4;
  uint64_t d = (c + (c >> 8)) & m8;
  uint32_t t = uint32_t((d >> 32) + (d >> 48));
  uint32_t s = 64;
  s -= ((t - r) & 256) >> 3; r -= (t & ((t - r) >> 8));
  t = uint32_t((d >> (s - 16)) & 0xff);
  s -= ((t - r) & 256) >> 4; r -= (t & ((t - r) >> 8));
  t = uint32_t((c >> (s - 8)) & 0xf);
  s -= ((t - r) & 256) >> 5; r -= (t & ((t - r) >> 8));
  t = uint32_t((b >> (s - 4)) & 0x7);
  s -= ((t - r) & 256) >> 6; r -= (t & ((t - r) >> 8));
  t = uint32_t((a >> (s - 2)) & 0x3);
  s -= ((t - r) & 256) >> 7; r -= (t & ((t - r) >> 8));
  t = uint32_t((v >> (s - 1)) & 0x1);
  s -= ((t - r) & 256) >> 8;
  return 64 - s;
}

}  // namespace pwmgpu
