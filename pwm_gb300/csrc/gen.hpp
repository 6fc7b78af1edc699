// Seeded synthetic texts: a counter-based splitmix64 stream (value i depends
// only on the seed and i, so host and device produce identical texts) mapped
// through inverse-CDF threshold tables of 53-bit integers.
//
// Plain C++ (no CUDA headers needed): the library compiles it for host and
// device; a CPU-only program can include it to produce the same texts.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <utility>
#include <vector>

#if defined(__CUDACC__)
#define PWMGPU_HD __host__ __device__
#else
#define PWMGPU_HD
#endif

namespace pwmgpu {

// Distribution ids (PWMGPU_GEN_* in include/pwmgpu.h).
enum : int { kGenUniform = 0, kGenDna4 = 1, kGenZipf256 = 2, kGenMix16 = 3 };

PWMGPU_HD inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// First index with u53 < thr[idx]; thr[nthr-1] == 2^53.
PWMGPU_HD inline uint32_t search_thresholds(const uint64_t* thr, uint32_t nthr, uint64_t u53) {
  uint32_t lo = 0, hi = nthr - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (u53 < thr[mid]) hi = mid; else lo = mid + 1;
  }
  return lo;
}

// Symbol i of distribution `dist`; key = mix64(seed).
PWMGPU_HD inline uint64_t gen_value(int dist, uint64_t key, uint64_t param, uint64_t i, const uint64_t* thr,
                                    uint32_t nthr, const uint32_t* perm) {
  const uint64_t r = mix64(key + i);
  switch (dist) {
    case kGenUniform: return param ? (r >> 11) % param : 0;                 // uniform [0, param)
    case kGenDna4: return search_thresholds(thr, nthr, r >> 11);            // DNA4
    case kGenZipf256: return perm[search_thresholds(thr, nthr, r >> 11)];   // Zipf(1.0) over 256, permuted
    default:                                                                // MIX16
      return (r & 1) ? ((r >> 16) & 0xFFFF) : search_thresholds(thr, nthr, mix64(r) >> 11);
  }
}

// Host thresholds / permutation of a distribution.  Every program that
// includes this header compiles it with -ffp-contract=off (GCC fuses
// multiply-adds on AArch64 by default), so that x86-64 and AArch64 hosts
// produce identical tables.
struct GenTables {
  std::vector<uint64_t> thr;
  std::vector<uint32_t> perm;
};

inline std::vector<uint64_t> thresholds_from_weights(const std::vector<double>& w) {
  double total = 0;
  for (double x : w) total += x;
  std::vector<uint64_t> thr(w.size());
  double cum = 0;
  const double scale = 9007199254740992.0;  // 2^53
  for (size_t i = 0; i < w.size(); ++i) {
    cum += w[i];
    double v = (cum / total) * scale;
    thr[i] = v >= scale ? (uint64_t(1) << 53) : uint64_t(v);
  }
  thr.back() = uint64_t(1) << 53;
  return thr;
}

inline GenTables gen_tables(int dist, uint64_t seed) {
  GenTables g;
  if (dist == kGenDna4) {
    g.thr = thresholds_from_weights({0.3, 0.2, 0.2, 0.3});
  } else if (dist == kGenZipf256) {
    std::vector<double> w(256);
    for (int r = 1; r <= 256; ++r) w[size_t(r - 1)] = 1.0 / double(r);
    g.thr = thresholds_from_weights(w);
    g.perm.resize(256);
    std::iota(g.perm.begin(), g.perm.end(), 0u);
    const uint64_t pkey = mix64(seed ^ 0x5bd1e9955bd1e995ull);
    for (uint32_t j = 255; j > 0; --j) {
      const uint32_t k = uint32_t(mix64(pkey + j) % (j + 1));
      std::swap(g.perm[j], g.perm[k]);
    }
  } else if (dist == kGenMix16) {
    // geometric(p = 0.01) on {0, 1, ...} clamped to 65535: cumulative
    // 1 - q^(k+1) with q^(k+1) by repeated multiplication.
    const double q = 0.99;
    std::vector<uint64_t> thr(65536);
    double qk = 1.0;
    const double scale = 9007199254740992.0;
    for (uint32_t k = 0; k < 65536; ++k) {
      qk *= q;
      double v = (1.0 - qk) * scale;
      thr[k] = v >= scale ? (uint64_t(1) << 53) : uint64_t(v);
    }
    thr.back() = uint64_t(1) << 53;
    g.thr = std::move(thr);
  }
  if (g.thr.empty()) g.thr.push_back(uint64_t(1) << 53);
  if (g.perm.empty()) g.perm.push_back(0);
  return g;
}

// n symbols of `dist` into a host array of `width`-byte symbols (1, 2, 4).
inline void generate_host(int dist, uint64_t seed, uint64_t param, uint64_t n, uint32_t width, void* out) {
  const GenTables g = gen_tables(dist, seed);
  const uint64_t key = mix64(seed);
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t v = gen_value(dist, key, param, i, g.thr.data(), uint32_t(g.thr.size()), g.perm.data());
    if (width == 1) static_cast<uint8_t*>(out)[i] = uint8_t(v);
    else if (width == 2) static_cast<uint16_t*>(out)[i] = uint16_t(v);
    else static_cast<uint32_t*>(out)[i] = uint32_t(v);
  }
}

// The batched workload: `count` 8-bit texts with log-normal lengths (median
// 2^16, sigma_ln 1.5, clamped to [2^10, 2^24]); 15% Zipf(1.0) byte texts with
// 8 levels, 85% DNA-like texts over {0..4} (symbol 4 in geometric runs of
// mean 50, about 2% of the symbols) with 3 levels.  Writes offsets (count+1)
// and levels (count); texts (offsets[count] bytes) may be null to size the
// batch.  The lengths go through libm's log/exp/cos, so they are exact only
// as far as the host's libm is.
inline void generate_batch_host(uint64_t seed, uint32_t count, uint64_t* offsets, uint32_t* levels, uint8_t* texts) {
  const uint64_t key = mix64(seed ^ 0x0ba7c4ull);
  const double two_pi = 6.283185307179586;
  offsets[0] = 0;
  for (uint32_t i = 0; i < count; ++i) {
    const double u1 = (double((mix64(key + 2ull * i) >> 11) + 1)) / 9007199254740993.0;
    const double u2 = double(mix64(key + 2ull * i + 1) >> 11) / 9007199254740992.0;
    const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(two_pi * u2);
    double len = std::floor(std::exp(std::log(65536.0) + 1.5 * z) + 0.5);
    len = std::min(std::max(len, 1024.0), 16777216.0);
    offsets[i + 1] = offsets[i] + uint64_t(len);
    levels[i] = (mix64(key ^ (0x5eedull + i)) % 100) < 15 ? 8 : 3;
  }
  if (!texts) return;
  const GenTables zipf = gen_tables(kGenZipf256, seed);
  const std::vector<uint64_t> dna = thresholds_from_weights({0.29, 0.2, 0.2, 0.29});
  // runs of symbol 4: a run starts with probability ps, lengths geometric
  // with mean 50; ps makes symbol 4 about 2% of the text
  const double ps = 0.02 / (50.0 * 0.98 + 0.02);
  const uint64_t ps_thr = uint64_t(ps * 9007199254740992.0);
  std::vector<uint64_t> geo(4096);
  {
    double qk = 1.0;
    for (size_t k = 0; k < geo.size(); ++k) {
      qk *= 0.98;
      geo[k] = uint64_t((1.0 - qk) * 9007199254740992.0);
    }
    geo.back() = uint64_t(1) << 53;
  }
  for (uint32_t i = 0; i < count; ++i) {
    uint8_t* out = texts + offsets[i];
    const uint64_t n = offsets[i + 1] - offsets[i];
    const uint64_t tkey = mix64(key + 0x9e37ull * (i + 1));
    if (levels[i] == 8) {
      for (uint64_t p = 0; p < n; ++p)
        out[p] = uint8_t(gen_value(kGenZipf256, tkey, 0, p, zipf.thr.data(), uint32_t(zipf.thr.size()),
                                   zipf.perm.data()));
      continue;
    }
    for (uint64_t p = 0; p < n;) {
      const uint64_t r = mix64(tkey + p);
      if ((r >> 11) < ps_thr) {
        const uint64_t run = 1 + search_thresholds(geo.data(), uint32_t(geo.size()), mix64(r) >> 11);
        for (uint64_t k = 0; k < run && p < n; ++k) out[p++] = 4;
      } else {
        out[p] = uint8_t(search_thresholds(dna.data(), uint32_t(dna.size()), mix64(r ^ 0xd1ceull) >> 11));
        ++p;
      }
    }
  }
}

}  // namespace pwmgpu
