// oracle/pwm_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of kurpicz/pwm's in-memory wavelet tree / wavelet matrix
// construction, its popcount rank/select support, its access/rank/select
// queries and its Huffman code builder.  Only the tests, the smoke check and
// the CPU-baseline leg of bench.py load this library; the GPU product never
// links it and has no CPU fallback.
//
// Every function cites the reference file:line it restates (paths relative to
// the pwm source tree).  Parity of this restatement is pinned against the
// reference itself: tests/golden/make_golden.py builds the reference headers
// into oracle/_ref/libpwmref.so and records its outputs on the reference's
// own fixture strings and on seeded inputs (tests/golden/*.json).
//
// Output layout (shared with the GPU library): all levels live in one array
// of u64 words; level l starts at offset[l] words, and every level is padded
// to a multiple of 16 words (128 bytes), exactly like pwm's
// flat_two_dim_array (include/arrays/flat_two_dim_array.hpp:117-156).
// Position i of a level is bit 63-(i&63) of word i>>6, the trailing partial
// word is left-aligned and zero padded (include/construction/
// building_blocks.hpp:18-50, include/util/common.hpp:60-68).

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <queue>
#include <unordered_map>
#include <vector>
#include <omp.h>

// The seeded input generator shared with the GPU library (plain C++): the
// oracle produces the same texts without loading the GPU library.
#include "../pwm_gb300/csrc/gen.hpp"

namespace {

inline uint64_t sym_at(const void* t, uint32_t w, uint64_t i) {
  switch (w) {
    case 1: return static_cast<const uint8_t*>(t)[i];
    case 2: return static_cast<const uint16_t*>(t)[i];
    case 4: return static_cast<const uint32_t*>(t)[i];
    default: return static_cast<const uint64_t*>(t)[i];
  }
}

inline uint64_t words_for(uint64_t bits) { return (bits + 63) >> 6; }
inline uint64_t padded_words(uint64_t bits) { return (words_for(bits) + 15) & ~uint64_t(15); }

// write_bits_wordwise (building_blocks.hpp:37-50): MSB-first packing, last
// partial word shifted left so that its unused low bits are zero.
template <typename F>
void write_bits(uint64_t* level, uint64_t size, F bit_of) {
  uint64_t pos = 0;
  for (; pos + 64 <= size; pos += 64) {
    uint64_t word = 0;
    for (uint64_t i = 0; i < 64; ++i) word = (word << 1) | bit_of(pos + i);
    level[pos >> 6] = word;
  }
  uint64_t rem = size & 63;
  if (rem) {
    uint64_t word = 0;
    for (uint64_t i = 0; i < rem; ++i) word = (word << 1) | bit_of(pos + i);
    level[pos >> 6] = word << (64 - rem);
  }
}

inline uint64_t reverse_bits(uint64_t v, uint32_t bits) {
  uint64_t r = 0;
  for (uint32_t i = 0; i < bits; ++i) { r = (r << 1) | (v & 1); v >>= 1; }
  return r;
}

inline bool bit_at(const uint64_t* level, uint64_t i) {
  return (level[i >> 6] >> (63 - (i & 63))) & 1ULL;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// Layout
// ---------------------------------------------------------------------------

// flat_two_dim_array level placement (flat_two_dim_array.hpp:117-156,
// 159-211): level_array_size = ceil(bits/64), padded up to the next 128-byte
// boundary.  Returns the total number of words.
uint64_t orc_layout(uint32_t levels, const uint64_t* level_bits, uint64_t* offsets) {
  uint64_t off = 0;
  for (uint32_t l = 0; l < levels; ++l) {
    offsets[l] = off;
    off += padded_words(level_bits[l]);
  }
  return off;
}

// ---------------------------------------------------------------------------
// Plain construction
// ---------------------------------------------------------------------------

}  // extern "C"

namespace {

// Prefix sorting, restating ps() (include/construction/ps.hpp:13-66) with the
// helpers scan_text_compute_first_level_bv_and_last_level_hist
// (building_blocks.hpp:72-85), compute_borders_optional_zeros_rho
// (building_blocks.hpp:87-119) and compute_last_level_zeros
// (building_blocks.hpp:155-162).  The WM visits prefix blocks in bit-reversed
// order: the live rho of ctx_generic.hpp:41-67 equals reverse_bits(i, level)
// at level `level` (permutation.hpp:16-29).  `bv` holds levels*stride words
// in the flat layout, `zeros` receives all L zero counts for a WM.  Templated
// on the symbol type like pwm's (the sorted copy holds symbols, ps.hpp:18).
// When `level_hist` is given it also keeps pwm's hist_at_level(l) for every
// level (ctx_options::hist::all_level, ctx_generic.hpp:126-255):
// level_hist[l][x] = symbols whose l-bit prefix is x, level_hist[0][0] = n
// (ps.hpp:64); wx_dd_ps merges with them.
template <typename T>
int ps_core(const T* text, uint64_t n, uint32_t levels, int is_tree, uint64_t* bv, const uint64_t* offsets,
            uint64_t* zeros, std::vector<std::vector<uint64_t>>* level_hist) {
  if (n == 0 || levels == 0) return 0;  // wx_ps.hpp:39-45: empty structure
  const uint64_t sigma = 1ULL << levels;
  std::vector<uint64_t> hist(sigma, 0), next(sigma, 0), borders(sigma, 0);
  std::vector<T> sorted(n);
  // Hot loop 1: level-0 bits plus the leaf histogram.
  write_bits(bv + offsets[0], n, [&](uint64_t i) {
    const uint64_t c = text[i];
    ++hist[c];
    return (c >> (levels - 1)) & 1ULL;
  });
  if (level_hist) {
    level_hist->assign(levels + 1, std::vector<uint64_t>());
    (*level_hist)[levels] = hist;
    (*level_hist)[0].assign(1, n);
  }
  if (!is_tree) {
    for (uint32_t l = 0; l < levels; ++l) zeros[l] = 0;
    for (uint64_t c = 0; c < sigma; c += 2) zeros[levels - 1] += hist[c];
  }
  uint64_t cur = sigma;
  for (uint32_t level = levels - 1; level > 0; --level) {
    cur >>= 1;
    for (uint64_t i = 0; i < cur; ++i) next[i] = hist[2 * i] + hist[2 * i + 1];
    std::swap(hist, next);
    if (level_hist) (*level_hist)[level].assign(hist.begin(), hist.begin() + cur);
    // borders in rho order
    uint64_t run = 0;
    for (uint64_t i = 0; i < cur; ++i) {
      uint64_t block = is_tree ? i : reverse_bits(i, level);
      borders[block] = run;
      run += hist[block];
    }
    if (!is_tree) zeros[level - 1] = borders[1];
    // Hot loop 2: stable counting sort by the level-bit prefix.
    const uint32_t shift = levels - level;
    for (uint64_t i = 0; i < n; ++i) {
      const T c = text[i];
      sorted[borders[uint64_t(c) >> shift]++] = c;
    }
    // Hot loop 3: pack the bits of the sorted sequence.
    const uint32_t bit = levels - 1 - level;
    write_bits(bv + offsets[level], n, [&](uint64_t i) { return (uint64_t(sorted[i]) >> bit) & 1ULL; });
  }
  return 0;
}

int ps_dispatch(const void* text, uint64_t n, uint32_t w, uint32_t levels, int is_tree, uint64_t* bv,
                const uint64_t* offsets, uint64_t* zeros, std::vector<std::vector<uint64_t>>* level_hist) {
  switch (w) {
    case 1: return ps_core(static_cast<const uint8_t*>(text), n, levels, is_tree, bv, offsets, zeros, level_hist);
    case 2: return ps_core(static_cast<const uint16_t*>(text), n, levels, is_tree, bv, offsets, zeros, level_hist);
    case 4: return ps_core(static_cast<const uint32_t*>(text), n, levels, is_tree, bv, offsets, zeros, level_hist);
    default: return ps_core(static_cast<const uint64_t*>(text), n, levels, is_tree, bv, offsets, zeros, level_hist);
  }
}

// Bits [src_off, src_off + len) of `src` into bits [dst_off, dst_off + len)
// of `dst` (MSB-first positions), OR-ed into destination words that start
// zeroed.  Callers give each thread whole destination words.
void or_bits(uint64_t* dst, uint64_t dst_off, const uint64_t* src, uint64_t src_off, uint64_t len) {
  while (len) {
    const uint64_t d = dst_off & 63, take = std::min<uint64_t>(64 - d, len);
    // `take` source bits starting at src_off, left-aligned
    const uint64_t s = src_off & 63;
    uint64_t v = src[src_off >> 6] << s;
    if (s && s + take > 64) v |= src[(src_off >> 6) + 1] >> (64 - s);
    v &= take == 64 ? ~0ULL : ~(~0ULL >> take);
    dst[dst_off >> 6] |= v >> d;
    dst_off += take;
    src_off += take;
    len -= take;
  }
}

}  // namespace

extern "C" {

int orc_wx_ps(const void* text, uint64_t n, uint32_t w, uint32_t levels, int is_tree,
              uint64_t* bv, const uint64_t* offsets, uint64_t* zeros) {
  return ps_dispatch(text, n, w, levels, is_tree, bv, offsets, zeros, nullptr);
}

// Domain decomposition, restating wx_dd_ps::compute (include/wx_dd_ps.hpp:
// 43-120) with merge_bit_vectors (include/construction/merge.hpp:192-465):
// `threads` shards; shard s builds the slice of n/threads symbols (one more
// for each of the first n%threads shards, wx_dd_ps.hpp:79-83) with ps(),
// keeping every level's prefix histogram; level l of the result is, block by
// block in the level's order (prefix order for the tree, bit-reversed prefix
// order for the matrix: rho, permutation.hpp:16-29), the concatenation of
// the shards' runs of that block; the matrix zeros are the shards' sums
// (wx_dd_ps.hpp:106-113).  As in pwm, the merge splits the destination into
// word-aligned ranges, one per thread (merge.hpp:296-306); the bit copy is
// this file's own.  threads <= 1 is plain ps (wx_dd_ps.hpp:57-62).
int orc_wx_dd_ps(const void* text, uint64_t n, uint32_t w, uint32_t levels, int is_tree, uint64_t* bv,
                 const uint64_t* offsets, uint64_t* zeros, int threads) {
  if (n == 0 || levels == 0) return 0;
  if (threads <= 0) threads = omp_get_max_threads();
  if (threads <= 1) return ps_dispatch(text, n, w, levels, is_tree, bv, offsets, zeros, nullptr);
  const uint64_t shards = uint64_t(threads);
  struct Shard {
    uint64_t size = 0, begin = 0;
    std::vector<uint64_t> words, offs, zeros;
    std::vector<std::vector<uint64_t>> hist;
  };
  std::vector<Shard> sh(shards);
  for (uint64_t s = 0; s < shards; ++s) {
    sh[s].size = n / shards + (s < n % shards ? 1 : 0);
    sh[s].begin = s * (n / shards) + std::min<uint64_t>(s, n % shards);
  }
#pragma omp parallel for schedule(static, 1) num_threads(threads)
  for (int64_t si = 0; si < int64_t(shards); ++si) {
    Shard& x = sh[size_t(si)];
    x.offs.resize(levels);
    uint64_t total = 0;
    for (uint32_t l = 0; l < levels; ++l) { x.offs[l] = total; total += padded_words(x.size); }
    x.words.assign(std::max<uint64_t>(total, 1), 0);
    x.zeros.assign(levels, 0);
    x.hist.assign(levels + 1, std::vector<uint64_t>());
    if (x.size) {
      ps_dispatch(static_cast<const uint8_t*>(text) + x.begin * w, x.size, w, levels, is_tree, x.words.data(),
                  x.offs.data(), x.zeros.data(), &x.hist);
    } else {
      for (uint32_t l = 0; l <= levels; ++l) x.hist[l].assign(size_t(1) << l, 0);
    }
  }
  // per level: (destination bit, shard, source bit, length) of every
  // non-empty run, in destination order
  struct Seg { uint64_t dst, shard, src, len; };
  std::vector<std::vector<Seg>> segs(levels);
  for (uint32_t l = 0; l < levels; ++l) {
    std::vector<uint64_t> cursor(shards, 0);
    uint64_t dst = 0;
    const uint64_t blocks = uint64_t(1) << l;
    for (uint64_t b = 0; b < blocks; ++b) {
      const uint64_t prefix = is_tree ? b : reverse_bits(b, l);
      for (uint64_t s = 0; s < shards; ++s) {
        const uint64_t len = sh[s].hist[l][prefix];
        if (len) segs[l].push_back({dst, s, cursor[s], len});
        dst += len;
        cursor[s] += len;
      }
    }
  }
  const uint64_t nw = words_for(n);
#pragma omp parallel for schedule(static, 1) num_threads(threads)
  for (int64_t t = 0; t < int64_t(shards); ++t) {
    const uint64_t w0 = uint64_t(t) * (nw / shards) + std::min<uint64_t>(uint64_t(t), nw % shards);
    const uint64_t w1 = w0 + nw / shards + (uint64_t(t) < nw % shards ? 1 : 0);
    const uint64_t lo = w0 * 64, hi = std::min(w1 * 64, n);
    for (uint32_t l = 0; l < levels; ++l) {
      uint64_t* out = bv + offsets[l];
      std::memset(out + w0, 0, (w1 - w0) * 8);
      if (lo >= hi) continue;
      const auto& sg = segs[l];
      // first segment ending after lo
      size_t k = size_t(std::upper_bound(sg.begin(), sg.end(), lo,
                                         [](uint64_t v, const Seg& g) { return v < g.dst + g.len; }) - sg.begin());
      for (; k < sg.size() && sg[k].dst < hi; ++k) {
        const Seg& g = sg[k];
        const uint64_t a = std::max(g.dst, lo), e = std::min(g.dst + g.len, hi);
        const Shard& x = sh[g.shard];
        or_bits(out, a, x.words.data() + x.offs[l], g.src + (a - g.dst), e - a);
      }
    }
  }
  if (!is_tree) {
    for (uint32_t l = 0; l < levels; ++l) {
      zeros[l] = 0;
      for (uint64_t s = 0; s < shards; ++s) zeros[l] += sh[s].zeros[l];
    }
  }
  return 0;
}

// Seeded synthetic texts, identical to the GPU library's pwmgpu_generate
// (same header): dist 0 uniform over [0, param), 1 DNA-like, 2 Zipf(1.0) over
// 256 symbols permuted, 3 the 16-bit mixture.
void orc_generate(int dist, uint64_t seed, uint64_t param, uint64_t n, uint32_t w, void* out, int threads) {
  if (threads <= 0) threads = omp_get_max_threads();
  const pwmgpu::GenTables g = pwmgpu::gen_tables(dist, seed);
  const uint64_t key = pwmgpu::mix64(seed);
#pragma omp parallel for schedule(static) num_threads(threads)
  for (int64_t i = 0; i < int64_t(n); ++i) {
    const uint64_t v = pwmgpu::gen_value(dist, key, param, uint64_t(i), g.thr.data(), uint32_t(g.thr.size()),
                                         g.perm.data());
    if (w == 1) static_cast<uint8_t*>(out)[i] = uint8_t(v);
    else if (w == 2) static_cast<uint16_t*>(out)[i] = uint16_t(v);
    else static_cast<uint32_t*>(out)[i] = uint32_t(v);
  }
}

// The batched workload's texts (pwmgpu_generate_batch, same header).
void orc_generate_batch(uint64_t seed, uint32_t count, uint64_t* offsets, uint32_t* levels, uint8_t* texts) {
  pwmgpu::generate_batch_host(seed, count, offsets, levels, texts);
}

// Prefix counting, restating pc() (include/construction/pc.hpp:12-56): the
// bit of symbol c at level `level` is OR-ed into position borders[prefix]++
// (write_symbol_bit, building_blocks.hpp:139-153) of a zeroed level.
int orc_wx_pc(const void* text, uint64_t n, uint32_t w, uint32_t levels, int is_tree,
              uint64_t* bv, const uint64_t* offsets, uint64_t* zeros) {
  if (n == 0 || levels == 0) return 0;
  const uint64_t sigma = 1ULL << levels;
  std::vector<uint64_t> hist(sigma, 0), next(sigma, 0), borders(sigma, 0);
  write_bits(bv + offsets[0], n, [&](uint64_t i) {
    uint64_t c = sym_at(text, w, i);
    ++hist[c];
    return (c >> (levels - 1)) & 1ULL;
  });
  if (!is_tree) {
    for (uint32_t l = 0; l < levels; ++l) zeros[l] = 0;
    for (uint64_t c = 0; c < sigma; c += 2) zeros[levels - 1] += hist[c];
  }
  for (uint32_t level = 1; level < levels; ++level)
    std::memset(bv + offsets[level], 0, words_for(n) * 8);
  uint64_t cur = sigma;
  for (uint32_t level = levels - 1; level > 0; --level) {
    cur >>= 1;
    for (uint64_t i = 0; i < cur; ++i) next[i] = hist[2 * i] + hist[2 * i + 1];
    std::swap(hist, next);
    uint64_t run = 0;
    for (uint64_t i = 0; i < cur; ++i) {
      uint64_t block = is_tree ? i : reverse_bits(i, level);
      borders[block] = run;
      run += hist[block];
    }
    if (!is_tree) zeros[level - 1] = borders[1];
    uint64_t* lv = bv + offsets[level];
    const uint32_t pshift = levels - level, bshift = pshift - 1;
    for (uint64_t i = 0; i < n; ++i) {
      uint64_t c = sym_at(text, w, i);
      uint64_t pos = borders[c >> pshift]++;
      lv[pos >> 6] |= ((c >> bshift) & 1ULL) << (63 - (pos & 63));
    }
  }
  return 0;
}

// Naive construction, restating wx_naive (include/wx_naive.hpp:21-78 for the
// WT, :81-153 for the WM): per level the MSB-first bits of the current
// sequence, then a stable bucketing by the (level+1)-bit prefix (WT) or a
// stable 0/1 partition (WM); WM zeros are counted directly.
int orc_wx_naive(const void* text, uint64_t n, uint32_t w, uint32_t levels, int is_tree,
                 uint64_t* bv, const uint64_t* offsets, uint64_t* zeros) {
  if (n == 0 || levels == 0) return 0;
  std::vector<uint64_t> cur(n), tmp(n);
  for (uint64_t i = 0; i < n; ++i) cur[i] = sym_at(text, w, i);
  for (uint32_t level = 0; level < levels; ++level) {
    const uint32_t shift = levels - (level + 1);
    write_bits(bv + offsets[level], n, [&](uint64_t i) { return (cur[i] >> shift) & 1ULL; });
    if (is_tree) {
      if (level + 1 < levels) {
        // stable bucket sort by (level+1)-bit prefix
        const uint64_t buckets = 1ULL << (level + 1);
        std::vector<uint64_t> count(buckets + 1, 0);
        for (uint64_t i = 0; i < n; ++i) ++count[(cur[i] >> shift) + 1];
        for (uint64_t b = 0; b < buckets; ++b) count[b + 1] += count[b];
        for (uint64_t i = 0; i < n; ++i) tmp[count[cur[i] >> shift]++] = cur[i];
        std::swap(cur, tmp);
      }
    } else {
      uint64_t z = 0;
      for (uint64_t i = 0; i < n; ++i) z += !((cur[i] >> shift) & 1ULL);
      zeros[level] = z;
      if (level + 1 < levels) {
        uint64_t p0 = 0, p1 = z;
        for (uint64_t i = 0; i < n; ++i) {
          if ((cur[i] >> shift) & 1ULL) tmp[p1++] = cur[i]; else tmp[p0++] = cur[i];
        }
        std::swap(cur, tmp);
      }
    }
  }
  return 0;
}

// Parallel prefix counting, an OpenMP restatement of ppc()
// (include/construction/ppc.hpp:19-90) used as the CPU baseline: per-thread
// leaf histograms while writing level 0, level histograms folded from the
// leaves, then every level filled independently (one level per thread,
// dynamic schedule) with write_symbol_bit semantics.  Like pwm's wx_ppc it
// does not compute zeros[L-1] (left 0, see ppc.hpp:19-90).
}  // extern "C"

namespace {

template <typename T>
int ppc_core(const T* text, uint64_t n, uint32_t levels, int is_tree, uint64_t* bv, const uint64_t* offsets,
             uint64_t* zeros, int threads) {
  const uint64_t sigma = 1ULL << levels;
  const uint64_t nw = words_for(n);
  std::vector<std::vector<uint64_t>> local(threads, std::vector<uint64_t>(sigma, 0));
  uint64_t* l0 = bv + offsets[0];
#pragma omp parallel num_threads(threads)
  {
    auto& h = local[omp_get_thread_num()];
#pragma omp for schedule(static)
    for (int64_t wi = 0; wi < int64_t(nw); ++wi) {
      uint64_t start = uint64_t(wi) * 64, end = std::min(n, start + 64), word = 0;
      for (uint64_t i = start; i < end; ++i) {
        const uint64_t c = text[i];
        ++h[c];
        word = (word << 1) | ((c >> (levels - 1)) & 1ULL);
      }
      l0[wi] = word << (64 - (end - start));
    }
  }
  std::vector<std::vector<uint64_t>> hist(levels + 1);
  hist[levels].assign(sigma, 0);
  for (int t = 0; t < threads; ++t)
    for (uint64_t c = 0; c < sigma; ++c) hist[levels][c] += local[t][c];
  for (int l = int(levels) - 1; l >= 1; --l) {
    hist[l].assign(1ULL << l, 0);
    for (uint64_t i = 0; i < (1ULL << l); ++i) hist[l][i] = hist[l + 1][2 * i] + hist[l + 1][2 * i + 1];
  }
  if (!is_tree) for (uint32_t l = 0; l < levels; ++l) zeros[l] = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int level = 1; level < int(levels); ++level) {
    const uint64_t blocks = 1ULL << level;
    std::vector<uint64_t> borders(blocks, 0);
    uint64_t run = 0;
    for (uint64_t i = 0; i < blocks; ++i) {
      uint64_t block = is_tree ? i : reverse_bits(i, level);
      borders[block] = run;
      run += hist[level][block];
    }
    if (!is_tree) zeros[level - 1] = borders[1];
    uint64_t* lv = bv + offsets[level];
    std::memset(lv, 0, nw * 8);
    const uint32_t pshift = levels - level, bshift = pshift - 1;
    for (uint64_t i = 0; i < n; ++i) {
      const uint64_t c = text[i];
      uint64_t pos = borders[c >> pshift]++;
      lv[pos >> 6] |= ((c >> bshift) & 1ULL) << (63 - (pos & 63));
    }
  }
  return 0;
}

}  // namespace

extern "C" {

int orc_wx_ppc(const void* text, uint64_t n, uint32_t w, uint32_t levels, int is_tree,
               uint64_t* bv, const uint64_t* offsets, uint64_t* zeros, int threads) {
  if (n == 0 || levels == 0) return 0;
  if (threads <= 0) threads = omp_get_max_threads();
  switch (w) {
    case 1: return ppc_core(static_cast<const uint8_t*>(text), n, levels, is_tree, bv, offsets, zeros, threads);
    case 2: return ppc_core(static_cast<const uint16_t*>(text), n, levels, is_tree, bv, offsets, zeros, threads);
    case 4: return ppc_core(static_cast<const uint32_t*>(text), n, levels, is_tree, bv, offsets, zeros, threads);
    default: return ppc_core(static_cast<const uint64_t*>(text), n, levels, is_tree, bv, offsets, zeros, threads);
  }
}

// ---------------------------------------------------------------------------
// Rank / select (Zhou-Andersen-Kaminsky popcount layout)
// ---------------------------------------------------------------------------
// popcnt_traits (include/queries/popcnt_traits.hpp:12-21): L2 = 512 bits
// (8 words), L1 = 2048 bits (32 words), L0 = 2^32-1 bits; the "block cover"
// constants are those bit sizes divided by 64 (integer division).
static const uint64_t kL2Bits = 512, kL1Bits = 2048, kL0Bits = 4294967295ULL;
static const uint64_t kL2Cover = 8, kL1Cover = 32, kL0Cover = 4294967295ULL / 64;
static const uint64_t kSampleRate = 8192;  // bin_select_popcnt.hpp:244

uint64_t orc_rank_l0_size(uint64_t nwords) { return nwords / kL0Cover + 1; }
uint64_t orc_rank_l12_size(uint64_t nwords) { return nwords / kL1Cover + 1; }

// bin_rank_popcnt constructor (include/queries/bin_rank_popcnt.hpp:54-86).
// l12 holds pairs of u32 {l1 cumulative count, three 10-bit L2 counts}
// (l12_entry, bin_rank_popcnt.hpp:32-47); entries past the loop stay zero.
void orc_rank_build(const uint64_t* data, uint64_t nwords, uint64_t* l0, uint32_t* l12) {
  const uint64_t n0 = orc_rank_l0_size(nwords), n12 = orc_rank_l12_size(nwords);
  std::memset(l0, 0, n0 * 8);
  std::memset(l12, 0, n12 * 8);
  uint64_t l0_pos = 0, l12_pos = 0, pos = 0;
  uint32_t l1_entry = 0;
  while (pos < nwords) {
    uint32_t new_l1 = l1_entry;
    uint32_t l2[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i) {
      for (uint64_t j = 0; j < kL2Cover && pos < nwords; ++j) l2[i] += __builtin_popcountll(data[pos++]);
      new_l1 += l2[i];
    }
    l12[2 * l12_pos] = l1_entry;
    l12[2 * l12_pos + 1] = (l2[0] & 1023u) | ((l2[1] & 1023u) << 10) | ((l2[2] & 1023u) << 20);
    ++l12_pos;
    l1_entry = new_l1;
    for (uint64_t j = 0; j < kL2Cover && pos < nwords; ++j) l1_entry += __builtin_popcountll(data[pos++]);
    if (l12_pos % kL0Cover == 0) {
      if (l0_pos > 0) l0[l0_pos] += l0[l0_pos - 1];
      l0[l0_pos++] += l1_entry;
      l1_entry = 0;
    }
  }
}

static inline uint32_t l2_of(const uint32_t* l12, uint64_t e, uint64_t i) {
  return (l12[2 * e + 1] >> (10 * i)) & 1023u;
}

// Number of real L1 blocks of a level; pwm's l12_ has one more, zeroed,
// entry when nwords is a multiple of 32 (bin_rank_popcnt.hpp:56, 63-85).
static inline uint64_t real_l1_blocks(uint64_t nwords) { return (nwords + kL1Cover - 1) / kL1Cover; }

// Total number of ones of a level, from its last real L1 entry.
uint64_t orc_total_ones(const uint64_t* data, uint64_t nwords, const uint32_t* l12) {
  if (nwords == 0) return 0;
  uint64_t last = real_l1_blocks(nwords) - 1, t = l12[2 * last];
  for (uint64_t w = last * kL1Cover; w < nwords; ++w) t += __builtin_popcountll(data[w]);
  return t;
}

// bin_rank_popcnt::rank1 (bin_rank_popcnt.hpp:98-128).  pwm answers
// rank1(n) with the zeroed extra L1 entry (0) when the level has a multiple
// of 2048 bits; here that index returns the level's total count `ones`
// instead.  Every other index gives pwm's value.
uint64_t orc_rank1(const uint64_t* data, uint64_t nwords, const uint64_t* l0, const uint32_t* l12, uint64_t ones,
                   uint64_t index) {
  uint64_t result = 0, rem = index;
  uint64_t l0_pos = rem / kL0Bits;
  rem -= l0_pos * kL0Bits;
  if (l0_pos > 0) result += l0[l0_pos - 1];
  uint64_t l1_pos = rem / kL1Bits;
  rem -= l1_pos * kL1Bits;
  if (l1_pos >= real_l1_blocks(nwords)) return ones;
  result += l12[2 * l1_pos];
  uint64_t l2_pos = rem / kL2Bits;
  rem -= l2_pos * kL2Bits;
  for (uint64_t i = 0; i < l2_pos; ++i) result += l2_of(l12, l1_pos, i);
  uint64_t off = l1_pos * kL1Cover + l2_pos * kL2Cover;
  while (rem >= 64) { result += __builtin_popcountll(data[off++]); rem -= 64; }
  if (rem > 0) result += __builtin_popcountll(data[off] >> (64 - rem));
  return result;
}

// Select the position (counted from the most significant bit) of the bit
// with the given 1-based rank inside a word.  This is the published
// branch-free "select the bit position with the given count" method from
// Sean Eron Anderson's Bit Twiddling Hacks, which pwm uses in
// bin_select_popcnt::word_select1 (bin_select_popcnt.hpp:123-164);
// restated step by step so that out-of-range ranks give the same value.
uint32_t orc_word_select1(uint64_t v, uint32_t rank) {
  const uint64_t m1 = ~0ULL / 3, m2 = ~0ULL / 5, m4 = ~0ULL / 0x11, m8 = ~0ULL / 0x101;
  unsigned r = rank;
  uint64_t a = v - ((v >> 1) & m1);
  uint64_t b = (a & m2) + ((a >> 2) & m2);
  uint64_t c = (b + (b >> 4)) & m4;
  uint64_t d = (c + (c >> 8)) & m8;
  unsigned t = unsigned((d >> 32) + (d >> 48));
  unsigned s = 64;
  s -= ((t - r) & 256) >> 3; r -= (t & ((t - r) >> 8));
  t = unsigned((d >> (s - 16)) & 0xff);
  s -= ((t - r) & 256) >> 4; r -= (t & ((t - r) >> 8));
  t = unsigned((c >> (s - 8)) & 0xf);
  s -= ((t - r) & 256) >> 5; r -= (t & ((t - r) >> 8));
  t = unsigned((b >> (s - 4)) & 0x7);
  s -= ((t - r) & 256) >> 6; r -= (t & ((t - r) >> 8));
  t = unsigned((a >> (s - 2)) & 0x3);
  s -= ((t - r) & 256) >> 7; r -= (t & ((t - r) >> 8));
  t = unsigned((v >> (s - 1)) & 0x1);
  s -= ((t - r) & 256) >> 8;
  return 64 - s;
}

// bin_select_popcnt constructor (bin_select_popcnt.hpp:38-107), select value
// 0 or 1: one sample (u32 position) every 8192 zeros/ones, taken in the L1
// block where the running count first exceeds the next sample number.
// Returns the number of samples; `samples` must hold at least
// nwords*64/8192 + 2 entries.
uint64_t orc_select_build(int value, const uint64_t* data, uint64_t nwords, const uint32_t* l12,
                          uint32_t* samples) {
  const uint64_t n12 = orc_rank_l12_size(nwords);
  uint64_t count = 0, next = 1, l0_pos = 0;
  for (uint64_t l1 = 0; l1 + 1 < n12;) {
    if (value == 0) {
      if (((l1 + 1) * kL1Bits) - l12[2 * (l1 + 1)] > next) {
        uint32_t rem = uint32_t(next - ((l1 * kL1Bits) - l12[2 * l1]));
        uint64_t l2 = 0;
        while (l2 < 3 && (kL2Bits - l2_of(l12, l1, l2)) < rem) rem -= uint32_t(kL2Bits - l2_of(l12, l1, l2++));
        uint64_t wp = l0_pos * kL0Cover + l1 * kL1Cover + l2 * kL2Cover;
        while (wp < nwords && rem > uint32_t(__builtin_popcountll(~data[wp]))) rem -= __builtin_popcountll(~data[wp++]);
        if (wp < nwords) {
          samples[count++] = uint32_t(orc_word_select1(~data[wp], rem) + 64 * (wp - (l0_pos * kL0Bits)));
          next += kSampleRate;
        }
      }
    } else {
      if (l12[2 * (l1 + 1)] > next) {
        uint32_t rem = uint32_t(next - l12[2 * l1]);
        uint64_t l2 = 0;
        while (l2 < 3 && l2_of(l12, l1, l2) < rem) rem -= l2_of(l12, l1, l2++);
        uint64_t wp = l0_pos * kL0Cover + l1 * kL1Cover + l2 * kL2Cover;
        while (wp < nwords && rem > uint32_t(__builtin_popcountll(data[wp]))) rem -= __builtin_popcountll(data[wp++]);
        if (wp < nwords) {
          samples[count++] = uint32_t(orc_word_select1(data[wp], rem) + 64 * (wp - (l0_pos * kL0Bits)));
          next += kSampleRate;
        }
      }
    }
    if (++l1 % kL0Cover == 0) ++l0_pos;
  }
  return count;
}

// bin_select_popcnt::select0/select1 (bin_select_popcnt.hpp:112-117,
// 166-241).  occ == 0 gives 0.
//
// Where pwm is defined this returns pwm's value bit for bit, including the
// direct return of a sample for occ = 8192k+1.  pwm has two undefined cases,
// both reads past an array: (a) samples_[occ/8192] beyond the sample table
// (always the case for bit vectors shorter than two L1 blocks), and (b) for
// occ = 8192k, a sample whose L1 block lies past the occ-th bit, after which
// the count underflows and the word walk runs off the data.  Here the block
// scan starts at sample (occ-1)/8192 (the same block for every defined case)
// or, past the table, at the last sample (block 0 without samples), which
// gives the correct position.  The forward block scan stops at the last
// real L1 block (pwm steps onto its zeroed extra entry there and then reads
// past the data).  An occurrence beyond the (padded) count returns
// UINT64_MAX instead of reading past the words.
uint64_t orc_select(int value, const uint64_t* data, uint64_t nwords, const uint64_t* l0, uint64_t n0,
                    const uint32_t* l12, const uint32_t* samples, uint64_t nsamples, uint64_t occ) {
  if (occ == 0) return 0;
  const uint64_t n12 = real_l1_blocks(nwords);
  uint64_t l0_pos = 0;
  while (l0_pos + 1 < n0 && l0[l0_pos + 1] < occ) ++l0_pos;
  occ -= l0[l0_pos];
  uint64_t l1;
  const uint64_t sidx = (occ - 1) / kSampleRate;
  if (sidx < nsamples) {
    l1 = samples[sidx];
    if ((occ - 1) % kSampleRate == 0) return l1;
    l1 /= kL1Bits;
  } else {
    l1 = nsamples ? samples[nsamples - 1] / kL1Bits : 0;
  }
  if (value == 0) {
    while (l1 + 1 < n12 && (((l1 + 1) * kL1Bits) - l12[2 * (l1 + 1)]) < occ) ++l1;
    occ -= (l1 * kL1Bits) - l12[2 * l1];
  } else {
    while (l1 + 1 < n12 && l12[2 * (l1 + 1)] < occ) ++l1;
    occ -= l12[2 * l1];
  }
  uint64_t l2 = 0;
  if (value == 0) {
    while (l2 < 3 && occ > kL2Bits - l2_of(l12, l1, l2)) occ -= kL2Bits - l2_of(l12, l1, l2++);
  } else {
    while (l2 < 3 && occ > l2_of(l12, l1, l2)) occ -= l2_of(l12, l1, l2++);
  }
  uint64_t last = kL2Cover * l2 + kL1Cover * l1 + kL0Cover * l0_pos;
  uint64_t extra = 0, pc = 0;
  for (;;) {
    if (last + extra >= nwords) return UINT64_MAX;
    uint64_t word = data[last + extra];
    if (value == 0) word = ~word;
    pc = __builtin_popcountll(word);
    if (pc >= occ) break;
    ++extra;
    occ -= pc;
  }
  uint64_t word = data[last + extra];
  if (value == 0) word = ~word;
  return kL2Bits * l2 + kL1Bits * l1 + kL0Bits * l0_pos + extra * 64 + orc_word_select1(word, uint32_t(occ));
}

// ---------------------------------------------------------------------------
// Queries over a whole structure (include/queries/query_support.hpp:18-186)
// ---------------------------------------------------------------------------
struct orc_qs_level {
  const uint64_t* data;
  uint64_t nwords, n0, ns0, ns1, ones;
  std::vector<uint64_t> l0;
  std::vector<uint32_t> l12, s0, s1;
  uint64_t rank1(uint64_t i) const { return orc_rank1(data, nwords, l0.data(), l12.data(), ones, i); }
  uint64_t rank0(uint64_t i) const { return i - rank1(i); }
  uint64_t select(int v, uint64_t occ) const {
    return orc_select(v, data, nwords, l0.data(), n0, l12.data(), v ? s1.data() : s0.data(), v ? ns1 : ns0, occ);
  }
};

struct orc_qs {
  uint32_t levels;
  int is_tree;
  uint64_t n;
  std::vector<uint64_t> zeros;
  std::vector<orc_qs_level> lv;
};

// query_support constructor (query_support.hpp:24-30): rank and both select
// supports for every level over ceil(n/64) words.
void* orc_qs_create(uint32_t levels, int is_tree, uint64_t n, const uint64_t* bv, const uint64_t* offsets,
                    const uint64_t* zeros) {
  auto* q = new orc_qs;
  q->levels = levels;
  q->is_tree = is_tree;
  q->n = n;
  if (!is_tree) q->zeros.assign(zeros, zeros + levels);
  q->lv.resize(levels);
  for (uint32_t l = 0; l < levels; ++l) {
    auto& L = q->lv[l];
    L.data = bv + offsets[l];
    L.nwords = words_for(n);
    L.n0 = orc_rank_l0_size(L.nwords);
    L.l0.resize(L.n0);
    L.l12.resize(2 * orc_rank_l12_size(L.nwords));
    orc_rank_build(L.data, L.nwords, L.l0.data(), L.l12.data());
    L.s0.resize(L.nwords * 64 / kSampleRate + 2);
    L.s1.resize(L.nwords * 64 / kSampleRate + 2);
    L.ns0 = orc_select_build(0, L.data, L.nwords, L.l12.data(), L.s0.data());
    L.ns1 = orc_select_build(1, L.data, L.nwords, L.l12.data(), L.s1.data());
    L.ones = orc_total_ones(L.data, L.nwords, L.l12.data());
  }
  return q;
}

void orc_qs_free(void* q) { delete static_cast<orc_qs*>(q); }

// Rank/select blocks of one level, for comparing layouts.
uint64_t orc_qs_blocks(void* qp, uint32_t level, uint64_t* l0, uint32_t* l12, uint32_t* s0, uint32_t* s1,
                       uint64_t* counts /* n0, n12, ns0, ns1 */) {
  auto* q = static_cast<orc_qs*>(qp);
  auto& L = q->lv[level];
  counts[0] = L.n0;
  counts[1] = L.l12.size() / 2;
  counts[2] = L.ns0;
  counts[3] = L.ns1;
  if (l0) std::memcpy(l0, L.l0.data(), L.n0 * 8);
  if (l12) std::memcpy(l12, L.l12.data(), L.l12.size() * 4);
  if (s0) std::memcpy(s0, L.s0.data(), L.ns0 * 4);
  if (s1) std::memcpy(s1, L.s1.data(), L.ns1 * 4);
  return 0;
}

// access (query_support.hpp:39-46, access_tree :72-91, access_matrix :93-104)
uint64_t orc_qs_access(void* qp, uint64_t index) {
  auto* q = static_cast<orc_qs*>(qp);
  uint64_t word = 0;
  if (q->is_tree) {
    uint64_t start = 0, end = q->n;
    for (uint32_t level = 0; level < q->levels; ++level) {
      const auto& L = q->lv[level];
      uint64_t left = L.rank0(start), right = L.rank0(end);
      word <<= 1;
      if (bit_at(L.data, start + index)) {
        word |= 1;
        uint64_t off = L.rank1(start + index);
        index = off - (start - left);
        start = start + right - left;
      } else {
        uint64_t off = L.rank0(start + index);
        index = off - left;
        end = start + right - left;
      }
    }
  } else {
    for (uint32_t level = 0; level < q->levels; ++level) {
      const auto& L = q->lv[level];
      word <<= 1;
      if (bit_at(L.data, index)) {
        word |= 1;
        index = L.rank1(index) + q->zeros[level];
      } else {
        index = L.rank0(index);
      }
    }
  }
  return word;
}

// rank (query_support.hpp:48-58, rank_tree :106-125, rank_matrix :127-140).
// pwm takes a uint8_t symbol; this restatement takes the full symbol.
uint64_t orc_qs_rank(void* qp, uint64_t symbol, uint64_t index) {
  auto* q = static_cast<orc_qs*>(qp);
  if (index == 0) return 0;
  if (q->is_tree) {
    uint64_t start = 0, end = q->n;
    for (uint32_t level = 0; level < q->levels; ++level) {
      const auto& L = q->lv[level];
      uint64_t left = L.rank0(start), right = L.rank0(end);
      if ((symbol >> (q->levels - level - 1)) & 1) {
        uint64_t off = L.rank1(start + index);
        index = off - (start - left);
        start = start + right - left;
      } else {
        uint64_t off = L.rank0(start + index);
        index = off - left;
        end = start + right - left;
      }
    }
    return index;
  }
  uint64_t offset = 0;
  for (uint32_t level = 0; level < q->levels; ++level) {
    const auto& L = q->lv[level];
    if ((symbol >> (q->levels - level - 1)) & 1) {
      index = q->zeros[level] + L.rank1(index);
      offset = q->zeros[level] + L.rank1(offset);
    } else {
      index = L.rank0(index);
      offset = L.rank0(offset);
    }
  }
  return index - offset;
}

// select (query_support.hpp:60-70, select_tree :142-161, select_matrix
// :163-178): descend computing the node ranges, then map the occurrence back
// up level by level.
uint64_t orc_qs_select(void* qp, uint64_t symbol, uint64_t occ) {
  auto* q = static_cast<orc_qs*>(qp);
  if (occ == 0) return 0;
  const uint32_t L = q->levels;
  if (q->is_tree) {
    std::vector<uint64_t> st(L), le(L), ri(L);
    uint64_t start = 0, end = q->n;
    for (uint32_t level = 0; level < L; ++level) {
      const auto& lv = q->lv[level];
      uint64_t left = lv.rank0(start), right = lv.rank0(end);
      st[level] = start; le[level] = left; ri[level] = right;
      if ((symbol >> (L - level - 1)) & 1) start = start + right - left;
      else end = start + right - left;
    }
    for (int level = int(L) - 1; level >= 0; --level) {
      const auto& lv = q->lv[level];
      uint64_t start_l = st[level], left = le[level];
      if ((symbol >> (L - level - 1)) & 1) occ = lv.select(1, start_l - left + occ) - start_l + (level == 0 ? 0 : 1);
      else occ = lv.select(0, left + occ) - start_l + (level == 0 ? 0 : 1);
    }
    return occ;
  }
  std::vector<uint64_t> offs(L);
  uint64_t offset = 0;
  for (uint32_t level = 0; level < L; ++level) {
    const auto& lv = q->lv[level];
    if ((symbol >> (L - level - 1)) & 1) offset = q->zeros[level] + lv.rank1(offset);
    else offset = lv.rank0(offset);
    offs[level] = offset;
  }
  occ = occ + offset;
  for (int level = int(L) - 1; level >= 0; --level) {
    const auto& lv = q->lv[level];
    if ((symbol >> (L - level - 1)) & 1) occ = lv.select(1, occ - q->zeros[level]) + (level == 0 ? 0 : 1);
    else occ = lv.select(0, occ) + (level == 0 ? 0 : 1);
  }
  return occ;
}

// ---------------------------------------------------------------------------
// Huffman shaping
// ---------------------------------------------------------------------------

// Canonical Huffman codes, restating histogram (include/util/histogram.hpp:
// 39-76), level_sizes_builder (include/huffman/huff_level_sizes_builder.hpp:
// 13-46) and canonical_huff_codes::compute_codes (include/huffman/
// huff_codes.hpp:140-285).  The tie-breaking of the reference comes from
// std::priority_queue, std::sort and (for symbols wider than 8 bits) the
// iteration order of std::unordered_map; the same standard containers are
// used here with the same insertion sequences.
// code_len/code_word receive max_symbol+1 entries (max_symbols is the
// capacity); level_sizes receives `levels` entries.  Returns max_symbol+1, or
// 0 for an empty text.
uint64_t orc_huff_codes(const void* text, uint64_t n, uint32_t w, int is_tree, uint64_t* code_len,
                        uint64_t* code_word, uint64_t max_symbols, uint64_t* level_sizes, uint32_t* levels_out) {
  *levels_out = 0;
  if (n == 0) return 0;
  std::vector<std::pair<uint64_t, uint64_t>> hist;  // (symbol, frequency) in histogram order
  uint64_t max_symbol = 0;
  if (w == 1) {
    std::vector<uint64_t> h(256, 0);
    for (uint64_t i = 0; i < n; ++i) {
      uint64_t c = sym_at(text, w, i);
      max_symbol = std::max(max_symbol, c);
      ++h[c];
    }
    for (uint64_t c = 0; c < 256; ++c) if (h[c]) hist.emplace_back(c, h[c]);
  } else {
    auto run = [&](auto tag) {
      using A = decltype(tag);
      std::unordered_map<A, uint64_t> m;
      for (uint64_t i = 0; i < n; ++i) {
        A c = A(sym_at(text, w, i));
        max_symbol = std::max<uint64_t>(max_symbol, c);
        auto it = m.find(c);
        if (it == m.end()) m.emplace(c, 1); else ++it->second;
      }
      for (const auto& e : m) hist.emplace_back(uint64_t(e.first), e.second);
    };
    if (w == 2) run(uint16_t(0)); else run(uint32_t(0));
  }
  const uint64_t nsym = max_symbol + 1;
  if (nsym > max_symbols) return 0;
  auto freq_of = [&](uint64_t s) {
    for (const auto& e : hist) if (e.first == s) return e.second;
    return uint64_t(0);
  };
  struct item {
    uint64_t occ;
    std::vector<uint64_t> syms;
    bool operator>(const item& o) const { return occ > o.occ; }
  };
  std::priority_queue<item, std::vector<item>, std::greater<item>> pq;
  std::vector<uint64_t> len(nsym, 0), word(nsym, 0);
  for (const auto& e : hist) pq.emplace(item{e.second, std::vector<uint64_t>{e.first}});
  if (pq.size() == 1) ++len[pq.top().syms.front()];
  while (pq.size() > 1) {
    auto a = pq.top(); pq.pop();
    auto b = pq.top(); pq.pop();
    std::move(b.syms.begin(), b.syms.end(), std::back_inserter(a.syms));
    for (auto c : a.syms) ++len[c];
    pq.emplace(item{a.occ + b.occ, a.syms});
  }
  std::vector<uint64_t> order(nsym);
  for (uint64_t i = 0; i < nsym; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) { return len[a] < len[b]; });
  const uint64_t levels = len[order.back()];
  std::vector<uint64_t> sizes(levels, 0);
  uint64_t k = 0;
  while (k < nsym && len[order[k]] == 0) ++k;
  if (!is_tree) {
    uint64_t cur = 1;
    std::vector<uint64_t> words{0, 1};
    while (k < nsym) {
      if (len[order[k]] > cur) {
        for (uint64_t i = cur; i < len[order[k]]; ++i) {
          std::vector<uint64_t> nw;
          nw.reserve(words.size() * 2);
          for (auto cw : words) nw.push_back(cw << 1);
          for (auto cw : words) nw.push_back((cw << 1) + 1);
          words = std::move(nw);
        }
        cur = len[order[k]];
      }
      while (k < nsym && len[order[k]] == cur) {
        uint64_t s = order[k++];
        word[s] = words.back();
        words.pop_back();
        sizes[len[s] - 1] += freq_of(s);
      }
    }
  } else {
    uint64_t cw = 0;
    auto gen = [&]() {
      uint64_t s = order[k];
      word[s] = (~cw) & ((1ULL << len[s]) - 1);
      sizes[len[s] - 1] += freq_of(s);
    };
    gen();
    for (++k; k < nsym; ++k) {
      cw = (cw + 1) << (len[order[k]] - len[order[k - 1]]);
      gen();
    }
  }
  for (uint64_t i = levels - 1; i > 0; --i) sizes[i - 1] += sizes[i];
  for (uint64_t s = 0; s < nsym; ++s) { code_len[s] = len[s]; code_word[s] = word[s]; }
  for (uint64_t l = 0; l < levels; ++l) level_sizes[l] = sizes[l];
  *levels_out = uint32_t(levels);
  return nsym;
}

// Huffman-shaped construction, restating huff_naive (include/huffman/
// huff_naive.hpp:19-126): level l holds bit l of every code that is longer
// than l; the WT keeps the next level stably bucketed by the (l+1)-bit code
// prefix, the WM by the current bit; WM zeros count the 0 bits of each level.
int orc_huff_naive(const void* text, uint64_t n, uint32_t w, int is_tree, const uint64_t* code_len,
                   const uint64_t* code_word, uint32_t levels, uint64_t* bv, const uint64_t* offsets,
                   uint64_t* zeros) {
  if (n == 0) return 0;
  std::vector<uint64_t> cur(n);
  for (uint64_t i = 0; i < n; ++i) cur[i] = sym_at(text, w, i);
  if (!is_tree) for (uint32_t l = 0; l < levels; ++l) zeros[l] = 0;
  auto bit = [&](uint64_t s, uint32_t level) { return (code_word[s] >> (code_len[s] - 1 - level)) & 1ULL; };
  for (uint32_t level = 0; level < levels; ++level) {
    const uint64_t size = cur.size();
    write_bits(bv + offsets[level], size, [&](uint64_t i) { return bit(cur[i], level); });
    if (!is_tree) {
      uint64_t z = 0;
      for (uint64_t i = 0; i < size; ++i) z += !bit(cur[i], level);
      zeros[level] = z;
    }
    std::vector<uint64_t> nxt;
    nxt.reserve(size);
    if (is_tree) {
      std::map<uint64_t, std::vector<uint64_t>> buckets;
      for (auto s : cur)
        if (code_len[s] > level + 1) buckets[code_word[s] >> (code_len[s] - (level + 1))].push_back(s);
      for (auto& b : buckets) nxt.insert(nxt.end(), b.second.begin(), b.second.end());
    } else {
      for (auto s : cur) if (code_len[s] > level + 1 && !bit(s, level)) nxt.push_back(s);
      for (auto s : cur) if (code_len[s] > level + 1 && bit(s, level)) nxt.push_back(s);
    }
    cur.swap(nxt);
  }
  return 0;
}

// Text reconstruction (include/util/decode.hpp:18-97 restated through the
// query recursion): decodes every position with access.  Test support.
void orc_decode(void* qp, uint64_t* out) {
  auto* q = static_cast<orc_qs*>(qp);
  for (uint64_t i = 0; i < q->n; ++i) out[i] = orc_qs_access(q, i);
}

}  // extern "C"

// pwm's copy_bits (include/construction/merge.hpp:19-190), the bit-range copy
// of the domain-decomposition merge: `len` bits from bit src_off of src to
// bit dst_off of dst (bit i of a word array is bit BITS-1-i%BITS of word
// i/BITS).  The destination words the range covers whole are stored; the
// partial words at its ends are OR-ed bit by bit.
template <typename W>
static void orc_copy_bits_t(W* dst, const W* src, uint64_t dst_off, uint64_t src_off, uint64_t len) {
  constexpr uint64_t B = sizeof(W) * 8;
  auto bit = [&](uint64_t i) -> W { return W((src[i / B] >> (B - 1 - i % B)) & 1u); };
  const uint64_t end = dst_off + len;
  while (dst_off % B != 0 && dst_off != end) {
    dst[dst_off / B] |= W(bit(src_off++) << (B - 1 - dst_off % B));
    ++dst_off;
  }
  while (end - dst_off >= B) {
    W v = 0;
    for (uint64_t k = 0; k < B; ++k) v = W((v << 1) | bit(src_off + k));
    dst[dst_off / B] = v;
    dst_off += B;
    src_off += B;
  }
  while (dst_off != end) {
    dst[dst_off / B] |= W(bit(src_off++) << (B - 1 - dst_off % B));
    ++dst_off;
  }
}

extern "C" {

void orc_copy_bits_u8(uint8_t* dst, const uint8_t* src, uint64_t dst_off, uint64_t src_off, uint64_t len) {
  orc_copy_bits_t(dst, src, dst_off, src_off, len);
}
void orc_copy_bits_u64(uint64_t* dst, const uint64_t* src, uint64_t dst_off, uint64_t src_off, uint64_t len) {
  orc_copy_bits_t(dst, src, dst_off, src_off, len);
}

// CPU-baseline step (bench.py's cpu_baseline leg and `--impl reference`):
// wavelet matrix and wavelet tree with pwm's parallel prefix counting
// (variant 0, orc_wx_ppc) or its domain decomposition (variant 1,
// orc_wx_dd_ps), then rank/select support (bin_rank_popcnt + both
// bin_select_popcnt) for every level of both, levels in parallel.  wm/wt hold
// levels*stride words each.
int orc_cpu_step(const void* text, uint64_t n, uint32_t w, uint32_t levels, int threads, uint64_t* wm,
                 uint64_t* wt, const uint64_t* offsets, uint64_t* zeros, int variant) {
  if (threads <= 0) threads = omp_get_max_threads();
  if (variant == 1) {
    orc_wx_dd_ps(text, n, w, levels, 0, wm, offsets, zeros, threads);
    orc_wx_dd_ps(text, n, w, levels, 1, wt, offsets, nullptr, threads);
  } else {
    orc_wx_ppc(text, n, w, levels, 0, wm, offsets, zeros, threads);
    orc_wx_ppc(text, n, w, levels, 1, wt, offsets, nullptr, threads);
  }
  const uint64_t nw = words_for(n);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int job = 0; job < int(2 * levels); ++job) {
    const uint64_t* data = (job < int(levels) ? wm : wt) + offsets[job % levels];
    std::vector<uint64_t> l0(orc_rank_l0_size(nw));
    std::vector<uint32_t> l12(2 * orc_rank_l12_size(nw)), s(nw * 64 / 8192 + 2);
    orc_rank_build(data, nw, l0.data(), l12.data());
    orc_select_build(0, data, nw, l12.data(), s.data());
    orc_select_build(1, data, nw, l12.data(), s.data());
  }
  return 0;
}

}  // extern "C"
