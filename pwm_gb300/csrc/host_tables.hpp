// Host-side O(2^L) and O(sigma * L) tables of a build: zero counts, the run
// starts of every split pass and the prefix-group segments that turn matrix
// levels into tree levels.  Pure integer code shared by the plain and the
// Huffman paths.
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "tile_layout.hpp"

namespace pwmgpu {

struct PassPlan {
  uint32_t level;  // first level of the pass
  int K;           // levels of the pass
  bool has_out;    // writes S_{level+K}
};

// Passes of up to kmax levels covering levels 0..L-1.
inline std::vector<PassPlan> plan_passes(uint32_t L, int kmax) {
  std::vector<PassPlan> p;
  for (uint32_t l = 0; l < L;) {
    int K = int(std::min<uint32_t>(uint32_t(kmax), L - l));
    p.push_back({l, K, l + K < L});
    l += uint32_t(K);
  }
  return p;
}

// The low `bits` bits of v reversed (bits <= 32), by byte table.
inline uint32_t rev_bits_host(uint64_t v, uint32_t bits) {
  static const auto table = []() {
    std::array<uint8_t, 256> t{};
    for (uint32_t b = 0; b < 256; ++b) {
      uint32_t r = 0;
      for (uint32_t i = 0; i < 8; ++i) r |= ((b >> i) & 1u) << (7 - i);
      t[b] = uint8_t(r);
    }
    return t;
  }();
  if (bits == 0) return 0;
  const uint32_t x = uint32_t(v);
  const uint32_t r = (uint32_t(table[x & 0xFF]) << 24) | (uint32_t(table[(x >> 8) & 0xFF]) << 16) |
                     (uint32_t(table[(x >> 16) & 0xFF]) << 8) | uint32_t(table[x >> 24]);
  return r >> (32 - bits);
}

// One weighted "code" of the text: the bits the levels test, its length
// (levels it is present on) and how often it occurs.  Plain symbols are codes
// of length L (the symbol's L low bits, MSB first).
struct WeightedCode {
  uint64_t word;   // code bits, MSB = level 0, right-aligned in `len` bits
  uint32_t len;
  uint64_t freq;
};

struct LevelTables {
  std::vector<uint64_t> zeros;                 // per level
  std::vector<uint64_t> level_bits;            // elements per level
  std::vector<std::vector<uint64_t>> starts;   // per pass: sum_j 2^j entries, j-major
  std::vector<std::vector<uint64_t>> seg_tree, seg_matrix;  // per level (level 0 unused)
};

inline uint32_t code_bit(const WeightedCode& c, uint32_t level) { return uint32_t(c.word >> (c.len - 1 - level)) & 1u; }

// Tables of a plain text from its leaf histogram (2^L counts): dense
// per-level prefix counts folded from the leaves.
inline LevelTables build_tables_plain(const std::vector<uint64_t>& hist, uint32_t L, const std::vector<PassPlan>& plan,
                                      bool want_tree) {
  LevelTables t;
  std::vector<std::vector<uint64_t>> cnt(L + 1);
  cnt[L] = hist;
  for (int m = int(L) - 1; m >= 0; --m) {
    cnt[m].assign(size_t(1) << m, 0);
    for (size_t p = 0; p < cnt[m].size(); ++p) cnt[m][p] = cnt[m + 1][2 * p] + cnt[m + 1][2 * p + 1];
  }
  const uint64_t n = cnt[0][0];
  t.level_bits.assign(L, n);
  t.zeros.assign(L, 0);
  for (uint32_t m = 0; m < L; ++m)
    for (size_t p = 0; p < cnt[m + 1].size(); p += 2) t.zeros[m] += cnt[m + 1][p];
  t.starts.resize(plan.size());
  for (size_t pi = 0; pi < plan.size(); ++pi) {
    const auto& p = plan[pi];
    std::vector<uint64_t> st(size_t((2 << p.K) - 2), 0);
    for (int j = 1; j <= p.K; ++j) {
      const auto& c = cnt[p.level + j];
      std::vector<uint64_t> k(size_t(1) << j, 0);
      const uint64_t mask = (uint64_t(1) << j) - 1;
      for (size_t q = 0; q < c.size(); ++q) k[rev_bits_host(q & mask, uint32_t(j))] += c[q];
      uint64_t run = 0;
      for (size_t v = 0; v < k.size(); ++v) { st[size_t((1 << j) - 2) + v] = run; run += k[v]; }
    }
    t.starts[pi] = std::move(st);
  }
  if (want_tree) {
    t.seg_tree.resize(L);
    t.seg_matrix.resize(L);
    for (uint32_t m = 1; m < L; ++m) {
      const auto& c = cnt[m];
      std::vector<uint64_t> mstart(c.size(), 0);
      uint64_t run = 0;
      for (size_t r = 0; r < c.size(); ++r) {
        size_t p = rev_bits_host(r, m);
        mstart[p] = run;
        run += c[p];
      }
      std::vector<uint64_t> st, sm;
      run = 0;
      for (size_t p = 0; p < c.size(); ++p) {
        if (c[p]) { st.push_back(run); sm.push_back(mstart[p]); }
        run += c[p];
      }
      if (st.empty()) { st.push_back(0); sm.push_back(0); }
      t.seg_tree[m] = std::move(st);
      t.seg_matrix[m] = std::move(sm);
    }
  }
  return t;
}

// The counts of one level (a view).
struct CountSpan {
  const uint64_t* p;
  size_t n;
  size_t size() const { return n; }
  const uint64_t& operator[](size_t i) const { return p[i]; }
  const uint64_t* begin() const { return p; }
  const uint64_t* end() const { return p + n; }
};

// Natural-order prefix counts of every level m = 0..L (2^m counts each),
// flat: level m at offset 2^m - 1.  Either owned (folded on the host) or a
// view of counts the device folded (fold_levels_kernel).
class PrefixCounts {
 public:
  PrefixCounts() = default;
  static PrefixCounts view(const uint64_t* flat, uint32_t L) {
    PrefixCounts c;
    c.ext_ = flat;
    c.L_ = L;
    return c;
  }
  static PrefixCounts fold(const uint64_t* hist, uint32_t L) {
    PrefixCounts c;
    c.L_ = L;
    c.own_.resize((size_t(2) << L) - 1);
    uint64_t* f = c.own_.data();
    std::copy(hist, hist + (size_t(1) << L), f + (size_t(1) << L) - 1);
    for (int m = int(L) - 1; m >= 0; --m) {
      const uint64_t* up = f + (size_t(2) << m) - 1;
      uint64_t* o = f + (size_t(1) << m) - 1;
      for (size_t x = 0; x < (size_t(1) << m); ++x) o[x] = up[2 * x] + up[2 * x + 1];
    }
    return c;
  }
  CountSpan operator[](uint32_t m) const { return {base() + (size_t(1) << m) - 1, size_t(1) << m}; }
  uint32_t levels() const { return L_; }
  bool empty() const { return !ext_ && own_.empty(); }

 private:
  const uint64_t* base() const { return ext_ ? ext_ : own_.data(); }
  const uint64_t* ext_ = nullptr;
  std::vector<uint64_t> own_;
  uint32_t L_ = 0;
};

inline PrefixCounts fold_prefix_counts(const uint64_t* hist, uint32_t L) { return PrefixCounts::fold(hist, L); }

// Tables of a plain build through the tile engine: zero counts, level sizes
// and the tree segments of the given levels (those the regroup writes).
// zeros: the zero bits of every level when the device counted them, else
// they are summed here.
inline LevelTables build_tables_tile(const PrefixCounts& cnt, uint32_t L, const std::vector<uint32_t>& tree_levels,
                                     const uint64_t* zeros = nullptr) {
  LevelTables t;
  const uint64_t n = cnt[0][0];
  t.level_bits.assign(L, n);
  t.zeros.assign(L, 0);
  if (zeros) {
    t.zeros.assign(zeros, zeros + L);
  } else {
    for (uint32_t m = 0; m < L; ++m) {
      const CountSpan c = cnt[m + 1];
      for (size_t p = 0; p < c.size(); p += 2) t.zeros[m] += c[p];
    }
  }
  t.seg_tree.resize(L);
  t.seg_matrix.resize(L);
  for (uint32_t m : tree_levels) {
    const CountSpan c = cnt[m];
    std::vector<uint64_t> mstart(c.size(), 0);
    uint64_t run = 0;
    for (size_t r = 0; r < c.size(); ++r) {
      const size_t p = rev_bits_host(r, m);
      mstart[p] = run;
      run += c[p];
    }
    std::vector<uint64_t> st, sm;
    run = 0;
    for (size_t p = 0; p < c.size(); ++p) {
      if (c[p]) { st.push_back(run); sm.push_back(mstart[p]); }
      run += c[p];
    }
    if (st.empty()) { st.push_back(0); sm.push_back(0); }
    t.seg_tree[m] = std::move(st);
    t.seg_matrix[m] = std::move(sm);
  }
  return t;
}

// ---------------------------------------------------------------------------
// Segmented tile passes of a plain text (levels <= kTilePlanMaxLevels).
// Pass (l, K) splits S_l through levels l..l+K-1.  A pass is "segmented" when
// each l-bit prefix group of S_l is its own segment: every run of those
// levels then has one start in the matrix and one in the tree, so the pass
// writes both.  Otherwise (l > 0 and groups too small or too many, or no
// tree) one segment covers S_l, the pass writes the matrix only and the tree
// levels of the pass come from the regroup.
// ---------------------------------------------------------------------------
constexpr uint32_t kTilePlanMaxLevels = 20;

struct TileSegHost {
  uint64_t in_begin, m, table;
  uint32_t tile0, text;
  uint64_t group = 0;  // the segment's group of level `level` (key order)
};

struct TilePassHost {
  uint32_t level = 0;
  int K = 0;
  bool out = false;
  bool segmented = false;
  uint32_t tiles = 0;
  std::vector<TileSegHost> segs;
  std::vector<uint64_t> table;  // per segment: tile_table_size(K) entries
};

// Start table of a matrix-only pass over all of S_l (one segment) from the
// counts of its natural K-bit digit (digit[d]: the symbols whose bits of
// levels l..l+K-1, level l's most significant, read d): the starts of the
// runs of key_j (the same bits, level l's least significant) in levels
// l..l+K-1 and, with `out`, in S_{l+K}.
inline void matrix_pass_table(const std::vector<uint64_t>& digit, int K, bool out, std::vector<uint64_t>& tab) {
  std::vector<uint64_t> ck(size_t(1) << K, 0);  // by key_K
  for (size_t r = 0; r < ck.size(); ++r) ck[rev_bits_host(r, uint32_t(K))] += digit[r];
  for (int j = 0; j <= K; ++j) {
    if (j < K || out) {
      uint64_t run = 0;
      for (int v = 0; v < (1 << j); ++v) {
        uint64_t cv = 0;  // key_j == v: the low j bits of key_K
        for (int h = 0; h < (1 << (K - j)); ++h) cv += ck[size_t(v + (h << j))];
        if (j < K) tab[size_t(tile_wm_entry(j, v))] = run;
        else tab[size_t(tile_out_entry(K, v))] = run;
        run += cv;
      }
    }
  }
}

// cnt: the folded prefix counts (fold_prefix_counts).  tile_keys(l): keys
// per tile of the pass starting at level l (its key width may narrow as the
// passes go on).  regroup: tree levels the passes leave to the regroup
// (empty without a tree).  Exclusive prefixes over all 2^m groups of a level
// are built only for the levels of segmented passes (few groups); a
// matrix-only pass needs only the counts of its own K bits, folded from one
// level, or given: digits[16 p + r] for pass p of plan_passes(L, kmax)
// (launch_flat_digits; passes of at most 4 levels).
template <typename TileKeys>
inline std::vector<TilePassHost> plan_tile_passes(const PrefixCounts& cnt, uint32_t L, int kmax,
                                                  TileKeys tile_keys, bool want_tree,
                                                  std::vector<uint32_t>* regroup,
                                                  const uint64_t* digits = nullptr) {
  const uint64_t n = cnt[0][0];
  std::vector<std::vector<uint64_t>> pren(L + 1), prek(L + 1);
  auto prefixes = [&](uint32_t m) {  // natural order (tree) and key order (matrix: reversed prefix)
    if (!prek[m].empty()) return;
    const size_t sz = cnt[m].size();
    pren[m].assign(sz + 1, 0);
    prek[m].assign(sz + 1, 0);
    for (size_t p = 0; p < sz; ++p) pren[m][p + 1] = pren[m][p] + cnt[m][p];
    for (size_t x = 0; x < sz; ++x) prek[m][x + 1] = prek[m][x] + cnt[m][rev_bits_host(x, m)];
  };
  std::vector<TilePassHost> passes;
  size_t pi = 0;
  for (const auto& pp : plan_passes(L, kmax)) {
    TilePassHost ps;
    ps.level = pp.level;
    ps.K = pp.K;
    ps.out = pp.has_out;
    const uint32_t l = pp.level;
    const int K = pp.K;
    const uint64_t groups = uint64_t(1) << l;
    const size_t pass_index = pi++;
    const uint32_t T = tile_keys(l);
    ps.segmented = want_tree && (l == 0 || (groups <= 65536 && n >= groups * 4 * uint64_t(T)));
    const int TS = tile_table_size(K);
    uint32_t tile = 0;
    auto add_segment = [&](uint64_t begin, uint64_t m, const std::vector<uint64_t>& tab, uint64_t group) {
      if (m == 0) return;
      ps.segs.push_back({begin, m, uint64_t(ps.table.size()), tile, 0u, group});
      ps.table.insert(ps.table.end(), tab.begin(), tab.end());
      tile += uint32_t((m + T - 1) / T);
    };
    std::vector<uint64_t> tab(size_t(TS), 0);
    if (ps.segmented) {
      for (uint32_t m = l; m <= l + uint32_t(K) && m <= L; ++m) prefixes(m);
      for (uint64_t g = 0; g < groups; ++g) {
        const uint64_t m = prek[l][g + 1] - prek[l][g];
        if (m == 0) continue;
        for (int j = 0; j < K; ++j)
          for (int v = 0; v < (1 << j); ++v) {
            const uint64_t x = (uint64_t(v) << l) | g;
            tab[size_t(tile_wm_entry(j, v))] = prek[l + j][x];
            tab[size_t(tile_wt_entry(K, j, v))] = pren[l + j][rev_bits_host(x, l + j)];
          }
        if (ps.out)
          for (int v = 0; v < (1 << K); ++v) tab[size_t(tile_out_entry(K, v))] = prek[l + K][(uint64_t(v) << l) | g];
        add_segment(prek[l][g], m, tab, g);
      }
    } else {
      // counts of the pass's natural K-bit digit (bits of levels l..l+K-1,
      // level l's most significant) over the whole text: the natural
      // prefixes of level l+K summed by their last K bits
      const uint32_t top = l + uint32_t(K);
      const size_t R = size_t(1) << K;
      std::vector<uint64_t> low(R, 0);
      if (digits && K <= 4) {  // (16 counts per pass)
        for (size_t r = 0; r < R; ++r) low[r] = digits[16 * pass_index + r];
      } else {
        const CountSpan c = cnt[top];
        for (size_t p = 0; p < c.size(); p += R)
          for (size_t r = 0; r < R; ++r) low[r] += c[p + r];
      }
      matrix_pass_table(low, K, ps.out, tab);
      add_segment(0, n, tab, 0);
      if (want_tree && regroup)
        for (int j = 0; j < K; ++j)
          if (l + uint32_t(j) > 0) regroup->push_back(l + uint32_t(j));
    }
    ps.tiles = tile;
    passes.push_back(std::move(ps));
  }
  return passes;
}

// Matrix-only passes (no tree) from the digit counts of each pass alone:
// digits[16 p + d] counts the natural K-bit digit d of pass p (the passes of
// plan_passes(L, kmax)); the same plan as plan_tile_passes without a tree.
template <typename TileKeys>
inline std::vector<TilePassHost> plan_matrix_passes(const uint64_t* digits, uint64_t n, uint32_t L, int kmax,
                                                    TileKeys tile_keys) {
  std::vector<TilePassHost> passes;
  size_t pi = 0;
  for (const auto& pp : plan_passes(L, kmax)) {
    TilePassHost ps;
    ps.level = pp.level;
    ps.K = pp.K;
    ps.out = pp.has_out;
    std::vector<uint64_t> tab(size_t(tile_table_size(pp.K)), 0);
    const std::vector<uint64_t> digit(digits + 16 * pi, digits + 16 * pi + (size_t(1) << pp.K));
    matrix_pass_table(digit, pp.K, ps.out, tab);
    if (n) {
      ps.segs.push_back({0, n, 0, 0u, 0u, 0});
      ps.table = tab;
      ps.tiles = uint32_t((n + tile_keys(pp.level) - 1) / tile_keys(pp.level));
    }
    passes.push_back(std::move(ps));
    ++pi;
  }
  return passes;
}

// Zero bits of every level from the same digit counts: level l+j of pass p
// is bit K-1-j of its digit.
inline std::vector<uint64_t> matrix_pass_zeros(const uint64_t* digits, uint32_t L, int kmax) {
  std::vector<uint64_t> z(L, 0);
  size_t pi = 0;
  for (const auto& pp : plan_passes(L, kmax)) {
    for (int j = 0; j < pp.K; ++j)
      for (int d = 0; d < (1 << pp.K); ++d)
        if (!((d >> (pp.K - 1 - j)) & 1)) z[pp.level + uint32_t(j)] += digits[16 * pi + size_t(d)];
    ++pi;
  }
  return z;
}

// The same with T keys per tile in every pass.
inline std::vector<TilePassHost> plan_tile_passes(const PrefixCounts& cnt, uint32_t L, int kmax, uint32_t T,
                                                  bool want_tree, std::vector<uint32_t>* regroup,
                                                  const uint64_t* digits = nullptr) {
  return plan_tile_passes(cnt, L, kmax, [T](uint32_t) { return T; }, want_tree, regroup, digits);
}

// One run of a merge of shards (pwm's merge_bit_vectors, include/
// construction/merge.hpp:192-465): bits [src_bit, src_bit + len) of level l of
// shard `shard` go to bit `dst` of level l of the merged structure.
struct MergeRun {
  uint64_t dst, shard, src_bit, len;
};

// The runs of level l of a merged structure, in destination order: block by
// block in the level's order (the tree's natural prefix order, the matrix's
// bit-reversed one), each block the shards' runs of it in shard order; a
// shard's level holds its runs in the same order, so its read position is the
// sum of its earlier runs.  cnt: the shards' prefix counts.
inline std::vector<MergeRun> plan_merge_level(const std::vector<PrefixCounts>& cnt, uint32_t l, bool tree) {
  std::vector<MergeRun> runs;
  std::vector<uint64_t> rd(cnt.size(), 0);
  uint64_t dst = 0;
  for (uint64_t b = 0; b < (uint64_t(1) << l); ++b) {
    const uint64_t pfx = tree ? b : rev_bits_host(b, l);
    for (size_t s = 0; s < cnt.size(); ++s) {
      const uint64_t len = cnt[s][l][pfx];
      if (!len) continue;
      runs.push_back({dst, uint64_t(s), rd[s], len});
      dst += len;
      rd[s] += len;
    }
  }
  return runs;
}

// Tables of a Huffman-shaped text from its weighted codes.  want_tree: also
// the segments.
inline LevelTables build_tables(const std::vector<WeightedCode>& codes, uint32_t L, const std::vector<PassPlan>& plan,
                                bool want_tree) {
  LevelTables t;
  t.zeros.assign(L, 0);
  t.level_bits.assign(L, 0);
  // One walk over the codes: per code its bits reversed (code bit m at bit m),
  // its zero bits, and per pass (l, K) the counts of its key_j values among
  // the codes alive at l+j (key_j: code bits l..l+j-1, bit l least
  // significant); the level sizes from the counts by length.
  std::vector<uint64_t> by_len(L + 1, 0);
  std::vector<std::vector<uint64_t>> cnts(plan.size());
  for (size_t pi = 0; pi < plan.size(); ++pi) cnts[pi].assign(size_t((2 << plan[pi].K) - 2), 0);
  for (const auto& c : codes) {
    const uint32_t top = std::min<uint32_t>(c.len, L);
    by_len[top] += c.freq;
    uint64_t rw = 0;
    for (uint32_t m = 0; m < top; ++m) rw |= uint64_t(code_bit(c, m)) << m;
    for (uint64_t z = ~rw & (top >= 64 ? ~uint64_t(0) : (uint64_t(1) << top) - 1); z; z &= z - 1)
      t.zeros[__builtin_ctzll(z)] += c.freq;
    for (size_t pi = 0; pi < plan.size(); ++pi) {
      const uint32_t l = plan[pi].level;
      if (l >= top) break;
      const uint32_t chunk = uint32_t(rw >> l);
      std::vector<uint64_t>& cn = cnts[pi];
      for (int j = 1; j <= plan[pi].K; ++j) {
        const uint32_t m = l + uint32_t(j) - 1;
        if (m >= top || m + 1 >= c.len) break;  // alive at l+j
        cn[size_t((1u << j) - 2 + (chunk & ((1u << j) - 1)))] += c.freq;
      }
    }
  }
  uint64_t run = 0;
  for (uint32_t m = L; m-- > 0;) {
    run += by_len[m + 1];
    t.level_bits[m] = run;
  }
  t.starts.resize(plan.size());
  for (size_t pi = 0; pi < plan.size(); ++pi) {
    const auto& p = plan[pi];
    const int C = (2 << p.K) - 2;
    const std::vector<uint64_t>& cnt = cnts[pi];
    std::vector<uint64_t> st(size_t(C), 0);
    for (int j = 1; j <= p.K; ++j) {
      uint64_t r = 0;
      for (int v = 0; v < (1 << j); ++v) {
        st[size_t((1 << j) - 2 + v)] = r;
        r += cnt[size_t((1 << j) - 2 + v)];
      }
    }
    t.starts[pi] = std::move(st);
  }
  if (want_tree) {
    t.seg_tree.resize(L);
    t.seg_matrix.resize(L);
    // codes longer than one bit by their left-aligned code word: at every
    // level the prefixes of the longer codes then come in prefix order, so no
    // level sorts them.  The words are distinct (the codes are prefix-free):
    // an LSD radix sort on their top maxlen bits, 11 bits a pass.
    uint32_t maxlen = 1;
    for (const auto& c : codes) maxlen = std::max<uint32_t>(maxlen, std::min<uint32_t>(c.len, 64));
    std::vector<std::pair<uint64_t, uint32_t>> by_word, tmpw;  // (left-aligned code word, code)
    by_word.reserve(codes.size());
    for (size_t i = 0; i < codes.size(); ++i)
      if (codes[i].len > 1) by_word.emplace_back(codes[i].word << (64 - codes[i].len), uint32_t(i));
    tmpw.resize(by_word.size());
    std::vector<uint32_t> rc(2049);
    for (uint32_t lo = 0; lo < maxlen; lo += 11) {
      const uint32_t sh = 64 - maxlen + lo;
      std::fill(rc.begin(), rc.end(), 0u);
      for (const auto& pw : by_word) ++rc[((pw.first >> sh) & 2047u) + 1];
      for (size_t i = 0; i < 2048; ++i) rc[i + 1] += rc[i];
      for (const auto& pw : by_word) tmpw[rc[(pw.first >> sh) & 2047u]++] = pw;
      by_word.swap(tmpw);
    }
    // The prefix groups of every level in one walk: with the codes in that
    // order, code i (longer than m) starts a new group at level m exactly
    // when m > b_i = min(common prefix with code i-1, length of code i-1 - 1)
    // -- a code between two codes sharing m bits would share them too and,
    // being no longer than m, be a prefix of them (the codes are prefix-free).
    std::vector<std::vector<uint64_t>> gpl(L), gcl(L);  // per level: group prefixes and counts
    {
      uint64_t prev_lw = 0;
      uint32_t prev_len = 0;
      for (size_t q = 0; q < by_word.size(); ++q) {
        const WeightedCode& c = codes[by_word[q].second];
        const uint64_t lw = by_word[q].first;
        const uint32_t b = q == 0 ? 0u : std::min<uint32_t>(uint32_t(__builtin_clzll(prev_lw ^ lw)), prev_len - 1);
        const uint32_t top = std::min<uint32_t>(c.len, L);  // levels 1..top-1 hold the code
        for (uint32_t m = 1; m < top; ++m) {
          if (m > b) {
            gpl[m].push_back(lw >> (64 - m));
            gcl[m].push_back(c.freq);
          } else {
            gcl[m].back() += c.freq;
          }
        }
        prev_lw = lw;
        prev_len = c.len;
      }
    }
    std::vector<uint64_t> gr, by_rev;  // per group of a level: bit-reversed prefix
    for (uint32_t m = 1; m < L; ++m) {
      const std::vector<uint64_t>& gp = gpl[m];
      const std::vector<uint64_t>& gc = gcl[m];
      const size_t G = gp.size();
      std::vector<uint64_t> st(G), sm(G);
      run = 0;
      for (size_t i = 0; i < G; ++i) {
        st[i] = run;
        run += gc[i];
      }
      gr.resize(G);
      for (size_t i = 0; i < G; ++i) gr[i] = rev_bits_host(gp[i], m);
      if (m <= 20 && (size_t(1) << m) <= 16 * G) {
        // the matrix orders the groups by bit-reversed prefix: counts
        // scattered to their reversed prefixes, exclusive sums in that order
        by_rev.assign(size_t(1) << m, 0);
        for (size_t i = 0; i < G; ++i) by_rev[gr[i]] = gc[i];
        run = 0;
        for (auto& x : by_rev) {
          const uint64_t v = x;
          x = run;
          run += v;
        }
        for (size_t i = 0; i < G; ++i) sm[i] = by_rev[gr[i]];
      } else {  // few groups for the reversed-prefix range: sort them
        std::vector<std::pair<uint64_t, size_t>> ro(G);
        for (size_t i = 0; i < G; ++i) ro[i] = {gr[i], i};
        std::sort(ro.begin(), ro.end());
        run = 0;
        for (const auto& r : ro) {
          sm[r.second] = run;
          run += gc[r.second];
        }
      }
      if (G == 0) {
        st.push_back(0);
        sm.push_back(0);
      }
      t.seg_tree[m] = std::move(st);
      t.seg_matrix[m] = std::move(sm);
    }
  }
  return t;
}

}  // namespace pwmgpu
