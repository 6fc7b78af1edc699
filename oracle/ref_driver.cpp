// oracle/ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A thin extern "C" shim over kurpicz/pwm's own in-memory construction,
// query and Huffman headers.  `make -C oracle ref REF=<pwm tree>` compiles it
// against the reference source tree into oracle/_ref/libpwmref.so (nothing of
// the reference is copied into this repository).  tests/golden/make_golden.py
// uses it to pin the oracle restatement and to record golden vectors; tests
// use it directly when the library is present.
//
// Layout of every returned structure: the flat 128-byte padded level layout
// of flat_two_dim_array (levels contiguous, each padded to 16 words).

#include <cstdint>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "wx_naive.hpp"
#include "wx_pc.hpp"
#include "wx_pc_ss.hpp"
#include "wx_ppc.hpp"
#include "wx_ppc_ss.hpp"
#include "wx_pps.hpp"
#include "wx_ps.hpp"
#include "wx_dd_pc.hpp"
#include "wx_dd_pc_ss.hpp"
#include "wx_dd_ps.hpp"
#include "wx_huff_naive.hpp"
#include "wx_huff_pc.hpp"
#include "wx_huff_ps.hpp"
#include "wx_huff_dd_ps.hpp"
#include "util/decode.hpp"
#include "huffman/huff_decode.hpp"
#define private public
#include "queries/query_support.hpp"
#undef private
#include "test/util/util.hpp"
// ref_stub/ shadows external_memory/stxxl_helper.hpp (declarations only)
#include "util/alphabet_util.hpp"

namespace {

std::vector<std::string>& fixtures() {
  static std::vector<std::string> f;
  if (f.empty()) test::roundtrip_batch([&](const std::string& s) { f.push_back(s); });
  return f;
}

// Copy a wavelet_structure into the flat padded layout; returns total words.
uint64_t export_ws(const wavelet_structure& ws, uint64_t* bv, uint64_t cap_words, uint64_t* level_bits,
                   uint64_t* zeros, uint32_t* levels_out) {
  const auto& b = ws.bvs();
  *levels_out = uint32_t(b.levels());
  uint64_t off = 0;
  for (uint64_t l = 0; l < b.levels(); ++l) {
    uint64_t bits = b.level_bit_size(l), words = (bits + 63) / 64, padded = (words + 15) & ~uint64_t(15);
    if (level_bits) level_bits[l] = bits;
    if (bv && off + padded <= cap_words) {
      std::memset(bv + off, 0, padded * 8);
      std::memcpy(bv + off, b[l].data(), words * 8);
      // pwm leaves the unused tail of an uninitialised level undefined; the
      // tail of the last word is always written as zero by the constructions.
    }
    off += padded;
  }
  if (zeros) {
    const auto& z = ws.zeros();
    for (size_t l = 0; l < z.size(); ++l) zeros[l] = z[l];
  }
  return off;
}

template <template <typename, bool> class Algo, typename A>
wavelet_structure run_plain(bool tree, const void* text, uint64_t n, uint64_t levels) {
  A* t = const_cast<A*>(static_cast<const A*>(text));
  if (tree) return Algo<A, true>::compute(t, n, levels);
  return Algo<A, false>::compute(t, n, levels);
}

template <typename A>
wavelet_structure dispatch_plain(int variant, bool tree, const void* text, uint64_t n, uint64_t levels) {
  switch (variant) {
    case 0: return run_plain<wx_ps, A>(tree, text, n, levels);
    case 1: return run_plain<wx_pc, A>(tree, text, n, levels);
    case 2: return run_plain<wx_naive, A>(tree, text, n, levels);
    case 3: return run_plain<wx_ppc, A>(tree, text, n, levels);
    case 4: return run_plain<wx_pps, A>(tree, text, n, levels);
    case 5: return run_plain<wx_dd_ps, A>(tree, text, n, levels);
    case 6: return run_plain<wx_dd_pc, A>(tree, text, n, levels);
    case 7: return run_plain<wx_pc_ss, A>(tree, text, n, levels);
    case 8: return run_plain<wx_ppc_ss, A>(tree, text, n, levels);
    default: return run_plain<wx_dd_pc_ss, A>(tree, text, n, levels);
  }
}

template <typename A>
wavelet_structure dispatch_huff(int variant, bool tree, const void* text, uint64_t n) {
  const A* t = static_cast<const A*>(text);
  switch (variant) {
    case 0: return tree ? wx_huff_naive<A, true>::compute(t, n, 0) : wx_huff_naive<A, false>::compute(t, n, 0);
    case 1: return tree ? wx_huff_ps<A, true>::compute(t, n, 0) : wx_huff_ps<A, false>::compute(t, n, 0);
    default: return tree ? wx_huff_pc<A, true>::compute(t, n, 0) : wx_huff_pc<A, false>::compute(t, n, 0);
  }
}

}  // namespace

extern "C" {

uint64_t pwmref_fixture_count() { return fixtures().size(); }

// Copies fixture i (bytes) into buf (cap bytes); returns its length.
uint64_t pwmref_fixture(uint64_t i, uint8_t* buf, uint64_t cap) {
  const auto& s = fixtures().at(i);
  if (buf) std::memcpy(buf, s.data(), std::min<uint64_t>(cap, s.size()));
  return s.size();
}

// variant: 0 ps, 1 pc, 2 naive, 3 ppc, 4 pps, 5 dd_ps, 6 dd_pc, 7 pc_ss,
// 8 ppc_ss, 9 dd_pc_ss.  Returns total words written (bv may be null to
// query the size).
uint64_t pwmref_build(int variant, uint32_t width, int is_tree, const void* text, uint64_t n, uint64_t levels,
                      uint64_t* bv, uint64_t cap_words, uint64_t* level_bits, uint64_t* zeros, uint32_t* levels_out) {
  wavelet_structure ws = width == 1   ? dispatch_plain<uint8_t>(variant, is_tree, text, n, levels)
                         : width == 2 ? dispatch_plain<uint16_t>(variant, is_tree, text, n, levels)
                                      : dispatch_plain<uint32_t>(variant, is_tree, text, n, levels);
  return export_ws(ws, bv, cap_words, level_bits, zeros, levels_out);
}

// variant: 0 huff_naive, 1 huff_ps, 2 huff_pc.  code_len/code_word receive
// the code table (max_symbol+1 entries, capacity cap_codes).
uint64_t pwmref_huff(int variant, uint32_t width, int is_tree, const void* text, uint64_t n, uint64_t* bv,
                     uint64_t cap_words, uint64_t* level_bits, uint64_t* zeros, uint32_t* levels_out,
                     uint64_t* code_len, uint64_t* code_word, uint64_t cap_codes, uint64_t* ncodes) {
  wavelet_structure ws = width == 1   ? dispatch_huff<uint8_t>(variant, is_tree, text, n)
                         : width == 2 ? dispatch_huff<uint16_t>(variant, is_tree, text, n)
                                      : dispatch_huff<uint32_t>(variant, is_tree, text, n);
  auto copy_codes = [&](const auto& cp) {
    *ncodes = cp.size();
    for (size_t s = 0; s < cp.size() && s < cap_codes; ++s) {
      code_len[s] = cp[s].code_length();
      code_word[s] = cp[s].code_word();
    }
  };
  if (width == 1) {
    if (is_tree) copy_codes(ws.codes<uint8_t, true>().code_pairs()); else copy_codes(ws.codes<uint8_t, false>().code_pairs());
  } else if (width == 2) {
    if (is_tree) copy_codes(ws.codes<uint16_t, true>().code_pairs()); else copy_codes(ws.codes<uint16_t, false>().code_pairs());
  } else {
    if (is_tree) copy_codes(ws.codes<uint32_t, true>().code_pairs()); else copy_codes(ws.codes<uint32_t, false>().code_pairs());
  }
  return export_ws(ws, bv, cap_words, level_bits, zeros, levels_out);
}

// Rank/select blocks of one bit vector (bin_rank_popcnt / bin_select_popcnt
// members read directly).  counts: n0, n12, ns0, ns1.
void pwmref_rank_select(const uint64_t* words, uint64_t nwords, uint64_t* l0, uint32_t* l12, uint32_t* s0,
                        uint32_t* s1, uint64_t* counts) {
  bin_rank_popcnt rank({words, nwords});
  bin_select0_popcnt sel0(rank);
  bin_select1_popcnt sel1(rank);
  counts[0] = rank.l0_.size();
  counts[1] = rank.l12_.size();
  counts[2] = sel0.samples_.size();
  counts[3] = sel1.samples_.size();
  if (l0) for (size_t i = 0; i < rank.l0_.size(); ++i) l0[i] = rank.l0_[i];
  if (l12) for (size_t i = 0; i < rank.l12_.size(); ++i) { l12[2 * i] = rank.l12_[i].l1_value; l12[2 * i + 1] = rank.l12_[i].l2_values; }
  if (s0) for (size_t i = 0; i < sel0.samples_.size(); ++i) s0[i] = sel0.samples_[i];
  if (s1) for (size_t i = 0; i < sel1.samples_.size(); ++i) s1[i] = sel1.samples_[i];
}

uint64_t pwmref_rank1(const uint64_t* words, uint64_t nwords, const uint64_t* idx, uint64_t count, uint64_t* out) {
  bin_rank_popcnt rank({words, nwords});
  for (uint64_t i = 0; i < count; ++i) out[i] = rank.rank1(idx[i]);
  return count;
}

uint64_t pwmref_select(int value, const uint64_t* words, uint64_t nwords, const uint64_t* occ, uint64_t count,
                       uint64_t* out) {
  bin_rank_popcnt rank({words, nwords});
  bin_select0_popcnt sel0(rank);
  bin_select1_popcnt sel1(rank);
  for (uint64_t i = 0; i < count; ++i) out[i] = value ? sel1.select(occ[i]) : sel0.select(occ[i]);
  return count;
}

// 8-bit queries through pwm's query_support on a structure built by
// wx_naive (query_support_tests.cpp:20-85).  op: 0 access(i), 1 rank(sym, i),
// 2 select(sym, occ).
uint64_t pwmref_queries(int is_tree, const uint8_t* text, uint64_t n, uint64_t levels, int op, const uint64_t* a,
                        const uint64_t* b, uint64_t count, uint64_t* out) {
  uint8_t* t = const_cast<uint8_t*>(text);
  wavelet_structure ws = is_tree ? wx_naive<uint8_t, true>::compute(t, n, levels)
                                 : wx_naive<uint8_t, false>::compute(t, n, levels);
  query_support<> qs(ws);
  for (uint64_t i = 0; i < count; ++i) {
    if (op == 0) out[i] = qs.access(a[i]);
    else if (op == 1) out[i] = qs.rank(uint8_t(a[i]), b[i]);
    else out[i] = qs.select(uint8_t(a[i]), b[i]);
  }
  return count;
}

// pwm's reduce_alphabet (include/util/alphabet_util.hpp:18-45) on a copy of
// the text, written back to `text`; returns pwm's max_char.  pwm's 8-bit
// table has 255 entries, so 8-bit texts must not hold symbol 255.
uint64_t pwmref_reduce_alphabet(uint32_t width, void* text, uint64_t n) {
  auto run = [&](auto* t) {
    using A = std::remove_pointer_t<decltype(t)>;
    std::vector<A> v(t, t + n);
    const uint64_t m = reduce_alphabet(v);
    std::memcpy(t, v.data(), n * sizeof(A));
    return m;
  };
  if (width == 1) return run(static_cast<uint8_t*>(text));
  if (width == 2) return run(static_cast<uint16_t*>(text));
  return run(static_cast<uint32_t*>(text));
}

// pwm's copy_bits (include/construction/merge.hpp:19-190), the bit-range copy
// of its domain-decomposition merge, on byte words (as test/bit_copy.cpp
// calls it) and on 64-bit words (as merge_bit_vectors calls it).
void pwmref_copy_bits_u8(uint8_t* dst, const uint8_t* src, uint64_t dst_off, uint64_t src_off, uint64_t len) {
  copy_bits<uint8_t>(dst, src, dst_off, src_off, len);
}
void pwmref_copy_bits_u64(uint64_t* dst, const uint64_t* src, uint64_t dst_off, uint64_t src_off, uint64_t len) {
  copy_bits<uint64_t>(dst, src, dst_off, src_off, len);
}

}  // extern "C"
