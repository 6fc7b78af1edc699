/*
 * wx_gpu.hpp -- drop-in construction classes for kurpicz/pwm backed by the
 * GB300 engine (libpwmgpu.so, include/pwmgpu.h).
 *
 * Include from inside pwm's source tree (it uses pwm's own containers):
 *
 *   #include "wx_gpu.hpp"
 *   using wm_gpu_8 = wx_gpu<uint8_t, false>;
 *   CONSTRUCTION_REGISTER("wm_gpu", "GB300 wavelet matrix", wm_gpu_8)
 *
 * The classes have the static interface of pwm's wx_* classes
 * (include/wx_ps.hpp:19-57: is_parallel, is_tree, word_width,
 * is_huffman_shaped, the wx_in_out_external<false,false> traits of
 * include/wx_base.hpp:13-23, and
 *   static wavelet_structure compute(text, size, levels)).
 * pwm has no error channel in compute(); a non-OK status of the engine is
 * thrown as std::runtime_error.
 */
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "pwmgpu.h"

#include "arrays/bit_vectors.hpp"
#include "construction/wavelet_structure.hpp"
#include "huffman/huff_bit_vectors.hpp"
#include "huffman/huff_codes.hpp"
#include "huffman/huff_level_sizes_builder.hpp"
#include "util/histogram.hpp"
#include "wx_base.hpp"

namespace pwmgpu_pwm {

// One engine context per process (device 0, its own stream).
inline pwmgpu_ctx* context() {
  static pwmgpu_ctx* ctx = [] {
    pwmgpu_ctx* c = nullptr;
    const pwmgpu_status st = pwmgpu_ctx_create(0, nullptr, &c);
    if (st != PWMGPU_OK) throw std::runtime_error(std::string("pwmgpu: ") + pwmgpu_status_string(st));
    return c;
  }();
  return ctx;
}

inline void check(pwmgpu_status st) {
  if (st != PWMGPU_OK)
    throw std::runtime_error(std::string("pwmgpu: ") + pwmgpu_status_string(st) + ": " +
                             pwmgpu_ctx_last_error(context()));
}

}  // namespace pwmgpu_pwm

// Plain wavelet matrix (is_tree == false) or levelwise wavelet tree.  Output
// is bit-identical to wx_ps / wx_pc (and the other plain variants), zeros
// include zeros[levels-1] like wx_ps.
template <typename AlphabetType, bool is_tree_>
class wx_gpu : public wx_in_out_external<false, false> {
 public:
  static constexpr bool is_parallel = true;
  static constexpr bool is_tree = is_tree_;
  static constexpr uint8_t word_width = sizeof(AlphabetType);
  static constexpr bool is_huffman_shaped = false;

  template <typename InputType>
  static wavelet_structure compute(const InputType& text, const uint64_t size, const uint64_t levels) {
    if (size == 0) {
      if constexpr (is_tree) return wavelet_structure_tree();
      else return wavelet_structure_matrix();
    }
    bit_vectors<false> bv(levels, size);
    std::vector<uint64_t> zeros(levels, 0);
    pwmgpu_pwm::check(pwmgpu_compute(pwmgpu_pwm::context(), &text[0], size, word_width, uint32_t(levels),
                                     is_tree ? 1 : 0, bv[0].data(), zeros.data()));
    if constexpr (is_tree) return wavelet_structure_tree(std::move(bv));
    else return wavelet_structure_matrix(std::move(bv), std::move(zeros));
  }
};

// Huffman-shaped wavelet matrix / tree.  Codes come from pwm's own builder
// (so the shape is exactly pwm's); levels follow the longest code and the
// `levels` argument is ignored, as in wx_huff_ps.  Output equals
// wx_huff_naive (and wx_huff_ps / wx_huff_pc for trees).
template <typename AlphabetType, bool is_tree_>
class wx_gpu_huff : public wx_in_out_external<false, false> {
 public:
  static constexpr bool is_parallel = true;
  static constexpr bool is_tree = is_tree_;
  static constexpr uint8_t word_width = sizeof(AlphabetType);
  static constexpr bool is_huffman_shaped = true;

  using huffman_codes = canonical_huff_codes<AlphabetType, is_tree>;

  static wavelet_structure compute(AlphabetType const* const text, const uint64_t size, const uint64_t /*levels*/) {
    histogram<AlphabetType> hist{text, size};
    level_sizes_builder<AlphabetType> builder{std::move(hist)};
    huffman_codes codes(builder);
    if (size == 0) {
      if constexpr (is_tree) return wavelet_structure_tree_huffman<AlphabetType>(std::move(codes));
      else return wavelet_structure_matrix_huffman<AlphabetType>(std::move(codes));
    }
    const auto& level_sizes = builder.level_sizes();
    const uint64_t levels = builder.levels();
    const auto& pairs = codes.code_pairs();
    std::vector<uint64_t> len(pairs.size()), word(pairs.size());
    for (size_t s = 0; s < pairs.size(); ++s) {
      len[s] = pairs[s].code_length();
      word[s] = pairs[s].code_word();
    }
    huff_bit_vectors<false> bv(levels, level_sizes);
    std::vector<uint64_t> zeros(levels, 0);
    pwmgpu_pwm::check(pwmgpu_compute_huffman(pwmgpu_pwm::context(), text, size, word_width, is_tree ? 1 : 0,
                                             len.data(), word.data(), len.size(), uint32_t(levels),
                                             level_sizes.data(), bv[0].data(), zeros.data()));
    if constexpr (is_tree) return wavelet_structure_tree_huffman<AlphabetType>(std::move(bv), std::move(codes));
    else return wavelet_structure_matrix_huffman<AlphabetType>(std::move(bv), std::move(zeros), std::move(codes));
  }
};
