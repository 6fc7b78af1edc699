// Test infrastructure only: pwm's canonical Huffman code table of a text,
// computed by the library's pwmgpu_huffman_codes (equal to pwm's builder,
// pinned by tests/golden), shared by the code-table stand-ins.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "pwmgpu.h"

struct standin_code_table {
  std::vector<uint64_t> len, word, level_sizes;
  uint64_t levels = 0;
};

inline pwmgpu_ctx* standin_context() {
  static pwmgpu_ctx* ctx = [] {
    pwmgpu_ctx* c = nullptr;
    if (pwmgpu_ctx_create(0, nullptr, &c) != PWMGPU_OK) throw std::runtime_error("pwmgpu context");
    return c;
  }();
  return ctx;
}

template <typename AlphabetType>
standin_code_table standin_codes(AlphabetType const* text, uint64_t size, bool is_tree) {
  standin_code_table t;
  if (size == 0) return t;
  const uint64_t cap = uint64_t(1) << (8 * sizeof(AlphabetType));
  t.len.resize(cap);
  t.word.resize(cap);
  t.level_sizes.resize(64);
  uint64_t num = 0;
  uint32_t levels = 0;
  if (pwmgpu_huffman_codes(standin_context(), text, size, sizeof(AlphabetType), is_tree ? 1 : 0, t.len.data(),
                           t.word.data(), cap, &num, t.level_sizes.data(), &levels) != PWMGPU_OK)
    throw std::runtime_error("pwmgpu_huffman_codes");
  t.len.resize(num);
  t.word.resize(num);
  t.level_sizes.resize(levels);
  t.levels = levels;
  return t;
}
