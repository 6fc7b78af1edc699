// Stand-in for pwm's canonical_huff_codes (test infrastructure only): the code
// pairs (length, word) of every symbol up to the largest one of the text.
#pragma once
#include <vector>

#include "huffman/huff_level_sizes_builder.hpp"

class code_pair {
 public:
  code_pair(uint64_t len, uint64_t word) : len_(len), word_(word) {}
  uint64_t code_length() const { return len_; }
  uint64_t code_word() const { return word_; }

 private:
  uint64_t len_, word_;
};

template <typename AlphabetType, bool is_tree>
class canonical_huff_codes {
 public:
  explicit canonical_huff_codes(level_sizes_builder<AlphabetType>& b) {
    const standin_code_table t = standin_codes(b.hist().text(), b.hist().size(), is_tree);
    for (size_t s = 0; s < t.len.size(); ++s) pairs_.emplace_back(t.len[s], t.word[s]);
  }
  const std::vector<code_pair>& code_pairs() const { return pairs_; }

 private:
  std::vector<code_pair> pairs_;
};
