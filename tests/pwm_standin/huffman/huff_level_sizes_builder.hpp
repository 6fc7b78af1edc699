// Stand-in for pwm's level_sizes_builder (test infrastructure only): the
// level sizes and level count of a text's Huffman shape.
#pragma once
#include <utility>

#include "huffman/pwm_codes.hpp"
#include "util/histogram.hpp"

template <typename AlphabetType>
class level_sizes_builder {
 public:
  explicit level_sizes_builder(histogram<AlphabetType>&& h)
      : hist_(std::move(h)), table_(standin_codes(hist_.text(), hist_.size(), false)) {}
  const std::vector<uint64_t>& level_sizes() const { return table_.level_sizes; }
  uint64_t levels() const { return table_.levels; }
  const histogram<AlphabetType>& hist() const { return hist_; }

 private:
  histogram<AlphabetType> hist_;
  standin_code_table table_;
};
