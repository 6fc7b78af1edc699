// Stand-in for pwm's huff_bit_vectors (test infrastructure only): levels of
// the given sizes, laid out like bit_vectors.
#pragma once
#include "arrays/bit_vectors.hpp"

template <bool is_bv_initialized = false>
class huff_bit_vectors : public base_bit_vectors {
 public:
  huff_bit_vectors(uint64_t levels, const std::vector<uint64_t>& level_sizes)
      : base_bit_vectors(std::vector<uint64_t>(level_sizes.begin(), level_sizes.begin() + levels)) {}
};
