// Stand-in for pwm's construction/wavelet_structure.hpp (test infrastructure
// only): the structure a construction returns (bit vectors, matrix zeros,
// shape flags) and the factories the constructions use.
#pragma once
#include <cstdint>
#include <memory>
#include <utility>
#include <vector>

#include "arrays/bit_vectors.hpp"

class wavelet_structure {
 public:
  wavelet_structure(base_bit_vectors&& bvs, std::vector<uint64_t>&& zeros, bool is_tree, bool is_huffman)
      : bvs_(std::move(bvs)), zeros_(std::move(zeros)), is_tree_(is_tree), is_huffman_(is_huffman) {}
  const base_bit_vectors& bvs() const { return bvs_; }
  const std::vector<uint64_t>& zeros() const { return zeros_; }
  uint64_t levels() const { return bvs_.levels(); }
  bool is_tree() const { return is_tree_; }
  bool is_huffman_shaped() const { return is_huffman_; }

 private:
  base_bit_vectors bvs_;
  std::vector<uint64_t> zeros_;
  bool is_tree_, is_huffman_;
};

class wavelet_structure_tree : public wavelet_structure {
 public:
  wavelet_structure_tree() : wavelet_structure(base_bit_vectors(), {}, true, false) {}
  explicit wavelet_structure_tree(base_bit_vectors&& bv) : wavelet_structure(std::move(bv), {}, true, false) {}
};

class wavelet_structure_matrix : public wavelet_structure {
 public:
  wavelet_structure_matrix() : wavelet_structure(base_bit_vectors(), {}, false, false) {}
  wavelet_structure_matrix(base_bit_vectors&& bv, std::vector<uint64_t>&& zeros)
      : wavelet_structure(std::move(bv), std::move(zeros), false, false) {}
};

template <typename AlphabetType>
class wavelet_structure_tree_huffman : public wavelet_structure {
 public:
  template <typename Codes>
  explicit wavelet_structure_tree_huffman(Codes&&) : wavelet_structure(base_bit_vectors(), {}, true, true) {}
  template <typename Codes>
  wavelet_structure_tree_huffman(base_bit_vectors&& bv, Codes&&)
      : wavelet_structure(std::move(bv), {}, true, true) {}
};

template <typename AlphabetType>
class wavelet_structure_matrix_huffman : public wavelet_structure {
 public:
  template <typename Codes>
  explicit wavelet_structure_matrix_huffman(Codes&&) : wavelet_structure(base_bit_vectors(), {}, false, true) {}
  template <typename Codes>
  wavelet_structure_matrix_huffman(base_bit_vectors&& bv, std::vector<uint64_t>&& zeros, Codes&&)
      : wavelet_structure(std::move(bv), std::move(zeros), false, true) {}
};
