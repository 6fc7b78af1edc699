// Stand-in for pwm's bit_vectors (test infrastructure only): the levels of a
// structure in one zeroed allocation, each level padded to 16 words (128
// bytes), level l addressed by operator[](l).data().
#pragma once
#include <cstdint>
#include <utility>
#include <vector>

class base_bit_vectors {
 public:
  struct level_ref {
    uint64_t* ptr;
    uint64_t words;
    uint64_t* data() const { return ptr; }
    uint64_t size() const { return words; }
    uint64_t& operator[](uint64_t i) const { return ptr[i]; }
  };

  base_bit_vectors() = default;
  explicit base_bit_vectors(std::vector<uint64_t> level_bits) : bits_(std::move(level_bits)) {
    uint64_t off = 0;
    for (uint64_t b : bits_) {
      offs_.push_back(off);
      off += (((b + 63) / 64) + 15) & ~uint64_t(15);
    }
    words_.assign(off ? off : 1, 0);
  }
  uint64_t levels() const { return bits_.size(); }
  uint64_t level_bit_size(uint64_t l) const { return bits_[l]; }
  level_ref operator[](uint64_t l) const {
    return level_ref{const_cast<uint64_t*>(words_.data()) + offs_[l], (bits_[l] + 63) / 64};
  }

 private:
  std::vector<uint64_t> bits_, offs_, words_;
};

template <bool is_bv_initialized = false>
class bit_vectors : public base_bit_vectors {
 public:
  bit_vectors() = default;
  bit_vectors(uint64_t levels, uint64_t size) : base_bit_vectors(std::vector<uint64_t>(levels, size)) {}
};
