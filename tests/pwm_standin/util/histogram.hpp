// Stand-in for pwm's util/histogram.hpp (test infrastructure only): keeps the
// text; the code-table stand-ins build pwm's table from it.
#pragma once
#include <cstdint>

template <typename AlphabetType>
class histogram {
 public:
  histogram(AlphabetType const* text, uint64_t size) : text_(text), size_(size) {}
  AlphabetType const* text() const { return text_; }
  uint64_t size() const { return size_; }

 private:
  AlphabetType const* text_;
  uint64_t size_;
};
