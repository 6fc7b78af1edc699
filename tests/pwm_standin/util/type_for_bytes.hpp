// Stand-in for pwm's util/type_for_bytes.hpp (test infrastructure only):
// uint40_t, five bytes packed little-endian (sizeof == 5).
#pragma once
#include <cstdint>
#include <cstring>

struct __attribute__((packed)) uint40_t {
  uint8_t b[5];
  uint40_t() = default;
  uint40_t(uint64_t v) {  // NOLINT: implicit like pwm's
    for (int i = 0; i < 5; ++i) b[i] = uint8_t(v >> (8 * i));
  }
  operator uint64_t() const {
    uint64_t v = 0;
    for (int i = 0; i < 5; ++i) v |= uint64_t(b[i]) << (8 * i);
    return v;
  }
};
static_assert(sizeof(uint40_t) == 5, "packed 40-bit symbols");
