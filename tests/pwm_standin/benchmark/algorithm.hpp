// Stand-in for pwm's benchmark/algorithm.hpp (test infrastructure only): the
// CONSTRUCTION_REGISTER contract (a static object per registration that adds
// the construction, with its static traits, to one process-wide list).
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "construction/wavelet_structure.hpp"
#include "util/type_for_bytes.hpp"

struct registered_construction {
  std::string name, description;
  uint64_t word_width;
  bool is_tree, is_huffman_shaped, is_parallel, external_in, external_out, stats_support, is_inplace;
  std::function<wavelet_structure(const void*, uint64_t, uint64_t)> compute;
};

inline std::vector<registered_construction>& construction_list() {
  static std::vector<registered_construction> list;
  return list;
}

// The alphabet type of a word width, as pwm's type_for_bytes gives it.
template <uint64_t W> struct standin_alphabet;
template <> struct standin_alphabet<1> { using type = uint8_t; };
template <> struct standin_alphabet<2> { using type = uint16_t; };
template <> struct standin_alphabet<4> { using type = uint32_t; };
template <> struct standin_alphabet<5> { using type = uint40_t; };

template <typename Algorithm>
struct concrete_construction {
  concrete_construction(const char* name, const char* description) {
    using A = typename standin_alphabet<Algorithm::word_width>::type;
    construction_list().push_back(registered_construction{
        name, description, Algorithm::word_width, Algorithm::is_tree, Algorithm::is_huffman_shaped,
        Algorithm::is_parallel, Algorithm::external_in, Algorithm::external_out, Algorithm::stats_support,
        Algorithm::is_inplace, [](const void* text, uint64_t n, uint64_t levels) {
          A* t = static_cast<A*>(const_cast<void*>(text));
          return Algorithm::compute(t, n, levels);
        }});
  }
};

#define CONSTRUCTION_REGISTER(algo_name, algo_description, ws) \
  static const auto _cstr_algo_##ws##_register = concrete_construction<ws>(algo_name, algo_description);
