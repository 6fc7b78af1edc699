// Test driver (test infrastructure only): runs one construction registered by
// integration/gpu_construction.cpp through CONSTRUCTION_REGISTER, as pwm's
// benchmark does, and writes its wavelet_structure to a file.
//
//   run_registered list
//       prints "name word_width is_tree is_huffman is_parallel ext_in ext_out stats inplace" per registration
//   run_registered <name> <word_width> <levels> <text file> <out file>
//       out: levels, then per level its bit size, then the zero count
//       and the zeros, then every level's ceil(bits/64) words (all u64)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "benchmark/algorithm.hpp"

int main(int argc, char** argv) {
  if (argc >= 2 && !strcmp(argv[1], "list")) {
    for (const auto& a : construction_list())
      printf("%s %llu %d %d %d %d %d %d %d\n", a.name.c_str(), (unsigned long long)a.word_width, a.is_tree,
             a.is_huffman_shaped, a.is_parallel, a.external_in, a.external_out, a.stats_support, a.is_inplace);
    return 0;
  }
  if (argc < 6) return 2;
  const std::string name = argv[1];
  const uint64_t width = strtoull(argv[2], nullptr, 10), levels = strtoull(argv[3], nullptr, 10);
  for (const auto& a : construction_list()) {
    if (a.name != name || a.word_width != width) continue;
    FILE* f = fopen(argv[4], "rb");
    if (!f) return 3;
    std::vector<unsigned char> text;
    unsigned char buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), f)) > 0) text.insert(text.end(), buf, buf + got);
    fclose(f);
    const uint64_t n = text.size() / width;
    try {
      const wavelet_structure ws = a.compute(text.empty() ? nullptr : text.data(), n, levels);
      FILE* o = fopen(argv[5], "wb");
      if (!o) return 3;
      auto put = [&](uint64_t v) { fwrite(&v, 8, 1, o); };
      const auto& b = ws.bvs();
      put(b.levels());
      for (uint64_t l = 0; l < b.levels(); ++l) put(b.level_bit_size(l));
      put(ws.zeros().size());
      for (uint64_t z : ws.zeros()) put(z);
      for (uint64_t l = 0; l < b.levels(); ++l) fwrite(b[l].data(), 8, (b.level_bit_size(l) + 63) / 64, o);
      fclose(o);
    } catch (const std::exception& e) {
      printf("runtime: %s\n", e.what());
      return 4;
    }
    return 0;
  }
  printf("not registered: %s/%llu\n", name.c_str(), (unsigned long long)width);
  return 5;
}
