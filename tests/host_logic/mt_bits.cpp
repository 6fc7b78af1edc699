// The bit vector of pwm's select test (test/bin_rank_select_tests.cpp:38-61):
// 2^27 bits, word by word from std::uniform_int_distribution<uint64_t>(0) over
// std::mt19937(44227).  Writes the 2^21 words (native byte order) to argv[1].
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const size_t words = (size_t(1024) * 1024 * 128) / 64;
  std::vector<uint64_t> w(words);
  std::mt19937 gen(44227);
  std::uniform_int_distribution<uint64_t> dis(0);
  for (auto& x : w) x = dis(gen);
  FILE* f = std::fopen(argv[1], "wb");
  if (!f) return 1;
  const size_t put = std::fwrite(w.data(), 8, w.size(), f);
  std::fclose(f);
  return put == w.size() ? 0 : 1;
}
