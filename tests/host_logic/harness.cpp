// Host-logic harness for tests/test_host_logic.py: runs the library's pure
// C++ host code (pwm_gb300/csrc/host_huffman.hpp, host_stream.hpp) on inputs
// from stdin and prints the results.
//
//   harness huff <is_tree> <width>   stdin: nsym, then "count first" per symbol
//                                    stdout: levels, level sizes, then "len word" per symbol
//   harness lc <seed> <trials>       randomized self-check of LevelCompletion
//   harness plan <L> <tree> <kmax> <T>  stdin: the 2^L leaf counts
//                                    stdout: the tile-pass plan (host_tables.hpp)
//   harness merge <L> <shards> <tree>    stdin: each shard's 2^L leaf counts
//                                    stdout: per level, the merge runs "dst shard src len"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "../../pwm_gb300/csrc/host_huffman.hpp"
#include "../../pwm_gb300/csrc/host_stream.hpp"
#include "../../pwm_gb300/csrc/host_tables.hpp"
#include "../../pwm_gb300/csrc/staging.hpp"

using namespace pwmgpu;

static int huff(bool is_tree, uint32_t width) {
  unsigned long long nsym = 0;
  if (scanf("%llu", &nsym) != 1) return 2;
  std::vector<uint64_t> count(nsym), first(nsym);
  uint64_t max_symbol = 0;
  for (uint64_t c = 0; c < nsym; ++c) {
    unsigned long long k = 0, f = 0;
    if (scanf("%llu %llu", &k, &f) != 2) return 2;
    count[c] = k;
    first[c] = f;
    if (k) max_symbol = c;
  }
  const auto entries = width == 1 ? histogram_order<uint8_t>(count, first, 1) : histogram_order<uint16_t>(count, first, 2);
  const HuffCodes h = build_huffman_codes(entries, max_symbol, is_tree);
  printf("%u\n", h.levels);
  for (uint64_t s : h.level_sizes) printf("%llu ", (unsigned long long)s);
  printf("\n");
  for (size_t c = 0; c < h.len.size(); ++c) printf("%llu %llu\n", (unsigned long long)h.len[c], (unsigned long long)h.word[c]);
  return 0;
}

// Random partitions of levels into bit ranges, recorded in random order: every
// word must be reported exactly once, only once all its bits are written, and
// overlapping or out-of-range ranges must be refused.
static int lc(uint64_t seed, int trials) {
  std::mt19937_64 rng(seed);
  for (int trial = 0; trial < trials; ++trial) {
    const uint64_t n = rng() % 3000 + 1;
    const uint64_t lw = (n + 63) / 64 + rng() % 4;
    std::vector<uint64_t> cuts{0, n};
    const int k = int(rng() % 16);
    for (int i = 0; i < k; ++i) cuts.push_back(rng() % (n + 1));
    std::sort(cuts.begin(), cuts.end());
    std::vector<std::pair<uint64_t, uint64_t>> parts;
    for (size_t i = 0; i + 1 < cuts.size(); ++i) parts.push_back({cuts[i], cuts[i + 1]});
    std::shuffle(parts.begin(), parts.end(), rng);
    LevelCompletion done(2, n);
    std::vector<int> sent(lw, 0), written(n, 0);
    for (auto& p : parts) {
      std::vector<std::pair<uint64_t, uint64_t>> out;
      if (!done.add(1, p.first, p.second, lw, out)) { printf("refused a valid range\n"); return 1; }
      for (uint64_t b = p.first; b < p.second; ++b) written[b] = 1;
      for (auto& w : out)
        for (uint64_t x = w.first; x < w.second; ++x) {
          if (x >= lw || sent[x]) { printf("word %llu reported twice or past the level\n", (unsigned long long)x); return 1; }
          for (uint64_t b = x * 64; b < x * 64 + 64 && b < n; ++b)
            if (!written[b]) { printf("word %llu reported early\n", (unsigned long long)x); return 1; }
          sent[x] = 1;
        }
    }
    for (uint64_t x = 0; x < lw; ++x)
      if (!sent[x]) { printf("word %llu never reported\n", (unsigned long long)x); return 1; }
    if (!done.complete(1)) { printf("level not complete\n"); return 1; }
    std::vector<std::pair<uint64_t, uint64_t>> out;
    if (parts.size() && parts[0].second > parts[0].first && done.add(1, parts[0].first, parts[0].second, lw, out)) {
      printf("accepted a range twice\n");
      return 1;
    }
    if (done.add(1, 0, n + 1, lw, out) || done.add(2, 0, 1, lw, out)) { printf("accepted an invalid range\n"); return 1; }
  }
  printf("ok\n");
  return 0;
}

// The plan of a plain tile build from its leaf histogram: zero counts, tree
// levels left to the regroup, and per pass its segments and start tables.
static int plan(uint32_t L, bool tree, int kmax, uint32_t T) {
  std::vector<uint64_t> hist(size_t(1) << L);
  for (auto& h : hist) {
    unsigned long long v = 0;
    if (scanf("%llu", &v) != 1) return 2;
    h = v;
  }
  const PrefixCounts cnt = fold_prefix_counts(hist.data(), L);
  std::vector<uint32_t> regroup;
  const auto passes = plan_tile_passes(cnt, L, kmax, T, tree, &regroup);
  // the same plan from every pass's digit counts, summed from the leaves
  // (what launch_flat_digits derives from the prefix counts on the device)
  {
    const auto shape = plan_passes(L, kmax);
    std::vector<uint64_t> digits(16 * shape.size(), 0);
    for (size_t s = 0; s < hist.size(); ++s)
      for (size_t p = 0; p < shape.size(); ++p)
        if (shape[p].K <= 4)
          digits[16 * p + ((s >> (L - shape[p].level - uint32_t(shape[p].K))) & ((size_t(1) << shape[p].K) - 1))] +=
              hist[s];
    std::vector<uint32_t> regroup2;
    const auto passes2 = plan_tile_passes(cnt, L, kmax, T, tree, &regroup2, digits.data());
    bool same = regroup2 == regroup && passes2.size() == passes.size();
    for (size_t p = 0; same && p < passes.size(); ++p)
      same = passes2[p].table == passes[p].table && passes2[p].segs.size() == passes[p].segs.size() &&
             passes2[p].tiles == passes[p].tiles;
    if (!same) {
      fprintf(stderr, "plan from digit counts differs\n");
      return 3;
    }
  }
  const LevelTables t = build_tables_tile(cnt, L, tree ? regroup : std::vector<uint32_t>{});
  printf("zeros");
  for (uint64_t z : t.zeros) printf(" %llu", (unsigned long long)z);
  printf("\nregroup");
  for (uint32_t r : regroup) printf(" %u", r);
  printf("\n");
  for (const auto& p : passes) {
    printf("pass %u %d %d %d %u %zu\n", p.level, p.K, int(p.out), int(p.segmented), p.tiles, p.segs.size());
    for (const auto& sg : p.segs) {
      printf("seg %llu %llu %u %llu\ntable", (unsigned long long)sg.in_begin, (unsigned long long)sg.m, sg.tile0,
             (unsigned long long)sg.group);
      for (int i = 0; i < tile_table_size(p.K); ++i) printf(" %llu", (unsigned long long)p.table[sg.table + i]);
      printf("\n");
    }
  }
  return 0;
}

// Matrix-only plans two ways from one leaf histogram: from the folded
// prefix counts of every level (plan_tile_passes) and from the digit counts
// of each pass alone (plan_matrix_passes, what the device counts for deep
// matrix-only builds); both plans and the zero counts must agree.
static int digits(uint32_t L, int kmax, uint32_t T) {
  std::vector<uint64_t> hist(size_t(1) << L);
  for (auto& h : hist) {
    unsigned long long v = 0;
    if (scanf("%llu", &v) != 1) return 2;
    h = v;
  }
  const PrefixCounts cnt = fold_prefix_counts(hist.data(), L);
  std::vector<uint32_t> regroup;
  const auto a = plan_tile_passes(cnt, L, kmax, T, false, &regroup);
  const auto shape = plan_passes(L, kmax);
  std::vector<uint64_t> dg(16 * shape.size(), 0);
  for (size_t p = 0; p < shape.size(); ++p)
    for (uint64_t x = 0; x < hist.size(); ++x)
      dg[16 * p + ((x >> (L - shape[p].level - uint32_t(shape[p].K))) & ((1u << shape[p].K) - 1))] += hist[x];
  const auto b = plan_matrix_passes(dg.data(), cnt[0][0], L, kmax, [T](uint32_t) { return T; });
  if (a.size() != b.size() || !regroup.empty()) { printf("pass count\n"); return 1; }
  for (size_t p = 0; p < a.size(); ++p) {
    if (a[p].level != b[p].level || a[p].K != b[p].K || a[p].out != b[p].out || a[p].tiles != b[p].tiles ||
        a[p].table != b[p].table || a[p].segs.size() != b[p].segs.size() || a[p].segmented || b[p].segmented) {
      printf("pass %zu differs\n", p);
      return 1;
    }
    for (size_t i = 0; i < a[p].segs.size(); ++i)
      if (a[p].segs[i].in_begin != b[p].segs[i].in_begin || a[p].segs[i].m != b[p].segs[i].m ||
          a[p].segs[i].table != b[p].segs[i].table || a[p].segs[i].tile0 != b[p].segs[i].tile0) {
        printf("pass %zu segment %zu differs\n", p, i);
        return 1;
      }
  }
  const LevelTables t = build_tables_tile(cnt, L, {});
  if (t.zeros != matrix_pass_zeros(dg.data(), L, kmax)) { printf("zeros differ\n"); return 1; }
  printf("ok %zu\n", a.size());
  return 0;
}

static int merge(uint32_t L, uint32_t shards, bool tree) {
  std::vector<PrefixCounts> cnt;
  std::vector<uint64_t> hist(size_t(1) << L);
  for (uint32_t s = 0; s < shards; ++s) {
    for (auto& h : hist) {
      unsigned long long v = 0;
      if (scanf("%llu", &v) != 1) return 2;
      h = v;
    }
    cnt.push_back(fold_prefix_counts(hist.data(), L));
  }
  for (uint32_t l = 0; l < L; ++l) {
    printf("level %u\n", l);
    for (const MergeRun& r : plan_merge_level(cnt, l, tree))
      printf("%llu %llu %llu %llu\n", (unsigned long long)r.dst, (unsigned long long)r.shard,
             (unsigned long long)r.src_bit, (unsigned long long)r.len);
  }
  return 0;
}

// The staging copy pool: every size around its slice and 4 KiB boundaries,
// with 1..9 threads, copies exactly the bytes asked for and nothing past them.
static int copy(unsigned seed) {
  std::mt19937_64 rng(seed);
  const uint64_t sizes[] = {0, 1, 4095, 4096, 4097, (1u << 20) - 1, 1u << 20, (1u << 20) + 1, 3u << 20,
                            (5u << 20) + 12345, 33u << 20};
  for (unsigned threads = 1; threads <= 9; ++threads) {
    pwmgpu::CopyPool pool(threads);
    if (pool.threads() != threads) return 3;
    for (uint64_t n : sizes) {
      std::vector<unsigned char> src(n + 64), dst(n + 64, 0xA5);
      for (auto& c : src) c = (unsigned char)(rng() & 0xFF);
      pool.copy(dst.data() + 7, src.data() + 7, n);
      for (uint64_t i = 0; i < n + 64; ++i) {
        const bool inside = i >= 7 && i < 7 + n;
        if (dst[i] != (inside ? src[i] : 0xA5)) {
          printf("threads %u size %llu byte %llu\n", threads, (unsigned long long)n, (unsigned long long)i);
          return 1;
        }
      }
    }
  }
  printf("ok\n");
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 3 && !strcmp(argv[1], "copy")) return copy(unsigned(atoi(argv[2])));
  if (argc >= 5 && !strcmp(argv[1], "digits"))
    return digits(uint32_t(atoi(argv[2])), atoi(argv[3]), uint32_t(atoi(argv[4])));
  if (argc >= 5 && !strcmp(argv[1], "merge"))
    return merge(uint32_t(atoi(argv[2])), uint32_t(atoi(argv[3])), atoi(argv[4]) != 0);
  if (argc >= 6 && !strcmp(argv[1], "plan"))
    return plan(uint32_t(atoi(argv[2])), atoi(argv[3]) != 0, atoi(argv[4]), uint32_t(atoi(argv[5])));
  if (argc >= 4 && !strcmp(argv[1], "huff")) return huff(atoi(argv[2]) != 0, uint32_t(atoi(argv[3])));
  if (argc >= 4 && !strcmp(argv[1], "lc")) return lc(strtoull(argv[2], nullptr, 10), atoi(argv[3]));
  fprintf(stderr, "usage: harness huff <is_tree> <width> | lc <seed> <trials> | plan <L> <tree> <kmax> <T>\n");
  return 2;
}
