// Huffman code tables on the host, as pwm builds them.  Pure C++ (tested on
// the host alone against pwm's code tables).
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <numeric>
#include <unordered_map>
#include <utility>
#include <vector>

namespace pwmgpu {

// ---------------------------------------------------------------------------
// Huffman codes: pwm's canonical_huff_codes (include/huffman/huff_codes.hpp:
// 140-285) with the same standard containers, so that priority-queue and
// sort ties break the same way.
// ---------------------------------------------------------------------------
struct HuffCodes {
  std::vector<uint64_t> len, word, level_sizes;
  uint32_t levels = 0;
};

// The merges of pwm's priority queue of items T (compare: "greater" by
// occurrences only, as std::greater on pwm's items): child[2i], child[2i+1]
// are the nodes merge i popped (leaves are nodes 0..leaves-1, merge i makes
// node leaves + i).  Returns the number of merges.
template <typename T, typename Cmp, typename Make, typename Occ, typename Node>
inline uint32_t huffman_merges(const std::vector<std::pair<uint64_t, uint64_t>>& entries, std::vector<uint32_t>& child,
                               Cmp comp, Make make, Occ occ, Node node) {
  std::vector<T> heap;
  heap.reserve(entries.size());
  auto push = [&](T it) {
    heap.push_back(it);
    std::push_heap(heap.begin(), heap.end(), comp);
  };
  auto pop = [&]() {
    std::pop_heap(heap.begin(), heap.end(), comp);
    const T it = heap.back();
    heap.pop_back();
    return it;
  };
  for (size_t i = 0; i < entries.size(); ++i) push(make(entries[i].second, uint32_t(i)));
  uint32_t merges = 0;
  while (heap.size() > 1) {
    const T a = pop();
    const T b = pop();
    child[2 * merges] = node(a);
    child[2 * merges + 1] = node(b);
    push(make(occ(a) + occ(b), uint32_t(entries.size() + merges)));
    ++merges;
  }
  return merges;
}

// entries: (symbol, frequency) in pwm's histogram order.
inline HuffCodes build_huffman_codes(const std::vector<std::pair<uint64_t, uint64_t>>& entries, uint64_t max_symbol,
                                     bool is_tree) {
  HuffCodes h;
  if (entries.empty()) return h;
  const uint64_t nsym = max_symbol + 1;
  std::vector<uint64_t> freq(nsym, 0);
  for (const auto& e : entries) freq[e.first] = e.second;
  // pwm merges the two least frequent items of a std::priority_queue<Item,
  // std::vector<Item>, std::greater<Item>> (ordered by occurrences only) and
  // lengthens the codes of all symbols of the merged item, so a code length
  // is the depth of the symbol's leaf in the tree of merges.  The same heap
  // operations (push: push_back + push_heap, pop: pop_heap + pop_back) on
  // (occurrences, node) items compared by occurrences only break ties
  // identically; the depths come from one pass over the merge tree, parents
  // before children.  Items are one 64-bit word (occurrences above the node
  // bits) when the text's total fits beside them: half the bytes the heap
  // moves, the same comparisons.
  h.len.assign(nsym, 0);
  h.word.assign(nsym, 0);
  const size_t leaves = entries.size();
  std::vector<uint32_t> child(2 * leaves, 0);  // node leaves + i: children of merge i at 2i, 2i + 1
  if (leaves == 1) ++h.len[entries[0].first];
  uint64_t total = 0;
  bool fits = true;
  for (const auto& e : entries) fits = fits && !__builtin_add_overflow(total, e.second, &total);
  uint32_t nb = 1;  // node bits
  while ((uint64_t(1) << nb) < 2 * leaves) ++nb;
  fits = fits && nb < 64 && total < (uint64_t(1) << (64 - nb));
  uint32_t merges = 0;
  if (fits) {
    const uint64_t nmask = (uint64_t(1) << nb) - 1;
    merges = huffman_merges<uint64_t>(
        entries, child, [nb](uint64_t a, uint64_t b) { return (a >> nb) > (b >> nb); },
        [nb](uint64_t occ, uint32_t node) { return (occ << nb) | node; }, [nb](uint64_t a) { return a >> nb; },
        [nmask](uint64_t a) { return uint32_t(a & nmask); });
  } else {
    struct Item {
      uint64_t occ;
      uint32_t node;
    };
    merges = huffman_merges<Item>(
        entries, child, [](const Item& a, const Item& b) { return a.occ > b.occ; },
        [](uint64_t occ, uint32_t node) { return Item{occ, node}; }, [](const Item& a) { return a.occ; },
        [](const Item& a) { return a.node; });
  }
  if (merges) {
    std::vector<uint64_t> depth(leaves + merges, 0);
    for (uint32_t i = merges; i-- > 0;)  // the last merge is the root
      for (int k = 0; k < 2; ++k) depth[child[2 * i + k]] = depth[leaves + i] + 1;
    for (size_t i = 0; i < leaves; ++i) h.len[entries[i].first] = depth[i];
  }
  std::vector<uint64_t> order(nsym);
  std::iota(order.begin(), order.end(), uint64_t(0));
  std::sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) { return h.len[a] < h.len[b]; });
  h.levels = uint32_t(h.len[order.back()]);
  std::vector<uint64_t> sizes(h.levels, 0);
  uint64_t k = 0;
  while (k < nsym && h.len[order[k]] == 0) ++k;
  if (!is_tree) {
    uint64_t cur = 1;
    std::vector<uint64_t> words{0, 1};
    while (k < nsym) {
      if (h.len[order[k]] > cur) {
        for (uint64_t i = cur; i < h.len[order[k]]; ++i) {
          std::vector<uint64_t> nw;
          nw.reserve(words.size() * 2);
          for (uint64_t cw : words) nw.push_back(cw << 1);
          for (uint64_t cw : words) nw.push_back((cw << 1) + 1);
          words = std::move(nw);
        }
        cur = h.len[order[k]];
      }
      while (k < nsym && h.len[order[k]] == cur) {
        const uint64_t sy = order[k++];
        h.word[sy] = words.back();
        words.pop_back();
        sizes[h.len[sy] - 1] += freq[sy];
      }
    }
  } else {
    uint64_t cw = 0;
    auto gen = [&]() {
      const uint64_t sy = order[k];
      h.word[sy] = (~cw) & ((uint64_t(1) << h.len[sy]) - 1);
      sizes[h.len[sy] - 1] += freq[sy];
    };
    gen();
    for (++k; k < nsym; ++k) {
      cw = (cw + 1) << (h.len[order[k]] - h.len[order[k - 1]]);
      gen();
    }
  }
  for (uint64_t i = h.levels - 1; i > 0; --i) sizes[i - 1] += sizes[i];
  h.level_sizes = sizes;
  return h;
}

// Allocator for pwm's histogram map: nodes come from one block that lives as
// long as the map (allocation does not change a std::unordered_map's bucket
// sequence, so the iteration order stays pwm's).
struct NodeArena {
  std::vector<std::max_align_t> block;
  size_t used = 0;  // in units of max_align_t
};
template <typename T>
struct ArenaAlloc {
  using value_type = T;
  NodeArena* arena;
  explicit ArenaAlloc(NodeArena* a) : arena(a) {}
  template <typename U>
  ArenaAlloc(const ArenaAlloc<U>& o) : arena(o.arena) {}
  T* allocate(size_t n) {
    const size_t units = (n * sizeof(T) + sizeof(std::max_align_t) - 1) / sizeof(std::max_align_t);
    if (alignof(T) <= alignof(std::max_align_t) && arena->used + units <= arena->block.size()) {
      T* p = reinterpret_cast<T*>(arena->block.data() + arena->used);
      arena->used += units;
      return p;
    }
    return static_cast<T*>(::operator new(n * sizeof(T)));
  }
  void deallocate(T* p, size_t) {
    const auto* b = reinterpret_cast<const std::max_align_t*>(p);
    if (b < arena->block.data() || b >= arena->block.data() + arena->block.size()) ::operator delete(p);
  }
  template <typename U>
  bool operator==(const ArenaAlloc<U>& o) const { return arena == o.arena; }
  template <typename U>
  bool operator!=(const ArenaAlloc<U>& o) const { return arena != o.arena; }
};

// pwm's histogram order (include/util/histogram.hpp:39-76): ascending symbols
// for 8-bit texts; for wider texts the iteration order of a
// std::unordered_map filled in order of first occurrence (a default map, as
// pwm's, so the same buckets and rehashes; first occurrences are distinct, so
// a radix sort of (first, symbol) gives the one insert order).
template <typename A>
inline std::vector<std::pair<uint64_t, uint64_t>> histogram_order(const std::vector<uint64_t>& count,
                                                                  const std::vector<uint64_t>& first, uint32_t width) {
  std::vector<std::pair<uint64_t, uint64_t>> out;
  if (width == 1) {
    for (uint64_t c = 0; c < count.size(); ++c)
      if (count[c]) out.emplace_back(c, count[c]);
    return out;
  }
  std::vector<std::pair<uint64_t, uint64_t>> fs, tmp;  // (first occurrence, symbol)
  uint64_t top = 0;
  for (uint64_t c = 0; c < count.size(); ++c)
    if (count[c]) {
      fs.emplace_back(first[c], c);
      top |= first[c];
    }
  tmp.resize(fs.size());
  std::vector<uint32_t> cnt(65537);
  for (int sh = 0; sh < 64 && (top >> sh); sh += 16) {  // LSD, 16-bit digits
    std::fill(cnt.begin(), cnt.end(), 0u);
    for (const auto& p : fs) ++cnt[((p.first >> sh) & 0xFFFF) + 1];
    for (size_t i = 0; i < 65536; ++i) cnt[i + 1] += cnt[i];
    for (const auto& p : fs) tmp[cnt[(p.first >> sh) & 0xFFFF]++] = p;
    fs.swap(tmp);
  }
  using Node = std::pair<const A, uint64_t>;
  NodeArena arena;
  arena.block.resize(fs.size() * ((sizeof(Node) + 2 * sizeof(void*) + sizeof(std::max_align_t) - 1) /
                                  sizeof(std::max_align_t)) + 64);
  {
    std::unordered_map<A, uint64_t, std::hash<A>, std::equal_to<A>, ArenaAlloc<Node>> m{ArenaAlloc<Node>(&arena)};
    for (const auto& p : fs) m.emplace(A(p.second), count[p.second]);
    out.reserve(m.size());
    for (const auto& e : m) out.emplace_back(uint64_t(e.first), e.second);
  }
  return out;
}

}  // namespace pwmgpu
