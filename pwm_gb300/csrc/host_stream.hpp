// Host side of streaming a build's levels to host memory while the passes
// still run: which words of a level are complete as bit ranges of it are
// written.  Pure C++ (tested on the host alone).
#pragma once

#include <algorithm>
#include <cstdint>
#include <iterator>
#include <map>
#include <utility>
#include <vector>

namespace pwmgpu {

// Words of a structure's levels that become complete as bit ranges of them
// are written: a word is complete once all its bits are (bits past the
// level's end count as written); each word is reported once.
class LevelCompletion {
 public:
  LevelCompletion(uint32_t levels, uint64_t nbits) : done_(levels), nbits_(nbits) {}
  // Bits [a, b) of level m (of level_words words) are written: appends the
  // words [w0, w1) of the level that this completes.  False (nothing
  // recorded) for a range past the level or one that overlaps a recorded one.
  bool add(uint32_t m, uint64_t a, uint64_t b, uint64_t level_words, std::vector<std::pair<uint64_t, uint64_t>>& out) {
    if (a >= b) return true;
    if (b > nbits_ || m >= done_.size()) return false;
    auto& iv = done_[m];
    uint64_t A = a, B = b;
    auto it = iv.upper_bound(a);
    if (it != iv.begin()) {
      auto pv = std::prev(it);
      if (pv->second > a) return false;
      if (pv->second == a) {
        A = pv->first;
        iv.erase(pv);
      }
    }
    while (it != iv.end() && it->first <= B) {
      if (it->first < B) return false;
      B = it->second;
      it = iv.erase(it);
    }
    iv[A] = B;
    // [a, b) touches words [a/64, ceil(b/64)) (to the level's end if it
    // reaches it), none complete before; those inside [A, B) are now
    const uint64_t c0 = (A + 63) / 64, c1 = B == nbits_ ? level_words : B / 64;
    const uint64_t w0 = std::max(c0, a / 64), w1 = std::min(c1, b == nbits_ ? level_words : (b + 63) / 64);
    if (w0 < w1) out.emplace_back(w0, w1);
    return true;
  }
  bool complete(uint32_t m) const {
    const auto& iv = done_[m];
    return nbits_ == 0 || (iv.size() == 1 && iv.begin()->first == 0 && iv.begin()->second == nbits_);
  }

 private:
  std::vector<std::map<uint64_t, uint64_t>> done_;
  uint64_t nbits_;
};

}  // namespace pwmgpu
