// Popcount rank/select support in pwm's layout and batched queries.
//
// Layout (include/queries/bin_rank_popcnt.hpp:32-86, popcnt_traits.hpp:
// 12-21): per level, one l12 entry per L1 block of 32 words (2048 bits): the
// u32 count of ones before the block (wrapping like pwm's u32) and the ones
// of its first three 512-bit L2 blocks in 10-bit fields.  When the level has
// a multiple of 32 words pwm keeps one more, zeroed, entry; so does this
// layout.  l0 is all zero for levels below 2^32-1 bits (the only sizes
// accepted).  Select samples (bin_select_popcnt.hpp:38-107): the position of
// every 8192nd zero/one, taken in the L1 block where the running count first
// exceeds the next sample number.
#include <algorithm>
#include <mutex>

#include "kernels.cuh"

namespace pwmgpu {

namespace {

constexpr uint64_t kL1Bits = 2048, kL2Bits = 512, kL1Cover = 32, kL2Cover = 8, kSampleRate = 8192;
constexpr int kRsThreads = 256;

__device__ __forceinline__ uint32_t l2_of(const uint32_t* l12, uint64_t e, uint32_t i) {
  return (l12[2 * e + 1] >> (10 * i)) & 1023u;
}

// Phase 1: per L1 block popcounts, l2 fields, and the exclusive prefix of
// block totals inside each CTA (256 blocks per CTA).  Warp w reads its 32
// blocks (8 KB) with coalesced 16-byte loads: in step i, lanes 0-15 read
// block 2i and lanes 16-31 block 2i+1, four lanes per 512-bit L2 block; the
// counts are then gathered so that lane b holds block b's.
__global__ void __launch_bounds__(kRsThreads) rs_blocks_kernel(const RankSelectLevel* lv, uint32_t* tmp,
                                                              uint64_t tmp_stride) {
  const RankSelectLevel L = lv[blockIdx.y];
  const uint64_t nreal = (L.nwords + kL1Cover - 1) / kL1Cover;
  const uint64_t first = uint64_t(blockIdx.x) * kRsThreads;
  if (first >= nreal) return;
  uint32_t* intra = tmp + blockIdx.y * tmp_stride;
  uint32_t* cta_tot = intra + nreal;
  __shared__ uint32_t tot[kRsThreads];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  {
    const uint64_t wb = first + 32 * uint64_t(warp);  // first block of this warp
    const uint64_t ww = wb * kL1Cover;                 // first word of this warp
    // 16-byte loads when the warp's words are all in the level and aligned
    const bool full = ww + 32 * kL1Cover <= L.nwords && (reinterpret_cast<uintptr_t>(L.data) & 15) == 0;
    uint32_t l2[4] = {0, 0, 0, 0};
    auto gather = [&](int i, uint32_t c) {
      c += __shfl_xor_sync(0xFFFFFFFFu, c, 1);
      c += __shfl_xor_sync(0xFFFFFFFFu, c, 2);
      // lane 2i takes block 2i's four counts (lanes 0,4,8,12), lane 2i+1 block 2i+1's (16,20,24,28)
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint32_t x = __shfl_sync(0xFFFFFFFFu, c, (lane & 1) * 16 + 4 * k);
        if ((lane >> 1) == i) l2[k] = x;
      }
    };
    if (full) {
      // all 16 loads of the lane in flight before the first popcount
      uint32_t c[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const uint4 v = __ldcs(reinterpret_cast<const uint4*>(L.data + ww + 2 * uint64_t(i * 32 + lane)));
        c[i] = __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) gather(i, c[i]);
    } else {
      for (int i = 0; i < 16; ++i) {
        const uint64_t w = ww + 2 * uint64_t(i * 32 + lane);  // first of this lane's two words
        gather(i, (w < L.nwords ? __popcll(L.data[w]) : 0) + (w + 1 < L.nwords ? __popcll(L.data[w + 1]) : 0));
      }
    }
    const uint64_t blk = wb + lane;
    if (blk < nreal) L.l12[2 * blk + 1] = (l2[0] & 1023u) | ((l2[1] & 1023u) << 10) | ((l2[2] & 1023u) << 20);
    tot[threadIdx.x] = blk < nreal ? l2[0] + l2[1] + l2[2] + l2[3] : 0u;
  }
  // exclusive scan of the 256 block totals (u32, wrapping)
  uint32_t v = tot[threadIdx.x];
  uint32_t x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
    if (lane >= d) x += y;
  }
  __shared__ uint32_t wsum[kRsThreads / 32];
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < kRsThreads / 32 ? wsum[lane] : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, d);
      if (lane >= d) s += y;
    }
    if (lane < kRsThreads / 32) wsum[lane] = s;  // inclusive
  }
  __syncthreads();
  const uint32_t warp_excl = warp ? wsum[warp - 1] : 0u;
  const uint64_t blk = first + threadIdx.x;
  if (blk < nreal) intra[blk] = warp_excl + x - v;
  if (threadIdx.x == kRsThreads - 1) cta_tot[blockIdx.x] = warp_excl + x;
}

// Phase 2: one CTA per level scans the CTA totals (exclusive, u32 wrap) and
// the exact u64 total of ones.
__global__ void __launch_bounds__(1024) rs_scan_kernel(const RankSelectLevel* lv, uint32_t* tmp,
                                                       uint64_t tmp_stride) {
  const RankSelectLevel L = lv[blockIdx.x];
  const uint64_t nreal = (L.nwords + kL1Cover - 1) / kL1Cover;
  const uint64_t ncta = (nreal + kRsThreads - 1) / kRsThreads;
  uint32_t* cta_tot = tmp + blockIdx.x * tmp_stride + nreal;
  // l0: all zero below 2^32-1 bits per level (the only sizes built); the
  // sample counts stay 0 for levels too short to examine a block
  // (rs_finish_kernel writes them otherwise)
  for (uint64_t i = threadIdx.x; i < L.nwords / (4294967295ull / 64) + 1; i += blockDim.x) L.l0[i] = 0;
  if (threadIdx.x == 0) {
    L.meta[0] = 0;
    L.meta[1] = 0;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ unsigned long long wsum[32];
  __shared__ unsigned long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint64_t base = 0; base < ncta; base += 1024) {
    const uint64_t i = base + threadIdx.x;
    const unsigned long long v = i < ncta ? cta_tot[i] : 0ull;
    unsigned long long x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      unsigned long long s = wsum[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, s, d);
        if (lane >= d) s += y;
      }
      wsum[lane] = s;
    }
    __syncthreads();
    const unsigned long long excl = carry + (warp ? wsum[warp - 1] : 0ull) + x - v;
    if (i < ncta) cta_tot[i] = uint32_t(excl);  // now the CTA's exclusive offset
    __syncthreads();
    if (threadIdx.x == 1023) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) L.meta[2] = carry;  // total ones of the level
}

__device__ __forceinline__ uint32_t l1_value(const uint32_t* intra, const uint32_t* cta_off, uint64_t nreal,
                                             uint64_t e) {
  // pwm's l1 value of entry e; the extra entry past the real blocks is 0.
  return e < nreal ? cta_off[e / kRsThreads] + intra[e] : 0u;
}

// Select-sample position inside L1 block b: the `rem`-th one (value 1) or
// zero (value 0) counted from the block's first word, found by one thread.
// pwm walks the L2 blocks and then the words of the block
// (bin_select_popcnt.hpp:55-99); skipping whole L2 blocks by their counts
// first does not change which word and rank it ends on, so this gives the
// same position.  Only words of the level count (the last block may be
// short).  rem == 0 is pwm's word_select1(first word, 0).  Returns false when
// the block ends before the rem-th bit (pwm then takes no sample).
__device__ __forceinline__ bool thread_block_select(const uint64_t* data, uint64_t nwords, const uint32_t* l12,
                                                    uint64_t b, int value, uint32_t rem, uint64_t* pos) {
  const uint64_t w0 = b * kL1Cover;
  if (rem == 0) {
    const uint64_t first = value ? data[w0] : ~data[w0];
    *pos = word_select1(first, 0) + 64 * w0;
    return true;
  }
  // skip whole L2 blocks (8 words) by their counts; the fourth has no field
  const uint32_t fields = l12[2 * b + 1];
  uint32_t sub = 0;
  for (; sub < 3; ++sub) {
    const uint64_t ws = w0 + kL2Cover * sub;
    const uint64_t left = ws >= nwords ? 0 : nwords - ws;
    const uint32_t words = uint32_t(left < kL2Cover ? left : kL2Cover);
    const uint32_t ones = (fields >> (10 * sub)) & 1023u;
    const uint32_t cnt = value ? ones : 64u * words - ones;
    if (rem <= cnt) break;
    rem -= cnt;
  }
  const uint64_t ws = w0 + kL2Cover * sub;
  for (uint32_t k = 0; k < kL2Cover; ++k) {
    if (ws + k >= nwords) return false;
    const uint64_t w = value ? data[ws + k] : ~data[ws + k];
    const uint32_t pc = uint32_t(__popcll(w));
    if (pc >= rem) {
      *pos = word_select1(w, rem) + 64 * (ws + k);
      return true;
    }
    rem -= pc;
  }
  return false;
}

// Phase 3: l1 values and the select samples, one thread per L1 block (the
// searches of a warp's blocks are independent, so their loads overlap).
__global__ void __launch_bounds__(kRsThreads) rs_finish_kernel(const RankSelectLevel* lv, const uint32_t* tmp,
                                                              uint64_t tmp_stride) {
  const RankSelectLevel L = lv[blockIdx.y];
  const uint64_t nreal = (L.nwords + kL1Cover - 1) / kL1Cover;
  const uint64_t n12 = L.nwords / kL1Cover + 1;
  const uint32_t* intra = tmp + blockIdx.y * tmp_stride;
  const uint32_t* cta_off = intra + nreal;
  const uint64_t b = uint64_t(blockIdx.x) * kRsThreads + threadIdx.x;
  if (b >= nreal) return;
  const uint64_t ones_before = l1_value(intra, cta_off, nreal, b);
  L.l12[2 * b] = uint32_t(ones_before);
  if (b == 0 && n12 > nreal) { L.l12[2 * nreal] = 0; L.l12[2 * nreal + 1] = 0; }
  if (b + 1 >= n12) return;  // pwm examines blocks 0 .. n12-2
  const uint64_t ones_through = l1_value(intra, cta_off, nreal, b + 1);
  // sample s is taken in the first block whose running count exceeds
  // 1 + 8192 s (bin_select_popcnt.hpp:55-99)
  const uint64_t s1 = ones_before == 0 ? 0 : (ones_before - 1 + kSampleRate - 1) / kSampleRate;
  const uint64_t next1 = 1 + kSampleRate * s1;
  const bool need1 = ones_through > next1;
  const uint64_t f_prev = b * kL1Bits - ones_before;
  const uint64_t f_here = (b + 1) * kL1Bits - ones_through;
  const uint64_t s0 = f_prev == 0 ? 0 : (f_prev - 1 + kSampleRate - 1) / kSampleRate;
  const uint64_t next0 = 1 + kSampleRate * s0;
  const bool need0 = f_here > next0;
  bool got1 = false, got0 = false;
  uint64_t pos;
  if (need1 && thread_block_select(L.data, L.nwords, L.l12, b, 1, uint32_t(next1 - ones_before), &pos)) {
    L.s1[s1] = uint32_t(pos);
    got1 = true;
  }
  if (need0 && thread_block_select(L.data, L.nwords, L.l12, b, 0, uint32_t(next0 - f_prev), &pos)) {
    L.s0[s0] = uint32_t(pos);
    got0 = true;
  }
  // samples are taken in block order, so the count is fixed by the last
  // block pwm examines (n12 - 2): the samples before it plus its own
  if (b == n12 - 2) {
    L.meta[1] = s1 + (got1 ? 1 : 0);
    L.meta[0] = s0 + (got0 ? 1 : 0);
  }
}

// ---------------------------------------------------------------------------
// Queries (include/queries/query_support.hpp:39-178)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t q_rank1(const QueryLevel& L, uint64_t index) {
  // bin_rank_popcnt::rank1 (bin_rank_popcnt.hpp:98-128); the index of pwm's
  // extra zeroed L1 entry answers with the level's total instead of 0.
  const uint64_t nreal = (L.nwords + kL1Cover - 1) / kL1Cover;
  if (index > L.nwords * 64) index = L.nwords * 64;  // past the level: the padding holds no ones
  const uint64_t l1 = index / kL1Bits;
  if (l1 >= nreal) return L.meta[2];
  uint64_t rem = index - l1 * kL1Bits;
  uint64_t result = L.l12[2 * l1];
  const uint64_t l2 = rem / kL2Bits;
  rem -= l2 * kL2Bits;
  for (uint32_t i = 0; i < l2; ++i) result += l2_of(L.l12, l1, i);
  uint64_t off = l1 * kL1Cover + l2 * kL2Cover;
  while (rem >= 64) { result += __popcll(L.data[off++]); rem -= 64; }
  if (rem > 0) result += __popcll(L.data[off] >> (64 - rem));
  return result;
}
__device__ __forceinline__ uint64_t q_rank0(const QueryLevel& L, uint64_t index) { return index - q_rank1(L, index); }

// bin_select_popcnt::select (bin_select_popcnt.hpp:112-117, 166-241), with
// the scan start at sample (occ-1)/8192 and the block scan and word walk
// bounded by the real data (pwm reads past its arrays there).
__device__ uint64_t q_select(const QueryLevel& L, int value, uint64_t occ) {
  if (occ == 0) return 0;
  const uint64_t nreal = (L.nwords + kL1Cover - 1) / kL1Cover;
  const uint64_t ns = L.meta[value ? 1 : 0];
  const uint32_t* samples = value ? L.s1 : L.s0;
  const uint64_t sidx = (occ - 1) / kSampleRate;
  uint64_t l1;
  if (sidx < ns) {
    l1 = samples[sidx];
    if ((occ - 1) % kSampleRate == 0) return l1;
    l1 /= kL1Bits;
  } else {
    l1 = ns ? samples[ns - 1] / kL1Bits : 0;
  }
  if (value == 0) {
    while (l1 + 1 < nreal && (((l1 + 1) * kL1Bits) - L.l12[2 * (l1 + 1)]) < occ) ++l1;
    occ -= (l1 * kL1Bits) - L.l12[2 * l1];
  } else {
    while (l1 + 1 < nreal && L.l12[2 * (l1 + 1)] < occ) ++l1;
    occ -= L.l12[2 * l1];
  }
  uint32_t l2 = 0;
  if (value == 0) {
    while (l2 < 3 && occ > kL2Bits - l2_of(L.l12, l1, l2)) occ -= kL2Bits - l2_of(L.l12, l1, l2++);
  } else {
    while (l2 < 3 && occ > l2_of(L.l12, l1, l2)) occ -= l2_of(L.l12, l1, l2++);
  }
  const uint64_t last = kL2Cover * l2 + kL1Cover * l1;
  uint64_t extra = 0;
  for (;;) {
    if (last + extra >= L.nwords) return ~0ull;
    uint64_t w = L.data[last + extra];
    if (value == 0) w = ~w;
    const uint64_t pc = __popcll(w);
    if (pc >= occ) return kL2Bits * l2 + kL1Bits * l1 + extra * 64 + word_select1(w, uint32_t(occ));
    ++extra;
    occ -= pc;
  }
}

__device__ __forceinline__ bool bit_at(const uint64_t* d, uint64_t i) { return (d[i >> 6] >> (63 - (i & 63))) & 1; }

// ops: the kind of each query (a mixed batch), or null for `op` throughout.
__global__ void query_kernel(QueryStructure q, int op0, const uint8_t* __restrict__ ops,
                             const uint64_t* __restrict__ a, const uint64_t* __restrict__ b, uint64_t count,
                             uint64_t* __restrict__ out) {
  const uint32_t Lv = q.levels;
  for (uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < count; t += uint64_t(gridDim.x) * blockDim.x) {
    const int op = ops ? int(ops[t]) : op0;
    uint64_t result = 0;
    if (op == 0 && a[t] >= q.n) {  // access past the text
      result = ~0ull;
    } else if (op == 0) {  // access
      uint64_t index = a[t], word = 0;
      if (q.is_tree) {
        uint64_t start = 0, end = q.n;
        for (uint32_t level = 0; level < Lv; ++level) {
          const QueryLevel& L = q.lv[level];
          const uint64_t left = q_rank0(L, start), right = q_rank0(L, end);
          word <<= 1;
          if (bit_at(L.data, start + index)) {
            word |= 1;
            index = q_rank1(L, start + index) - (start - left);
            start = start + right - left;
          } else {
            index = q_rank0(L, start + index) - left;
            end = start + right - left;
          }
        }
      } else {
        for (uint32_t level = 0; level < Lv; ++level) {
          const QueryLevel& L = q.lv[level];
          word <<= 1;
          if (bit_at(L.data, index)) {
            word |= 1;
            index = q_rank1(L, index) + q.zeros[level];
          } else {
            index = q_rank0(L, index);
          }
        }
      }
      result = word;
    } else if (op == 1) {  // rank(symbol, index)
      const uint64_t sym = a[t];
      uint64_t index = b[t];
      if (index != 0) {
        if (q.is_tree) {
          uint64_t start = 0, end = q.n;
          for (uint32_t level = 0; level < Lv; ++level) {
            const QueryLevel& L = q.lv[level];
            const uint64_t left = q_rank0(L, start), right = q_rank0(L, end);
            if ((sym >> (Lv - level - 1)) & 1) {
              index = q_rank1(L, start + index) - (start - left);
              start = start + right - left;
            } else {
              index = q_rank0(L, start + index) - left;
              end = start + right - left;
            }
          }
          result = index;
        } else {
          uint64_t offset = 0;
          for (uint32_t level = 0; level < Lv; ++level) {
            const QueryLevel& L = q.lv[level];
            if ((sym >> (Lv - level - 1)) & 1) {
              index = q.zeros[level] + q_rank1(L, index);
              offset = q.zeros[level] + q_rank1(L, offset);
            } else {
              index = q_rank0(L, index);
              offset = q_rank0(L, offset);
            }
          }
          result = index - offset;
        }
      }
    } else {  // select(symbol, occ)
      const uint64_t sym = a[t];
      uint64_t occ = b[t];
      if (occ != 0) {
        uint64_t st[64], le[64];
        if (q.is_tree) {
          uint64_t start = 0, end = q.n;
          for (uint32_t level = 0; level < Lv; ++level) {
            const QueryLevel& L = q.lv[level];
            const uint64_t left = q_rank0(L, start), right = q_rank0(L, end);
            st[level] = start;
            le[level] = left;
            if ((sym >> (Lv - level - 1)) & 1) start = start + right - left;
            else end = start + right - left;
          }
          for (int level = int(Lv) - 1; level >= 0; --level) {
            const QueryLevel& L = q.lv[level];
            const uint64_t adj = level == 0 ? 0 : 1;
            if ((sym >> (Lv - level - 1)) & 1) occ = q_select(L, 1, st[level] - le[level] + occ) - st[level] + adj;
            else occ = q_select(L, 0, le[level] + occ) - st[level] + adj;
          }
        } else {
          uint64_t offset = 0;
          for (uint32_t level = 0; level < Lv; ++level) {
            const QueryLevel& L = q.lv[level];
            if ((sym >> (Lv - level - 1)) & 1) offset = q.zeros[level] + q_rank1(L, offset);
            else offset = q_rank0(L, offset);
          }
          occ += offset;
          for (int level = int(Lv) - 1; level >= 0; --level) {
            const QueryLevel& L = q.lv[level];
            const uint64_t adj = level == 0 ? 0 : 1;
            if ((sym >> (Lv - level - 1)) & 1) occ = q_select(L, 1, occ - q.zeros[level]) + adj;
            else occ = q_select(L, 0, occ) + adj;
          }
        }
        result = occ;
      }
    }
    out[t] = result;
  }
}

// ---------------------------------------------------------------------------
// Queries on Huffman-shaped structures (pwm's query_support has none: it
// prints "NOT YET IMPLEMENTED", include/queries/query_support.hpp:43,55,67).
//
// Level l holds bit l of every code longer than l.  In both shapes the codes
// that end at a level sort behind all codes that go on: the matrix's codes
// (huff_codes.hpp:204-245) take, length by length, the largest bit-reversed
// words, and the tree's are negated canonical codes (:246-283), the largest
// prefixes.  So level l + 1 is a prefix of level l's entries reordered as the
// plain structures reorder them (the matrix by its stable 0/1 partition, the
// tree within each node), and the plain position arithmetic holds; a code
// ends where its position falls past the next level's size.
// ---------------------------------------------------------------------------
__device__ uint64_t huff_decode(const HuffQueryTables& h, uint32_t len, uint64_t word) {
  const uint64_t key = (uint64_t(len) << 56) | word;
  uint64_t lo = 0, hi = h.ndec;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (h.dec_key[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo < h.ndec && h.dec_key[lo] == key ? h.dec_sym[lo] : ~0ull;
}

__global__ void huff_query_kernel(QueryStructure q, HuffQueryTables h, int op, const uint64_t* __restrict__ a,
                                  const uint64_t* __restrict__ b, uint64_t count, uint64_t* __restrict__ out) {
  const uint32_t Lv = q.levels;
  for (uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < count; t += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t result = ~0ull;
    if (op == 0) {  // access: read bits until the code ends
      if (a[t] < q.n) {
        uint64_t index = a[t], word = 0;
        if (q.is_tree) {
          uint64_t start = 0, end = q.n;
          for (uint32_t level = 0; level < Lv; ++level) {
            const QueryLevel& L = q.lv[level];
            const uint64_t left = q_rank0(L, start), right = q_rank0(L, end);
            const bool one = bit_at(L.data, start + index);
            word = (word << 1) | (one ? 1u : 0u);
            if (one) {
              index = q_rank1(L, start + index) - (start - left);
              start = start + right - left;
            } else {
              index = q_rank0(L, start + index) - left;
              end = start + right - left;
            }
            if (level + 1 == Lv || start + index >= h.level_bits[level + 1]) {
              result = huff_decode(h, level + 1, word);
              break;
            }
          }
        } else {
          for (uint32_t level = 0; level < Lv; ++level) {
            const QueryLevel& L = q.lv[level];
            const bool one = bit_at(L.data, index);
            word = (word << 1) | (one ? 1u : 0u);
            index = one ? q.zeros[level] + q_rank1(L, index) : q_rank0(L, index);
            if (level + 1 == Lv || index >= h.level_bits[level + 1]) {
              result = huff_decode(h, level + 1, word);
              break;
            }
          }
        }
      }
      out[t] = result;
      continue;
    }
    // rank(symbol, index) / select(symbol, occurrence): walk the symbol's code
    const uint64_t sym = a[t];
    const uint32_t len = sym < h.nsym ? uint32_t(h.code_len[sym]) : 0u;
    const uint64_t code = len ? h.code_word[sym] : 0;
    if (len == 0 || len > Lv) {  // a symbol without a code does not occur
      out[t] = (op == 1 || b[t] == 0) ? 0 : ~0ull;
      continue;
    }
    auto bit = [&](uint32_t level) { return (code >> (len - 1 - level)) & 1; };
    if (op == 1) {
      uint64_t index = b[t] < q.n ? b[t] : q.n;
      if (q.is_tree) {
        uint64_t start = 0, end = q.n;
        for (uint32_t level = 0; level < len && index; ++level) {
          const QueryLevel& L = q.lv[level];
          const uint64_t left = q_rank0(L, start), right = q_rank0(L, end);
          if (bit(level)) {
            index = q_rank1(L, start + index) - (start - left);
            start = start + right - left;
          } else {
            index = q_rank0(L, start + index) - left;
            end = start + right - left;
          }
        }
        result = index;
      } else {
        uint64_t offset = 0;
        for (uint32_t level = 0; level < len; ++level) {
          const QueryLevel& L = q.lv[level];
          if (bit(level)) {
            index = q.zeros[level] + q_rank1(L, index);
            offset = q.zeros[level] + q_rank1(L, offset);
          } else {
            index = q_rank0(L, index);
            offset = q_rank0(L, offset);
          }
        }
        result = index - offset;
      }
    } else {
      uint64_t occ = b[t];
      if (occ == 0) {
        result = 0;  // as the plain structures' select
      } else {
        if (q.is_tree) {
          uint64_t st[64], le[64];
          uint64_t start = 0, end = q.n;
          for (uint32_t level = 0; level < len; ++level) {
            const QueryLevel& L = q.lv[level];
            const uint64_t left = q_rank0(L, start), right = q_rank0(L, end);
            st[level] = start;
            le[level] = left;
            if (bit(level)) start = start + right - left;
            else end = start + right - left;
          }
          if (occ <= end - start) {  // the symbol's node holds its occurrences
            for (int level = int(len) - 1; level >= 0; --level) {
              const QueryLevel& L = q.lv[level];
              const uint64_t adj = level == 0 ? 0 : 1;
              if (bit(uint32_t(level))) occ = q_select(L, 1, st[level] - le[level] + occ) - st[level] + adj;
              else occ = q_select(L, 0, le[level] + occ) - st[level] + adj;
            }
            result = occ;
          }
        } else {
          uint64_t offset = 0, end = q.n;
          for (uint32_t level = 0; level < len; ++level) {
            const QueryLevel& L = q.lv[level];
            if (bit(level)) {
              offset = q.zeros[level] + q_rank1(L, offset);
              end = q.zeros[level] + q_rank1(L, end);
            } else {
              offset = q_rank0(L, offset);
              end = q_rank0(L, end);
            }
          }
          if (occ <= end - offset) {
            occ += offset;
            for (int level = int(len) - 1; level >= 0; --level) {
              const QueryLevel& L = q.lv[level];
              const uint64_t adj = level == 0 ? 0 : 1;
              if (bit(uint32_t(level))) occ = q_select(L, 1, occ - q.zeros[level]) + adj;
              else occ = q_select(L, 0, occ) + adj;
            }
            result = occ;
          }
        }
      }
    }
    out[t] = result;
  }
}

}  // namespace

void launch_huff_queries(const QueryStructure& q, const HuffQueryTables& h, int op, const uint64_t* a,
                         const uint64_t* b, uint64_t count, uint64_t* out, cudaStream_t s, uint64_t* launches) {
  if (count == 0) return;
  uint64_t blocks = (count + 127) / 128;
  if (blocks > 65535) blocks = 65535;
  huff_query_kernel<<<unsigned(blocks), 128, 0, s>>>(q, h, op, a, b, count, out);
  ++*launches;
}

void launch_rank_select(const RankSelectLevel* host_levels, uint32_t count, RankSelectLevel* dev_levels,
                        uint32_t* tmp, uint64_t tmp_words_per_level, cudaStream_t s, uint64_t* launches) {
  if (count == 0) return;
  uint64_t max_real = 0;
  for (uint32_t i = 0; i < count; ++i) {
    uint64_t nreal = (host_levels[i].nwords + kL1Cover - 1) / kL1Cover;
    if (nreal > max_real) max_real = nreal;
  }
  if (max_real == 0) return;
  const uint64_t ctas = (max_real + kRsThreads - 1) / kRsThreads;
  dim3 g1(unsigned(ctas), count);
  rs_blocks_kernel<<<g1, kRsThreads, 0, s>>>(dev_levels, tmp, tmp_words_per_level);
  rs_scan_kernel<<<count, 1024, 0, s>>>(dev_levels, tmp, tmp_words_per_level);
  rs_finish_kernel<<<g1, kRsThreads, 0, s>>>(dev_levels, tmp, tmp_words_per_level);
  *launches += 3;
}

void launch_queries(const QueryStructure& q, int op, const uint64_t* a, const uint64_t* b, uint64_t count,
                    uint64_t* out, cudaStream_t s, uint64_t* launches, const uint8_t* ops) {
  if (count == 0) return;
  uint64_t blocks = (count + 127) / 128;
  if (blocks > 65535) blocks = 65535;
  query_kernel<<<unsigned(blocks), 128, 0, s>>>(q, op, ops, a, b, count, out);
  ++*launches;
}


// ===========================================================================
// Allocation-free rank/select build (pwmgpu_rank_select_build_noalloc).
//
// For callers that must not allocate device memory while they run:
// allocator-less plugins that receive every buffer from their host framework,
// and latency-critical serving loops that cannot afford an allocator's
// implicit synchronisation.  The per-L1-block prefix counts the build needs
// live in a fixed, file-scope device array instead of context scratch, and
// the level descriptor the kernels read lives in a file-scope device slot.
// Both are resident on every GPU that loads this library until the process
// exits.  Every call shares them: calls that overlap on the GPU (different
// streams, or different host threads on one device) race and must be
// serialised by the caller.
// ===========================================================================
namespace {

// 4 MiB: prefix counts for up to kNoAllocMaxL1Blocks L1 blocks plus their
// per-CTA totals.
constexpr uint64_t kNoAllocScratchWords = uint64_t(1) << 20;
constexpr uint64_t kNoAllocMaxL1Blocks = (uint64_t(1) << 20) - (uint64_t(1) << 12);

static __device__ __align__(256) uint32_t g_noalloc_rs_scratch[kNoAllocScratchWords];
static __device__ __align__(256) RankSelectLevel g_noalloc_rs_level[1];

// Stores the level descriptor into its file-scope slot in stream order: the
// values travel as a kernel parameter, so no host buffer has to outlive the
// call.
__global__ void noalloc_set_level_kernel(RankSelectLevel level) { g_noalloc_rs_level[0] = level; }

struct NoAllocSymbols {
  bool ready = false;
  uint32_t* scratch = nullptr;
  RankSelectLevel* level = nullptr;
};

}  // namespace

// Device addresses of the file-scope arrays for the current device, looked
// up once per device (the first call on a device does it) and kept for the
// life of the process: after a cudaDeviceReset the module may load at other
// addresses, so the entry point must not be used across a device reset.
cudaError_t noalloc_rank_select_symbols(uint32_t** scratch, RankSelectLevel** level) {
  static std::mutex mu;
  static NoAllocSymbols per_device[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  NoAllocSymbols& s = per_device[dev];
  if (!s.ready) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_rs_scratch);
    if (e != cudaSuccess) return e;
    s.scratch = static_cast<uint32_t*>(p);
    e = cudaGetSymbolAddress(&p, g_noalloc_rs_level);
    if (e != cudaSuccess) return e;
    s.level = static_cast<RankSelectLevel*>(p);
    s.ready = true;
  }
  *scratch = s.scratch;
  *level = s.level;
  return cudaSuccess;
}

uint64_t noalloc_rank_select_max_words() { return kNoAllocMaxL1Blocks * kL1Cover; }

// Enqueues the build of one level's blocks on `stream` using only the
// file-scope arrays; outputs that must start at zero (l0, counts) are cleared
// here.  Returns cudaErrorInvalidValue for levels above the limit.
cudaError_t noalloc_rank_select_build(const uint64_t* words, uint64_t nwords, uint64_t* l0, uint32_t* l12,
                                      uint32_t* s0, uint32_t* s1, unsigned long long* counts, cudaStream_t stream) {
  if (nwords > noalloc_rank_select_max_words()) return cudaErrorInvalidValue;
  uint32_t* scratch = nullptr;
  RankSelectLevel* dev_level = nullptr;
  cudaError_t e = noalloc_rank_select_symbols(&scratch, &dev_level);
  if (e != cudaSuccess) return e;
  const uint64_t n0 = nwords / (4294967295ull / 64) + 1;
  e = cudaMemsetAsync(l0, 0, n0 * 8, stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(counts, 0, 3 * 8, stream);
  if (e != cudaSuccess) return e;
  if (nwords == 0) {
    // pwm keeps one zeroed l12 entry for an empty level; no kernel runs
    e = cudaMemsetAsync(l12, 0, 2 * sizeof(uint32_t), stream);
    return e;
  }
  RankSelectLevel host{words, nwords, l0, l12, s0, s1, counts};
  noalloc_set_level_kernel<<<1, 1, 0, stream>>>(host);
  const uint64_t nreal = (nwords + kL1Cover - 1) / kL1Cover;
  const uint64_t stride = nreal + (nreal + kRsThreads - 1) / kRsThreads + 1;
  uint64_t launches = 0;
  launch_rank_select(&host, 1, dev_level, scratch, stride, stream, &launches);
  return cudaGetLastError();
}

}  // namespace pwmgpu
