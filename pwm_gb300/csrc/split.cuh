// Fused multi-level split pass of the wavelet matrix construction.
//
// The level-l sequence S_l of a wavelet matrix is the text stably sorted by
// its reversed l-bit prefix: S_{l+1} is the stable 0/1 partition of S_l by
// bit l (pwm's naive definition, include/wx_naive.hpp:81-153; the prefix
// sorting of include/construction/ps.hpp:13-66 with the bit-reversal rho of
// include/util/permutation.hpp:16-51 produces the same sequences).  One pass
// of this kernel reads a tile of S_l from HBM once and produces the bit
// vectors of K consecutive levels l..l+K-1 plus S_{l+K}:
//
//   * level l's bits are in tile order: each warp ballots 32 positions and
//     stores the bit-reversed mask as one coalesced 32-bit chunk;
//   * level l+j (0 < j < K) of S_{l+j} is S_l stably sorted by key_j = bits
//     l..l+j-1 (bit l least significant): the tile contributes one run per
//     value v of key_j, run v holding bit l+j of the tile's elements with
//     key_j == v in tile order, and it lands at
//         start_j[v] + (count of key_j == v in earlier tiles).
//     The runs are built without moving keys: per round of 32 elements a warp
//     ballots the members of every run and compacts their bits with one
//     redux.sync.or (each member shifts its bit to its rank in the run);
//   * only the final order (key_K, the sequence S_{l+K} for the next pass) is
//     materialised: each key is stored once into its run in shared memory and
//     the runs are copied out coalesced;
//   * the per-tile run counts are exchanged between tiles with a decoupled
//     look-back (one counter per finest run), walked 32 predecessors at a time
//     by one warp per counter, so every tile learns its global run offsets
//     with a single read of its input.
//
// Huffman-shaped matrices use the same pass over packed code keys: an
// element is alive at level m while its code is longer than m, and the runs
// of level l+j count only elements alive there (include/huffman/
// huff_naive.hpp:19-126: finished codes leave the next level).
#pragma once

#include "common.cuh"

namespace pwmgpu {

// Plain symbols: level m tests bit L-1-m of the symbol.
template <typename KeyT>
struct PlainKeys {
  uint32_t L;
  __device__ __forceinline__ uint32_t bit(KeyT k, uint32_t level) const {
    return uint32_t(uint64_t(k) >> (L - 1 - level)) & 1u;
  }
  __device__ __forceinline__ bool alive(KeyT, uint32_t) const { return true; }
  static constexpr bool kDrops = false;
};

// Huffman keys: code left-aligned in the top (bits-8) bits, code length in
// the low 8 bits.  Level m tests code bit m; the element is alive at level m
// while length > m.
template <typename KeyT>
struct HuffKeys {
  uint32_t L;  // unused; keeps the layout of PlainKeys
  static constexpr uint32_t kTop = sizeof(KeyT) * 8 - 1;
  __device__ __forceinline__ uint32_t bit(KeyT k, uint32_t level) const {
    return uint32_t(uint64_t(k) >> (kTop - level)) & 1u;
  }
  __device__ __forceinline__ bool alive(KeyT k, uint32_t level) const { return uint32_t(k & 0xFFu) > level; }
  static constexpr bool kDrops = true;
};

constexpr int kMaxPassLevels = 4;

struct SplitArgs {
  const void* in;            // S_l (m keys)
  void* out;                 // S_{l+K} or nullptr for the last pass
  uint64_t m;                // |S_l|
  uint32_t level;            // l
  uint32_t levels_here;      // K' <= K actually present (last pass may be shorter)
  uint64_t* bv[kMaxPassLevels];  // matrix level arrays for l .. l+K'-1
  uint64_t* tree_level0;     // optional second destination of level 0 (tree)
  const uint64_t* starts;    // sum_{j=1..K} 2^j entries, j-major (offset 2^j-2)
  unsigned long long* lookback;  // [tiles][NLB] state words, zeroed
  uint32_t* tile_counter;    // zeroed
  uint64_t level_size[kMaxPassLevels + 1];  // elements of levels l..l+K (K: S_out)
  uint32_t* status;
  uint32_t tiles;
};

template <typename KeyT, typename Traits, int K, int THREADS, int ITEMS>
struct SplitPass {
  static constexpr int T = THREADS * ITEMS;          // tile size (elements)
  static constexpr int WARPS = THREADS / 32;
  static constexpr int C = (2 << K) - 2;             // runs of all levels j = 1..K
  static constexpr int NLB = Traits::kDrops ? C : (1 << K);  // look-back counters
  static constexpr int SWORDS = T / 32 + 2;          // words of one inner-level bit stream
  static_assert(T % 64 == 0 && (T / WARPS) % 32 == 0, "tile must cover whole words and warp rounds");
  static constexpr size_t smem_bytes() {
    return size_t(2) * T * sizeof(KeyT) + size_t(K > 1 ? K - 1 : 1) * SWORDS * 4;
  }
};

__device__ __forceinline__ constexpr int run_offset(int j) { return (1 << j) - 2; }

// 32 stream bits starting at (possibly negative) bit offset `src` of sbits.
__device__ __forceinline__ uint32_t extract32(const uint32_t* sbits, int64_t src) {
  if (src < 0) {
    uint32_t w0 = sbits[0];
    return (src <= -32) ? 0u : (w0 >> uint32_t(-src));
  }
  uint64_t s = uint64_t(src);
  uint32_t w0 = sbits[s >> 5], w1 = sbits[(s >> 5) + 1];
  return __funnelshift_l(w1, w0, uint32_t(s & 31));
}

// Exclusive prefix over predecessor tiles of look-back counter `c`, walked by
// one warp 32 tiles at a time; publishes this tile's inclusive value.
__device__ __forceinline__ uint64_t warp_lookback(unsigned long long* lb, int nlb, uint32_t tile, int c, uint64_t mine,
                                                  uint32_t* status) {
  const int lane = threadIdx.x & 31;
  unsigned long long* row = lb + uint64_t(tile) * nlb + c;
  if (tile == 0) {
    if (lane == 0) st_volatile(row, kFlagPrefix | mine);
    return 0;
  }
  uint64_t excl = 0;
  int64_t base = int64_t(tile) - 1;
  while (true) {
    const int64_t t = base - lane;
    uint64_t s = kFlagPrefix;  // before tile 0: an empty inclusive prefix
    if (t >= 0) s = lookback_wait(lb + uint64_t(t) * nlb + c, status);
    const uint32_t pmask = __ballot_sync(0xFFFFFFFFu, (s >> 62) == 2);
    const int stop = pmask ? __ffs(pmask) - 1 : 31;
    uint64_t v = lane <= stop ? (s & kCountMask) : 0;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
    excl += v;
    if (pmask) break;
    base -= 32;
  }
  if (lane == 0) st_volatile(row, kFlagPrefix | (excl + mine));
  return excl;
}

template <typename KeyT, typename Traits, int K, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS) split_pass_kernel(SplitArgs a, Traits tr) {
  using P = SplitPass<KeyT, Traits, K, THREADS, ITEMS>;
  constexpr int T = P::T, C = P::C, NLB = P::NLB, WARPS = P::WARPS, SWORDS = P::SWORDS;
  constexpr int FIN = run_offset(K);            // first finest run
  constexpr int PER = T / WARPS;                // elements per warp
  extern __shared__ __align__(16) unsigned char smem_raw[];
  KeyT* keys = reinterpret_cast<KeyT*>(smem_raw);
  KeyT* sorted = keys + T;
  uint32_t* sbits = reinterpret_cast<uint32_t*>(sorted + T);

  __shared__ uint32_t s_tile;
  __shared__ uint32_t cntw[WARPS][C];          // run sizes per warp
  __shared__ uint32_t basew[WARPS][C];         // tile-local start of each warp's part of a run
  __shared__ uint32_t cnt[C];                  // run sizes of the tile
  __shared__ uint32_t lstart[C];               // tile-local run starts
  __shared__ unsigned long long gpos[C];       // global run starts
  __shared__ unsigned long long pre[NLB];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const bool has_out = a.out != nullptr;

  if (tid == 0) s_tile = atomicAdd(a.tile_counter, 1u);
  for (int i = tid; i < (K > 1 ? K - 1 : 0) * SWORDS; i += THREADS) sbits[i] = 0;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint64_t tile_start = uint64_t(tile) * T;
  const uint64_t remain = a.m - tile_start;
  const uint32_t n = remain < uint64_t(T) ? uint32_t(remain) : uint32_t(T);
  const KeyT* in = static_cast<const KeyT*>(a.in) + tile_start;

  // ---- load the tile (16-byte vectors where the tile is full) ----------
  if (n == T && (reinterpret_cast<uintptr_t>(in) & 15) == 0) {
    const uint4* src = reinterpret_cast<const uint4*>(in);
    uint4* dst = reinterpret_cast<uint4*>(keys);
    constexpr int V = T * sizeof(KeyT) / 16;
#pragma unroll 4
    for (int i = tid; i < V; i += THREADS) dst[i] = __ldcs(src + i);
  } else {
    for (uint32_t i = tid; i < n; i += THREADS) keys[i] = in[i];
  }
  __syncthreads();

  const uint32_t w0 = uint32_t(warp) * PER;
  const uint32_t w1 = min(n, w0 + PER);

  // ---- per-warp run counts (ballots per run value) ----------------------
  {
    uint32_t acc[C];
#pragma unroll
    for (int c = 0; c < C; ++c) acc[c] = 0;
    for (uint32_t base = w0; base < w1; base += 32) {
      const uint32_t e = base + lane;
      const bool ok = e < w1;
      const KeyT k = ok ? keys[e] : KeyT(0);
      uint32_t key = 0;
#pragma unroll
      for (int j = 1; j <= K; ++j) {
        key |= tr.bit(k, a.level + j - 1) << (j - 1);
        if (Traits::kDrops || j == K) {
          const bool al = ok && tr.alive(k, a.level + j);
#pragma unroll
          for (int v = 0; v < (1 << j); ++v)
            acc[run_offset(j) + v] += __popc(__ballot_sync(0xFFFFFFFFu, al && key == uint32_t(v)));
        }
      }
    }
    if (!Traits::kDrops) {
      // runs of levels j < K are unions of finest runs (key_j = low j bits)
#pragma unroll
      for (int j = 1; j < K; ++j)
#pragma unroll
        for (int v = 0; v < (1 << j); ++v) {
          uint32_t s = 0;
#pragma unroll
          for (int h = 0; h < (1 << (K - j)); ++h) s += acc[FIN + v + (h << j)];
          acc[run_offset(j) + v] = s;
        }
    }
    if (lane == 0) {
#pragma unroll
      for (int c = 0; c < C; ++c) cntw[warp][c] = acc[c];
    }
  }
  __syncthreads();

  // ---- tile totals, local run starts, per-warp bases ---------------------
  if (tid < C) {
    uint32_t t = 0;
    for (int w = 0; w < WARPS; ++w) t += cntw[w][tid];
    cnt[tid] = t;
  }
  __syncthreads();
  if (tid < C) {
    int j = 1;
    while (tid >= run_offset(j + 1)) ++j;
    const int v = tid - run_offset(j);
    uint32_t s = 0;
    for (int u = 0; u < v; ++u) s += cnt[run_offset(j) + u];
    lstart[tid] = s;
    for (int w = 0; w < WARPS; ++w) {
      basew[w][tid] = s;
      s += cntw[w][tid];
    }
  }
  // publish this tile's aggregates; successors' walks need them
  if (tid < NLB && tile != 0) {
    const int c = Traits::kDrops ? tid : FIN + tid;
    uint32_t t = 0;
    for (int w = 0; w < WARPS; ++w) t += cntw[w][c];
    st_volatile(a.lookback + uint64_t(tile) * NLB + tid, kFlagAggregate | t);
  }
  __syncthreads();

  // ---- look-back right after the counts, so that inclusive prefixes travel
  // ---- quickly down the tile chain; the other warps start their chunk -----
  for (int c = warp; c < NLB; c += WARPS) {
    const int cc = Traits::kDrops ? c : FIN + c;
    const uint64_t p = warp_lookback(a.lookback, NLB, tile, c, cnt[cc], a.status);
    if (lane == 0) pre[c] = p;
  }

  // ---- one pass over the tile: level l bits, inner runs, final order ------
  {
    uint32_t run_off[C];
#pragma unroll
    for (int c = 0; c < C; ++c) run_off[c] = basew[warp][c];
    uint32_t* dst0 = reinterpret_cast<uint32_t*>(a.bv[0]);
    uint32_t* dst_tree = reinterpret_cast<uint32_t*>(a.tree_level0);
    const uint64_t q0 = tile_start >> 5;
    const uint32_t wend = ((min(n, w0 + PER) + 63) & ~63u);  // whole words of level l (zero padded)
    for (uint32_t base = w0; base < wend && base < w0 + PER; base += 32) {
      const uint32_t e = base + lane;
      const bool ok = e < w1;
      const KeyT k = ok ? keys[e] : KeyT(0);
      // level l: tile order
      const uint32_t m0 = __brev(__ballot_sync(0xFFFFFFFFu, ok && tr.bit(k, a.level)));
      if (lane == 0) {
        dst0[chunk_u32_index(q0 + (base >> 5))] = m0;
        if (dst_tree) dst_tree[chunk_u32_index(q0 + (base >> 5))] = m0;
      }
      if (base >= w1) continue;
      uint32_t key = 0;
#pragma unroll
      for (int j = 1; j <= K; ++j) {
        key |= tr.bit(k, a.level + j - 1) << (j - 1);
        const bool al = ok && tr.alive(k, a.level + j);
        if (j < K) {
          const uint32_t b = tr.bit(k, a.level + j);
          uint32_t* sb = sbits + (j - 1) * SWORDS;
#pragma unroll
          for (int v = 0; v < (1 << j); ++v) {
            const int c = run_offset(j) + v;
            const bool member = al && key == uint32_t(v);
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, member);
            if (m == 0) continue;
            const uint32_t r = __popc(m & lt);
            const uint32_t bits = __reduce_or_sync(0xFFFFFFFFu, (member && b) ? (0x80000000u >> r) : 0u);
            if (lane == 0) {
              const uint32_t pos = run_off[c], sh = pos & 31, cntm = __popc(m);
              atomicOr(&sb[pos >> 5], bits >> sh);
              if (sh + cntm > 32) atomicOr(&sb[(pos >> 5) + 1], bits << (32 - sh));
            }
            run_off[c] += __popc(m);
          }
        } else if (has_out) {
#pragma unroll
          for (int v = 0; v < (1 << K); ++v) {
            const int c = FIN + v;
            const bool member = al && key == uint32_t(v);
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, member);
            if (m == 0) continue;
            if (member) sorted[run_off[c] + __popc(m & lt)] = k;
            run_off[c] += __popc(m);
          }
        }
      }
    }
  }

  __syncthreads();  // pre[] (look-back) and the local runs are complete
  if (tid < C) {
    int j = 1;
    while (tid >= run_offset(j + 1)) ++j;
    const int v = tid - run_offset(j);
    uint64_t p;
    if (Traits::kDrops) {
      p = pre[tid];
    } else {
      p = 0;
      for (int h = 0; h < (1 << (K - j)); ++h) p += pre[v + (h << j)];
    }
    gpos[tid] = a.starts[tid] + p;
  }
  __syncthreads();

  // ---- inner-level runs to HBM: plain stores for whole chunks, OR at edges ---
#pragma unroll 1
  for (int c = 0; c < FIN; ++c) {
    const uint32_t len = cnt[c];
    if (len == 0) continue;
    int j = 1;
    while (c >= run_offset(j + 1)) ++j;
    const uint64_t g = gpos[c];
    if (g + len > a.level_size[j]) {  // inconsistent run tables: never write out of range
      if (tid == 0) atomicOr(a.status, kErrBounds);
      continue;
    }
    const uint32_t* sb = sbits + (j - 1) * SWORDS;
    const uint64_t qa = g >> 5, qb = (g + len - 1) >> 5;
    uint32_t* dst = reinterpret_cast<uint32_t*>(a.bv[j]);
    for (uint64_t q = qa + tid; q <= qb; q += THREADS) {
      const int64_t d = int64_t(q << 5) - int64_t(g);  // chunk start relative to the run start
      const uint32_t val = d < 0 ? (extract32(sb, int64_t(lstart[c])) >> uint32_t(-d))
                                 : extract32(sb, int64_t(lstart[c]) + d);
      const uint32_t lo = d < 0 ? uint32_t(-d) : 0u;
      const int64_t hi64 = int64_t(len) - d;
      const uint32_t hi = hi64 >= 32 ? 32u : uint32_t(hi64);
      const uint32_t mask = chunk_mask(lo, hi);
      if (mask == 0xFFFFFFFFu) dst[chunk_u32_index(q)] = val;
      else atomicOr(&dst[chunk_u32_index(q)], val & mask);
    }
  }

  // ---- S_{l+K}: runs of the final order to their global positions ---------
  if (has_out) {
    KeyT* out = static_cast<KeyT*>(a.out);
#pragma unroll 1
    for (int v = 0; v < (1 << K); ++v) {
      const uint32_t len = cnt[FIN + v];
      if (len == 0) continue;
      const uint64_t g = gpos[FIN + v];
      if (g + len > a.level_size[K]) {
        if (tid == 0) atomicOr(a.status, kErrBounds);
        continue;
      }
      const KeyT* src = sorted + lstart[FIN + v];
      for (uint32_t i = tid; i < len; i += THREADS) out[g + i] = src[i];
    }
  }
}

}  // namespace pwmgpu
