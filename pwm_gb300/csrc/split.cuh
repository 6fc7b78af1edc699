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
//   * the tile is then stably split K times in shared memory (LSD order, bit
//     l first); after split j the tile is sorted by key_j = bits l..l+j-1
//     (bit l least significant) and holds 2^j runs, and run v of level l+j
//     lands at  start_j[v] + (count of key_j == v in earlier tiles);
//   * the per-tile run counts are exchanged between tiles with a decoupled
//     look-back (one counter per run), so every tile learns its global run
//     offsets with a single read of its input.
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
  static constexpr int CHUNKS = T / 32;
  static_assert(T % 64 == 0, "tile must cover whole words");
  static constexpr size_t smem_bytes() {
    return size_t(2) * T * sizeof(KeyT) + size_t(K > 1 ? K - 1 : 1) * (CHUNKS + 1) * 4;
  }
};

__device__ __forceinline__ int run_offset(int j) { return (1 << j) - 2; }

// Stable split of in[0..n) by `bit` (zeros first) keeping only elements alive
// at `keep_level`; returns the number of elements written to out.
template <typename KeyT, typename Traits, int THREADS>
__device__ __forceinline__ uint32_t block_split(const KeyT* in, KeyT* out, uint32_t n, const Traits& tr,
                                                uint32_t bit_level, uint32_t keep_level, uint32_t* wz, uint32_t* wo) {
  constexpr int WARPS = THREADS / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t per = ((n + WARPS - 1) / WARPS + 31) & ~31u;
  const uint32_t b0 = min(n, per * warp), b1 = min(n, b0 + per);
  uint32_t z = 0, o = 0;
  for (uint32_t base = b0; base < b1; base += 32) {
    uint32_t e = base + lane;
    bool in_range = e < b1;
    KeyT k = in_range ? in[e] : KeyT(0);
    bool keep = in_range && tr.alive(k, keep_level);
    uint32_t b = tr.bit(k, bit_level);
    z += __popc(__ballot_sync(0xFFFFFFFFu, keep && !b));
    o += __popc(__ballot_sync(0xFFFFFFFFu, keep && b));
  }
  if (lane == 0) { wz[warp] = z; wo[warp] = o; }
  __syncthreads();
  if (warp == 0) {
    uint32_t vz = lane < WARPS ? wz[lane] : 0, vo = lane < WARPS ? wo[lane] : 0;
    uint32_t sz = vz, so = vo;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      uint32_t tz = __shfl_up_sync(0xFFFFFFFFu, sz, d), to = __shfl_up_sync(0xFFFFFFFFu, so, d);
      if (lane >= d) { sz += tz; so += to; }
    }
    uint32_t total_z = __shfl_sync(0xFFFFFFFFu, sz, 31), total_o = __shfl_sync(0xFFFFFFFFu, so, 31);
    if (lane < WARPS) { wz[lane] = sz - vz; wo[lane] = total_z + so - vo; }
    if (lane == 0) { wz[WARPS] = total_z + total_o; }
  }
  __syncthreads();
  uint32_t zb = wz[warp], ob = wo[warp];
  for (uint32_t base = b0; base < b1; base += 32) {
    uint32_t e = base + lane;
    bool in_range = e < b1;
    KeyT k = in_range ? in[e] : KeyT(0);
    bool keep = in_range && tr.alive(k, keep_level);
    uint32_t b = tr.bit(k, bit_level);
    uint32_t m0 = __ballot_sync(0xFFFFFFFFu, keep && !b);
    uint32_t m1 = __ballot_sync(0xFFFFFFFFu, keep && b);
    if (keep) out[b ? ob + __popc(m1 & lt) : zb + __popc(m0 & lt)] = k;
    zb += __popc(m0);
    ob += __popc(m1);
  }
  uint32_t total = wz[WARPS];
  __syncthreads();
  return total;
}

// Pack bit `level` of keys[0..n) into sbits (position i at bit 31-(i%32) of
// word i/32); words up to ceil(n/32) are written, the next one is zeroed.
template <typename KeyT, typename Traits, int THREADS>
__device__ __forceinline__ void pack_bits(const KeyT* keys, uint32_t n, const Traits& tr, uint32_t level,
                                          uint32_t* sbits) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nchunks = (n + 31) / 32;
  for (uint32_t c = warp; c <= nchunks; c += THREADS / 32) {
    uint32_t e = c * 32 + lane;
    bool v = e < n && tr.bit(keys[e], level);
    uint32_t mask = __ballot_sync(0xFFFFFFFFu, v);
    if (lane == 0) sbits[c] = __brev(mask);
  }
}

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

template <typename KeyT, typename Traits, int K, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS) split_pass_kernel(SplitArgs a, Traits tr) {
  using P = SplitPass<KeyT, Traits, K, THREADS, ITEMS>;
  constexpr int T = P::T, C = P::C, NLB = P::NLB, WARPS = P::WARPS, CHUNKS = P::CHUNKS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  KeyT* buf0 = reinterpret_cast<KeyT*>(smem_raw);
  KeyT* buf1 = buf0 + T;
  uint32_t* sbits = reinterpret_cast<uint32_t*>(buf1 + T);

  __shared__ uint32_t s_tile;
  __shared__ uint32_t cnt[C];          // run sizes of this tile, all levels j=1..K
  __shared__ uint32_t lstart[C];       // run starts inside the tile
  __shared__ unsigned long long gpos[C];  // global start of every run
  __shared__ unsigned long long pre[NLB];
  __shared__ uint32_t wz[WARPS + 1], wo[WARPS + 1];
  __shared__ uint32_t nstage[K + 1];
  __shared__ uint32_t chunk_prefix[C + 1];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int Kp = int(a.levels_here);   // levels present in this pass (1..K)
  const bool has_out = a.out != nullptr;
  const int splits = has_out ? Kp : Kp - 1;

  if (tid == 0) s_tile = atomicAdd(a.tile_counter, 1u);
  for (int c = tid; c < C; c += THREADS) cnt[c] = 0;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint64_t tile_start = uint64_t(tile) * T;
  const uint64_t remain = a.m - tile_start;
  const uint32_t n = remain < uint64_t(T) ? uint32_t(remain) : uint32_t(T);
  const KeyT* in = static_cast<const KeyT*>(a.in) + tile_start;

  // ---- load the tile (16-byte vectors where the tile is full) ----------
  if (n == T && (reinterpret_cast<uintptr_t>(in) & 15) == 0) {
    const uint4* src = reinterpret_cast<const uint4*>(in);
    uint4* dst = reinterpret_cast<uint4*>(buf0);
    constexpr int V = T * sizeof(KeyT) / 16;
#pragma unroll 4
    for (int i = tid; i < V; i += THREADS) dst[i] = __ldcs(src + i);
  } else {
    for (uint32_t i = tid; i < n; i += THREADS) buf0[i] = in[i];
  }
  __syncthreads();

  // ---- run counts of every level of the pass (warp ballots) ------------
  {
    uint32_t acc[C];
#pragma unroll
    for (int c = 0; c < C; ++c) acc[c] = 0;
    const uint32_t per = ((n + WARPS - 1) / WARPS + 31) & ~31u;
    const uint32_t b0 = min(n, per * warp), b1 = min(n, b0 + per);
    for (uint32_t base = b0; base < b1; base += 32) {
      uint32_t e = base + lane;
      bool ok = e < b1;
      KeyT k = ok ? buf0[e] : KeyT(0);
      uint32_t key = 0;
#pragma unroll
      for (int j = 1; j <= K; ++j) {
        key |= tr.bit(k, a.level + j - 1) << (j - 1);
        if (Traits::kDrops || j == K) {
          bool al = ok && j <= Kp && tr.alive(k, a.level + j);
#pragma unroll
          for (int v = 0; v < (1 << j); ++v)
            acc[run_offset(j) + v] += __popc(__ballot_sync(0xFFFFFFFFu, al && key == uint32_t(v)));
        }
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int c = 0; c < C; ++c)
        if (acc[c]) atomicAdd(&cnt[c], acc[c]);
    }
  }
  __syncthreads();
  if (!Traits::kDrops) {
    // derive the run counts of levels j < K from the finest runs
    for (int c = tid; c < C - (1 << K); c += THREADS) {
      int j = 1;
      while (c >= run_offset(j + 1)) ++j;
      int v = c - run_offset(j);
      uint32_t s = 0;
      for (int h = 0; h < (1 << (K - j)); ++h) s += cnt[run_offset(K) + v + (h << j)];
      cnt[c] = s;
    }
    __syncthreads();
  }

  // ---- publish the tile's counts and look back over predecessors ---------
  if (tid < NLB) {
    const int c = Traits::kDrops ? tid : run_offset(K) + tid;
    const uint64_t mine = cnt[c];
    unsigned long long* row = a.lookback + uint64_t(tile) * NLB;
    if (tile == 0) {
      st_volatile(row + tid, kFlagPrefix | mine);
      pre[tid] = 0;
    } else {
      st_volatile(row + tid, kFlagAggregate | mine);
      uint64_t excl = 0;
      for (int64_t t = int64_t(tile) - 1; t >= 0; --t) {
        uint64_t s = lookback_wait(a.lookback + uint64_t(t) * NLB + tid, a.status);
        excl += s & kCountMask;
        if ((s >> 62) == 2) break;
      }
      st_volatile(row + tid, kFlagPrefix | (excl + mine));
      pre[tid] = excl;
    }
  }

  // ---- level l bits in tile order (independent of the look-back) ---------
  {
    uint32_t* dst = reinterpret_cast<uint32_t*>(a.bv[0]);
    uint32_t* dst_tree = reinterpret_cast<uint32_t*>(a.tree_level0);
    const uint64_t q0 = tile_start >> 5;
    const uint32_t nch = ((n + 63) / 64) * 2;  // whole words (zero padded)
    for (uint32_t c = warp; c < nch; c += WARPS) {
      uint32_t e = c * 32 + lane;
      bool v = e < n && tr.bit(buf0[e], a.level);
      uint32_t mask = __brev(__ballot_sync(0xFFFFFFFFu, v));
      if (lane == 0) {
        dst[chunk_u32_index(q0 + c)] = mask;
        if (dst_tree) dst_tree[chunk_u32_index(q0 + c)] = mask;
      }
    }
  }

  // ---- local splits; pack the bits of the inner levels -------------------
  KeyT* cur = buf0;
  KeyT* nxt = buf1;
  if (tid == 0) nstage[0] = n;
  uint32_t ncur = n;
  for (int j = 1; j <= splits; ++j) {
    ncur = block_split<KeyT, Traits, THREADS>(cur, nxt, ncur, tr, a.level + j - 1, a.level + j, wz, wo);
    KeyT* t = cur; cur = nxt; nxt = t;
    if (j < Kp) pack_bits<KeyT, Traits, THREADS>(cur, ncur, tr, a.level + j, sbits + (j - 1) * (CHUNKS + 1));
    if (tid == 0) nstage[j] = ncur;
  }

  // ---- run starts inside the tile and global run positions ---------------
  __syncthreads();  // pre[] complete, splits done
  if (tid < C) {
    int j = 1;
    while (tid >= run_offset(j + 1)) ++j;
    int v = tid - run_offset(j);
    uint32_t s = 0;
    for (int u = 0; u < v; ++u) s += cnt[run_offset(j) + u];
    lstart[tid] = s;
    uint64_t p;
    if (Traits::kDrops) {
      p = pre[tid];
    } else {
      p = 0;
      for (int h = 0; h < (1 << (K - j)); ++h) p += pre[v + (h << j)];
    }
    gpos[tid] = (j <= Kp) ? a.starts[tid] + p : 0;
  }
  __syncthreads();

  // ---- inner-level bit runs: plain stores for whole chunks, OR at edges ---
  if (Kp > 1) {
    if (tid == 0) {
      uint32_t q = 0;
      for (int c = 0; c < C; ++c) {
        chunk_prefix[c] = q;
        int j = 1;
        while (c >= run_offset(j + 1)) ++j;
        uint32_t len = cnt[c];
        if (j < Kp && len > 0) {
          uint64_t g = gpos[c];
          q += uint32_t(((g + len - 1) >> 5) - (g >> 5) + 1);
        }
      }
      chunk_prefix[C] = q;
    }
    __syncthreads();
    const uint32_t total_chunks = chunk_prefix[C];
    for (uint32_t qi = tid; qi < total_chunks; qi += THREADS) {
      int c = 0;
      while (chunk_prefix[c + 1] <= qi) ++c;
      int j = 1;
      while (c >= run_offset(j + 1)) ++j;
      const uint64_t g = gpos[c];
      const uint32_t len = cnt[c];
      if (g + len > a.level_size[j]) {  // inconsistent run tables: never write out of range
        atomicOr(a.status, kErrBounds);
        continue;
      }
      const uint64_t q = (g >> 5) + (qi - chunk_prefix[c]);
      const int64_t d = int64_t(q << 5) - int64_t(g);         // chunk start relative to run start
      const uint32_t* sb = sbits + (j - 1) * (CHUNKS + 1);
      uint32_t val = extract32(sb, int64_t(lstart[c]) + d);
      if (d < 0) val = extract32(sb, int64_t(lstart[c])) >> uint32_t(-d);
      const uint32_t lo = d < 0 ? uint32_t(-d) : 0u;
      const int64_t hi64 = int64_t(len) - d;
      const uint32_t hi = hi64 >= 32 ? 32u : uint32_t(hi64);
      const uint32_t mask = chunk_mask(lo, hi);
      uint32_t* dst = reinterpret_cast<uint32_t*>(a.bv[j]) + chunk_u32_index(q);
      if (mask == 0xFFFFFFFFu) *dst = val;
      else atomicOr(dst, val & mask);
    }
  }

  // ---- S_{l+K}: runs of the final split to their global positions --------
  if (has_out) {
    KeyT* out = static_cast<KeyT*>(a.out);
    const uint32_t nout = nstage[Kp];
    constexpr int R = 1 << K;
    for (uint32_t e = tid; e < nout; e += THREADS) {
      int v = 0;
      while (v + 1 < R && lstart[run_offset(K) + v + 1] <= e) ++v;
      const uint64_t dst = gpos[run_offset(K) + v] + (e - lstart[run_offset(K) + v]);
      if (dst < a.level_size[K]) out[dst] = cur[e];
      else atomicOr(a.status, kErrBounds);
    }
  }
}

}  // namespace pwmgpu
