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
//   * the tile is stably split by bit l, l+1, ... in shared memory (LSD
//     order): after split j it is sorted by key_j = bits l..l+j-1 (bit l least
//     significant) and holds one run per value v of key_j; run v of level
//     l+j lands at  start_j[v] + (count of key_j == v in earlier tiles);
//   * every split reads 16 bytes of keys per lane (one 128-bit shared load),
//     extracts the split bit of all of them at once, ranks them with one
//     packed warp scan of (zeros, ones) counts and stores each key once; the
//     same read yields the bits of the level being split, in that level's
//     order, so no separate bit-packing pass exists;
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
    if constexpr (sizeof(KeyT) <= 4) return (uint32_t(k) >> (L - 1 - level)) & 1u;
    else return uint32_t(uint64_t(k) >> (L - 1 - level)) & 1u;
  }
  __device__ __forceinline__ bool alive(KeyT, uint32_t) const { return true; }
  static constexpr bool kDrops = false;
};

// Huffman keys with a stop bit: ((code << 1) | 1) << (L - length), L the
// longest code.  Level m tests bit L - m; the element is alive at level m
// while a bit below that one is set (the stop bit lies below every code
// bit of the element and nothing lies below the stop bit).  A pass needs
// only the bits of its levels and below, so it writes S_{l+K} in the
// narrowest keys that hold the L - (l + K) + 1 low bits, and the bit a
// level tests keeps its position.
template <typename KeyT>
struct HuffKeys {
  uint32_t L;
  __device__ __forceinline__ uint32_t bit(KeyT k, uint32_t level) const {
    return uint32_t(uint64_t(k) >> (L - level)) & 1u;
  }
  __device__ __forceinline__ bool alive(KeyT k, uint32_t level) const {
    return (uint64_t(k) & ((uint64_t(1) << (L - level)) - 1u)) != 0;
  }
  static constexpr bool kDrops = true;
};

constexpr int kMaxPassLevels = 4;

struct SplitArgs {
  const void* in;            // S_l (m keys)
  void* out;                 // S_{l+K} or nullptr for the last pass
  uint64_t m;                // |S_l|
  uint32_t level;            // l
  uint32_t levels_here;      // K (levels of this pass)
  uint64_t* bv[kMaxPassLevels];  // matrix level arrays for l .. l+K-1
  uint64_t* tree_level0;     // optional second destination of level 0 (tree)
  const uint64_t* starts;    // sum_{j=1..K} 2^j entries, j-major (offset 2^j-2)
  unsigned long long* lookback;  // [tiles][NLB] state words, zeroed
  uint32_t* tile_counter;    // zeroed
  uint64_t level_size[kMaxPassLevels + 1];  // elements of levels l..l+K (K: S_out)
  uint32_t* status;
  uint32_t tiles;
  uint32_t L;                // levels of the text (plain keys)
};

template <typename KeyT, typename Traits, int K, int THREADS, int ITEMS>
struct SplitPass {
  static constexpr int T = THREADS * ITEMS;           // tile size (elements)
  static constexpr int WARPS = THREADS / 32;
  static constexpr int PERW = T / WARPS;              // elements of one warp's slice
  static constexpr int KPL = 16 / int(sizeof(KeyT));  // keys per lane per round (one 16-byte load)
  static constexpr int ROUND = 32 * KPL;              // keys per warp round
  static constexpr int C = (2 << K) - 2;              // runs of all levels j = 1..K
  static constexpr int NLB = Traits::kDrops ? C : (1 << K);  // look-back counters per tile row
  static constexpr int SW = PERW / 32 + 2;            // words of one warp's inner-level bit stream
  static constexpr int RUNS = 1 << (K > 1 ? K - 1 : 0);  // runs a split can refine
  static constexpr int MASKW = PERW / KPL;            // mask words of one warp (one per lane-round)
  static_assert(PERW % ROUND == 0, "a warp slice is whole rounds");
  static_assert(KPL <= 16, "split and alive masks share one word");
  static constexpr size_t smem_bytes() {
    return size_t(2) * T * sizeof(KeyT) + size_t(K > 1 ? K - 1 : 1) * WARPS * SW * 4 + size_t(WARPS) * MASKW * 4;
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
// one warp 32 tiles at a time; publishes this tile's aggregate first and its
// inclusive value at the end.
__device__ __forceinline__ uint64_t warp_lookback(unsigned long long* lb, int nlb, uint32_t tile, int c, uint64_t mine,
                                                  uint32_t* status) {
  const int lane = threadIdx.x & 31;
  unsigned long long* row = lb + uint64_t(tile) * nlb + c;
  if (tile == 0) {
    if (lane == 0) st_volatile(row, kFlagPrefix | mine);
    return 0;
  }
  if (lane == 0) st_volatile(row, kFlagAggregate | mine);
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

// The KPL keys of a lane, kept as the four 32-bit words of one 16-byte load.
template <typename KeyT, typename Traits, int KPL>
struct LaneKeys {
  uint32_t w[4];
  __device__ __forceinline__ void load(const KeyT* p) {
    const uint4 v = *reinterpret_cast<const uint4*>(p);
    w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
  }
  __device__ __forceinline__ KeyT key(int i) const {
    if constexpr (sizeof(KeyT) == 1) return KeyT((w[i >> 2] >> (8 * (i & 3))) & 0xFFu);
    else if constexpr (sizeof(KeyT) == 2) return KeyT((w[i >> 1] >> (16 * (i & 1))) & 0xFFFFu);
    else if constexpr (sizeof(KeyT) == 4) return KeyT(w[i]);
    else return KeyT(uint64_t(w[2 * i]) | (uint64_t(w[2 * i + 1]) << 32));
  }
  // bit k of the result: split bit of key k
  __device__ __forceinline__ uint32_t bits(const Traits& tr, uint32_t level) const {
    if constexpr (sizeof(KeyT) == 1 && !Traits::kDrops) {
      // four keys per word; the chosen bit of each byte gathered by a multiply
      const uint32_t sh = tr.L - 1 - level;
      if (sh >= 8) return 0u;  // above the key width every bit is 0
      uint32_t m = 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) m |= ((((w[q] >> sh) & 0x01010101u) * 0x10204080u) >> 28) << (4 * q);
      return m;
    } else {
      uint32_t m = 0;
#pragma unroll
      for (int i = 0; i < KPL; ++i) m |= tr.bit(key(i), level) << i;
      return m;
    }
  }
  __device__ __forceinline__ uint32_t alive(const Traits& tr, uint32_t level) const {
    if constexpr (!Traits::kDrops) {
      return (1u << KPL) - 1u;
    } else {
      uint32_t m = 0;
#pragma unroll
      for (int i = 0; i < KPL; ++i) m |= uint32_t(tr.alive(key(i), level)) << i;
      return m;
    }
  }
  // key_j (bits level0 .. level0+j-1, the first least significant) of key i
  __device__ __forceinline__ uint32_t digit(const Traits& tr, int i, uint32_t level0, int j) const {
    uint32_t d = 0;
    const KeyT k = key(i);
    for (int b = 0; b < j; ++b) d |= tr.bit(k, level0 + uint32_t(b)) << b;
    return d;
  }
};

// The bits of one warp round in MSB-first stream order: lane i holds KPL bits
// (bit k = stream position i*KPL + k of the round).  The 32/KPL lanes of one
// 32-bit chunk are combined with shuffles; the first lane of each chunk gets
// the chunk (returns true and sets *value).
template <int KPL>
__device__ __forceinline__ bool round_chunk(uint32_t lane_bits, uint32_t* value) {
  const int lane = threadIdx.x & 31;
  constexpr int LPC = 32 / KPL;  // lanes per 32-bit chunk
  uint32_t v = (__brev(lane_bits) >> (32 - KPL)) << (32 - KPL * (lane % LPC + 1));
#pragma unroll
  for (int d = 1; d < LPC; d <<= 1) v |= __shfl_down_sync(0xFFFFFFFFu, v, d);
  *value = v;
  return lane % LPC == 0;
}

// Copy `len` bytes from shared memory to global memory by one warp: byte
// stores up to a 4-byte aligned destination, then 32-bit stores whose source
// bytes are funnel-shifted out of aligned shared words, then the tail.
__device__ __forceinline__ void copy_run_bytes(unsigned char* dst, const unsigned char* src, uint32_t len) {
  const int lane = threadIdx.x & 31;
  const uint32_t head = min(len, uint32_t((4 - (reinterpret_cast<uintptr_t>(dst) & 3)) & 3));
  if (uint32_t(lane) < head) dst[lane] = src[lane];
  const uint32_t body = (len - head) >> 2;
  const uint32_t so0 = uint32_t(reinterpret_cast<uintptr_t>(src + head) & 3);
  const uint32_t* s32 = reinterpret_cast<const uint32_t*>(src + head - so0);
  uint32_t* d32 = reinterpret_cast<uint32_t*>(dst + head);
  for (uint32_t k = lane; k < body; k += 32) {
    const uint32_t lo = s32[k], hi = so0 ? s32[k + 1] : 0u;
    d32[k] = __funnelshift_r(lo, hi, 8 * so0);
  }
  const uint32_t done = head + 4 * body;
  if (uint32_t(lane) < len - done) dst[done + lane] = src[done + lane];
}

template <typename KeyT, typename Traits, int K, int THREADS, int ITEMS, typename KeyO = KeyT>
__device__ __forceinline__ void split_pass_tile(const SplitArgs& a, const Traits& tr, uint32_t tile);

// One text: tiles are taken in launch order from a.tile_counter.  KeyO: the
// key type of S_{l+K} (KeyT, or narrower for Huffman keys, their low bits).
template <typename KeyT, typename Traits, int K, int THREADS, int ITEMS, typename KeyO = KeyT>
__global__ void __launch_bounds__(THREADS, K <= 2 ? 4 : 3) split_pass_kernel(SplitArgs a, Traits tr) {
  __shared__ uint32_t s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(a.tile_counter, 1u);
  __syncthreads();
  split_pass_tile<KeyT, Traits, K, THREADS, ITEMS, KeyO>(a, tr, s_tile);
}

// A batch of texts: global tile g belongs to the text whose range
// [tile_base[t], tile_base[t+1]) holds it; tiles are taken in launch order
// from one counter, so the predecessors of a tile inside its text were taken
// earlier (the look-back waits end).
template <typename KeyT, typename Traits, int K, int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS, K <= 2 ? 4 : 3)
    split_pass_batched_kernel(const SplitArgs* __restrict__ args, const uint32_t* __restrict__ tile_base,
                              uint32_t ntexts, uint32_t* tile_counter) {
  __shared__ uint32_t s_tile, s_text;
  __shared__ SplitArgs s_args;
  if (threadIdx.x == 0) {
    const uint32_t g = atomicAdd(tile_counter, 1u);
    uint32_t lo = 0, hi = ntexts;  // last text with tile_base <= g
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (tile_base[mid] <= g) lo = mid; else hi = mid;
    }
    s_text = lo;
    s_tile = g - tile_base[lo];
  }
  __syncthreads();
  if (threadIdx.x == 0) s_args = args[s_text];
  __syncthreads();
  const Traits tr{s_args.L};
  split_pass_tile<KeyT, Traits, K, THREADS, ITEMS>(s_args, tr, s_tile);
}

template <typename KeyT, typename Traits, int K, int THREADS, int ITEMS, typename KeyO>
__device__ __forceinline__ void split_pass_tile(const SplitArgs& a, const Traits& tr, const uint32_t tile) {
  using P = SplitPass<KeyT, Traits, K, THREADS, ITEMS>;
  constexpr int T = P::T, C = P::C, WARPS = P::WARPS, SW = P::SW, KPL = P::KPL, ROUND = P::ROUND;
  constexpr int RUNS = P::RUNS, PERW = P::PERW, MASKW = P::MASKW;
  constexpr uint32_t FULL = (1u << KPL) - 1u;
  using LK = LaneKeys<KeyT, Traits, KPL>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  KeyT* bufA = reinterpret_cast<KeyT*>(smem_raw);
  KeyT* bufB = bufA + T;
  uint32_t* sbits_all = reinterpret_cast<uint32_t*>(bufB + T);
  uint32_t* masks_all = sbits_all + (K > 1 ? K - 1 : 1) * WARPS * SW;

  __shared__ uint32_t runz[WARPS][K + 1][RUNS], runo[WARPS][K + 1][RUNS];  // per warp, per split
  __shared__ uint32_t cntw[WARPS][C];          // run sizes per warp
  __shared__ uint32_t cnt[C];                  // run sizes of the tile
  __shared__ unsigned long long gpos[C];       // global run starts of the tile
  __shared__ unsigned long long pre[P::NLB];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool has_out = a.out != nullptr;
  const int D = has_out ? K : K - 1;  // splits of this pass

  for (int i = tid; i < WARPS * (K + 1) * RUNS; i += THREADS) {
    (&runz[0][0][0])[i] = 0;
    (&runo[0][0][0])[i] = 0;
  }
  __syncthreads();
  const uint64_t tile_start = uint64_t(tile) * T;
  const uint64_t remain = a.m - tile_start;
  const uint32_t n = remain < uint64_t(T) ? uint32_t(remain) : uint32_t(T);

  // ---- this warp's slice [w0, w0 + nw) of the tile -----------------------
  const uint32_t w0 = uint32_t(warp) * PERW;
  const uint32_t nw = n > w0 ? min(n - w0, uint32_t(PERW)) : 0u;
  KeyT* cur = bufA + w0;
  KeyT* nxt = bufB + w0;
  uint32_t* sbits = sbits_all + warp * SW;      // stream m-1 at sbits + (m-1) * WARPS * SW
  uint32_t* masks = masks_all + warp * MASKW;
  {
    const KeyT* in = static_cast<const KeyT*>(a.in) + tile_start + w0;
    if (nw == PERW && (reinterpret_cast<uintptr_t>(in) & 15) == 0) {
      const uint4* src = reinterpret_cast<const uint4*>(in);
      uint4* dst = reinterpret_cast<uint4*>(cur);
      constexpr int V = PERW * sizeof(KeyT) / 16;
#pragma unroll 4
      for (int i = lane; i < V; i += 32) dst[i] = __ldcs(src + i);
    } else {
      for (uint32_t i = lane; i < nw; i += 32) cur[i] = in[i];
    }
    for (int m = 0; m < K - 1; ++m)
      for (int i = lane; i < SW; i += 32) sbits[m * WARPS * SW + i] = 0;
  }
  __syncwarp();

  const uint64_t level0_chunks = 2 * words_for(a.level_size[0]);
  uint32_t* g0 = reinterpret_cast<uint32_t*>(a.bv[0]);
  uint32_t* gt = reinterpret_cast<uint32_t*>(a.tree_level0);
  const uint64_t q0 = (tile_start + w0) >> 5;

  // ---- split j reads the order of key_{j-1}: it emits the bits of level
  // ---- l+j-1 and, for j <= D, partitions by that bit (warp-local) --------
  uint32_t nin = nw;
#pragma unroll 1
  for (int j = 1; j <= (has_out ? D : D + 1); ++j) {
    const bool scatter = j <= D;
    const int m = j - 1;  // level l+m is emitted
    const uint32_t bl = a.level + uint32_t(m), al = a.level + uint32_t(j);
    uint32_t z = 0, o = 0;
    for (uint32_t base = 0; base < nin; base += ROUND) {
      const uint32_t e0 = base + uint32_t(lane) * KPL;
      LK lk;
      lk.load(cur + e0);
      const uint32_t vmask = e0 >= nin ? 0u : (nin - e0 >= uint32_t(KPL) ? FULL : ((1u << (nin - e0)) - 1u));
      const uint32_t b = lk.bits(tr, bl) & vmask;
      {
        uint32_t v;
        if (round_chunk<KPL>(b, &v)) {
          const uint32_t chunk = e0 >> 5;
          if (m == 0) {
            const uint64_t q = q0 + chunk;
            if (q < level0_chunks) {
              g0[chunk_u32_index(q)] = v;
              if (gt) gt[chunk_u32_index(q)] = v;
            }
          } else {
            sbits[(m - 1) * WARPS * SW + chunk] = v;
          }
        }
      }
      if (!scatter) continue;
      const uint32_t am = lk.alive(tr, al) & vmask;
      masks[base / KPL + lane] = b | (am << 16);
      const uint32_t c0 = __popc(am & ~b), c1 = __popc(am & b);
      z += c0;
      o += c1;
      if (m > 0 && vmask) {
        // zeros / ones per run of key_m; the slice is sorted by key_m
        const int last = 31 - __clz(vmask);
        const uint32_t u0 = lk.digit(tr, 0, a.level, m), u1 = lk.digit(tr, last, a.level, m);
        if (u0 == u1) {
          if (c0) atomicAdd(&runz[warp][j][u0], c0);
          if (c1) atomicAdd(&runo[warp][j][u0], c1);
        } else {
#pragma unroll
          for (int i = 0; i < KPL; ++i) {
            if (!((am >> i) & 1u)) continue;
            const uint32_t u = lk.digit(tr, i, a.level, m);
            if ((b >> i) & 1u) atomicAdd(&runo[warp][j][u], 1u);
            else atomicAdd(&runz[warp][j][u], 1u);
          }
        }
      }
    }
    if (!scatter) break;
    z = __reduce_add_sync(0xFFFFFFFFu, z);
    o = __reduce_add_sync(0xFFFFFFFFu, o);
    if (j == 1 && lane == 0) { runz[warp][1][0] = z; runo[warp][1][0] = o; }
    __syncwarp();
    uint32_t pz = 0, po = z;
    for (uint32_t base = 0; base < nin; base += ROUND) {
      const uint32_t e0 = base + uint32_t(lane) * KPL;
      LK lk;
      lk.load(cur + e0);
      const uint32_t bm = masks[base / KPL + lane];
      const uint32_t b = bm & 0xFFFFu, am = bm >> 16;
      const uint32_t packed = __popc(am & ~b) | (__popc(am & b) << 16);
      uint32_t x = packed;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if (lane >= d) x += y;
      }
      const uint32_t total = __shfl_sync(0xFFFFFFFFu, x, 31);
      const uint32_t ex = x - packed;
      uint32_t dz = pz + (ex & 0xFFFFu), dn = po + (ex >> 16);
      if (!Traits::kDrops && am == FULL) {
#pragma unroll
        for (int i = 0; i < KPL; ++i) {
          const bool one = (b >> i) & 1u;
          nxt[one ? dn : dz] = lk.key(i);
          dn += one;
          dz += !one;
        }
      } else {
#pragma unroll
        for (int i = 0; i < KPL; ++i) {
          if ((am >> i) & 1u) {
            if ((b >> i) & 1u) nxt[dn++] = lk.key(i);
            else nxt[dz++] = lk.key(i);
          }
        }
      }
      pz += total & 0xFFFFu;
      po += total >> 16;
    }
    nin = z + o;
    __syncwarp();
    KeyT* t = cur; cur = nxt; nxt = t;
  }

  // ---- run sizes of this warp for levels j = 1..D --------------------------
  for (int c = lane; c < C; c += 32) {
    int j = 1;
    while (c >= run_offset(j + 1)) ++j;
    const int v = c - run_offset(j);
    uint32_t r = 0;
    if (j <= D) {
      const int half = 1 << (j - 1);
      r = v < half ? runz[warp][j][v] : runo[warp][j][v - half];
    }
    cntw[warp][c] = r;
  }
  __syncthreads();
  if (tid < C) {
    uint32_t t = 0;
    for (int w = 0; w < WARPS; ++w) t += cntw[w][tid];
    cnt[tid] = t;
  }
  __syncthreads();

  // ---- look-back over the finest runs of this pass --------------------------
  const int nlb = D == 0 ? 0 : (Traits::kDrops ? (2 << D) - 2 : (1 << D));
  const int fin = D == 0 ? 0 : run_offset(D);
  for (int c = warp; c < nlb; c += WARPS) {
    const int cc = Traits::kDrops ? c : fin + c;
    const uint64_t p = warp_lookback(a.lookback, P::NLB, tile, c, cnt[cc], a.status);
    if (lane == 0) pre[c] = p;
  }
  __syncthreads();
  if (tid < C) {
    int j = 1;
    while (tid >= run_offset(j + 1)) ++j;
    const int v = tid - run_offset(j);
    uint64_t p = 0;
    if (j <= D) {
      if (Traits::kDrops) {
        p = pre[tid];
      } else {
        for (int h = 0; h < (1 << (D - j)); ++h) p += pre[v + (h << j)];
      }
    }
    gpos[tid] = a.starts[tid] + p;
  }
  __syncthreads();

  // ---- this warp's parts of the runs to HBM --------------------------------
  // warp w's part of run c starts at gpos[c] + (earlier warps' parts) and at
  // (earlier runs of the same level in this warp) in the warp's own order
  uint32_t local = 0;  // start of the current run in this warp's order
  int cur_level = 0;
#pragma unroll 1
  for (int c = 0; c < C; ++c) {
    int j = 1;
    while (c >= run_offset(j + 1)) ++j;
    if (j != cur_level) { cur_level = j; local = 0; }
    const uint32_t len = cntw[warp][c];
    if (len == 0) continue;
    uint64_t g = gpos[c];
    for (int w = 0; w < warp; ++w) g += cntw[w][c];
    const uint32_t start = local;
    local += len;
    if (j < K) {
      // bits of inner level l+j
      if (g + len > a.level_size[j]) {  // inconsistent run tables: never write out of range
        if (lane == 0) atomicOr(a.status, kErrBounds);
        continue;
      }
      const uint32_t* sb = sbits + (j - 1) * WARPS * SW;
      const uint64_t qa = g >> 5, qb = (g + len - 1) >> 5;
      uint32_t* dst = reinterpret_cast<uint32_t*>(a.bv[j]);
      for (uint64_t q = qa + lane; q <= qb; q += 32) {
        const int64_t d = int64_t(q << 5) - int64_t(g);  // chunk start relative to the part start
        const uint32_t val = d < 0 ? (extract32(sb, int64_t(start)) >> uint32_t(-d)) : extract32(sb, int64_t(start) + d);
        const uint32_t lo = d < 0 ? uint32_t(-d) : 0u;
        const int64_t hi64 = int64_t(len) - d;
        const uint32_t hi = hi64 >= 32 ? 32u : uint32_t(hi64);
        const uint32_t mask = chunk_mask(lo, hi);
        if (mask == 0xFFFFFFFFu) dst[chunk_u32_index(q)] = val;
        else atomicOr(&dst[chunk_u32_index(q)], val & mask);
      }
    } else if (has_out) {
      // keys of S_{l+K}
      if (g + len > a.level_size[K]) {
        if (lane == 0) atomicOr(a.status, kErrBounds);
        continue;
      }
      if constexpr (sizeof(KeyO) == sizeof(KeyT)) {
        copy_run_bytes(reinterpret_cast<unsigned char*>(static_cast<KeyT*>(a.out) + g),
                       reinterpret_cast<const unsigned char*>(cur + start), len * uint32_t(sizeof(KeyT)));
      } else {
        KeyO* dst = static_cast<KeyO*>(a.out) + g;
        for (uint32_t i = uint32_t(lane); i < len; i += 32) dst[i] = KeyO(cur[start + i]);
      }
    }
  }
}

}  // namespace pwmgpu
