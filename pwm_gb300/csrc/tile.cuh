// Segmented multi-level split pass for plain keys: one CTA sorts one tile of
// a level sequence through K levels in shared memory and writes the bits of
// those K levels straight into BOTH the wavelet matrix and the wavelet tree.
//
// Background (pwm's naive definition, include/wx_naive.hpp:81-153, and the
// prefix sorting of include/construction/ps.hpp:13-66 with the bit-reversal
// rho of include/util/permutation.hpp:16-51): the level-m sequence S_m of a
// wavelet matrix is the text stably sorted by key_m, the first m symbol bits
// read with the first bit least significant; level m holds bit m of every
// element in S_m order.  The tree level m holds the same bits grouped by the
// natural m-bit prefix instead.  Inside one group (one prefix) both keep text
// order, so a group is one contiguous run in either structure and only the
// run starts differ.
//
// A pass covers levels l..l+K-1 of one "segment" of S_l: either all of S_l
// (the first pass, or any pass whose tree levels are left to a regroup), or
// one l-bit prefix group of S_l, whose elements share key_l and therefore
// land in every later level at group-specific run starts of both structures.
// Per tile the kernel
//   * loads the tile into shared memory (one TMA bulk copy when the tile is
//     16-byte aligned whole blocks, else 16-byte vectors, misaligned segments
//     realigned with funnel shifts);
//   * runs D = K (or K-1 in the last pass) CTA-wide stable 1-bit splits in
//     LSD order.  Each thread keeps V 16-byte vectors of keys in registers in
//     a striped layout (conflict-free 128-bit shared loads), extracts the
//     split bit of 16 bytes at once, ranks its keys with one packed warp scan
//     of zero counts per two vectors plus a CTA scan of 8 warp totals, and
//     stores every key once;
//   * emits the bits of each level from the same register copy, in that
//     level's order, into a shared bit stream;
//   * tracks the tile's run sizes of key_1..key_D from the split counts;
//   * counts the tile's finest runs (key_D digits) right after loading it and
//     publishes them at once; after its splits and the write of the level-l
//     run (which needs no prefix) the CTA completes the decoupled look-back
//     (restarted at every segment's first tile; counter-major state, one
//     coalesced load per counter, 256 predecessors per round trip);
//   * writes every run of every level to the matrix and the tree at
//     table start + look-back prefix in 64-bit words, and the runs of
//     S_{l+K} to the next pass's input (one warp per run, round-robin; the
//     level words word-parallel in passes of 5-8 levels and over 2- and
//     4-byte keys).
// A pass that writes no S_{l+K} over 1-byte keys (the last pass of every
// text whose remaining levels fit a byte) runs the splits on bit planes
// instead (tile_planes_splits): the K bits of every key as K planes of 32-key
// words, each split a stable partition of the later planes' words; the
// streams of the levels are then the planes themselves.
#pragma once

#include "common.cuh"
#include "tile_layout.hpp"

namespace pwmgpu {


struct TileSeg {
  uint64_t in_begin;  // first key of the segment in the pass input
  uint64_t m;         // keys of the segment
  uint64_t table;     // offset of the segment's start table
  uint32_t tile0;     // first global tile of the segment
  uint32_t text;      // index of the structure pair the segment belongs to
};

struct TileText {
  uint64_t* wm;     // matrix level l of the pass; level l+j at wm + j * stride
  uint64_t* wt;     // tree level l (nullptr: no tree levels from this pass)
  uint64_t stride;  // words between consecutive levels
  uint64_t nbits;   // bits of every level
  uint32_t shift;   // level l+j tests key bit (shift - j)
  // Batched passes (tile_pass_body with BATCH) only; zero otherwise:
  uint32_t vpt;         // 16-byte vectors per thread of this text's tiles (1, 2 or 4)
  uint32_t wait_idx;    // ~0u, or a counter in TileArgs::done this pass waits for ...
  uint32_t signal_idx;  // ~0u, or a counter each of its tiles adds one to when done
  uint32_t blk0;        // with TileArgs::text_blocks: the text's first block of given prefixes
};

struct TileArgs {
  const void* in;
  void* out;          // S_{l+K}; nullptr in the last pass
  uint64_t out_size;  // keys of `out` (bounds check)
  const TileSeg* segs;
  const TileText* texts;
  const uint64_t* tables;
  unsigned long long* lookback;  // [1 << D][tiles] (counter-major), zeroed
  uint32_t* tile_counter;        // zeroed
  uint32_t* status;
  uint32_t nsegs;
  uint32_t tiles;       // tiles of the whole pass (the look-back state's stride)
  uint32_t tile_base;   // this launch takes tiles [tile_base, tile_base + launch_tiles)
  uint32_t launch_tiles;
  // Optional (first pass of a text with one segment): the finest-run counts
  // of every tile and their exclusive prefixes, from the histogram kernel:
  // prefix = blockpre[tile / tiles_per_block] + relpre[tile].  The pass then
  // neither counts nor looks back.
  const unsigned long long* blockpre;
  const uint32_t* relpre;
  const uint32_t* tilecnt;
  uint32_t tiles_per_block;
  // 0: tile g's block is g / tiles_per_block; 1 (the first pass of a
  // batch's texts, blocks restarting at every text): TileText::blk0 + the
  // tile's index in its segment / tiles_per_block.
  uint32_t text_blocks;
  uint32_t first_level_written;  // level l is already written (by the histogram kernel)
  uint32_t clear_edges;          // the levels were not zeroed: shared words are cleared before they are set
  // Optional: words [0, zero_words) at zero_a (and zero_b) are zeroed, tile g
  // taking words [g * zero_per_tile, (g + 1) * zero_per_tile): the levels of
  // the next pass, whose edge words it ORs.  16-byte aligned, even counts.
  uint64_t* zero_a;
  uint64_t* zero_b;
  uint64_t zero_words;
  uint32_t zero_per_tile;
  uint32_t spin_limit;  // polls of one look-back wait before it gives up (kErrTimeout)
  // Batched passes: the per-(text, pass) tile counters (TileText::wait_idx /
  // signal_idx) and the tiles each counter must reach.
  unsigned int* done;
  const unsigned int* need;
};

template <typename KeyT, int K, bool OUT, int THREADS, int V>
struct TileCfg {
  static constexpr int D = OUT ? K : K - 1;             // splits
  static constexpr int KPL = 16 / int(sizeof(KeyT));    // keys per 16-byte vector
  static constexpr int ITEMS = V * KPL;                  // keys per thread
  static constexpr int T = THREADS * ITEMS;              // keys per tile
  static constexpr int WARPS = THREADS / 32;
  static constexpr int WSLICE = 32 * ITEMS;              // keys per warp
  static constexpr int NVEC = THREADS * V;               // vectors per tile
  static constexpr int SBW = T / 32 + 2;                 // stream words per level (+2 for funnel reads)
  static constexpr int NLB = 1 << D;                     // look-back counters per tile
  static constexpr int LPC = 32 / KPL;                   // lanes per 32-bit stream word
  static_assert(T <= 32768, "zero counts are packed in 16 bits");
  static_assert(K >= 1 && K <= kTileGivenMaxLevels && (K <= kTileMaxLevels || !OUT),
                "1..4 levels per pass; up to 8 in a last pass with given prefixes");
  static_assert(V % 2 == 0, "vectors are scanned in pairs");
  static constexpr size_t smem_bytes() {
    return deep_offset() + (K > kTileMaxLevels ? 0 : deep_bytes());
  }
  // key form, K <= 4: the run records after the streams, 16-byte aligned
  static constexpr size_t deep_offset() { return (size_t(T) * sizeof(KeyT) + stream_area() + 15) & ~size_t(15);
  }
  // One key buffer (a split reads all its keys into registers before its
  // first barrier, then scatters into the same buffer), then the K streams
  // and the per-vector zero prefixes; before the splits the same bytes hold
  // the finest-run counters (16 bits per thread and run).
  static constexpr size_t stream_area() {
    const size_t s = size_t(K) * SBW * 4 + (D >= 2 ? size_t(NVEC) * 4 : 0);
    const size_t c = size_t(1 << D) * THREADS * 2;
    return s > c ? s : c;
  }
  // Levels 1..K-1 written word-parallel (tile_pass_body): passes of 5..8
  // levels (levels 1..JW still a warp per run), and passes over 2- and
  // 4-byte keys, whose smaller tiles give runs too short for a warp each
  // (measured: 16-bit, 16 levels 4.48 -> 4.38 ms of passes; 32-bit, 20 levels
  // 1.64 -> 1.58; slower over 1-byte keys: 4.71 -> 4.80 ms at 8 levels).
  static constexpr bool WORD_PARALLEL = K > kTileMaxLevels || (K > 1 && sizeof(KeyT) > 1);
  static constexpr int JW = K > kTileMaxLevels ? 3 : 0;
  // run records and word prefixes of the word-parallel writes
  static constexpr size_t deep_bytes() {
    return WORD_PARALLEL ? size_t(2 * ((1 << K) - 2)) * 16 + size_t(2 * (K - 1 - JW)) * ((1 << (K - 1)) + 1) * 4 : 0;
  }
  // the bit-plane form (tile_pass_body with PLANES): two sets of K planes, a
  // zero count per plane word, the 256-entry compress table, then the deep
  // records
  static constexpr size_t plane_area() { return size_t(2) * K * SBW * 4 + size_t(T / 32) * 4 + 256 * 4; }
  static constexpr size_t plane_smem_bytes() { return plane_area() + deep_bytes(); }
};

// Bit q of the 8 keys of w0 (keys 0-3, key k in byte k) and w1 (keys 4-7),
// key 0 in bit 7 of the result (higher bits are not cleared).  The 8 bits are
// spread to byte bit 0 (w1) and bit 4 (w0) and collected by one 32x32->64-bit
// multiply by 2^4 + 2^13 + 2^22 + 2^31: the 32 partial products land on
// distinct bit positions, so no carries disturb bits 28-35.
__device__ __forceinline__ uint32_t key_bits8(uint32_t w0, uint32_t w1, int q) {
  const uint32_t t0 = (w0 >> q) & 0x01010101u, t1 = (w1 >> q) & 0x01010101u;
  return uint32_t((uint64_t(t0 * 16u + t1) * 0x80402010ull) >> 28);
}

// Split bits of the keys of one 16-byte vector, MSB first: bit KPL-1-i is the
// bit of key i.
template <typename KeyT>
__device__ __forceinline__ uint32_t vector_bits(const uint4& v, uint32_t sh) {
  if (sh >= 8 * sizeof(KeyT)) return 0u;  // above the key width every bit is 0
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
  uint32_t m = 0;
  if constexpr (sizeof(KeyT) == 1) {
    // byte k of a word lands at bit 3-k: ((w >> sh) & 0x01010101) * 0x80402010 >> 28
    // (one 32-bit multiply per word measured faster in this form than
    // key_bits8's 64-bit multiply per two words)
#pragma unroll
    for (int q = 0; q < 4; ++q) m |= ((((w[q] >> sh) & 0x01010101u) * 0x80402010u) >> 28) << (12 - 4 * q);
  } else if constexpr (sizeof(KeyT) == 2) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t t = (w[q] >> sh) & 0x00010001u;
      m |= (((t << 1) | (t >> 16)) & 3u) << (6 - 2 * q);
    }
  } else if constexpr (sizeof(KeyT) == 4) {
#pragma unroll
    for (int q = 0; q < 4; ++q) m |= ((w[q] >> sh) & 1u) << (3 - q);
  } else {
    m = (uint32_t(((uint64_t(w[1]) << 32 | w[0]) >> sh) & 1u) << 1) | uint32_t(((uint64_t(w[3]) << 32 | w[2]) >> sh) & 1u);
  }
  return m;
}

// D-bit fields [lo, lo+D) of the keys of one 16-byte vector (fmask: the
// field mask clipped to the key width).
template <typename KeyT>
__device__ __forceinline__ void vector_fields(const uint4& v, uint32_t lo, uint32_t fmask,
                                              uint32_t (&f)[16 / sizeof(KeyT)]) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if constexpr (sizeof(KeyT) == 1) {
      const uint32_t x = (w[q] >> lo) & (fmask * 0x01010101u);
#pragma unroll
      for (int k = 0; k < 4; ++k) f[4 * q + k] = __byte_perm(x, 0u, 0x4440u + k);
    } else if constexpr (sizeof(KeyT) == 2) {
      const uint32_t x = (w[q] >> lo) & (fmask * 0x00010001u);
      f[2 * q] = x & 0xFFFFu;
      f[2 * q + 1] = x >> 16;
    } else {
      f[q] = (w[q] >> lo) & fmask;
    }
  }
}

// Key i of a 16-byte vector, as the low bits of a 32-bit register (64-bit
// keys: the full key).  i is a constant after unrolling.
template <typename KeyT>
__device__ __forceinline__ auto vector_key(const uint4& v, int i) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
  if constexpr (sizeof(KeyT) == 1) return uint32_t(w[i >> 2] >> (8 * (i & 3)));
  else if constexpr (sizeof(KeyT) == 2) return uint32_t(w[i >> 1] >> (16 * (i & 1)));
  else if constexpr (sizeof(KeyT) == 4) return w[i];
  else return uint64_t(w[2 * i]) | (uint64_t(w[2 * i + 1]) << 32);
}

__device__ __forceinline__ void st_shared_key(uint32_t addr, uint32_t v, int bytes) {
  if (bytes == 1) asm volatile("st.shared.u8 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
  else if (bytes == 2) asm volatile("st.shared.u16 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
  else asm volatile("st.shared.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ void st_shared_key(uint32_t addr, uint64_t v, int) {
  asm volatile("st.shared.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}

// Stable 1-bit split of the keys of one vector: key i goes to the one cursor
// plus the ones before it, or to the zero cursor plus the zeros before it
// (shared byte addresses).  FULL: all KPL keys are valid; otherwise the
// first `valid`.
template <typename KeyT, int KPL, bool FULL>
__device__ __forceinline__ void scatter_vector(const uint4& v, uint32_t mb, uint32_t zd, uint32_t od, int valid) {
  constexpr uint32_t KB = sizeof(KeyT);
#pragma unroll
  for (int i = 0; i < KPL; ++i) {
    if (!FULL && i >= valid) break;
    const uint32_t c = i ? __popc(mb >> (KPL - i)) : 0u;  // ones before key i
    const uint32_t one = (mb >> (KPL - 1 - i)) & 1u;
    st_shared_key(one ? od + c * KB : zd + (uint32_t(i) - c) * KB, vector_key<KeyT>(v, i), int(KB));
  }
}

// Decoupled look-back of all NLB counters of a tile by the whole CTA.  The
// state is counter-major (counter c of tile t at lb[c * tiles + t]): warp w
// examines predecessors base-32w-31 .. base-32w, one coalesced load per
// counter, so one round trip covers 32*WARPS predecessors (the inclusive
// prefixes must propagate faster than tiles complete).  Per counter the walk
// stops at the nearest inclusive prefix.  A segment's first tile publishes
// its inclusive values at once, so no walk crosses a segment start.  The
// tile's own aggregates (mine, at most one tile of keys each) were published
// when it counted its keys.  Leaves the exclusive prefixes in pre[0..NLB)
// and publishes the inclusive ones.  Called by every thread of the CTA.  A
// wait gives up after `spin_limit` polls (~64 ns apart): kErrTimeout, and the
// missing counts are taken as zero, so the kernel always returns.
template <int NLB, int WARPS>
__device__ __forceinline__ void segment_lookback_cta(unsigned long long* lb, uint32_t tiles, uint32_t tile,
                                                     uint32_t first, const uint32_t* mine, unsigned long long* pre,
                                                     unsigned long long (*wsum)[NLB], uint32_t* wmask,
                                                     uint32_t* s_open, uint32_t* status, uint32_t spin_limit) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid < NLB) pre[tid] = 0;
  if (tile == first) return;  // its inclusive values went out with its counts
  if (tid == 0) *s_open = (1u << NLB) - 1u;
  __syncthreads();
  int64_t base = int64_t(tile) - 1;
  for (;;) {
    const uint32_t open = *s_open;
    if (!open) break;
    const int64_t t = base - 32 * warp - lane;
    const bool real = t >= int64_t(first);
    const unsigned long long* col = lb + (real ? t : 0);
    uint64_t v[NLB];
#pragma unroll
    for (int c = 0; c < NLB; ++c)
      v[c] = (real && ((open >> c) & 1u)) ? ld_volatile(col + uint64_t(c) * tiles) : kFlagPrefix;
    // wait (bounded) for counters a predecessor has not published yet
    for (uint32_t spins = 0;; ++spins) {
      bool missing = false;
#pragma unroll
      for (int c = 0; c < NLB; ++c) missing |= (v[c] >> 62) == 0;
      if (!missing) break;
      if (spins >= spin_limit) {
        atomicOr(status, kErrTimeout);
#pragma unroll
        for (int c = 0; c < NLB; ++c)
          if ((v[c] >> 62) == 0) v[c] = kFlagPrefix;
        break;
      }
      __nanosleep(64);
#pragma unroll
      for (int c = 0; c < NLB; ++c)
        if ((v[c] >> 62) == 0) v[c] = ld_volatile(col + uint64_t(c) * tiles);
    }
    uint32_t pbits = 0;
#pragma unroll
    for (int c = 0; c < NLB; ++c) {
      if (!((open >> c) & 1u)) continue;
      const bool isp = (v[c] >> 62) == 2;
      const uint32_t pmask = __ballot_sync(0xFFFFFFFFu, isp);
      const int stop = pmask ? __ffs(pmask) - 1 : 32;  // nearest inclusive prefix in this window
      // aggregates before it are single-tile counts: a 32-bit warp sum
      const uint32_t agg = __reduce_add_sync(0xFFFFFFFFu, (lane < stop && !isp) ? uint32_t(v[c]) : 0u);
      const uint64_t pv = __shfl_sync(0xFFFFFFFFu, v[c] & kCountMask, pmask ? stop : 0);
      if (lane == 0) wsum[warp][c] = uint64_t(agg) + (pmask ? pv : 0ull);
      pbits |= pmask ? (1u << c) : 0u;
    }
    if (lane == 0) wmask[warp] = pbits;
    __syncthreads();
    if (tid < NLB && ((open >> tid) & 1u)) {
      uint64_t e = pre[tid];
      bool closed = false;
      for (int w = 0; w < WARPS && !closed; ++w) {
        e += wsum[w][tid];
        closed = (wmask[w] >> tid) & 1u;
      }
      pre[tid] = e;
      if (closed) atomicAnd(s_open, ~(1u << tid));
    }
    __syncthreads();
    base -= 32 * WARPS;
  }
  if (tid < NLB) st_volatile(lb + uint64_t(tid) * tiles + tile, kFlagPrefix | (pre[tid] + mine[tid]));
}

// 64 stream bits starting at bit `x` of a shared bit stream (MSB first).
__device__ __forceinline__ uint64_t stream64(const uint32_t* sb, uint32_t x) {
  const uint32_t i = x >> 5, sh = x & 31;
  const uint32_t w0 = sb[i], w1 = sb[i + 1], w2 = sb[i + 2];
  const uint32_t hi = __funnelshift_l(w1, w0, sh), lo = __funnelshift_l(w2, w1, sh);
  return (uint64_t(hi) << 32) | lo;
}

// Stream bits [src, src+len) to level bits [dst, dst+len), 64-bit words
// k = k0, k0 + step, ... of the destination range.  Words the run covers
// whole are stored (the lean path); so is the level's last word when the run
// fills it up to the level's end; the (at most two) words shared with other
// runs are OR-ed, so those must be zero before the pass.  (Clearing the run's
// own bits with an AND first would make zeroing unnecessary, but costs each
// pass more in L2 atomics than the zeroing costs.)
__device__ __forceinline__ void write_bits64(uint64_t* level, uint64_t nbits, uint64_t dst, const uint32_t* sb,
                                             uint32_t src, uint32_t len, uint32_t k0, uint32_t step,
                                             uint32_t* status) {
  if (len == 0) return;
  if (dst + len > nbits) {
    if (k0 == 0) atomicOr(status, kErrBounds);
    return;
  }
  uint64_t* out = level + (dst >> 6);
  const uint32_t lead = uint32_t(dst & 63);
  const uint32_t nwords = (lead + len + 63) >> 6;
  const uint32_t tail = (lead + len) & 63;  // bits of the last word covered (0: all 64)
  const bool at_end = dst + len == nbits;   // the run ends the level: the rest of its last word is padding
  // whole words: [kb, ke)
  const uint32_t kb = lead ? 1u : 0u;
  const uint32_t ke = (tail == 0 || (at_end && nwords > kb)) ? nwords : nwords - 1;
  const uint32_t base = src - lead;  // stream bit of destination word 0's first bit (+64k)
  for (uint32_t k = k0; k < nwords; k += step) {
    if (k >= kb && k < ke) {
      const uint32_t x = base + 64 * k;
      const uint32_t i = x >> 5, sh = x & 31;
      const uint32_t w0 = sb[i], w1 = sb[i + 1], w2 = sb[i + 2];
      uint64_t val = (uint64_t(__funnelshift_l(w1, w0, sh)) << 32) | __funnelshift_l(w2, w1, sh);
      if (k == nwords - 1 && tail) val &= ~(~0ull >> tail);  // owned last word: clear the padding
      out[k] = val;
    } else {
      uint64_t val = k ? stream64(sb, base + 64 * k) : (stream64(sb, src) >> lead);
      uint64_t mask = k ? ~0ull : (~0ull >> lead);
      if (k == nwords - 1 && tail) mask &= ~(~0ull >> tail);
      atomicOr(reinterpret_cast<unsigned long long*>(out + k), (unsigned long long)(val & mask));
    }
  }
}

// write_bits64 for levels that were not zeroed: a shared word is cleared in
// the run's bits before they are set.
__device__ __forceinline__ void write_bits64_clear(uint64_t* level, uint64_t nbits, uint64_t dst, const uint32_t* sb,
                                                   uint32_t src, uint32_t len, uint32_t k0, uint32_t step,
                                                   uint32_t* status) {
  if (len == 0) return;
  if (dst + len > nbits) {
    if (k0 == 0) atomicOr(status, kErrBounds);
    return;
  }
  uint64_t* out = level + (dst >> 6);
  const uint32_t lead = uint32_t(dst & 63);
  const uint32_t nwords = (lead + len + 63) >> 6;
  const uint32_t tail = (lead + len) & 63;
  const bool at_end = dst + len == nbits;
  const uint32_t kb = lead ? 1u : 0u;
  const uint32_t ke = (tail == 0 || (at_end && nwords > kb)) ? nwords : nwords - 1;
  const uint32_t base = src - lead;
  for (uint32_t k = k0; k < nwords; k += step) {
    const uint64_t tmask = (k == nwords - 1 && tail) ? ~(~0ull >> tail) : ~0ull;
    if (k >= kb && k < ke) {
      out[k] = stream64(sb, base + 64 * k) & tmask;
    } else {
      const uint64_t val = k ? stream64(sb, base + 64 * k) : (stream64(sb, src) >> lead);
      const uint64_t mask = (k ? ~0ull : (~0ull >> lead)) & tmask;
      atomicAnd(reinterpret_cast<unsigned long long*>(out + k), (unsigned long long)~mask);
      atomicOr(reinterpret_cast<unsigned long long*>(out + k), (unsigned long long)(val & mask));
    }
  }
}

// One warp copies `len` bytes from shared memory to global memory: byte
// stores up to a 4-byte aligned destination, then 32-bit stores whose source
// bytes are funnel-shifted out of aligned shared words, then the tail.
__device__ __forceinline__ void write_key_run(unsigned char* dst, const unsigned char* src, uint32_t len) {
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

// One warp copies `len` keys from shared memory to global memory, each
// narrowed to its low 8 * sizeof(KeyO) bits (the bits of the levels the
// following passes still split on): a key per lane and step.
template <typename KeyT, typename KeyO>
__device__ __forceinline__ void write_key_run_narrow(KeyO* dst, const KeyT* src, uint32_t len) {
  for (uint32_t i = threadIdx.x & 31; i < len; i += 32) dst[i] = KeyO(src[i]);
}

// Bytes [off, off + 16) of the 32 bytes lo:hi (off < 16, the same for the
// whole tile): a two-stage word shifter (by 2, then by 1 word) and one
// funnel shift per output word.
__device__ __forceinline__ uint4 realign16(const uint4& lo, const uint4& hi, uint32_t off) {
  const uint32_t w[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
  const bool s2 = (off & 8u) != 0, s1 = (off & 4u) != 0;
  uint32_t g[6], f[5];
#pragma unroll
  for (int i = 0; i < 6; ++i) g[i] = s2 ? w[i + 2] : w[i];
#pragma unroll
  for (int i = 0; i < 5; ++i) f[i] = s1 ? g[i + 1] : g[i];
  const uint32_t bsh = 8u * (off & 3u);
  return make_uint4(__funnelshift_r(f[0], f[1], bsh), __funnelshift_r(f[1], f[2], bsh),
                    __funnelshift_r(f[2], f[3], bsh), __funnelshift_r(f[3], f[4], bsh));
}

// Load `bytes` bytes from global `src` (any alignment) into the 16-byte
// aligned shared buffer `dst`, 16 bytes per thread step.  Bytes past the end
// of the tile are not read beyond the 16-byte block that holds the last one.
template <int THREADS>
__device__ __forceinline__ void load_tile_bytes(uint4* dst, const unsigned char* src, uint32_t bytes) {
  const uint32_t nv = (bytes + 15) >> 4;
  const uintptr_t sa = reinterpret_cast<uintptr_t>(src);
  const uint32_t off = uint32_t(sa & 15);
  const uint4* a = reinterpret_cast<const uint4*>(sa - off);
  if (off == 0) {
    for (uint32_t k = threadIdx.x; k < nv; k += THREADS) dst[k] = __ldcs(a + k);
    return;
  }
  const uint32_t last_block = uint32_t((off + bytes - 1) >> 4);  // last aligned block holding tile bytes
  for (uint32_t k = threadIdx.x; k < nv; k += THREADS) {
    const uint4 lo = __ldcs(a + k);
    const uint4 hi = k + 1 <= last_block ? __ldcs(a + k + 1) : make_uint4(0, 0, 0, 0);
    dst[k] = realign16(lo, hi, off);
  }
}

// A contiguous tile by one TMA bulk copy (cp.async.bulk) into shared memory:
// thread 0 arms the mbarrier with the byte count and issues the copy, every
// thread waits for the barrier's first phase.  Both addresses must be
// 16-byte aligned and `bytes` a multiple of 16 (the caller checks).  The
// wait is bounded (the context's limit, at least 2^16 polls): on expiry
// kErrTimeout is recorded and the thread waits once more (bounded, ~1 s) for
// the copy in flight, so that no copy outlives the tile; the tile then goes
// on (its results are void, the status says so) and publishes its prefixes.
__device__ __forceinline__ void bulk_load_tile(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                               uint32_t spin_limit, uint32_t* status) {
  const uint32_t b = uint32_t(__cvta_generic_to_shared(bar));
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     uint32_t(__cvta_generic_to_shared(dst))),
                 "l"(src), "r"(bytes), "r"(b)
                 : "memory");
  }
  auto done = [&]() {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(b)
        : "memory");
    return ok != 0;
  };
  const uint32_t limit = spin_limit > (1u << 16) ? spin_limit : (1u << 16);
  for (uint32_t spins = 0; !done();) {
    if (++spins >= limit) {
      atomicOr(status, kErrTimeout);
      for (uint32_t k = 0; k < (1u << 20) && !done(); ++k) __nanosleep(1000);
      return;
    }
  }
}

// ---- bit planes (the last pass of 1-byte keys) -----------------------------
// A plane holds one level's bit of every key of the tile, 32 keys per word,
// the first key in bit 31.  A 1-bit split of the keys then becomes a stable
// partition of each later plane's words by the split plane's word: its bits
// under zeros packed to the top ("compress", Hacker's Delight 7-4, mirrored to
// pack toward bit 31) and appended to the zero part of the new plane, the
// bits under ones to the one part.  The compress runs inside each byte (three
// rounds of moves by 1, 2 and 4 bits), then shifts the four byte pieces
// together; the move masks of a byte depend on its mask byte only and come
// from a 256-entry table, so a mask word costs four table reads and a byte
// transpose, once per word and polarity, for every plane that moves.

// Table entry of mask byte b: the move masks of compress toward bit 7 inside
// the byte (Hacker's Delight 7-4 with every shift mirrored: round i moves the
// selected bits whose remaining distance has bit i set) in bytes 0-2, the
// number of selected bits in byte 3.
__device__ __forceinline__ uint32_t compress_lut_entry(uint32_t b) {
  uint32_t m = b, mk = (~b & 0xFFu) >> 1, e = uint32_t(__popc(b)) << 24;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    uint32_t mp = mk ^ (mk >> 1);
    mp ^= mp >> 2;
    mp ^= mp >> 4;
    const uint32_t v = mp & m;
    m = ((m ^ v) | (v << (1 << i))) & 0xFFu;
    e |= v << (8 * i);
    mk &= ~mp;
  }
  return e;
}
// The byte move masks of mask word m (mv[0..2], byte k from the entry of mask
// byte k: a 4x4 byte transpose of the four entries) and the shifts that join
// the byte pieces (mv[3..5] for bytes 2, 1, 0: the bits not selected in the
// bytes above, summed from the top by one multiply).
__device__ __forceinline__ void compress_masks(const uint32_t* lut, uint32_t m, uint32_t (&mv)[6]) {
  const uint32_t e0 = lut[m & 0xFFu], e1 = lut[(m >> 8) & 0xFFu], e2 = lut[(m >> 16) & 0xFFu], e3 = lut[m >> 24];
  const uint32_t l01 = __byte_perm(e0, e1, 0x5140), l23 = __byte_perm(e2, e3, 0x5140);
  const uint32_t h01 = __byte_perm(e0, e1, 0x7362), h23 = __byte_perm(e2, e3, 0x7362);
  mv[0] = __byte_perm(l01, l23, 0x5410);
  mv[1] = __byte_perm(l01, l23, 0x7632);
  mv[2] = __byte_perm(h01, h23, 0x5410);
  const uint32_t sh = __byte_perm(0x08080808u - __byte_perm(h01, h23, 0x7632), 0u, 0x0123) * 0x01010101u;
  mv[3] = sh & 0xFFu;
  mv[4] = (sh >> 8) & 0xFFu;
  mv[5] = (sh >> 16) & 0xFFu;
}

// The bits of x under m, in order, packed to the top of the word (mv: the
// masks of m).
__device__ __forceinline__ uint32_t compress_apply(uint32_t x, uint32_t m, const uint32_t (&mv)[6]) {
  x &= m;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const uint32_t t = x & mv[i];
    x = (x ^ t) | (t << (1 << i));
  }
  return (x & 0xFF000000u) | ((x & 0x00FF0000u) << mv[3]) | ((x & 0x0000FF00u) << mv[4]) | ((x & 0xFFu) << mv[5]);
}

// OR the top `len` bits of v into a zeroed shared bit stream at bit `pos`
// (other threads fill the rest of the words it touches).
__device__ __forceinline__ void or_stream_bits(uint32_t* sb, uint32_t pos, uint32_t v, uint32_t len) {
  if (len == 0) return;
  const uint32_t i = pos >> 5, sh = pos & 31;
  atomicOr(sb + i, v >> sh);
  if (sh + len > 32) atomicOr(sb + i + 1, v << (32 - sh));
}

// Exclusive prefix of in[0..count) into out (count <= 128) by one warp, lane
// i taking entries 4i..4i+3.
__device__ __forceinline__ void warp_exclusive_scan(const uint32_t* in, uint32_t* out, int count, int lane) {
  uint32_t v[4], sum = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = 4 * lane + q;
    v[q] = i < count ? in[i] : 0u;
    sum += v[q];
  }
  uint32_t x = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
    if (lane >= d) x += y;
  }
  uint32_t run = x - sum;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = 4 * lane + q;
    if (i < count) out[i] = run;
    run += v[q];
  }
}

// The load and the splits of a tile in bit-plane form (tile_pass_body with
// PLANES; 1-byte keys, no S_{l+K}).  Leaves the streams of levels l..l+K-1
// (plane j of set j % 2), the run sizes and starts of key_1..key_D, and the
// finest-run counts (counted and published for the look-back, or given).
// Per split s the thread owning plane words [tid * WPT, (tid + 1) * WPT)
// reads its words of plane s (the split bit, in S_{l+s} order) and of the
// later planes, scans the zero counts over the CTA, and ORs the compressed
// zero and one parts of each later plane into the other set at the word's
// zero and one cursors; its own words of the read set are then cleared for
// the split after next.  BATCH: the tile has VP <= V vectors per thread, so
// NWt = THREADS * VP / 2 plane words, max(VP / 2, 1) per thread (VP = 1:
// the first half of the threads own one word each); the words above NWt stay
// zero.
template <int K, int THREADS, int V, bool BATCH>
__device__ __forceinline__ void tile_planes_splits(const TileArgs& a, const TileText& s_tx, const TileSeg& s_sg,
                                                   uint32_t g, uint32_t tl, uint64_t tstart, uint32_t n, int VP,
                                                   uint32_t shift, bool given, uint32_t* sbits, uint32_t* s_cnt,
                                                   unsigned long long* pre, uint32_t* s_wz, uint32_t* s_ztot,
                                                   uint32_t (*rsz)[1 << (K - 1)], uint32_t (*rst)[1 << (K - 1)]) {
  using C = TileCfg<uint8_t, K, false, THREADS, V>;
  constexpr int D = C::D, T = C::T, WARPS = C::WARPS, SBW = C::SBW, NLB = C::NLB;
  constexpr int NW = T / 32;         // plane words of a tile of V vectors per thread
  constexpr int WPT = NW / THREADS;  // plane words per thread in the splits
  static_assert(K >= 1 && K <= kTileGivenMaxLevels && WPT * THREADS == NW, "up to 8 levels; whole words per thread");
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t NWt = BATCH ? uint32_t(THREADS * VP / 2) : uint32_t(NW);  // plane words of this tile
  const int wpt = BATCH ? (VP >= 2 ? VP / 2 : 1) : WPT;                     // of them per thread
  uint32_t* zpos = sbits + 2 * K * SBW;  // zeros before each plane word, current split
  uint32_t* s_clut = zpos + NW;          // compress table
  for (int b = tid; b < 256; b += THREADS) s_clut[b] = compress_lut_entry(uint32_t(b));
  const uint32_t nfull = n >> 5, nrem = n & 31;
  auto word_valid = [&](uint32_t w) -> uint32_t {
    return w < nfull ? ~0u : ((w == nfull && nrem) ? ~0u << (32 - nrem) : 0u);
  };

  // set 1 and the words of set 0 above the tile's start cleared
  for (int i = tid; i < K * SBW; i += THREADS) sbits[K * SBW + i] = 0u;
  if (BATCH && NWt < uint32_t(NW)) {
    const uint32_t pad = uint32_t(SBW) - NWt;
    for (uint32_t i = tid; i < K * pad; i += THREADS) sbits[(i / pad) * SBW + NWt + i % pad] = 0u;
  } else if (tid < 2 * K) {
    sbits[(tid >> 1) * SBW + NW + (tid & 1)] = 0u;
  }
  if (tid == 0) {
    rsz[0][0] = n;
    rst[0][0] = 0;
  }

  // ---- load; planes 0..K-1 in text order (set 0) ---------------------------
  {
    const uintptr_t sa = reinterpret_cast<uintptr_t>(static_cast<const unsigned char*>(a.in) + s_sg.in_begin + tstart);
    const uint32_t off = uint32_t(sa & 15);
    const uint4* av = reinterpret_cast<const uint4*>(sa - off);
    const uint32_t nvec = (n + 15) >> 4;
    const uint32_t last_block = uint32_t((uint64_t(off) + n + 15) >> 4) - 1;  // last aligned block holding tile bytes
    const uint32_t lo = shift - uint32_t(K - 1);  // plane j is key bit lo + K-1-j
#pragma unroll
    for (int r = 0; r < V; ++r) {
      if (BATCH && r >= VP) break;  // uniform over the CTA
      const int gv = (warp * VP + r) * 32 + lane;
      uint4 kv = make_uint4(0u, 0u, 0u, 0u);
      if (uint32_t(gv) < nvec) {
        const uint4 x0 = __ldcs(av + gv);
        if (off == 0) {
          kv = x0;
        } else {
          const uint4 x1 = uint32_t(gv) + 1 <= last_block ? __ldcs(av + gv + 1) : make_uint4(0u, 0u, 0u, 0u);
          kv = realign16(x0, x1, off);
        }
      }
      const int rem = int(n) - gv * 16;
      const int nvv = rem >= 16 ? 16 : (rem > 0 ? rem : 0);
      const uint32_t vm = 0xFFFFu & ~((1u << (16 - nvv)) - 1u);  // valid keys, key 0 in bit 15
      const uint32_t w0 = kv.x >> lo, w1 = kv.y >> lo, w2 = kv.z >> lo, w3 = kv.w >> lo;
      uint32_t b[K];
#pragma unroll
      for (int j = 0; j < K; ++j)
        b[j] = __byte_perm(key_bits8(w2, w3, K - 1 - j), key_bits8(w0, w1, K - 1 - j), 0x0040) & vm;
      // an even lane's vector is the upper half of the plane word, its odd
      // neighbour's the lower half: one shuffle per two planes
      const uint32_t pwi = uint32_t(gv) >> 1;
#pragma unroll
      for (int j = 0; j < K; j += 2) {
        if (j + 1 < K) {
          const uint32_t odd = __shfl_down_sync(0xFFFFFFFFu, b[j] | (b[j + 1] << 16), 1);
          if (!(lane & 1)) {
            sbits[j * SBW + pwi] = (b[j] << 16) | (odd & 0xFFFFu);
            sbits[(j + 1) * SBW + pwi] = (b[j + 1] << 16) | (odd >> 16);
          }
        } else {
          const uint32_t odd = __shfl_down_sync(0xFFFFFFFFu, b[j], 1);
          if (!(lane & 1)) sbits[j * SBW + pwi] = (b[j] << 16) | odd;
        }
      }
    }
  }
  __syncthreads();

  // ---- counts of the finest runs (key_D: bit t of the digit is plane t) -----
  if constexpr (D >= 1) {
    if (given) {
      for (int c = tid; c < NLB; c += THREADS) {
        const uint64_t blk = a.text_blocks ? uint64_t(s_tx.blk0) + tl / a.tiles_per_block : g / a.tiles_per_block;
        s_cnt[c] = a.tilecnt[uint64_t(g) * NLB + c];
        pre[c] = a.blockpre[blk * NLB + c] + a.relpre[uint64_t(g) * NLB + c];
      }
    } else if constexpr (K > kTileMaxLevels) {  // deeper passes need their prefixes given
      if (tid == 0) atomicOr(a.status, kErrBounds);
      for (int c = tid; c < NLB; c += THREADS) s_cnt[c] = 0, pre[c] = 0;
    } else {
      // per-warp counts in the zero-count words (first written after split 0's barrier)
      uint32_t (*s_wcnt)[NLB] = reinterpret_cast<uint32_t (*)[NLB]>(zpos);
      static_assert(WARPS * NLB <= NW, "the counts fit the zero-count words");
      uint32_t cnt[NLB];
#pragma unroll
      for (int c = 0; c < NLB; ++c) cnt[c] = 0;
#pragma unroll
      for (int k = 0; k < WPT; ++k) {
        if (BATCH && k >= wpt) break;
        const uint32_t w = uint32_t(tid) * wpt + k;
        const uint32_t vmk = word_valid(w);  // 0 above the tile's words
        uint32_t pl[D];
#pragma unroll
        for (int t = 0; t < D; ++t) pl[t] = sbits[t * SBW + w];
#pragma unroll
        for (int c = 0; c < NLB; ++c) {
          uint32_t mt = vmk;
#pragma unroll
          for (int t = 0; t < D; ++t) mt &= ((c >> t) & 1) ? pl[t] : ~pl[t];
          cnt[c] += __popc(mt);
        }
      }
#pragma unroll
      for (int c = 0; c < NLB; ++c) {
        const uint32_t x = __reduce_add_sync(0xFFFFFFFFu, cnt[c]);
        if (lane == 0) s_wcnt[warp][c] = x;
      }
      __syncthreads();
      if (tid < NLB) {
        uint32_t t = 0;
#pragma unroll
        for (int w = 0; w < WARPS; ++w) t += s_wcnt[w][tid];
        s_cnt[tid] = t;
        st_volatile(a.lookback + uint64_t(tid) * a.tiles + g, (g == s_sg.tile0 ? kFlagPrefix : kFlagAggregate) | t);
      }
    }
  }

  // ---- the splits -------------------------------------------------------------
#pragma unroll
  for (int s = 0; s < D; ++s) {
    uint32_t* Pc = sbits + (s & 1) * K * SBW;        // planes in S_{l+s} order
    uint32_t* Pn = sbits + ((s & 1) ^ 1) * K * SBW;  // planes s+1.. in S_{l+s+1} order
    uint32_t m[WPT], vmk[WPT], zc[WPT], pw[K][WPT];
    uint32_t tsum = 0;
#pragma unroll
    for (int k = 0; k < WPT; ++k) {
      const uint32_t w = uint32_t(tid) * wpt + k;  // < NW: every word read is inside the planes
      vmk[k] = (BATCH && k >= wpt) ? 0u : word_valid(w);
      m[k] = (BATCH && k >= wpt) ? 0u : Pc[s * SBW + w];
      zc[k] = __popc(~m[k] & vmk[k]);
      tsum += zc[k];
#pragma unroll
      for (int p = s + 1; p < K; ++p) pw[p][k] = (BATCH && k >= wpt) ? 0u : Pc[p * SBW + w];
    }
    uint32_t x = tsum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) s_wz[warp] = x;
    __syncthreads();  // (A)
    uint32_t ztot = 0, zpre = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t z = s_wz[w];
      ztot += z;
      zpre += w < warp ? z : 0u;
    }
    if (tid == 0) *s_ztot = ztot;
    if constexpr (K > kTileMaxLevels) {  // up to 64 runs: a warp scan
      if (s >= 2 && warp == 0) warp_exclusive_scan(rsz[s], rst[s], 1 << s, lane);
    } else if (s >= 2 && tid == 0) {
      uint32_t run = 0;
      for (int v = 0; v < (1 << s); ++v) {
        rst[s][v] = run;
        run += rsz[s][v];
      }
    }
    uint32_t zp = zpre + x - tsum;  // zeros before this thread's first word
#pragma unroll
    for (int k = 0; k < WPT; ++k) {
      if (BATCH && k >= wpt) break;
      const uint32_t w = uint32_t(tid) * wpt + k;
      zpos[w] = zp;
#pragma unroll
      for (int p = s + 1; p < K; ++p) Pc[p * SBW + w] = 0u;  // read above; set again two splits on
      if (s + 1 < K) {
        const uint32_t mz = ~m[k] & vmk[k], mo = m[k];
        const uint32_t nz = zc[k], no = __popc(mo);
        const uint32_t opos = ztot + 32u * w - zp;  // every word before w is whole
        uint32_t mvz[6], mvo[6];
        compress_masks(s_clut, mz, mvz);
        compress_masks(s_clut, mo, mvo);
#pragma unroll
        for (int p = s + 1; p < K; ++p) {
          or_stream_bits(Pn + p * SBW, zp, compress_apply(pw[p][k], mz, mvz), nz);
          or_stream_bits(Pn + p * SBW, opos, compress_apply(pw[p][k], mo, mvo), no);
        }
      }
      zp += zc[k];
    }
    __syncthreads();  // (B)
    // ---- run sizes of key_{s+1} -------------------------------------------
    if (s == 0) {
      if (tid == 0) {
        rsz[1][0] = ztot;
        rsz[1][1] = n - ztot;
        rst[1][0] = 0;
        rst[1][1] = ztot;
      }
    } else if (tid < (2 << s)) {
      const int v = tid & ((1 << s) - 1);
      const uint32_t st = rst[s][v], en = st + rsz[s][v];
      auto zb = [&](uint32_t p) -> uint32_t {  // zeros of plane s before position p (S_{l+s} order)
        if (p >= n) return *s_ztot;
        const uint32_t w = p >> 5, k = p & 31;
        return zpos[w] + k - (k ? __popc(Pc[s * SBW + w] >> (32 - k)) : 0u);
      };
      const uint32_t zin = zb(en) - zb(st);
      rsz[s + 1][tid] = (tid >> s) ? rsz[s][v] - zin : zin;
    }
  }
}

// One tile of a pass: tile g of the launch's segments.  BATCH: a pass of a
// batch of texts inside the persistent kernel (tile_batch.cu): the tile size
// is the text's own (TileText::vpt vectors per thread, a warp's slice
// shrinking with it), the tile first waits until every tile of the text's
// previous pass is done and afterwards counts itself done; otherwise
// TileText's batch fields are ignored.
// KeyO: the key type of S_{l+K} (KeyT, or narrower when the levels left
// after this pass fit it).  PLANES (1-byte keys, a pass without S_{l+K}, up
// to 4 levels): the splits move bit planes instead of keys.
template <typename KeyT, int K, bool OUT, int THREADS, int V, bool BATCH, typename KeyO = KeyT, bool PLANES = false>
__device__ __forceinline__ void tile_pass_body(const TileArgs& a, uint32_t g_in) {
  using C = TileCfg<KeyT, K, OUT, THREADS, V>;
  constexpr int D = C::D, KPL = C::KPL, T = C::T, WARPS = C::WARPS, WSLICE = C::WSLICE, SBW = C::SBW;
  constexpr int NLB = C::NLB, LPC = C::LPC;
  constexpr uint32_t FULLV = (1u << KPL) - 1u;
  constexpr int KB = int(sizeof(KeyT));

  extern __shared__ __align__(16) unsigned char smem_raw[];
  KeyT* buf0 = reinterpret_cast<KeyT*>(smem_raw);
  // K streams of SBW words (PLANES: two sets of K planes, the stream of level
  // l+j being plane j of set j % 2)
  uint32_t* sbits = reinterpret_cast<uint32_t*>(smem_raw + (PLANES ? size_t(0) : size_t(T) * KB));
  uint32_t* meta = sbits + K * SBW;  // D >= 2: per vector
  auto stream = [&](int j) -> const uint32_t* { return sbits + ((PLANES ? (j & 1) * K : 0) + j) * SBW; };

  __shared__ uint32_t s_tile, s_seg;
  __shared__ TileSeg s_sg;
  __shared__ TileText s_tx;
  __shared__ uint32_t s_wz[WARPS];
  __shared__ uint32_t s_ztot;
  __shared__ uint32_t rsz[D + 1][1 << D], rst[D + 1][1 << D];
  __shared__ unsigned long long pre[NLB];
  __shared__ unsigned long long s_table[tile_table_size(K)];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (warp == 0) {
    // the last segment with tile0 <= g, by a 32-way search of warp 0 (a
    // batch has thousands of segments: three dependent loads, not twelve).
    // Invariant: segs[lo].tile0 <= g < segs[hi].tile0 (hi = nsegs: none).
    const uint32_t g = g_in;
    uint32_t lo = 0, hi = a.nsegs;
    while (hi - lo > 1) {
      const uint32_t span = hi - lo;
      const uint32_t idx = span <= 32 ? lo + uint32_t(lane) : lo + uint32_t((uint64_t(span) * uint32_t(lane)) >> 5);
      const bool le = idx < hi && (idx == lo || a.segs[idx].tile0 <= g);
      const uint32_t m = __ballot_sync(0xFFFFFFFFu, le);
      const int k = 31 - __clz(m);  // the last probe at or before the answer (lane 0 always is)
      const uint32_t nxt = __shfl_sync(0xFFFFFFFFu, idx, k < 31 ? k + 1 : 31);
      lo = __shfl_sync(0xFFFFFFFFu, idx, k);
      if (k < 31) hi = min(hi, nxt);
    }
    if (lane == 0) {
      s_tile = g;
      s_seg = lo;
    }
  }
  __syncthreads();
  const uint32_t g = s_tile;
  if (tid == 0) {
    s_sg = a.segs[s_seg];
    s_tx = a.texts[s_sg.text];
  }
  __syncthreads();
  if constexpr (BATCH) {
    if (s_tx.wait_idx != ~0u) {  // the text's previous pass wrote this pass's input
      if (tid == 0) {
        const volatile unsigned int* dp = a.done + s_tx.wait_idx;
        const unsigned int need = a.need[s_tx.wait_idx];
        for (uint32_t spins = 0; *dp < need; ++spins) {
          if (spins >= a.spin_limit) {
            atomicOr(a.status, kErrTimeout);
            break;
          }
          __nanosleep(128);
        }
        __threadfence();
      }
      __syncthreads();
    }
  }
  const int VP = BATCH ? int(s_tx.vpt) : V;  // vectors per thread of this tile
  const uint32_t TT = BATCH ? uint32_t(THREADS * VP * KPL) : uint32_t(T);
  const uint32_t tl = g - s_sg.tile0;
  const uint64_t tstart = uint64_t(tl) * TT;
  const uint32_t n = s_sg.m - tstart < uint64_t(TT) ? uint32_t(s_sg.m - tstart) : TT;
  for (int i = tid; i < tile_table_size(K); i += THREADS) s_table[i] = a.tables[s_sg.table + i];

  const uint32_t shift = s_tx.shift;
  __shared__ uint32_t s_cnt[NLB];
  const bool given = a.blockpre != nullptr;  // prefixes from the histogram kernel
  int cur = 0;
  if constexpr (PLANES) {
    static_assert(sizeof(KeyT) == 1 && !OUT, "bit planes: passes over 1-byte keys without S_{l+K}");
    static_assert(K <= kTileMaxLevels || !BATCH, "batched passes take at most 4 levels");
    tile_planes_splits<K, THREADS, V, BATCH>(a, s_tx, s_sg, g, tl, tstart, n, VP, shift, given, sbits, s_cnt, pre,
                                             s_wz, &s_ztot, rsz, rst);
  } else {
  {
    const unsigned char* src = static_cast<const unsigned char*>(a.in) + (s_sg.in_begin + tstart) * KB;
    const uint32_t bytes = n * uint32_t(KB);
    // a 16-byte aligned tile of whole 16-byte blocks (every tile of a first
    // pass but the text's last): one TMA bulk copy; otherwise vector loads
    if (!BATCH && (reinterpret_cast<uintptr_t>(src) & 15) == 0 && (bytes & 15) == 0 && bytes) {
      __shared__ __align__(8) uint64_t s_bar;
      bulk_load_tile(buf0, src, bytes, &s_bar, a.spin_limit, a.status);
    } else {
      load_tile_bytes<THREADS>(reinterpret_cast<uint4*>(buf0), src, bytes);
    }
  }
  if (tid == 0) {
    rsz[0][0] = n;
    rst[0][0] = 0;
  }
  __syncthreads();

  const uint32_t smem_base = uint32_t(__cvta_generic_to_shared(smem_raw));

  // ---- counts of the finest runs (key_D), published before the splits -----
  // Every thread counts its keys into its own 16-bit column of 2^D counters
  // in the stream area (free until the first split emits a stream).
  if (D >= 1 && given) {
    if (tid < NLB) {
      const uint64_t blk = a.text_blocks ? uint64_t(s_tx.blk0) + tl / a.tiles_per_block : g / a.tiles_per_block;
      s_cnt[tid] = a.tilecnt[uint64_t(g) * NLB + tid];
      pre[tid] = a.blockpre[blk * NLB + tid] + a.relpre[uint64_t(g) * NLB + tid];
    }
  } else if constexpr (D >= 1 && D <= kTileMaxLevels) {
    __shared__ uint32_t s_wcnt[WARPS][NLB];
    constexpr int NB = 1 << D;
    // bin b of thread t: half (t & 1) of word b * THREADS/2 + t/2 (a thread
    // counts at most 64 keys)
    uint32_t* cnt = sbits;
#pragma unroll
    for (int b = 0; b < NB; b += 2) cnt[b * (THREADS / 2) + tid] = 0;
    const uint32_t lo = shift - uint32_t(D - 1);  // field bit D-1 is level l
    const uint32_t fmask = uint32_t(NB - 1) & (KB < 4 ? (0xFFFFFFFFu >> (32 - 8 * KB)) >> lo : 0xFFFFFFFFu);
    const uint32_t cbase = smem_base + uint32_t(T * KB) + uint32_t(tid >> 1) * 4u;
    const uint32_t one = 1u << (16 * (tid & 1));
    __syncthreads();  // the counters are cleared by other threads
#pragma unroll
    for (int r = 0; r < V; ++r) {
      if (BATCH && r >= VP) break;
      const int gv = (warp * VP + r) * 32 + lane;
      const uint4 kv = reinterpret_cast<const uint4*>(buf0)[gv];
      const int rem = int(n) - gv * KPL;
      const int nvv = rem >= KPL ? KPL : (rem > 0 ? rem : 0);
      uint32_t f[KPL];
      vector_fields<KeyT>(kv, lo, fmask, f);
#pragma unroll
      for (int i = 0; i < KPL; ++i)
        if (i < nvv) asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(cbase + f[i] * uint32_t(THREADS * 2)), "r"(one) : "memory");
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const uint32_t x = __reduce_add_sync(0xFFFFFFFFu, (cnt[b * (THREADS / 2) + (tid >> 1)] >> (16 * (tid & 1))) & 0xFFFFu);
      if (lane == 0) s_wcnt[warp][b] = x;
    }
    __syncthreads();
    if (tid < NB) {
      uint32_t t = 0;
#pragma unroll
      for (int w = 0; w < WARPS; ++w) t += s_wcnt[w][tid];
      const int c = int(reverse_low_bits(uint32_t(tid), uint32_t(D)));  // key_D has level l least significant
      s_cnt[c] = t;
      st_volatile(a.lookback + uint64_t(c) * a.tiles + g, (g == s_sg.tile0 ? kFlagPrefix : kFlagAggregate) | t);
    }
    // the first split's scatter into the counter area follows its barrier (A)
  } else if constexpr (D > kTileMaxLevels) {
    if (tid == 0) atomicOr(a.status, kErrBounds);  // deeper passes need their prefixes given
  }
  // valid keys of this warp and before it
  const uint32_t wslice = BATCH ? uint32_t(32 * VP * KPL) : uint32_t(WSLICE);
  const uint32_t wbeg = uint32_t(warp) * wslice;
  const uint32_t nw = n > wbeg ? min(n - wbeg, wslice) : 0u;
  const uint32_t vbefore = min(n, wbeg);

#pragma unroll 1
  for (int s = 0; s < K; ++s) {
    const bool split = s < D;
    const KeyT* cb = buf0 + cur * T;
    const uint32_t sh = shift - uint32_t(s);
    uint4 kv[V];
    uint32_t mb[V];
    int nv[V];
#pragma unroll
    for (int r = 0; r < V; ++r) {
      if (BATCH && r >= VP) {  // beyond this tile's vectors (uniform over the CTA)
        kv[r] = make_uint4(0u, 0u, 0u, 0u);
        nv[r] = 0;
        mb[r] = 0;
        continue;
      }
      const int gv = (warp * VP + r) * 32 + lane;
      kv[r] = reinterpret_cast<const uint4*>(cb)[gv];
      const int rem = int(n) - gv * KPL;
      nv[r] = rem >= KPL ? KPL : (rem > 0 ? rem : 0);
      const uint32_t vm = nv[r] == KPL ? FULLV : (FULLV & ~((1u << (KPL - nv[r])) - 1u));
      mb[r] = vector_bits<KeyT>(kv[r], sh) & vm;
      // level l+s bits of this vector into stream s
      uint32_t x = mb[r] << (32 - KPL * (1 + (lane % LPC)));
#pragma unroll
      for (int d = 1; d < LPC; d <<= 1) x |= __shfl_down_sync(0xFFFFFFFFu, x, d);
      if (lane % LPC == 0) sbits[s * SBW + gv / LPC] = x;
    }
    if (!split) break;

    // ---- zero counts, warp scan over (round, lane) order ------------------
    uint32_t zc[V], ex[V];
#pragma unroll
    for (int r = 0; r < V; ++r) zc[r] = uint32_t(nv[r]) - __popc(mb[r]);
    uint32_t rb = 0;
#pragma unroll
    for (int q = 0; q < V / 2; ++q) {
      const uint32_t p = zc[2 * q] | (zc[2 * q + 1] << 16);
      uint32_t x = p;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if (lane >= d) x += y;
      }
      const uint32_t tot = __shfl_sync(0xFFFFFFFFu, x, 31);
      const uint32_t e = x - p;
      ex[2 * q] = rb + (e & 0xFFFFu);
      rb += tot & 0xFFFFu;
      ex[2 * q + 1] = rb + (e >> 16);
      rb += tot >> 16;
    }
    if (lane == 0) s_wz[warp] = rb;
    __syncthreads();  // (A)
    uint32_t ztot = 0, zpre = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t z = s_wz[w];
      ztot += z;
      zpre += w < warp ? z : 0u;
    }
    if (tid == 0) s_ztot = ztot;
    // starts of the key_s runs (sizes written after the previous split): a
    // warp scan for the many runs of deep passes, else thread 0
    if constexpr (K > kTileMaxLevels) {
      if (s >= 2 && warp == 0) warp_exclusive_scan(rsz[s], rst[s], 1 << s, lane);
    } else if (s >= 2 && tid == 0) {
      uint32_t run = 0;
      for (int v = 0; v < (1 << s); ++v) { rst[s][v] = run; run += rsz[s][v]; }
    }
    const uint32_t opre = vbefore - zpre;
    const uint32_t nb = smem_base;  // the keys are in registers: scatter into the same buffer
#pragma unroll
    for (int r = 0; r < V; ++r) {
      if (BATCH && r >= VP) break;
      const int gv = (warp * VP + r) * 32 + lane;
      const uint32_t before = min(nw, uint32_t((r * 32 + lane) * KPL));  // valid keys of the warp before the vector
      const uint32_t zd = nb + (zpre + ex[r]) * KB;
      const uint32_t od = nb + (ztot + opre + before - ex[r]) * KB;
      if constexpr (D >= 2) {
        if (s >= 1) meta[gv] = ((zpre + ex[r]) << 16) | mb[r];
      }
      if (nv[r] == KPL) scatter_vector<KeyT, KPL, true>(kv[r], mb[r], zd, od, KPL);
      else if (nv[r] > 0) scatter_vector<KeyT, KPL, false>(kv[r], mb[r], zd, od, nv[r]);
    }
    __syncthreads();  // (B)
    // ---- run sizes of key_{s+1} -------------------------------------------
    if (s == 0) {
      if (tid == 0) {
        rsz[1][0] = ztot;
        rsz[1][1] = n - ztot;
        rst[1][0] = 0;
        rst[1][1] = ztot;
      }
    } else if (tid < (2 << s)) {
      const int v = tid & ((1 << s) - 1);
      const uint32_t st = rst[s][v], en = st + rsz[s][v];
      auto zb = [&](uint32_t p) -> uint32_t {  // zeros before tile position p in the pre-split order
        if (p >= n) return s_ztot;
        const uint32_t w = meta[p / KPL], k = p % KPL;
        const uint32_t ones = k ? __popc((w & FULLV) >> (KPL - k)) : 0u;
        return (w >> 16) + k - ones;
      };
      const uint32_t zin = zb(en) - zb(st);
      rsz[s + 1][tid] = (tid >> s) ? rsz[s][v] - zin : zin;
    }
  }
  }  // !PLANES
  __syncthreads();
  if constexpr (D >= 2) {
    if constexpr (K > kTileMaxLevels) {
      if (warp == 0) warp_exclusive_scan(rsz[D], rst[D], 1 << D, lane);
    } else if (tid == 0) {
      uint32_t run = 0;
      for (int v = 0; v < (1 << D); ++v) { rst[D][v] = run; run += rsz[D][v]; }
    }
  }

  // ---- level l (one run, needs no prefix), then the look-back -------------
  const int nstruct = s_tx.wt ? 2 : 1;
  for (int st = 0; st < (a.first_level_written ? 0 : nstruct); ++st) {
    const uint64_t dst = s_table[st ? tile_wt_entry(K, 0, 0) : tile_wm_entry(0, 0)] + tstart;
    if (a.clear_edges)
      write_bits64_clear(st ? s_tx.wt : s_tx.wm, s_tx.nbits, dst, stream(0), 0, n, uint32_t(tid), uint32_t(THREADS),
                         a.status);
    else
      write_bits64(st ? s_tx.wt : s_tx.wm, s_tx.nbits, dst, stream(0), 0, n, uint32_t(tid), uint32_t(THREADS),
                   a.status);
  }
  if constexpr (D >= 1) {
    if (tid < NLB && s_cnt[tid] != rsz[D][tid]) atomicOr(a.status, kErrBounds);  // counts must agree
  }
  if constexpr (D >= 1 && D <= kTileMaxLevels) {
    __shared__ unsigned long long wsum[WARPS][NLB];
    __shared__ uint32_t wmask[WARPS], s_open;
    if (!given)
      segment_lookback_cta<NLB, WARPS>(a.lookback, a.tiles, g, s_sg.tile0, s_cnt, pre, wsum, wmask, &s_open,
                                       a.status, a.spin_limit);
  }
  __syncthreads();

  // ---- runs of S_{l+K} and of levels 1..K-1, round-robin over the warps ---
  // prefix of run v of key_j (j >= 1): the finest runs with key_j == v
  __shared__ unsigned long long runpre[(1 << K)];
  constexpr int NINNER = (1 << K) - 2;  // runs of levels 1..K-1 of one structure
  if (tid < NINNER) {
    int j = 1;
    while (tid + 2 >= (2 << j)) ++j;
    const int v = tid + 2 - (1 << j);
    uint64_t p = 0;
    for (int h = 0; h < (1 << (D - j)); ++h) p += pre[v + (h << j)];
    runpre[tid] = p;
  }
  __syncthreads();
  if constexpr (C::WORD_PARALLEL) {
    // Levels 1..K-1 of both structures, word-parallel: a deep level has up to
    // 2^(K-1) runs, most of them a few words long (and the tiles of 2- and
    // 4-byte keys are short), so instead of a warp per run every thread
    // takes destination words of the concatenated runs.  Per (structure,
    // level) list one warp scans the runs' word counts and stores a 16-byte
    // record per run (first destination word, stream bit of that word, last
    // whole word, lead and tail bits); a thread then finds its word's run by
    // binary search.  A word shared with other runs is cleared in this run's
    // bits, then set, whether or not the level was zeroed (writers of one
    // word touch disjoint bits, so the atomics commute, and the runs of a
    // level cover all of its bits).  In passes of 5..8 levels, levels 1..JW
    // (runs of 32 words and more on average) go a warp per run.
    constexpr int JW = C::JW;
    constexpr int NCJ = K - 1 - JW;         // word-parallel levels per structure
    constexpr int NC = 2 * NCJ;             // lists
    constexpr int MAXR = 1 << (K - 1);      // runs of the deepest level
    constexpr int RPL = (MAXR + 31) / 32;   // runs per lane in a scan
    constexpr int NREC = 2 * ((1 << K) - 2);
    static_assert(PLANES || K <= kTileMaxLevels || size_t(NREC) * 16 + size_t(NC) * (MAXR + 1) * 4 <= size_t(T) * KB,
                  "run records and word prefixes fit the key buffer");
    static_assert(size_t(NREC) * 16 + size_t(NC) * (MAXR + 1) * 4 == C::deep_bytes(), "deep record layout");
    // bit planes: after the planes; key form: 5..8 levels in the key buffer
    // (free after the splits), up to 4 after the streams
    unsigned char* deep = smem_raw + (PLANES ? C::plane_area() : (K > kTileMaxLevels ? size_t(0) : C::deep_offset()));
    static_assert(C::plane_area() % 16 == 0 && C::deep_offset() % 16 == 0, "16-byte records");
    uint4* rec = reinterpret_cast<uint4*>(deep);                   // [NREC]
    uint32_t* wp = reinterpret_cast<uint32_t*>(deep + NREC * 16);  // [NC][MAXR + 1]
    __shared__ uint32_t s_cw[NC + 1];
    const uint64_t nbits = s_tx.nbits;
    for (int c = warp; c < NC; c += WARPS) {
      const int st = c / NCJ, j = JW + 1 + c % NCJ;
      uint64_t* level = (st ? s_tx.wt : s_tx.wm) + uint64_t(j) * s_tx.stride;
      uint4* rc = rec + st * ((1 << K) - 2) + (1 << j) - 2;
      uint32_t cw[RPL], sum = 0;
#pragma unroll
      for (int q = 0; q < RPL; ++q) {
        const int v = lane * RPL + q;
        uint32_t w = 0;
        if (st < nstruct && v < (1 << j)) {
          const uint32_t len = rsz[j][v];
          const uint64_t dst = s_table[st ? tile_wt_entry(K, j, v) : tile_wm_entry(j, v)] + runpre[(1 << j) - 2 + v];
          if (len && dst + len > nbits) {
            atomicOr(a.status, kErrBounds);
          } else if (len) {
            const uint32_t lead = uint32_t(dst & 63), tail = (lead + len) & 63;
            w = (lead + len + 63) >> 6;
            const uint32_t kb = lead ? 1u : 0u;
            const uint32_t ke = (tail == 0 || (dst + len == nbits && w > kb)) ? w : w - 1;
            const uint64_t out = reinterpret_cast<uint64_t>(level + (dst >> 6));
            rc[v] = make_uint4(uint32_t(out), uint32_t(out >> 32), rst[j][v] - lead, ke | (lead << 16) | (tail << 24));
          }
        }
        cw[q] = w;
        sum += w;
      }
      uint32_t x = sum;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if (lane >= d) x += y;
      }
      uint32_t* w = wp + c * (MAXR + 1);
      uint32_t run = x - sum;
#pragma unroll
      for (int q = 0; q < RPL; ++q) {
        const int v = lane * RPL + q;
        if (v < (1 << j)) w[v] = run;
        run += cw[q];
      }
      if (lane == 31) {
        w[1 << j] = x;
        s_cw[c + 1] = x;
      }
    }
    __syncthreads();
    if (tid == 0) {
      s_cw[0] = 0;
      for (int c = 1; c <= NC; ++c) s_cw[c] += s_cw[c - 1];
    }
    __syncthreads();
    // levels 1..JW: a warp per run, round-robin
    constexpr int NSH = (2 << JW) - 2;  // runs of levels 1..JW of one structure
#pragma unroll 1
    for (int it = warp; it < nstruct * NSH; it += WARPS) {
      const int e = it % NSH, st = it / NSH;
      int j = 1;
      while (e + 2 >= (2 << j)) ++j;
      const int v = e + 2 - (1 << j);
      uint64_t* level = (st ? s_tx.wt : s_tx.wm) + uint64_t(j) * s_tx.stride;
      const uint64_t dst = s_table[st ? tile_wt_entry(K, j, v) : tile_wm_entry(j, v)] + runpre[e];
      write_bits64_clear(level, s_tx.nbits, dst, stream(j), rst[j][v], rsz[j][v], uint32_t(lane), 32u, a.status);
    }
    const uint32_t total = s_cw[NC];
    int c = 0;
#pragma unroll 1
    for (uint32_t f = uint32_t(tid); f < total; f += THREADS) {
      while (s_cw[c + 1] <= f) ++c;
      const int st = c / NCJ, j = JW + 1 + c % NCJ;
      const uint32_t* w = wp + c * (MAXR + 1);
      const uint32_t k0 = f - s_cw[c];
      int lo = 0, hi = 1 << j;  // the last run starting at or before word k0
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (w[mid] <= k0) lo = mid; else hi = mid;
      }
      const uint32_t k = k0 - w[lo], nw = w[lo + 1] - w[lo];
      const uint4 r = rec[st * ((1 << K) - 2) + (1 << j) - 2 + lo];
      uint64_t* out = reinterpret_cast<uint64_t*>(uint64_t(r.x) | (uint64_t(r.y) << 32));
      const uint32_t base = r.z, ke = r.w & 0xFFFFu, lead = (r.w >> 16) & 0xFFu, tail = r.w >> 24;
      const uint32_t* sb = stream(j);
      const uint64_t tmask = (k == nw - 1 && tail) ? ~(~0ull >> tail) : ~0ull;  // bits of the last word
      if (k >= (lead ? 1u : 0u) && k < ke) {
        out[k] = stream64(sb, base + 64 * k) & tmask;
      } else {
        const uint64_t val = k ? stream64(sb, base + 64 * k) : (stream64(sb, base + lead) >> lead);
        const uint64_t mask = (k ? ~0ull : (~0ull >> lead)) & tmask;
        atomicAnd(reinterpret_cast<unsigned long long*>(out + k), (unsigned long long)~mask);
        atomicOr(reinterpret_cast<unsigned long long*>(out + k), (unsigned long long)(val & mask));
      }
    }
    if constexpr (OUT) {
      const KeyT* cb = buf0 + cur * T;
#pragma unroll 1
      for (int v = warp; v < (1 << K); v += WARPS) {
        const uint32_t len = rsz[D][v];
        if (len == 0) continue;
        const uint64_t dst = s_table[tile_out_entry(K, v)] + pre[v];
        if (dst + len > a.out_size) {
          if (lane == 0) atomicOr(a.status, kErrBounds);
          continue;
        }
        if constexpr (sizeof(KeyO) == sizeof(KeyT))
          write_key_run(reinterpret_cast<unsigned char*>(static_cast<KeyT*>(a.out) + dst),
                        reinterpret_cast<const unsigned char*>(cb + rst[D][v]), len * uint32_t(KB));
        else
          write_key_run_narrow<KeyT, KeyO>(static_cast<KeyO*>(a.out) + dst, cb + rst[D][v], len);
      }
    }
  } else {
  constexpr int NOUT = OUT ? (1 << K) : 0;
  const int items = NOUT + nstruct * NINNER;
  const KeyT* cb = buf0 + cur * T;
#pragma unroll 1
  for (int it = warp; it < items; it += WARPS) {
    if (it < NOUT) {
      const int v = it;
      const uint32_t len = rsz[D][v];
      if (len == 0) continue;
      const uint64_t dst = s_table[tile_out_entry(K, v)] + pre[v];
      if (dst + len > a.out_size) {
        if (lane == 0) atomicOr(a.status, kErrBounds);
        continue;
      }
      if constexpr (sizeof(KeyO) == sizeof(KeyT))
        write_key_run(reinterpret_cast<unsigned char*>(static_cast<KeyT*>(a.out) + dst),
                      reinterpret_cast<const unsigned char*>(cb + rst[D][v]), len * uint32_t(KB));
      else
        write_key_run_narrow<KeyT, KeyO>(static_cast<KeyO*>(a.out) + dst, cb + rst[D][v], len);
    } else {
      const int e = (it - NOUT) % (NINNER > 0 ? NINNER : 1);
      const int st = (it - NOUT) / (NINNER > 0 ? NINNER : 1);
      int j = 1;
      while (e + 2 >= (2 << j)) ++j;
      const int v = e + 2 - (1 << j);
      uint64_t* level = (st ? s_tx.wt : s_tx.wm) + uint64_t(j) * s_tx.stride;
      const uint64_t dst = s_table[st ? tile_wt_entry(K, j, v) : tile_wm_entry(j, v)] + runpre[e];
      if (a.clear_edges)
        write_bits64_clear(level, s_tx.nbits, dst, stream(j), rst[j][v], rsz[j][v], uint32_t(lane), 32u,
                           a.status);
      else
        write_bits64(level, s_tx.nbits, dst, stream(j), rst[j][v], rsz[j][v], uint32_t(lane), 32u, a.status);
    }
  }
  }

  // ---- this tile's slab of the next pass's levels --------------------------
  if (a.zero_words) {
    const uint64_t z0 = uint64_t(g) * a.zero_per_tile;
    const uint64_t z1 = z0 + a.zero_per_tile < a.zero_words ? z0 + a.zero_per_tile : a.zero_words;
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    for (uint64_t w = z0 + 2 * uint64_t(tid); w < z1; w += 2 * THREADS) {
      *reinterpret_cast<uint4*>(a.zero_a + w) = zero;
      if (a.zero_b) *reinterpret_cast<uint4*>(a.zero_b + w) = zero;
    }
  }
  if constexpr (BATCH) {
    if (s_tx.signal_idx != ~0u) {  // every thread's writes are visible before the count
      __threadfence();
      __syncthreads();
      if (tid == 0) atomicAdd(a.done + s_tx.signal_idx, 1u);
    }
  }
}

// A launch of one pass: each CTA takes the next tile from the launch's tile
// counter.  CTAs per SM (registers a thread): the bit-plane form 6 (40), 4
// (64) for 5-8 levels; the key form over 1-byte keys 5 (48), over wider keys
// 4 (64; at 48 they spill more and measured slower), 3 for 5-8 levels.
template <typename KeyT, int K, bool OUT, int THREADS, int V, typename KeyO = KeyT, bool PLANES = false>
__global__ void __launch_bounds__(THREADS, (K > kTileMaxLevels ? (PLANES ? 1024 : 768)
                                                                 : (PLANES ? 1536 : (sizeof(KeyT) == 1 ? 1280 : 1024))) /
                                               THREADS) tile_pass_kernel(TileArgs a) {
  __shared__ uint32_t s_g;
  if (threadIdx.x == 0) s_g = a.tile_base + atomicAdd(a.tile_counter, 1u);
  __syncthreads();
  tile_pass_body<KeyT, K, OUT, THREADS, V, false, KeyO, PLANES>(a, s_g);
}

}  // namespace pwmgpu
