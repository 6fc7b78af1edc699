// Histogram, wavelet-tree regroup, Huffman key and generator kernels.
#include <algorithm>

#include "gen.hpp"
#include "kernels.cuh"

namespace pwmgpu {

namespace {

constexpr int kHistThreads = 512;

template <typename T, typename F>
__device__ __forceinline__ void for_each_symbol_vec(const T* text, uint64_t n, uint64_t tid, uint64_t nthreads,
                                                    F&& f) {
  // 16-byte vectors over the aligned body, then the tail element by element.
  constexpr int PER = 16 / sizeof(T);
  const uint64_t nvec = (reinterpret_cast<uintptr_t>(text) % 16 == 0) ? n / PER : 0;
  const uint4* v = reinterpret_cast<const uint4*>(text);
  for (uint64_t i = tid; i < nvec; i += nthreads) {
    uint4 x = __ldcs(v + i);
    const T* s = reinterpret_cast<const T*>(&x);
#pragma unroll
    for (int k = 0; k < PER; ++k) f(uint64_t(s[k]));
  }
  for (uint64_t i = nvec * PER + tid; i < n; i += nthreads) f(uint64_t(text[i]));
}

// L <= 8: one 256-bin sub-histogram per warp; 9..13: one per CTA.
template <typename T, int BINS, bool PER_WARP>
__global__ void __launch_bounds__(kHistThreads) leaf_hist_smem(const T* text, uint64_t n, uint32_t levels,
                                                               unsigned long long* hist, uint32_t* status) {
  constexpr int WARPS = kHistThreads / 32;
  constexpr int COPIES = PER_WARP ? WARPS : 1;
  __shared__ uint32_t h[COPIES * BINS];
  for (int i = threadIdx.x; i < COPIES * BINS; i += kHistThreads) h[i] = 0;
  __syncthreads();
  uint32_t* mine = h + (PER_WARP ? (threadIdx.x >> 5) * BINS : 0);
  const uint64_t limit = 1ull << levels;
  bool bad = false;
  for_each_symbol_vec<T>(text, n, uint64_t(blockIdx.x) * kHistThreads + threadIdx.x,
                         uint64_t(gridDim.x) * kHistThreads, [&](uint64_t c) {
                           if (c >= limit) { bad = true; return; }
                           atomicAdd(&mine[c], 1u);
                         });
  if (bad) atomicOr(status, kErrSymbol);
  __syncthreads();
  for (int b = threadIdx.x; b < int(limit); b += kHistThreads) {
    uint64_t s = 0;
    for (int w = 0; w < COPIES; ++w) s += h[w * BINS + b];
    if (s) atomicAdd(&hist[b], (unsigned long long)s);
  }
}

// L >= 14: global atomics, lanes holding the same symbol combined first.
template <typename T>
__global__ void __launch_bounds__(kHistThreads) leaf_hist_global(const T* text, uint64_t n, uint32_t levels,
                                                                 unsigned long long* hist, uint32_t* status) {
  const uint64_t limit = 1ull << levels;
  const int lane = threadIdx.x & 31;
  const uint64_t warp_id = (uint64_t(blockIdx.x) * kHistThreads + threadIdx.x) >> 5;
  const uint64_t warps = (uint64_t(gridDim.x) * kHistThreads) >> 5;
  bool bad = false;
  for (uint64_t base = warp_id * 32; base < n; base += warps * 32) {
    uint64_t i = base + lane;
    uint64_t c = i < n ? uint64_t(text[i]) : ~0ull;
    bool ok = i < n && c < limit;
    if (i < n && c >= limit) bad = true;
    uint32_t key = ok ? uint32_t(c) : 0xFFFFFFFFu;
    uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
    if (ok && lane == __ffs(peers) - 1) atomicAdd(&hist[c], (unsigned long long)__popc(peers));
  }
  if (bad) atomicOr(status, kErrSymbol);
}

// Leaf histogram (levels <= 8) that also counts, per tile of the first
// tile pass (tile_keys symbols), its finest runs: the 2^D values of the first
// D symbol bits read with the first bit least significant.  Block b walks
// tiles [b*tiles_per_block, ...) in order; per tile it writes the counts and
// their prefix inside the block, at the end the block's totals.
constexpr int kTileHistThreads = 256;

// BYTES8: 8-bit symbols and 8 levels, so that every byte is a bin: a key
// costs a byte extract, an address and the atomic.
template <typename T, bool BYTES8>
__global__ void __launch_bounds__(kTileHistThreads) tile_hist_kernel(const T* text, uint64_t n, uint32_t levels,
                                                                 uint32_t D, uint32_t tile_keys,
                                                                 uint32_t tiles_per_block, uint32_t block0,
                                                                 unsigned long long* hist, uint32_t* tilecnt,
                                                                 uint32_t* relpre, unsigned long long* blocksum,
                                                                 uint64_t* level0_a, uint64_t* level0_b,
                                                                 uint32_t* status) {
  constexpr int WARPS = kTileHistThreads / 32;
  constexpr int BINS = 256;
  // One counter per (bin, lane) shared by the block's warps: lane k counts
  // into column k, so the 32 lanes of an atomic never meet on an address or
  // a bank, however skewed the text (at most 8 warps x 64 symbols x 16
  // tiles = 8192 per counter).
  __shared__ __align__(16) uint32_t h[BINS * 32];
  __shared__ uint32_t s_tc[BINS / 2];  // runs of the first D <= 7 bits
  const int tid = threadIdx.x;
  for (int i = tid; i < BINS * 32; i += kTileHistThreads) h[i] = 0;
  if (tid < BINS / 2) s_tc[tid] = 0;
  __syncthreads();
  uint32_t* mine = h + (tid & 31);
  const uint32_t bins = 1u << levels, NB = 1u << D, binmask = bins - 1;
  uint32_t prev = 0;  // thread b < bins: the block's count of symbol b so far
  uint32_t rel = 0;   // thread c < NB: the block's count of run c before the current tile
  uint32_t seen = 0;  // OR of the thread's symbols: one >= 2^levels sets a bit above the bins
  const uint32_t block = block0 + blockIdx.x;
  const uint64_t first_tile = uint64_t(block) * tiles_per_block;
  const int lane = tid & 31, warp = tid >> 5;
  const uint32_t l0shift = levels - 1;  // level 0 holds the symbols' top bit
  // Level 0 of the structures (text order, MSB first): word of 64 symbols
  // out of 64 / PER threads' vector bit masks.
  auto store_level0 = [&](uint64_t word_index, uint64_t word) {
    level0_a[word_index] = word;
    if (level0_b) level0_b[word_index] = word;
  };
  auto count = [&](uint32_t c) {
    seen |= c;
    atomicAdd(&mine[(c & binmask) * 32], 1u);  // an out-of-range symbol fails the build below
  };
  constexpr int PER = 16 / sizeof(T);
  // whole aligned tiles of HV 16-byte vectors per thread, loaded one tile
  // ahead so that the loads overlap the counting of the previous tile
  constexpr int HV = 4;
  const uint32_t tile_vecs = uint32_t(tile_keys * sizeof(T) / 16);
  const bool vec = tile_keys * sizeof(T) % (16 * kTileHistThreads) == 0 && tile_vecs <= HV * kTileHistThreads &&
                   (reinterpret_cast<uintptr_t>(text) % 16) == 0;
  const int nv = int(tile_vecs / kTileHistThreads);  // vectors per thread (1..HV)
  auto full_tile = [&](uint64_t tile) { return vec && (tile + 1) * tile_keys <= n; };
  uint4 ahead[HV];
  if (full_tile(first_tile)) {
    const uint4* p = reinterpret_cast<const uint4*>(text + first_tile * tile_keys);
#pragma unroll
    for (int v = 0; v < HV; ++v)
      if (v < nv) ahead[v] = __ldcs(p + tid + v * kTileHistThreads);
  }
  for (uint32_t k = 0; k < tiles_per_block; ++k) {
    const uint64_t tile = first_tile + k;
    const uint64_t start = tile * tile_keys;
    if (start >= n) break;
    const uint64_t len = n - start < tile_keys ? n - start : tile_keys;
    const T* p = text + start;
    if (full_tile(tile)) {
      uint4 cur[HV];
#pragma unroll
      for (int v = 0; v < HV; ++v) cur[v] = ahead[v];
      if (k + 1 < tiles_per_block && full_tile(tile + 1)) {
        const uint4* q = reinterpret_cast<const uint4*>(text + (tile + 1) * tile_keys);
#pragma unroll
        for (int v = 0; v < HV; ++v)
          if (v < nv) ahead[v] = __ldcs(q + tid + v * kTileHistThreads);
      }
      if (level0_a) {
        constexpr int LPC = 32 / PER;  // threads per 32 symbols
#pragma unroll
        for (int v = 0; v < HV; ++v) {
          if (v >= nv) break;
          uint32_t x = vector_bits<T>(cur[v], l0shift) << (32 - PER * (1 + (lane % LPC)));
#pragma unroll
          for (int d = 1; d < LPC; d <<= 1) x |= __shfl_down_sync(0xFFFFFFFFu, x, d);
          const uint32_t lo = __shfl_down_sync(0xFFFFFFFFu, x, LPC);
          if (lane % (2 * LPC) == 0)
            store_level0((start + uint64_t(tid + v * kTileHistThreads) * PER) >> 6, (uint64_t(x) << 32) | lo);
        }
      }
#pragma unroll
      for (int v = 0; v < HV; ++v) {
        if (v >= nv) break;
        if constexpr (BYTES8) {
          const uint32_t w[4] = {cur[v].x, cur[v].y, cur[v].z, cur[v].w};
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int k = 0; k < 4; ++k) atomicAdd(&mine[__byte_perm(w[q], 0u, 0x4440u + k) * 32], 1u);
        } else {
          const T* s = reinterpret_cast<const T*>(&cur[v]);
#pragma unroll
          for (int q = 0; q < PER; ++q) count(uint32_t(s[q]));
        }
      }
    } else {
      const uint64_t nvec = (reinterpret_cast<uintptr_t>(p) % 16 == 0) ? len / PER : 0;
      for (uint64_t i = tid; i < nvec; i += kTileHistThreads) {
        const uint4 x = __ldcs(reinterpret_cast<const uint4*>(p) + i);
        const T* s = reinterpret_cast<const T*>(&x);
#pragma unroll
        for (int q = 0; q < PER; ++q) count(uint32_t(s[q]));
      }
      for (uint64_t i = nvec * PER + tid; i < len; i += kTileHistThreads) count(uint32_t(p[i]));
      if (level0_a) {
        // a word of 64 symbols per warp from two ballots (bit k of a ballot
        // is lane k: reversed, the first symbol is the most significant)
        const uint64_t nw = (len + 63) >> 6;
        for (uint64_t j = warp; j < nw; j += WARPS) {
          const uint64_t i0 = j * 64 + lane, i1 = i0 + 32;
          const bool b0 = i0 < len && ((uint32_t(p[i0]) >> l0shift) & 1u);
          const bool b1 = i1 < len && ((uint32_t(p[i1]) >> l0shift) & 1u);
          const uint32_t hi = __brev(__ballot_sync(0xFFFFFFFFu, b0)), lo = __brev(__ballot_sync(0xFFFFFFFFu, b1));
          if (lane == 0) store_level0((start >> 6) + j, (uint64_t(hi) << 32) | lo);
        }
      }
    }
    __syncthreads();
    if (tid < int(bins)) {
      // row of 32 counters, its 16-byte pieces read in a rotated order so
      // that the 8 threads of a quarter warp hit different banks
      const uint4* row = reinterpret_cast<const uint4*>(h + tid * 32);
      uint32_t tot = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const uint4 r = row[(k + tid) & 7];
        tot += r.x + r.y + r.z + r.w;
      }
      const uint32_t x = tot - prev;
      prev = tot;
      // run of symbol b: its top D bits, first bit least significant
      const uint32_t run = reverse_low_bits(uint32_t(tid) >> (levels - D), D);
      if (x) atomicAdd(&s_tc[run], x);
    }
    __syncthreads();
    if (tid < int(NB)) {
      const uint32_t c = s_tc[tid];
      tilecnt[tile * NB + tid] = c;
      relpre[tile * NB + tid] = rel;
      rel += c;
      s_tc[tid] = 0;
    }
    __syncthreads();
  }
  if (seen >> levels) atomicOr(status, kErrSymbol);
  if (tid < int(NB)) blocksum[uint64_t(block) * NB + tid] = rel;
  if (tid < int(bins) && prev) atomicAdd(&hist[tid], (unsigned long long)prev);
}

// After the tile histogram, one launch of NB + 1 CTAs of 1024 threads:
//  * CTA c < NB: the exclusive prefix, per column c, of the nblocks x NB
//    block totals (in place), each thread a run of up to 4 consecutive
//    blocks (more in a loop for longer texts);
//  * CTA NB: the start table of the first tile pass of a text with levels
//    <= 8 (one segment, the whole text) from the leaf histogram, the entries
//    the host's plan gives that pass: matrix runs of key_j in key order, tree
//    runs in natural prefix order, runs of S_K; tree entries 0 without a
//    tree.  A key_j run is a contiguous range of bins (those with the same
//    j-bit prefix), so its count is a difference of the bins' prefix sums,
//    and the tree's starts are those prefix sums themselves.
template <int W>
__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long v, unsigned long long* wsum,
                                                                   unsigned long long* total) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, d);
    if (lane >= uint32_t(d)) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < uint32_t(W) ? wsum[lane] : 0ull;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, w, d);
      if (lane >= uint32_t(d)) w += y;
    }
    if (lane < uint32_t(W)) wsum[lane] = w;  // inclusive
  }
  __syncthreads();
  if (total) *total = wsum[W - 1];
  return (warp ? wsum[warp - 1] : 0ull) + x - v;
}

__global__ void __launch_bounds__(1024) tile_block_scan_kernel(unsigned long long* blocksum, uint32_t nblocks,
                                                               uint32_t NB, const unsigned long long* hist,
                                                               uint32_t levels, uint32_t K, uint32_t out,
                                                               uint32_t tree, uint64_t* table) {
  __shared__ unsigned long long wsum[32];
  const uint32_t tid = threadIdx.x;
  if (blockIdx.x < NB) {
    const uint32_t c = blockIdx.x;
    const uint32_t per = (nblocks + 1023) / 1024;
    const uint32_t b0 = min(nblocks, tid * per), b1 = min(nblocks, b0 + per);
    unsigned long long v[4] = {0, 0, 0, 0}, sum = 0;
    if (per <= 4) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (b0 + q < b1) v[q] = blocksum[uint64_t(b0 + q) * NB + c];
      sum = v[0] + v[1] + v[2] + v[3];
    } else {
      for (uint32_t b = b0; b < b1; ++b) sum += blocksum[uint64_t(b) * NB + c];
    }
    unsigned long long run = block_exclusive_scan<32>(sum, wsum, nullptr);
    if (per <= 4) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (b0 + q < b1) {
          blocksum[uint64_t(b0 + q) * NB + c] = run;
          run += v[q];
        }
    } else {
      for (uint32_t b = b0; b < b1; ++b) {
        const unsigned long long x = blocksum[uint64_t(b) * NB + c];
        blocksum[uint64_t(b) * NB + c] = run;
        run += x;
      }
    }
    return;
  }
  if (!table) return;
  // prefix sums over the bins in natural order: P[b] = bins before b
  __shared__ unsigned long long P[(1 << kTileGivenMaxLevels) + 1];
  const uint32_t bins = 1u << levels;
  const unsigned long long cnt = tid < bins ? hist[tid] : 0ull;
  unsigned long long total;
  const unsigned long long ex = block_exclusive_scan<32>(cnt, wsum, &total);
  if (tid < bins) P[tid] = ex;
  if (tid == 0) P[bins] = total;
  __syncthreads();
  // warp j: level j (j < K: matrix and tree starts; j == K: runs of S_K)
  const uint32_t warp = tid >> 5, lane = tid & 31;
  if (warp > K || (warp == K && !out)) return;
  const uint32_t j = warp, R = 1u << j, sh = levels - j;
  // key order x: the run of natural prefix p = rev(x); lane takes x = 8 lane + q
  unsigned long long v[8], sum = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const uint32_t x = 8 * lane + q;
    v[q] = 0;
    if (x < R) {
      const uint32_t p = reverse_low_bits(x, j);
      v[q] = P[(p + 1) << sh] - P[p << sh];
    }
    sum += v[q];
  }
  unsigned long long xs = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, xs, d);
    if (lane >= uint32_t(d)) xs += y;
  }
  unsigned long long run = xs - sum;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const uint32_t x = 8 * lane + q;
    if (x < R) {
      if (j < K) {
        table[tile_wm_entry(int(j), int(x))] = run;
        table[tile_wt_entry(int(K), int(j), int(x))] = tree ? P[reverse_low_bits(x, j) << sh] : 0ull;
      } else {
        table[tile_out_entry(int(K), int(x))] = run;
      }
    }
    run += v[q];
  }
}

// Start table of a first tile pass from folded prefix counts: warp j takes
// level j (2^j <= 16 prefixes, a lane each).  Key order x holds the natural
// prefix p = rev(x): the matrix starts are exclusive sums in key order, the
// tree starts exclusive sums in natural order; warp K gives the runs of S_K.
__global__ void __launch_bounds__(160) tile_first_table_kernel(const uint64_t* flat, uint32_t K, uint32_t out,
                                                                uint32_t tree, uint64_t* table) {
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp > K || (warp == K && !out)) return;
  const uint32_t j = warp, R = 1u << j;
  const uint64_t* c = flat + (R - 1);
  const uint32_t p = lane < R ? reverse_low_bits(lane, j) : 0u;
  const unsigned long long in_key = lane < R ? c[p] : 0ull, in_nat = lane < R ? c[lane] : 0ull;
  unsigned long long xk = in_key, xn = in_nat;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long yk = __shfl_up_sync(0xFFFFFFFFu, xk, d);
    const unsigned long long yn = __shfl_up_sync(0xFFFFFFFFu, xn, d);
    if (lane >= uint32_t(d)) {
      xk += yk;
      xn += yn;
    }
  }
  const unsigned long long key_pre = xk - in_key;
  const unsigned long long nat_pre_p = __shfl_sync(0xFFFFFFFFu, xn - in_nat, p);  // natural prefix before p
  if (lane >= R) return;
  if (j < K) {
    table[tile_wm_entry(int(j), int(lane))] = key_pre;
    table[tile_wt_entry(int(K), int(j), int(lane))] = tree ? nat_pre_p : 0ull;
  } else {
    table[tile_out_entry(int(K), int(lane))] = key_pre;
  }
}

// 14..16 levels: the bins split into ranges of 2^15 u32 counters held in
// shared memory (128 KB); grid row r counts the symbols of range r in its
// chunk of the text and adds its nonzero bins to the global histogram.
// Skewed texts keep their hot bins on chip instead of contending in L2.
constexpr int kRangeBins = 1 << 15;
constexpr int kRangeThreads = 1024;

template <typename T>
__global__ void __launch_bounds__(kRangeThreads) leaf_hist_ranges(const T* text, uint64_t n, uint32_t levels,
                                                                 uint64_t chunk, unsigned long long* hist,
                                                                 uint32_t* status) {
  extern __shared__ uint32_t hr[];
  for (int i = threadIdx.x; i < kRangeBins; i += kRangeThreads) hr[i] = 0;
  __syncthreads();
  const uint64_t lo = uint64_t(blockIdx.y) * kRangeBins;
  const uint64_t limit = 1ull << levels;
  const uint64_t b = uint64_t(blockIdx.x) * chunk;
  const uint64_t e = b + chunk < n ? b + chunk : n;
  bool bad = false;
  if (b < e)
    for_each_symbol_vec<T>(text + b, e - b, threadIdx.x, kRangeThreads, [&](uint64_t c) {
      if (c >= limit) { bad = true; return; }
      const uint64_t r = c - lo;
      if (r < kRangeBins) atomicAdd(&hr[r], 1u);
    });
  if (bad && blockIdx.y == 0) atomicOr(status, kErrSymbol);
  __syncthreads();
  for (int i = threadIdx.x; i < kRangeBins; i += kRangeThreads)
    if (hr[i] && lo + i < limit) atomicAdd(&hist[lo + i], (unsigned long long)hr[i]);
}

int hist_grid(uint64_t n, uint32_t width) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  uint64_t per_block = uint64_t(kHistThreads) * (16 / width) * 4;
  uint64_t want = (n + per_block - 1) / per_block;
  uint64_t cap = uint64_t(sms > 0 ? sms : 148) * 4;
  return int(want < 1 ? 1 : (want > cap ? cap : want));
}

template <typename T>
void hist_dispatch(const T* text, uint64_t n, uint32_t levels, unsigned long long* hist, uint32_t* status,
                   cudaStream_t s) {
  int grid = hist_grid(n, sizeof(T));
  if (levels <= 8)
    leaf_hist_smem<T, 256, true><<<grid, kHistThreads, 0, s>>>(text, n, levels, hist, status);
  else if (levels <= 13)
    leaf_hist_smem<T, 8192, false><<<grid, kHistThreads, 0, s>>>(text, n, levels, hist, status);
  else if (levels <= 16) {
    static bool configured = false;
    if (!configured) {
      cudaFuncSetAttribute(leaf_hist_ranges<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRangeBins * 4);
      configured = true;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t ranges = uint32_t(((uint64_t(1) << levels) + kRangeBins - 1) / kRangeBins);
    const uint64_t blocks = std::max<uint64_t>(1, std::min<uint64_t>(uint64_t(sms > 0 ? sms : 148),
                                                                    (n + 65535) / 65536));
    const uint64_t chunk = (((n + blocks - 1) / blocks) + 15) & ~uint64_t(15);  // keeps 16-byte alignment
    dim3 g(unsigned((n + chunk - 1) / chunk), ranges);
    leaf_hist_ranges<T><<<g, kRangeThreads, kRangeBins * 4, s>>>(text, n, levels, chunk, hist, status);
  } else
    leaf_hist_global<T><<<grid, kHistThreads, 0, s>>>(text, n, levels, hist, status);
}

// ---------------------------------------------------------------------------
// Tree level from the matrix level: one thread per output word gathers the
// bit ranges of the prefix groups that cover it.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t bits_at(const uint64_t* level, uint64_t src, uint32_t take) {
  // `take` (1..64) bits starting at bit position src, left-aligned.
  const uint64_t w = src >> 6;
  const uint32_t sh = uint32_t(src & 63);
  uint64_t v = level[w] << sh;
  if (sh != 0 && sh + take > 64) v |= level[w + 1] >> (64 - sh);
  return take == 64 ? v : (v & ~(~0ull >> take));
}

constexpr int kRegroupWords = 8;  // consecutive output words per thread

__global__ void regroup_kernel(const uint64_t* __restrict__ matrix_level, uint64_t* __restrict__ tree_level,
                               uint64_t nbits, const uint64_t* __restrict__ seg_tree,
                               const uint64_t* __restrict__ seg_matrix, uint64_t nseg, uint32_t* status) {
  const uint64_t nwords = (nbits + 63) >> 6;
  const uint64_t first = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) * kRegroupWords;
  if (first >= nwords) return;
  // last segment starting at or before the first bit of this thread
  uint64_t lo = 0, hi = nseg;
  const uint64_t p0 = first << 6;
  while (hi - lo > 1) {
    const uint64_t mid = (lo + hi) >> 1;
    if (seg_tree[mid] <= p0) lo = mid; else hi = mid;
  }
  uint64_t seg = lo;
  uint64_t seg_start = seg_tree[seg];
  uint64_t seg_end = seg + 1 < nseg ? seg_tree[seg + 1] : nbits;
  const uint64_t last = min(nwords, first + kRegroupWords);
  for (uint64_t w = first; w < last; ++w) {
    const uint64_t wp = w << 6, end = min(wp + 64, nbits);
    uint64_t pos = wp, acc = 0;
    while (pos < end) {
      if (pos >= seg_end) {
        // the last segment starting at or before pos, searched from the next
        // one by galloping (runs of empty segments cost their logarithm)
        uint64_t a = seg + 1, b = a + 1, step = 1;  // seg_tree[a] == seg_end <= pos
        while (b < nseg && seg_tree[b] <= pos) {
          a = b;
          step <<= 1;
          b = a + step;
        }
        b = min(b, nseg);
        while (b - a > 1) {
          const uint64_t mid = (a + b) >> 1;
          if (seg_tree[mid] <= pos) a = mid; else b = mid;
        }
        seg = a;
        seg_start = seg_tree[seg];
        seg_end = seg + 1 < nseg ? seg_tree[seg + 1] : nbits;
      }
      const uint64_t stop = min(end, seg_end);
      const uint32_t take = uint32_t(stop - pos);
      const uint64_t src = seg_matrix[seg] + (pos - seg_start);
      if (src + take > nbits) {  // inconsistent segments: never read out of range
        atomicOr(status, kErrBounds);
        break;
      }
      acc |= bits_at(matrix_level, src, take) >> (pos - wp);
      pos = stop;
    }
    tree_level[w] = acc;
  }
}

// The same for levels of many small (or empty) segments: one thread per tree
// bit, each searching its segment on its own, so that no thread walks a long
// chain of segments.  A warp covers 32 consecutive bits (one half of a word,
// written as the word's upper or lower 32 bits); the grid covers every word.
__global__ void __launch_bounds__(256) regroup_bits_kernel(const uint64_t* __restrict__ matrix_level,
                                                           uint32_t* __restrict__ tree_halves, uint64_t nbits,
                                                           const uint64_t* __restrict__ seg_tree,
                                                           const uint64_t* __restrict__ seg_matrix, uint64_t nseg,
                                                           uint32_t* status) {
  const uint64_t pos = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  bool bit = false;
  if (pos < nbits) {
    uint64_t lo = 0, hi = nseg;
    while (hi - lo > 1) {
      const uint64_t mid = (lo + hi) >> 1;
      if (seg_tree[mid] <= pos) lo = mid; else hi = mid;
    }
    const uint64_t src = seg_matrix[lo] + (pos - seg_tree[lo]);
    if (src >= nbits) atomicOr(status, kErrBounds);  // inconsistent segments: never read out of range
    else bit = (matrix_level[src >> 6] >> (63 - (src & 63))) & 1u;
  }
  const uint32_t m = __ballot_sync(0xFFFFFFFFu, bit);
  // bits pos..pos+31 of a word are its upper half when pos % 64 < 32
  // (the first bit of a word is its most significant)
  if ((threadIdx.x & 31) == 0) tree_halves[2 * (pos >> 6) + ((pos & 32) ? 0 : 1)] = __brev(m);
}

// ---- every pass's digit counts from the prefix counts ---------------------------
// digits[16 p + r]: the symbols whose bits of levels l..l+K-1 of pass p
// (level l's most significant) read r: the natural prefix counts of level
// l+K summed by their last K bits.  Blocks take chunks of kDigitChunk counts
// of one pass; a thread's counts share one residue (the stride is a multiple
// of 16), lanes 16 apart share it too.
constexpr uint32_t kDigitThreads = 256, kDigitChunk = kDigitThreads * 16;

struct FlatDigitPlan {
  uint32_t count;
  uint32_t top[kPassDigitsMaxPasses];  // level l+K of each pass
  uint32_t K[kPassDigitsMaxPasses];
  uint32_t chunk0[kPassDigitsMaxPasses + 1];
};

__global__ void __launch_bounds__(kDigitThreads) flat_digits_kernel(const uint64_t* __restrict__ flat,
                                                                    FlatDigitPlan p,
                                                                    unsigned long long* __restrict__ digits) {
  __shared__ unsigned long long s_d[16];
  uint32_t i = 0;
  while (i + 1 < p.count && p.chunk0[i + 1] <= blockIdx.x) ++i;
  if (threadIdx.x < 16) s_d[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t ne = 1ull << p.top[i];
  const uint64_t* c = flat + (ne - 1);
  const uint64_t x0 = uint64_t(blockIdx.x - p.chunk0[i]) * kDigitChunk + threadIdx.x;
  uint64_t v = 0;
#pragma unroll 4
  for (uint32_t k = 0; k < kDigitChunk / kDigitThreads; ++k) {
    const uint64_t x = x0 + uint64_t(k) * kDigitThreads;
    if (x < ne) v += c[x];
  }
  v += __shfl_xor_sync(0xFFFFFFFFu, v, 16);
  const uint32_t mask = (1u << p.K[i]) - 1u;
  if ((threadIdx.x & 31) < 16 && v) atomicAdd(&s_d[threadIdx.x & mask], (unsigned long long)v);
  __syncthreads();
  if (threadIdx.x <= mask && s_d[threadIdx.x]) atomicAdd(&digits[16 * i + threadIdx.x], s_d[threadIdx.x]);
}

// ---- the regroup's segments, on the device -------------------------------------
// Level m of the tree holds the groups of the m-bit natural prefixes in
// natural order; the matrix level holds the same groups in key order (the
// prefix bit-reversed, as pwm's matrix orders level m by the bit of level m-1
// first); both keep text order inside a group.  So group p starts in the tree
// at the exclusive prefix of the level's counts in natural order, and in the
// matrix at the exclusive prefix, in key order, at rev_m(p).  Blocks take
// chunks of kSegChunk groups of every listed level: chunk sums, then each
// level's chunk offsets, then the starts.
constexpr uint32_t kSegThreads = 256, kSegPer = 8, kSegChunk = kSegThreads * kSegPer;
constexpr uint32_t kSegMaxLevels = 32;

struct RegroupSegPlan {
  uint32_t count;
  uint32_t m[kSegMaxLevels];
  uint32_t chunk0[kSegMaxLevels + 1];  // first block of each level; chunk0[count]: all blocks
  uint64_t out[kSegMaxLevels];         // tree starts at out[i], matrix starts at out[i] + 2^m
};

__device__ __forceinline__ uint32_t seg_rev(uint32_t x, uint32_t m) { return __brev(x) >> (32 - m); }

__device__ __forceinline__ uint32_t seg_level_of(const RegroupSegPlan& p, uint32_t b) {
  uint32_t i = 0;
  while (i + 1 < p.count && p.chunk0[i + 1] <= b) ++i;
  return i;
}

// Exclusive scan of the pairs (a, b) over the block, in place; ta, tb: totals.
__device__ __forceinline__ void seg_block_scan(uint64_t& a, uint64_t& b, uint64_t& ta, uint64_t& tb) {
  __shared__ uint64_t wa[kSegThreads / 32], wb[kSegThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t ia = a, ib = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t ya = __shfl_up_sync(0xFFFFFFFFu, ia, o), yb = __shfl_up_sync(0xFFFFFFFFu, ib, o);
    if (lane >= o) {
      ia += ya;
      ib += yb;
    }
  }
  if (lane == 31) {
    wa[warp] = ia;
    wb[warp] = ib;
  }
  __syncthreads();
  uint64_t oa = 0, ob = 0;
  ta = tb = 0;
#pragma unroll
  for (int w = 0; w < int(kSegThreads / 32); ++w) {
    if (w < warp) {
      oa += wa[w];
      ob += wb[w];
    }
    ta += wa[w];
    tb += wb[w];
  }
  a = oa + ia - a;
  b = ob + ib - b;
  __syncthreads();  // wa, wb free for the next call
}

__global__ void __launch_bounds__(kSegThreads) regroup_seg_sums_kernel(const uint64_t* __restrict__ flat,
                                                                       RegroupSegPlan p, uint64_t* __restrict__ sums) {
  const uint32_t i = seg_level_of(p, blockIdx.x);
  const uint32_t m = p.m[i];
  const uint64_t ng = 1ull << m;
  const uint64_t* c = flat + (ng - 1);
  const uint64_t x0 = uint64_t(blockIdx.x - p.chunk0[i]) * kSegChunk + threadIdx.x * kSegPer;
  uint64_t a = 0, b = 0;
#pragma unroll
  for (uint32_t k = 0; k < kSegPer; ++k) {
    const uint64_t x = x0 + k;
    if (x < ng) {
      a += c[x];
      b += c[seg_rev(uint32_t(x), m)];
    }
  }
  uint64_t ta, tb;
  seg_block_scan(a, b, ta, tb);
  if (threadIdx.x == 0) {
    sums[2 * uint64_t(blockIdx.x)] = ta;
    sums[2 * uint64_t(blockIdx.x) + 1] = tb;
  }
}

// One block per level: its chunk sums become exclusive chunk offsets.
__global__ void __launch_bounds__(kSegThreads) regroup_seg_offsets_kernel(RegroupSegPlan p,
                                                                          uint64_t* __restrict__ sums) {
  const uint32_t c0 = p.chunk0[blockIdx.x], c1 = p.chunk0[blockIdx.x + 1];
  uint64_t carry_a = 0, carry_b = 0;
  for (uint32_t base = c0; base < c1; base += kSegThreads) {
    const uint32_t k = base + threadIdx.x;
    uint64_t a = k < c1 ? sums[2 * uint64_t(k)] : 0, b = k < c1 ? sums[2 * uint64_t(k) + 1] : 0;
    uint64_t ta, tb;
    seg_block_scan(a, b, ta, tb);
    if (k < c1) {
      sums[2 * uint64_t(k)] = carry_a + a;
      sums[2 * uint64_t(k) + 1] = carry_b + b;
    }
    carry_a += ta;
    carry_b += tb;
  }
}

__global__ void __launch_bounds__(kSegThreads) regroup_seg_write_kernel(const uint64_t* __restrict__ flat,
                                                                        RegroupSegPlan p,
                                                                        const uint64_t* __restrict__ sums,
                                                                        uint64_t* __restrict__ out) {
  const uint32_t i = seg_level_of(p, blockIdx.x);
  const uint32_t m = p.m[i];
  const uint64_t ng = 1ull << m;
  const uint64_t* c = flat + (ng - 1);
  uint64_t* st = out + p.out[i];
  uint64_t* sm = st + ng;
  const uint64_t x0 = uint64_t(blockIdx.x - p.chunk0[i]) * kSegChunk + threadIdx.x * kSegPer;
  uint64_t va[kSegPer], vb[kSegPer], a = 0, b = 0;
#pragma unroll
  for (uint32_t k = 0; k < kSegPer; ++k) {
    const uint64_t x = x0 + k;
    va[k] = x < ng ? c[x] : 0;
    vb[k] = x < ng ? c[seg_rev(uint32_t(x), m)] : 0;
    a += va[k];
    b += vb[k];
  }
  uint64_t ta, tb;
  seg_block_scan(a, b, ta, tb);
  a += sums[2 * uint64_t(blockIdx.x)];
  b += sums[2 * uint64_t(blockIdx.x) + 1];
#pragma unroll
  for (uint32_t k = 0; k < kSegPer; ++k) {
    const uint64_t x = x0 + k;
    if (x < ng) {
      st[x] = a;                         // group x (natural) in the tree
      sm[seg_rev(uint32_t(x), m)] = b;  // group rev(x), key position x, in the matrix
    }
    a += va[k];
    b += vb[k];
  }
}

// ---------------------------------------------------------------------------
// Huffman code keys
// ---------------------------------------------------------------------------
// Key of symbol c with code (word, len), L the longest code: the code
// followed by a stop bit, ((word << 1) | 1) << (L - len), in L + 1 <= 8 *
// sizeof(K) bits (split.cuh HuffKeys).
template <typename T, typename K>
__global__ void huffman_keys_kernel(const T* text, uint64_t n, const uint64_t* code_len, const uint64_t* code_word,
                                    uint64_t ncodes, uint32_t L, K* keys, uint32_t* status) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t c = uint64_t(text[i]);
    uint64_t len = c < ncodes ? code_len[c] : 0;
    if (len == 0 || len > L) {
      atomicOr(status, kErrSymbol);
      keys[i] = K(0);
      continue;
    }
    keys[i] = K(((uint64_t(code_word[c]) << 1) | 1u) << (L - len));
  }
}

// First occurrence of every symbol: an atomicMin only where the index is
// below the value already there, read with a plain (L1-cacheable) load, so
// that the hot symbols, whose first occurrence the early blocks set, cost
// neither atomics nor L2 traffic.  A stale cached value is never below the
// current one (values only decrease), so it costs at most an extra atomic.
template <typename T>
__global__ void first_occurrence_kernel(const T* text, uint64_t n, unsigned long long* first) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    unsigned long long* f = &first[uint64_t(text[i])];
    if (i < *f) atomicMin(f, (unsigned long long)i);
  }
}

template <typename T>
__global__ void symbol_hist_kernel(const T* text, uint64_t n, uint64_t nsym, unsigned long long* hist,
                                   unsigned long long* first) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t c = uint64_t(text[i]);
    if (c < nsym) {
      atomicAdd(&hist[c], 1ull);
      if (first) atomicMin(&first[c], (unsigned long long)i);
    }
  }
}

// n words and a status word into host-mapped memory: small results the host
// waits for, written by the SMs instead of a copy engine, so that they do not
// queue behind bulk downloads.
// Matrix-only builds of more than 8 levels need, per pass, only the counts
// of its natural K-bit digit (the bits of its levels, the first most
// significant), not a leaf histogram of 2^L bins.  Each thread counts into
// its own column of (pass, digit) counters (counter (e, lane) at e * 32 +
// lane: the lanes of an atomic never share a bank), a CTA adds its totals to
// `digits` in global memory, and the last CTA to finish writes, into mapped
// host memory, the natural prefix counts of levels 0..K0 (flat: level m at
// 2^m - 1; the first pass's start table reads them), the zero bits of every
// level, the status word and the digit counts.
// NP: the passes' count bound, so that the per-symbol loop over the passes
// unrolls (6 covers every text up to 24 levels in passes of 4).
template <int NP>
__global__ void __launch_bounds__(256) pass_digits_kernel(const unsigned char* __restrict__ text, uint64_t n,
                                                          uint32_t width, PassDigitsArgs pd,
                                                          unsigned long long* digits, unsigned int* done,
                                                          uint32_t* status, uint64_t* out) {
  extern __shared__ uint32_t dcnt[];  // [npasses * 16][32]
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  const uint32_t ncnt = pd.npasses * 16;
  for (uint32_t i = tid; i < ncnt * 32; i += blockDim.x) dcnt[i] = 0;
  __syncthreads();
  const uint32_t base = uint32_t(__cvta_generic_to_shared(dcnt)) + lane * 4;
  // a symbol >= 2^L sets a bit of `seen` at or above L (its digits still
  // count, into counters whose values the failed build never uses)
  uint32_t seen = 0;
  uint32_t lo[NP], mask[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    lo[p] = p < int(pd.npasses) ? pd.lo[p] : 0u;
    mask[p] = p < int(pd.npasses) ? pd.mask[p] : 0u;
  }
  auto count = [&](uint32_t x) {
    seen |= x;
#pragma unroll
    for (int p = 0; p < NP; ++p)
      if (p < int(pd.npasses))
        asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(base + ((uint32_t(p) * 16 + ((x >> lo[p]) & mask[p])) << 7))
                     : "memory");
  };
  // 16-byte vectors between the unaligned ends of the text
  const uint32_t E = 16 / width;
  const uint64_t head = min(n, uint64_t((16u - (reinterpret_cast<uintptr_t>(text) & 15u)) & 15u) / width);
  const uint64_t nv = (n - head) / E;
  auto sym = [&](uint64_t i) {
    return width == 1 ? uint32_t(text[i]) : width == 2 ? uint32_t(reinterpret_cast<const uint16_t*>(text)[i])
                                                       : reinterpret_cast<const uint32_t*>(text)[i];
  };
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x, gid = uint64_t(blockIdx.x) * blockDim.x + tid;
  if (gid < head) count(sym(gid));
  const uint4* v = reinterpret_cast<const uint4*>(text + head * width);
  for (uint64_t k = gid; k < nv; k += stride) {
    const uint4 x = __ldcs(v + k);
    const uint32_t w[4] = {x.x, x.y, x.z, x.w};
    if (width == 1) {
#pragma unroll
      for (int e = 0; e < 16; ++e) count((w[e >> 2] >> (8 * (e & 3))) & 0xFFu);
    } else if (width == 2) {
#pragma unroll
      for (int e = 0; e < 8; ++e) count((w[e >> 1] >> (16 * (e & 1))) & 0xFFFFu);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) count(w[e]);
    }
  }
  for (uint64_t i = head + nv * E + gid; i < n; i += stride) count(sym(i));
  if (pd.L < 32 && (seen >> pd.L)) atomicOr(status, kErrSymbol);
  __syncthreads();
  for (uint32_t e = tid; e < ncnt; e += blockDim.x) {
    uint32_t sum = 0;
    for (uint32_t l = 0; l < 32; ++l) sum += dcnt[e * 32 + ((l + e) & 31)];
    if (sum) atomicAdd(&digits[e], (unsigned long long)sum);
  }
  __threadfence();
  __syncthreads();
  __shared__ bool last;
  if (tid == 0) last = atomicAdd(done, 1u) + 1 == gridDim.x;
  __syncthreads();
  if (!last) return;
  __threadfence();
  const volatile unsigned long long* dg = digits;
  // flat natural prefix counts of levels 0..K0 (the first pass, from level 0)
  const uint32_t K0 = pd.K[0];
  uint64_t* flat = out;
  for (uint32_t i = tid; i < (2u << K0) - 1; i += blockDim.x) {
    const uint32_t m = 31 - __clz(i + 1), q = i + 1 - (1u << m);  // level m, prefix q
    unsigned long long c = 0;
    for (uint32_t d = 0; d < (1u << K0); ++d)
      if ((d >> (K0 - m)) == q) c += dg[d];
    flat[i] = c;
  }
  uint64_t* zeros = out + (2u << K0) - 1;
  for (uint32_t p = 0; p < pd.npasses; ++p)
    for (uint32_t j = tid; j < pd.K[p]; j += blockDim.x) {
      unsigned long long z = 0;
      for (uint32_t d = 0; d < (1u << pd.K[p]); ++d)
        if (!((d >> (pd.K[p] - 1 - j)) & 1u)) z += dg[p * 16 + d];
      zeros[pd.level[p] + j] = z;
    }
  uint64_t* rest = zeros + pd.L;
  if (tid == 0) rest[0] = *static_cast<volatile uint32_t*>(status);
  for (uint32_t e = tid; e < ncnt; e += blockDim.x) rest[1 + e] = dg[e];
}

__global__ void readback_kernel(const unsigned long long* src, uint64_t n, const uint32_t* status, uint64_t* dst) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    dst[i] = src[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) dst[n] = status ? *status : 0u;
}

// Natural-prefix counts of every level from the leaf histogram, flat (level
// m's 2^m counts at offset 2^m - 1), and the zero bits of every level
// (zeros[m]: the counts of the even prefixes of level m + 1).  One launch
// folds level `top` (read from `leaves`, and then copied to the flat array,
// or from the flat array) `down` <= 10 levels down; a block takes 1024
// entries of level top, halves them `down` times in shared memory and adds
// its even entries of each level into zeros with one atomic per level.
__global__ void __launch_bounds__(256) fold_levels_kernel(uint64_t* flat, uint64_t* flat_dev,
                                                          const unsigned long long* leaves, uint32_t top,
                                                          uint32_t down, unsigned long long* zeros) {
  __shared__ uint64_t v[1024];
  __shared__ unsigned long long s_even;
  const uint64_t n_top = 1ull << top;
  const uint64_t base = uint64_t(blockIdx.x) * 1024;
  const uint64_t* src = leaves ? reinterpret_cast<const uint64_t*>(leaves) : (flat_dev ? flat_dev : flat) + (n_top - 1);
  for (int i = threadIdx.x; i < 1024; i += 256) {
    const uint64_t x = base + i < n_top ? src[base + i] : 0;
    v[i] = x;
    if (leaves && base + i < n_top) {
      flat[n_top - 1 + base + i] = x;
      if (flat_dev) flat_dev[n_top - 1 + base + i] = x;
    }
  }
  __syncthreads();
  for (uint32_t d = 1; d <= down; ++d) {
    const uint32_t k = 1024u >> d;  // entries of level top - d in this block
    if (threadIdx.x == 0) s_even = 0;
    __syncthreads();
    uint64_t sums[2], even = 0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const uint32_t i = threadIdx.x + 256u * r;
      sums[r] = i < k ? v[2 * i] + v[2 * i + 1] : 0;
      even += i < k ? v[2 * i] : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) even += __shfl_xor_sync(0xFFFFFFFFu, even, o);
    if ((threadIdx.x & 31) == 0 && even) atomicAdd(&s_even, (unsigned long long)even);
    __syncthreads();  // every read of the level above is done
    const uint32_t m = top - d;
    const uint64_t n_m = 1ull << m, b_m = base >> d;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const uint32_t i = threadIdx.x + 256u * r;
      if (i < k) {
        v[i] = sums[r];
        if (b_m + i < n_m) {
          flat[n_m - 1 + b_m + i] = sums[r];
          if (flat_dev) flat_dev[n_m - 1 + b_m + i] = sums[r];
        }
      }
    }
    if (threadIdx.x == 0 && s_even) atomicAdd(&zeros[m], s_even);
    __syncthreads();
  }
}

// 40-bit symbols (pwm's uint40_t: 5 little-endian bytes, packed) widened to
// 32 bits; a value of 2^32 or more becomes 0xFFFFFFFF, which the histogram
// rejects as a symbol past the levels (at most 24).
__global__ void widen40_kernel(const uint8_t* in, uint64_t n, uint32_t* out) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint8_t* r = in + 5 * i;
    const uint32_t v = uint32_t(r[0]) | (uint32_t(r[1]) << 8) | (uint32_t(r[2]) << 16) | (uint32_t(r[3]) << 24);
    out[i] = r[4] ? 0xFFFFFFFFu : v;
  }
}

// Alphabet reduction of arbitrary 32- and 40-bit symbols: an open-addressing
// hash table (power-of-two capacity, at least twice the text) keyed by the
// symbol, each slot keeping the symbol's first position.  Probing is linear
// and bounded by the capacity; a table that fills up sets the status.
__device__ __forceinline__ uint64_t symbol_at(const uint8_t* text, uint32_t width, uint64_t i) {
  if (width == 4) return reinterpret_cast<const uint32_t*>(text)[i];
  const uint8_t* r = text + 5 * i;  // 40-bit: 5 little-endian bytes
  return uint64_t(r[0]) | (uint64_t(r[1]) << 8) | (uint64_t(r[2]) << 16) | (uint64_t(r[3]) << 24) |
         (uint64_t(r[4]) << 32);
}
__device__ __forceinline__ uint64_t slot_hash(uint64_t v) {  // splitmix64 finaliser
  v ^= v >> 30;
  v *= 0xbf58476d1ce4e5b9ull;
  v ^= v >> 27;
  v *= 0x94d049bb133111ebull;
  return v ^ (v >> 31);
}
constexpr uint64_t kEmptySlot = ~0ull;  // no symbol has 64 bits

__global__ void alphabet_insert_kernel(const uint8_t* text, uint32_t width, uint64_t n, unsigned long long* keys,
                                       unsigned long long* first, uint64_t mask, uint32_t* status) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t v = symbol_at(text, width, i);
    uint64_t h = slot_hash(v) & mask;
    bool placed = false;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
      // a slot, once set, never changes: a value read past L1 is final unless
      // empty, and then the CAS decides (its return value, not a re-read)
      unsigned long long k = *reinterpret_cast<volatile unsigned long long*>(&keys[h]);
      if (k == kEmptySlot) {
        const unsigned long long old = atomicCAS(&keys[h], kEmptySlot, (unsigned long long)v);
        k = old == kEmptySlot ? v : old;
      }
      if (k == v) {
        // first positions only decrease, so a stale value costs an extra atomic at most
        if (i < first[h]) atomicMin(&first[h], (unsigned long long)i);
        placed = true;
        break;
      }
      h = (h + 1) & mask;
    }
    if (!placed) atomicOr(status, kErrBounds);
  }
}

// The occupied slots, compacted: (slot, symbol, first position) per distinct symbol.
__global__ void alphabet_collect_kernel(const unsigned long long* keys, const unsigned long long* first, uint64_t cap,
                                        unsigned long long* count, uint64_t* out) {
  for (uint64_t h = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; h < cap; h += uint64_t(gridDim.x) * blockDim.x) {
    if (keys[h] == kEmptySlot) continue;
    const unsigned long long k = atomicAdd(count, 1ull);
    out[3 * k] = h;
    out[3 * k + 1] = keys[h];
    out[3 * k + 2] = first[h];
  }
}

// Each symbol replaced by its slot's id, written in the text's width.
__global__ void alphabet_remap_kernel(const uint8_t* text, uint32_t width, uint64_t n, const unsigned long long* keys,
                                      const uint32_t* ids, uint64_t mask, uint8_t* out, uint32_t* status) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t v = symbol_at(text, width, i);
    uint64_t h = slot_hash(v) & mask;
    uint32_t id = 0;
    bool found = false;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
      const unsigned long long k = keys[h];
      if (k == v) {
        id = ids[h];
        found = true;
        break;
      }
      if (k == kEmptySlot) break;
      h = (h + 1) & mask;
    }
    if (!found) atomicOr(status, kErrBounds);
    if (width == 4) {
      reinterpret_cast<uint32_t*>(out)[i] = id;
    } else {
      uint8_t* r = out + 5 * i;
      r[0] = uint8_t(id);
      r[1] = uint8_t(id >> 8);
      r[2] = uint8_t(id >> 16);
      r[3] = uint8_t(id >> 24);
      r[4] = 0;
    }
  }
}

__global__ void scatter_ids_kernel(const uint64_t* slots, const uint32_t* ids, uint64_t count, uint32_t* slot_ids) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += uint64_t(gridDim.x) * blockDim.x)
    slot_ids[slots[i]] = ids[i];
}

// Largest symbol of a 32-bit text (warp maxima, one atomic per warp).
__global__ void max_symbol_kernel(const uint32_t* text, uint64_t n, unsigned int* out) {
  uint32_t m = 0;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    m = max(m, text[i]);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, d));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// out[i] = map[text[i]] (pwm's reduce_alphabet renumbering); symbols past the
// map set the status and write 0.
template <typename T>
__global__ void remap_kernel(const T* text, uint64_t n, const uint32_t* map, uint64_t nmap, T* out,
                             uint32_t* status) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t c = uint64_t(text[i]);
    if (c < nmap) {
      out[i] = T(map[c]);
    } else {
      atomicOr(status, kErrSymbol);
      out[i] = T(0);
    }
  }
}

// ---------------------------------------------------------------------------
// Generators (gen.hpp)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void generate_kernel(int dist, uint64_t key, uint64_t param, uint64_t n, T* out, const uint64_t* thr,
                                uint32_t nthr, const uint32_t* perm) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    out[i] = T(gen_value(dist, key, param, i, thr, nthr, perm));
}

int grid_for(uint64_t n, int threads) {
  uint64_t b = (n + threads - 1) / threads;
  if (b > 4096) b = 4096;
  return int(b < 1 ? 1 : b);
}

}  // namespace

uint32_t tile_hist_tiles_per_block() { return 16; }

uint32_t tile_hist_blocks(uint64_t n, uint32_t tile_keys) {
  const uint64_t tiles = (n + tile_keys - 1) / tile_keys;
  return uint32_t((tiles + tile_hist_tiles_per_block() - 1) / tile_hist_tiles_per_block());
}

void launch_tile_histogram_blocks(const void* text, uint64_t n, uint32_t width, uint32_t levels, uint32_t D,
                                  uint32_t tile_keys, uint32_t block0, uint32_t nblk, unsigned long long* hist,
                                  uint32_t* tilecnt, uint32_t* relpre, unsigned long long* blocksum,
                                  uint64_t* level0_a, uint64_t* level0_b, uint32_t* status, cudaStream_t s,
                                  uint64_t* launches) {
  if (n == 0 || nblk == 0) return;
  const uint32_t per = tile_hist_tiles_per_block();
#define PWMGPU_TH(T, B8)                                                                                       \
  tile_hist_kernel<T, B8><<<nblk, kTileHistThreads, 0, s>>>(static_cast<const T*>(text), n, levels, D, tile_keys, \
                                                            per, block0, hist, tilecnt, relpre, blocksum,       \
                                                            level0_a, level0_b, status)
  if (width == 1 && levels == 8) PWMGPU_TH(uint8_t, true);
  else if (width == 1) PWMGPU_TH(uint8_t, false);
  else if (width == 2) PWMGPU_TH(uint16_t, false);
  else PWMGPU_TH(uint32_t, false);
#undef PWMGPU_TH
  ++*launches;
}

void launch_tile_block_scan(unsigned long long* blocksum, uint32_t nblocks, uint32_t D, const unsigned long long* hist,
                            uint32_t levels, uint32_t K, bool out, bool tree, uint64_t* table, cudaStream_t s,
                            uint64_t* launches) {
  if (nblocks == 0) return;
  tile_block_scan_kernel<<<(1u << D) + (table ? 1u : 0u), 1024, 0, s>>>(blocksum, nblocks, 1u << D, hist, levels, K,
                                                                        out ? 1u : 0u, tree ? 1u : 0u, table);
  ++*launches;
}

void launch_tile_first_table(const uint64_t* flat, uint32_t K, bool out, bool tree, uint64_t* table, cudaStream_t s,
                             uint64_t* launches) {
  tile_first_table_kernel<<<1, 32 * (K + 1), 0, s>>>(flat, K, out ? 1u : 0u, tree ? 1u : 0u, table);
  ++*launches;
}

void launch_leaf_histogram(const void* text, uint64_t n, uint32_t width, uint32_t levels, unsigned long long* hist,
                           uint32_t* status, cudaStream_t s, uint64_t* launches) {
  if (n == 0) return;
  switch (width) {
    case 1: hist_dispatch(static_cast<const uint8_t*>(text), n, levels, hist, status, s); break;
    case 2: hist_dispatch(static_cast<const uint16_t*>(text), n, levels, hist, status, s); break;
    default: hist_dispatch(static_cast<const uint32_t*>(text), n, levels, hist, status, s); break;
  }
  ++*launches;
}

void launch_regroup(const uint64_t* matrix_level, uint64_t* tree_level, uint64_t nbits, const uint64_t* seg_tree,
                    const uint64_t* seg_matrix, uint64_t nseg, uint32_t* status, cudaStream_t s, uint64_t* launches) {
  const uint64_t nwords = (nbits + 63) >> 6;
  if (nwords == 0) return;
  if (nseg * 64 > nbits && nbits <= (uint64_t(1) << 22)) {  // groups of under 64 bits on average
    regroup_bits_kernel<<<unsigned((nwords * 64 + 255) / 256), 256, 0, s>>>(
        matrix_level, reinterpret_cast<uint32_t*>(tree_level), nbits, seg_tree, seg_matrix, nseg, status);
    ++*launches;
    return;
  }
  const uint64_t threads = (nwords + kRegroupWords - 1) / kRegroupWords;
  regroup_kernel<<<unsigned((threads + 255) / 256), 256, 0, s>>>(matrix_level, tree_level, nbits, seg_tree, seg_matrix,
                                                                 nseg, status);
  ++*launches;
}

bool launch_flat_digits(const uint64_t* flat, uint32_t L, const uint32_t* level, const uint32_t* K, uint32_t count,
                        unsigned long long* digits, cudaStream_t s, uint64_t* launches) {
  if (count == 0) return true;
  if (count > kPassDigitsMaxPasses) return false;
  FlatDigitPlan p{};
  p.count = count;
  uint64_t blocks = 0;
  for (uint32_t i = 0; i < count; ++i) {
    if (K[i] < 1 || K[i] > 4 || level[i] + K[i] > L || L > 31) return false;
    p.top[i] = level[i] + K[i];
    p.K[i] = K[i];
    p.chunk0[i] = uint32_t(blocks);
    blocks += ((uint64_t(1) << p.top[i]) + kDigitChunk - 1) / kDigitChunk;
  }
  p.chunk0[count] = uint32_t(blocks);
  if (cudaMemsetAsync(digits, 0, size_t(count) * 16 * 8, s) != cudaSuccess) return false;
  flat_digits_kernel<<<unsigned(blocks), kDigitThreads, 0, s>>>(flat, p, digits);
  ++*launches;
  return true;
}

static uint64_t regroup_seg_chunks(uint32_t m) { return ((uint64_t(1) << m) + kSegChunk - 1) / kSegChunk; }

uint64_t regroup_segs_offset(const uint32_t* levels, uint32_t i) {
  uint64_t o = 0;
  for (uint32_t k = 0; k < i; ++k) o += uint64_t(2) << levels[k];
  return o;
}

uint64_t regroup_segs_words(const uint32_t* levels, uint32_t count) { return regroup_segs_offset(levels, count); }

uint64_t regroup_segs_scratch_words(const uint32_t* levels, uint32_t count) {
  uint64_t c = 0;
  for (uint32_t k = 0; k < count; ++k) c += regroup_seg_chunks(levels[k]);
  return 2 * c;
}

bool launch_regroup_segs(const uint64_t* flat, const uint32_t* levels, uint32_t count, uint64_t* out,
                         uint64_t* scratch, cudaStream_t s, uint64_t* launches) {
  if (count == 0) return true;
  if (count > kSegMaxLevels) return false;
  RegroupSegPlan p{};
  p.count = count;
  uint64_t blocks = 0;
  for (uint32_t k = 0; k < count; ++k) {
    if (levels[k] < 1 || levels[k] > 31) return false;
    p.m[k] = levels[k];
    p.chunk0[k] = uint32_t(blocks);
    p.out[k] = regroup_segs_offset(levels, k);
    blocks += regroup_seg_chunks(levels[k]);
  }
  if (blocks >= (uint64_t(1) << 31)) return false;
  p.chunk0[count] = uint32_t(blocks);
  regroup_seg_sums_kernel<<<unsigned(blocks), kSegThreads, 0, s>>>(flat, p, scratch);
  regroup_seg_offsets_kernel<<<count, kSegThreads, 0, s>>>(p, scratch);
  regroup_seg_write_kernel<<<unsigned(blocks), kSegThreads, 0, s>>>(flat, p, scratch, out);
  *launches += 3;
  return true;
}

template <typename T, typename K>
void launch_hk(const void* text, uint64_t n, const uint64_t* code_len, const uint64_t* code_word, uint64_t ncodes,
               uint32_t L, void* keys, uint32_t* status, cudaStream_t s) {
  huffman_keys_kernel<T, K><<<grid_for(n, 256), 256, 0, s>>>(static_cast<const T*>(text), n, code_len, code_word,
                                                             ncodes, L, static_cast<K*>(keys), status);
}

template <typename T>
void launch_hk_width(uint32_t key_bytes, const void* text, uint64_t n, const uint64_t* code_len,
                     const uint64_t* code_word, uint64_t ncodes, uint32_t L, void* keys, uint32_t* status,
                     cudaStream_t s) {
  switch (key_bytes) {
    case 1: launch_hk<T, uint8_t>(text, n, code_len, code_word, ncodes, L, keys, status, s); break;
    case 2: launch_hk<T, uint16_t>(text, n, code_len, code_word, ncodes, L, keys, status, s); break;
    case 4: launch_hk<T, uint32_t>(text, n, code_len, code_word, ncodes, L, keys, status, s); break;
    default: launch_hk<T, uint64_t>(text, n, code_len, code_word, ncodes, L, keys, status, s); break;
  }
}

void launch_huffman_keys(const void* text, uint64_t n, uint32_t width, const uint64_t* code_len,
                         const uint64_t* code_word, uint64_t ncodes, uint32_t levels, uint32_t key_bytes, void* keys,
                         uint32_t* status, cudaStream_t s, uint64_t* launches) {
  if (n == 0) return;
  if (width == 1) launch_hk_width<uint8_t>(key_bytes, text, n, code_len, code_word, ncodes, levels, keys, status, s);
  else if (width == 2)
    launch_hk_width<uint16_t>(key_bytes, text, n, code_len, code_word, ncodes, levels, keys, status, s);
  else launch_hk_width<uint32_t>(key_bytes, text, n, code_len, code_word, ncodes, levels, keys, status, s);
  ++*launches;
}

void launch_symbol_histogram(const void* text, uint64_t n, uint32_t width, uint64_t nsym, unsigned long long* hist,
                             unsigned long long* first, uint32_t* status, cudaStream_t s, uint64_t* launches) {
  if (n == 0) return;
  const int g = grid_for(n, 256);
  if (width <= 2) {
    // every value is a bin: the shared-memory leaf histograms of 8 / 16 levels
    launch_leaf_histogram(text, n, width, 8 * width, hist, status, s, launches);
    if (first) {
      if (width == 1) first_occurrence_kernel<<<g, 256, 0, s>>>(static_cast<const uint8_t*>(text), n, first);
      else first_occurrence_kernel<<<g, 256, 0, s>>>(static_cast<const uint16_t*>(text), n, first);
      ++*launches;
    }
    return;
  }
  symbol_hist_kernel<<<g, 256, 0, s>>>(static_cast<const uint32_t*>(text), n, nsym, hist, first);
  ++*launches;
}

void launch_pass_digits(const void* text, uint64_t n, uint32_t width, const PassDigitsArgs& pd,
                        unsigned long long* digits, unsigned int* done, uint32_t* status, uint64_t* out,
                        cudaStream_t s, uint64_t* launches) {
  const size_t smem = size_t(pd.npasses) * 16 * 32 * 4;
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(pass_digits_kernel<kPassDigitsMaxPasses>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         int(kPassDigitsMaxPasses * 16 * 32 * 4));
    configured = true;
  }
  const uint64_t vecs = (n * width + 15) / 16;
  const uint64_t want = (vecs + 255) / 256;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const uint64_t cap = uint64_t(sms > 0 ? sms : 1) * 4;
  const unsigned grid = unsigned(std::max<uint64_t>(1, std::min(want, cap)));
  if (pd.npasses <= 6)
    pass_digits_kernel<6><<<grid, 256, smem, s>>>(static_cast<const unsigned char*>(text), n, width, pd, digits, done,
                                                  status, out);
  else
    pass_digits_kernel<kPassDigitsMaxPasses><<<grid, 256, smem, s>>>(static_cast<const unsigned char*>(text), n, width,
                                                                     pd, digits, done, status, out);
  ++*launches;
}

void launch_readback(const unsigned long long* src, uint64_t n, const uint32_t* status, uint64_t* dst,
                     cudaStream_t s, uint64_t* launches) {
  const uint64_t blocks = (n + 255) / 256;
  readback_kernel<<<unsigned(blocks < 1024 ? (blocks ? blocks : 1) : 1024), 256, 0, s>>>(src, n, status, dst);
  ++*launches;
}

void launch_widen40(const void* in, uint64_t n, uint32_t* out, cudaStream_t s, uint64_t* launches) {
  if (n == 0) return;
  widen40_kernel<<<grid_for(n, 256), 256, 0, s>>>(static_cast<const uint8_t*>(in), n, out);
  ++*launches;
}

void launch_fold_levels(const unsigned long long* hist, uint32_t levels, uint64_t* flat, unsigned long long* zeros,
                        cudaStream_t s, uint64_t* launches, uint64_t* flat_dev) {
  uint32_t top = levels;
  bool first = true;
  for (;;) {
    const uint32_t down = top < 10u ? top : 10u;
    const uint64_t blocks = ((1ull << top) + 1023) / 1024;
    fold_levels_kernel<<<unsigned(blocks), 256, 0, s>>>(flat, flat_dev, first ? hist : nullptr, top, down, zeros);
    ++*launches;
    first = false;
    if (down == top) break;  // level 0 written
    top -= down;
  }
}

void launch_alphabet_insert(const void* text, uint32_t width, uint64_t n, unsigned long long* keys,
                            unsigned long long* first, uint64_t cap, uint32_t* status, cudaStream_t s,
                            uint64_t* launches) {
  if (n == 0) return;
  alphabet_insert_kernel<<<grid_for(n, 256), 256, 0, s>>>(static_cast<const uint8_t*>(text), width, n, keys, first,
                                                         cap - 1, status);
  ++*launches;
}

void launch_alphabet_collect(const unsigned long long* keys, const unsigned long long* first, uint64_t cap,
                             unsigned long long* count, uint64_t* out, cudaStream_t s, uint64_t* launches) {
  alphabet_collect_kernel<<<grid_for(cap, 256), 256, 0, s>>>(keys, first, cap, count, out);
  ++*launches;
}

void launch_scatter_ids(const uint64_t* slots, const uint32_t* ids, uint64_t count, uint32_t* slot_ids, cudaStream_t s,
                        uint64_t* launches) {
  if (count == 0) return;
  scatter_ids_kernel<<<grid_for(count, 256), 256, 0, s>>>(slots, ids, count, slot_ids);
  ++*launches;
}

void launch_alphabet_remap(const void* text, uint32_t width, uint64_t n, const unsigned long long* keys,
                           const uint32_t* slot_ids, uint64_t cap, void* out, uint32_t* status, cudaStream_t s,
                           uint64_t* launches) {
  if (n == 0) return;
  alphabet_remap_kernel<<<grid_for(n, 256), 256, 0, s>>>(static_cast<const uint8_t*>(text), width, n, keys, slot_ids,
                                                        cap - 1, static_cast<uint8_t*>(out), status);
  ++*launches;
}

void launch_max_symbol(const uint32_t* text, uint64_t n, unsigned int* out, cudaStream_t s, uint64_t* launches) {
  if (n == 0) return;
  max_symbol_kernel<<<grid_for(n, 256), 256, 0, s>>>(text, n, out);
  ++*launches;
}

void launch_remap(const void* text, uint64_t n, uint32_t width, const uint32_t* map, uint64_t nmap, void* out,
                  uint32_t* status, cudaStream_t s, uint64_t* launches) {
  if (n == 0) return;
  const int g = grid_for(n, 256);
  if (width == 1)
    remap_kernel<<<g, 256, 0, s>>>(static_cast<const uint8_t*>(text), n, map, nmap, static_cast<uint8_t*>(out), status);
  else if (width == 2)
    remap_kernel<<<g, 256, 0, s>>>(static_cast<const uint16_t*>(text), n, map, nmap, static_cast<uint16_t*>(out),
                                   status);
  else
    remap_kernel<<<g, 256, 0, s>>>(static_cast<const uint32_t*>(text), n, map, nmap, static_cast<uint32_t*>(out),
                                   status);
  ++*launches;
}

void launch_generate(int dist, uint64_t seed, uint64_t param, uint64_t n, uint32_t width, void* out,
                     const uint64_t* thresholds, uint32_t nthr, const uint32_t* perm, cudaStream_t s,
                     uint64_t* launches) {
  if (n == 0) return;
  const uint64_t key = mix64(seed);
  const int g = grid_for(n, 256);
  if (width == 1) generate_kernel<<<g, 256, 0, s>>>(dist, key, param, n, static_cast<uint8_t*>(out), thresholds, nthr, perm);
  else if (width == 2) generate_kernel<<<g, 256, 0, s>>>(dist, key, param, n, static_cast<uint16_t*>(out), thresholds, nthr, perm);
  else generate_kernel<<<g, 256, 0, s>>>(dist, key, param, n, static_cast<uint32_t*>(out), thresholds, nthr, perm);
  ++*launches;
}

}  // namespace pwmgpu
