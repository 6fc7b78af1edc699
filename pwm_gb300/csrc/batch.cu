// Kernels of the batched construction: many independent texts, each built
// exactly like a single text (same split passes), with the per-text tables
// that a single build derives on the host computed on the device instead, so
// that a whole batch is one CUDA graph without host round trips.
#include "kernels.cuh"

namespace pwmgpu {

namespace {

constexpr int kBatchThreads = 256;

__device__ __forceinline__ uint32_t rev_bits_dev(uint32_t v, uint32_t bits) {
  return bits == 0 ? 0u : (__brev(v) >> (32 - bits));
}

// Leaf histogram of one chunk of one text (2^L <= 4096 bins in shared
// memory).  The bins are kept in 4096 >> L interleaved copies (at most one
// per thread; bin s of copy c at s * copies + c, so the lanes of a warp hit
// different banks), which spreads the atomics of texts with few levels over
// the copies instead of piling them on a handful of words.  The chunk is
// read in 16-byte vectors between its unaligned ends.  A chunk of a tile
// batch also counts, per first-pass tile, the tile's finest runs (the
// D-bit digit of the top symbol bits, counter = the digit bit-reversed), a
// column per lane, for the pass's given prefixes.
constexpr uint32_t kHistTileCounters = 16 * 16 * 32;  // tiles x counters x lanes
template <typename T>
__global__ void __launch_bounds__(kBatchThreads) batch_hist_kernel(const T* __restrict__ texts,
                                                                   const BatchChunk* __restrict__ chunks,
                                                                   const BatchText* __restrict__ info,
                                                                   unsigned long long* hist, uint32_t* tilecnt,
                                                                   uint32_t* relpre, unsigned long long* blocksum,
                                                                   uint32_t* status) {
  constexpr uint32_t E = 16 / sizeof(T);  // symbols per vector
  extern __shared__ uint32_t hsm[];
  uint32_t* h = hsm;               // [4096]
  uint32_t* tc = hsm + 4096;       // [16 tiles][16 counters][32 lanes]
  const BatchChunk c = chunks[blockIdx.x];
  const BatchText t = info[c.text];
  const uint32_t bins = 1u << t.levels;
  const uint32_t copies = min(uint32_t(kBatchThreads), 4096u >> t.levels);
  const uint32_t mine = threadIdx.x % copies, lane = threadIdx.x & 31;
  const uint32_t D = c.D, dsh = t.levels - c.D;  // the digit: symbol bits [L-D, L)
  const uint32_t ntiles = D ? uint32_t((c.len + (uint64_t(1) << c.log2T) - 1) >> c.log2T) : 0u;
  // Up to 16 bins: one counter per (tile, bin, lane) serves both the text's
  // histogram and the tiles' finest-run counts (each a sum over bins), one
  // shared atomic per symbol; else a text histogram (per-thread copies) and
  // the tiles' digit counters.
  const bool by_tile = D && bins <= 16;
  if (!by_tile)
    for (uint32_t i = threadIdx.x; i < bins * copies; i += kBatchThreads) h[i] = 0;
  for (uint32_t i = threadIdx.x; i < ntiles * 16 * 32; i += kBatchThreads) tc[i] = 0;
  __syncthreads();
  // Branch-free: every symbol counts into bin (symbol mod 2^L), and `seen`
  // collects the bits of all of them (of whole words: 2^L - 1 per symbol
  // lane of a word is the allowed part), so one test at the end finds a
  // symbol >= 2^L (the counts are then not used).
  uint32_t seen = 0;
  const uint32_t bmask = bins - 1;
  // the allowed bits of one symbol lane of a word (2^L - 1, at most the lane)
  const uint32_t lmask = sizeof(T) == 4 ? bmask : min(bmask, (1u << (8 * sizeof(T))) - 1u);
  const uint32_t tcb = uint32_t(__cvta_generic_to_shared(tc)) + lane * 4;
  auto count = [&](uint32_t s, uint32_t i) {  // symbol s at chunk position i
    if (by_tile) {
      asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(tcb + (((i >> c.log2T) * 16 + (s & bmask)) << 7)) : "memory");
      return;
    }
    atomicAdd(&h[(s & bmask) * copies + mine], 1u);
    if (D) {
      const uint32_t cn = __brev((s >> dsh) & ((1u << D) - 1u)) >> (32 - D);
      asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(tcb + (((i >> c.log2T) * 16 + cn) << 7)) : "memory");
    }
  };
  const T* p = texts + t.offset + c.start;
  const uint64_t head = min(c.len, uint64_t((16u - (reinterpret_cast<uintptr_t>(p) & 15u)) & 15u) / sizeof(T));
  const uint64_t nv = (c.len - head) / E;
  if (threadIdx.x < head) {
    seen |= uint32_t(p[threadIdx.x]);
    count(uint32_t(p[threadIdx.x]), threadIdx.x);
  }
  const uint4* v = reinterpret_cast<const uint4*>(p + head);
  uint32_t seen_w = 0;  // the OR of whole vector words
  for (uint32_t k = threadIdx.x; k < nv; k += kBatchThreads) {
    const uint4 x = __ldcs(v + k);
    const uint32_t w[4] = {x.x, x.y, x.z, x.w};
    seen_w |= x.x | x.y | x.z | x.w;
    const uint32_t i0 = uint32_t(head) + k * E;
#pragma unroll
    for (uint32_t e = 0; e < E; ++e) {
      if constexpr (sizeof(T) == 1) count((w[e >> 2] >> (8 * (e & 3))) & lmask, i0 + e);
      else if constexpr (sizeof(T) == 2) count((w[e >> 1] >> (16 * (e & 1))) & lmask, i0 + e);
      else count(w[e], i0 + e);
    }
  }
  for (uint64_t i = head + nv * E + threadIdx.x; i < c.len; i += kBatchThreads) {
    seen |= uint32_t(p[i]);
    count(uint32_t(p[i]), uint32_t(i));
  }
  const uint32_t lanes = sizeof(T) == 1 ? 0x01010101u : (sizeof(T) == 2 ? 0x00010001u : 1u);
  if ((seen & ~bmask) || (seen_w & ~(lanes * lmask))) atomicOr(status, kErrSymbol);
  __syncthreads();
  unsigned long long* out = hist + t.hist_off;
  if (by_tile) {
    // per (tile, bin) the lanes' sum into lane column 0, then the text's
    // histogram over the tiles and each tile's counters over the bins of
    // each digit (the slots of unused tiles and bins are zero)
    for (uint32_t e = threadIdx.x; e < ntiles * 16; e += kBatchThreads) {
      uint32_t sum = 0;
      for (uint32_t l = 0; l < 32; ++l) sum += tc[e * 32 + l];
      h[e] = sum;  // h (free in this mode): [tile][bin]
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < bins; b += kBatchThreads) {
      uint32_t sum = 0;
      for (uint32_t tile = 0; tile < ntiles; ++tile) sum += h[tile * 16 + b];
      if (sum) atomicAdd(&out[b], (unsigned long long)sum);
    }
    const uint32_t nb = 1u << D;
    for (uint32_t e = threadIdx.x; e < ntiles * nb; e += kBatchThreads) {
      const uint32_t tile = e >> D, cn = e & (nb - 1);
      uint32_t sum = 0;
      for (uint32_t b = 0; b < bins; ++b)
        if ((__brev((b >> dsh) & (nb - 1u)) >> (32 - D)) == cn) sum += h[tile * 16 + b];
      tilecnt[c.cnt_off + e] = sum;
      tc[(tile * 16 + cn) * 32 + ((e + 1) & 31)] = sum;  // read back below by the prefix loop
    }
    __syncthreads();
    if (threadIdx.x < nb) {
      const uint32_t cn = threadIdx.x;
      uint32_t run = 0;
      for (uint32_t tile = 0; tile < ntiles; ++tile) {
        const uint32_t e = tile * nb + cn;
        relpre[c.cnt_off + e] = run;
        run += tc[(tile * 16 + cn) * 32 + ((e + 1) & 31)];
      }
      blocksum[c.blk_off + cn] = run;
    }
    return;
  }
  for (uint32_t s = threadIdx.x; s < bins; s += kBatchThreads) {
    uint32_t sum = 0;
    for (uint32_t k = 0; k < copies; ++k) sum += h[s * copies + k];
    if (sum) atomicAdd(&out[s], (unsigned long long)sum);
  }
  // per tile and counter the lanes' sum (into lane column 0), then per
  // counter the block's exclusive prefixes over its tiles and its total
  const uint32_t nb = 1u << D;
  for (uint32_t e = threadIdx.x; e < ntiles * nb; e += kBatchThreads) {
    const uint32_t tile = e >> D, cn = e & (nb - 1);
    uint32_t sum = 0;
    for (uint32_t l = 0; l < 32; ++l) sum += tc[(tile * 16 + cn) * 32 + ((l + e) & 31)];
    tilecnt[c.cnt_off + e] = sum;
    tc[(tile * 16 + cn) * 32 + ((e + 1) & 31)] = sum;  // a lane this thread read last: no other thread reads it
  }
  __syncthreads();
  if (threadIdx.x < nb && D) {
    const uint32_t cn = threadIdx.x;
    uint32_t run = 0;
    for (uint32_t tile = 0; tile < ntiles; ++tile) {
      const uint32_t e = tile * nb + cn;
      relpre[c.cnt_off + e] = run;
      run += tc[(tile * 16 + cn) * 32 + ((e + 1) & 31)];
    }
    blocksum[c.blk_off + cn] = run;
  }
}

// Per-text tables from the leaf histogram (one CTA per text, L <= 12):
// matrix zero counts, the run starts of every split pass (passes of at most
// kmax levels from level 0, the same plan as a single build) and the
// tree's dense group segments of levels 1..L-1 (tree start, matrix start).
__global__ void __launch_bounds__(kBatchThreads) batch_tables_kernel(const unsigned long long* __restrict__ hist,
                                                                     const BatchText* __restrict__ info, int kmax,
                                                                     uint64_t* zeros, uint64_t* starts,
                                                                     uint64_t* segs) {
  extern __shared__ unsigned long long cnt[];  // heap layout: node (m, p) at (1 << m) + p, m in [0, L]
  const BatchText t = info[blockIdx.x];
  const uint32_t L = t.levels;
  const unsigned long long* h = hist + t.hist_off;
  for (uint32_t p = threadIdx.x; p < (1u << L); p += kBatchThreads) cnt[(1u << L) + p] = h[p];
  __syncthreads();
  for (int m = int(L) - 1; m >= 0; --m) {
    for (uint32_t p = threadIdx.x; p < (1u << m); p += kBatchThreads)
      cnt[(1u << m) + p] = cnt[(2u << m) + 2 * p] + cnt[(2u << m) + 2 * p + 1];
    __syncthreads();
  }
  // zeros[m]: symbols whose bit for level m is 0 = even (m+1)-prefixes
  for (uint32_t m = threadIdx.x; m < L; m += kBatchThreads) {
    unsigned long long z = 0;
    for (uint32_t p = 0; p < (1u << (m + 1)); p += 2) z += cnt[(2u << m) + p];
    zeros[t.zeros_off + m] = z;
  }
  // run starts: pass (l, K), level l+j, value v of key_j (bit l least
  // significant) counts the (l+j)-prefixes q with rev_j(q mod 2^j) == v
  {
    uint32_t l = 0;
    uint64_t off = t.starts_off;
    for (uint32_t pass = 0; l < L; ++pass) {
      const int K = int(min(uint32_t(kmax), L - l));
      for (int j = 1 + int(threadIdx.x); j <= K; j += kBatchThreads) {
        const uint32_t lev = l + uint32_t(j);
        uint64_t* st = starts + off + ((1u << j) - 2);
        if (lev <= L) {
          unsigned long long run = 0;
          for (uint32_t v = 0; v < (1u << j); ++v) {
            unsigned long long c = 0;
            const uint32_t q0 = rev_bits_dev(v, uint32_t(j));
            for (uint32_t q = q0; q < (1u << lev); q += (1u << j)) c += cnt[(1u << lev) + q];
            st[v] = run;
            run += c;
          }
        } else {
          for (uint32_t v = 0; v < (1u << j); ++v) st[v] = 0;
        }
      }
      off += (2u << K) - 2;
      l += uint32_t(K);
    }
  }
  // tree segments, level m: groups in natural prefix order; the matrix holds
  // them in bit-reversed order
  for (uint32_t m = 1 + threadIdx.x; m < L; m += kBatchThreads) {
    uint64_t* tree_start = segs + t.segs_off + 2 * ((1u << m) - 2);
    uint64_t* matrix_start = tree_start + (1u << m);
    unsigned long long run = 0;
    for (uint32_t p = 0; p < (1u << m); ++p) {
      tree_start[p] = run;
      run += cnt[(1u << m) + p];
    }
    run = 0;
    for (uint32_t r = 0; r < (1u << m); ++r) {
      const uint32_t p = rev_bits_dev(r, m);
      matrix_start[p] = run;
      run += cnt[(1u << m) + p];
    }
  }
}

__device__ __forceinline__ uint64_t bits_at_dev(const uint64_t* level, uint64_t src, uint32_t take) {
  const uint64_t w = src >> 6;
  const uint32_t sh = uint32_t(src & 63);
  uint64_t v = level[w] << sh;
  if (sh != 0 && sh + take > 64) v |= level[w + 1] >> (64 - sh);
  return take == 64 ? v : (v & ~(~0ull >> take));
}

// Tree level m of one text from its matrix level, one thread per word.
__global__ void __launch_bounds__(kBatchThreads) batch_regroup_kernel(const BatchRegroup* __restrict__ items,
                                                                      uint32_t* status) {
  const BatchRegroup it = items[blockIdx.x];
  const uint64_t nwords = (it.nbits + 63) >> 6;
  const uint64_t nseg = it.nseg;
  for (uint64_t w = it.word_begin + threadIdx.x; w < it.word_end && w < nwords; w += kBatchThreads) {
    const uint64_t p0 = w << 6, end = min(p0 + 64, it.nbits);
    uint64_t pos = p0, acc = 0;
    while (pos < end) {
      uint64_t lo = 0, hi = nseg;
      while (hi - lo > 1) {
        const uint64_t mid = (lo + hi) >> 1;
        if (it.seg_tree[mid] <= pos) lo = mid; else hi = mid;
      }
      const uint64_t seg_end = lo + 1 < nseg ? it.seg_tree[lo + 1] : it.nbits;
      const uint64_t stop = min(end, seg_end);
      const uint32_t take = uint32_t(stop - pos);
      const uint64_t src = it.seg_matrix[lo] + (pos - it.seg_tree[lo]);
      if (take == 0 || src + take > it.nbits) {
        atomicOr(status, kErrBounds);
        break;
      }
      acc |= bits_at_dev(it.matrix, src, take) >> (pos - p0);
      pos = stop;
    }
    it.tree[w] = acc;
  }
}

}  // namespace

template <typename T>
void launch_hist_w(const void* texts, const BatchChunk* chunks, uint32_t nchunks, const BatchText* info,
                   unsigned long long* hist, uint32_t* tilecnt, uint32_t* relpre, unsigned long long* blocksum,
                   uint32_t* status, cudaStream_t s) {
  constexpr size_t smem = (4096 + kHistTileCounters) * 4;
  static bool configured = false;  // attribute set once per width
  if (!configured) {
    cudaFuncSetAttribute(batch_hist_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    configured = true;
  }
  batch_hist_kernel<T><<<nchunks, kBatchThreads, smem, s>>>(static_cast<const T*>(texts), chunks, info, hist, tilecnt,
                                                            relpre, blocksum, status);
}

void launch_batch_hist(const void* texts, uint32_t width, const BatchChunk* chunks, uint32_t nchunks,
                       const BatchText* info, unsigned long long* hist, uint32_t* tilecnt, uint32_t* relpre,
                       unsigned long long* blocksum, uint32_t* status, cudaStream_t s, uint64_t* launches) {
  if (nchunks == 0) return;
  if (width == 1) launch_hist_w<uint8_t>(texts, chunks, nchunks, info, hist, tilecnt, relpre, blocksum, status, s);
  else if (width == 2) launch_hist_w<uint16_t>(texts, chunks, nchunks, info, hist, tilecnt, relpre, blocksum, status, s);
  else launch_hist_w<uint32_t>(texts, chunks, nchunks, info, hist, tilecnt, relpre, blocksum, status, s);
  ++*launches;
}

void launch_batch_tables(const unsigned long long* hist, const BatchText* info, uint32_t ntexts, uint32_t max_levels,
                         int kmax, uint64_t* zeros, uint64_t* starts, uint64_t* segs, cudaStream_t s,
                         uint64_t* launches) {
  if (ntexts == 0) return;
  const size_t smem = (size_t(2) << max_levels) * 8;
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(batch_tables_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(8 << 13));
    configured = true;
  }
  batch_tables_kernel<<<ntexts, kBatchThreads, smem, s>>>(hist, info, kmax, zeros, starts, segs);
  ++*launches;
}

void launch_batch_regroup(const BatchRegroup* items, uint32_t nitems, uint32_t* status, cudaStream_t s,
                          uint64_t* launches) {
  if (nitems == 0) return;
  batch_regroup_kernel<<<nitems, kBatchThreads, 0, s>>>(items, status);
  ++*launches;
}

}  // namespace pwmgpu
