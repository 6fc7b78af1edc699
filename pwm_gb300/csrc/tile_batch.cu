// Batched construction on the tile engine: many independent texts built by
// one persistent kernel that takes (text, pass, tile) items from a device
// work queue, with every table the single-text host planner would compute
// derived on the device from the texts' leaf histograms, so that a whole
// batch is one CUDA graph without host round trips.
//
// Work items: the tiles of every (text, pass), grouped by pass shape (pass
// index, levels K, whether it writes S_{l+K}) and queued group by group in
// pass order, so that when a tile of pass p of a text is dequeued every tile
// of pass p-1 of that text has been dequeued before it; the tile waits
// (bounded) until those are done and counts itself done afterwards.  A
// waiting CTA never holds an item an earlier item waits for, so the queue
// always drains.
#include "kernels.cuh"
#include "tile_batch.cuh"

namespace pwmgpu {

namespace {

constexpr int kPlanThreads = 256;

// The per-thread partial sums part[0..kPlanThreads) replaced by their
// exclusive prefixes (warp 0, 8 per lane, one shuffle scan); returns the
// total.  Called by every thread after part is written.
__device__ unsigned long long scan_parts(unsigned long long* part) {
  static_assert(kPlanThreads == 256, "8 partial sums per lane of one warp");
  __shared__ unsigned long long total;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = int(threadIdx.x);
    unsigned long long v[8], sum = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      v[q] = part[8 * lane + q];
      sum += v[q];
    }
    unsigned long long x = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (lane >= d) x += y;
    }
    unsigned long long run = x - sum;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      part[8 * lane + q] = run;
      run += v[q];
    }
    if (lane == 31) total = x;
  }
  __syncthreads();
  return total;
}

__device__ __forceinline__ uint32_t rev_bits(uint32_t v, uint32_t bits) {
  return bits == 0 ? 0u : (__brev(v) >> (32 - bits));
}

// Exclusive prefix sums of a[0..len) into out[0..len), the total into
// out[len], by one warp: lane i sums a run of consecutive elements, one
// shuffle scan of the run sums, then each lane writes its run.
template <typename F>
__device__ void warp_exclusive_scan_u64(uint64_t len, F fetch, uint64_t* out, uint32_t lane) {
  const uint64_t per = (len + 31) / 32;
  const uint64_t b = min(len, uint64_t(lane) * per), e = min(len, b + per);
  unsigned long long sum = 0;
  for (uint64_t i = b; i < e; ++i) sum += fetch(i);
  unsigned long long x = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, d);
    if (int(lane) >= d) x += y;
  }
  unsigned long long run = x - sum;
  for (uint64_t i = b; i < e; ++i) {
    const unsigned long long v = fetch(i);
    out[i] = run;
    run += v;
  }
  if (lane == 31) out[len] = x;
}

// Per text, one warp (at most 2^12 leaves, 128 per lane): the natural
// prefix counts of every level folded from its leaf histogram, the matrix
// zero counts, and the exclusive prefixes of every level in natural (tree)
// and key (matrix: bit-reversed prefix) order.  A CTA of 256 threads per
// text spent its time in barriers: most texts have a few dozen leaves.
__global__ void __launch_bounds__(256) tile_batch_fold_kernel(const TileBatchText* __restrict__ texts, uint32_t ntexts,
                                                              const unsigned long long* __restrict__ hist, uint64_t* pfx,
                                                              uint64_t* zeros,
                                                              const unsigned long long* __restrict__ blocksum,
                                                              unsigned long long* blockpre) {
  const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= ntexts) return;
  const TileBatchText t = texts[w];
  const uint32_t L = t.levels;
  uint64_t* cnt = pfx + t.pfx_off;  // level m at 2^m - 1
  uint64_t* pn = cnt + tile_batch_counts(L);
  uint64_t* pk = pn + tile_batch_prefixes(L);
  const unsigned long long* h = hist + t.hist_off;
  for (uint64_t p = lane; p < (uint64_t(1) << L); p += 32) cnt[(uint64_t(1) << L) - 1 + p] = h[p];
  __syncwarp();
  for (int m = int(L) - 1; m >= 0; --m) {
    const uint64_t* up = cnt + (uint64_t(2) << m) - 1;
    uint64_t* o = cnt + (uint64_t(1) << m) - 1;
    for (uint64_t p = lane; p < (uint64_t(1) << m); p += 32) o[p] = up[2 * p] + up[2 * p + 1];
    __syncwarp();
  }
  // zeros of level m: the symbols whose (m+1)-bit prefix is even
  for (uint32_t m = 0; m < L; ++m) {
    const uint64_t* c = cnt + (uint64_t(2) << m) - 1;
    unsigned long long z = 0;
    for (uint64_t p = 2 * lane; p < (uint64_t(2) << m); p += 64) z += c[p];
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) z += __shfl_xor_sync(0xFFFFFFFFu, z, d);
    if (lane == 0) zeros[t.zeros_off + m] = z;
  }
  for (uint32_t m = 0; m <= L; ++m) {
    const uint64_t* c = cnt + (uint64_t(1) << m) - 1;
    const uint64_t len = uint64_t(1) << m;
    warp_exclusive_scan_u64(len, [&](uint64_t i) { return c[i]; }, pn + tile_batch_level_at(m), lane);
    warp_exclusive_scan_u64(len, [&](uint64_t i) { return c[rev_bits(uint32_t(i), m)]; }, pk + tile_batch_level_at(m),
                            lane);
  }
  // the first pass's block prefixes: per counter, exclusive sums over the
  // text's blocks of tiles (lane i takes a run of consecutive blocks)
  const uint32_t nb = t.nb0, nt = t.nblk0;
  for (uint32_t cn = 0; cn < nb; ++cn) {
    const uint32_t per = (nt + 31) / 32, b = min(nt, lane * per), e = min(nt, b + per);
    unsigned long long sum = 0;
    for (uint32_t i = b; i < e; ++i) sum += blocksum[t.blk_off + uint64_t(i) * nb + cn];
    unsigned long long x = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (int(lane) >= d) x += y;
    }
    unsigned long long run = x - sum;
    for (uint32_t i = b; i < e; ++i) {
      const uint64_t at = t.blk_off + uint64_t(i) * nb + cn;
      const unsigned long long v = blocksum[at];
      blockpre[at] = run;
      run += v;
    }
  }
}

// Per (text, pass): its segments (one per prefix group of its first level,
// in key order, empty ones kept with no tiles), their start tables and tile
// counts, and the tiles of the pass (what the next pass of the text waits
// for).  The tables are those of the single-text planner's segmented passes
// (plan_tile_passes, host_tables.hpp).
__global__ void __launch_bounds__(kPlanThreads) tile_batch_segments_kernel(
    const TileBatchText* __restrict__ texts, const TileBatchPass* __restrict__ passes,
    const TileBatchGroup* __restrict__ groups, const uint64_t* __restrict__ pfx, uint32_t key_bytes, unsigned* need) {
  __shared__ unsigned long long part[kPlanThreads];
  const TileBatchPass p = passes[blockIdx.x];
  const TileBatchText t = texts[p.text];
  const TileBatchGroup gr = groups[p.group];
  const uint32_t L = t.levels, l = p.level, K = gr.K;
  const uint64_t* pn = pfx + t.pfx_off + tile_batch_counts(L);
  const uint64_t* pk = pn + tile_batch_prefixes(L);
  auto PK = [&](uint32_t m, uint64_t x) { return pk[tile_batch_level_at(m) + x]; };
  auto PN = [&](uint32_t m, uint64_t x) { return pn[tile_batch_level_at(m) + x]; };
  const int TS = tile_table_size(int(K));
  const uint64_t TT = uint64_t(256) * p.vpt * (16 / key_bytes);
  unsigned long long tiles = 0;
  for (uint64_t g = threadIdx.x; g < (uint64_t(1) << l); g += kPlanThreads) {
    const uint64_t m = PK(l, g + 1) - PK(l, g);
    const uint64_t tab = p.table_base + g * uint64_t(TS);
    TileSeg sg;
    sg.in_begin = (l == 0 ? t.text_begin : t.key_begin) + PK(l, g);
    sg.m = m;
    sg.table = tab;
    sg.tile0 = 0;  // tile_batch_scan_kernel
    sg.text = p.tt_index;
    gr.segs[p.seg_base + g] = sg;
    const uint32_t nt = uint32_t((m + TT - 1) / TT);
    gr.seg_tiles[p.seg_base + g] = nt;
    tiles += nt;
    uint64_t* tb = gr.tables + tab;
    for (uint32_t j = 0; j < K; ++j)
      for (uint32_t v = 0; v < (1u << j); ++v) {
        const uint64_t x = (uint64_t(v) << l) | g;
        tb[tile_wm_entry(int(j), int(v))] = PK(l + j, x);
        tb[tile_wt_entry(int(K), int(j), int(v))] = PN(l + j, rev_bits(uint32_t(x), l + j));
      }
    if (gr.out)
      for (uint32_t v = 0; v < (1u << K); ++v) tb[tile_out_entry(int(K), int(v))] = t.key_begin + PK(l + K, (uint64_t(v) << l) | g);
  }
  part[threadIdx.x] = tiles;
  const unsigned long long total = scan_parts(part);
  if (threadIdx.x == 0) need[p.slot] = unsigned(total);
}

// Per group: the first tile of every segment (exclusive sums of the tile
// counts) and the group's tiles.
__global__ void __launch_bounds__(1024) tile_batch_scan_kernel(const TileBatchGroup* __restrict__ groups,
                                                               unsigned* group_tiles) {
  __shared__ unsigned long long part[1024];
  const TileBatchGroup gr = groups[blockIdx.x];
  const uint32_t tid = threadIdx.x;
  const uint64_t per = (uint64_t(gr.nsegs) + 1023) / 1024;
  const uint64_t b = min(uint64_t(gr.nsegs), tid * per), e = min(uint64_t(gr.nsegs), b + per);
  unsigned long long sum = 0;
  for (uint64_t i = b; i < e; ++i) sum += gr.seg_tiles[i];
  part[tid] = sum;
  __syncthreads();
  for (uint32_t d = 1; d < 1024; d <<= 1) {  // inclusive scan (Hillis-Steele)
    const unsigned long long y = tid >= d ? part[tid - d] : 0ull;
    __syncthreads();
    part[tid] += y;
    __syncthreads();
  }
  unsigned long long run = part[tid] - sum;
  for (uint64_t i = b; i < e; ++i) {
    gr.segs[i].tile0 = uint32_t(run);
    run += gr.seg_tiles[i];
  }
  if (tid == 1023) group_tiles[blockIdx.x] = unsigned(part[1023]);
}

// The persistent kernel: a CTA per resident slot (5 per SM, 48 registers a
// thread) takes items until the queue is drained.  Item i of group k is tile
// i - base(k) of that group's pass.
template <typename KeyT>
__global__ void __launch_bounds__(256, 5) tile_batch_kernel(TileBatchQueue q) {
  __shared__ uint32_t s_base[kTileBatchMaxGroups + 1];
  __shared__ uint32_t s_item, s_gi;
  __shared__ __align__(16) TileArgs s_args;
  // (Claiming the next item while the current one runs was slower: a tile
  // waiting for a text's previous pass then also waits for items that other
  // CTAs hold unstarted.)
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (uint32_t k = 0; k < q.ngroups; ++k) {
      s_base[k] = run;
      run += q.group_tiles[k];
    }
    s_base[q.ngroups] = run;
  }
  uint32_t have = ~0u;  // the group whose arguments s_args holds
  for (;;) {
    __syncthreads();  // s_base is set; the previous item is done with shared memory
    if (threadIdx.x == 0) {
      const uint32_t item = atomicAdd(q.head, 1u);
      uint32_t k = 0;
      while (k < q.ngroups && item >= s_base[k + 1]) ++k;
      s_item = item;
      s_gi = k;
    }
    __syncthreads();
    const uint32_t k = s_gi;
    if (k >= q.ngroups) break;
    if (k != have) {
      const uint32_t* src = reinterpret_cast<const uint32_t*>(q.args + k);
      uint32_t* dst = reinterpret_cast<uint32_t*>(&s_args);
      for (uint32_t i = threadIdx.x; i < sizeof(TileArgs) / 4; i += blockDim.x) dst[i] = src[i];
      have = k;
      __syncthreads();
    }
    const uint32_t g = s_item - s_base[k];
    // passes without S_{l+K} over 1-byte keys split bit planes
    constexpr bool PL = sizeof(KeyT) == 1;
    switch (q.variant[k]) {
      case kTileBatchK4Out: tile_pass_body<KeyT, 4, true, 256, 4, true>(s_args, g); break;
      case kTileBatchK4: tile_pass_body<KeyT, 4, false, 256, 4, true, KeyT, PL>(s_args, g); break;
      case kTileBatchK3: tile_pass_body<KeyT, 3, false, 256, 4, true, KeyT, PL>(s_args, g); break;
      case kTileBatchK2: tile_pass_body<KeyT, 2, false, 256, 4, true, KeyT, PL>(s_args, g); break;
      default: tile_pass_body<KeyT, 1, false, 256, 4, true, KeyT, PL>(s_args, g); break;
    }
  }
}

template <typename KeyT>
size_t batch_kernel_smem() {
  using C = TileCfg<KeyT, 4, true, 256, 4>;  // the largest shape's buffers
  static bool configured = false;  // attribute set once per key width
  if (!configured) {
    cudaFuncSetAttribute(tile_batch_kernel<KeyT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(C::smem_bytes()));
    configured = true;
  }
  return C::smem_bytes();
}

template <typename KeyT>
void launch_batch_kernel(const TileBatchQueue& q, uint32_t ctas, cudaStream_t s) {
  const size_t smem = batch_kernel_smem<KeyT>();
  tile_batch_kernel<KeyT><<<ctas, 256, smem, s>>>(q);
}

template <typename KeyT>
int batch_kernel_occupancy() {
  int blocks = 0;
  const size_t smem = batch_kernel_smem<KeyT>();
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, tile_batch_kernel<KeyT>, 256, smem) == cudaSuccess
             ? blocks
             : 0;
}

}  // namespace

void launch_tile_batch_plan(const TileBatchText* texts, uint32_t ntexts, const TileBatchPass* passes,
                            uint32_t npasses, const TileBatchGroup* groups, uint32_t ngroups,
                            const unsigned long long* hist, uint64_t* pfx, uint64_t* zeros, uint32_t key_bytes,
                            unsigned* need, unsigned* group_tiles, const unsigned long long* blocksum,
                            unsigned long long* blockpre, cudaStream_t s, uint64_t* launches) {
  if (ntexts == 0) return;
  tile_batch_fold_kernel<<<(ntexts + 7) / 8, 256, 0, s>>>(texts, ntexts, hist, pfx, zeros, blocksum, blockpre);
  tile_batch_segments_kernel<<<npasses, kPlanThreads, 0, s>>>(texts, passes, groups, pfx, key_bytes, need);
  tile_batch_scan_kernel<<<ngroups, 1024, 0, s>>>(groups, group_tiles);
  *launches += 3;
}

void launch_tile_batch(uint32_t key_bytes, const TileBatchQueue& q, uint32_t ctas, cudaStream_t s,
                       uint64_t* launches) {
  if (q.ngroups == 0 || ctas == 0) return;
  if (key_bytes == 1) launch_batch_kernel<uint8_t>(q, ctas, s);
  else if (key_bytes == 2) launch_batch_kernel<uint16_t>(q, ctas, s);
  else launch_batch_kernel<uint32_t>(q, ctas, s);
  ++*launches;
}

int tile_batch_ctas_per_sm(uint32_t key_bytes) {
  if (key_bytes == 1) return batch_kernel_occupancy<uint8_t>();
  if (key_bytes == 2) return batch_kernel_occupancy<uint16_t>();
  return batch_kernel_occupancy<uint32_t>();
}

}  // namespace pwmgpu
