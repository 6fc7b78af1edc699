// Descriptors of the batched tile engine (tile_batch.cu): texts, their
// passes, the pass groups and the work queue of the persistent kernel.
#pragma once

#include <cstdint>

#include "tile.cuh"

namespace pwmgpu {

constexpr uint32_t kTileBatchMaxLevels = 12;  // a text's prefix tables fit one CTA's planning
constexpr uint32_t kTileBatchMaxGroups = 16;  // pass groups of one batch

// Pass shapes of the persistent kernel: passes of 4 levels that write the
// next sequence, and last passes of 1..4 levels.
enum : uint8_t { kTileBatchK4Out = 0, kTileBatchK4 = 1, kTileBatchK3 = 2, kTileBatchK2 = 3, kTileBatchK1 = 4 };

// Offsets of a text's planning scratch: the natural prefix counts of levels
// 0..L (level m at 2^m - 1), then the exclusive prefixes of every level in
// natural and in key order (level m at tile_batch_level_at(m), 2^m + 1
// entries: the last one is the total).
__host__ __device__ inline uint64_t tile_batch_counts(uint32_t L) { return (uint64_t(2) << L) - 1; }
__host__ __device__ inline uint64_t tile_batch_level_at(uint32_t m) { return (uint64_t(1) << m) - 1 + m; }
__host__ __device__ inline uint64_t tile_batch_prefixes(uint32_t L) { return tile_batch_level_at(L + 1); }
__host__ __device__ inline uint64_t tile_batch_scratch(uint32_t L) {
  return tile_batch_counts(L) + 2 * tile_batch_prefixes(L);
}

struct TileBatchText {
  uint64_t text_begin;  // first symbol of the text in the batch's text buffer
  uint64_t key_begin;   // ... and in the key buffers of the passes after the first
  uint64_t n;           // symbols
  uint32_t levels;
  uint32_t pad;
  uint64_t hist_off;   // its 2^levels leaf counts in the batch's histogram array
  uint64_t pfx_off;    // its planning scratch (tile_batch_scratch words)
  uint64_t zeros_off;  // its matrix zero counts
  // its first pass's given prefixes: the histogram kernel's totals of its
  // nblk0 blocks of tiles at blocksum[blk_off + block * nb0 + counter],
  // their exclusive prefixes to the same place in blockpre (nb0 = 0: the
  // first pass counts and looks back)
  uint64_t blk_off;
  uint32_t nblk0, nb0;
};

struct TileBatchPass {  // one pass of one text
  uint32_t text, group;  // indices into the text and group arrays
  uint32_t level;        // first level of the pass
  uint32_t vpt;          // vectors per thread of its tiles
  uint32_t seg_base;     // its first segment in the group's segment array (2^level segments)
  uint32_t tt_index;     // its TileText in the group's array
  uint32_t slot;         // its counter in the done / need arrays
  uint32_t pad;
  uint64_t table_base;   // its first segment's start table in the group's table array
};

struct TileBatchGroup {  // the passes of one shape: one TileArgs of the persistent kernel
  TileSeg* segs;
  uint64_t* tables;
  uint32_t* seg_tiles;   // tiles of every segment (planning)
  uint32_t nsegs;
  uint32_t K;
  uint32_t out;
  uint32_t pad;
};

struct TileBatchQueue {
  const TileArgs* args;          // device: one per group, in queue order
  const unsigned* group_tiles;   // device: tiles of every group (planning)
  unsigned* head;                // device: the queue's next item, zeroed before each build
  uint32_t ngroups;
  uint8_t variant[kTileBatchMaxGroups];  // kTileBatch* shape of every group
};

// Planning on the device: prefix tables and zero counts of every text, the
// segments and start tables of every pass, the first tile of every segment
// and the tiles of every group and of every (text, pass) (`need`).
void launch_tile_batch_plan(const TileBatchText* texts, uint32_t ntexts, const TileBatchPass* passes,
                            uint32_t npasses, const TileBatchGroup* groups, uint32_t ngroups,
                            const unsigned long long* hist, uint64_t* pfx, uint64_t* zeros, uint32_t key_bytes,
                            unsigned* need, unsigned* group_tiles, const unsigned long long* blocksum,
                            unsigned long long* blockpre, cudaStream_t s, uint64_t* launches);
// The persistent kernel on `ctas` CTAs.
void launch_tile_batch(uint32_t key_bytes, const TileBatchQueue& q, uint32_t ctas, cudaStream_t s,
                       uint64_t* launches);
// CTAs of the persistent kernel that fit one SM.
int tile_batch_ctas_per_sm(uint32_t key_bytes);

}  // namespace pwmgpu
