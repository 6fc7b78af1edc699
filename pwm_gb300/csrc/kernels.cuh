// Declarations of the kernel launchers shared by the host orchestration.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "split.cuh"
#include "tile.cuh"

namespace pwmgpu {

// ---- histogram of the text ------------------------------------------------
// Leaf histogram (2^levels bins, u64) of a device text; records kErrSymbol in
// *status when a symbol is >= 2^levels.  hist must be zeroed.
void launch_leaf_histogram(const void* text, uint64_t n, uint32_t width, uint32_t levels,
                           unsigned long long* hist, uint32_t* status, cudaStream_t s, uint64_t* launches);

// Leaf histogram of a text with levels <= 8 that also counts, per tile of
// tile_keys symbols (a multiple of 64), the 2^D runs of the first D symbol
// bits (first bit least significant): tilecnt[tile][run], relpre[tile][run]
// (prefix inside a block of tile_hist_tiles_per_block() tiles) and
// blocksum[block][run].  Blocks [block0, block0 + nblk) of the
// tile_hist_blocks(n, tile_keys) blocks run, so a text can be counted piece
// by piece as it arrives; when level0_a is set, they also write level 0
// (the symbols' top bits in text order) to level0_a and level0_b (if set).
// hist must be zeroed.  launch_tile_block_scan then turns blocksum into each
// block's exclusive prefix.
uint32_t tile_hist_tiles_per_block();
// 40-bit symbols (5 little-endian bytes each) widened to 32 bits (values of
// 2^32 and more become 0xFFFFFFFF).
void launch_widen40(const void* in, uint64_t n, uint32_t* out, cudaStream_t s, uint64_t* launches);
// Prefix counts of levels 0..levels from the leaf histogram into `flat`
// (level m at offset 2^m - 1; host-mapped memory allowed) and, when given,
// the same into device memory `flat_dev`; the zero bits of each level added
// into zeros[0..levels) (zeroed by the caller).
void launch_fold_levels(const unsigned long long* hist, uint32_t levels, uint64_t* flat, unsigned long long* zeros,
                        cudaStream_t s, uint64_t* launches, uint64_t* flat_dev = nullptr);
// dst[0..n) = src[0..n), dst[n] = *status (dst: host-mapped memory).
void launch_readback(const unsigned long long* src, uint64_t n, const uint32_t* status, uint64_t* dst,
                     cudaStream_t s, uint64_t* launches);
// Alphabet reduction of 32- or 40-bit symbols (width 4 or 5) through a hash
// table of `cap` (a power of two, at least twice the text) slots: keys set to
// all ones and first positions to all ones by the caller; insert, collect the
// occupied slots as (slot, symbol, first) triples (count zeroed by the
// caller), scatter the ids the host assigns to their slots, remap.
void launch_alphabet_insert(const void* text, uint32_t width, uint64_t n, unsigned long long* keys,
                            unsigned long long* first, uint64_t cap, uint32_t* status, cudaStream_t s,
                            uint64_t* launches);
void launch_alphabet_collect(const unsigned long long* keys, const unsigned long long* first, uint64_t cap,
                             unsigned long long* count, uint64_t* out, cudaStream_t s, uint64_t* launches);
void launch_scatter_ids(const uint64_t* slots, const uint32_t* ids, uint64_t count, uint32_t* slot_ids, cudaStream_t s,
                        uint64_t* launches);
void launch_alphabet_remap(const void* text, uint32_t width, uint64_t n, const unsigned long long* keys,
                           const uint32_t* slot_ids, uint64_t cap, void* out, uint32_t* status, cudaStream_t s,
                           uint64_t* launches);
// Largest symbol of a 32-bit text into *out (zeroed by the caller).
void launch_max_symbol(const uint32_t* text, uint64_t n, unsigned int* out, cudaStream_t s, uint64_t* launches);
// out[i] = map[text[i]] (same width; in place allowed).
void launch_remap(const void* text, uint64_t n, uint32_t width, const uint32_t* map, uint64_t nmap, void* out,
                  uint32_t* status, cudaStream_t s, uint64_t* launches);
uint32_t tile_hist_blocks(uint64_t n, uint32_t tile_keys);
void launch_tile_histogram_blocks(const void* text, uint64_t n, uint32_t width, uint32_t levels, uint32_t D,
                                  uint32_t tile_keys, uint32_t block0, uint32_t nblk, unsigned long long* hist,
                                  uint32_t* tilecnt, uint32_t* relpre, unsigned long long* blocksum,
                                  uint64_t* level0_a, uint64_t* level0_b, uint32_t* status, cudaStream_t s,
                                  uint64_t* launches);
// With `table` set, the same launch also writes the start table
// (tile_table_size(K) entries) of the first tile pass of the text (levels <=
// 8, one segment) from its leaf histogram.
void launch_tile_block_scan(unsigned long long* blocksum, uint32_t nblocks, uint32_t D, const unsigned long long* hist,
                            uint32_t levels, uint32_t K, bool out, bool tree, uint64_t* table, cudaStream_t s,
                            uint64_t* launches);
// The start table of the first tile pass of a text of any level count (one
// segment: the whole text) from the natural prefix counts of its levels 0..K
// (`flat`: level m at offset 2^m - 1, as launch_fold_levels writes them), so
// that the pass can start before the host plans the later ones.
void launch_tile_first_table(const uint64_t* flat, uint32_t K, bool out, bool tree, uint64_t* table, cudaStream_t s,
                             uint64_t* launches);

// ---- merge of shards (merge.cu) -----------------------------------------------
// A run of one shard's level in the merged level: destination bit `dst`,
// its first bit `src_bit` in the shard's level `src`.  Sorted by dst; no
// empty runs.
struct MergeSeg {
  uint64_t dst;
  uint64_t src_bit;
  const uint64_t* src;
};

// A bit range of a built piece bound for host arrays (semi-external builds):
// `len` bits from bit `src_bit` of `src` go to bit `dst_bit` of a host level;
// the destination words [dst_bit / 64, ceil((dst_bit + len) / 64)) are staged
// from staging word `stage` on, bits outside the range zero.
struct StageSeg {
  const uint64_t* src;
  uint64_t src_bit, dst_bit, len, stage;
};
// Segments sorted by `stage`; total: staging words (the end of the last).
void launch_stage_segments(const StageSeg* segs, uint64_t nseg, uint64_t* staging, uint64_t total, uint32_t* status,
                           cudaStream_t s, uint64_t* launches);
// out[i] = words[idx[i]].
void launch_gather_words(const uint64_t* words, const uint64_t* idx, uint64_t count, uint64_t* out, cudaStream_t s,
                         uint64_t* launches);
// pwm's copy_bits (merge.hpp:19-190) on 64-bit words: whole destination
// words stored, the partial words at the ends OR-ed.
void launch_copy_bits(uint64_t* dst, const uint64_t* src, uint64_t dst_off, uint64_t src_off, uint64_t len,
                      cudaStream_t s);
// One merged level of nbits bits.
void launch_merge_gather(const MergeSeg* segs, uint64_t nseg, uint64_t* dst, uint64_t nbits, uint32_t* status,
                         cudaStream_t s, uint64_t* launches);

// ---- split passes -----------------------------------------------------------
// Geometry of the split pass for a key width: tile size in elements.
uint32_t split_tile_elems(uint32_t key_bytes);
// Dynamic shared memory of one CTA.
size_t split_smem_bytes(uint32_t key_bytes, int K);
void launch_split_pass(uint32_t key_bytes, uint32_t out_bytes, bool huffman, int K, const SplitArgs& a, uint32_t L,
                       cudaStream_t s,
                       uint64_t* launches);
// Plain keys of a batch of texts: args[t] describes text t's pass, its tiles
// are [tile_base[t], tile_base[t+1]) of the launch; counter zeroed.
void launch_split_pass_batched(uint32_t key_bytes, int K, const SplitArgs* args, const uint32_t* tile_base,
                               uint32_t ntexts, uint32_t tiles, uint32_t* counter, cudaStream_t s,
                               uint64_t* launches);

// ---- segmented tile passes (plain keys, matrix and tree together) ------------
// Keys of one tile for a key width.
uint32_t tile_pass_elems(uint32_t key_bytes);
// One pass of K levels over a.tiles tiles; `out`: the pass writes S_{l+K}.
// Digit counts of the passes of a matrix-only build (pass_digits_kernel):
// pass p covers levels level[p]..level[p]+K[p]-1, its natural digit is
// (symbol >> lo[p]) & mask[p].
constexpr uint32_t kPassDigitsMaxPasses = 24;
struct PassDigitsArgs {
  uint32_t npasses, L;
  uint32_t level[kPassDigitsMaxPasses], K[kPassDigitsMaxPasses], lo[kPassDigitsMaxPasses],
      mask[kPassDigitsMaxPasses];
};
// digits: npasses * 16 zeroed counters; done: a zeroed counter; out (device
// view of mapped host memory): flat prefix counts of levels 0..K[0]
// (2^(K[0]+1) - 1 words), the zeros of every level (L words), the status
// word, the digit counts (npasses * 16).
void launch_pass_digits(const void* text, uint64_t n, uint32_t width, const PassDigitsArgs& pd,
                        unsigned long long* digits, unsigned int* done, uint32_t* status, uint64_t* out,
                        cudaStream_t s, uint64_t* launches);

// Every pass's digit counts (16 per pass, pass i at 16 i: the symbols whose
// bits of levels level[i]..level[i]+K[i]-1 read r, level[i]'s most
// significant) from the device prefix counts `flat` of an L-level text
// (level m at 2^m - 1).  digits is zeroed here.  False (nothing launched) for
// more than kPassDigitsMaxPasses passes or K outside 1..4.
bool launch_flat_digits(const uint64_t* flat, uint32_t L, const uint32_t* level, const uint32_t* K, uint32_t count,
                        unsigned long long* digits, cudaStream_t s, uint64_t* launches);

// The narrowest key width (1, 2 or 4 bytes) holding `bits` bits.
uint32_t tile_key_bytes(uint32_t bits);
// One tile pass over keys of key_bytes; a pass writing S_{l+K} (out) writes
// it in keys of out_bytes <= key_bytes, their low bits.
void launch_tile_pass(uint32_t key_bytes, uint32_t out_bytes, int K, bool out, const TileArgs& a, cudaStream_t s,
                      uint64_t* launches);

// ---- wavelet tree from the matrix --------------------------------------------
// Level `m` of the tree: the matrix level with its prefix groups reordered.
// seg_tree/seg_matrix: nseg (>=1) group starts sorted by seg_tree, seg_tree[0] == 0.
void launch_regroup(const uint64_t* matrix_level, uint64_t* tree_level, uint64_t nbits, const uint64_t* seg_tree,
                    const uint64_t* seg_matrix, uint64_t nseg, uint32_t* status, cudaStream_t s, uint64_t* launches);
// The segments of the regroup of levels[0..count) (each 1..23, ascending not
// required) from the device prefix counts `flat` (level m at 2^m - 1, as
// launch_fold_levels writes them): at out + regroup_segs_offset(levels, i),
// level m = levels[i] gets 2^m group starts in the tree level (natural
// prefix order) followed by the 2^m starts of the same groups in the matrix
// level (key order: the bit-reversed prefix), empty groups included.
// scratch: regroup_segs_scratch_words(levels, count) words.  False (nothing
// launched) for more than 32 levels or a level outside 1..31.
uint64_t regroup_segs_words(const uint32_t* levels, uint32_t count);
uint64_t regroup_segs_offset(const uint32_t* levels, uint32_t i);
uint64_t regroup_segs_scratch_words(const uint32_t* levels, uint32_t count);
bool launch_regroup_segs(const uint64_t* flat, const uint32_t* levels, uint32_t count, uint64_t* out,
                         uint64_t* scratch, cudaStream_t s, uint64_t* launches);

// ---- Huffman keys -------------------------------------------------------------
// key = ((code << 1) | 1) << (levels - len) for every text symbol, in keys
// of key_bytes >= (levels + 1) / 8 bytes.
void launch_huffman_keys(const void* text, uint64_t n, uint32_t width, const uint64_t* code_len,
                         const uint64_t* code_word, uint64_t ncodes, uint32_t levels, uint32_t key_bytes, void* keys,
                         uint32_t* status, cudaStream_t s, uint64_t* launches);
// Histogram of the symbols (u64 counts; 8- and 16-bit texts: all 2^8 / 2^16
// values, so hist needs that many entries; 32-bit texts: symbols below nsym)
// and, with `first` (filled with UINT64_MAX), the first position of every
// symbol.  hist must be zeroed.
void launch_symbol_histogram(const void* text, uint64_t n, uint32_t width, uint64_t nsym,
                             unsigned long long* hist, unsigned long long* first, uint32_t* status, cudaStream_t s,
                             uint64_t* launches);

// ---- rank / select --------------------------------------------------------------
struct RankSelectLevel {
  const uint64_t* data;   // level words
  uint64_t nwords;
  uint64_t* l0;           // n0 = nwords / 67108863 + 1 entries
  uint32_t* l12;          // 2 * (nwords / 32 + 1) u32
  uint32_t* s0;           // capacity nwords * 64 / 8192 + 2
  uint32_t* s1;
  unsigned long long* meta;  // [0] ns0, [1] ns1, [2] total ones
};
// Builds pwm's rank/select blocks for `count` levels.  tmp must hold
// max(ceil(nwords/32)) + 1 u32 per level plus per-CTA totals (see .cu).
void launch_rank_select(const RankSelectLevel* host_levels, uint32_t count, RankSelectLevel* dev_levels,
                        uint32_t* tmp, uint64_t tmp_words_per_level, cudaStream_t s, uint64_t* launches);

struct QueryLevel {
  const uint64_t* data;
  uint64_t nwords;
  const uint64_t* l0;
  uint64_t n0;
  const uint32_t* l12;
  const uint32_t* s0;
  const uint32_t* s1;
  const unsigned long long* meta;
};
struct QueryStructure {
  uint32_t levels;
  uint32_t is_tree;
  uint64_t n;
  const QueryLevel* lv;        // device array of `levels`
  const uint64_t* zeros;       // device array of `levels` (matrix)
};
// ops: each query's kind (a mixed batch), or null for `op` throughout.
void launch_queries(const QueryStructure& q, int op, const uint64_t* a, const uint64_t* b, uint64_t count,
                    uint64_t* out, cudaStream_t s, uint64_t* launches, const uint8_t* ops = nullptr);

// Code table of a Huffman-shaped structure, as its queries read it.
struct HuffQueryTables {
  const uint64_t* code_len;    // per symbol (0: no code)
  const uint64_t* code_word;   // per symbol: code_len bits, level 0's bit most significant
  uint64_t nsym;
  const uint64_t* dec_key;     // (length << 56) | word of every code, ascending
  const uint64_t* dec_sym;     // the symbol of dec_key[i]
  uint64_t ndec;
  const uint64_t* level_bits;  // bits of each level
};
void launch_huff_queries(const QueryStructure& q, const HuffQueryTables& h, int op, const uint64_t* a,
                         const uint64_t* b, uint64_t count, uint64_t* out, cudaStream_t s, uint64_t* launches);

// Allocation-free single-level rank/select build on file-scope device arrays
// (see ranksel.cu); limit in words.
uint64_t noalloc_rank_select_max_words();
cudaError_t noalloc_rank_select_build(const uint64_t* words, uint64_t nwords, uint64_t* l0, uint32_t* l12,
                                      uint32_t* s0, uint32_t* s1, unsigned long long* counts, cudaStream_t stream);

// ---- batches -------------------------------------------------------------------------
struct BatchText {
  uint64_t offset;      // first symbol of the text in the concatenated batch
  uint64_t n;           // symbols
  uint32_t levels;
  uint32_t pad;
  uint64_t hist_off;    // 2^levels leaf counts
  uint64_t zeros_off;   // levels matrix zero counts
  uint64_t starts_off;  // run starts of all passes
  uint64_t segs_off;    // tree segments of levels 1..levels-1 (2*(2^levels - 2))
};
struct BatchChunk {
  uint32_t text;
  uint32_t pad;
  uint64_t start;  // symbol offset inside the text
  uint64_t len;
  // Tile batches: the chunk is a block of whole first-pass tiles of 2^log2T
  // symbols (at most 16), whose counts of the pass's finest runs (2^D
  // counters per tile; D = 0: none) go to tilecnt[cnt_off + tile * 2^D +
  // counter], their exclusive prefixes within the block to relpre (same
  // place) and the block's totals to blocksum[blk_off + counter].
  uint64_t cnt_off, blk_off;
  uint32_t D, log2T;
};
struct BatchRegroup {
  const uint64_t* matrix;
  uint64_t* tree;
  uint64_t nbits;
  const uint64_t* seg_tree;
  const uint64_t* seg_matrix;
  uint64_t nseg;
  uint64_t word_begin, word_end;
};
void launch_batch_hist(const void* texts, uint32_t width, const BatchChunk* chunks, uint32_t nchunks,
                       const BatchText* info, unsigned long long* hist, uint32_t* tilecnt, uint32_t* relpre,
                       unsigned long long* blocksum, uint32_t* status, cudaStream_t s, uint64_t* launches);
void launch_batch_tables(const unsigned long long* hist, const BatchText* info, uint32_t ntexts, uint32_t max_levels,
                         int kmax, uint64_t* zeros, uint64_t* starts, uint64_t* segs, cudaStream_t s,
                         uint64_t* launches);
void launch_batch_regroup(const BatchRegroup* items, uint32_t nitems, uint32_t* status, cudaStream_t s,
                          uint64_t* launches);

// ---- generators -------------------------------------------------------------------
void launch_generate(int dist, uint64_t seed, uint64_t param, uint64_t n, uint32_t width, void* out,
                     const uint64_t* thresholds, uint32_t nthr, const uint32_t* perm, cudaStream_t s,
                     uint64_t* launches);

}  // namespace pwmgpu
