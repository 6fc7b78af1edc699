/*
 * pwmgpu.h -- C ABI of the GB300 wavelet tree / wavelet matrix engine.
 *
 * Plain pointers and sizes only.  Every call returns a pwmgpu_status; the
 * text of the last error of a context is available from
 * pwmgpu_ctx_last_error().  All work of a context runs in order on the CUDA
 * stream it was created with.
 *
 * Output layout (identical to pwm's bit_vectors, include/arrays/
 * flat_two_dim_array.hpp:110-213 in kurpicz/pwm): the levels of one
 * structure are contiguous u64 arrays; level l has ceil(bits_l/64) words and
 * is padded to a multiple of 16 words (128 bytes) before level l+1 starts.
 * Position i of a level is bit 63-(i%64) of word i/64; the unused low bits of
 * the last word are zero (include/construction/building_blocks.hpp:18-50).
 * A caller holding a pwm bit_vectors object passes bvs[0].data() as `bv`.
 */
#ifndef PWMGPU_H
#define PWMGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define PWMGPU_API __attribute__((visibility("default")))
#else
#define PWMGPU_API
#endif

typedef enum pwmgpu_status {
  PWMGPU_OK = 0,
  PWMGPU_ERR_ARG = 1,       /* invalid argument: null pointer, width, levels, sizes  */
  PWMGPU_ERR_OOM = 2,       /* a device allocation failed                             */
  PWMGPU_ERR_CUDA = 3,      /* a CUDA runtime call failed                             */
  PWMGPU_ERR_TIMEOUT = 4,   /* a bounded device-side wait gave up (status word set)   */
  PWMGPU_ERR_SYMBOL = 5,    /* a text symbol is >= 2^levels                           */
  PWMGPU_ERR_NO_DEVICE = 6, /* no CUDA device / the library was built for another GPU */
  PWMGPU_ERR_BUSY = 7       /* serving: admission refused (HBM budget or queue full)  */
} pwmgpu_status;

/* Which structures a device build produces. */
#define PWMGPU_MATRIX 0x1u      /* wavelet matrix: bit vectors + zero counts        */
#define PWMGPU_TREE 0x2u        /* levelwise wavelet tree: bit vectors              */
#define PWMGPU_RANK_SELECT 0x4u /* popcount rank/select support for every level     */
#define PWMGPU_HUFFMAN 0x8u     /* Huffman-shaped levels (codes given or built)     */
#define PWMGPU_KEEP_HISTOGRAM 0x10u /* keep the leaf histogram on the host after a build
                                     * (a shard to merge, pwmgpu_wx_merge)              */

/* Query kinds for pwmgpu_wx_query. */
#define PWMGPU_Q_ACCESS 0
#define PWMGPU_Q_RANK 1
#define PWMGPU_Q_SELECT 2

typedef struct pwmgpu_ctx pwmgpu_ctx;
typedef struct pwmgpu_wx pwmgpu_wx;

/* Read-only view of one built structure (device pointers). */
typedef struct pwmgpu_view {
  uint32_t levels;
  uint32_t is_tree;
  uint32_t is_huffman;
  uint32_t has_rank_select;
  uint64_t size;               /* text length n                                   */
  uint64_t total_words;        /* words of the whole level array                  */
  const uint64_t* words;       /* device: all levels, flat padded layout          */
  const uint64_t* level_offset;/* host: word offset of every level (levels)       */
  const uint64_t* level_bits;  /* host: bits of every level (levels)              */
  const uint64_t* zeros;       /* host: zero count per level (matrix), else NULL  */
} pwmgpu_view;

/* ---------------------------------------------------------------------- */
/* Context                                                                 */
/* ---------------------------------------------------------------------- */

/* Creates a context on `device`.  `cuda_stream` is a cudaStream_t to run
 * on, or NULL for a stream owned by the context.  Scratch memory is cached
 * in the context and reused by later builds. */
PWMGPU_API pwmgpu_status pwmgpu_ctx_create(int device, void* cuda_stream, pwmgpu_ctx** out);
PWMGPU_API void pwmgpu_ctx_destroy(pwmgpu_ctx* ctx);
PWMGPU_API const char* pwmgpu_ctx_last_error(const pwmgpu_ctx* ctx);
PWMGPU_API const char* pwmgpu_status_string(pwmgpu_status s);
/* Waits for all work of the context. */
PWMGPU_API pwmgpu_status pwmgpu_ctx_sync(pwmgpu_ctx* ctx);
/* Number of kernels this library launched on the context so far. */
PWMGPU_API uint64_t pwmgpu_ctx_launch_count(const pwmgpu_ctx* ctx);
/* Profiling: while enabled, CUDA events are recorded on the context's stream
 * around every kernel launch group.  pwmgpu_ctx_profile_read synchronises and
 * writes one line per group name, "name groups launches total_ms
 * algorithmic_bytes", then clears the record. */
PWMGPU_API pwmgpu_status pwmgpu_ctx_profile(pwmgpu_ctx* ctx, int enable);
PWMGPU_API pwmgpu_status pwmgpu_ctx_profile_read(pwmgpu_ctx* ctx, char* buf, uint64_t cap);
/* Tuning: levels fused into one split pass (1..4; 0 restores the default).
 * A pass reads its input sequence once and writes the bits of that many
 * levels.  Sets the width of both engines.  Defaults: the tile engine builds
 * a text of up to 7 levels in one pass of all its levels and deeper texts in
 * passes of 4; the warp-pass engine uses passes of 2. */
PWMGPU_API pwmgpu_status pwmgpu_ctx_set_pass_levels(pwmgpu_ctx* ctx, int levels_per_pass);

/* Stream-ordered device allocations (cudaMallocAsync / cudaFreeAsync on the
 * context's stream) for the structures and scratch of this context: freeing
 * does not synchronise the device, so contexts on other streams keep running.
 * Freed memory stays in the process's default pool. */
PWMGPU_API pwmgpu_status pwmgpu_ctx_set_stream_ordered_alloc(pwmgpu_ctx* ctx, int enable);

/* Split engines of plain builds.  TILE (default): CTA-wide splits of whole
 * tiles that write matrix and tree levels together (levels <= 20).  WARP:
 * warp-autonomous split passes that write the matrix, with the tree levels
 * regrouped from it (every plain build; Huffman builds and batches always use
 * it).  Both give identical structures. */
#define PWMGPU_ENGINE_TILE 0
#define PWMGPU_ENGINE_WARP 1
PWMGPU_API pwmgpu_status pwmgpu_ctx_set_engine(pwmgpu_ctx* ctx, int engine);

/* Bytes of text per piece when a pinned host text is uploaded in pieces
 * (default 64 MiB; rounded to the histogram's blocks of 2^18 symbols). */
PWMGPU_API pwmgpu_status pwmgpu_ctx_set_upload_piece_bytes(pwmgpu_ctx* ctx, uint64_t bytes);

/* Host threads that move pageable host buffers (host-to-host builds,
 * downloads) through the context's ring of 4 pinned 16 MiB staging pieces,
 * one piece filled or drained on the host while the copy engine moves the
 * one before: -1 (default) up to 8 threads, as the host has cores; 0 hands
 * pageable buffers to cudaMemcpyAsync unstaged.  Pinned buffers and copies
 * under one piece are never staged. */
PWMGPU_API pwmgpu_status pwmgpu_ctx_set_host_copy_threads(pwmgpu_ctx* ctx, int threads);

/* Chunks (1..16, default 4) in which a host-to-host build with pinned
 * outputs launches its first pass (and later passes of at most 64
 * segments), so that the words each chunk completes go back while the next
 * chunks run; 1 launches each pass whole and streams level groups per pass. */
PWMGPU_API pwmgpu_status pwmgpu_ctx_set_stream_chunks(pwmgpu_ctx* ctx, uint32_t chunks);

/* Bound on the polls of one decoupled look-back wait of the tile engine
 * (each poll sleeps about 64 ns; 0 restores the default of 2^24, about a
 * second).  A wait that runs out records a timeout in the context's status
 * word and the kernel carries on with a zero prefix, so it always returns;
 * the call that reads the status (pwmgpu_wx_check, the host-to-host calls)
 * returns PWMGPU_ERR_TIMEOUT and the context stays usable. */
PWMGPU_API pwmgpu_status pwmgpu_ctx_set_spin_limit(pwmgpu_ctx* ctx, uint32_t polls);

/* Failure injection for tests, on the host side: while enabled, every
 * look-back pass of a device-text plain build is launched without its first
 * tile, so that tile never publishes its counts and the tiles of its segment
 * wait until the spin limit.  The build then reports PWMGPU_ERR_TIMEOUT (its
 * output is undefined, every write stays in bounds).  Off by default. */
PWMGPU_API pwmgpu_status pwmgpu_ctx_test_withhold_tile(pwmgpu_ctx* ctx, int enable);

/* Frees what the context keeps between calls (scratch buffers, cached shard
 * structures of sharded and semi-external builds, pinned staging) after its
 * streams finish; later calls allocate again. */
PWMGPU_API pwmgpu_status pwmgpu_ctx_release_scratch(pwmgpu_ctx* ctx);

/* ---------------------------------------------------------------------- */
/* Drop-in construction (host text in, host bit vectors out)               */
/* ---------------------------------------------------------------------- */

/* Replaces the compute() of pwm's plain construction classes:
 *   wx_ps  include/wx_ps.hpp:37-56      wx_pc   include/wx_pc.hpp:36-57
 *   wx_ppc include/wx_ppc.hpp:36-58     wx_pps  include/wx_pps.hpp:38-69
 *   wx_pc_ss / wx_ppc_ss / wx_dd_ps / wx_dd_pc / wx_dd_pc_ss (same output)
 * `text`: host array of `size` symbols of `word_width` bytes (1, 2, 4, or 5
 * for pwm's packed little-endian uint40_t, registered by pwm for wm_pc /
 * wt_pc: src/register/sequential_prefix_counting.cpp:16-47, widened to 32
 * bits on the device), each < 2^levels.  `bv`: host array of levels * round_up(ceil(size/64), 16)
 * words.  `zeros`: host array of `levels` u64 for a matrix (is_tree == 0),
 * ignored for a tree; all L entries are written, like wx_ps / wx_pc.
 * size == 0 writes nothing (pwm returns an empty structure). */
PWMGPU_API pwmgpu_status pwmgpu_compute(pwmgpu_ctx* ctx, const void* text, uint64_t size, uint32_t word_width,
                                        uint32_t levels, int is_tree, uint64_t* bv, uint64_t* zeros);

/* Canonical Huffman codes of a text, as pwm's histogram +
 * level_sizes_builder + canonical_huff_codes compute them
 * (include/util/histogram.hpp:39-76, include/huffman/
 * huff_level_sizes_builder.hpp:13-46, include/huffman/huff_codes.hpp:
 * 140-285), including pwm's tie-breaking.  Writes max_symbol+1 entries of
 * code_len / code_word (capacity `cap`), the per-level sizes (up to 64) and
 * the number of levels (= longest code). */
PWMGPU_API pwmgpu_status pwmgpu_huffman_codes(pwmgpu_ctx* ctx, const void* text, uint64_t size, uint32_t word_width,
                                              int is_tree, uint64_t* code_len, uint64_t* code_word, uint64_t cap,
                                              uint64_t* num_codes, uint64_t* level_sizes, uint32_t* levels);

/* Replaces the compute() of pwm's Huffman-shaped construction classes:
 *   wx_huff_ps include/wx_huff_ps.hpp:45-79, wx_huff_pc include/wx_huff_pc.hpp:
 *   45-80, wx_huff_naive include/wx_huff_naive.hpp:45-79 (and wx_huff_dd_*).
 * Level l holds bit l of every code longer than l.  The tree orders each level
 * stably by code prefix, the matrix by the previous code bit with finished
 * codes dropped (huff_naive semantics, include/huffman/huff_naive.hpp:19-126);
 * matrix zeros are the 0 bits of each level.  Codes come from the caller
 * (code_len/code_word, num_codes entries, e.g. pwm's own builder) or, when
 * code_len is NULL, from pwmgpu_huffman_codes.  `bv` is laid out with the
 * per-level sizes in `level_sizes`. */
PWMGPU_API pwmgpu_status pwmgpu_compute_huffman(pwmgpu_ctx* ctx, const void* text, uint64_t size, uint32_t word_width,
                                                int is_tree, const uint64_t* code_len, const uint64_t* code_word,
                                                uint64_t num_codes, uint32_t levels, const uint64_t* level_sizes,
                                                uint64_t* bv, uint64_t* zeros);

/* ---------------------------------------------------------------------- */
/* Device-resident structures (batching, serving, benchmarking)            */
/* ---------------------------------------------------------------------- */

/* Allocates device storage for a build of `size` symbols with `levels`
 * levels; shape_flags: PWMGPU_MATRIX and/or PWMGPU_TREE, optionally
 * PWMGPU_RANK_SELECT.  word_width 1, 2, 4 or 5 (40-bit symbols: the builds,
 * host or device text, widen them to 32 bits first). */
PWMGPU_API pwmgpu_status pwmgpu_wx_create(pwmgpu_ctx* ctx, uint64_t size, uint32_t word_width, uint32_t levels,
                                          uint32_t shape_flags, pwmgpu_wx** out);
/* Builds into `wx` from a device text (same size/width/levels as created).
 * Asynchronous on the context's stream; errors detected on the device are
 * reported by the next call that synchronises (pwmgpu_wx_check). */
PWMGPU_API pwmgpu_status pwmgpu_wx_build(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* d_text);
/* Same as pwmgpu_wx_build from a host text (copied in by the library; from
 * pinned host memory in pieces that the histogram follows as they arrive). */
PWMGPU_API pwmgpu_status pwmgpu_wx_build_host(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* host_text);
/* Host text in, host structures out: builds into `wx` and copies the matrix
 * words (wm_bv, with its zeros) and the tree words (wt_bv) in the layout of
 * pwmgpu_wx_download; any output may be NULL.  With pinned host arrays the
 * text is uploaded in pieces and every level group is copied back as soon as
 * its pass completes, overlapping the rest of the build.  Returns when the
 * outputs are on the host. */
PWMGPU_API pwmgpu_status pwmgpu_wx_compute_host(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* host_text,
                                                uint64_t* wm_bv, uint64_t* wm_zeros, uint64_t* wt_bv);
/* Synchronises and reports device-side errors (bad symbol, timeout). */
PWMGPU_API pwmgpu_status pwmgpu_wx_check(pwmgpu_ctx* ctx, pwmgpu_wx* wx);
/* which: 0 = matrix, 1 = tree. */
PWMGPU_API pwmgpu_status pwmgpu_wx_view(const pwmgpu_wx* wx, int which, pwmgpu_view* view);
/* Copies the bit vectors (and matrix zeros) of one structure to the host. */
PWMGPU_API pwmgpu_status pwmgpu_wx_download(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, int which, uint64_t* bv,
                                            uint64_t* zeros);
/* Rank/select blocks of one level, in pwm's layout (bin_rank_popcnt.hpp:
 * 32-86, bin_select_popcnt.hpp:38-107): l0 (u64), l12 (pairs of u32: l1
 * count, three 10-bit l2 counts), select0 and select1 samples (u32).
 * counts receives n_l0, n_l12, n_select0, n_select1.  Any output may be NULL
 * to query the counts. */
PWMGPU_API pwmgpu_status pwmgpu_wx_rank_select_blocks(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, int which,
                                                      uint32_t level, uint64_t* l0, uint32_t* l12, uint32_t* s0,
                                                      uint32_t* s1, uint64_t* counts);
/* Batched queries on device arrays (query_support, include/queries/
 * query_support.hpp:39-178): ACCESS(a[i]) ; RANK(symbol a[i], index b[i]) ;
 * SELECT(symbol a[i], occurrence b[i]).  Needs PWMGPU_RANK_SELECT. */
PWMGPU_API pwmgpu_status pwmgpu_wx_query(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, int which, int op, const uint64_t* d_a,
                                         const uint64_t* d_b, uint64_t count, uint64_t* d_out);
/* The same on host arrays, through the context's scratch and stream;
 * returns when out[] holds the answers. */
PWMGPU_API pwmgpu_status pwmgpu_wx_query_host(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, int which, int op,
                                              const uint64_t* a, const uint64_t* b, uint64_t count, uint64_t* out);
/* A mixed batch on host arrays: query i is of kind ops[i] (PWMGPU_Q_*) with
 * operands a[i], b[i] (b may be NULL when every query is an ACCESS); one
 * upload, one launch, one download.  Plain (not Huffman-shaped) structures. */
PWMGPU_API pwmgpu_status pwmgpu_wx_query_batch_host(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, int which,
                                                    const uint8_t* ops, const uint64_t* a, const uint64_t* b,
                                                    uint64_t count, uint64_t* out);
/* pwm's reduce_alphabet (include/util/alphabet_util.hpp:18-45) on the
 * device: the symbols of d_text renumbered 0, 1, ... in order of first
 * occurrence into d_out (same width; d_out == d_text allowed); *max_char
 * receives the number of distinct symbols - 1, what pwm returns (all ones
 * for an empty text).  8-bit symbol 255 is renumbered like any other (pwm's
 * table stops at 254).  word_width 1, 2, 4 or 5 (pwm's 40-bit uint40_t, packed
 * little-endian); 32-bit symbols from 2^24 up and 40-bit symbols go through a
 * device hash table (texts of at most 2^30 symbols). */
PWMGPU_API pwmgpu_status pwmgpu_reduce_alphabet(pwmgpu_ctx* ctx, const void* d_text, uint64_t size, uint32_t word_width,
                                                void* d_out, uint64_t* max_char);

/* Semi-external construction of a host text larger than the device memory
 * (pwm's semi_in, include/external_memory/semi_in/pc_semi_external.hpp:16-230,
 * which reads its text twice).  The text streams through the GPU in pieces
 * that fit about `device_budget` bytes (0: half the free device memory):
 * once for the leaf histogram, once to build each piece, whose runs go to
 * the host arrays at their global positions.  wm_bv / wt_bv (either may be
 * NULL, not both) receive the structures in the layout of
 * pwmgpu_wx_download (levels of round_up(ceil(size/64), 16) words),
 * wm_zeros (may be NULL) the matrix zeros.  The result equals a plain
 * build's bit for bit.  The budget must hold a piece of 2^16 symbols.  The
 * context keeps the piece buffers for the next call (pwmgpu_ctx_release_scratch
 * frees them). */
PWMGPU_API pwmgpu_status pwmgpu_compute_semi_external(pwmgpu_ctx* ctx, const void* text, uint64_t size,
                                                      uint32_t word_width, uint32_t levels, uint64_t* wm_bv,
                                                      uint64_t* wm_zeros, uint64_t* wt_bv, uint64_t device_budget);

/* Device-resident Huffman-shaped structure: exactly one of PWMGPU_MATRIX or
 * PWMGPU_TREE (pwm's matrix and tree use different codes), optionally
 * PWMGPU_RANK_SELECT, built from a non-empty device text.  Codes come from
 * the caller (code_len/code_word, num_codes entries; levels = the longest
 * code of a symbol that occurs) or, when code_len is NULL, from the builder
 * of pwmgpu_huffman_codes (8- and 16-bit texts).  The levels are those of
 * pwmgpu_compute_huffman (pwmgpu_wx_view / _download read them).  With
 * rank/select, pwmgpu_wx_query answers ACCESS (the symbol), RANK (occurrences
 * before an index, the index clamped to the size) and SELECT (position of the
 * b-th occurrence, b >= 1; all ones when there are fewer; 0 for b = 0) by
 * walking the symbol's code: pwm's query_support has no Huffman queries
 * (include/queries/query_support.hpp:43,55,67 print "NOT YET IMPLEMENTED").
 * Plain builds (pwmgpu_wx_build and the like) refuse such a wx. */
PWMGPU_API pwmgpu_status pwmgpu_wx_build_huffman(pwmgpu_ctx* ctx, const void* d_text, uint64_t size,
                                                 uint32_t word_width, uint32_t shape_flags, const uint64_t* code_len,
                                                 const uint64_t* code_word, uint64_t num_codes, pwmgpu_wx** out);
/* The code table of a Huffman-shaped wx: num_codes receives its entries;
 * code_len / code_word (both or neither) receive them when cap allows. */
PWMGPU_API pwmgpu_status pwmgpu_wx_codes(const pwmgpu_wx* wx, uint64_t* code_len, uint64_t* code_word, uint64_t cap,
                                         uint64_t* num_codes);
PWMGPU_API void pwmgpu_wx_free(pwmgpu_wx* wx);

/* ---------------------------------------------------------------------- */
/* Domain decomposition (pwm's wx_dd_ps / wx_dd_pc: include/wx_dd_ps.hpp:  */
/* 43-120, include/construction/merge.hpp:192-465)                        */
/* ---------------------------------------------------------------------- */
/* Structures built independently from consecutive slices of one text merge
 * into the structures of the whole text, bit for bit those of one build:
 * level l of the result is, block by block in the level's order (prefix
 * order for the tree, bit-reversed prefix order for the matrix), the
 * concatenation of the shards' runs of that block.  shards[i] holds slice i
 * (created with PWMGPU_KEEP_HISTOGRAM and built), all of out's word width and
 * levels and holding the structures out holds; out's size is the sum of
 * theirs; the matrix zeros are summed.  Plain structures of at most 16
 * levels.  Builds out's rank/select support when out has it. */
PWMGPU_API pwmgpu_status pwmgpu_wx_merge(pwmgpu_ctx* ctx, const pwmgpu_wx* const* shards, uint32_t count,
                                         pwmgpu_wx* out);
/* pwmgpu_wx_build of a device text as `shards` slices built one by one and
 * merged (pwm's slices: size/shards symbols, one more for each of the first
 * size%shards). */
PWMGPU_API pwmgpu_status pwmgpu_wx_build_sharded(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* d_text,
                                                 uint32_t shards);
/* pwm's copy_bits (merge.hpp:19-190) on device arrays of 64-bit words: len
 * bits from bit src_off of d_src to bit dst_off of d_dst (bit i is bit
 * 63 - i%64 of word i/64); destination words the range covers whole are
 * stored, the partial words at its ends OR-ed.  Asynchronous on cuda_stream
 * (NULL: the default stream). */
PWMGPU_API pwmgpu_status pwmgpu_copy_bits(uint64_t* d_dst, const uint64_t* d_src, uint64_t dst_off, uint64_t src_off,
                                          uint64_t len, void* cuda_stream);

/* ---------------------------------------------------------------------- */
/* Serving: continuous batching over device-resident structures            */
/* ---------------------------------------------------------------------- */
/* A server runs `slots` worker threads, each with its own context and CUDA
 * stream.  Requests wait in one FIFO queue; the head is admitted when a slot
 * is idle and its device bytes fit the HBM budget beside the resident
 * structures and the requests in flight, so admitted requests overlap on the
 * device.  A build request copies its text, builds the structure(s) with
 * rank/select support, answers its first query batch and leaves the
 * structure resident until pwmgpu_server_release; query requests answer
 * further batches against a resident structure.  Answers are those of the
 * same calls made alone (pwmgpu_wx_create / _build_host / _query_host). */
typedef struct pwmgpu_server pwmgpu_server;
typedef struct {
  const void* text;          /* host symbols; valid until the request is done */
  uint64_t size;             /* symbols (>= 1) */
  uint32_t word_width;       /* 1, 2 or 4 */
  uint32_t levels;           /* 1..24 */
  uint32_t shape_flags;      /* PWMGPU_MATRIX and/or PWMGPU_TREE (rank/select implied) */
  uint32_t query_structure;  /* 0: the matrix answers the queries, 1: the tree */
  uint64_t nqueries;
  const uint8_t* query_ops;  /* PWMGPU_Q_ACCESS / _RANK / _SELECT per query */
  const uint64_t* query_a;   /* access: position; rank, select: symbol */
  const uint64_t* query_b;   /* rank: position; select: occurrence; NULL if only accesses */
  uint64_t* results;         /* host: nqueries answers, valid once the request is done */
} pwmgpu_request;
typedef struct {
  uint64_t id;
  int status;                /* pwmgpu_status of the request */
  uint32_t slot;             /* worker that ran it */
  double submit_s, start_s, done_s;  /* seconds since the server started */
  uint64_t device_bytes;     /* resident bytes the request holds (build requests) */
} pwmgpu_request_info;
typedef struct {
  uint64_t budget_bytes, in_use_bytes, peak_bytes;
  uint64_t queued, running, completed;
} pwmgpu_server_stats_t;

PWMGPU_API pwmgpu_status pwmgpu_server_create(int device, uint64_t hbm_budget_bytes, uint32_t slots,
                                              pwmgpu_server** out);
/* ERR_OOM when the request can never fit the budget. */
PWMGPU_API pwmgpu_status pwmgpu_server_submit(pwmgpu_server* s, const pwmgpu_request* req, uint64_t* id);
PWMGPU_API pwmgpu_status pwmgpu_server_submit_queries(pwmgpu_server* s, uint64_t structure_id,
                                                      uint32_t query_structure, uint64_t nqueries,
                                                      const uint8_t* ops, const uint64_t* a, const uint64_t* b,
                                                      uint64_t* results, uint64_t* id);
/* Blocks until the request is done; returns its status. */
PWMGPU_API pwmgpu_status pwmgpu_server_wait(pwmgpu_server* s, uint64_t id, pwmgpu_request_info* info);
/* ERR_BUSY while the request is queued or running. */
PWMGPU_API pwmgpu_status pwmgpu_server_poll(pwmgpu_server* s, uint64_t id, pwmgpu_request_info* info);
PWMGPU_API const char* pwmgpu_server_error(pwmgpu_server* s, uint64_t id);
/* Done build request: frees its structure (after its query requests);
 * done query request: forgets it. */
PWMGPU_API pwmgpu_status pwmgpu_server_release(pwmgpu_server* s, uint64_t id);
PWMGPU_API pwmgpu_status pwmgpu_server_stats(pwmgpu_server* s, pwmgpu_server_stats_t* stats);
PWMGPU_API void pwmgpu_server_destroy(pwmgpu_server* s);

/* ---------------------------------------------------------------------- */
/* Batches: many independent plain texts built by one CUDA graph           */
/* ---------------------------------------------------------------------- */

/* Texts i = 0..count-1 occupy symbols [offsets[i], offsets[i+1]) of one
 * device buffer of word_width-byte symbols; text i has levels[i] (1..12)
 * levels.  Every text gets a wavelet matrix (PWMGPU_MATRIX is required) and,
 * with PWMGPU_TREE, a levelwise wavelet tree, each bit-identical to a single
 * pwmgpu_compute of that text (pwm's wx_ps::compute, include/wx_ps.hpp:37-56,
 * text by text).
 *
 * Engines (the context's, pwmgpu_ctx_set_engine, at creation): TILE (default)
 * builds every pass of every text in one persistent kernel that takes
 * (text, pass, tile) items from a device work queue, passes of 4 levels, the
 * tables of every pass derived on the device; the tile size of each text
 * (1, 2 or 4 16-byte vectors per thread) is the fastest measured for its
 * (word width, levels, log2 length) class, measured on the first build that
 * meets the class and cached in the context.  WARP runs a kernel per pass
 * shape with passes of levels_per_pass (1..4) levels and regroups the trees
 * from the matrices; levels_per_pass applies to it only. */
typedef struct pwmgpu_batch pwmgpu_batch;
PWMGPU_API pwmgpu_status pwmgpu_batch_create(pwmgpu_ctx* ctx, uint32_t count, const uint64_t* offsets,
                                             const uint32_t* levels, uint32_t word_width, uint32_t shape_flags,
                                             int levels_per_pass, pwmgpu_batch** out);
/* Builds all texts of the batch from the device buffer d_texts.  The first
 * call (and a call with another buffer or pass width) runs the build and
 * records it as a CUDA graph; later calls replay the graph (one graph launch
 * per batch).  Asynchronous; pwmgpu_batch_check synchronises and reports
 * device-side errors. */
PWMGPU_API pwmgpu_status pwmgpu_batch_build(pwmgpu_ctx* ctx, pwmgpu_batch* batch, const void* d_texts);
PWMGPU_API pwmgpu_status pwmgpu_batch_set_levels_per_pass(pwmgpu_batch* batch, int levels_per_pass);
/* Tile engine: every text's tiles take vectors_per_thread (1, 2 or 4) 16-byte
 * vectors per thread instead of the tuned size (0: tuned again); the next
 * build plans and records the batch anew. */
PWMGPU_API pwmgpu_status pwmgpu_batch_set_tile_vectors(pwmgpu_batch* batch, uint32_t vectors_per_thread);
/* The vectors per thread text `index` was built with (0 on the warp engine,
 * or before the first build). */
PWMGPU_API pwmgpu_status pwmgpu_batch_tile_vectors(const pwmgpu_batch* batch, uint32_t index,
                                                   uint32_t* vectors_per_thread);
PWMGPU_API pwmgpu_status pwmgpu_batch_check(pwmgpu_ctx* ctx, pwmgpu_batch* batch);
/* Text `index`'s matrix (which = 0, with its zero counts) or tree (which = 1)
 * in pwm's bit_vectors layout. */
PWMGPU_API pwmgpu_status pwmgpu_batch_download(pwmgpu_ctx* ctx, const pwmgpu_batch* batch, uint32_t index, int which,
                                               uint64_t* bv, uint64_t* zeros);
PWMGPU_API void pwmgpu_batch_free(pwmgpu_batch* batch);
/* Seeded batch of `count` 8-bit texts: log-normal lengths (median 2^16,
 * sigma_ln 1.5, clamped to [2^10, 2^24]); 15% Zipf(1.0) byte texts with 8
 * levels, 85% DNA-like texts over {0..4} (symbol 4 in geometric runs of mean
 * 50, about 2% of the symbols) with 3 levels.  Writes offsets (count+1) and
 * levels (count); texts (offsets[count] bytes) may be NULL to size the batch. */
PWMGPU_API pwmgpu_status pwmgpu_generate_batch(uint64_t seed, uint32_t count, uint64_t* offsets, uint32_t* levels,
                                               uint8_t* texts);

/* Allocation-free rank/select build of one bit vector (device pointers).
 *
 * No counterpart in the reference: pwm builds rank/select support on the
 * host with std::vector.  This entry point exists for callers that cannot
 * allocate device memory while they run -- plugins whose host framework owns
 * every device buffer and hands them in, serving loops that cannot afford an
 * allocator's implicit synchronisation.  It calls no cudaMalloc/cudaFree and
 * needs no context: its scratch is a fixed 4 MiB array in the library's
 * device image, resident on every GPU that loads the library until the
 * process exits.
 *
 * Input: `nwords` words of one level (pwm layout).  Outputs (caller
 * allocated, device memory), identical to pwm's bin_rank_popcnt /
 * bin_select_popcnt blocks and to pwmgpu_wx_rank_select_blocks:
 *   d_l0       nwords/67108863 + 1 u64 (cleared here)
 *   d_l12      2 * (nwords/32 + 1) u32 (for nwords == 0 one zeroed entry)
 *   d_select0, d_select1   nwords*64/8192 + 2 u32 each
 *   d_counts   3 u64: select0 samples, select1 samples, total ones (cleared here)
 * Work is enqueued on `cuda_stream` (NULL: the default stream) of the current
 * device.  The first call on a device looks up the scratch array's device
 * address and keeps it for the life of the process; make that first call
 * before any stream capture, and do not call this entry point again after a
 * cudaDeviceReset.  All calls share the scratch and keep the last call's
 * contents: calls that overlap on the GPU race, so serialise them (one
 * stream, or events).  nwords above PWMGPU_NOALLOC_RS_MAX_WORDS (about 2.1e9
 * bits) returns PWMGPU_ERR_ARG without enqueuing anything. */
#define PWMGPU_NOALLOC_RS_MAX_WORDS 33423360ull
PWMGPU_API pwmgpu_status pwmgpu_rank_select_build_noalloc(const uint64_t* d_words, uint64_t nwords, uint64_t* d_l0,
                                                          uint32_t* d_l12, uint32_t* d_select0, uint32_t* d_select1,
                                                          uint64_t* d_counts, void* cuda_stream);

/* ---------------------------------------------------------------------- */
/* Seeded synthetic texts (counter-based, identical on host and device)     */
/* ---------------------------------------------------------------------- */

#define PWMGPU_GEN_UNIFORM 0   /* uniform over [0, param)                         */
#define PWMGPU_GEN_DNA4 1      /* {0,1,2,3} with p = (0.3, 0.2, 0.2, 0.3)          */
#define PWMGPU_GEN_ZIPF256 2   /* Zipf(1.0) ranks over 256 symbols, permuted       */
#define PWMGPU_GEN_MIX16 3     /* 50/50 uniform u16 / geometric(p=0.01) clamped    */

/* Fills `out` (host when on_device == 0, device otherwise) with n symbols of
 * word_width bytes. */
PWMGPU_API pwmgpu_status pwmgpu_generate(pwmgpu_ctx* ctx, int dist, uint64_t seed, uint64_t param, uint64_t n,
                                         uint32_t word_width, void* out, int on_device);

#ifdef __cplusplus
}
#endif

#endif /* PWMGPU_H */
