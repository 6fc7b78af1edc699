// Internal interface of the engine's host side, shared by its translation
// units: the context and structure types behind the C ABI's opaque handles,
// error handling, allocation of structures and their rank/select storage,
// and the build entry points of each subsystem (plain.cu, huffman.cu,
// shards.cu, batch_host.cu; the C ABI itself is in abi.cu).
#pragma once

#include <algorithm>
#include <array>
#include <functional>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <queue>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/pwmgpu.h"
#include "gen.hpp"
#include "host_huffman.hpp"
#include "host_stream.hpp"
#include "host_tables.hpp"
#include "kernels.cuh"
#include "staging.hpp"

namespace pwmgpu {

constexpr uint32_t kMaxLevels = 64;
constexpr uint32_t kMaxPlainLevels = 24;  // the leaf histogram has 2^L bins
constexpr int kDefaultPassLevels = 2;  // fastest measured width of the warp-pass engine for 8-bit text
constexpr int kDefaultTileLevels = 4;  // levels per segmented tile pass
constexpr uint32_t kSinglePassMaxLevels = 7;  // one tile pass for texts of at most this many levels
constexpr uint32_t kMaxStreamChunks = 16;  // chunks of a pass whose finished words stream to pinned outputs
constexpr uint64_t kAlphabetMaxSymbol = uint64_t(1) << 24;  // 32-bit alphabet reduction: one bin per value below
constexpr uint64_t kAlphabetHashMaxSymbols = uint64_t(1) << 30;  // wider symbols: through a hash table
constexpr uint64_t kStagePiece = uint64_t(16) << 20;  // bytes of one pinned staging piece
constexpr unsigned kStagePieces = 4;                  // pieces in the staging ring
constexpr unsigned kStageAutoThreads = 8;             // host copy threads by default (at most)

struct Fail {
  pwmgpu_status st;
  std::string msg;
};

#define CUDA_TRY(expr)                                                                          \
  do {                                                                                          \
    cudaError_t _e = (expr);                                                                    \
    if (_e != cudaSuccess) {                                                                    \
      throw Fail{_e == cudaErrorMemoryAllocation ? PWMGPU_ERR_OOM : PWMGPU_ERR_CUDA,            \
                 std::string(#expr) + ": " + cudaGetErrorString(_e)};                           \
    }                                                                                           \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct ProfRecord {
  const char* name;
  uint64_t bytes;
  uint64_t launches;
  cudaEvent_t a, b;
};

}  // namespace pwmgpu

using namespace pwmgpu;

struct pwmgpu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  uint64_t launches = 0;
  uint32_t* d_status = nullptr;
  std::map<std::string, DevBuf> scratch;
  int pass_levels = kDefaultPassLevels;
  int tile_levels = 0;  // 0: automatic
  int engine = PWMGPU_ENGINE_TILE;
  uint64_t upload_piece = uint64_t(64) << 20;  // bytes of text per uploaded piece
  uint32_t stream_chunks = 4;                   // chunks of a pass whose words stream to pinned outputs
  uint32_t spin_limit = kSpinLimit;             // polls of one look-back wait of the tile engine
  // batched tile engine: vectors per thread of the tiles of each (key width,
  // levels, log2 length) class, measured on first use
  std::map<uint32_t, uint32_t> batch_tune;
  bool withhold_first_tile = false;             // test hook: look-back passes skip their first tile
  // pageable host buffers move through pinned staging pieces filled and
  // drained by host threads (-1: automatic count, 0: the driver copies them)
  int host_copy_threads = -1;
  std::unique_ptr<CopyPool> copy_pool;
  void* stage = nullptr;
  cudaEvent_t stage_ev[kStagePieces] = {};
  bool async_alloc = false;  // stream-ordered allocations on `stream`
  uint64_t scratch_bytes = 0;
  pwmgpu_wx* compute_cache = nullptr;  // reused by pwmgpu_compute for equal shapes
  std::vector<std::unique_ptr<pwmgpu_wx>> shard_cache;  // reused by pwmgpu_wx_build_sharded
  std::unique_ptr<pwmgpu_wx> semi_shard[2];             // semi-external pieces: full-size and last
  // CUDA-event timing of every launch group while profiling is on
  bool profiling = false;
  std::vector<ProfRecord> prof;
  std::vector<cudaEvent_t> event_pool;
  cudaEvent_t take_event() {
    if (!event_pool.empty()) {
      cudaEvent_t e = event_pool.back();
      event_pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    CUDA_TRY(cudaEventCreate(&e));
    return e;
  }

  // Grow-only pinned host buffer (contents undefined).
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
  void* grow_pinned(size_t bytes) {
    if (pinned_bytes < bytes) {
      if (pinned) {
        CUDA_TRY(cudaStreamSynchronize(stream));
        CUDA_TRY(cudaFreeHost(pinned));
      }
      pinned = nullptr;
      pinned_bytes = 0;
      CUDA_TRY(cudaMallocHost(&pinned, bytes));
      pinned_bytes = bytes;
    }
    return pinned;
  }

  // Grow-only named pinned host buffers (contents undefined); the caller
  // makes sure no copy uses one that grows.
  std::map<std::string, std::pair<void*, size_t>> pinned_named;
  void* grow_pinned_named(const std::string& name, size_t bytes) {
    auto& b = pinned_named[name];
    if (b.second < bytes) {
      if (b.first) CUDA_TRY(cudaFreeHost(b.first));
      b.first = nullptr;
      b.second = 0;
      CUDA_TRY(cudaMallocHost(&b.first, bytes));
      b.second = bytes;
    }
    return b.first;
  }
  // Grow-only host buffer the device writes directly (mapped): results the
  // host waits for that must not queue behind bulk copies.
  void* mapped = nullptr;
  uint64_t* mapped_dev = nullptr;
  size_t mapped_bytes = 0;
  uint64_t* grow_mapped(size_t bytes) {
    if (mapped_bytes < bytes) {
      if (mapped) {
        CUDA_TRY(cudaStreamSynchronize(stream));
        CUDA_TRY(cudaFreeHost(mapped));
      }
      mapped = nullptr;
      mapped_dev = nullptr;
      mapped_bytes = 0;
      CUDA_TRY(cudaHostAlloc(&mapped, bytes, cudaHostAllocMapped));
      void* dp = nullptr;
      CUDA_TRY(cudaHostGetDevicePointer(&dp, mapped, 0));
      mapped_dev = static_cast<uint64_t*>(dp);
      mapped_bytes = bytes;
    }
    return static_cast<uint64_t*>(mapped);
  }
  void release_pinned() {
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    pinned_bytes = 0;
    if (mapped) cudaFreeHost(mapped);
    mapped = nullptr;
    mapped_dev = nullptr;
    mapped_bytes = 0;
    for (auto& kv : pinned_named)
      if (kv.second.first) cudaFreeHost(kv.second.first);
    pinned_named.clear();
  }

  // Grow-only named scratch buffer (contents undefined).
  void* grow(const std::string& name, size_t bytes) {
    auto& b = scratch[name];
    if (b.bytes < bytes) {
      if (b.p) {
        if (async_alloc) {
          CUDA_TRY(cudaFreeAsync(b.p, stream));
        } else {
          CUDA_TRY(cudaStreamSynchronize(stream));
          CUDA_TRY(cudaFree(b.p));
        }
        scratch_bytes -= b.bytes;
      }
      b.p = nullptr;
      b.bytes = 0;
      const size_t want = std::max<size_t>(bytes, 256);
      if (async_alloc) CUDA_TRY(cudaMallocAsync(&b.p, want, stream));
      else CUDA_TRY(cudaMalloc(&b.p, want));
      b.bytes = want;
      scratch_bytes += want;
    }
    return b.p;
  }
  // Transfer streams of host-to-host builds (uploads, downloads) and the
  // events that order them against the main stream; every call that uses
  // them waits for them before it returns, so the events are reused.
  cudaStream_t up = nullptr, down = nullptr;
  // A stream for rank/select of the levels the first passes complete, which
  // runs beside the last pass (integer-bound, while rank/select is
  // memory-bound); created on first use.
  cudaStream_t side = nullptr;
  cudaEvent_t side_go = nullptr, side_done = nullptr;
  void side_init() {
    if (side) return;
    CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&side_go, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&side_done, cudaEventDisableTiming));
  }
  // recorded after the histogram of a build reaches the host
  cudaEvent_t hist_ready = nullptr;
  cudaEvent_t hist_event() {
    if (!hist_ready) CUDA_TRY(cudaEventCreateWithFlags(&hist_ready, cudaEventDisableTiming));
    return hist_ready;
  }
  std::vector<cudaEvent_t> xev;
  size_t xev_used = 0;
  void xfer_init() {
    if (!up) {
      CUDA_TRY(cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking));
      CUDA_TRY(cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking));
    }
    xev_used = 0;
  }
  // an event recorded on `after`'s current work
  cudaEvent_t mark(cudaStream_t after) {
    if (xev_used == xev.size()) {
      cudaEvent_t e;
      CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      xev.push_back(e);
    }
    cudaEvent_t e = xev[xev_used++];
    CUDA_TRY(cudaEventRecord(e, after));
    return e;
  }
  ~pwmgpu_ctx();
};

namespace pwmgpu {

// One built structure (matrix or tree) in device memory.
struct Structure {
  bool present = false;
  bool is_tree = false;
  bool huffman = false;
  uint32_t levels = 0;
  uint64_t n = 0;
  std::vector<uint64_t> bits, offs;
  uint64_t total_words = 0;
  uint64_t* d_words = nullptr;
  std::vector<uint64_t> zeros;   // host (matrix)
  uint64_t* d_zeros = nullptr;   // device copy (matrix), read by queries
  // rank/select
  bool rs = false;
  void* d_rs = nullptr;          // l0, l12, samples and meta of all levels
  size_t rs_bytes = 0;
  std::vector<RankSelectLevel> rs_levels;
  RankSelectLevel* d_rs_levels = nullptr;
  QueryLevel* d_q_levels = nullptr;
  std::vector<QueryLevel> q_host;   // source of the asynchronous copy to d_q_levels
  cudaStream_t alloc_stream = nullptr;  // stream-ordered allocations (nullptr: cudaMalloc)

  void set_layout(const std::vector<uint64_t>& level_bits) {
    levels = uint32_t(level_bits.size());
    bits = level_bits;
    offs.assign(levels, 0);
    uint64_t off = 0;
    for (uint32_t l = 0; l < levels; ++l) { offs[l] = off; off += padded_words(bits[l]); }
    total_words = off;
  }
  void release() {
    auto fr = [&](void* p) {
      if (!p) return;
      if (alloc_stream) cudaFreeAsync(p, alloc_stream);
      else cudaFree(p);
    };
    fr(d_words);
    fr(d_zeros);
    fr(d_rs);
    fr(d_rs_levels);
    fr(d_q_levels);
    d_words = nullptr; d_zeros = nullptr; d_rs = nullptr; d_rs_levels = nullptr; d_q_levels = nullptr;
    rs = false;
    rs_bytes = 0;
  }
};


}  // namespace pwmgpu

struct pwmgpu_wx {
  pwmgpu_ctx* ctx = nullptr;
  uint64_t n = 0;
  uint32_t width = 1;     // key bytes of the build
  uint32_t in_width = 0;  // bytes of an input symbol when they differ (5: pwm's uint40_t, widened to 4)
  uint32_t levels = 0;
  uint32_t flags = 0;
  bool huffman = false;
  Structure wm, wt;
  uint32_t input_width() const { return in_width ? in_width : width; }
  bool wm_internal = false;  // matrix built only as the source of the tree
  bool keep_hist = false;    // PWMGPU_KEEP_HISTOGRAM: the leaf histogram of the last build, for merges
  std::vector<uint64_t> hist;
  // Huffman-shaped: the code table, and its device copy for queries
  std::vector<uint64_t> code_len, code_word;
  uint64_t* d_huff = nullptr;
  HuffQueryTables hq{};
  ~pwmgpu_wx() {
    wm.release();
    wt.release();
    if (d_huff) cudaFree(d_huff);
  }
};

namespace pwmgpu {

inline pwmgpu_status fail(pwmgpu_ctx* ctx, pwmgpu_status st, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return st;
}

template <typename F>
pwmgpu_status guarded(pwmgpu_ctx* ctx, F&& f) {
  try {
    if (ctx) CUDA_TRY(cudaSetDevice(ctx->device));
    return f();
  } catch (const Fail& e) {
    return fail(ctx, e.st, e.msg);
  } catch (const std::bad_alloc&) {
    return fail(ctx, PWMGPU_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {  // nothing else may cross the C ABI
    return fail(ctx, PWMGPU_ERR_CUDA, std::string("host error: ") + e.what());
  }
}

inline bool valid_width(uint32_t w) { return w == 1 || w == 2 || w == 4; }
// Plain builds also take pwm's 40-bit symbols (uint40_t), widened to 32 bits
// on the device first.
inline bool valid_plain_width(uint32_t w) { return valid_width(w) || w == 5; }

// Records CUDA events on the context's stream around one launch group when
// profiling is on; `bytes` is the algorithmic traffic of the group.
struct ProfScope {
  pwmgpu_ctx* ctx;
  ProfRecord rec{};
  uint64_t launches_before = 0;
  ProfScope(pwmgpu_ctx* c, const char* name, uint64_t bytes) : ctx(c) {
    if (!ctx->profiling) return;
    rec.name = name;
    rec.bytes = bytes;
    rec.a = ctx->take_event();
    rec.b = ctx->take_event();
    launches_before = ctx->launches;
    CUDA_TRY(cudaEventRecord(rec.a, ctx->stream));
  }
  ~ProfScope() {
    if (!ctx->profiling || !rec.a) return;
    cudaEventRecord(rec.b, ctx->stream);
    rec.launches = ctx->launches - launches_before;
    ctx->prof.push_back(rec);
  }
};

// ---------------------------------------------------------------------------
// Rank/select storage of a structure
// ---------------------------------------------------------------------------
inline uint64_t rs_n0(uint64_t nwords) { return nwords / (4294967295ull / 64) + 1; }
inline uint64_t rs_n12(uint64_t nwords) { return nwords / 32 + 1; }
inline uint64_t rs_ns(uint64_t nwords) { return nwords * 64 / 8192 + 2; }

// cudaMalloc, or a stream-ordered allocation on `stream` (no device-wide
// synchronisation when freed).
template <typename P>
void dev_alloc(P** p, size_t bytes, cudaStream_t stream) {
  void* v = nullptr;
  if (stream) CUDA_TRY(cudaMallocAsync(&v, bytes, stream));
  else CUDA_TRY(cudaMalloc(&v, bytes));
  *p = static_cast<P*>(v);
}

// ---- structures and rank/select storage (engine.cu) ------------------------
void alloc_rank_select(Structure& s);
void alloc_structure(Structure& s, const std::vector<uint64_t>& level_bits, uint64_t n, bool tree, bool huff,
                     bool rank_select, cudaStream_t alloc_stream = nullptr);
// Rank/select blocks of every level of the given structures (asynchronous),
// all levels in one launch sequence.  share_level0: a plain matrix and tree,
// whose level 0 is the same bit vector: the tree's blocks of level 0 are a
// copy of the matrix's.  Levels [lo, hi) only, on `stream` (default: the
// context's) with scratch buffers named after `tag`.
void build_rank_select(pwmgpu_ctx* ctx, Structure* wm, Structure* wt = nullptr, bool share_level0 = false,
                       uint32_t lo = 0, uint32_t hi = ~0u, cudaStream_t stream = nullptr, const char* tag = "");
uint32_t read_status(pwmgpu_ctx* ctx);
void throw_status(uint32_t st);
void check_device_status(pwmgpu_ctx* ctx);
// The warp-pass matrix passes and the tree regroup, shared by plain and
// Huffman builds (engine.cu).
void run_passes(pwmgpu_ctx* ctx, const void* keys, uint32_t key_bytes, uint32_t text_bytes, bool huff, uint32_t L,
                const std::vector<PassPlan>& plan, const LevelTables& tabs, Structure& wm, Structure* wt);

// ---- plain builds (plain.cu) -------------------------------------------------
void validate_plain(uint64_t n, uint32_t width, uint32_t levels, bool allow40 = false);
// Host ends of a plain build.  `text` (pinned: uploaded in pieces that the
// histogram follows; else in one copy) is copied into the build's device
// text; `wm` / `wt` receive the structures' words in their device layout,
// streamed level group by level group as the passes complete when they are
// pinned, else copied at the end.  The build returns once they are on the
// host.
struct HostIO {
  const void* text = nullptr;
  uint64_t* wm = nullptr;
  uint64_t* wt = nullptr;
};
// Plain build of a wx from a device text (with `io`: from a host text, into
// host arrays; d_text is then the device copy to fill).
void build_plain(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* d_text, const HostIO* io = nullptr);

// Bytes of the narrowest Huffman key holding `bits` bits (1, 2, 4 or 8).
inline uint32_t huff_key_bytes(uint32_t bits) { return bits <= 8 ? 1u : bits <= 16 ? 2u : bits <= 32 ? 4u : 8u; }

// ---- host copies (staging.cu) -----------------------------------------------------
bool host_pinned(const void* p);
// Host to device on `s`; returns once `h_src` may be reused.  Pageable
// memory of a piece or more goes through the pinned staging ring.
void host_to_device(pwmgpu_ctx* ctx, void* d_dst, const void* h_src, uint64_t bytes, cudaStream_t s);
// Device to host after the work on `s`; returns once `h_dst` holds the bytes.
void device_to_host(pwmgpu_ctx* ctx, void* h_dst, const void* d_src, uint64_t bytes, cudaStream_t s);
void release_staging(pwmgpu_ctx* ctx);

// ---- Huffman-shaped builds (huffman.cu) ------------------------------------------
// Symbol histogram + first occurrences of a device text on the GPU, then the
// code table on the host.
HuffCodes huffman_codes_device(pwmgpu_ctx* ctx, const void* d_text, uint64_t n, uint32_t width, bool is_tree,
                               uint64_t* max_symbol_out);
// Huffman build of one structure (matrix, or tree through the matrix).
void build_huffman(pwmgpu_ctx* ctx, const void* d_text, uint64_t n, uint32_t width, bool is_tree,
                   const std::vector<uint64_t>& code_len, const std::vector<uint64_t>& code_word, uint32_t levels,
                   Structure& wm, Structure* wt, bool rank_select);

// ---- shards, semi-external builds, alphabet reduction (shards.cu) -----------------
std::unique_ptr<pwmgpu_wx> make_wx(pwmgpu_ctx* ctx, uint64_t size, uint32_t word_width, uint32_t levels,
                                   uint32_t shape_flags);
void semi_external(pwmgpu_ctx* ctx, const void* text, uint64_t n, uint32_t width, uint32_t L, uint64_t* out_wm,
                   uint64_t* wm_zeros, uint64_t* out_wt, uint64_t budget);
const void* build_input(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, const void* d_text);
const void* upload_wide_host_text(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, const void* host_text);
void merge_shards(pwmgpu_ctx* ctx, const std::vector<const pwmgpu_wx*>& sh, pwmgpu_wx* out);
uint64_t reduce_alphabet_hashed(pwmgpu_ctx* ctx, const void* d_text, uint64_t n, uint32_t width, void* d_out);

}  // namespace pwmgpu
