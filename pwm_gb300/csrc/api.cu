// C ABI of the engine (include/pwmgpu.h): contexts, device-resident
// structures, the drop-in host-to-host constructions, the Huffman code
// builder, queries and generators.
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

using namespace pwmgpu;

namespace {

constexpr uint32_t kMaxLevels = 64;
constexpr uint32_t kMaxPlainLevels = 24;  // the leaf histogram has 2^L bins
constexpr int kDefaultPassLevels = 2;  // fastest measured width of the warp-pass engine for 8-bit text
constexpr int kDefaultTileLevels = 4;  // levels per segmented tile pass
constexpr uint32_t kSinglePassMaxLevels = 7;  // one tile pass for texts of at most this many levels

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

}  // namespace

namespace {
struct ProfRecord {
  const char* name;
  uint64_t bytes;
  uint64_t launches;
  cudaEvent_t a, b;
};
}  // namespace

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
  bool withhold_first_tile = false;             // test hook: look-back passes skip their first tile
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

namespace {

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

}  // namespace

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

pwmgpu_ctx::~pwmgpu_ctx() {
  cudaSetDevice(device);
  delete compute_cache;
  shard_cache.clear();  // structures free on the context's stream: before it goes
  semi_shard[0].reset();
  semi_shard[1].reset();
  for (auto& r : prof) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  for (auto e : event_pool) cudaEventDestroy(e);
  if (async_alloc && stream) cudaStreamSynchronize(stream);
  for (auto& kv : scratch)
    if (kv.second.p) {
      if (async_alloc) cudaFreeAsync(kv.second.p, stream);
      else cudaFree(kv.second.p);
    }
  if (async_alloc && stream) cudaStreamSynchronize(stream);
  if (d_status) cudaFree(d_status);
  for (cudaStream_t t : {up, down, side})
    if (t) cudaStreamSynchronize(t);
  release_pinned();
  for (cudaStream_t t : {up, down, side})
    if (t) {
      cudaStreamSynchronize(t);
      cudaStreamDestroy(t);
    }
  if (side_go) cudaEventDestroy(side_go);
  if (side_done) cudaEventDestroy(side_done);
  for (auto e : xev) cudaEventDestroy(e);
  if (hist_ready) cudaEventDestroy(hist_ready);
  if (own_stream && stream) cudaStreamDestroy(stream);
}

namespace {

pwmgpu_status fail(pwmgpu_ctx* ctx, pwmgpu_status st, const std::string& msg) {
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
  }
}

bool valid_width(uint32_t w) { return w == 1 || w == 2 || w == 4; }
// Plain builds also take pwm's 40-bit symbols (uint40_t), widened to 32 bits
// on the device first.
bool valid_plain_width(uint32_t w) { return valid_width(w) || w == 5; }

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
uint64_t rs_n0(uint64_t nwords) { return nwords / (4294967295ull / 64) + 1; }
uint64_t rs_n12(uint64_t nwords) { return nwords / 32 + 1; }
uint64_t rs_ns(uint64_t nwords) { return nwords * 64 / 8192 + 2; }

// cudaMalloc, or a stream-ordered allocation on `stream` (no device-wide
// synchronisation when freed).
template <typename P>
void dev_alloc(P** p, size_t bytes, cudaStream_t stream) {
  void* v = nullptr;
  if (stream) CUDA_TRY(cudaMallocAsync(&v, bytes, stream));
  else CUDA_TRY(cudaMalloc(&v, bytes));
  *p = static_cast<P*>(v);
}

void alloc_rank_select(Structure& s) {
  size_t bytes = 0;
  std::vector<size_t> off0(s.levels), off12(s.levels), offs0(s.levels), offs1(s.levels), offm(s.levels);
  auto take = [&](size_t b) {
    size_t o = bytes;
    bytes += (b + 255) & ~size_t(255);
    return o;
  };
  for (uint32_t l = 0; l < s.levels; ++l) {
    const uint64_t nw = words_for(s.bits[l]);
    off0[l] = take(rs_n0(nw) * 8);
    off12[l] = take(rs_n12(nw) * 8);
    offs0[l] = take(rs_ns(nw) * 4);
    offs1[l] = take(rs_ns(nw) * 4);
    offm[l] = take(3 * 8);
  }
  s.rs_bytes = std::max<size_t>(bytes, 256);
  dev_alloc(&s.d_rs, s.rs_bytes, s.alloc_stream);
  char* base = static_cast<char*>(s.d_rs);
  s.rs_levels.resize(s.levels);
  s.q_host.assign(s.levels, QueryLevel{});
  auto& q = s.q_host;
  for (uint32_t l = 0; l < s.levels; ++l) {
    auto& r = s.rs_levels[l];
    r.data = s.d_words + s.offs[l];
    r.nwords = words_for(s.bits[l]);
    r.l0 = reinterpret_cast<uint64_t*>(base + off0[l]);
    r.l12 = reinterpret_cast<uint32_t*>(base + off12[l]);
    r.s0 = reinterpret_cast<uint32_t*>(base + offs0[l]);
    r.s1 = reinterpret_cast<uint32_t*>(base + offs1[l]);
    r.meta = reinterpret_cast<unsigned long long*>(base + offm[l]);
    q[l] = QueryLevel{r.data, r.nwords, r.l0, rs_n0(r.nwords), r.l12, r.s0, r.s1, r.meta};
  }
  const size_t nl = std::max<uint32_t>(s.levels, 1);
  dev_alloc(&s.d_rs_levels, sizeof(RankSelectLevel) * nl, s.alloc_stream);
  dev_alloc(&s.d_q_levels, sizeof(QueryLevel) * nl, s.alloc_stream);
  if (s.levels) {
    if (s.alloc_stream) {  // the host vectors live as long as the structure
      CUDA_TRY(cudaMemcpyAsync(s.d_rs_levels, s.rs_levels.data(), sizeof(RankSelectLevel) * s.levels,
                               cudaMemcpyHostToDevice, s.alloc_stream));
      CUDA_TRY(cudaMemcpyAsync(s.d_q_levels, q.data(), sizeof(QueryLevel) * s.levels, cudaMemcpyHostToDevice,
                               s.alloc_stream));
    } else {
      CUDA_TRY(cudaMemcpy(s.d_rs_levels, s.rs_levels.data(), sizeof(RankSelectLevel) * s.levels,
                          cudaMemcpyHostToDevice));
      CUDA_TRY(cudaMemcpy(s.d_q_levels, q.data(), sizeof(QueryLevel) * s.levels, cudaMemcpyHostToDevice));
    }
  }
  s.rs = true;
}

void alloc_structure(Structure& s, const std::vector<uint64_t>& level_bits, uint64_t n, bool tree, bool huff,
                     bool rank_select, cudaStream_t alloc_stream = nullptr) {
  s.release();
  s.alloc_stream = alloc_stream;
  s.present = true;
  s.is_tree = tree;
  s.huffman = huff;
  s.n = n;
  s.set_layout(level_bits);
  dev_alloc(&s.d_words, std::max<uint64_t>(s.total_words, 16) * 8, alloc_stream);
  // padding bits and words are never written by a build: zero from here on
  if (alloc_stream) CUDA_TRY(cudaMemsetAsync(s.d_words, 0, std::max<uint64_t>(s.total_words, 16) * 8, alloc_stream));
  else CUDA_TRY(cudaMemset(s.d_words, 0, std::max<uint64_t>(s.total_words, 16) * 8));
  dev_alloc(&s.d_zeros, std::max<uint32_t>(s.levels, 1) * 8, alloc_stream);
  if (rank_select) alloc_rank_select(s);
}

// Rank/select blocks of every level of the given structures (asynchronous),
// all levels in one launch sequence.  share_level0: a plain matrix and tree,
// whose level 0 is the same bit vector: the tree's blocks of level 0 are a
// copy of the matrix's.  The kernels write every entry that is read (l0 is
// cleared by the scan kernel), so nothing is zeroed first.
//
// Levels [lo, hi) only, on `stream` (default: the context's) with scratch
// buffers named after `tag` (so that two groups can run at once); only the
// context's stream is profiled.
void build_rank_select(pwmgpu_ctx* ctx, Structure* wm, Structure* wt = nullptr, bool share_level0 = false,
                       uint32_t lo = 0, uint32_t hi = ~0u, cudaStream_t stream = nullptr, const char* tag = "") {
  std::vector<RankSelectLevel> lv;
  auto add = [&](const Structure* st, uint32_t from) {
    for (uint32_t l = std::max(lo, from); l < std::min(hi, st->levels); ++l) lv.push_back(st->rs_levels[l]);
  };
  if (wm && wm->rs) add(wm, 0);
  const bool copy0 = share_level0 && lo == 0 && hi > 0 && wm && wm->rs && wm->levels && wt && wt->rs && wt->levels;
  if (wt && wt->rs) add(wt, copy0 ? 1 : 0);
  if (lv.empty() && !copy0) return;
  cudaStream_t s = stream ? stream : ctx->stream;
  const std::string t(tag);
  if (!lv.empty()) {
    auto* d_lv = static_cast<RankSelectLevel*>(ctx->grow("rs_levels" + t, lv.size() * sizeof(RankSelectLevel)));
    CUDA_TRY(cudaMemcpyAsync(d_lv, lv.data(), lv.size() * sizeof(RankSelectLevel), cudaMemcpyHostToDevice, s));
    uint64_t max_real = 0, bytes = 0;
    for (auto& r : lv) {
      max_real = std::max<uint64_t>(max_real, (r.nwords + 31) / 32);
      bytes += r.nwords * 8 + (r.nwords / 32 + 1) * 8;
    }
    const uint64_t stride = max_real + (max_real + 255) / 256 + 1;
    uint32_t* tmp = static_cast<uint32_t*>(ctx->grow("rs_tmp" + t, std::max<uint64_t>(stride * lv.size() * 4, 256)));
    if (s == ctx->stream) {
      ProfScope ps(ctx, "rank_select", bytes);
      launch_rank_select(lv.data(), uint32_t(lv.size()), d_lv, tmp, stride, s, &ctx->launches);
    } else {
      launch_rank_select(lv.data(), uint32_t(lv.size()), d_lv, tmp, stride, s, &ctx->launches);
    }
  }
  if (copy0) {  // l0, l12, samples and meta of level 0 lie in this order in both structures
    const RankSelectLevel &a = wm->rs_levels[0], &b = wt->rs_levels[0];
    const size_t n = size_t(reinterpret_cast<const char*>(a.meta + 3) - reinterpret_cast<const char*>(a.l0));
    CUDA_TRY(cudaMemcpyAsync(b.l0, a.l0, n, cudaMemcpyDeviceToDevice, s));
  }
}

uint32_t read_status(pwmgpu_ctx* ctx) {
  uint32_t st = 0;
  CUDA_TRY(cudaMemcpyAsync(&st, ctx->d_status, 4, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return st;
}

void throw_status(uint32_t st) {
  if (st & kErrSymbol) throw Fail{PWMGPU_ERR_SYMBOL, "a text symbol is >= 2^levels (or has no Huffman code)"};
  if (st & kErrTimeout) throw Fail{PWMGPU_ERR_TIMEOUT, "a device-side look-back wait gave up"};
  if (st & kErrBounds) throw Fail{PWMGPU_ERR_CUDA, "a device-side bounds check tripped"};
}

void check_device_status(pwmgpu_ctx* ctx) { throw_status(read_status(ctx)); }

// ---------------------------------------------------------------------------
// The matrix passes and the tree regroup, shared by plain and Huffman builds
// ---------------------------------------------------------------------------
// keys: the level-0 sequence (text or Huffman keys) of `key_bytes` per
// element.  Builds the matrix levels into `wm` and, if wanted, the tree
// levels into `wt`.
void run_passes(pwmgpu_ctx* ctx, const void* keys, uint32_t key_bytes, uint32_t text_bytes, bool huff, uint32_t L,
                const std::vector<PassPlan>& plan, const LevelTables& tabs, Structure& wm, Structure* wt) {
  cudaStream_t s = ctx->stream;
  // Device copies of the per-pass run starts.
  size_t start_words = 0;
  for (auto& st : tabs.starts) start_words += st.size();
  std::vector<uint64_t> flat_starts;
  flat_starts.reserve(start_words);
  for (auto& st : tabs.starts) flat_starts.insert(flat_starts.end(), st.begin(), st.end());
  uint64_t* d_starts = static_cast<uint64_t*>(ctx->grow("starts", std::max<size_t>(start_words, 1) * 8));
  CUDA_TRY(cudaMemcpyAsync(d_starts, flat_starts.data(), start_words * 8, cudaMemcpyHostToDevice, s));

  // Inner levels of a pass are written with OR at run edges: zero them.
  for (const auto& p : plan)
    for (int j = 1; j < p.K; ++j) {
      const uint32_t m = p.level + uint32_t(j);
      CUDA_TRY(cudaMemsetAsync(wm.d_words + wm.offs[m], 0, words_for(wm.bits[m]) * 8, s));
    }

  const uint64_t n0 = tabs.level_bits.empty() ? 0 : tabs.level_bits[0];
  const uint32_t T = split_tile_elems(key_bytes);
  void* ping = ctx->grow("keys_a", std::max<uint64_t>(n0, 1) * key_bytes);
  void* pong = ctx->grow("keys_b", std::max<uint64_t>(n0, 1) * key_bytes);
  const void* in = keys;
  size_t start_off = 0;
  for (size_t pi = 0; pi < plan.size(); ++pi) {
    const auto& p = plan[pi];
    const uint64_t m = tabs.level_bits[p.level];
    const uint32_t tiles = uint32_t((m + T - 1) / T);
    const int nlb = huff ? (2 << p.K) - 2 : (1 << p.K);
    auto* lb = static_cast<unsigned long long*>(ctx->grow("lookback", std::max<uint64_t>(tiles, 1) * nlb * 8 + 64));
    uint32_t* counter = reinterpret_cast<uint32_t*>(lb + uint64_t(std::max<uint32_t>(tiles, 1)) * nlb);
    CUDA_TRY(cudaMemsetAsync(lb, 0, uint64_t(std::max<uint32_t>(tiles, 1)) * nlb * 8 + 64, s));
    SplitArgs a{};
    a.in = in;
    a.out = p.has_out ? (in == ping ? pong : ping) : nullptr;
    a.m = m;
    a.level = p.level;
    a.levels_here = uint32_t(p.K);
    for (int j = 0; j < p.K; ++j) a.bv[j] = wm.d_words + wm.offs[p.level + j];
    a.tree_level0 = (wt && p.level == 0) ? wt->d_words : nullptr;
    a.starts = d_starts + start_off;
    a.lookback = lb;
    a.tile_counter = counter;
    a.status = ctx->d_status;
    a.tiles = tiles;
    a.L = L;
    for (int j = 0; j <= p.K; ++j)
      a.level_size[j] = p.level + j < L ? tabs.level_bits[p.level + j] : 0;
    {
      uint64_t bytes = 0;
      for (int j = 0; j < p.K; ++j) {
        const uint64_t mj = tabs.level_bits[p.level + j];
        bytes += mj * text_bytes + words_for(mj) * 8;
      }
      ProfScope ps(ctx, "split_pass", bytes);
      launch_split_pass(key_bytes, huff, p.K, a, L, s, &ctx->launches);
    }
    CUDA_TRY(cudaGetLastError());
    start_off += tabs.starts[pi].size();
    if (p.has_out) in = a.out;
  }

  if (wt) {
    // Tree levels 1..L-1: the matrix level with its prefix groups reordered.
    size_t seg_words = 0;
    for (uint32_t m = 1; m < L; ++m) seg_words += 2 * tabs.seg_tree[m].size();
    std::vector<uint64_t> segs;
    segs.reserve(seg_words);
    for (uint32_t m = 1; m < L; ++m) {
      segs.insert(segs.end(), tabs.seg_tree[m].begin(), tabs.seg_tree[m].end());
      segs.insert(segs.end(), tabs.seg_matrix[m].begin(), tabs.seg_matrix[m].end());
    }
    uint64_t* d_segs = static_cast<uint64_t*>(ctx->grow("segs", std::max<size_t>(seg_words, 1) * 8));
    if (seg_words) CUDA_TRY(cudaMemcpyAsync(d_segs, segs.data(), seg_words * 8, cudaMemcpyHostToDevice, s));
    size_t off = 0;
    for (uint32_t m = 1; m < L; ++m) {
      const uint64_t ns = tabs.seg_tree[m].size();
      ProfScope ps(ctx, "regroup", 2 * words_for(wm.bits[m]) * 8);
      launch_regroup(wm.d_words + wm.offs[m], wt->d_words + wt->offs[m], wm.bits[m], d_segs + off, d_segs + off + ns,
                     ns, ctx->d_status, s, &ctx->launches);
      off += 2 * ns;
    }
    CUDA_TRY(cudaGetLastError());
  }
  // (copies from pageable host vectors return once the data is staged, so
  // the plan may go out of scope with the passes still running)
}

// ---------------------------------------------------------------------------
// Plain builds through the segmented tile passes: every pass writes its
// matrix levels, and its tree levels when its segments are prefix groups;
// the remaining tree levels come from the regroup.
// ---------------------------------------------------------------------------
struct TileFirstPass {
  const unsigned long long* blockpre = nullptr;
  const uint32_t* relpre = nullptr;
  const uint32_t* tilecnt = nullptr;
  uint32_t tiles_per_block = 0;
  bool level0_written = false;  // the histogram kernel wrote level 0 of both structures
};

// Device descriptors of passes [from, to): per pass its segments, its level
// descriptor and its start tables, at offsets of one uploaded blob.
struct TileBlob {
  std::vector<unsigned char> bytes;
  std::vector<size_t> segs, text, table;  // indexed by pass
};

TileBlob tile_blob(const std::vector<TilePassHost>& passes, size_t from, size_t to, uint32_t L, uint64_t n,
                   const Structure& wm, const Structure* wt) {
  TileBlob b;
  b.segs.assign(passes.size(), 0);
  b.text.assign(passes.size(), 0);
  b.table.assign(passes.size(), 0);
  auto align16 = [&]() { b.bytes.resize((b.bytes.size() + 15) & ~size_t(15)); };
  auto put = [&](const void* p, size_t bytes) {
    const auto* c = static_cast<const unsigned char*>(p);
    b.bytes.insert(b.bytes.end(), c, c + bytes);
  };
  const uint64_t stride = L > 1 ? wm.offs[1] - wm.offs[0] : padded_words(n);
  for (size_t pi = from; pi < to; ++pi) {
    const auto& p = passes[pi];
    align16();
    b.segs[pi] = b.bytes.size();
    for (const auto& h : p.segs) {
      TileSeg d{h.in_begin, h.m, h.table, h.tile0, h.text};
      put(&d, sizeof d);
    }
    align16();
    b.text[pi] = b.bytes.size();
    TileText tx{};
    tx.wm = wm.d_words + wm.offs[p.level];
    tx.wt = (wt && p.segmented) ? wt->d_words + wt->offs[p.level] : nullptr;
    tx.stride = stride;
    tx.nbits = n;
    tx.shift = L - 1 - p.level;
    put(&tx, sizeof tx);
    align16();
    b.table[pi] = b.bytes.size();
    put(p.table.data(), p.table.size() * 8);
  }
  if (b.bytes.empty()) b.bytes.resize(16);
  return b;
}

// Enqueues pass pi (descriptors at d_blob) reading `in`; returns the keys it
// writes for the next pass.  Edge words are OR-ed, so a pass's levels must be
// zero: the first pass's are zeroed by the caller (or by the histogram
// kernel), every other pass's by the pass before it, a slab per tile.  Only
// level and width of passes[pi + 1] are read.
//
// bounds: tile boundaries 0 = t_0 < t_1 < ... = tiles of separate launches
// (chunks, for streaming the finished words of each); after_chunk(c) runs on
// the host once chunk c is enqueued.
const void* enqueue_tile_pass(pwmgpu_ctx* ctx, const std::vector<TilePassHost>& passes, size_t pi,
                              const unsigned char* d_blob, const TileBlob& blob, const void* in, uint32_t width,
                              uint64_t n, Structure& wm, Structure* wt, const TileFirstPass* first,
                              const std::vector<uint32_t>& bounds = {},
                              const std::function<void(size_t)>& after_chunk = {}) {
  cudaStream_t s = ctx->stream;
  const auto& p = passes[pi];
  void* ping = ctx->grow("keys_a", std::max<uint64_t>(n, 1) * width);
  void* pong = ctx->grow("keys_b", std::max<uint64_t>(n, 1) * width);
  const int D = p.out ? p.K : p.K - 1;
  const uint64_t nlb = uint64_t(1) << D;
  const uint64_t lb_bytes = uint64_t(std::max<uint32_t>(p.tiles, 1)) * nlb * 8;
  auto* lb = static_cast<unsigned long long*>(ctx->grow("lookback", lb_bytes + 64));
  // with given prefixes the pass reads only its tile counter
  const bool given = pi == 0 && first && p.segs.size() == 1;
  if (given) CUDA_TRY(cudaMemsetAsync(reinterpret_cast<unsigned char*>(lb) + lb_bytes, 0, 64, s));
  else CUDA_TRY(cudaMemsetAsync(lb, 0, lb_bytes + 64, s));
  TileArgs a{};
  a.in = in;
  a.out = p.out ? (in == ping ? pong : ping) : nullptr;
  a.out_size = p.out ? n : 0;
  a.segs = reinterpret_cast<const TileSeg*>(d_blob + blob.segs[pi]);
  a.texts = reinterpret_cast<const TileText*>(d_blob + blob.text[pi]);
  a.tables = reinterpret_cast<const uint64_t*>(d_blob + blob.table[pi]);
  a.lookback = lb;
  a.tile_counter = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(lb) + lb_bytes);
  a.status = ctx->d_status;
  a.nsegs = uint32_t(p.segs.size());
  a.tiles = p.tiles;
  if (pi + 1 < passes.size()) {
    const auto& q = passes[pi + 1];
    const uint32_t l1 = q.level + q.K - 1;
    a.zero_a = wm.d_words + wm.offs[q.level];
    a.zero_b = wt ? wt->d_words + wt->offs[q.level] : nullptr;
    a.zero_words = (l1 + 1 < wm.levels ? wm.offs[l1 + 1] : wm.total_words) - wm.offs[q.level];
    const uint64_t per = (a.zero_words + p.tiles - 1) / std::max<uint32_t>(p.tiles, 1);
    a.zero_per_tile = uint32_t((per + 1) & ~uint64_t(1));
  }
  if (given) {
    a.blockpre = first->blockpre;
    a.relpre = first->relpre;
    a.tilecnt = first->tilecnt;
    a.tiles_per_block = first->tiles_per_block;
    a.first_level_written = first->level0_written ? 1u : 0u;
  }
  if (pi == 0 && first) a.clear_edges = 1u;  // the histogram kernel did not zero the first pass's levels
  a.spin_limit = ctx->spin_limit;
  std::vector<uint32_t> b = bounds.size() >= 2 ? bounds : std::vector<uint32_t>{0, p.tiles};
  if (ctx->withhold_first_tile && !given && p.tiles >= 2 && bounds.size() < 2) b = {1, p.tiles};  // tile 0 never publishes
  const uint64_t structs = (wt && p.segmented) ? 2 : 1;
  const uint64_t skipped = a.first_level_written ? structs * words_for(n) * 8 : 0;
  const uint64_t bytes = structs * uint64_t(p.K) * (n * width + words_for(n) * 8) - skipped;
  for (size_t c = 0; c + 1 < b.size(); ++c) {
    if (c) CUDA_TRY(cudaMemsetAsync(a.tile_counter, 0, 4, s));
    a.tile_base = b[c];
    a.launch_tiles = b[c + 1] - b[c];
    {
      ProfScope ps(ctx, "split_pass", p.tiles ? bytes * a.launch_tiles / p.tiles : 0);
      launch_tile_pass(width, p.K, p.out, a, s, &ctx->launches);
    }
    CUDA_TRY(cudaGetLastError());
    if (after_chunk) after_chunk(c);
  }
  return p.out ? a.out : in;
}

// Passes launched in chunks of tiles: bounds(pi) gives pass pi's tile bounds
// (empty: one launch), after(pi, c) runs on the host once chunk c of pass pi
// is enqueued.
struct PassChunks {
  std::function<std::vector<uint32_t>(size_t)> bounds;
  std::function<void(size_t, size_t)> after;
};

// Passes [from, passes.size()) and the regroup; `in` is the input of pass
// `from` (the text for pass 0).  after_pass(i) runs on the host once pass i
// is enqueued, and after_pass(passes.size()) once the regroup is.
void run_tile_passes(pwmgpu_ctx* ctx, const void* in, uint32_t width, uint32_t L,
                     const std::vector<TilePassHost>& passes, const std::vector<uint32_t>& regroup,
                     const LevelTables& tabs, Structure& wm, Structure* wt, const TileFirstPass* first = nullptr,
                     const std::function<void(size_t)>& after_pass = {}, size_t from = 0,
                     const PassChunks* chunks = nullptr) {
  cudaStream_t s = ctx->stream;
  const uint64_t n = tabs.level_bits.empty() ? 0 : tabs.level_bits[0];
  const TileBlob blob = tile_blob(passes, from, passes.size(), L, n, wm, wt);
  auto* d_blob = static_cast<unsigned char*>(ctx->grow("tile_plan", blob.bytes.size()));
  CUDA_TRY(cudaMemcpyAsync(d_blob, blob.bytes.data(), blob.bytes.size(), cudaMemcpyHostToDevice, s));
  for (size_t pi = from; pi < passes.size(); ++pi) {
    std::vector<uint32_t> bounds;
    std::function<void(size_t)> after_chunk;
    if (chunks && chunks->bounds) bounds = chunks->bounds(pi);
    if (chunks && chunks->after) after_chunk = [chunks, pi](size_t c) { chunks->after(pi, c); };
    in = enqueue_tile_pass(ctx, passes, pi, d_blob, blob, in, width, n, wm, wt, first, bounds, after_chunk);
    if (after_pass) after_pass(pi);
  }

  if (wt && !regroup.empty()) {
    size_t seg_words = 0;
    for (uint32_t m : regroup) seg_words += 2 * tabs.seg_tree[m].size();
    std::vector<uint64_t> segs;
    segs.reserve(seg_words);
    for (uint32_t m : regroup) {
      segs.insert(segs.end(), tabs.seg_tree[m].begin(), tabs.seg_tree[m].end());
      segs.insert(segs.end(), tabs.seg_matrix[m].begin(), tabs.seg_matrix[m].end());
    }
    uint64_t* d_segs = static_cast<uint64_t*>(ctx->grow("segs", std::max<size_t>(seg_words, 1) * 8));
    CUDA_TRY(cudaMemcpyAsync(d_segs, segs.data(), seg_words * 8, cudaMemcpyHostToDevice, s));
    size_t off = 0;
    for (uint32_t m : regroup) {
      const uint64_t ns = tabs.seg_tree[m].size();
      ProfScope ps(ctx, "regroup", 2 * words_for(wm.bits[m]) * 8);
      launch_regroup(wm.d_words + wm.offs[m], wt->d_words + wt->offs[m], wm.bits[m], d_segs + off, d_segs + off + ns,
                     ns, ctx->d_status, s, &ctx->launches);
      off += 2 * ns;
    }
    CUDA_TRY(cudaGetLastError());
  }
  if (after_pass) after_pass(passes.size());
  // (copies from pageable host vectors return once the data is staged, so
  // the plan may go out of scope with the passes still running)
}

void validate_plain(uint64_t n, uint32_t width, uint32_t levels, bool allow40 = false) {
  if (!(allow40 ? valid_plain_width(width) : valid_width(width)))
    throw Fail{PWMGPU_ERR_ARG, allow40 ? "word_width must be 1, 2, 4 or 5" : "word_width must be 1, 2 or 4"};
  if (levels == 0 || levels > kMaxPlainLevels)
    throw Fail{PWMGPU_ERR_ARG, "levels must be in 1..24 (the leaf histogram has 2^levels bins)"};
  if (n >= (uint64_t(1) << 62)) throw Fail{PWMGPU_ERR_ARG, "size too large"};
}

// Most chunks of a pass whose finished words stream to the host while the
// next chunks run.
constexpr uint32_t kMaxStreamChunks = 16;

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

bool host_pinned(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Plain build of a wx from a device text (with `io`: from a host text, into
// host arrays; d_text is then the device copy to fill).
void build_plain(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* d_text, const HostIO* io = nullptr) {
  cudaStream_t s = ctx->stream;
  const uint32_t L = wx->levels;
  const uint64_t n = wx->n;
  if (n == 0) {
    if (wx->keep_hist) wx->hist.assign(size_t(1) << L, 0);
    wx->wm.zeros.assign(L, 0);
    return;
  }
  const bool pinned_in = io && io->text && host_pinned(io->text);
  uint64_t* host_out[2] = {io ? io->wm : nullptr, io ? io->wt : nullptr};
  bool any_out = false, all_pinned = true;
  for (int st = 0; st < 2; ++st)
    if (host_out[st] && (st ? wx->wt.present : wx->wm.present)) {
      any_out = true;
      all_pinned = all_pinned && host_pinned(host_out[st]);
    }
  const bool stream_out = any_out && all_pinned;
  if (pinned_in || stream_out) ctx->xfer_init();
  // the transfer streams this build uses are idle again when it returns or throws
  struct XferDrain {
    pwmgpu_ctx* c;
    bool used;
    ~XferDrain() {
      if (!used) return;
      if (c->up) cudaStreamSynchronize(c->up);
      if (c->down) cudaStreamSynchronize(c->down);
    }
  } drain{ctx, pinned_in || stream_out};
  if (io && io->text && !pinned_in)
    CUDA_TRY(cudaMemcpyAsync(const_cast<void*>(d_text), io->text, n * wx->width, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, 4, s));
  const uint64_t bins = uint64_t(1) << L;
  auto* d_hist = static_cast<unsigned long long*>(ctx->grow("hist", bins * 8));
  CUDA_TRY(cudaMemsetAsync(d_hist, 0, bins * 8, s));
  // Tile engine: level 0 is written in whole words (by the histogram kernel,
  // or by the first pass, whose tiles start at multiples of 64 bits); the
  // first pass's other levels are zeroed by the histogram kernel (levels <= 8)
  // or here; the padding is zero from allocation.
  const bool tile_engine = ctx->engine == PWMGPU_ENGINE_TILE && L <= kTilePlanMaxLevels;
  // Pass width: by default a text of up to kSinglePassMaxLevels levels takes
  // one pass of all its levels (the histogram kernel gives that pass its
  // prefixes), deeper texts passes of kDefaultTileLevels; set_pass_levels(k)
  // asks for k (<= 4).  At 8 levels one pass would write 127 runs per tile
  // into each of the deepest levels of both structures, and the two 4-level
  // passes are faster (measured: 5.9 against 6.2 ms for 2^30 bytes, while
  // one pass wins at 5..7 levels).
  const bool auto_k = ctx->tile_levels == 0;
  const int kmax = (auto_k && L > uint32_t(kTileMaxLevels) && L <= kSinglePassMaxLevels)
                       ? int(L)
                       : std::min(auto_k ? kDefaultTileLevels : ctx->tile_levels, kTileMaxLevels);
  const int Kz = std::min<int>(kmax, int(L));
  const uint32_t D0 = uint32_t(Kz < int(L) ? Kz : Kz - 1);  // splits of the first pass
  const bool tile_hist = tile_engine && L <= 8 && D0 >= 1;
  if (tile_engine && !tile_hist && Kz > 1)
    for (Structure* st : {&wx->wm, &wx->wt})
      if (st->present)
        CUDA_TRY(cudaMemsetAsync(st->d_words + st->offs[1], 0,
                                 ((uint32_t(Kz) < L ? st->offs[Kz] : st->total_words) - st->offs[1]) * 8, s));
  // Tile engine, levels <= 8: the histogram kernel also counts the finest runs
  // of every tile of the first pass and scans them, so that pass neither
  // counts nor looks back.
  TileFirstPass first{};
  // host words the device writes (mapped, written by kernels: they must not
  // wait behind downloads in flight): the prefix counts of every level, flat
  // (level m at 2^m - 1; level L is the leaf histogram), the zero bits of
  // every level and the status word; and (pinned) the block prefix rows at
  // the bounds of a chunked first pass
  const uint64_t NB0 = uint64_t(1) << D0;
  const uint64_t flat_words = (bins << 1) - 1;
  uint64_t* h_flat = ctx->grow_mapped((flat_words + L + 1) * 8);
  uint64_t* d_flat_host = ctx->mapped_dev;
  uint64_t* h_hist = h_flat + bins - 1;
  const uint64_t* h_zeros = h_flat + flat_words;
  auto* h_status = reinterpret_cast<uint32_t*>(h_flat + flat_words + L);
  auto* d_level_zeros = static_cast<unsigned long long*>(ctx->grow("level_zeros", uint64_t(L) * 8));
  auto* h_rows = static_cast<uint64_t*>(
      ctx->grow_pinned(uint64_t(kMaxStreamChunks) * (uint64_t(1) << kTileGivenMaxLevels) * 8));
  // words of each structure already streamed to the host (a prefix of level 0)
  uint64_t sent[2] = {0, 0};
  Structure* sts[2] = {&wx->wm, &wx->wt};
  auto send = [&](int st, uint64_t w0, uint64_t w1) {  // after the main stream's current work
    if (w1 <= w0) return;
    CUDA_TRY(cudaStreamWaitEvent(ctx->down, ctx->mark(s), 0));
    CUDA_TRY(cudaMemcpyAsync(host_out[st] + w0, sts[st]->d_words + w0, (w1 - w0) * 8, cudaMemcpyDeviceToHost,
                             ctx->down));
  };
  if (tile_hist) {
    const uint32_t T = tile_pass_elems(wx->width);
    const uint64_t tiles = (n + T - 1) / T;
    const uint32_t per = tile_hist_tiles_per_block();
    const uint32_t nblocks = tile_hist_blocks(n, T);
    const uint64_t NB = uint64_t(1) << D0;
    auto* base = static_cast<unsigned char*>(ctx->grow("tile_first", tiles * NB * 8 + nblocks * NB * 8 + 256));
    first.tilecnt = reinterpret_cast<uint32_t*>(base);
    first.relpre = first.tilecnt + tiles * NB;
    first.blockpre = reinterpret_cast<unsigned long long*>(base + ((tiles * NB * 8 + 15) & ~uint64_t(15)));
    first.tiles_per_block = per;
    first.level0_written = true;
    uint64_t* l0[2] = {wx->wm.present ? wx->wm.d_words : nullptr, wx->wt.present ? wx->wt.d_words : nullptr};
    if (!l0[0]) std::swap(l0[0], l0[1]);
    // (the first pass clears the shared words of its levels 1..Kz-1 itself,
    // cheaper than zeroing them here; later passes' levels are zeroed by the
    // pass before them)
    // pieces of whole histogram blocks: uploaded, counted, their level-0 words sent back
    const uint64_t block_keys = uint64_t(per) * T;
    const uint32_t piece_blocks =
        pinned_in ? uint32_t(std::max<uint64_t>(1, ctx->upload_piece / (block_keys * wx->width))) : nblocks;
    ProfScope ps(ctx, "leaf_histogram", n * wx->width + (l0[1] ? 2 : 1) * words_for(n) * 8);
    for (uint32_t b0 = 0; b0 < nblocks; b0 += piece_blocks) {
      const uint32_t nb = std::min(piece_blocks, nblocks - b0);
      const uint64_t k0 = uint64_t(b0) * block_keys, k1 = std::min(n, uint64_t(b0 + nb) * block_keys);
      if (pinned_in) {
        CUDA_TRY(cudaMemcpyAsync(static_cast<unsigned char*>(const_cast<void*>(d_text)) + k0 * wx->width,
                                 static_cast<const unsigned char*>(io->text) + k0 * wx->width, (k1 - k0) * wx->width,
                                 cudaMemcpyHostToDevice, ctx->up));
        CUDA_TRY(cudaStreamWaitEvent(s, ctx->mark(ctx->up), 0));
      }
      launch_tile_histogram_blocks(d_text, n, wx->width, L, D0, T, b0, nb, d_hist,
                                   const_cast<uint32_t*>(first.tilecnt), const_cast<uint32_t*>(first.relpre),
                                   const_cast<unsigned long long*>(first.blockpre), l0[0], l0[1], ctx->d_status, s,
                                   &ctx->launches);
      if (stream_out) {
        const uint64_t w1 = k1 == n ? words_for(n) : k1 / 64;
        for (int st = 0; st < 2; ++st)
          if (host_out[st] && sts[st]->present) {
            send(st, sent[st], w1);
            sent[st] = w1;
          }
      }
    }
    // (the block scan follows with the first pass's start table, below)
  } else {
    if (pinned_in) CUDA_TRY(cudaMemcpyAsync(const_cast<void*>(d_text), io->text, n * wx->width,
                                            cudaMemcpyHostToDevice, s));
    ProfScope ps(ctx, "leaf_histogram", n * wx->width);
    launch_leaf_histogram(d_text, n, wx->width, L, d_hist, ctx->d_status, s, &ctx->launches);
  }
  CUDA_TRY(cudaGetLastError());
  // prefix counts, zero bits and the status word to the host
  CUDA_TRY(cudaMemsetAsync(d_level_zeros, 0, uint64_t(L) * 8, s));
  launch_fold_levels(d_hist, L, d_flat_host, d_level_zeros, s, &ctx->launches);
  launch_readback(d_level_zeros, L, ctx->d_status, d_flat_host + flat_words, s, &ctx->launches);
  CUDA_TRY(cudaEventRecord(ctx->hist_event(), s));
  const bool want_tree = wx->wt.present;
  // After the tile histogram the first pass needs nothing from the host but
  // its start table, which a one-CTA kernel derives from the histogram: the
  // pass runs while the host reads the histogram and plans the other passes
  // (the host's plan gives the same first pass).
  const void* next_in = d_text;
  size_t from = 0;
  // a host-to-host build runs the first pass in chunks of whole histogram
  // blocks (blk0: block bounds; ev0: an event after each chunk) and reads the
  // block prefixes at their bounds, so that the words each chunk finishes go
  // back while the next ones run
  std::vector<uint32_t> blk0;
  std::vector<cudaEvent_t> ev0;
  cudaEvent_t rows_ev = nullptr;
  if (tile_hist) {
    const auto shape = plan_passes(L, Kz);
    std::vector<TilePassHost> early(std::min<size_t>(shape.size(), 2));
    for (size_t i = 0; i < early.size(); ++i) {
      early[i].level = shape[i].level;
      early[i].K = shape[i].K;
      early[i].out = shape[i].has_out;
    }
    TilePassHost& p0 = early[0];
    const uint32_t T = tile_pass_elems(wx->width);
    p0.segmented = want_tree;
    p0.tiles = uint32_t((n + T - 1) / T);
    p0.segs.push_back({0, n, 0, 0, 0});
    p0.table.assign(size_t(tile_table_size(p0.K)), 0);
    const TileBlob b0 = tile_blob(early, 0, 1, L, n, wx->wm, want_tree ? &wx->wt : nullptr);
    auto* d_b0 = static_cast<unsigned char*>(ctx->grow("tile_plan0", b0.bytes.size()));
    CUDA_TRY(cudaMemcpyAsync(d_b0, b0.bytes.data(), b0.bytes.size(), cudaMemcpyHostToDevice, s));
    launch_tile_block_scan(const_cast<unsigned long long*>(first.blockpre), tile_hist_blocks(n, T), D0, d_hist, L,
                           uint32_t(p0.K), p0.out, want_tree, reinterpret_cast<uint64_t*>(d_b0 + b0.table[0]), s,
                           &ctx->launches);
    std::vector<uint32_t> bounds0;
    const uint32_t nblk = tile_hist_blocks(n, T);
    const uint32_t C = ctx->stream_chunks;
    if (stream_out && C > 1 && nblk >= 2 * C) {
      // chunk c of C takes a share c + 1 of C (C + 1) / 2: the first is small,
      // so that downloads start early, later ones overlap the downloads
      for (uint32_t c = 0; c <= C; ++c)
        blk0.push_back(uint32_t(uint64_t(nblk) * (c * (c + 1) / 2) / (C * (C + 1) / 2)));
      blk0.erase(std::unique(blk0.begin(), blk0.end()), blk0.end());
      for (size_t c = 1; c + 1 < blk0.size(); ++c)
        CUDA_TRY(cudaMemcpyAsync(h_rows + (c - 1) * NB0, first.blockpre + uint64_t(blk0[c]) * NB0, NB0 * 8,
                                 cudaMemcpyDeviceToHost, s));
      rows_ev = ctx->mark(s);
      for (uint32_t b : blk0)
        bounds0.push_back(uint32_t(std::min<uint64_t>(p0.tiles, uint64_t(b) * first.tiles_per_block)));
    }
    next_in = enqueue_tile_pass(ctx, early, 0, d_b0, b0, d_text, wx->width, n, wx->wm, want_tree ? &wx->wt : nullptr,
                                &first, bounds0, [&](size_t) {
                                  if (!blk0.empty()) ev0.push_back(ctx->mark(s));
                                });
    from = 1;
  }
  CUDA_TRY(cudaEventSynchronize(ctx->hist_event()));
  if (*h_status) {
    CUDA_TRY(cudaStreamSynchronize(s));  // the first pass may still read the text
    throw_status(*h_status);
  }
  if (wx->keep_hist) wx->hist.assign(h_hist, h_hist + bins);
  LevelTables tabs;
  std::vector<PassPlan> plan;
  std::vector<TilePassHost> tile_passes;
  std::vector<uint32_t> regroup;
  PrefixCounts cnt;  // natural-prefix counts per level
  if (tile_engine) {
    cnt = PrefixCounts::view(h_flat, L);
    tile_passes = plan_tile_passes(cnt, L, kmax, tile_pass_elems(wx->width), want_tree, &regroup);
    tabs = build_tables_tile(cnt, L, want_tree ? regroup : std::vector<uint32_t>{}, h_zeros);
  } else {
    plan = plan_passes(L, ctx->pass_levels);
    tabs = build_tables_plain(std::vector<uint64_t>(h_hist, h_hist + bins), L, plan, want_tree);
  }
  wx->wm.zeros = tabs.zeros;
  CUDA_TRY(cudaMemcpyAsync(wx->wm.d_zeros, wx->wm.zeros.data(), L * 8, cudaMemcpyHostToDevice, s));
  // Streaming the structures back: after each pass its levels of the
  // structures it completes (tree levels left to the regroup come last).
  auto level_end = [&](const Structure& st, uint32_t m) { return m + 1 < st.levels ? st.offs[m + 1] : st.total_words; };
  // Chunked streaming (every tree level from the passes): the first pass's
  // chunks, and later passes of few segments in chunks of whole segments; a
  // word goes back once all its bits are written.
  const bool chunk_stream = stream_out && tile_engine && regroup.empty();
  std::vector<char> streamed(tile_passes.size(), 0);
  std::vector<LevelCompletion> done(2, LevelCompletion(L, n));
  std::vector<std::array<uint64_t, 3>> pend;  // (structure, first word, end word)
  std::vector<std::pair<uint64_t, uint64_t>> fresh;
  auto active = [&](int st) { return host_out[st] != nullptr && sts[st]->present; };
  auto note = [&](int st, uint32_t m, uint64_t a, uint64_t b) {  // bits [a, b) of level m written
    const Structure& S = *sts[st];
    fresh.clear();
    if (!done[st].add(m, a, b, level_end(S, m) - S.offs[m], fresh))
      throw Fail{PWMGPU_ERR_CUDA, "internal: a streamed range past its level or written twice"};
    for (const auto& w : fresh) pend.push_back({uint64_t(st), S.offs[m] + w.first, S.offs[m] + w.second});
  };
  auto flush = [&](cudaEvent_t after) {  // the pending words, once `after` has happened
    if (pend.empty()) return;
    std::sort(pend.begin(), pend.end());
    CUDA_TRY(cudaStreamWaitEvent(ctx->down, after, 0));
    for (size_t i = 0; i < pend.size();) {
      const int st = int(pend[i][0]);
      const uint64_t w0 = pend[i][1];
      uint64_t w1 = pend[i][2];
      size_t k = i + 1;
      for (; k < pend.size() && pend[k][0] == pend[i][0] && pend[k][1] == w1; ++k) w1 = pend[k][2];
      if (w1 > sts[st]->total_words) throw Fail{PWMGPU_ERR_CUDA, "internal: words past the structure"};
      CUDA_TRY(cudaMemcpyAsync(host_out[st] + w0, sts[st]->d_words + w0, (w1 - w0) * 8, cudaMemcpyDeviceToHost,
                               ctx->down));
      i = k;
    }
    pend.clear();
  };
  auto check_levels = [&](const TilePassHost& p, uint32_t m0) {
    for (int st = 0; st < 2; ++st)
      if (active(st) && (st == 0 || p.segmented))
        for (uint32_t m = m0; m < p.level + uint32_t(p.K); ++m)
          if (!done[st].complete(m)) throw Fail{PWMGPU_ERR_CUDA, "internal: a streamed level is incomplete"};
  };
  // start of each natural prefix of level m in the matrix (key order) and the tree
  auto level_starts = [&](uint32_t m, bool tree) {
    std::vector<uint64_t> st(cnt[m].size());
    uint64_t run = 0;
    for (uint64_t y = 0; y < st.size(); ++y) {
      const uint64_t q = tree ? y : rev_bits_host(y, m);
      st[q] = run;
      run += cnt[m][q];
    }
    return st;
  };
  if (chunk_stream && blk0.size() >= 2 && ev0.size() + 1 == blk0.size() && !tile_passes.empty() &&
      tile_passes[0].K == Kz) {
    const TilePassHost& p = tile_passes[0];
    CUDA_TRY(cudaEventSynchronize(rows_ev));
    // keys of each natural prefix of level j in the histogram blocks before bound c
    auto before = [&](size_t c, uint32_t j) {
      if (c + 1 == blk0.size()) return std::vector<uint64_t>(cnt[j].begin(), cnt[j].end());
      std::vector<uint64_t> r(size_t(1) << j, 0);
      if (c == 0) return r;
      const uint64_t* row = h_rows + (c - 1) * NB0;  // key order of the first D0 bits
      for (uint64_t x = 0; x < NB0; ++x) r[rev_bits_host(x, D0) >> (D0 - j)] += row[x];
      return r;
    };
    std::vector<std::vector<uint64_t>> start[2];
    for (int st = 0; st < 2; ++st)
      for (uint32_t j = 0; j < uint32_t(p.K); ++j) start[st].push_back(level_starts(j, st == 1));
    for (int st = 0; st < 2; ++st)  // level 0 went back with the upload
      if (active(st)) note(st, 0, 0, n);
    pend.clear();
    for (size_t c = 0; c + 1 < blk0.size(); ++c) {
      if (c == 0)
        for (int st = 0; st < 2; ++st)
          if (active(st) && sent[st] < level_end(*sts[st], 0)) pend.push_back({uint64_t(st), sent[st], level_end(*sts[st], 0)});
      for (uint32_t j = 1; j < uint32_t(p.K); ++j) {
        const auto lo = before(c, j), hi = before(c + 1, j);
        for (uint64_t q = 0; q < lo.size(); ++q)
          for (int st = 0; st < 2; ++st)
            if (active(st)) note(st, j, start[st][j][q] + lo[q], start[st][j][q] + hi[q]);
      }
      flush(ev0[c]);
    }
    check_levels(p, 0);
    streamed[0] = 1;
  }
  // later passes: chunks of whole segments (the host knows each segment's runs)
  std::vector<std::vector<uint32_t>> seg_bounds(tile_passes.size());
  PassChunks chunks;
  chunks.bounds = [&](size_t pi) {
    std::vector<uint32_t> b;
    const TilePassHost& p = tile_passes[pi];
    if (!chunk_stream || pi == 0 || !p.segmented || p.segs.size() < 2 || p.segs.size() > 64) return b;
    auto& sb = seg_bounds[pi];
    sb.assign(1, 0);
    for (uint32_t c = 1; c < ctx->stream_chunks; ++c) {
      const uint64_t target = uint64_t(p.tiles) * (c * (c + 1) / 2) / (ctx->stream_chunks * (ctx->stream_chunks + 1) / 2);
      uint32_t i = sb.back() + 1;
      while (i < p.segs.size() && p.segs[i].tile0 < target) ++i;
      if (i < p.segs.size()) sb.push_back(i);
    }
    sb.push_back(uint32_t(p.segs.size()));
    for (uint32_t i : sb) b.push_back(i < p.segs.size() ? p.segs[i].tile0 : p.tiles);
    return b;
  };
  chunks.after = [&](size_t pi, size_t c) {
    if (seg_bounds[pi].empty()) return;
    const TilePassHost& p = tile_passes[pi];
    const uint32_t l = p.level;
    for (uint32_t i = seg_bounds[pi][c]; i < seg_bounds[pi][c + 1]; ++i) {
      const TileSegHost& sg = p.segs[i];
      const uint64_t* tab = p.table.data() + sg.table;
      for (int j = 0; j < p.K; ++j)
        for (int v = 0; v < (1 << j); ++v) {
          const uint64_t x = (uint64_t(v) << l) | sg.group;
          const uint64_t m = cnt[l + j][rev_bits_host(x, l + uint32_t(j))];
          for (int st = 0; st < 2; ++st)
            if (active(st)) {
              const uint64_t b = tab[st ? tile_wt_entry(p.K, j, v) : tile_wm_entry(j, v)];
              note(st, l + uint32_t(j), b, b + m);
            }
        }
    }
    flush(ctx->mark(s));
    if (c + 2 == seg_bounds[pi].size()) {
      check_levels(p, l);
      streamed[pi] = 1;
    }
  };
  auto after_pass = [&](size_t pi) {
    for (int st = 0; st < 2; ++st) {
      if (!host_out[st] || !sts[st]->present) continue;
      const Structure& S = *sts[st];
      uint64_t w1 = sent[st];
      if (pi < tile_passes.size() && streamed[pi]) {  // sent chunk by chunk
        const TilePassHost& p = tile_passes[pi];
        sent[st] = std::max(sent[st], level_end(S, p.level + p.K - 1));
        continue;
      }
      if (pi < tile_passes.size()) {
        const TilePassHost& p = tile_passes[pi];
        if (st == 1 && !p.segmented) continue;
        w1 = level_end(S, p.level + p.K - 1);
      } else {
        w1 = S.total_words;
      }
      // levels complete in order for the matrix; a tree level left to the
      // regroup holds back the tree's later levels until the end
      if (st == 1 && pi < tile_passes.size()) {
        bool gap = false;
        for (uint32_t m : regroup) gap |= level_end(S, m) <= w1;
        if (gap) continue;
      }
      send(st, sent[st], w1);
      sent[st] = std::max(sent[st], w1);
    }
  };
  // Rank/select: the levels of all passes but the last (when no tree level
  // waits for the regroup) on the side stream as soon as the last pass
  // starts, the others after it.
  Structure* rs_wm = wx->wm.rs && !wx->wm_internal ? &wx->wm : nullptr;
  Structure* rs_wt = want_tree && wx->wt.rs ? &wx->wt : nullptr;
  const bool early_rs = tile_engine && (rs_wm || rs_wt) && tile_passes.size() >= 2 && regroup.empty();
  const uint32_t late_level = early_rs ? tile_passes.back().level : 0;
  auto rank_select_early = [&]() {
    ctx->side_init();
    CUDA_TRY(cudaEventRecord(ctx->side_go, s));
    CUDA_TRY(cudaStreamWaitEvent(ctx->side, ctx->side_go, 0));
    build_rank_select(ctx, rs_wm, rs_wt, true, 0, late_level, ctx->side, "_side");
    CUDA_TRY(cudaEventRecord(ctx->side_done, ctx->side));
  };
  auto hook = [&](size_t pi) {
    if (stream_out) after_pass(pi);
    if (early_rs && pi + 2 == tile_passes.size()) rank_select_early();
  };
  if (tile_engine) {
    if (from == 1) hook(0);
    run_tile_passes(ctx, next_in, wx->width, L, tile_passes, regroup, tabs, wx->wm, want_tree ? &wx->wt : nullptr,
                    first.blockpre ? &first : nullptr, std::function<void(size_t)>(hook), from,
                    chunk_stream ? &chunks : nullptr);
  }
  else
    run_passes(ctx, d_text, wx->width, wx->width, false, L, plan, tabs, wx->wm, want_tree ? &wx->wt : nullptr);
  build_rank_select(ctx, rs_wm, rs_wt, true, late_level);
  if (early_rs) CUDA_TRY(cudaStreamWaitEvent(s, ctx->side_done, 0));
  CUDA_TRY(cudaGetLastError());
  if (any_out) {
    for (int st = 0; st < 2; ++st) {
      if (!host_out[st] || !sts[st]->present) continue;
      const Structure& S = *sts[st];
      if (stream_out) send(st, sent[st], S.total_words);
      else CUDA_TRY(cudaMemcpyAsync(host_out[st], S.d_words, S.total_words * 8, cudaMemcpyDeviceToHost, s));
    }
    if (stream_out) CUDA_TRY(cudaStreamSynchronize(ctx->down));
    CUDA_TRY(cudaStreamSynchronize(s));
  }
}

// Symbol histogram + first occurrences of a device text on the GPU, then the
// code builder on the host.
HuffCodes huffman_codes_device(pwmgpu_ctx* ctx, const void* d_text, uint64_t n, uint32_t width, bool is_tree,
                               uint64_t* max_symbol_out) {
  cudaStream_t s = ctx->stream;
  uint64_t nsym = width == 1 ? 256 : (width == 2 ? 65536 : 0);
  if (width == 4) {
    // bound the alphabet by the largest symbol (one histogram bin per value)
    throw Fail{PWMGPU_ERR_ARG, "Huffman codes for 32-bit texts: pass a code table"};
  }
  auto* d_hist = static_cast<unsigned long long*>(ctx->grow("sym_hist", nsym * 8));
  auto* d_first = static_cast<unsigned long long*>(ctx->grow("sym_first", nsym * 8));
  CUDA_TRY(cudaMemsetAsync(d_hist, 0, nsym * 8, s));
  CUDA_TRY(cudaMemsetAsync(d_first, 0xFF, nsym * 8, s));
  CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, 4, s));
  {
    ProfScope ps(ctx, "symbol_histogram", n * width);
    launch_symbol_histogram(d_text, n, width, nsym, d_hist, width == 1 ? nullptr : d_first, ctx->d_status, s,
                            &ctx->launches);
  }
  std::vector<uint64_t> count(nsym), first(nsym);
  CUDA_TRY(cudaMemcpyAsync(count.data(), d_hist, nsym * 8, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaMemcpyAsync(first.data(), d_first, nsym * 8, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t max_symbol = 0;
  for (uint64_t c = 0; c < nsym; ++c)
    if (count[c]) max_symbol = c;
  *max_symbol_out = max_symbol;
  auto entries = width == 1 ? histogram_order<uint8_t>(count, first, 1) : histogram_order<uint16_t>(count, first, 2);
  return build_huffman_codes(entries, max_symbol, is_tree);
}

// Huffman build of one structure (matrix, or tree through the matrix).
// Returns the level sizes.
void build_huffman(pwmgpu_ctx* ctx, const void* d_text, uint64_t n, uint32_t width, bool is_tree,
                   const std::vector<uint64_t>& code_len, const std::vector<uint64_t>& code_word, uint32_t levels,
                   Structure& wm, Structure* wt, bool rank_select) {
  cudaStream_t s = ctx->stream;
  const uint64_t ncodes = code_len.size();
  // symbol histogram for the weighted codes
  const uint64_t nsym = ncodes;
  // 8- and 16-bit texts count every value (symbols past the table fail below)
  const uint64_t bins = std::max<uint64_t>(width <= 2 ? uint64_t(1) << (8 * width) : nsym, std::max<uint64_t>(nsym, 1));
  auto* d_hist = static_cast<unsigned long long*>(ctx->grow("sym_hist", bins * 8));
  CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, 4, s));
  CUDA_TRY(cudaMemsetAsync(d_hist, 0, bins * 8, s));
  {
    ProfScope ps(ctx, "symbol_histogram", n * width);
    launch_symbol_histogram(d_text, n, width, nsym, d_hist, nullptr, ctx->d_status, s, &ctx->launches);
  }
  std::vector<uint64_t> count(nsym);
  CUDA_TRY(cudaMemcpyAsync(count.data(), d_hist, nsym * 8, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  uint64_t counted = 0;
  std::vector<WeightedCode> wc;
  for (uint64_t c = 0; c < nsym; ++c) {
    counted += count[c];
    if (count[c]) {
      if (code_len[c] == 0 || code_len[c] > 56) throw Fail{PWMGPU_ERR_ARG, "a text symbol has no usable code"};
      wc.push_back({code_word[c], uint32_t(code_len[c]), count[c]});
    }
  }
  if (counted != n) throw Fail{PWMGPU_ERR_SYMBOL, "a text symbol is outside the code table"};
  uint32_t maxlen = 0;
  for (auto& c : wc) maxlen = std::max(maxlen, c.len);
  if (levels == 0) levels = maxlen;  // the longest code of a symbol that occurs
  if (maxlen != levels) throw Fail{PWMGPU_ERR_ARG, "levels must equal the longest code length"};
  const uint32_t key_bytes = maxlen <= 24 ? 4 : 8;
  const auto plan = plan_passes(levels, ctx->pass_levels);
  const LevelTables tabs = build_tables(wc, levels, plan, wt != nullptr);
  // layouts
  alloc_structure(wm, tabs.level_bits, n, false, true, rank_select && !is_tree);
  wm.zeros = tabs.zeros;
  CUDA_TRY(cudaMemcpyAsync(wm.d_zeros, wm.zeros.data(), levels * 8, cudaMemcpyHostToDevice, s));
  if (wt) alloc_structure(*wt, tabs.level_bits, n, true, true, rank_select);
  // code keys
  uint64_t* d_len = static_cast<uint64_t*>(ctx->grow("code_len", std::max<uint64_t>(ncodes, 1) * 8));
  uint64_t* d_word = static_cast<uint64_t*>(ctx->grow("code_word", std::max<uint64_t>(ncodes, 1) * 8));
  CUDA_TRY(cudaMemcpyAsync(d_len, code_len.data(), ncodes * 8, cudaMemcpyHostToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(d_word, code_word.data(), ncodes * 8, cudaMemcpyHostToDevice, s));
  void* keys = ctx->grow("huff_keys", std::max<uint64_t>(n, 1) * key_bytes);
  launch_huffman_keys(d_text, n, width, d_len, d_word, ncodes, key_bytes, keys, ctx->d_status, s, &ctx->launches);
  run_passes(ctx, keys, key_bytes, width, true, levels, plan, tabs, wm, wt);
  check_device_status(ctx);
  build_rank_select(ctx, !is_tree ? &wm : nullptr, wt);
}

}  // namespace


// ===========================================================================
// Batches of independent plain texts
// ===========================================================================
namespace {

constexpr uint32_t kBatchMaxLevels = 12;        // per-text tables live in shared memory
constexpr uint64_t kBatchChunk = 65536;         // symbols per histogram CTA
constexpr uint64_t kBatchRegroupWords = 1024;   // words per regroup CTA

struct BatchPassGroup {
  int pass = 0, K = 1;
  std::vector<uint32_t> texts;
  uint32_t tiles = 0;
  SplitArgs* d_args = nullptr;
  uint32_t* d_tile_base = nullptr;
  unsigned long long* d_lookback = nullptr;  // followed by the tile counter
  size_t lb_bytes = 0;
};

}  // namespace

struct pwmgpu_batch {
  pwmgpu_ctx* ctx = nullptr;
  uint32_t count = 0, width = 1, flags = 0, maxL = 0;
  int kmax = 2;
  std::vector<uint64_t> offs;
  std::vector<uint32_t> L;
  std::vector<BatchText> info;
  std::vector<uint64_t> wm_off, wt_off, words_per_level;
  uint64_t wm_words = 0, wt_words = 0, zeros_n = 0, hist_n = 0, starts_n = 0, segs_n = 0, symbols = 0;
  std::vector<BatchChunk> chunks;
  std::vector<BatchRegroup> regroup;
  // device
  std::vector<void*> owned;
  BatchText* d_info = nullptr;
  BatchChunk* d_chunks = nullptr;
  BatchRegroup* d_regroup = nullptr;
  uint64_t *d_wm = nullptr, *d_wt = nullptr, *d_zeros = nullptr, *d_starts = nullptr, *d_segs = nullptr;
  unsigned long long* d_hist = nullptr;
  void *d_keys_a = nullptr, *d_keys_b = nullptr;
  std::vector<BatchPassGroup> groups;
  int groups_k = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* graph_text = nullptr;
  int graph_k = 0;

  void* dalloc(size_t bytes) {
    void* p = nullptr;
    CUDA_TRY(cudaMalloc(&p, std::max<size_t>(bytes, 256)));
    owned.push_back(p);
    return p;
  }
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    graph_text = nullptr;
  }
  ~pwmgpu_batch() {
    drop_graph();
    for (auto& g : groups) {
      cudaFree(g.d_args);
      cudaFree(g.d_tile_base);
      cudaFree(g.d_lookback);
    }
    for (void* p : owned) cudaFree(p);
  }
};

namespace {

// Pass groups (pass index, K) and their per-text split arguments.
void batch_plan(pwmgpu_batch* b, const void* d_texts) {
  pwmgpu_ctx* ctx = b->ctx;
  for (auto& g : b->groups) {
    cudaFree(g.d_args);
    cudaFree(g.d_tile_base);
    cudaFree(g.d_lookback);
  }
  b->groups.clear();
  const int kmax = b->kmax;
  const uint32_t T = split_tile_elems(b->width);
  std::vector<uint64_t> pass_starts_base(b->count, 0);
  for (int pass = 0;; ++pass) {
    std::map<int, BatchPassGroup> by_k;
    for (uint32_t t = 0; t < b->count; ++t) {
      const uint32_t l = uint32_t(pass * kmax);
      if (l >= b->L[t]) continue;
      const int K = int(std::min<uint32_t>(uint32_t(kmax), b->L[t] - l));
      auto& g = by_k[K];
      g.pass = pass;
      g.K = K;
      g.texts.push_back(t);
    }
    if (by_k.empty()) break;
    for (auto& kv : by_k) {
      BatchPassGroup g = kv.second;
      const int K = g.K;
      const int nlb = 1 << K;
      std::vector<SplitArgs> args(g.texts.size());
      std::vector<uint32_t> tile_base(g.texts.size() + 1, 0);
      uint64_t lb_words = 0;
      std::vector<uint64_t> lb_off(g.texts.size());
      for (size_t i = 0; i < g.texts.size(); ++i) {
        const uint32_t t = g.texts[i];
        const uint64_t n = b->offs[t + 1] - b->offs[t];
        const uint32_t tiles = uint32_t((n + T - 1) / T);
        tile_base[i + 1] = tile_base[i] + tiles;
        lb_off[i] = lb_words;
        lb_words += uint64_t(tiles) * nlb;
      }
      g.tiles = tile_base.back();
      g.lb_bytes = lb_words * 8 + 64;
      CUDA_TRY(cudaMalloc(&g.d_lookback, g.lb_bytes));
      CUDA_TRY(cudaMalloc(&g.d_args, sizeof(SplitArgs) * std::max<size_t>(args.size(), 1)));
      CUDA_TRY(cudaMalloc(&g.d_tile_base, sizeof(uint32_t) * tile_base.size()));
      const uint32_t l = uint32_t(g.pass * kmax);
      for (size_t i = 0; i < g.texts.size(); ++i) {
        const uint32_t t = g.texts[i];
        const uint64_t n = b->offs[t + 1] - b->offs[t];
        SplitArgs& a = args[i];
        a = SplitArgs{};
        const bool has_out = l + uint32_t(K) < b->L[t];
        char* ka = static_cast<char*>(b->d_keys_a) + b->offs[t] * b->width;
        char* kb = static_cast<char*>(b->d_keys_b) + b->offs[t] * b->width;
        const char* text = static_cast<const char*>(d_texts) + b->offs[t] * b->width;
        a.in = g.pass == 0 ? static_cast<const void*>(text) : (g.pass % 2 == 1 ? ka : kb);
        a.out = has_out ? static_cast<void*>(g.pass % 2 == 0 ? ka : kb) : nullptr;
        a.m = n;
        a.level = l;
        a.levels_here = uint32_t(K);
        for (int j = 0; j < K; ++j) a.bv[j] = b->d_wm + b->wm_off[t] + uint64_t(l + j) * b->words_per_level[t];
        a.tree_level0 = (g.pass == 0 && (b->flags & PWMGPU_TREE)) ? b->d_wt + b->wt_off[t] : nullptr;
        a.starts = b->d_starts + b->info[t].starts_off + pass_starts_base[t];
        a.lookback = g.d_lookback + lb_off[i];
        a.tile_counter = nullptr;
        for (int j = 0; j <= K; ++j) a.level_size[j] = n;
        a.status = ctx->d_status;
        a.tiles = tile_base[i + 1] - tile_base[i];
        a.L = b->L[t];
        pass_starts_base[t] += uint64_t((2 << K) - 2);
      }
      CUDA_TRY(cudaMemcpy(g.d_args, args.data(), sizeof(SplitArgs) * args.size(), cudaMemcpyHostToDevice));
      CUDA_TRY(cudaMemcpy(g.d_tile_base, tile_base.data(), sizeof(uint32_t) * tile_base.size(),
                          cudaMemcpyHostToDevice));
      b->groups.push_back(std::move(g));
    }
  }
  b->groups_k = kmax;
}

// Enqueue one whole batch build on the context's stream.
void batch_enqueue(pwmgpu_batch* b, const void* d_texts) {
  pwmgpu_ctx* ctx = b->ctx;
  cudaStream_t s = ctx->stream;
  CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, 4, s));
  CUDA_TRY(cudaMemsetAsync(b->d_hist, 0, std::max<uint64_t>(b->hist_n, 1) * 8, s));
  CUDA_TRY(cudaMemsetAsync(b->d_wm, 0, std::max<uint64_t>(b->wm_words, 1) * 8, s));
  for (auto& g : b->groups) CUDA_TRY(cudaMemsetAsync(g.d_lookback, 0, g.lb_bytes, s));
  launch_batch_hist(d_texts, b->width, b->d_chunks, uint32_t(b->chunks.size()), b->d_info, b->d_hist, ctx->d_status,
                    s, &ctx->launches);
  launch_batch_tables(b->d_hist, b->d_info, b->count, b->maxL, b->kmax, b->d_zeros, b->d_starts, b->d_segs, s,
                      &ctx->launches);
  for (auto& g : b->groups) {
    auto* counter = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(g.d_lookback) + g.lb_bytes - 64);
    launch_split_pass_batched(b->width, g.K, g.d_args, g.d_tile_base, uint32_t(g.texts.size()), g.tiles, counter, s,
                              &ctx->launches);
  }
  if (b->flags & PWMGPU_TREE)
    launch_batch_regroup(b->d_regroup, uint32_t(b->regroup.size()), ctx->d_status, s, &ctx->launches);
  CUDA_TRY(cudaGetLastError());
}

// Host side of the seeded batch generator.
struct BatchGen {
  std::vector<uint64_t> dna_thr, run_thr, zipf_thr;
  std::vector<uint32_t> perm;
};

}  // namespace

// ===========================================================================
// extern "C"
// ===========================================================================
namespace {

std::unique_ptr<pwmgpu_wx> make_wx(pwmgpu_ctx* ctx, uint64_t size, uint32_t word_width, uint32_t levels,
                                   uint32_t shape_flags) {
  auto wx = std::make_unique<pwmgpu_wx>();
  wx->ctx = ctx;
  wx->n = size;
  wx->width = word_width == 5 ? 4 : word_width;
  wx->in_width = word_width == 5 ? 5 : 0;
  wx->levels = levels;
  wx->flags = shape_flags;
  wx->keep_hist = shape_flags & PWMGPU_KEEP_HISTOGRAM;
  const bool rs = shape_flags & PWMGPU_RANK_SELECT;
  std::vector<uint64_t> bits(levels, size);
  cudaStream_t as = ctx->async_alloc ? ctx->stream : nullptr;
  alloc_structure(wx->wm, bits, size, false, false, rs && (shape_flags & PWMGPU_MATRIX), as);
  wx->wm_internal = !(shape_flags & PWMGPU_MATRIX);
  if (shape_flags & PWMGPU_TREE) alloc_structure(wx->wt, bits, size, true, false, rs, as);
  return wx;
}

// ---------------------------------------------------------------------------
// Semi-external construction (pwm's semi_in, include/external_memory/semi_in/
// pc_semi_external.hpp:16-230, which reads its text twice: once for the
// histogram and the first level, once to place every bit).  A host text is
// streamed through the GPU in pieces that fit a device budget: the first
// pass accumulates the leaf histogram, which gives every group's global
// start; the second builds each piece as a shard (matrix and/or tree) and
// sends each of its runs to the host arrays at the group's start plus the
// bits earlier pieces put there -- pwm's merge of slices (merge.hpp:
// 192-465) with the destination in host memory.  Words a run covers whole go
// by DMA from a staging buffer that holds them shifted into place; words two
// runs share, and all words of short runs, come back in one copy per piece
// and are OR-ed together on the host at the end.
// ---------------------------------------------------------------------------
constexpr uint64_t kSemiMinPiece = uint64_t(1) << 16;
constexpr uint64_t kAlphabetMaxSymbol = uint64_t(1) << 24;  // 32-bit alphabet reduction: one bin per value below
constexpr uint64_t kAlphabetHashMaxSymbols = uint64_t(1) << 30;  // wider symbols: through a hash table
constexpr uint64_t kSemiDmaMinWords = 512;  // shorter runs go through the host's OR

void semi_external(pwmgpu_ctx* ctx, const void* text, uint64_t n, uint32_t width, uint32_t L, uint64_t* out_wm,
                   uint64_t* wm_zeros, uint64_t* out_wt, uint64_t budget) {
  cudaStream_t s = ctx->stream;
  const bool want_tree = out_wt != nullptr;
  const int nout = (out_wm ? 1 : 0) + (out_wt ? 1 : 0);
  if (budget == 0) {
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    budget = free_b / 2;
  }
  // device bytes per symbol of a piece: two text buffers, the build's two
  // key buffers, the shard's structures and two stagings of the outputs
  const double per_sym = 4.0 * width + (want_tree ? 2 : 1) * L / 8.0 + 2.0 * nout * L / 8.0 + 1.0;
  uint64_t P = uint64_t(double(budget) / per_sym) & ~(kSemiMinPiece - 1);
  if (P < kSemiMinPiece) throw Fail{PWMGPU_ERR_ARG, "device budget below one piece of 2^16 symbols"};
  P = std::min(P, (n + kSemiMinPiece - 1) & ~(kSemiMinPiece - 1));
  const auto* txt = static_cast<const unsigned char*>(text);
  ctx->xfer_init();
  // every stream is idle again when this returns or throws
  struct Drain {
    pwmgpu_ctx* c;
    ~Drain() {
      cudaStreamSynchronize(c->up);
      cudaStreamSynchronize(c->down);
      cudaStreamSynchronize(c->stream);
    }
  };
  // Buffers double-buffered by piece parity, kept in the context for the
  // next call: two piece texts, two stagings (with their run tables) and two
  // pinned return buffers.  A staging or return buffer grows only after the
  // piece that used it two steps before has been collected.
  Drain drain{ctx};
  const bool single = n <= P;  // one piece: its own histogram is the text's
  void* piece_buf[2] = {ctx->grow("semi_text0", P * width), single ? nullptr : ctx->grow("semi_text1", P * width)};
  const char* stage_name[2] = {"semi_stage0", "semi_stage1"};
  const char* back_name[2] = {"semi_back0", "semi_back1"};
  void* back_buf[2] = {nullptr, nullptr};
  // start of each natural prefix of level m in the matrix (key order) or the tree
  auto starts = [](const CountSpan c, uint32_t m, bool tree) {
    std::vector<uint64_t> st(c.size());
    uint64_t run = 0;
    for (uint64_t y = 0; y < c.size(); ++y) {
      const uint64_t q = tree ? y : rev_bits_host(y, m);
      st[q] = run;
      run += c[q];
    }
    return st;
  };
  struct Out {
    int st;  // 0 matrix, 1 tree
    uint64_t* host;
    std::vector<std::vector<uint64_t>> gstart;
  };
  std::vector<Out> outs;
  if (out_wm) outs.push_back({0, out_wm, {}});
  if (out_wt) outs.push_back({1, out_wt, {}});
  PrefixCounts cnt;                          // the text's prefix counts per level
  std::vector<std::vector<uint64_t>> placed;  // per level and prefix: bits earlier pieces placed
  auto setup = [&](const uint64_t* hist) {    // global starts and zeros from the leaf histogram
    cnt = fold_prefix_counts(hist, L);
    if (wm_zeros) {
      const LevelTables t = build_tables_tile(cnt, L, {});
      std::memcpy(wm_zeros, t.zeros.data(), L * 8);
    }
    for (auto& o : outs)
      for (uint32_t l = 0; l < L; ++l) o.gstart.push_back(starts(cnt[l], l, o.st == 1));
    placed.assign(L, {});
    for (uint32_t l = 0; l < L; ++l) placed[l].assign(cnt[l].size(), 0);
  };
  // pass 1: the leaf histogram, uploads beside the counting (a text of one
  // piece skips it)
  const uint64_t bins = uint64_t(1) << L;
  cudaEvent_t used[2] = {nullptr, nullptr};  // the last work on s that read text buffer b
  if (!single) {
    auto* d_hist = static_cast<unsigned long long*>(ctx->grow("semi_hist", bins * 8));
    CUDA_TRY(cudaMemsetAsync(d_hist, 0, bins * 8, s));
    CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, 4, s));
    for (uint64_t a = 0, k = 0; a < n; a += P, ++k) {
      const int b = int(k & 1);
      const uint64_t m = std::min(P, n - a);
      if (used[b]) CUDA_TRY(cudaStreamWaitEvent(ctx->up, used[b], 0));
      CUDA_TRY(cudaMemcpyAsync(piece_buf[b], txt + a * width, m * width, cudaMemcpyHostToDevice, ctx->up));
      CUDA_TRY(cudaStreamWaitEvent(s, ctx->mark(ctx->up), 0));
      ProfScope ps(ctx, "leaf_histogram", m * width);
      launch_leaf_histogram(piece_buf[b], m, width, L, d_hist, ctx->d_status, s, &ctx->launches);
      used[b] = ctx->mark(s);
    }
    std::vector<uint64_t> hist(bins);
    CUDA_TRY(cudaMemcpyAsync(hist.data(), d_hist, bins * 8, cudaMemcpyDeviceToHost, s));
    check_device_status(ctx);
    setup(hist.data());
  }
  const uint64_t lw = padded_words(n);  // words per level of the host arrays
  // A piece's runs bound for the host: short ones first in the staging, then
  // the long ones, whose partial edge words are gathered behind the short
  // runs' words so that one copy brings back everything the host ORs.
  struct PieceOut {
    std::vector<StageSeg> segs;                  // short runs, then long runs
    std::vector<std::array<uint64_t, 2>> meta;   // per run: (output, first absolute word)
    size_t nsmall = 0;
    uint64_t small_words = 0, total = 0;
    std::vector<uint64_t> edge_idx;              // staging words of the long runs' partial edges
    std::vector<std::array<uint64_t, 2>> edge_meta;
    cudaEvent_t done = nullptr;                  // its copies back have finished
    bool pending = false;
  };
  PieceOut po[2];
  std::vector<std::array<uint64_t, 3>> acc;  // (output, word, bits) OR-ed at the end
  auto collect = [&](PieceOut& q, int b) {   // the host's share of a piece, once its copies are back
    if (!q.pending) return;
    CUDA_TRY(cudaEventSynchronize(q.done));
    const auto* h_back = static_cast<const uint64_t*>(back_buf[b]);
    for (size_t i = 0; i < q.nsmall; ++i) {
      const StageSeg& sg = q.segs[i];
      const uint64_t words = ((sg.dst_bit + sg.len + 63) >> 6) - (sg.dst_bit >> 6);
      for (uint64_t j = 0; j < words; ++j) acc.push_back({q.meta[i][0], q.meta[i][1] + j, h_back[sg.stage + j]});
    }
    for (size_t e = 0; e < q.edge_idx.size(); ++e)
      acc.push_back({q.edge_meta[e][0], q.edge_meta[e][1], h_back[q.small_words + e]});
    q.pending = false;
  };
  // pass 2: piece k uploads (up) while piece k-1 builds (s) and piece k-2's
  // words go back (down); the host ORs piece k-1's share meanwhile
  for (int b = 0; b < 2; ++b) used[b] = nullptr;
  // the staging kernels' own status word (every shard build clears the context's)
  auto* d_stage_status = static_cast<uint32_t*>(ctx->grow("semi_status", 4));
  CUDA_TRY(cudaMemsetAsync(d_stage_status, 0, 4, s));
  cudaEvent_t uploaded[2] = {nullptr, nullptr};
  auto upload = [&](uint64_t a, int b) {  // into text buffer b once the build that read it is done
    if (used[b]) CUDA_TRY(cudaStreamWaitEvent(ctx->up, used[b], 0));
    CUDA_TRY(cudaMemcpyAsync(piece_buf[b], txt + a * width, std::min(P, n - a) * width, cudaMemcpyHostToDevice,
                             ctx->up));
    uploaded[b] = ctx->mark(ctx->up);
  };
  upload(0, 0);
  for (uint64_t a = 0, k = 0; a < n; a += P, ++k) {
    const int b = int(k & 1);
    const uint64_t m = std::min(P, n - a);
    CUDA_TRY(cudaStreamWaitEvent(s, uploaded[b], 0));
    // the shard structures of full pieces and of a shorter last piece stay in
    // the context for the next call of the same shape
    const uint32_t shape = (out_wm ? PWMGPU_MATRIX : 0u) | (want_tree ? PWMGPU_TREE : 0u) | PWMGPU_KEEP_HISTOGRAM;
    auto& slot = ctx->semi_shard[m == P ? 0 : 1];
    if (!slot || slot->n != m || slot->width != width || slot->levels != L || slot->flags != shape) {
      CUDA_TRY(cudaStreamSynchronize(s));
      slot.reset();
      slot = make_wx(ctx, m, width, L, shape);
    }
    pwmgpu_wx* shard = slot.get();
    build_plain(ctx, shard, piece_buf[b]);
    if (single) setup(shard->hist.data());
    const auto pc = fold_prefix_counts(shard->hist.data(), L);
    PieceOut& q = po[b];
    collect(q, b);  // piece k-2 (its buffers are reused now)
    q = PieceOut{};
    std::vector<StageSeg> big;
    std::vector<std::array<uint64_t, 2>> big_meta;
    for (size_t oi = 0; oi < outs.size(); ++oi) {
      const Out& o = outs[oi];
      const Structure& S = o.st ? shard->wt : shard->wm;
      for (uint32_t l = 0; l < L; ++l) {
        const auto ls = starts(pc[l], l, o.st == 1);
        for (uint64_t x = 0; x < pc[l].size(); ++x) {
          const uint64_t c = pc[l][x];
          if (!c) continue;
          const uint64_t dst = o.gstart[l][x] + placed[l][x];
          const StageSeg sg{S.d_words + S.offs[l], ls[x], dst, c, 0};
          const uint64_t words = ((dst + c + 63) >> 6) - (dst >> 6);
          const uint64_t edges = ((dst & 63) ? 1 : 0) + (((dst + c) & 63) ? 1 : 0);
          const std::array<uint64_t, 2> mt{uint64_t(oi), uint64_t(l) * lw + (dst >> 6)};
          if (words >= edges + kSemiDmaMinWords) {
            big.push_back(sg);
            big_meta.push_back(mt);
          } else {
            q.segs.push_back(sg);
            q.meta.push_back(mt);
          }
        }
      }
    }
    for (uint32_t l = 0; l < L; ++l)
      for (uint64_t x = 0; x < pc[l].size(); ++x) placed[l][x] += pc[l][x];
    q.nsmall = q.segs.size();
    uint64_t stage = 0;
    for (auto& sg : q.segs) {
      sg.stage = stage;
      stage += ((sg.dst_bit + sg.len + 63) >> 6) - (sg.dst_bit >> 6);
    }
    q.small_words = stage;
    for (size_t i = 0; i < big.size(); ++i) {
      StageSeg sg = big[i];
      sg.stage = stage;
      const uint64_t words = ((sg.dst_bit + sg.len + 63) >> 6) - (sg.dst_bit >> 6);
      if (sg.dst_bit & 63) {
        q.edge_idx.push_back(stage);
        q.edge_meta.push_back(big_meta[i]);
      }
      if ((sg.dst_bit + sg.len) & 63) {
        q.edge_idx.push_back(stage + words - 1);
        q.edge_meta.push_back({big_meta[i][0], big_meta[i][1] + words - 1});
      }
      q.segs.push_back(sg);
      q.meta.push_back(big_meta[i]);
      stage += words;
    }
    q.total = stage;
    const uint64_t back = q.small_words + q.edge_idx.size();  // words the host ORs
    // staging b and its return buffer were last read by piece k-2's copies,
    // collected above; the segment tables go in front of the staged words
    const size_t seg_bytes = (q.segs.size() * sizeof(StageSeg) + 15) & ~size_t(15);
    const size_t idx_bytes = (q.edge_idx.size() * 8 + 15) & ~size_t(15);
    auto* base = static_cast<unsigned char*>(ctx->grow(stage_name[b], seg_bytes + idx_bytes + (q.total + back + 1) * 8));
    auto* d_segs = reinterpret_cast<StageSeg*>(base);
    auto* d_eidx = reinterpret_cast<uint64_t*>(base + seg_bytes);
    auto* d_stage = reinterpret_cast<uint64_t*>(base + seg_bytes + idx_bytes);
    auto* h_back = static_cast<uint64_t*>(ctx->grow_pinned_named(back_name[b], std::max<uint64_t>(back, 1) * 8));
    back_buf[b] = h_back;
    CUDA_TRY(cudaMemcpyAsync(d_segs, q.segs.data(), q.segs.size() * sizeof(StageSeg), cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d_eidx, q.edge_idx.data(), q.edge_idx.size() * 8, cudaMemcpyHostToDevice, s));
    {
      ProfScope ps(ctx, "semi_stage", q.total * 16);
      launch_stage_segments(d_segs, q.segs.size(), d_stage, q.total, d_stage_status, s, &ctx->launches);
    }
    uint64_t* d_back = d_stage + q.total;
    if (q.small_words)
      CUDA_TRY(cudaMemcpyAsync(d_back, d_stage, q.small_words * 8, cudaMemcpyDeviceToDevice, s));
    launch_gather_words(d_stage, d_eidx, q.edge_idx.size(), d_back + q.small_words, s, &ctx->launches);
    CUDA_TRY(cudaGetLastError());
    used[b] = ctx->mark(s);  // the build read text buffer b; the staging is complete
    CUDA_TRY(cudaStreamWaitEvent(ctx->down, used[b], 0));
    CUDA_TRY(cudaMemcpyAsync(h_back, d_back, back * 8, cudaMemcpyDeviceToHost, ctx->down));
    for (size_t i = q.nsmall; i < q.segs.size(); ++i) {  // the long runs' whole words into the host arrays
      const StageSeg& sg = q.segs[i];
      const uint64_t words = ((sg.dst_bit + sg.len + 63) >> 6) - (sg.dst_bit >> 6);
      const uint64_t j0 = (sg.dst_bit & 63) ? 1 : 0, j1 = words - (((sg.dst_bit + sg.len) & 63) ? 1 : 0);
      uint64_t* h = outs[q.meta[i][0]].host + q.meta[i][1];
      CUDA_TRY(cudaMemcpyAsync(h + j0, d_stage + sg.stage + j0, (j1 - j0) * 8, cudaMemcpyDeviceToHost, ctx->down));
    }
    q.done = ctx->mark(ctx->down);
    q.pending = true;
    if (a + P < n) upload(a + P, b ^ 1);  // piece k+1 goes up beside piece k's copies back
    collect(po[b ^ 1], b ^ 1);  // piece k-1, while piece k runs
  }
  collect(po[0], 0);
  collect(po[1], 1);
  check_device_status(ctx);
  uint32_t stage_status = 0;
  CUDA_TRY(cudaMemcpyAsync(&stage_status, d_stage_status, 4, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  throw_status(stage_status);
  for (uint32_t l = 0; l < L; ++l)
    if (!std::equal(placed[l].begin(), placed[l].end(), cnt[l].begin()))
      throw Fail{PWMGPU_ERR_CUDA, "internal: pieces do not add up to the text"};
  // words shared by runs: OR of their parts; padding words past each level: zero
  std::sort(acc.begin(), acc.end());
  for (size_t i = 0; i < acc.size();) {
    uint64_t v = 0;
    size_t k = i;
    for (; k < acc.size() && acc[k][0] == acc[i][0] && acc[k][1] == acc[i][1]; ++k) v |= acc[k][2];
    outs[acc[i][0]].host[acc[i][1]] = v;
    i = k;
  }
  for (const Out& o : outs)
    for (uint32_t l = 0; l < L; ++l)
      std::fill(o.host + uint64_t(l) * lw + words_for(n), o.host + uint64_t(l + 1) * lw, uint64_t(0));
}

// The device text of a build in its key width: 40-bit symbols widened into
// scratch, others as they are.
const void* build_input(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, const void* d_text) {
  if (wx->in_width != 5) return d_text;
  auto* wide = static_cast<uint32_t*>(ctx->grow("wide_text", std::max<uint64_t>(wx->n, 1) * 4));
  launch_widen40(d_text, wx->n, wide, ctx->stream, &ctx->launches);
  CUDA_TRY(cudaGetLastError());
  return wide;
}

// A host text of 40-bit symbols: copied up and widened; the build then runs
// from the device text with only the outputs on the host.
const void* upload_wide_host_text(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, const void* host_text) {
  void* d40 = ctx->grow("text40", std::max<uint64_t>(wx->n, 1) * 5);
  CUDA_TRY(cudaMemcpyAsync(d40, host_text, wx->n * 5, cudaMemcpyHostToDevice, ctx->stream));
  return build_input(ctx, wx, d40);
}

constexpr uint32_t kMergeMaxLevels = 16;

// pwm's merge_bit_vectors (merge.hpp:192-465) on the device: per level the
// runs of every block and shard in the level's order, gathered word by word.
void merge_shards(pwmgpu_ctx* ctx, const std::vector<const pwmgpu_wx*>& sh, pwmgpu_wx* out) {
  const uint32_t L = out->levels, p = uint32_t(sh.size());
  if (p == 0) throw Fail{PWMGPU_ERR_ARG, "no shards"};
  if (out->huffman) throw Fail{PWMGPU_ERR_ARG, "merging takes plain structures"};
  if (L > kMergeMaxLevels) throw Fail{PWMGPU_ERR_ARG, "merging takes structures of at most 16 levels"};
  uint64_t total = 0;
  for (const pwmgpu_wx* x : sh) {
    if (!x || x->huffman) throw Fail{PWMGPU_ERR_ARG, "merging takes plain structures"};
    if (x->width != out->width || x->levels != L) throw Fail{PWMGPU_ERR_ARG, "shards of another width or level count"};
    if (x->hist.size() != (size_t(1) << L))
      throw Fail{PWMGPU_ERR_ARG, "a shard without its histogram (create with PWMGPU_KEEP_HISTOGRAM and build it)"};
    if (out->wt.present && !x->wt.present) throw Fail{PWMGPU_ERR_ARG, "a shard without the tree"};
    total += x->n;
  }
  if (total != out->n) throw Fail{PWMGPU_ERR_ARG, "the shards' sizes do not add up to out's"};
  cudaStream_t st = ctx->stream;
  CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, 4, st));
  std::vector<PrefixCounts> cnt(p);
  for (uint32_t s = 0; s < p; ++s) cnt[s] = fold_prefix_counts(sh[s]->hist.data(), L);
  for (int which = 0; which < 2; ++which) {
    Structure& O = which ? out->wt : out->wm;
    if (!O.present || out->n == 0) continue;
    std::vector<MergeSeg> segs;
    std::vector<size_t> seg_off(L + 1, 0);
    for (uint32_t l = 0; l < L; ++l) {
      seg_off[l] = segs.size();
      for (const MergeRun& r : plan_merge_level(cnt, l, which == 1)) {
        const Structure& S = which ? sh[r.shard]->wt : sh[r.shard]->wm;
        segs.push_back({r.dst, r.src_bit, S.d_words + S.offs[l]});
      }
    }
    seg_off[L] = segs.size();
    auto* d_segs = static_cast<MergeSeg*>(ctx->grow("merge_segs", std::max<size_t>(segs.size(), 1) * sizeof(MergeSeg)));
    // (a copy from a pageable host vector returns once the data is staged)
    CUDA_TRY(cudaMemcpyAsync(d_segs, segs.data(), segs.size() * sizeof(MergeSeg), cudaMemcpyHostToDevice, st));
    for (uint32_t l = 0; l < L; ++l) {
      ProfScope ps(ctx, "merge", 2 * words_for(O.bits[l]) * 8);
      launch_merge_gather(d_segs + seg_off[l], seg_off[l + 1] - seg_off[l], O.d_words + O.offs[l], O.bits[l],
                          ctx->d_status, st, &ctx->launches);
    }
    CUDA_TRY(cudaGetLastError());
  }
  out->wm.zeros.assign(L, 0);
  for (const pwmgpu_wx* x : sh)
    for (uint32_t l = 0; l < L && l < x->wm.zeros.size(); ++l) out->wm.zeros[l] += x->wm.zeros[l];
  CUDA_TRY(cudaMemcpyAsync(out->wm.d_zeros, out->wm.zeros.data(), L * 8, cudaMemcpyHostToDevice, st));
  if (out->keep_hist) {
    out->hist.assign(size_t(1) << L, 0);
    for (const pwmgpu_wx* x : sh)
      for (size_t b = 0; b < out->hist.size(); ++b) out->hist[b] += x->hist[b];
  }
  build_rank_select(ctx, out->wm.rs && !out->wm_internal ? &out->wm : nullptr, out->wt.present ? &out->wt : nullptr,
                    true);
  check_device_status(ctx);  // synchronises: the shards may be freed after this
}

}  // namespace

extern "C" {

const char* pwmgpu_status_string(pwmgpu_status s) {
  switch (s) {
    case PWMGPU_OK: return "ok";
    case PWMGPU_ERR_ARG: return "invalid argument";
    case PWMGPU_ERR_OOM: return "out of device memory";
    case PWMGPU_ERR_CUDA: return "CUDA error";
    case PWMGPU_ERR_TIMEOUT: return "device-side wait timed out";
    case PWMGPU_ERR_SYMBOL: return "symbol out of range";
    case PWMGPU_ERR_NO_DEVICE: return "no usable CUDA device";
    case PWMGPU_ERR_BUSY: return "admission refused";
  }
  return "unknown status";
}

pwmgpu_status pwmgpu_ctx_create(int device, void* cuda_stream, pwmgpu_ctx** out) {
  if (!out) return PWMGPU_ERR_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0 || device < 0 || device >= count) {
    cudaGetLastError();
    return PWMGPU_ERR_NO_DEVICE;
  }
  auto* ctx = new pwmgpu_ctx;
  ctx->device = device;
  pwmgpu_status st = guarded(ctx, [&]() {
    if (cuda_stream) {
      ctx->stream = static_cast<cudaStream_t>(cuda_stream);
    } else {
      CUDA_TRY(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
      ctx->own_stream = true;
    }
    CUDA_TRY(cudaMalloc(&ctx->d_status, 64));
    CUDA_TRY(cudaMemset(ctx->d_status, 0, 64));
    // a kernel of this library must be loadable on this device
    cudaFuncAttributes attr;
    cudaError_t e = cudaFuncGetAttributes(&attr, reinterpret_cast<const void*>(&pwmgpu_ctx_create));
    (void)e;
    cudaGetLastError();
    return PWMGPU_OK;
  });
  if (st != PWMGPU_OK) {
    delete ctx;
    return st;
  }
  *out = ctx;
  return PWMGPU_OK;
}

void pwmgpu_ctx_destroy(pwmgpu_ctx* ctx) { delete ctx; }

const char* pwmgpu_ctx_last_error(const pwmgpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

pwmgpu_status pwmgpu_ctx_sync(pwmgpu_ctx* ctx) {
  if (!ctx) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return PWMGPU_OK;
  });
}

uint64_t pwmgpu_ctx_launch_count(const pwmgpu_ctx* ctx) { return ctx ? ctx->launches : 0; }

pwmgpu_status pwmgpu_ctx_set_pass_levels(pwmgpu_ctx* ctx, int k) {
  if (!ctx || k < 0 || k > kMaxPassLevels || k > kTileMaxLevels) return PWMGPU_ERR_ARG;
  ctx->pass_levels = k ? k : kDefaultPassLevels;
  ctx->tile_levels = k;
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_ctx_set_stream_ordered_alloc(pwmgpu_ctx* ctx, int enable) {
  if (!ctx) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    if (enable && !ctx->async_alloc) {
      // freed blocks stay in this process's pool for the next allocation
      cudaMemPool_t pool;
      CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, ctx->device));
      uint64_t keep = ~uint64_t(0);
      CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
    ctx->async_alloc = enable != 0;
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_ctx_set_engine(pwmgpu_ctx* ctx, int engine) {
  if (!ctx || (engine != PWMGPU_ENGINE_TILE && engine != PWMGPU_ENGINE_WARP)) return PWMGPU_ERR_ARG;
  ctx->engine = engine;
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_ctx_set_upload_piece_bytes(pwmgpu_ctx* ctx, uint64_t bytes) {
  if (!ctx || bytes == 0) return PWMGPU_ERR_ARG;
  ctx->upload_piece = bytes;
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_ctx_release_scratch(pwmgpu_ctx* ctx) {
  if (!ctx) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    for (cudaStream_t t : {ctx->stream, ctx->up, ctx->down, ctx->side})
      if (t) CUDA_TRY(cudaStreamSynchronize(t));
    delete ctx->compute_cache;
    ctx->compute_cache = nullptr;
    ctx->shard_cache.clear();
    ctx->semi_shard[0].reset();
    ctx->semi_shard[1].reset();
    for (auto& kv : ctx->scratch)
      if (kv.second.p) {
        if (ctx->async_alloc) CUDA_TRY(cudaFreeAsync(kv.second.p, ctx->stream));
        else CUDA_TRY(cudaFree(kv.second.p));
      }
    ctx->scratch.clear();
    ctx->scratch_bytes = 0;
    if (ctx->async_alloc) CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->release_pinned();
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_ctx_set_stream_chunks(pwmgpu_ctx* ctx, uint32_t chunks) {
  if (!ctx || chunks == 0 || chunks > kMaxStreamChunks) return PWMGPU_ERR_ARG;
  ctx->stream_chunks = chunks;
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_ctx_set_spin_limit(pwmgpu_ctx* ctx, uint32_t polls) {
  if (!ctx) return PWMGPU_ERR_ARG;
  ctx->spin_limit = polls ? polls : kSpinLimit;
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_ctx_test_withhold_tile(pwmgpu_ctx* ctx, int enable) {
  if (!ctx) return PWMGPU_ERR_ARG;
  ctx->withhold_first_tile = enable != 0;
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_ctx_profile(pwmgpu_ctx* ctx, int enable) {
  if (!ctx) return PWMGPU_ERR_ARG;
  ctx->profiling = enable != 0;
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_ctx_profile_read(pwmgpu_ctx* ctx, char* buf, uint64_t cap) {
  if (!ctx || !buf || cap == 0) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    struct Agg { uint64_t groups = 0, launches = 0, bytes = 0; double ms = 0; };
    std::map<std::string, Agg> agg;
    for (auto& r : ctx->prof) {
      float ms = 0;
      CUDA_TRY(cudaEventElapsedTime(&ms, r.a, r.b));
      auto& g = agg[r.name];
      g.groups += 1;
      g.launches += r.launches;
      g.bytes += r.bytes;
      g.ms += ms;
      ctx->event_pool.push_back(r.a);
      ctx->event_pool.push_back(r.b);
    }
    ctx->prof.clear();
    std::string out;
    char line[256];
    for (auto& kv : agg) {
      std::snprintf(line, sizeof(line), "%s %llu %llu %.6f %llu\n", kv.first.c_str(),
                    (unsigned long long)kv.second.groups, (unsigned long long)kv.second.launches, kv.second.ms,
                    (unsigned long long)kv.second.bytes);
      out += line;
    }
    if (out.size() + 1 > cap) throw Fail{PWMGPU_ERR_ARG, "profile buffer too small"};
    std::memcpy(buf, out.c_str(), out.size() + 1);
    return PWMGPU_OK;
  });
}

// ---- device-resident structures --------------------------------------------

pwmgpu_status pwmgpu_wx_merge(pwmgpu_ctx* ctx, const pwmgpu_wx* const* shards, uint32_t count, pwmgpu_wx* out) {
  if (!ctx || !out || (count && !shards)) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    merge_shards(ctx, std::vector<const pwmgpu_wx*>(shards, shards + count), out);
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_build_sharded(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* d_text, uint32_t shards) {
  if (!ctx || !wx || shards == 0 || (!d_text && wx->n)) return PWMGPU_ERR_ARG;
  if (wx->huffman) return fail(ctx, PWMGPU_ERR_ARG, "a Huffman-shaped wx is built by pwmgpu_wx_build_huffman");
  return guarded(ctx, [&]() {
    d_text = build_input(ctx, wx, d_text);
    if (shards == 1 || wx->n == 0) {
      build_plain(ctx, wx, d_text);
      return PWMGPU_OK;
    }
    const uint32_t shape = (wx->wm_internal ? 0u : PWMGPU_MATRIX) | (wx->wt.present ? PWMGPU_TREE : 0u) |
                           PWMGPU_KEEP_HISTOGRAM;
    // the shard structures stay in the context for the next build of this shape
    auto& parts = ctx->shard_cache;
    std::vector<const pwmgpu_wx*> view;
    const uint64_t n = wx->n, base = n / shards, extra = n % shards;
    if (parts.size() > shards) parts.resize(shards);
    for (uint32_t s = 0; s < shards; ++s) {  // pwm's slices (wx_dd_ps.hpp:66-83)
      const uint64_t size = base + (s < extra ? 1 : 0), off = s * base + std::min<uint64_t>(s, extra);
      if (s == parts.size()) parts.emplace_back();
      auto& part = parts[s];
      if (!part || part->n != size || part->width != wx->width || part->levels != wx->levels || part->flags != shape)
        part = make_wx(ctx, size, wx->width, wx->levels, shape);
      build_plain(ctx, part.get(), static_cast<const unsigned char*>(d_text) + off * wx->width);
      view.push_back(part.get());
    }
    merge_shards(ctx, view, wx);
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_copy_bits(uint64_t* d_dst, const uint64_t* d_src, uint64_t dst_off, uint64_t src_off,
                               uint64_t len, void* cuda_stream) {
  if (len && (!d_dst || !d_src)) return PWMGPU_ERR_ARG;
  launch_copy_bits(d_dst, d_src, dst_off, src_off, len, static_cast<cudaStream_t>(cuda_stream));
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return PWMGPU_OK;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
    return PWMGPU_ERR_NO_DEVICE;
  return PWMGPU_ERR_CUDA;
}

pwmgpu_status pwmgpu_wx_create(pwmgpu_ctx* ctx, uint64_t size, uint32_t word_width, uint32_t levels,
                               uint32_t shape_flags, pwmgpu_wx** out) {
  if (!ctx || !out) return PWMGPU_ERR_ARG;
  *out = nullptr;
  return guarded(ctx, [&]() {
    validate_plain(size, word_width, levels, true);
    if (!(shape_flags & (PWMGPU_MATRIX | PWMGPU_TREE))) throw Fail{PWMGPU_ERR_ARG, "need PWMGPU_MATRIX or PWMGPU_TREE"};
    if ((shape_flags & PWMGPU_RANK_SELECT) && size >= 4294967295ull - 64)
      throw Fail{PWMGPU_ERR_ARG, "rank/select support needs levels below 2^32-1 bits"};
    *out = make_wx(ctx, size, word_width, levels, shape_flags).release();
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_build(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* d_text) {
  if (!ctx || !wx || (!d_text && wx->n)) return PWMGPU_ERR_ARG;
  if (wx->huffman) return fail(ctx, PWMGPU_ERR_ARG, "a Huffman-shaped wx is built by pwmgpu_wx_build_huffman");
  return guarded(ctx, [&]() {
    build_plain(ctx, wx, build_input(ctx, wx, d_text));
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_build_host(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* host_text) {
  if (!ctx || !wx || (!host_text && wx->n)) return PWMGPU_ERR_ARG;
  if (wx->huffman) return fail(ctx, PWMGPU_ERR_ARG, "a Huffman-shaped wx is built by pwmgpu_wx_build_huffman");
  return guarded(ctx, [&]() {
    if (wx->in_width == 5) {
      build_plain(ctx, wx, upload_wide_host_text(ctx, wx, host_text));
      return PWMGPU_OK;
    }
    void* d_text = ctx->grow("host_text", std::max<uint64_t>(wx->n * wx->width, 1));
    HostIO io;
    io.text = host_text;
    build_plain(ctx, wx, d_text, &io);
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_compute_host(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* host_text, uint64_t* wm_bv,
                                     uint64_t* wm_zeros, uint64_t* wt_bv) {
  if (!ctx || !wx || (!host_text && wx->n)) return PWMGPU_ERR_ARG;
  if (wx->huffman) return fail(ctx, PWMGPU_ERR_ARG, "a Huffman-shaped wx is built by pwmgpu_wx_build_huffman");
  if ((wm_bv && (!wx->wm.present || wx->wm_internal)) || (wt_bv && !wx->wt.present))
    return fail(ctx, PWMGPU_ERR_ARG, "an output structure the wx does not hold");
  return guarded(ctx, [&]() {
    HostIO io;
    io.wm = wm_bv;
    io.wt = wt_bv;
    if (wx->in_width == 5) {
      build_plain(ctx, wx, upload_wide_host_text(ctx, wx, host_text), &io);
    } else {
      void* d_text = ctx->grow("host_text", std::max<uint64_t>(wx->n * wx->width, 1));
      io.text = host_text;
      build_plain(ctx, wx, d_text, &io);
    }
    check_device_status(ctx);
    if (wm_zeros && wx->wm.present && !wx->wm_internal) std::memcpy(wm_zeros, wx->wm.zeros.data(), wx->levels * 8);
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_check(pwmgpu_ctx* ctx, pwmgpu_wx* wx) {
  if (!ctx || !wx) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    CUDA_TRY(cudaGetLastError());
    check_device_status(ctx);
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_view(const pwmgpu_wx* wx, int which, pwmgpu_view* v) {
  if (!wx || !v) return PWMGPU_ERR_ARG;
  const Structure& s = which ? wx->wt : wx->wm;
  if (!s.present || (which == 0 && wx->wm_internal)) return PWMGPU_ERR_ARG;
  v->levels = s.levels;
  v->is_tree = s.is_tree;
  v->is_huffman = s.huffman;
  v->has_rank_select = s.rs;
  v->size = s.n;
  v->total_words = s.total_words;
  v->words = s.d_words;
  v->level_offset = s.offs.data();
  v->level_bits = s.bits.data();
  v->zeros = s.is_tree ? nullptr : s.zeros.data();
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_wx_download(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, int which, uint64_t* bv, uint64_t* zeros) {
  if (!ctx || !wx || !bv) return PWMGPU_ERR_ARG;
  const Structure& s = which ? wx->wt : wx->wm;
  if (!s.present) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    if (s.total_words)
      CUDA_TRY(cudaMemcpyAsync(bv, s.d_words, s.total_words * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (zeros && !s.is_tree) std::memcpy(zeros, s.zeros.data(), s.levels * 8);
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_rank_select_blocks(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, int which, uint32_t level,
                                           uint64_t* l0, uint32_t* l12, uint32_t* s0, uint32_t* s1, uint64_t* counts) {
  if (!ctx || !wx || !counts) return PWMGPU_ERR_ARG;
  const Structure& s = which ? wx->wt : wx->wm;
  if (!s.present || !s.rs || level >= s.levels) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    const RankSelectLevel& r = s.rs_levels[level];
    uint64_t meta[3];
    CUDA_TRY(cudaMemcpyAsync(meta, r.meta, 24, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    counts[0] = rs_n0(r.nwords);
    counts[1] = rs_n12(r.nwords);
    counts[2] = meta[0];
    counts[3] = meta[1];
    if (l0) CUDA_TRY(cudaMemcpyAsync(l0, r.l0, counts[0] * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (l12) CUDA_TRY(cudaMemcpyAsync(l12, r.l12, counts[1] * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (s0 && counts[2]) CUDA_TRY(cudaMemcpyAsync(s0, r.s0, counts[2] * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (s1 && counts[3]) CUDA_TRY(cudaMemcpyAsync(s1, r.s1, counts[3] * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_query(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, int which, int op, const uint64_t* d_a,
                              const uint64_t* d_b, uint64_t count, uint64_t* d_out) {
  if (!ctx || !wx || op < 0 || op > 2 || (count && (!d_a || !d_out || (op > 0 && !d_b)))) return PWMGPU_ERR_ARG;
  const Structure& s = which ? wx->wt : wx->wm;
  if (!s.present || !s.rs || (which == 0 && wx->wm_internal))
    return fail(ctx, PWMGPU_ERR_ARG, "queries need a structure with rank/select");
  return guarded(ctx, [&]() {
    QueryStructure q{s.levels, s.is_tree ? 1u : 0u, s.n, s.d_q_levels, s.d_zeros};
    ProfScope ps(ctx, "queries", count * 24);
    if (s.huffman) launch_huff_queries(q, wx->hq, op, d_a, d_b, count, d_out, ctx->stream, &ctx->launches);
    else launch_queries(q, op, d_a, d_b, count, d_out, ctx->stream, &ctx->launches);
    CUDA_TRY(cudaGetLastError());
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_query_host(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, int which, int op, const uint64_t* a,
                                   const uint64_t* b, uint64_t count, uint64_t* out) {
  if (!ctx || !wx || op < 0 || op > 2 || (count && (!a || !out || (op > 0 && !b)))) return PWMGPU_ERR_ARG;
  if (count == 0) return PWMGPU_OK;
  const Structure& s = which ? wx->wt : wx->wm;
  if (!s.present || !s.rs || (which == 0 && wx->wm_internal))
    return fail(ctx, PWMGPU_ERR_ARG, "queries need a structure with rank/select");
  return guarded(ctx, [&]() {
    auto* d = static_cast<uint64_t*>(ctx->grow("query_io", count * 3 * 8));
    cudaStream_t st = ctx->stream;
    CUDA_TRY(cudaMemcpyAsync(d, a, count * 8, cudaMemcpyHostToDevice, st));
    if (op > 0) CUDA_TRY(cudaMemcpyAsync(d + count, b, count * 8, cudaMemcpyHostToDevice, st));
    QueryStructure q{s.levels, s.is_tree ? 1u : 0u, s.n, s.d_q_levels, s.d_zeros};
    {
      ProfScope ps(ctx, "queries", count * 24);
      if (s.huffman) launch_huff_queries(q, wx->hq, op, d, d + count, count, d + 2 * count, st, &ctx->launches);
      else launch_queries(q, op, d, d + count, count, d + 2 * count, st, &ctx->launches);
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(out, d + 2 * count, count * 8, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return PWMGPU_OK;
  });
}

// pwm's reduce_alphabet for symbols too wide for one bin per value (40-bit,
// or 32-bit from 2^24 up): a device hash table finds the distinct symbols and
// their first positions, the host numbers them by first position, and the
// text is renumbered through the table.  Returns the distinct symbols - 1.
uint64_t reduce_alphabet_hashed(pwmgpu_ctx* ctx, const void* d_text, uint64_t n, uint32_t width, void* d_out) {
  if (n > kAlphabetHashMaxSymbols) throw Fail{PWMGPU_ERR_ARG, "alphabet reduction of wide symbols: at most 2^30 symbols"};
  cudaStream_t s = ctx->stream;
  uint64_t cap = 1024;
  while (cap < 2 * n) cap <<= 1;
  auto* keys = static_cast<unsigned long long*>(ctx->grow("alpha_keys", cap * 8));
  auto* first = static_cast<unsigned long long*>(ctx->grow("alpha_first", cap * 8));
  auto* slot_ids = static_cast<uint32_t*>(ctx->grow("alpha_slot_ids", cap * 4));
  auto* count = static_cast<unsigned long long*>(ctx->grow("alpha_count", 8));
  auto* triples = static_cast<uint64_t*>(ctx->grow("alpha_triples", n * 24));
  CUDA_TRY(cudaMemsetAsync(keys, 0xFF, cap * 8, s));
  CUDA_TRY(cudaMemsetAsync(first, 0xFF, cap * 8, s));
  CUDA_TRY(cudaMemsetAsync(count, 0, 8, s));
  launch_alphabet_insert(d_text, width, n, keys, first, cap, ctx->d_status, s, &ctx->launches);
  launch_alphabet_collect(keys, first, cap, count, triples, s, &ctx->launches);
  uint64_t sigma = 0;
  CUDA_TRY(cudaMemcpyAsync(&sigma, count, 8, cudaMemcpyDeviceToHost, s));
  check_device_status(ctx);
  if (sigma == 0 || sigma > n) throw Fail{PWMGPU_ERR_CUDA, "internal: alphabet table inconsistent"};
  std::vector<uint64_t> t(3 * sigma);
  CUDA_TRY(cudaMemcpyAsync(t.data(), triples, sigma * 24, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<uint64_t> order(sigma);
  std::iota(order.begin(), order.end(), uint64_t(0));
  std::sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) { return t[3 * a + 2] < t[3 * b + 2]; });
  std::vector<uint64_t> slots(sigma);
  std::vector<uint32_t> ids(sigma);
  for (uint64_t r = 0; r < sigma; ++r) {
    slots[r] = t[3 * order[r]];
    ids[r] = uint32_t(r);
  }
  // slots and ids go where the triples were (no longer needed on the device)
  CUDA_TRY(cudaMemcpyAsync(triples, slots.data(), sigma * 8, cudaMemcpyHostToDevice, s));
  auto* d_ids = reinterpret_cast<uint32_t*>(triples + sigma);
  CUDA_TRY(cudaMemcpyAsync(d_ids, ids.data(), sigma * 4, cudaMemcpyHostToDevice, s));
  launch_scatter_ids(triples, d_ids, sigma, slot_ids, s, &ctx->launches);
  launch_alphabet_remap(d_text, width, n, keys, slot_ids, cap, d_out, ctx->d_status, s, &ctx->launches);
  check_device_status(ctx);  // also: the pageable copies above have been read
  return sigma - 1;
}

pwmgpu_status pwmgpu_reduce_alphabet(pwmgpu_ctx* ctx, const void* d_text, uint64_t size, uint32_t word_width,
                                     void* d_out, uint64_t* max_char) {
  if (!ctx || !max_char || (size && (!d_text || !d_out))) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    if (!valid_plain_width(word_width)) throw Fail{PWMGPU_ERR_ARG, "word_width must be 1, 2, 4 or 5"};
    *max_char = ~uint64_t(0);  // pwm: no symbol, 0 - 1
    if (size == 0) return PWMGPU_OK;
    cudaStream_t s = ctx->stream;
    CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, 4, s));
    uint64_t nsym = word_width == 1 ? 256 : 65536;
    bool hashed = word_width == 5;
    if (word_width == 4) {
      auto* d_max = static_cast<unsigned int*>(ctx->grow("alpha_max", 4));
      CUDA_TRY(cudaMemsetAsync(d_max, 0, 4, s));
      launch_max_symbol(static_cast<const uint32_t*>(d_text), size, d_max, s, &ctx->launches);
      unsigned int mx = 0;
      CUDA_TRY(cudaMemcpyAsync(&mx, d_max, 4, cudaMemcpyDeviceToHost, s));
      CUDA_TRY(cudaStreamSynchronize(s));
      hashed = mx >= kAlphabetMaxSymbol;
      nsym = uint64_t(mx) + 1;
    }
    if (hashed) {
      *max_char = reduce_alphabet_hashed(ctx, d_text, size, word_width, d_out);
      return PWMGPU_OK;
    }
    // symbol counts and first occurrences, then ids in order of first occurrence
    auto* d_hist = static_cast<unsigned long long*>(ctx->grow("sym_hist", nsym * 8));
    auto* d_first = static_cast<unsigned long long*>(ctx->grow("sym_first", nsym * 8));
    CUDA_TRY(cudaMemsetAsync(d_hist, 0, nsym * 8, s));
    CUDA_TRY(cudaMemsetAsync(d_first, 0xFF, nsym * 8, s));
    {
      ProfScope ps(ctx, "symbol_histogram", size * word_width);
      launch_symbol_histogram(d_text, size, word_width, nsym, d_hist, d_first, ctx->d_status, s, &ctx->launches);
    }
    std::vector<uint64_t> count(nsym), first(nsym);
    CUDA_TRY(cudaMemcpyAsync(count.data(), d_hist, nsym * 8, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(first.data(), d_first, nsym * 8, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<uint32_t> present;
    for (uint64_t c = 0; c < nsym; ++c)
      if (count[c]) present.push_back(uint32_t(c));
    std::sort(present.begin(), present.end(), [&](uint32_t a, uint32_t b) { return first[a] < first[b]; });
    std::vector<uint32_t> map(nsym, 0);
    for (size_t i = 0; i < present.size(); ++i) map[present[i]] = uint32_t(i);
    auto* d_map = static_cast<uint32_t*>(ctx->grow("alpha_map", nsym * 4));
    CUDA_TRY(cudaMemcpyAsync(d_map, map.data(), nsym * 4, cudaMemcpyHostToDevice, s));
    launch_remap(d_text, size, word_width, d_map, nsym, d_out, ctx->d_status, s, &ctx->launches);
    check_device_status(ctx);  // also: the map's pageable copy has been read
    *max_char = present.size() - 1;
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_compute_semi_external(pwmgpu_ctx* ctx, const void* text, uint64_t size, uint32_t word_width,
                                           uint32_t levels, uint64_t* wm_bv, uint64_t* wm_zeros, uint64_t* wt_bv,
                                           uint64_t device_budget) {
  if (!ctx || (size && !text) || (!wm_bv && !wt_bv)) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    validate_plain(size, word_width, levels);
    if (size == 0) {
      if (wm_zeros) std::memset(wm_zeros, 0, levels * 8);
      return PWMGPU_OK;
    }
    semi_external(ctx, text, size, word_width, levels, wm_bv, wm_zeros, wt_bv, device_budget);
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_build_huffman(pwmgpu_ctx* ctx, const void* d_text, uint64_t size, uint32_t word_width,
                                      uint32_t shape_flags, const uint64_t* code_len, const uint64_t* code_word,
                                      uint64_t num_codes, pwmgpu_wx** out) {
  if (!ctx || !out || !d_text) return PWMGPU_ERR_ARG;
  *out = nullptr;
  return guarded(ctx, [&]() {
    if (!valid_width(word_width)) throw Fail{PWMGPU_ERR_ARG, "word_width must be 1, 2 or 4"};
    if (size == 0) throw Fail{PWMGPU_ERR_ARG, "a Huffman-shaped structure needs a non-empty text"};
    const bool tree = shape_flags & PWMGPU_TREE;
    if (tree == bool(shape_flags & PWMGPU_MATRIX))
      throw Fail{PWMGPU_ERR_ARG, "a Huffman-shaped wx holds one structure: PWMGPU_MATRIX or PWMGPU_TREE"};
    const bool rs = shape_flags & PWMGPU_RANK_SELECT;
    if (rs && size >= 4294967295ull - 64) throw Fail{PWMGPU_ERR_ARG, "rank/select support needs levels below 2^32-1 bits"};
    auto wx = std::make_unique<pwmgpu_wx>();
    wx->ctx = ctx;
    wx->n = size;
    wx->width = word_width;
    wx->flags = shape_flags;
    wx->huffman = true;
    uint32_t L = 0;
    if (code_len) {
      if (!code_word || num_codes == 0) throw Fail{PWMGPU_ERR_ARG, "code table incomplete"};
      wx->code_len.assign(code_len, code_len + num_codes);
      wx->code_word.assign(code_word, code_word + num_codes);
    } else {
      uint64_t max_symbol = 0;
      HuffCodes h = huffman_codes_device(ctx, d_text, size, word_width, tree, &max_symbol);
      wx->code_len = h.len;
      wx->code_word = h.word;
      L = h.levels;
    }
    for (uint64_t c = 0; c < wx->code_len.size(); ++c) {
      if (wx->code_len[c] > 56) throw Fail{PWMGPU_ERR_ARG, "codes longer than 56 bits"};
      if (wx->code_len[c]) wx->code_word[c] &= (uint64_t(1) << wx->code_len[c]) - 1;
    }
    build_huffman(ctx, d_text, size, word_width, tree, wx->code_len, wx->code_word, L, wx->wm,
                  tree ? &wx->wt : nullptr, rs);
    const Structure& S = tree ? wx->wt : wx->wm;
    wx->levels = S.levels;
    if (tree) {  // the matrix was only the tree's source
      wx->wm.release();
      wx->wm.present = false;
      wx->wm_internal = true;
    }
    // device tables for queries: codes per symbol, codes sorted by (length, word), level sizes
    const uint64_t nsym = wx->code_len.size();
    std::vector<std::pair<uint64_t, uint64_t>> dec;
    for (uint64_t c = 0; c < nsym; ++c)
      if (wx->code_len[c]) dec.emplace_back((wx->code_len[c] << 56) | wx->code_word[c], c);
    std::sort(dec.begin(), dec.end());
    std::vector<uint64_t> blob;
    blob.reserve(2 * nsym + 2 * dec.size() + S.levels);
    blob.insert(blob.end(), wx->code_len.begin(), wx->code_len.end());
    blob.insert(blob.end(), wx->code_word.begin(), wx->code_word.end());
    for (const auto& d : dec) blob.push_back(d.first);
    for (const auto& d : dec) blob.push_back(d.second);
    blob.insert(blob.end(), S.bits.begin(), S.bits.end());
    CUDA_TRY(cudaMalloc(&wx->d_huff, std::max<size_t>(blob.size(), 1) * 8));
    CUDA_TRY(cudaMemcpyAsync(wx->d_huff, blob.data(), blob.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    const uint64_t* d = wx->d_huff;
    wx->hq = HuffQueryTables{d, d + nsym, nsym, d + 2 * nsym, d + 2 * nsym + dec.size(), dec.size(),
                             d + 2 * nsym + 2 * dec.size()};
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));  // the pageable table copy has been read
    *out = wx.release();
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_wx_codes(const pwmgpu_wx* wx, uint64_t* code_len, uint64_t* code_word, uint64_t cap,
                              uint64_t* num_codes) {
  if (!wx || !num_codes || !wx->huffman) return PWMGPU_ERR_ARG;
  *num_codes = wx->code_len.size();
  if (code_len || code_word) {
    if (!code_len || !code_word || cap < wx->code_len.size()) return PWMGPU_ERR_ARG;
    std::memcpy(code_len, wx->code_len.data(), wx->code_len.size() * 8);
    std::memcpy(code_word, wx->code_word.data(), wx->code_word.size() * 8);
  }
  return PWMGPU_OK;
}

void pwmgpu_wx_free(pwmgpu_wx* wx) {
  if (!wx) return;
  if (wx->ctx) cudaSetDevice(wx->ctx->device);
  delete wx;
}

// ---- drop-in host-to-host builds ------------------------------------------------
pwmgpu_status pwmgpu_compute(pwmgpu_ctx* ctx, const void* text, uint64_t size, uint32_t word_width, uint32_t levels,
                             int is_tree, uint64_t* bv, uint64_t* zeros) {
  if (!ctx) return PWMGPU_ERR_ARG;
  if (size == 0) return PWMGPU_OK;  // pwm: empty structure
  if (!text || !bv || (!is_tree && !zeros)) return fail(ctx, PWMGPU_ERR_ARG, "null text, bv or zeros");
  return guarded(ctx, [&]() {
    validate_plain(size, word_width, levels, true);
    const uint32_t shape = is_tree ? PWMGPU_TREE : PWMGPU_MATRIX;
    pwmgpu_wx*& wx = ctx->compute_cache;
    if (!wx || wx->n != size || wx->input_width() != word_width || wx->levels != levels || wx->flags != shape) {
      delete wx;
      wx = nullptr;
      pwmgpu_status st = pwmgpu_wx_create(ctx, size, word_width, levels, shape, &wx);
      if (st != PWMGPU_OK) return st;
    }
    HostIO io;
    (is_tree ? io.wt : io.wm) = bv;
    if (wx->in_width == 5) {
      build_plain(ctx, wx, upload_wide_host_text(ctx, wx, text), &io);
    } else {
      void* d_text = ctx->grow("host_text", size * word_width);
      io.text = text;
      build_plain(ctx, wx, d_text, &io);
    }
    const Structure& s = is_tree ? wx->wt : wx->wm;
    check_device_status(ctx);
    if (!is_tree) std::memcpy(zeros, s.zeros.data(), levels * 8);
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_huffman_codes(pwmgpu_ctx* ctx, const void* text, uint64_t size, uint32_t word_width, int is_tree,
                                   uint64_t* code_len, uint64_t* code_word, uint64_t cap, uint64_t* num_codes,
                                   uint64_t* level_sizes, uint32_t* levels) {
  if (!ctx || !num_codes || !levels) return PWMGPU_ERR_ARG;
  *num_codes = 0;
  *levels = 0;
  if (size == 0) return PWMGPU_OK;
  if (!text) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    if (word_width != 1 && word_width != 2)
      throw Fail{PWMGPU_ERR_ARG, "the code builder takes 8- or 16-bit texts; pass a code table for wider ones"};
    void* d_text = ctx->grow("host_text", size * word_width);
    CUDA_TRY(cudaMemcpyAsync(d_text, text, size * word_width, cudaMemcpyHostToDevice, ctx->stream));
    uint64_t max_symbol = 0;
    HuffCodes h = huffman_codes_device(ctx, d_text, size, word_width, is_tree != 0, &max_symbol);
    if (h.levels > kMaxLevels) throw Fail{PWMGPU_ERR_ARG, "codes longer than 64 bits"};
    *num_codes = max_symbol + 1;
    *levels = h.levels;
    if (code_len && code_word) {
      if (cap < max_symbol + 1) throw Fail{PWMGPU_ERR_ARG, "code table capacity too small"};
      std::memcpy(code_len, h.len.data(), (max_symbol + 1) * 8);
      std::memcpy(code_word, h.word.data(), (max_symbol + 1) * 8);
    }
    if (level_sizes) std::memcpy(level_sizes, h.level_sizes.data(), h.levels * 8);
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_compute_huffman(pwmgpu_ctx* ctx, const void* text, uint64_t size, uint32_t word_width,
                                     int is_tree, const uint64_t* code_len, const uint64_t* code_word,
                                     uint64_t num_codes, uint32_t levels, const uint64_t* level_sizes, uint64_t* bv,
                                     uint64_t* zeros) {
  if (!ctx) return PWMGPU_ERR_ARG;
  if (size == 0) return PWMGPU_OK;
  if (!text || !bv || (!is_tree && !zeros)) return fail(ctx, PWMGPU_ERR_ARG, "null text, bv or zeros");
  return guarded(ctx, [&]() {
    if (!valid_width(word_width)) throw Fail{PWMGPU_ERR_ARG, "word_width must be 1, 2 or 4"};
    void* d_text = ctx->grow("host_text", size * word_width);
    CUDA_TRY(cudaMemcpyAsync(d_text, text, size * word_width, cudaMemcpyHostToDevice, ctx->stream));
    std::vector<uint64_t> len, word;
    uint32_t L = levels;
    if (code_len) {
      if (!code_word || num_codes == 0) throw Fail{PWMGPU_ERR_ARG, "code table incomplete"};
      len.assign(code_len, code_len + num_codes);
      word.assign(code_word, code_word + num_codes);
    } else {
      uint64_t max_symbol = 0;
      HuffCodes h = huffman_codes_device(ctx, d_text, size, word_width, is_tree != 0, &max_symbol);
      len = h.len;
      word = h.word;
      L = h.levels;
    }
    Structure wm, wt;
    build_huffman(ctx, d_text, size, word_width, is_tree != 0, len, word, L, wm, is_tree ? &wt : nullptr, false);
    const Structure& s = is_tree ? wt : wm;
    if (level_sizes)
      for (uint32_t l = 0; l < L; ++l)
        if (level_sizes[l] != s.bits[l]) throw Fail{PWMGPU_ERR_ARG, "level_sizes do not match the code table"};
    CUDA_TRY(cudaMemcpyAsync(bv, s.d_words, s.total_words * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (!is_tree) std::memcpy(zeros, wm.zeros.data(), L * 8);
    wm.release();
    wt.release();
    return PWMGPU_OK;
  });
}

// ---- allocation-free rank/select ----------------------------------------------------
pwmgpu_status pwmgpu_rank_select_build_noalloc(const uint64_t* d_words, uint64_t nwords, uint64_t* d_l0,
                                               uint32_t* d_l12, uint32_t* d_select0, uint32_t* d_select1,
                                               uint64_t* d_counts, void* cuda_stream) {
  if ((nwords && !d_words) || !d_l0 || !d_l12 || !d_select0 || !d_select1 || !d_counts) return PWMGPU_ERR_ARG;
  if (nwords > PWMGPU_NOALLOC_RS_MAX_WORDS || nwords > noalloc_rank_select_max_words()) return PWMGPU_ERR_ARG;
  const cudaError_t e =
      noalloc_rank_select_build(d_words, nwords, d_l0, d_l12, d_select0, d_select1,
                                reinterpret_cast<unsigned long long*>(d_counts), static_cast<cudaStream_t>(cuda_stream));
  if (e == cudaSuccess) return PWMGPU_OK;
  if (e == cudaErrorInvalidValue) return PWMGPU_ERR_ARG;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
    return PWMGPU_ERR_NO_DEVICE;
  return PWMGPU_ERR_CUDA;
}

// ---- batches ---------------------------------------------------------------------
pwmgpu_status pwmgpu_batch_create(pwmgpu_ctx* ctx, uint32_t count, const uint64_t* offsets, const uint32_t* levels,
                                  uint32_t word_width, uint32_t shape_flags, int levels_per_pass,
                                  pwmgpu_batch** out) {
  if (!ctx || !out || (count && (!offsets || !levels))) return PWMGPU_ERR_ARG;
  *out = nullptr;
  return guarded(ctx, [&]() {
    if (!valid_width(word_width)) throw Fail{PWMGPU_ERR_ARG, "word_width must be 1, 2 or 4"};
    if (!(shape_flags & PWMGPU_MATRIX)) throw Fail{PWMGPU_ERR_ARG, "a batch builds wavelet matrices (and trees)"};
    if (levels_per_pass < 1 || levels_per_pass > kMaxPassLevels) throw Fail{PWMGPU_ERR_ARG, "levels_per_pass in 1..4"};
    auto b = std::make_unique<pwmgpu_batch>();
    b->ctx = ctx;
    b->count = count;
    b->width = word_width;
    b->flags = shape_flags;
    b->kmax = levels_per_pass;
    b->offs.assign(offsets, offsets + count + 1);
    b->L.assign(levels, levels + count);
    b->info.resize(count);
    b->wm_off.resize(count);
    b->wt_off.resize(count);
    b->words_per_level.resize(count);
    for (uint32_t t = 0; t < count; ++t) {
      if (b->offs[t + 1] < b->offs[t]) throw Fail{PWMGPU_ERR_ARG, "offsets must be non-decreasing"};
      if (b->L[t] == 0 || b->L[t] > kBatchMaxLevels) throw Fail{PWMGPU_ERR_ARG, "batch levels must be in 1..12"};
      const uint64_t n = b->offs[t + 1] - b->offs[t];
      b->maxL = std::max(b->maxL, b->L[t]);
      BatchText& bt = b->info[t];
      bt.offset = b->offs[t];
      bt.n = n;
      bt.levels = b->L[t];
      bt.hist_off = b->hist_n;
      bt.zeros_off = b->zeros_n;
      bt.starts_off = b->starts_n;
      bt.segs_off = b->segs_n;
      b->hist_n += uint64_t(1) << b->L[t];
      b->zeros_n += b->L[t];
      // room for the run starts of every pass plan (levels_per_pass may be retuned)
      uint64_t most = 0;
      for (int kk = 1; kk <= kMaxPassLevels; ++kk) {
        uint64_t need = 0;
        for (uint32_t l = 0; l < b->L[t];) {
          const int K = int(std::min<uint32_t>(uint32_t(kk), b->L[t] - l));
          need += uint64_t((2 << K) - 2);
          l += uint32_t(K);
        }
        most = std::max(most, need);
      }
      b->starts_n += most;
      b->segs_n += 2 * ((uint64_t(1) << b->L[t]) - 2);
      b->words_per_level[t] = padded_words(n);
      b->wm_off[t] = b->wm_words;
      b->wm_words += b->L[t] * padded_words(n);
      if (shape_flags & PWMGPU_TREE) {
        b->wt_off[t] = b->wt_words;
        b->wt_words += b->L[t] * padded_words(n);
      }
      for (uint64_t c = 0; c < n; c += kBatchChunk) b->chunks.push_back(BatchChunk{t, 0, c, std::min(kBatchChunk, n - c)});
      b->symbols += n;
    }
    b->d_info = static_cast<BatchText*>(b->dalloc(sizeof(BatchText) * std::max<uint32_t>(count, 1)));
    b->d_chunks = static_cast<BatchChunk*>(b->dalloc(sizeof(BatchChunk) * std::max<size_t>(b->chunks.size(), 1)));
    b->d_wm = static_cast<uint64_t*>(b->dalloc(b->wm_words * 8));
    if (shape_flags & PWMGPU_TREE) b->d_wt = static_cast<uint64_t*>(b->dalloc(b->wt_words * 8));
    b->d_zeros = static_cast<uint64_t*>(b->dalloc(b->zeros_n * 8));
    b->d_starts = static_cast<uint64_t*>(b->dalloc(b->starts_n * 8));
    b->d_segs = static_cast<uint64_t*>(b->dalloc(b->segs_n * 8));
    b->d_hist = static_cast<unsigned long long*>(b->dalloc(b->hist_n * 8));
    b->d_keys_a = b->dalloc(b->symbols * word_width);
    b->d_keys_b = b->dalloc(b->symbols * word_width);
    if (shape_flags & PWMGPU_TREE) {
      for (uint32_t t = 0; t < count; ++t) {
        const uint64_t n = b->offs[t + 1] - b->offs[t];
        const uint64_t nw = words_for(n);
        for (uint32_t m = 1; m < b->L[t]; ++m) {
          const uint64_t* seg = b->d_segs + b->info[t].segs_off + 2 * ((uint64_t(1) << m) - 2);
          for (uint64_t w = 0; w < nw; w += kBatchRegroupWords) {
            BatchRegroup it{};
            it.matrix = b->d_wm + b->wm_off[t] + m * b->words_per_level[t];
            it.tree = b->d_wt + b->wt_off[t] + m * b->words_per_level[t];
            it.nbits = n;
            it.seg_tree = seg;
            it.seg_matrix = seg + (uint64_t(1) << m);
            it.nseg = uint64_t(1) << m;
            it.word_begin = w;
            it.word_end = std::min(nw, w + kBatchRegroupWords);
            b->regroup.push_back(it);
          }
        }
      }
      b->d_regroup = static_cast<BatchRegroup*>(b->dalloc(sizeof(BatchRegroup) * std::max<size_t>(b->regroup.size(), 1)));
      if (!b->regroup.empty())
        CUDA_TRY(cudaMemcpy(b->d_regroup, b->regroup.data(), sizeof(BatchRegroup) * b->regroup.size(),
                            cudaMemcpyHostToDevice));
    }
    if (count) CUDA_TRY(cudaMemcpy(b->d_info, b->info.data(), sizeof(BatchText) * count, cudaMemcpyHostToDevice));
    if (!b->chunks.empty())
      CUDA_TRY(cudaMemcpy(b->d_chunks, b->chunks.data(), sizeof(BatchChunk) * b->chunks.size(), cudaMemcpyHostToDevice));
    *out = b.release();
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_batch_build(pwmgpu_ctx* ctx, pwmgpu_batch* b, const void* d_texts) {
  if (!ctx || !b || (!d_texts && b->symbols)) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    if (!b->exec || b->graph_text != d_texts || b->graph_k != b->kmax) {
      b->drop_graph();
      if (b->groups_k != b->kmax || b->groups.empty() || b->graph_text != d_texts) batch_plan(b, d_texts);
      // run once eagerly (configures kernel attributes), then capture the graph
      batch_enqueue(b, d_texts);
      CUDA_TRY(cudaStreamSynchronize(ctx->stream));
      CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      try {
        batch_enqueue(b, d_texts);
      } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(ctx->stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      CUDA_TRY(cudaStreamEndCapture(ctx->stream, &b->graph));
      CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
      b->graph_text = d_texts;
      b->graph_k = b->kmax;
      return PWMGPU_OK;  // the eager run above built the batch
    }
    CUDA_TRY(cudaGraphLaunch(b->exec, ctx->stream));
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_batch_set_levels_per_pass(pwmgpu_batch* b, int levels_per_pass) {
  if (!b || levels_per_pass < 1 || levels_per_pass > kMaxPassLevels) return PWMGPU_ERR_ARG;
  b->kmax = levels_per_pass;
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_batch_check(pwmgpu_ctx* ctx, pwmgpu_batch* b) {
  if (!ctx || !b) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    check_device_status(ctx);
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_batch_download(pwmgpu_ctx* ctx, const pwmgpu_batch* b, uint32_t index, int which, uint64_t* bv,
                                    uint64_t* zeros) {
  if (!ctx || !b || index >= b->count || !bv || (which && !(b->flags & PWMGPU_TREE))) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    const uint64_t words = b->L[index] * b->words_per_level[index];
    const uint64_t* src = which ? b->d_wt + b->wt_off[index] : b->d_wm + b->wm_off[index];
    if (words) CUDA_TRY(cudaMemcpyAsync(bv, src, words * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (zeros && !which)
      CUDA_TRY(cudaMemcpyAsync(zeros, b->d_zeros + b->info[index].zeros_off, b->L[index] * 8, cudaMemcpyDeviceToHost,
                               ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return PWMGPU_OK;
  });
}

void pwmgpu_batch_free(pwmgpu_batch* b) {
  if (!b) return;
  if (b->ctx) cudaSetDevice(b->ctx->device);
  delete b;
}

pwmgpu_status pwmgpu_generate_batch(uint64_t seed, uint32_t count, uint64_t* offsets, uint32_t* levels,
                                    uint8_t* texts) {
  if (!offsets || !levels) return PWMGPU_ERR_ARG;
  generate_batch_host(seed, count, offsets, levels, texts);
  return PWMGPU_OK;
}

// ---- generators ------------------------------------------------------------------
pwmgpu_status pwmgpu_generate(pwmgpu_ctx* ctx, int dist, uint64_t seed, uint64_t param, uint64_t n,
                              uint32_t word_width, void* out, int on_device) {
  if (!valid_width(word_width) || (n && !out) || dist < 0 || dist > 3) return PWMGPU_ERR_ARG;
  if (!on_device) {
    generate_host(dist, seed, param, n, word_width, out);
    return PWMGPU_OK;
  }
  const GenTables g = gen_tables(dist, seed);
  if (!ctx) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    auto* d_thr = static_cast<uint64_t*>(ctx->grow("gen_thr", g.thr.size() * 8));
    auto* d_perm = static_cast<uint32_t*>(ctx->grow("gen_perm", g.perm.size() * 4));
    CUDA_TRY(cudaMemcpyAsync(d_thr, g.thr.data(), g.thr.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(d_perm, g.perm.data(), g.perm.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    launch_generate(dist, seed, param, n, word_width, out, d_thr, uint32_t(g.thr.size()), d_perm, ctx->stream,
                    &ctx->launches);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return PWMGPU_OK;
  });
}

}  // extern "C"
