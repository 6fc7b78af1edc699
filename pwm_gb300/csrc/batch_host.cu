// Batches of independent plain texts built by one CUDA graph, and the seeded
// generators of the C ABI.
#include "engine.hpp"

using namespace pwmgpu;

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

extern "C" {

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
