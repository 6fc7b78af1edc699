// Batches of independent plain texts built by one CUDA graph, and the seeded
// generators of the C ABI.  Two engines: the tile engine (default: one
// persistent kernel over a device work queue of (text, pass, tile) items,
// tile_batch.cu, with the tile size of every text chosen by measurement and
// cached in the context) and the warp-pass engine (a kernel per pass shape,
// the tree regrouped from the matrix).
#include "engine.hpp"
#include "tile_batch.cuh"

using namespace pwmgpu;

// ===========================================================================
// Batches of independent plain texts
// ===========================================================================
namespace {

constexpr uint32_t kBatchMaxLevels = 12;        // per-text tables live in shared memory
constexpr uint64_t kBatchChunk = 65536;         // symbols per histogram CTA
constexpr size_t kTuneMaxTexts = 4096;           // texts of a tuning sub-batch (at most)
constexpr uint64_t kTuneSymbols = uint64_t(1) << 26;  // symbols of a tuning sub-batch (about)
constexpr uint32_t kGivenBlockTiles = 16;        // first-pass tiles per histogram block (a CTA's)
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
  // tile engine
  bool tile = true;
  uint32_t force_vpt = 0;            // 0: the tuned tile size of each text's class
  std::vector<uint32_t> vpt;         // vectors per thread of every text (planned)
  std::vector<void*> tile_owned;     // device arrays of the current tile plan
  TileBatchQueue queue{};
  uint32_t tile_ctas = 0, ntextpasses = 0, ngroups = 0;
  TileBatchText* d_tb_texts = nullptr;
  TileBatchPass* d_tb_passes = nullptr;
  TileBatchGroup* d_tb_groups = nullptr;
  uint64_t* d_pfx = nullptr;
  unsigned *d_done = nullptr, *d_need = nullptr, *d_group_tiles = nullptr, *d_head = nullptr;
  // histogram chunks of whole first-pass tiles, and those tiles' finest-run
  // counts and prefixes (the first pass's given prefixes)
  std::vector<BatchChunk> tchunks;
  BatchChunk* d_tchunks = nullptr;
  uint32_t *d_tilecnt = nullptr, *d_relpre = nullptr;
  unsigned long long *d_blocksum = nullptr, *d_blockpre = nullptr;
  std::vector<std::pair<void*, size_t>> lookback;  // per group
  const void* tile_text = nullptr;   // the text buffer the plan was made for
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
  void* talloc(size_t bytes) {
    void* p = nullptr;
    CUDA_TRY(cudaMalloc(&p, std::max<size_t>(bytes, 256)));
    tile_owned.push_back(p);
    return p;
  }
  void drop_tile_plan() {
    for (void* p : tile_owned) cudaFree(p);
    tile_owned.clear();
    lookback.clear();
    tile_text = nullptr;
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
    drop_tile_plan();
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
        char* ka = static_cast<char*>(b->d_keys_a) + (b->offs[t] - b->offs[0]) * b->width;
        char* kb = static_cast<char*>(b->d_keys_b) + (b->offs[t] - b->offs[0]) * b->width;
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
  launch_batch_hist(d_texts, b->width, b->d_chunks, uint32_t(b->chunks.size()), b->d_info, b->d_hist, nullptr, nullptr,
                    nullptr, ctx->d_status, s, &ctx->launches);
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

// ---- tile engine ------------------------------------------------------------
uint32_t floor_log2(uint64_t x) {
  uint32_t r = 0;
  while (x >>= 1) ++r;
  return r;
}

// Tuning class of a text: key width, levels and log2 of its length.
uint32_t tune_key(uint32_t width, uint32_t L, uint64_t n) {
  return (width << 16) | (L << 8) | floor_log2(std::max<uint64_t>(n, 1));
}

// Passes of one text on the tile engine: 4 levels each, the last one what is
// left; a pass writes the next sequence unless it is the last.
uint32_t tile_npass(uint32_t L) { return (L + uint32_t(kTileMaxLevels) - 1) / uint32_t(kTileMaxLevels); }

uint8_t tile_variant(uint32_t K, bool out) {
  if (out) return kTileBatchK4Out;  // only passes of kTileMaxLevels levels write S_{l+K}
  return K == 4 ? kTileBatchK4 : K == 3 ? kTileBatchK3 : K == 2 ? kTileBatchK2 : kTileBatchK1;
}

// Device descriptors of the batch's passes: groups of one pass shape in queue
// order (pass index first, so that a text's earlier passes come first), the
// segments, start tables, texts and look-back state of every group, and the
// queue.  The segments and tables themselves are filled on the device by the
// planning kernels of every build.
void tile_plan(pwmgpu_batch* b, const void* d_texts) {
  pwmgpu_ctx* ctx = b->ctx;
  b->drop_tile_plan();
  const uint32_t KPL = 16 / b->width;
  struct Item {
    uint32_t t, p, l, K;
    bool out;
  };
  std::map<std::pair<uint32_t, uint8_t>, std::vector<Item>> by;
  std::vector<uint32_t> first_slot(b->count, 0);
  uint32_t slots = 0;
  for (uint32_t t = 0; t < b->count; ++t) {
    const uint32_t L = b->L[t], np = tile_npass(L);
    first_slot[t] = slots;
    slots += np;
    for (uint32_t p = 0; p < np; ++p) {
      const uint32_t l = p * uint32_t(kTileMaxLevels), K = std::min<uint32_t>(uint32_t(kTileMaxLevels), L - l);
      const bool out = l + K < L;
      by[{p, tile_variant(K, out)}].push_back({t, p, l, K, out});
    }
  }
  if (by.size() > kTileBatchMaxGroups) throw Fail{PWMGPU_ERR_ARG, "too many pass shapes in one batch"};
  b->ntextpasses = slots;
  b->ngroups = uint32_t(by.size());
  // texts
  std::vector<TileBatchText> texts(b->count);
  uint64_t pfx = 0, key = 0;
  for (uint32_t t = 0; t < b->count; ++t) {
    TileBatchText& x = texts[t];
    x.text_begin = b->info[t].offset;
    x.key_begin = key;
    x.n = b->info[t].n;
    x.levels = b->L[t];
    x.hist_off = b->info[t].hist_off;
    x.pfx_off = pfx;
    x.zeros_off = b->info[t].zeros_off;
    pfx += tile_batch_scratch(b->L[t]);
    key += x.n;
  }
  std::vector<TileBatchPass> passes;
  std::vector<TileBatchGroup> groups;
  std::vector<TileArgs> args;
  TileBatchQueue q{};
  b->d_done = static_cast<unsigned*>(b->talloc(std::max<uint32_t>(slots, 1) * 4));
  b->d_need = static_cast<unsigned*>(b->talloc(std::max<uint32_t>(slots, 1) * 4));
  b->d_group_tiles = static_cast<unsigned*>(b->talloc(kTileBatchMaxGroups * 4));
  b->d_head = static_cast<unsigned*>(b->talloc(4));
  uint64_t tiles_all = 0;
  uint32_t gi = 0;
  // first passes: each text's tiles get given prefixes (counted by the
  // histogram kernel in chunks of whole tiles), at counter offsets of one
  // array for all first-pass groups
  uint64_t cnt_total = 0, blk_total = 0;
  struct GivenGroup {
    size_t arg;
    uint64_t cnt_off, blk_off;
  };
  std::vector<GivenGroup> given_groups;
  b->tchunks.clear();
  for (const auto& kv : by) {
    const auto& items = kv.second;
    const uint32_t K = items[0].K;
    const bool out = items[0].out;
    const uint32_t p = items[0].p;
    const int TS = tile_table_size(int(K));
    uint64_t nsegs = 0, tiles_ub = 1;
    for (const Item& it : items) {
      const uint64_t TT = uint64_t(256) * b->vpt[it.t] * KPL;
      nsegs += uint64_t(1) << it.l;
      tiles_ub += (b->info[it.t].n + TT - 1) / TT + (uint64_t(1) << it.l);
    }
    if (tiles_ub >= (uint64_t(1) << 31)) throw Fail{PWMGPU_ERR_ARG, "batch too large"};
    TileBatchGroup g{};
    g.segs = static_cast<TileSeg*>(b->talloc(nsegs * sizeof(TileSeg)));
    g.tables = static_cast<uint64_t*>(b->talloc(nsegs * uint64_t(TS) * 8));
    g.seg_tiles = static_cast<uint32_t*>(b->talloc(nsegs * 4));
    g.nsegs = uint32_t(nsegs);
    g.K = K;
    g.out = out ? 1u : 0u;
    auto* d_tx = static_cast<TileText*>(b->talloc(items.size() * sizeof(TileText)));
    std::vector<TileText> tx(items.size());
    uint64_t seg_base = 0;
    const uint32_t D = out ? K : K - 1;
    const bool given = p == 0 && D >= 1;
    const uint64_t group_cnt_off = cnt_total, group_blk_off = blk_total;
    uint64_t group_tile = 0, group_blk = 0;  // tiles and blocks of the group's texts so far (device order)
    for (size_t i = 0; i < items.size(); ++i) {
      const Item& it = items[i];
      const uint32_t t = it.t;
      const uint64_t wpl = b->words_per_level[t];
      TileText& x = tx[i];
      x.wm = b->d_wm + b->wm_off[t] + it.l * wpl;
      x.wt = (b->flags & PWMGPU_TREE) ? b->d_wt + b->wt_off[t] + it.l * wpl : nullptr;
      x.stride = wpl;
      x.nbits = b->info[t].n;
      x.shift = b->L[t] - 1 - it.l;
      x.vpt = b->vpt[t];
      x.wait_idx = it.p ? first_slot[t] + it.p - 1 : ~0u;
      x.signal_idx = it.p + 1 < tile_npass(b->L[t]) ? first_slot[t] + it.p : ~0u;
      TileBatchPass P{};
      P.text = t;
      P.group = gi;
      P.level = it.l;
      P.vpt = b->vpt[t];
      P.seg_base = uint32_t(seg_base);
      P.tt_index = uint32_t(i);
      P.slot = first_slot[t] + it.p;
      P.table_base = seg_base * uint64_t(TS);
      passes.push_back(P);
      seg_base += uint64_t(1) << it.l;
      if (given) {
        // blocks of kGivenBlockTiles tiles, one histogram CTA each
        const uint64_t TT = uint64_t(256) * b->vpt[t] * KPL, n = b->info[t].n, NB = uint64_t(1) << D;
        const uint64_t nt = (n + TT - 1) / TT, nblk = (nt + kGivenBlockTiles - 1) / kGivenBlockTiles;
        uint32_t log2T = 0;
        while ((uint64_t(1) << log2T) < TT) ++log2T;
        TileBatchText& x0 = texts[t];
        x0.blk_off = group_blk_off + group_blk * NB;
        x0.nblk0 = uint32_t(nblk);
        x0.nb0 = uint32_t(NB);
        tx[i].blk0 = uint32_t(group_blk);
        for (uint64_t k = 0; k < nblk; ++k) {
          BatchChunk ch{};
          ch.text = t;
          ch.start = k * kGivenBlockTiles * TT;
          ch.len = std::min<uint64_t>(kGivenBlockTiles * TT, n - ch.start);
          ch.cnt_off = group_cnt_off + (group_tile + k * kGivenBlockTiles) * NB;
          ch.blk_off = x0.blk_off + k * NB;
          ch.D = D;
          ch.log2T = log2T;
          b->tchunks.push_back(ch);
        }
        group_tile += nt;
        group_blk += nblk;
      }
    }
    if (given) {
      cnt_total += group_tile * (uint64_t(1) << D);
      blk_total += group_blk * (uint64_t(1) << D);
    }
    CUDA_TRY(cudaMemcpy(d_tx, tx.data(), tx.size() * sizeof(TileText), cudaMemcpyHostToDevice));
    const size_t lb_bytes = (uint64_t(1) << D) * tiles_ub * 8;
    void* lb = b->talloc(lb_bytes);
    b->lookback.push_back({lb, lb_bytes});
    TileArgs a{};
    a.in = p == 0 ? d_texts : (p % 2 == 1 ? b->d_keys_a : b->d_keys_b);
    a.out = out ? (p % 2 == 0 ? b->d_keys_a : b->d_keys_b) : nullptr;
    a.out_size = out ? b->symbols : 0;
    a.segs = g.segs;
    a.texts = d_tx;
    a.tables = g.tables;
    a.lookback = static_cast<unsigned long long*>(lb);
    a.status = ctx->d_status;
    a.nsegs = g.nsegs;
    a.tiles = uint32_t(tiles_ub);
    a.clear_edges = 1;  // levels are not zeroed between builds: shared words are cleared, then set
    a.spin_limit = ctx->spin_limit;
    a.done = b->d_done;
    a.need = b->d_need;
    if (given) {
      a.tiles_per_block = kGivenBlockTiles;
      a.text_blocks = 1;
      given_groups.push_back({args.size(), group_cnt_off, group_blk_off});  // arrays set below
    }
    args.push_back(a);
    groups.push_back(g);
    q.variant[gi] = kv.first.second;
    tiles_all += tiles_ub;
    ++gi;
  }
  // texts whose first pass takes no given prefixes (D = 0), and the rest of
  // the histogram chunks: whole texts in chunks of kBatchChunk symbols
  for (uint32_t t = 0; t < b->count; ++t)
    if (texts[t].nb0 == 0)
      for (uint64_t c0 = 0; c0 < b->info[t].n; c0 += kBatchChunk) {
        BatchChunk ch{};
        ch.text = t;
        ch.start = c0;
        ch.len = std::min<uint64_t>(kBatchChunk, b->info[t].n - c0);
        b->tchunks.push_back(ch);
      }
  b->d_tchunks = static_cast<BatchChunk*>(b->talloc(std::max<size_t>(b->tchunks.size(), 1) * sizeof(BatchChunk)));
  if (!b->tchunks.empty())
    CUDA_TRY(cudaMemcpy(b->d_tchunks, b->tchunks.data(), b->tchunks.size() * sizeof(BatchChunk),
                        cudaMemcpyHostToDevice));
  b->d_tilecnt = static_cast<uint32_t*>(b->talloc(std::max<uint64_t>(cnt_total, 1) * 4));
  b->d_relpre = static_cast<uint32_t*>(b->talloc(std::max<uint64_t>(cnt_total, 1) * 4));
  b->d_blocksum = static_cast<unsigned long long*>(b->talloc(std::max<uint64_t>(blk_total, 1) * 8));
  b->d_blockpre = static_cast<unsigned long long*>(b->talloc(std::max<uint64_t>(blk_total, 1) * 8));
  for (const auto& gg : given_groups) {
    args[gg.arg].tilecnt = b->d_tilecnt + gg.cnt_off;
    args[gg.arg].relpre = b->d_relpre + gg.cnt_off;
    args[gg.arg].blockpre = b->d_blockpre + gg.blk_off;
  }
  b->d_tb_texts = static_cast<TileBatchText*>(b->talloc(std::max<size_t>(texts.size(), 1) * sizeof(TileBatchText)));
  b->d_tb_passes = static_cast<TileBatchPass*>(b->talloc(std::max<size_t>(passes.size(), 1) * sizeof(TileBatchPass)));
  b->d_tb_groups = static_cast<TileBatchGroup*>(b->talloc(std::max<size_t>(groups.size(), 1) * sizeof(TileBatchGroup)));
  b->d_pfx = static_cast<uint64_t*>(b->talloc(std::max<uint64_t>(pfx, 1) * 8));
  auto* d_args = static_cast<TileArgs*>(b->talloc(std::max<size_t>(args.size(), 1) * sizeof(TileArgs)));
  if (!texts.empty())
    CUDA_TRY(cudaMemcpy(b->d_tb_texts, texts.data(), texts.size() * sizeof(TileBatchText), cudaMemcpyHostToDevice));
  if (!passes.empty())
    CUDA_TRY(cudaMemcpy(b->d_tb_passes, passes.data(), passes.size() * sizeof(TileBatchPass), cudaMemcpyHostToDevice));
  if (!groups.empty()) {
    CUDA_TRY(cudaMemcpy(b->d_tb_groups, groups.data(), groups.size() * sizeof(TileBatchGroup), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(d_args, args.data(), args.size() * sizeof(TileArgs), cudaMemcpyHostToDevice));
  }
  q.args = d_args;
  q.group_tiles = b->d_group_tiles;
  q.head = b->d_head;
  q.ngroups = b->ngroups;
  b->queue = q;
  int sms = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int per_sm = std::max(1, tile_batch_ctas_per_sm(b->width));
  b->tile_ctas = uint32_t(std::min<uint64_t>(uint64_t(sms) * per_sm, std::max<uint64_t>(tiles_all, 1)));
  b->tile_text = d_texts;
}

// One whole build on the tile engine, enqueued on the context's stream.
void tile_enqueue(pwmgpu_batch* b, const void* d_texts) {
  pwmgpu_ctx* ctx = b->ctx;
  cudaStream_t s = ctx->stream;
  CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, 4, s));
  CUDA_TRY(cudaMemsetAsync(b->d_hist, 0, std::max<uint64_t>(b->hist_n, 1) * 8, s));
  for (const auto& lb : b->lookback) CUDA_TRY(cudaMemsetAsync(lb.first, 0, lb.second, s));
  CUDA_TRY(cudaMemsetAsync(b->d_done, 0, std::max<uint32_t>(b->ntextpasses, 1) * 4, s));
  CUDA_TRY(cudaMemsetAsync(b->d_head, 0, 4, s));
  launch_batch_hist(d_texts, b->width, b->d_tchunks, uint32_t(b->tchunks.size()), b->d_info, b->d_hist, b->d_tilecnt,
                    b->d_relpre, b->d_blocksum, ctx->d_status, s, &ctx->launches);
  launch_tile_batch_plan(b->d_tb_texts, b->count, b->d_tb_passes, b->ntextpasses, b->d_tb_groups, b->ngroups, b->d_hist,
                         b->d_pfx, b->d_zeros, b->width, b->d_need, b->d_group_tiles, b->d_blocksum, b->d_blockpre, s,
                         &ctx->launches);
  launch_tile_batch(b->width, b->queue, b->tile_ctas, s, &ctx->launches);
  CUDA_TRY(cudaGetLastError());
}

std::unique_ptr<pwmgpu_batch> make_batch(pwmgpu_ctx* ctx, uint32_t count, const uint64_t* begin, const uint64_t* len,
                                         const uint32_t* levels, uint32_t word_width, uint32_t shape_flags, int kmax,
                                         bool tile);

// Tile size of every text: per (key width, levels, log2 length) class the
// fastest of 1, 2 or 4 vectors per thread (4096, 8192 or 16384 bytes of keys
// a tile), measured on up to 64 texts of the class (2^24 symbols at most) the
// first time a context meets the class, and cached in the context.
void tune_tile_sizes(pwmgpu_batch* b, const void* d_texts) {
  pwmgpu_ctx* ctx = b->ctx;
  std::map<uint32_t, std::vector<uint32_t>> cls;
  for (uint32_t t = 0; t < b->count; ++t) cls[tune_key(b->width, b->L[t], b->info[t].n)].push_back(t);
  for (const auto& kv : cls) {
    if (ctx->batch_tune.count(kv.first)) continue;
    // The class's texts, repeated (the same input, separate outputs) until
    // the sub-batch is about as large as a batch that fills the GPU many
    // times over: timed alone, a sub-batch of a few waves of tiles favours
    // small tiles through its tail, which a full batch does not have.
    std::vector<uint64_t> bg, ln;
    std::vector<uint32_t> lv;
    uint64_t sym = 0;
    for (size_t k = 0; bg.size() < kTuneMaxTexts && sym < kTuneSymbols; ++k) {
      const uint32_t t = kv.second[k % kv.second.size()];
      bg.push_back(b->info[t].offset);
      ln.push_back(b->info[t].n);
      lv.push_back(b->L[t]);
      sym += b->info[t].n;
    }
    uint32_t best = 4;
    float best_ms = 0;
    bool valid = true;
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    for (uint32_t v : {4u, 2u, 1u}) {
      auto sub = make_batch(ctx, uint32_t(bg.size()), bg.data(), ln.data(), lv.data(), b->width,
                            b->flags & PWMGPU_TREE ? (PWMGPU_MATRIX | PWMGPU_TREE) : PWMGPU_MATRIX, b->kmax, true);
      sub->force_vpt = v;
      sub->vpt.assign(sub->count, v);
      tile_plan(sub.get(), d_texts);
      tile_enqueue(sub.get(), d_texts);  // warm-up (kernel attributes, caches)
      CUDA_TRY(cudaEventRecord(e0, ctx->stream));
      for (int r = 0; r < 3; ++r) tile_enqueue(sub.get(), d_texts);
      CUDA_TRY(cudaEventRecord(e1, ctx->stream));
      CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0;
      CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
      // A text the build rejects (a symbol >= 2^levels) makes the timing
      // meaningless: keep the default for this batch, cache nothing, and let
      // the build's own run report the status to the caller's check.
      if (read_status(ctx) != 0) {
        valid = false;
        break;
      }
      if (v == 4u || ms < best_ms) {
        best = v;
        best_ms = ms;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (valid) ctx->batch_tune[kv.first] = best;
  }
  for (uint32_t t = 0; t < b->count; ++t) {
    const auto it = ctx->batch_tune.find(tune_key(b->width, b->L[t], b->info[t].n));
    b->vpt[t] = it == ctx->batch_tune.end() ? 4u : it->second;
  }
}

std::unique_ptr<pwmgpu_batch> make_batch(pwmgpu_ctx* ctx, uint32_t count, const uint64_t* begin, const uint64_t* len,
                                         const uint32_t* levels, uint32_t word_width, uint32_t shape_flags, int kmax,
                                         bool tile) {
    if (!valid_width(word_width)) throw Fail{PWMGPU_ERR_ARG, "word_width must be 1, 2 or 4"};
    if (!(shape_flags & PWMGPU_MATRIX)) throw Fail{PWMGPU_ERR_ARG, "a batch builds wavelet matrices (and trees)"};
    auto b = std::make_unique<pwmgpu_batch>();
    b->ctx = ctx;
    b->count = count;
    b->width = word_width;
    b->flags = shape_flags;
    b->kmax = kmax;
    b->tile = tile;
    b->L.assign(levels, levels + count);
    b->vpt.assign(count, 4);
    b->info.resize(count);
    b->wm_off.resize(count);
    b->wt_off.resize(count);
    b->words_per_level.resize(count);
    for (uint32_t t = 0; t < count; ++t) {
      if (b->L[t] == 0 || b->L[t] > kBatchMaxLevels) throw Fail{PWMGPU_ERR_ARG, "batch levels must be in 1..12"};
      const uint64_t n = len[t];
      b->maxL = std::max(b->maxL, b->L[t]);
      BatchText& bt = b->info[t];
      bt.offset = begin[t];
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
    if (!tile) {
      b->d_starts = static_cast<uint64_t*>(b->dalloc(b->starts_n * 8));
      b->d_segs = static_cast<uint64_t*>(b->dalloc(b->segs_n * 8));
    } else {
      // the tile engine never writes padding words: zero once
      CUDA_TRY(cudaMemset(b->d_wm, 0, std::max<uint64_t>(b->wm_words, 1) * 8));
      if (b->d_wt) CUDA_TRY(cudaMemset(b->d_wt, 0, std::max<uint64_t>(b->wt_words, 1) * 8));
    }
    b->d_hist = static_cast<unsigned long long*>(b->dalloc(b->hist_n * 8));
    b->d_keys_a = b->dalloc(b->symbols * word_width);
    b->d_keys_b = b->dalloc(b->symbols * word_width);
    if ((shape_flags & PWMGPU_TREE) && !tile) {
      for (uint32_t t = 0; t < count; ++t) {
        const uint64_t n = len[t];
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
    return b;
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
    if (levels_per_pass < 1 || levels_per_pass > kMaxPassLevels) throw Fail{PWMGPU_ERR_ARG, "levels_per_pass in 1..4"};
    std::vector<uint64_t> begin(count), len(count);
    for (uint32_t t = 0; t < count; ++t) {
      if (offsets[t + 1] < offsets[t]) throw Fail{PWMGPU_ERR_ARG, "offsets must be non-decreasing"};
      begin[t] = offsets[t];
      len[t] = offsets[t + 1] - offsets[t];
    }
    auto b = make_batch(ctx, count, begin.data(), len.data(), levels, word_width, shape_flags, levels_per_pass,
                        ctx->engine == PWMGPU_ENGINE_TILE);
    b->offs.assign(offsets, offsets + count + 1);
    *out = b.release();
    return PWMGPU_OK;
  });
}

pwmgpu_status pwmgpu_batch_build(pwmgpu_ctx* ctx, pwmgpu_batch* b, const void* d_texts) {
  if (!ctx || !b || (!d_texts && b->symbols)) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    const bool replan = b->tile ? (b->tile_text != d_texts) : (b->graph_k != b->kmax);
    if (!b->exec || b->graph_text != d_texts || replan) {
      b->drop_graph();
      if (b->tile) {
        if (b->force_vpt) b->vpt.assign(b->count, b->force_vpt);
        else tune_tile_sizes(b, d_texts);
        tile_plan(b, d_texts);
      } else if (b->groups_k != b->kmax || b->groups.empty() || b->graph_text != d_texts) {
        batch_plan(b, d_texts);
      }
      auto enqueue = [&]() {
        if (b->tile) tile_enqueue(b, d_texts);
        else batch_enqueue(b, d_texts);
      };
      // run once eagerly (configures kernel attributes), then capture the graph
      enqueue();
      CUDA_TRY(cudaStreamSynchronize(ctx->stream));
      CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      try {
        enqueue();
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

pwmgpu_status pwmgpu_batch_set_tile_vectors(pwmgpu_batch* b, uint32_t vectors_per_thread) {
  if (!b || !(vectors_per_thread == 0 || vectors_per_thread == 1 || vectors_per_thread == 2 ||
              vectors_per_thread == 4))
    return PWMGPU_ERR_ARG;
  if (b->force_vpt != vectors_per_thread) {
    b->force_vpt = vectors_per_thread;
    b->tile_text = nullptr;  // replan at the next build
  }
  return PWMGPU_OK;
}

pwmgpu_status pwmgpu_batch_tile_vectors(const pwmgpu_batch* b, uint32_t index, uint32_t* vectors_per_thread) {
  if (!b || index >= b->count || !vectors_per_thread) return PWMGPU_ERR_ARG;
  *vectors_per_thread = b->tile ? b->vpt[index] : 0;
  return PWMGPU_OK;
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
