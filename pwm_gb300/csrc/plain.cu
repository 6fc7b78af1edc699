// Plain builds: the segmented tile passes (tile.cuh) planned on the host from
// the device's prefix counts, the warp-pass engine for deeper texts, and the
// host ends of host-to-host builds (pieces uploaded as the histogram follows,
// finished words streamed back while later passes run).
#include "engine.hpp"

using namespace pwmgpu;

namespace {

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

// Key width of S_l for the pass starting at level l of an L-level text of
// `width`-byte symbols: the text itself at l = 0; later the narrowest width
// that holds the L - l bits the remaining levels split on (a pass writes
// only the low bits of its keys), never wider than the text.
uint32_t tile_pass_key_bytes(uint32_t width, uint32_t L, uint32_t l) {
  return l == 0 ? width : std::min(width, tile_key_bytes(L - l));
}

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
  const uint32_t in_bytes = tile_pass_key_bytes(width, wm.levels, pi == 0 ? 0u : p.level);
  const uint32_t out_bytes = tile_pass_key_bytes(width, wm.levels, p.level + uint32_t(p.K));
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
      launch_tile_pass(in_bytes, out_bytes, p.K, p.out, a, s, &ctx->launches);
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
                     const uint64_t* d_segs, const LevelTables& tabs, Structure& wm, Structure* wt,
                     const TileFirstPass* first = nullptr,
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

  if (wt && !regroup.empty()) {  // d_segs: every group of each level (launch_regroup_segs)
    if (!d_segs) throw Fail{PWMGPU_ERR_CUDA, "internal: the regroup has no segments"};
    for (uint32_t i = 0; i < uint32_t(regroup.size()); ++i) {
      const uint32_t m = regroup[i];
      const uint64_t ns = uint64_t(1) << m;
      const uint64_t* seg = d_segs + regroup_segs_offset(regroup.data(), i);
      ProfScope ps(ctx, "regroup", 2 * words_for(wm.bits[m]) * 8);
      launch_regroup(wm.d_words + wm.offs[m], wt->d_words + wt->offs[m], wm.bits[m], seg, seg + ns, ns,
                     ctx->d_status, s, &ctx->launches);
    }
    CUDA_TRY(cudaGetLastError());
  }
  if (after_pass) after_pass(passes.size());
  // (copies from pageable host vectors return once the data is staged, so
  // the plan may go out of scope with the passes still running)
}

}  // namespace

namespace pwmgpu {

void validate_plain(uint64_t n, uint32_t width, uint32_t levels, bool allow40) {
  if (!(allow40 ? valid_plain_width(width) : valid_width(width)))
    throw Fail{PWMGPU_ERR_ARG, allow40 ? "word_width must be 1, 2, 4 or 5" : "word_width must be 1, 2 or 4"};
  if (levels == 0 || levels > kMaxPlainLevels)
    throw Fail{PWMGPU_ERR_ARG, "levels must be in 1..24 (the leaf histogram has 2^levels bins)"};
  if (n >= (uint64_t(1) << 62)) throw Fail{PWMGPU_ERR_ARG, "size too large"};
}

// Plain build of a wx from a device text (with `io`: from a host text, into
// host arrays; d_text is then the device copy to fill).
void build_plain(pwmgpu_ctx* ctx, pwmgpu_wx* wx, const void* d_text, const HostIO* io) {
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
  if (io && io->text && !pinned_in) host_to_device(ctx, const_cast<void*>(d_text), io->text, n * wx->width, s);
  CUDA_TRY(cudaMemsetAsync(ctx->d_status, 0, 4, s));
  const uint64_t bins = uint64_t(1) << L;
  // Tile engine: level 0 is written in whole words (by the histogram kernel,
  // or by the first pass, whose tiles start at multiples of 64 bits); the
  // first pass's other levels are zeroed by the histogram kernel (levels <= 8)
  // or here; the padding is zero from allocation.
  // Deeper than the tile planner's folded prefix counts reach: the tile
  // engine still builds a matrix alone from every pass's digit counts
  // (digit_plan below), the warp-pass engine the rest.
  const bool tile_engine =
      ctx->engine == PWMGPU_ENGINE_TILE &&
      (L <= kTilePlanMaxLevels || (!wx->wt.present && !wx->keep_hist && !stream_out));
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
  const bool want_tree = wx->wt.present;
  // Matrix-only, more than 8 levels, no host streaming: the passes need only
  // the counts of their own digits, not a leaf histogram of 2^L bins
  // (plan_matrix_passes).
  const bool digit_plan = tile_engine && !want_tree && L > 8 && !wx->keep_hist && !stream_out;
  // A tree of more than 8 levels: the device also sums every pass's digit
  // counts from the prefix counts (the planner's matrix-only passes would
  // otherwise sum up to 2^L counts on the host: ~0.5 ms at 20 levels).
  const bool tree_digits = tile_engine && want_tree && !digit_plan && L > 8;
  const auto digit_shape = digit_plan || tree_digits ? plan_passes(L, kmax) : std::vector<PassPlan>{};
  auto* d_hist = digit_plan ? nullptr : static_cast<unsigned long long*>(ctx->grow("hist", bins * 8));
  if (!digit_plan) CUDA_TRY(cudaMemsetAsync(d_hist, 0, bins * 8, s));
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
  // (with digit_plan: the prefix counts of levels 0..Kz only, then the
  // zero bits, the status word and every pass's digit counts)
  const uint64_t NB0 = uint64_t(1) << D0;
  const uint64_t flat_words = digit_plan ? (uint64_t(2) << Kz) - 1 : (bins << 1) - 1;
  uint64_t* h_flat = ctx->grow_mapped((flat_words + L + 1 + 16 * digit_shape.size() + 1) * 8);
  uint64_t* d_flat_host = ctx->mapped_dev;
  uint64_t* h_hist = digit_plan ? nullptr : h_flat + bins - 1;
  const uint64_t* h_zeros = h_flat + flat_words;
  auto* h_status = reinterpret_cast<uint32_t*>(h_flat + flat_words + L);
  const uint64_t* h_digits = h_flat + flat_words + L + 1;
  auto* d_level_zeros = static_cast<unsigned long long*>(ctx->grow("level_zeros", uint64_t(L) * 8));
  // a tree's prefix counts also in device memory: the regroup's segments
  // (every group of a level, in both orders) are derived from them there
  bool tree_digits_ok = false;  // h_digits holds every pass's digit counts of a tree
  uint64_t* d_flat = tile_engine && want_tree && !digit_plan
                         ? static_cast<uint64_t*>(ctx->grow("flat_dev", flat_words * 8))
                         : nullptr;
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
  } else if (digit_plan) {
    if (pinned_in) CUDA_TRY(cudaMemcpyAsync(const_cast<void*>(d_text), io->text, n * wx->width,
                                            cudaMemcpyHostToDevice, s));
    PassDigitsArgs pd{};
    pd.npasses = uint32_t(digit_shape.size());
    pd.L = L;
    for (uint32_t p = 0; p < pd.npasses; ++p) {
      pd.level[p] = digit_shape[p].level;
      pd.K[p] = uint32_t(digit_shape[p].K);
      pd.lo[p] = L - digit_shape[p].level - pd.K[p];
      pd.mask[p] = (1u << pd.K[p]) - 1u;
    }
    auto* d_digits = static_cast<unsigned long long*>(ctx->grow("pass_digits", (16 * kPassDigitsMaxPasses + 2) * 8));
    CUDA_TRY(cudaMemsetAsync(d_digits, 0, (16 * pd.npasses + 2) * 8, s));
    ProfScope ps(ctx, "leaf_histogram", n * wx->width);
    launch_pass_digits(d_text, n, wx->width, pd, d_digits, reinterpret_cast<unsigned int*>(d_digits + 16 * pd.npasses),
                       ctx->d_status, d_flat_host, s, &ctx->launches);
  } else {
    if (pinned_in) CUDA_TRY(cudaMemcpyAsync(const_cast<void*>(d_text), io->text, n * wx->width,
                                            cudaMemcpyHostToDevice, s));
    ProfScope ps(ctx, "leaf_histogram", n * wx->width);
    launch_leaf_histogram(d_text, n, wx->width, L, d_hist, ctx->d_status, s, &ctx->launches);
  }
  CUDA_TRY(cudaGetLastError());
  if (!digit_plan) {
    // prefix counts, zero bits and the status word to the host
    CUDA_TRY(cudaMemsetAsync(d_level_zeros, 0, uint64_t(L) * 8, s));
    launch_fold_levels(d_hist, L, d_flat_host, d_level_zeros, s, &ctx->launches, d_flat);
    launch_readback(d_level_zeros, L, ctx->d_status, d_flat_host + flat_words, s, &ctx->launches);
    if (tree_digits) {
      std::vector<uint32_t> lv, kk;
      for (const auto& ps : digit_shape) {
        lv.push_back(ps.level);
        kk.push_back(uint32_t(ps.K));
      }
      const uint64_t nd = 16 * lv.size();
      auto* d_dg = static_cast<unsigned long long*>(ctx->grow("tree_digits", nd * 8));
      tree_digits_ok = launch_flat_digits(d_flat, L, lv.data(), kk.data(), uint32_t(lv.size()), d_dg, s,
                                          &ctx->launches);
      if (tree_digits_ok)
        launch_readback(d_dg, nd, ctx->d_status, d_flat_host + flat_words + L + 1, s, &ctx->launches);
    }
  }
  CUDA_TRY(cudaEventRecord(ctx->hist_event(), s));
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
  } else if (tile_engine && !stream_out && L > 8 && Kz < int(L)) {
    // Deeper texts: the first pass counts its tiles and looks back (the tile
    // histogram covers at most 8 levels), but its start table still follows
    // from the device's prefix counts of levels 0..Kz, so it starts before
    // the host reads them and plans the later passes (which took the GPU
    // idle for ~1.3 ms at 16 levels, 2^28 symbols).  The memset above zeroed
    // its levels 1..Kz-1.
    const auto shape = plan_passes(L, Kz);
    std::vector<TilePassHost> early(2);
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
    launch_tile_first_table(d_flat_host, uint32_t(p0.K), p0.out, want_tree,
                            reinterpret_cast<uint64_t*>(d_b0 + b0.table[0]), s, &ctx->launches);
    // the look-back state sized for every later pass now (a later pass has at
    // most 2^16 segments, each adding at most one partial tile), so that no
    // later pass reallocates it, which would wait for this one
    ctx->grow("lookback", (uint64_t(p0.tiles) + 65536 + 16) * (uint64_t(1) << kTileMaxLevels) * 8 + 64);
    next_in = enqueue_tile_pass(ctx, early, 0, d_b0, b0, d_text, wx->width, n, wx->wm, want_tree ? &wx->wt : nullptr,
                                nullptr);
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
  uint64_t* d_segs = nullptr;  // the regroup's segments (device)
  PrefixCounts cnt;  // natural-prefix counts per level
  const uint32_t w = wx->width;
  auto tile_keys = [&](uint32_t l) { return tile_pass_elems(tile_pass_key_bytes(w, L, l)); };
  if (digit_plan) {
    tile_passes = plan_matrix_passes(h_digits, n, L, kmax, tile_keys);
    tabs.level_bits.assign(L, n);
    tabs.zeros.assign(h_zeros, h_zeros + L);
    tabs.seg_tree.resize(L);
    tabs.seg_matrix.resize(L);
  } else if (tile_engine) {
    cnt = PrefixCounts::view(h_flat, L);
    tile_passes = plan_tile_passes(cnt, L, kmax, tile_keys, want_tree, &regroup, tree_digits_ok ? h_digits : nullptr);
    tabs = build_tables_tile(cnt, L, {}, h_zeros);
    if (want_tree && !regroup.empty()) {
      const auto nr = uint32_t(regroup.size());
      const uint64_t words = regroup_segs_words(regroup.data(), nr);
      d_segs = static_cast<uint64_t*>(
          ctx->grow("regroup_segs", (words + regroup_segs_scratch_words(regroup.data(), nr)) * 8));
      if (!d_flat || !launch_regroup_segs(d_flat, regroup.data(), nr, d_segs, d_segs + words, s, &ctx->launches))
        throw Fail{PWMGPU_ERR_CUDA, "internal: regroup segments"};
    }
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
    run_tile_passes(ctx, next_in, wx->width, L, tile_passes, regroup, d_segs, tabs, wx->wm, want_tree ? &wx->wt : nullptr,
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
      else device_to_host(ctx, host_out[st], S.d_words, S.total_words * 8, s);
    }
    if (stream_out) CUDA_TRY(cudaStreamSynchronize(ctx->down));
    CUDA_TRY(cudaStreamSynchronize(s));
  }
}

}  // namespace pwmgpu
