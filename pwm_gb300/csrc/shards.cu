// Structures built from shards: semi-external construction of host texts
// larger than the device memory, the merge of independently built slices
// (pwm's wx_dd_*), 40-bit inputs, and alphabet reduction of wide symbols.
#include "engine.hpp"

using namespace pwmgpu;

namespace pwmgpu {

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
  host_to_device(ctx, d40, host_text, wx->n * 5, ctx->stream);
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

}  // namespace pwmgpu
