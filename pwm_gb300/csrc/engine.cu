// Contexts' teardown, structures and their rank/select storage, device status,
// and the warp-pass matrix passes shared by plain and Huffman builds.
#include "engine.hpp"

using namespace pwmgpu;

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
  release_staging(this);
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

namespace pwmgpu {

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
                     bool rank_select, cudaStream_t alloc_stream) {
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
void build_rank_select(pwmgpu_ctx* ctx, Structure* wm, Structure* wt, bool share_level0, uint32_t lo, uint32_t hi,
                       cudaStream_t stream, const char* tag) {
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
  // Huffman keys narrow as the passes go: the pass from level l reads keys
  // of the L - l + 1 low bits (its levels, the later ones, the stop bit)
  auto in_bytes = [&](uint32_t l) {
    return (huff && l > 0) ? std::min(key_bytes, huff_key_bytes(L - l + 1)) : key_bytes;
  };
  void* ping = ctx->grow("keys_a", std::max<uint64_t>(n0, 1) * key_bytes);
  void* pong = ctx->grow("keys_b", std::max<uint64_t>(n0, 1) * key_bytes);
  const void* in = keys;
  size_t start_off = 0;
  for (size_t pi = 0; pi < plan.size(); ++pi) {
    const auto& p = plan[pi];
    const uint64_t m = tabs.level_bits[p.level];
    const uint32_t kb = in_bytes(p.level), kbo = in_bytes(p.level + uint32_t(p.K));
    const uint32_t T = split_tile_elems(kb);
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
      launch_split_pass(kb, kbo, huff, p.K, a, L, s, &ctx->launches);
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

}  // namespace pwmgpu
