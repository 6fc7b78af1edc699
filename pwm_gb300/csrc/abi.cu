// C ABI of the engine (include/pwmgpu.h): contexts, device-resident
// structures, the drop-in host-to-host constructions, the Huffman code
// builder, queries and alphabet reduction.  The build work itself lives in
// plain.cu, huffman.cu and shards.cu; batches and generators in
// batch_host.cu.
#include <cstring>
#include "engine.hpp"

using namespace pwmgpu;

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

pwmgpu_status pwmgpu_ctx_set_host_copy_threads(pwmgpu_ctx* ctx, int threads) {
  if (!ctx || threads < -1 || threads > 256) return PWMGPU_ERR_ARG;
  return guarded(ctx, [&]() {
    if (threads != ctx->host_copy_threads) ctx->copy_pool.reset();
    ctx->host_copy_threads = threads;
    return PWMGPU_OK;
  });
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
    device_to_host(ctx, bv, s.d_words, s.total_words * 8, ctx->stream);
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

pwmgpu_status pwmgpu_wx_query_batch_host(pwmgpu_ctx* ctx, const pwmgpu_wx* wx, int which, const uint8_t* ops,
                                         const uint64_t* a, const uint64_t* b, uint64_t count, uint64_t* out) {
  if (!ctx || !wx || (count && (!ops || !a || !out))) return PWMGPU_ERR_ARG;
  if (count == 0) return PWMGPU_OK;
  for (uint64_t i = 0; i < count; ++i)
    if (ops[i] > PWMGPU_Q_SELECT || (ops[i] != PWMGPU_Q_ACCESS && !b)) return PWMGPU_ERR_ARG;
  const Structure& s = which ? wx->wt : wx->wm;
  if (!s.present || !s.rs || (which == 0 && wx->wm_internal))
    return fail(ctx, PWMGPU_ERR_ARG, "queries need a structure with rank/select");
  if (s.huffman) return fail(ctx, PWMGPU_ERR_ARG, "mixed query batches need a plain structure");
  return guarded(ctx, [&]() {
    // a, b and the kinds staged in pinned memory and uploaded in one copy;
    // on the device the answers follow them (8-byte aligned)
    const uint64_t in_bytes = count * 16 + count, out_off = count * 2 + (count + 7) / 8;
    auto* h = static_cast<unsigned char*>(ctx->grow_pinned_named("query_io", std::max(in_bytes, count * 8)));
    std::memcpy(h, a, count * 8);
    if (b) std::memcpy(h + count * 8, b, count * 8);
    else std::memset(h + count * 8, 0, count * 8);
    std::memcpy(h + count * 16, ops, count);
    auto* d = static_cast<uint64_t*>(ctx->grow("query_io", (out_off + count) * 8));
    cudaStream_t st = ctx->stream;
    CUDA_TRY(cudaMemcpyAsync(d, h, in_bytes, cudaMemcpyHostToDevice, st));
    QueryStructure q{s.levels, s.is_tree ? 1u : 0u, s.n, s.d_q_levels, s.d_zeros};
    {
      ProfScope ps(ctx, "queries", count * 25);
      launch_queries(q, 0, d, d + count, count, d + out_off, st, &ctx->launches,
                     reinterpret_cast<const uint8_t*>(d + 2 * count));
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(h, d + out_off, count * 8, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    std::memcpy(out, h, count * 8);
    return PWMGPU_OK;
  });
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
    host_to_device(ctx, d_text, text, size * word_width, ctx->stream);
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
    host_to_device(ctx, d_text, text, size * word_width, ctx->stream);
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
    device_to_host(ctx, bv, s.d_words, s.total_words * 8, ctx->stream);
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


}  // extern "C"
