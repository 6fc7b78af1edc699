// Copies between pageable host memory and the device through a ring of
// pinned staging pieces: the context's host threads fill (or drain) one piece
// while the copy engine moves the one before, so a host-to-host build pays
// the larger of the two rates instead of the driver's single-threaded staging
// of pageable memory.  Pinned host memory goes straight to cudaMemcpyAsync.
#include <thread>

#include "engine.hpp"

namespace pwmgpu {

namespace {

unsigned copy_threads(const pwmgpu_ctx* ctx) {
  if (ctx->host_copy_threads >= 0) return unsigned(ctx->host_copy_threads);
  const unsigned hw = std::thread::hardware_concurrency();
  return std::max(1u, std::min(kStageAutoThreads, hw ? hw : 1u));
}

char* stage_ring(pwmgpu_ctx* ctx, unsigned threads) {
  if (!ctx->copy_pool || ctx->copy_pool->requested() != threads) {
    ctx->copy_pool.reset();
    ctx->copy_pool = std::make_unique<CopyPool>(threads);
  }
  if (!ctx->stage) {
    CUDA_TRY(cudaMallocHost(&ctx->stage, kStagePiece * kStagePieces));
    for (auto& e : ctx->stage_ev) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  return static_cast<char*>(ctx->stage);
}

}  // namespace

bool host_pinned(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

void host_to_device(pwmgpu_ctx* ctx, void* d_dst, const void* h_src, uint64_t bytes, cudaStream_t s) {
  if (!bytes) return;
  const unsigned threads = copy_threads(ctx);
  if (threads == 0 || bytes < kStagePiece || host_pinned(h_src)) {
    CUDA_TRY(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, s));
    return;
  }
  char* ring = stage_ring(ctx, threads);
  const char* src = static_cast<const char*>(h_src);
  char* dst = static_cast<char*>(d_dst);
  for (uint64_t off = 0, i = 0; off < bytes; off += kStagePiece, ++i) {
    const unsigned b = unsigned(i % kStagePieces);
    const uint64_t len = std::min(kStagePiece, bytes - off);
    CUDA_TRY(cudaEventSynchronize(ctx->stage_ev[b]));  // the piece's previous copy is done
    ctx->copy_pool->copy(ring + b * kStagePiece, src + off, len);
    CUDA_TRY(cudaMemcpyAsync(dst + off, ring + b * kStagePiece, len, cudaMemcpyHostToDevice, s));
    CUDA_TRY(cudaEventRecord(ctx->stage_ev[b], s));
  }
}

void device_to_host(pwmgpu_ctx* ctx, void* h_dst, const void* d_src, uint64_t bytes, cudaStream_t s) {
  const unsigned threads = copy_threads(ctx);
  if (bytes && !(threads == 0 || bytes < kStagePiece || host_pinned(h_dst))) {
    char* ring = stage_ring(ctx, threads);
    const char* src = static_cast<const char*>(d_src);
    char* dst = static_cast<char*>(h_dst);
    const uint64_t pieces = (bytes + kStagePiece - 1) / kStagePiece;
    auto issue = [&](uint64_t i) {
      const unsigned b = unsigned(i % kStagePieces);
      const uint64_t off = i * kStagePiece;
      CUDA_TRY(cudaStreamWaitEvent(s, ctx->stage_ev[b], 0));  // a copy out of the piece on another stream
      CUDA_TRY(cudaMemcpyAsync(ring + b * kStagePiece, src + off, std::min(kStagePiece, bytes - off),
                               cudaMemcpyDeviceToHost, s));
      CUDA_TRY(cudaEventRecord(ctx->stage_ev[b], s));
    };
    for (uint64_t i = 0; i < std::min<uint64_t>(pieces, kStagePieces); ++i) issue(i);
    for (uint64_t i = 0; i < pieces; ++i) {
      const unsigned b = unsigned(i % kStagePieces);
      const uint64_t off = i * kStagePiece;
      CUDA_TRY(cudaEventSynchronize(ctx->stage_ev[b]));
      ctx->copy_pool->copy(dst + off, ring + b * kStagePiece, std::min(kStagePiece, bytes - off));
      if (i + kStagePieces < pieces) issue(i + kStagePieces);
    }
    return;
  }
  if (bytes) CUDA_TRY(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
}

void release_staging(pwmgpu_ctx* ctx) {
  ctx->copy_pool.reset();
  if (ctx->stage) {
    for (auto e : ctx->stage_ev) cudaEventSynchronize(e);
    cudaFreeHost(ctx->stage);
    ctx->stage = nullptr;
  }
  for (auto& e : ctx->stage_ev)
    if (e) {
      cudaEventDestroy(e);
      e = nullptr;
    }
}

}  // namespace pwmgpu
