// Huffman-shaped builds: the code table from the device's symbol histogram
// (pwm's builder restated on the host) and the warp-pass engine on packed
// code keys.
#include "engine.hpp"

using namespace pwmgpu;

namespace pwmgpu {


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
  // keys: the code and a stop bit, levels + 1 bits (split.cuh HuffKeys)
  const uint32_t key_bytes = huff_key_bytes(levels + 1);
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
  launch_huffman_keys(d_text, n, width, d_len, d_word, ncodes, levels, key_bytes, keys, ctx->d_status, s,
                      &ctx->launches);
  run_passes(ctx, keys, key_bytes, width, true, levels, plan, tabs, wm, wt);
  check_device_status(ctx);
  build_rank_select(ctx, !is_tree ? &wm : nullptr, wt);
}

}  // namespace pwmgpu
