// Instantiations and launcher of the fused split pass (split.cuh).
#include "kernels.cuh"

namespace pwmgpu {

namespace {

constexpr int kSplitThreads = 256;

template <int KB>
struct SplitGeometry;
template <> struct SplitGeometry<1> { static constexpr int ITEMS = 64; using Key = uint8_t; };
template <> struct SplitGeometry<2> { static constexpr int ITEMS = 64; using Key = uint16_t; };
template <> struct SplitGeometry<4> { static constexpr int ITEMS = 32; using Key = uint32_t; };
template <> struct SplitGeometry<8> { static constexpr int ITEMS = 16; using Key = uint64_t; };

template <int KB, bool HUFF, int K, int KBO = KB>
void launch_one(const SplitArgs& a, uint32_t L, cudaStream_t s) {
  using G = SplitGeometry<KB>;
  using Key = typename G::Key;
  using KeyO = typename SplitGeometry<KBO>::Key;
  using Tr = typename std::conditional<HUFF, HuffKeys<Key>, PlainKeys<Key>>::type;
  using P = SplitPass<Key, Tr, K, kSplitThreads, G::ITEMS>;
  auto kern = split_pass_kernel<Key, Tr, K, kSplitThreads, G::ITEMS, KeyO>;
  static bool configured = false;  // one attribute call per instantiation and process
  const size_t smem = P::smem_bytes();
  if (!configured) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    configured = true;
  }
  Tr tr{L};
  kern<<<a.tiles, kSplitThreads, smem, s>>>(a, tr);
}

template <int KB, bool HUFF, int K>
void launch_batched_one(const SplitArgs* args, const uint32_t* tile_base, uint32_t ntexts, uint32_t tiles,
                        uint32_t* counter, cudaStream_t s) {
  using G = SplitGeometry<KB>;
  using Key = typename G::Key;
  using Tr = typename std::conditional<HUFF, HuffKeys<Key>, PlainKeys<Key>>::type;
  using P = SplitPass<Key, Tr, K, kSplitThreads, G::ITEMS>;
  auto kern = split_pass_batched_kernel<Key, Tr, K, kSplitThreads, G::ITEMS>;
  static bool configured = false;
  const size_t smem = P::smem_bytes();
  if (!configured) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    configured = true;
  }
  kern<<<tiles, kSplitThreads, smem, s>>>(args, tile_base, ntexts, counter);
}

template <int KB, bool HUFF, int KBO = KB>
void launch_k(int K, const SplitArgs& a, uint32_t L, cudaStream_t s) {
  switch (K) {
    case 1: launch_one<KB, HUFF, 1, KBO>(a, L, s); break;
    case 2: launch_one<KB, HUFF, 2, KBO>(a, L, s); break;
    case 3: launch_one<KB, HUFF, 3, KBO>(a, L, s); break;
    default: launch_one<KB, HUFF, 4, KBO>(a, L, s); break;
  }
}

}  // namespace

void launch_split_pass_batched(uint32_t key_bytes, int K, const SplitArgs* args, const uint32_t* tile_base,
                               uint32_t ntexts, uint32_t tiles, uint32_t* counter, cudaStream_t s,
                               uint64_t* launches) {
  if (tiles == 0) return;
#define PWMGPU_BK(KB)                                                                              \
  switch (K) {                                                                                     \
    case 1: launch_batched_one<KB, false, 1>(args, tile_base, ntexts, tiles, counter, s); break;   \
    case 2: launch_batched_one<KB, false, 2>(args, tile_base, ntexts, tiles, counter, s); break;   \
    case 3: launch_batched_one<KB, false, 3>(args, tile_base, ntexts, tiles, counter, s); break;   \
    default: launch_batched_one<KB, false, 4>(args, tile_base, ntexts, tiles, counter, s); break;  \
  }
  switch (key_bytes) {
    case 1: PWMGPU_BK(1) break;
    case 2: PWMGPU_BK(2) break;
    default: PWMGPU_BK(4) break;
  }
#undef PWMGPU_BK
  ++*launches;
}

uint32_t split_tile_elems(uint32_t key_bytes) {
  switch (key_bytes) {
    case 1: return kSplitThreads * SplitGeometry<1>::ITEMS;
    case 2: return kSplitThreads * SplitGeometry<2>::ITEMS;
    case 4: return kSplitThreads * SplitGeometry<4>::ITEMS;
    default: return kSplitThreads * SplitGeometry<8>::ITEMS;
  }
}

size_t split_smem_bytes(uint32_t key_bytes, int K) {
  const size_t T = split_tile_elems(key_bytes);
  return 2 * T * key_bytes + size_t(K > 1 ? K - 1 : 1) * (T / 32 + 1) * 4;
}

void launch_split_pass(uint32_t key_bytes, uint32_t out_bytes, bool huffman, int K, const SplitArgs& a, uint32_t L,
                       cudaStream_t s, uint64_t* launches) {
  if (a.tiles == 0) return;
  if (huffman) {
    // a pass without S_{l+K} has no output keys: the input width alone
    const uint32_t o = a.out ? std::min(out_bytes, key_bytes) : key_bytes;
    if (key_bytes == 8) {
      if (o == 8) launch_k<8, true>(K, a, L, s); else launch_k<8, true, 4>(K, a, L, s);
    } else if (key_bytes == 4) {
      if (o == 4) launch_k<4, true>(K, a, L, s);
      else if (o == 2) launch_k<4, true, 2>(K, a, L, s);
      else launch_k<4, true, 1>(K, a, L, s);
    } else if (key_bytes == 2) {
      if (o == 2) launch_k<2, true>(K, a, L, s); else launch_k<2, true, 1>(K, a, L, s);
    } else {
      launch_k<1, true>(K, a, L, s);
    }
  } else {
    switch (key_bytes) {
      case 1: launch_k<1, false>(K, a, L, s); break;
      case 2: launch_k<2, false>(K, a, L, s); break;
      default: launch_k<4, false>(K, a, L, s); break;
    }
  }
  ++*launches;
}

}  // namespace pwmgpu
