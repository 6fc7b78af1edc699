// Launch of one tile-pass instantiation (shared by tile.cu and tile_deep.cu,
// which instantiate the pass widths in separate translation units so that
// they compile in parallel).
#pragma once
#include "tile.cuh"

namespace pwmgpu {

constexpr int kTileThreads = 256;
constexpr int kTileVectors = 4;  // 16-byte vectors per thread: 64 bytes of keys

// PLANES: the bit-plane form of a pass without S_{l+K} over 1-byte keys.
template <typename KeyT, int K, bool OUT, typename KeyO = KeyT, bool PLANES = false>
void launch_tile_one(const TileArgs& a, cudaStream_t s) {
  using C = TileCfg<KeyT, K, OUT, kTileThreads, kTileVectors>;
  auto kern = tile_pass_kernel<KeyT, K, OUT, kTileThreads, kTileVectors, KeyO, PLANES>;
  constexpr size_t smem = PLANES ? C::plane_smem_bytes() : C::smem_bytes();
  static bool configured = false;  // attribute set once per instantiation
  if (!configured) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    configured = true;
  }
  kern<<<a.launch_tiles, kTileThreads, smem, s>>>(a);
}

// Last passes of 5..8 levels with given prefixes (tile_deep.cu).
void launch_tile_pass_deep(uint32_t key_bytes, int K, const TileArgs& a, cudaStream_t s);

}  // namespace pwmgpu
