// Launch of one tile-pass instantiation (shared by tile.cu and tile_deep.cu,
// which instantiate the pass widths in separate translation units so that
// they compile in parallel).
#pragma once
#include "tile.cuh"

namespace pwmgpu {

constexpr int kTileThreads = 256;
constexpr int kTileVectors = 4;  // 16-byte vectors per thread: 64 bytes of keys

template <typename KeyT, int K, bool OUT, typename KeyO = KeyT>
void launch_tile_one(const TileArgs& a, cudaStream_t s) {
  using C = TileCfg<KeyT, K, OUT, kTileThreads, kTileVectors>;
  auto kern = tile_pass_kernel<KeyT, K, OUT, kTileThreads, kTileVectors, KeyO>;
  static bool configured = false;  // attribute set once per instantiation
  if (!configured) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(C::smem_bytes()));
    configured = true;
  }
  kern<<<a.launch_tiles, kTileThreads, C::smem_bytes(), s>>>(a);
}

// Last passes of 5..8 levels with given prefixes (tile_deep.cu).
void launch_tile_pass_deep(uint32_t key_bytes, int K, const TileArgs& a, cudaStream_t s);

}  // namespace pwmgpu
