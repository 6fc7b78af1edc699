// Launchers of the segmented tile pass (tile.cuh) for 1-, 2- and 4-byte keys.
#include "kernels.cuh"
#include "tile_launch.cuh"

namespace pwmgpu {

namespace {

template <typename KeyT, bool OUT>
void launch_k(int K, const TileArgs& a, cudaStream_t s) {
  switch (K) {
    case 1: launch_tile_one<KeyT, 1, OUT>(a, s); break;
    case 2: launch_tile_one<KeyT, 2, OUT>(a, s); break;
    case 3: launch_tile_one<KeyT, 3, OUT>(a, s); break;
    default: launch_tile_one<KeyT, 4, OUT>(a, s); break;
  }
}

template <typename KeyT>
void launch_key(int K, bool out, const TileArgs& a, cudaStream_t s) {
  if (out) launch_k<KeyT, true>(K, a, s);
  else launch_k<KeyT, false>(K, a, s);
}

}  // namespace

uint32_t tile_pass_elems(uint32_t key_bytes) {
  return uint32_t(kTileThreads * kTileVectors * (16 / key_bytes));
}

void launch_tile_pass(uint32_t key_bytes, int K, bool out, const TileArgs& a, cudaStream_t s, uint64_t* launches) {
  if (a.launch_tiles == 0) return;
  if (K > kTileMaxLevels) {
    // only as the last pass of a text whose prefixes the histogram gives
    if (out || !a.blockpre || K > kTileGivenMaxLevels) return;
    launch_tile_pass_deep(key_bytes, K, a, s);
  } else if (key_bytes == 1) launch_key<uint8_t>(K, out, a, s);
  else if (key_bytes == 2) launch_key<uint16_t>(K, out, a, s);
  else launch_key<uint32_t>(K, out, a, s);
  ++*launches;
}

}  // namespace pwmgpu
