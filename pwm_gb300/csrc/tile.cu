// Launchers of the segmented tile pass (tile.cuh) for 1-, 2- and 4-byte keys.
#include "kernels.cuh"
#include "tile_launch.cuh"

namespace pwmgpu {

namespace {

template <typename KeyT, bool OUT, typename KeyO = KeyT, bool PLANES = false>
void launch_k(int K, const TileArgs& a, cudaStream_t s) {
  switch (K) {
    case 1: launch_tile_one<KeyT, 1, OUT, KeyO, PLANES>(a, s); break;
    case 2: launch_tile_one<KeyT, 2, OUT, KeyO, PLANES>(a, s); break;
    case 3: launch_tile_one<KeyT, 3, OUT, KeyO, PLANES>(a, s); break;
    default: launch_tile_one<KeyT, 4, OUT, KeyO, PLANES>(a, s); break;
  }
}

// A pass writing S_{l+K} in keys of out_bytes (<= the input's key width).  A
// pass over 1-byte keys without S_{l+K} moves bit planes.
template <typename KeyT>
void launch_key(int K, bool out, uint32_t out_bytes, const TileArgs& a, cudaStream_t s) {
  if (!out) {
    if constexpr (sizeof(KeyT) == 1) launch_k<KeyT, false, KeyT, true>(K, a, s);
    else launch_k<KeyT, false>(K, a, s);
  }
  else if (out_bytes >= sizeof(KeyT)) launch_k<KeyT, true>(K, a, s);
  else if constexpr (sizeof(KeyT) >= 2) {
    if (out_bytes == 1) launch_k<KeyT, true, uint8_t>(K, a, s);
    else if constexpr (sizeof(KeyT) == 4) launch_k<KeyT, true, uint16_t>(K, a, s);
  }
}

}  // namespace

uint32_t tile_pass_elems(uint32_t key_bytes) {
  return uint32_t(kTileThreads * kTileVectors * (16 / key_bytes));
}

uint32_t tile_key_bytes(uint32_t bits) { return bits <= 8 ? 1u : (bits <= 16 ? 2u : 4u); }

void launch_tile_pass(uint32_t key_bytes, uint32_t out_bytes, int K, bool out, const TileArgs& a, cudaStream_t s,
                      uint64_t* launches) {
  if (a.launch_tiles == 0) return;
  if (K > kTileMaxLevels) {
    // only as the last pass of a text whose prefixes the histogram gives
    if (out || !a.blockpre || K > kTileGivenMaxLevels) return;
    launch_tile_pass_deep(key_bytes, K, a, s);
  } else if (key_bytes == 1) launch_key<uint8_t>(K, out, out_bytes, a, s);
  else if (key_bytes == 2) launch_key<uint16_t>(K, out, out_bytes, a, s);
  else launch_key<uint32_t>(K, out, out_bytes, a, s);
  ++*launches;
}

}  // namespace pwmgpu
