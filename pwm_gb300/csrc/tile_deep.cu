// Tile passes of 5..8 levels (a whole text of at most 8 levels in one pass,
// its finest-run prefixes given by the histogram kernel).
#include "kernels.cuh"
#include "tile_launch.cuh"

namespace pwmgpu {

namespace {

// 1-byte keys in the bit-plane form
template <typename KeyT>
void launch_deep_key(int K, const TileArgs& a, cudaStream_t s) {
  constexpr bool PL = sizeof(KeyT) == 1;
  switch (K) {
    case 5: launch_tile_one<KeyT, 5, false, KeyT, PL>(a, s); break;
    case 6: launch_tile_one<KeyT, 6, false, KeyT, PL>(a, s); break;
    case 7: launch_tile_one<KeyT, 7, false, KeyT, PL>(a, s); break;
    default: launch_tile_one<KeyT, 8, false, KeyT, PL>(a, s); break;
  }
}

}  // namespace

void launch_tile_pass_deep(uint32_t key_bytes, int K, const TileArgs& a, cudaStream_t s) {
  if (key_bytes == 1) launch_deep_key<uint8_t>(K, a, s);
  else if (key_bytes == 2) launch_deep_key<uint16_t>(K, a, s);
  else launch_deep_key<uint32_t>(K, a, s);
}

}  // namespace pwmgpu
