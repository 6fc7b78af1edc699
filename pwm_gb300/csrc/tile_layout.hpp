// Layout of the tile passes' per-segment start tables and their level limits,
// shared by the kernels and the host planner (compiles with or without CUDA).
#pragma once

#if defined(__CUDACC__)
#define PWMGPU_HOST_DEVICE __host__ __device__
#else
#define PWMGPU_HOST_DEVICE
#endif

namespace pwmgpu {

constexpr int kTileMaxLevels = 4;
// A last pass whose finest-run prefixes are given (the histogram kernel's, for
// texts of at most 8 levels) neither counts nor looks back, and may split up
// to 7 times: all levels of such a text in one pass.
constexpr int kTileGivenMaxLevels = 8;

// Table entries of one segment: matrix starts (level j, run v) at
// (1 << j) - 1 + v, tree starts after them, then the S_out starts (2^K).
PWMGPU_HOST_DEVICE constexpr int tile_table_size(int K) { return 2 * ((1 << K) - 1) + (1 << K); }
PWMGPU_HOST_DEVICE constexpr int tile_wm_entry(int j, int v) { return (1 << j) - 1 + v; }
PWMGPU_HOST_DEVICE constexpr int tile_wt_entry(int K, int j, int v) { return (1 << K) - 1 + (1 << j) - 1 + v; }
PWMGPU_HOST_DEVICE constexpr int tile_out_entry(int K, int v) { return 2 * ((1 << K) - 1) + v; }

}  // namespace pwmgpu
