/*
 * gpu_construction.cpp -- registration unit for kurpicz/pwm.
 *
 * Copy to pwm's src/register/ and add it to INTERNAL_SRCS in
 * src/CMakeLists.txt and to CONSTRUCTION_ALGORITHMS in
 * test/util/testsuite.cmake, with this repository's include/ on the include
 * path and pwm_gb300/libpwmgpu.so linked; pwm's benchmark and `make check`
 * then run the GB300 engine like every other registered construction.  The
 * pattern is pwm's own (src/register/sequential_prefix_counting.cpp:10-48):
 * one alias and one CONSTRUCTION_REGISTER per alphabet width, the 40-bit
 * width (pwm's uint40_t) included for the plain structures.
 */
#include "util/type_for_bytes.hpp"
#include "benchmark/algorithm.hpp"
#include "wx_gpu.hpp"

using wm_gpu_8 = wx_gpu<uint8_t, false>;
using wm_gpu_16 = wx_gpu<uint16_t, false>;
using wm_gpu_32 = wx_gpu<uint32_t, false>;
using wm_gpu_40 = wx_gpu<uint40_t, false>;
using wt_gpu_8 = wx_gpu<uint8_t, true>;
using wt_gpu_16 = wx_gpu<uint16_t, true>;
using wt_gpu_32 = wx_gpu<uint32_t, true>;
using wt_gpu_40 = wx_gpu<uint40_t, true>;

CONSTRUCTION_REGISTER("wm_gpu", "GB300 wavelet matrix construction with 8-bit alphabet.", wm_gpu_8)
CONSTRUCTION_REGISTER("wm_gpu", "GB300 wavelet matrix construction with 16-bit alphabet.", wm_gpu_16)
CONSTRUCTION_REGISTER("wm_gpu", "GB300 wavelet matrix construction with 32-bit alphabet.", wm_gpu_32)
CONSTRUCTION_REGISTER("wm_gpu", "GB300 wavelet matrix construction with 40-bit alphabet.", wm_gpu_40)
CONSTRUCTION_REGISTER("wt_gpu", "GB300 wavelet tree construction with 8-bit alphabet.", wt_gpu_8)
CONSTRUCTION_REGISTER("wt_gpu", "GB300 wavelet tree construction with 16-bit alphabet.", wt_gpu_16)
CONSTRUCTION_REGISTER("wt_gpu", "GB300 wavelet tree construction with 32-bit alphabet.", wt_gpu_32)
CONSTRUCTION_REGISTER("wt_gpu", "GB300 wavelet tree construction with 40-bit alphabet.", wt_gpu_40)

using wm_gpu_huff_8 = wx_gpu_huff<uint8_t, false>;
using wm_gpu_huff_16 = wx_gpu_huff<uint16_t, false>;
using wt_gpu_huff_8 = wx_gpu_huff<uint8_t, true>;
using wt_gpu_huff_16 = wx_gpu_huff<uint16_t, true>;

CONSTRUCTION_REGISTER("wm_gpu_huff", "GB300 Huffman-shaped wavelet matrix construction with 8-bit alphabet.",
                      wm_gpu_huff_8)
CONSTRUCTION_REGISTER("wm_gpu_huff", "GB300 Huffman-shaped wavelet matrix construction with 16-bit alphabet.",
                      wm_gpu_huff_16)
CONSTRUCTION_REGISTER("wt_gpu_huff", "GB300 Huffman-shaped wavelet tree construction with 8-bit alphabet.",
                      wt_gpu_huff_8)
CONSTRUCTION_REGISTER("wt_gpu_huff", "GB300 Huffman-shaped wavelet tree construction with 16-bit alphabet.",
                      wt_gpu_huff_16)
