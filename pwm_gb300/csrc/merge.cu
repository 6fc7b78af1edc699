// Merge of independently built shards (pwm's domain decomposition,
// include/construction/merge.hpp) and pwm's bit-range copy on the device.
#include "kernels.cuh"

namespace pwmgpu {

namespace {

// `take` (1..64) bits from bit `pos` of a word array, in the high bits of the
// result (bit i is bit 63-i%64 of word i/64); reads the second word only for
// bits that lie in it.
__device__ __forceinline__ uint64_t bits_from(const uint64_t* w, uint64_t pos, uint32_t take) {
  const uint64_t i = pos >> 6;
  const uint32_t sh = uint32_t(pos & 63);
  uint64_t v = w[i] << sh;
  if (sh && sh + take > 64) v |= w[i + 1] >> (64 - sh);
  return take == 64 ? v : v & ~(~0ull >> take);
}

// Destination word k of [dst_off, dst_off + len), thread per word: whole
// words are stored, the partial words at the ends OR-ed (copy_bits,
// merge.hpp:19-190).
__global__ void copy_bits_kernel(uint64_t* dst, const uint64_t* src, uint64_t dst_off, uint64_t src_off,
                                 uint64_t len) {
  const uint64_t end = dst_off + len;
  const uint64_t w0 = dst_off >> 6, w1 = (end + 63) >> 6;
  for (uint64_t w = w0 + uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < w1;
       w += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t lo = w * 64 > dst_off ? w * 64 : dst_off, hi = w * 64 + 64 < end ? w * 64 + 64 : end;
    const uint32_t take = uint32_t(hi - lo);
    const uint64_t bits = bits_from(src, src_off + (lo - dst_off), take) >> (lo - w * 64);
    if (take == 64) dst[w] = bits;
    else dst[w] |= bits;
  }
}

constexpr uint32_t kMergeCtaWords = 8192;  // destination words per CTA
constexpr uint32_t kMergeCtaSegs = 256;    // segments a CTA stages in shared memory

// The last segment starting at or before bit `pos`.
__device__ __forceinline__ uint64_t find_seg(const MergeSeg* segs, uint64_t nseg, uint64_t pos) {
  uint64_t lo = 0, hi = nseg;
  while (hi - lo > 1) {
    const uint64_t mid = (lo + hi) >> 1;
    if (segs[mid].dst <= pos) lo = mid; else hi = mid;
  }
  return lo;
}

// One level of the merge.  A CTA writes kMergeCtaWords consecutive
// destination words, thread t the words w0 + t + 256 i (loads and stores
// coalesce); the segments that cover them (usually one or two) are staged in
// shared memory, and each thread walks them forward.  Bits past the level
// (nbits) stay 0.
__global__ void __launch_bounds__(256) merge_gather_kernel(const MergeSeg* segs, uint64_t nseg, uint64_t* dst,
                                                           uint64_t nbits, uint32_t* status) {
  __shared__ MergeSeg s_seg[kMergeCtaSegs + 1];
  __shared__ uint64_t s_first;
  __shared__ uint32_t s_count;
  const uint64_t nwords = (nbits + 63) >> 6;
  const uint64_t w0 = uint64_t(blockIdx.x) * kMergeCtaWords;
  const uint64_t w1 = w0 + kMergeCtaWords < nwords ? w0 + kMergeCtaWords : nwords;
  if (threadIdx.x == 0) {
    const uint64_t first = find_seg(segs, nseg, w0 << 6);
    const uint64_t last = find_seg(segs, nseg, (w1 << 6) - 1);  // the segment of the CTA's last bit
    s_first = first;
    s_count = uint32_t(last - first + 1 < kMergeCtaSegs ? last - first + 1 : 0);  // 0: too many to stage
  }
  __syncthreads();
  const uint64_t first = s_first;
  const uint32_t count = s_count;
  for (uint32_t k = threadIdx.x; k <= count && count; k += blockDim.x)  // + the next one's start (segment end)
    s_seg[k] = first + k < nseg ? segs[first + k] : MergeSeg{nbits, 0, nullptr};
  __syncthreads();
  uint32_t si = 0;          // staged index
  uint64_t gi = first;      // global index (when not staged)
  for (uint64_t w = w0 + threadIdx.x; w < w1; w += blockDim.x) {
    const uint64_t wp = w << 6, end = wp + 64 < nbits ? wp + 64 : nbits;
    uint64_t pos = wp, acc = 0;
    while (pos < end) {
      MergeSeg sg;
      uint64_t seg_end;
      if (count) {
        while (si + 1 < count && s_seg[si + 1].dst <= pos) ++si;
        sg = s_seg[si];
        seg_end = s_seg[si + 1].dst;
      } else {
        while (gi + 1 < nseg && segs[gi + 1].dst <= pos) ++gi;
        sg = segs[gi];
        seg_end = gi + 1 < nseg ? segs[gi + 1].dst : nbits;
      }
      if (sg.dst > pos || seg_end <= pos) {  // inconsistent segments: never read out of range
        atomicOr(status, kErrBounds);
        return;
      }
      const uint64_t stop = end < seg_end ? end : seg_end;
      acc |= bits_from(sg.src, sg.src_bit + (pos - sg.dst), uint32_t(stop - pos)) >> (pos - wp);
      pos = stop;
    }
    dst[w] = acc;
  }
}

}  // namespace

void launch_copy_bits(uint64_t* dst, const uint64_t* src, uint64_t dst_off, uint64_t src_off, uint64_t len,
                      cudaStream_t s) {
  if (len == 0) return;
  const uint64_t words = ((dst_off + len + 63) >> 6) - (dst_off >> 6);
  const uint64_t blocks = (words + 255) / 256;
  copy_bits_kernel<<<unsigned(blocks < 65535 ? blocks : 65535), 256, 0, s>>>(dst, src, dst_off, src_off, len);
}

void launch_merge_gather(const MergeSeg* segs, uint64_t nseg, uint64_t* dst, uint64_t nbits, uint32_t* status,
                         cudaStream_t s, uint64_t* launches) {
  const uint64_t nwords = (nbits + 63) >> 6;
  if (nwords == 0 || nseg == 0) return;
  merge_gather_kernel<<<unsigned((nwords + kMergeCtaWords - 1) / kMergeCtaWords), 256, 0, s>>>(segs, nseg, dst, nbits,
                                                                                              status);
  ++*launches;
}

}  // namespace pwmgpu
