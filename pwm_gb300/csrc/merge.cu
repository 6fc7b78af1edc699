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

// Staging word w, thread per word: the segment whose staged words hold it
// (binary search over the stage offsets), then its bits shifted into place.
__global__ void stage_segments_kernel(const StageSeg* segs, uint64_t nseg, uint64_t* staging, uint64_t total,
                                      uint32_t* status) {
  for (uint64_t w = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < total;
       w += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t lo = 0, hi = nseg;  // the last segment with stage <= w
    while (hi - lo > 1) {
      const uint64_t mid = (lo + hi) >> 1;
      if (segs[mid].stage <= w) lo = mid; else hi = mid;
    }
    const StageSeg sg = segs[lo];
    const uint64_t dw = (sg.dst_bit >> 6) + (w - sg.stage);
    const uint64_t end = sg.dst_bit + sg.len;
    const uint64_t b0 = dw * 64 > sg.dst_bit ? dw * 64 : sg.dst_bit, b1 = dw * 64 + 64 < end ? dw * 64 + 64 : end;
    if (sg.stage > w || b0 >= b1) {  // inconsistent layout: never read out of range
      atomicOr(status, kErrBounds);
      staging[w] = 0;
      continue;
    }
    staging[w] = bits_from(sg.src, sg.src_bit + (b0 - sg.dst_bit), uint32_t(b1 - b0)) >> (b0 - dw * 64);
  }
}

__global__ void gather_words_kernel(const uint64_t* words, const uint64_t* idx, uint64_t count, uint64_t* out) {
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += uint64_t(gridDim.x) * blockDim.x)
    out[i] = words[idx[i]];
}

}  // namespace

void launch_stage_segments(const StageSeg* segs, uint64_t nseg, uint64_t* staging, uint64_t total, uint32_t* status,
                           cudaStream_t s, uint64_t* launches) {
  if (nseg == 0 || total == 0) return;
  const uint64_t blocks = (total + 255) / 256;
  stage_segments_kernel<<<unsigned(blocks < 65535 ? blocks : 65535), 256, 0, s>>>(segs, nseg, staging, total, status);
  ++*launches;
}

void launch_gather_words(const uint64_t* words, const uint64_t* idx, uint64_t count, uint64_t* out, cudaStream_t s,
                         uint64_t* launches) {
  if (count == 0) return;
  const uint64_t blocks = (count + 255) / 256;
  gather_words_kernel<<<unsigned(blocks < 4096 ? blocks : 4096), 256, 0, s>>>(words, idx, count, out);
  ++*launches;
}

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
