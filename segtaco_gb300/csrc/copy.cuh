// copy.cuh -- many host<->device copies in one launch, driven by the SMs.
//
// On a Grace-Blackwell node pinned host memory is mapped into the GPU's
// address space and reached over NVLink-C2C, so a kernel can move a batch's
// dense operands between host and device itself: one launch for any number of
// segments instead of one copy-engine call per operand.  The segments are cut
// into 64 KiB chunks; CTAs take chunks in a grid-stride loop (a chunk -> its
// segment by binary search over the chunk prefix), and each thread moves
// 16-byte vectors when both ends are 16-byte aligned, bytes otherwise.
#pragma once

#include <stdint.h>

namespace segtaco {

struct CopySeg {
  const char *src;
  char *dst;
  long long bytes;
  long long chunk_begin;  // first chunk of this segment (prefix over segments)
};

constexpr long long kCopyChunk = 64 * 1024;

inline long long copy_chunks(long long bytes) { return (bytes + kCopyChunk - 1) / kCopyChunk; }

__global__ void __launch_bounds__(256) copy_segments_kernel(const CopySeg *__restrict__ segs,
                                                            int nsegs, long long total_chunks) {
  for (long long c = blockIdx.x; c < total_chunks; c += gridDim.x) {
    int lo = 0, hi = nsegs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (segs[mid].chunk_begin <= c)
        lo = mid;
      else
        hi = mid - 1;
    }
    const CopySeg sg = segs[lo];
    const long long off = (c - sg.chunk_begin) * kCopyChunk;
    const long long n = sg.bytes - off < kCopyChunk ? sg.bytes - off : kCopyChunk;
    const char *s = sg.src + off;
    char *d = sg.dst + off;
    if (((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d)) & 15) == 0) {
      const long long nv = n >> 4;
      const uint4 *s4 = reinterpret_cast<const uint4 *>(s);
      uint4 *d4 = reinterpret_cast<uint4 *>(d);
      for (long long i = threadIdx.x; i < nv; i += blockDim.x) d4[i] = s4[i];
      for (long long i = (nv << 4) + threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
    } else {
      for (long long i = threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
    }
  }
}

}  // namespace segtaco
