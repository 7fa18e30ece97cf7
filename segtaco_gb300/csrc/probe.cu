// probe.cu -- segtaco_probe_gather: the random-row gather ceiling of the GPU.
//
// SpMM over a CSR with scattered columns gathers one dense row slice per
// nonzero; its speed is set by how many such gathers the L2 and HBM serve per
// second, not by the streamed bytes.  This kernel does only that: warps load
// rows of `row_bytes` bytes at pseudo-random positions of a buffer (a hash of
// the gather index, so no index stream competes) with four sixteen-byte loads
// per lane in flight, and fold them into one value per warp.  Timing it over
// buffers smaller and larger than the L2 gives the two ceilings that bound the
// SpMM kernels.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace segtaco {
namespace {

__device__ __forceinline__ unsigned int mix32(unsigned int x) {
  // "lowbias32" integer hash (C. Wellons, 2018): two multiplies, three shifts
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

template <int LPR>  // lanes per row: row_bytes / 16
__global__ void __launch_bounds__(256, 4) gather_probe_kernel(const uint4 *__restrict__ buf,
                                                           long long rows, long long n,
                                                           unsigned int seed,
                                                           float *__restrict__ sink) {
  constexpr int RPW = 32 / LPR;  // rows per warp step
  constexpr int U = 8;
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  float acc = 0.f;
  for (long long base = warp * RPW * U; base < n; base += nwarps * RPW * U) {
    uint4 v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long long e = base + u * RPW + lane / LPR;
      if (e < n) {
        // multiply-high maps the 32-bit hash uniformly onto [0, rows)
        const long long r = (long long)__umulhi(mix32((unsigned int)e ^ seed), (unsigned int)rows);
        v[u] = __ldg(buf + r * LPR + (lane % LPR));
      } else {
        v[u] = make_uint4(0, 0, 0, 0);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
      acc += __uint_as_float(v[u].x) + __uint_as_float(v[u].y) + __uint_as_float(v[u].z) +
             __uint_as_float(v[u].w);
  }
  if (acc == 1234.5f) sink[threadIdx.x & 31] = acc;  // keeps the loads live
}

}  // namespace
}  // namespace segtaco

using namespace segtaco;

extern "C" int segtaco_probe_gather(const void *buf, int64_t rows, int32_t row_bytes, int64_t n,
                                    uint32_t seed, float *sink, int32_t blocks, void *stream) {
  if (!buf || !sink || rows <= 0 || n < 0 || blocks < 0)
    return set_error(SEGTACO_EINVAL, "probe: bad arguments");
  if ((reinterpret_cast<uintptr_t>(buf) & 15) != 0)
    return set_error(SEGTACO_EINVAL, "probe: buffer must be 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const auto *b = static_cast<const uint4 *>(buf);
  if (rows > 0xffffffffLL) return set_error(SEGTACO_EINVAL, "probe: at most 2^32 - 1 rows");
  const unsigned int sd = 0x9e3779b9u * (seed + 1);
  // blocks == 0: one resident wave (every SM full, no second wave).
  auto grid = [&](const void *fn) {
    if (blocks > 0) return blocks;
    int per_sm = 1, dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0);
    return std::max(1, per_sm) * sms;
  };
#define SEGTACO_PROBE(L)                                                       \
  gather_probe_kernel<L><<<grid((const void *)gather_probe_kernel<L>), 256, 0, s>>>( \
      b, rows, n, sd, sink);                                                   \
  break;
  switch (row_bytes) {
    case 16: SEGTACO_PROBE(1)
    case 32: SEGTACO_PROBE(2)
    case 64: SEGTACO_PROBE(4)
    case 128: SEGTACO_PROBE(8)
    case 256: SEGTACO_PROBE(16)
    case 512: SEGTACO_PROBE(32)
    default: return set_error(SEGTACO_EINVAL, "probe: row_bytes must be 16..512, a power of two");
  }
#undef SEGTACO_PROBE
  return check_launch("gather_probe_kernel");
}

#include "copy.cuh"

namespace segtaco {
// The address a kernel uses for `p`: device memory as is, pinned host memory
// through its mapping; anything else (pageable host memory) is refused, so no
// kernel ever dereferences memory the GPU cannot reach.
int device_view(const void *p, void **out) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return set_error(SEGTACO_EINVAL, "pointer %p is not known to CUDA", p);
  }
  if ((a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged ||
       a.type == cudaMemoryTypeHost) && a.devicePointer != nullptr) {
    *out = a.devicePointer;
    return SEGTACO_OK;
  }
  return set_error(SEGTACO_EINVAL, "pointer %p is neither device nor mapped pinned memory", p);
}
}  // namespace segtaco

// Diagnostic: one segment moved by copy_segments_kernel (src/dst may be mapped
// pinned host memory or device memory); the segment descriptor is staged in
// `desc` (device memory, at least 64 bytes).
extern "C" int segtaco_probe_copy(void *dst, const void *src, int64_t bytes, void *desc,
                                  int32_t blocks, void *stream) {
  using namespace segtaco;
  if (!dst || !src || !desc || bytes < 0 || blocks <= 0)
    return set_error(SEGTACO_EINVAL, "probe_copy: bad arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void *vs = nullptr, *vd = nullptr;
  SEGTACO_TRY(device_view(src, &vs));
  SEGTACO_TRY(device_view(dst, &vd));
  CopySeg sg{static_cast<const char *>(vs), static_cast<char *>(vd), bytes, 0};
  SEGTACO_TRY(check_cuda(cudaMemcpyAsync(desc, &sg, sizeof(sg), cudaMemcpyHostToDevice, s),
                         "probe_copy descriptor"));
  const long long chunks = copy_chunks(bytes);
  if (chunks == 0) return SEGTACO_OK;
  copy_segments_kernel<<<blocks, 256, 0, s>>>(static_cast<const CopySeg *>(desc), 1, chunks);
  return check_launch("copy_segments_kernel");
}
