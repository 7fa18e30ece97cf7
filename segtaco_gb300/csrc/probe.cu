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
#include "common.cuh"
#include "internal.h"

namespace segtaco {
namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  // splitmix64 finaliser (Steele, Lea, Flood 2014)
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ULL;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebULL;
  x ^= x >> 31;
  return x;
}

template <int LPR>  // lanes per row: row_bytes / 16
__global__ void __launch_bounds__(256) gather_probe_kernel(const uint4 *__restrict__ buf,
                                                           long long rows, long long n,
                                                           unsigned long long seed,
                                                           float *__restrict__ sink) {
  constexpr int RPW = 32 / LPR;  // rows per warp step
  constexpr int U = 4;
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
        // multiply-high maps the hash uniformly onto [0, rows)
        const long long r = (long long)__umul64hi(mix64((unsigned long long)e ^ seed),
                                                  (unsigned long long)rows);
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
  if (!buf || !sink || rows <= 0 || n < 0 || blocks <= 0)
    return set_error(SEGTACO_EINVAL, "probe: bad arguments");
  if ((reinterpret_cast<uintptr_t>(buf) & 15) != 0)
    return set_error(SEGTACO_EINVAL, "probe: buffer must be 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const auto *b = static_cast<const uint4 *>(buf);
  const unsigned long long sd = 0x9e3779b97f4a7c15ULL * (seed + 1);
  switch (row_bytes) {
    case 16: gather_probe_kernel<1><<<blocks, 256, 0, s>>>(b, rows, n, sd, sink); break;
    case 32: gather_probe_kernel<2><<<blocks, 256, 0, s>>>(b, rows, n, sd, sink); break;
    case 64: gather_probe_kernel<4><<<blocks, 256, 0, s>>>(b, rows, n, sd, sink); break;
    case 128: gather_probe_kernel<8><<<blocks, 256, 0, s>>>(b, rows, n, sd, sink); break;
    case 256: gather_probe_kernel<16><<<blocks, 256, 0, s>>>(b, rows, n, sd, sink); break;
    case 512: gather_probe_kernel<32><<<blocks, 256, 0, s>>>(b, rows, n, sd, sink); break;
    default: return set_error(SEGTACO_EINVAL, "probe: row_bytes must be 16..512, a power of two");
  }
  return check_launch("gather_probe_kernel");
}
