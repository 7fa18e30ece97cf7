// common.cuh -- device helpers shared by the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "segtaco.h"

namespace segtaco {

constexpr int kCta = 256;  // threads per CTA for every streaming kernel

// ---------------------------------------------------------------------------
// Loads with explicit cache behaviour (PTX ISA "ld" with cache operators).
// ---------------------------------------------------------------------------

// CSR index / value streams are read once per column slab: cache-streaming.
__device__ __forceinline__ int ld_stream(const int *p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float *p) { return __ldcs(p); }

// L2 policy for the gathered dense rows: keep them (evict_last) so that the
// slab of B being gathered stays L2-resident while the CSR streams pass by.
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

__device__ __forceinline__ uint64_t l2_policy_evict_normal() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ uint64_t l2_policy(int evict_last) {
  return evict_last ? l2_policy_evict_last() : l2_policy_evict_normal();
}

template <bool kHint>
__device__ __forceinline__ float4 ld_b4(const float *p, uint64_t pol) {
  float4 r;
  if (kHint) {
    asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
                 : "l"(p), "l"(pol));
  } else {
    r = __ldg(reinterpret_cast<const float4 *>(p));
  }
  return r;
}
template <bool kHint>
__device__ __forceinline__ float2 ld_b2(const float *p, uint64_t pol) {
  float2 r;
  if (kHint) {
    asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0,%1}, [%2], %3;"
                 : "=f"(r.x), "=f"(r.y)
                 : "l"(p), "l"(pol));
  } else {
    r = __ldg(reinterpret_cast<const float2 *>(p));
  }
  return r;
}
template <bool kHint>
__device__ __forceinline__ float ld_b1(const float *p, uint64_t pol) {
  float r;
  if (kHint) {
    asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(r) : "l"(p), "l"(pol));
  } else {
    r = __ldg(p);
  }
  return r;
}
template <bool kHint>
__device__ __forceinline__ uint4 ld_u4(const uint16_t *p, uint64_t pol) {
  uint4 r;
  if (kHint) {
    asm volatile("ld.global.nc.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "l"(p), "l"(pol));
  } else {
    r = __ldg(reinterpret_cast<const uint4 *>(p));
  }
  return r;
}
template <bool kHint>
__device__ __forceinline__ uint2 ld_u2(const uint16_t *p, uint64_t pol) {
  uint2 r;
  if (kHint) {
    asm volatile("ld.global.nc.L2::cache_hint.v2.u32 {%0,%1}, [%2], %3;"
                 : "=r"(r.x), "=r"(r.y)
                 : "l"(p), "l"(pol));
  } else {
    r = __ldg(reinterpret_cast<const uint2 *>(p));
  }
  return r;
}
template <bool kHint>
__device__ __forceinline__ uint32_t ld_u1(const uint16_t *p, uint64_t pol) {
  uint32_t r;
  if (kHint) {
    asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
  } else {
    r = __ldg(reinterpret_cast<const unsigned int *>(p));
  }
  return r;
}

// Predicated loads of the dense operand: the destination registers are zeroed
// and the load runs only where `ok` holds, so a lane with no nonzero to
// gather moves no data through the load/store pipe (an unpredicated dummy
// load of a cached row still costs its data-stage wavefronts).
// PTR, POL and OK name the operand numbers that follow the outputs.
#define SEGTACO_PRED_LD(TYPE, VEC, OUTS, ZEROS, PTR, POL, OK, ...)                       \
  asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.b32 q, " OK ", 0;\n\t" ZEROS               \
               "@q ld.global.nc.L2::cache_hint" VEC "." TYPE " " OUTS ", [" PTR "], " POL   \
               ";\n\t}"                                                                  \
               : __VA_ARGS__                                                             \
               : "l"(p), "l"(pol), "r"((int)ok))
__device__ __forceinline__ float4 ld_b4_if(const float *p, uint64_t pol, bool ok) {
  float4 r;
  SEGTACO_PRED_LD("f32", ".v4", "{%0,%1,%2,%3}",
                  "mov.b32 %0, 0;\n\tmov.b32 %1, 0;\n\tmov.b32 %2, 0;\n\tmov.b32 %3, 0;\n\t",
                  "%4", "%5", "%6", "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w));
  return r;
}
__device__ __forceinline__ float2 ld_b2_if(const float *p, uint64_t pol, bool ok) {
  float2 r;
  SEGTACO_PRED_LD("f32", ".v2", "{%0,%1}", "mov.b32 %0, 0;\n\tmov.b32 %1, 0;\n\t", "%2", "%3", "%4", "=f"(r.x),
                  "=f"(r.y));
  return r;
}
__device__ __forceinline__ float ld_b1_if(const float *p, uint64_t pol, bool ok) {
  float r;
  SEGTACO_PRED_LD("f32", "", "%0", "mov.b32 %0, 0;\n\t", "%1", "%2", "%3", "=f"(r));
  return r;
}
__device__ __forceinline__ uint4 ld_u4_if(const uint16_t *p, uint64_t pol, bool ok) {
  uint4 r;
  SEGTACO_PRED_LD("u32", ".v4", "{%0,%1,%2,%3}",
                  "mov.b32 %0, 0;\n\tmov.b32 %1, 0;\n\tmov.b32 %2, 0;\n\tmov.b32 %3, 0;\n\t",
                  "%4", "%5", "%6", "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w));
  return r;
}
__device__ __forceinline__ uint2 ld_u2_if(const uint16_t *p, uint64_t pol, bool ok) {
  uint2 r;
  SEGTACO_PRED_LD("u32", ".v2", "{%0,%1}", "mov.b32 %0, 0;\n\tmov.b32 %1, 0;\n\t", "%2", "%3", "%4", "=r"(r.x),
                  "=r"(r.y));
  return r;
}
__device__ __forceinline__ uint32_t ld_u1_if(const uint16_t *p, uint64_t pol, bool ok) {
  uint32_t r;
  SEGTACO_PRED_LD("u32", "", "%0", "mov.b32 %0, 0;\n\t", "%1", "%2", "%3", "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t ld_h1_if(const uint16_t *p, uint64_t pol, bool ok) {
  uint32_t r;
  SEGTACO_PRED_LD("u16", "", "%0", "mov.b32 %0, 0;\n\t", "%1", "%2", "%3", "=r"(r));
  return r;
}

// bf16 bit pattern -> float (exact: bf16 is the top half of a float).
__device__ __forceinline__ float bf16lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

// V consecutive dense elements as one raw vector load (kept raw in registers
// until used, so a bf16 x 8 load costs 4 registers, like an fp32 x 4 one).
// float: V in {1,2,4}; bf16 (uint16_t): V in {1,2,4,8}.
template <typename BT, int V> struct Dense;

// fp32 x 8: two sixteen-byte loads per lane, so a 32-column slab needs only
// G = 4 lanes per nonzero and a warp has P = 8 slots.
struct F8 {
  float4 a, b;
};
template <> struct Dense<float, 8> {
  using raw_t = F8;
  // One 32-byte load (ld.global.v8.f32, sm_100+): p is 32-byte aligned.
  static __device__ __forceinline__ raw_t load(const float *p, uint64_t pol) {
    F8 r;
    asm volatile("ld.global.nc.L2::cache_hint.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
                 : "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x),
                   "=f"(r.b.y), "=f"(r.b.z), "=f"(r.b.w)
                 : "l"(p), "l"(pol));
    return r;
  }
  static __device__ __forceinline__ raw_t load_if(const float *p, uint64_t pol, bool ok) {
    F8 r;
    SEGTACO_PRED_LD("f32", ".v8", "{%0,%1,%2,%3,%4,%5,%6,%7}",
                    "mov.b32 %0, 0;\n\tmov.b32 %1, 0;\n\tmov.b32 %2, 0;\n\tmov.b32 %3, 0;\n\t"
                    "mov.b32 %4, 0;\n\tmov.b32 %5, 0;\n\tmov.b32 %6, 0;\n\tmov.b32 %7, 0;\n\t",
                    "%8", "%9", "%10", "=f"(r.a.x), "=f"(r.a.y), "=f"(r.a.z), "=f"(r.a.w), "=f"(r.b.x), "=f"(r.b.y),
                    "=f"(r.b.z), "=f"(r.b.w));
    return r;
  }
  // The same slice from shared memory (32-byte aligned).
  static __device__ __forceinline__ raw_t lds(const float *p) {
    F8 r;
    r.a = *reinterpret_cast<const float4 *>(p);
    r.b = *reinterpret_cast<const float4 *>(p + 4);
    return r;
  }
  static __device__ __forceinline__ float get(const raw_t &r, int v) {
    const float4 &h = v < 4 ? r.a : r.b;
    const int w = v & 3;
    return w == 0 ? h.x : w == 1 ? h.y : w == 2 ? h.z : h.w;
  }
};
template <> struct Dense<float, 4> {
  using raw_t = float4;
  static __device__ __forceinline__ raw_t load(const float *p, uint64_t pol) {
    return ld_b4<true>(p, pol);
  }
  static __device__ __forceinline__ raw_t load_if(const float *p, uint64_t pol, bool ok) {
    return ld_b4_if(p, pol, ok);
  }
  static __device__ __forceinline__ raw_t lds(const float *p) {
    return *reinterpret_cast<const float4 *>(p);
  }
  static __device__ __forceinline__ float get(const raw_t &r, int v) {
    return v == 0 ? r.x : v == 1 ? r.y : v == 2 ? r.z : r.w;
  }
};
template <> struct Dense<float, 2> {
  using raw_t = float2;
  static __device__ __forceinline__ raw_t load(const float *p, uint64_t pol) {
    return ld_b2<true>(p, pol);
  }
  static __device__ __forceinline__ raw_t load_if(const float *p, uint64_t pol, bool ok) {
    return ld_b2_if(p, pol, ok);
  }
  static __device__ __forceinline__ raw_t lds(const float *p) {
    return *reinterpret_cast<const float2 *>(p);
  }
  static __device__ __forceinline__ float get(const raw_t &r, int v) { return v == 0 ? r.x : r.y; }
};
template <> struct Dense<float, 1> {
  using raw_t = float;
  static __device__ __forceinline__ raw_t load(const float *p, uint64_t pol) {
    return ld_b1<true>(p, pol);
  }
  static __device__ __forceinline__ raw_t load_if(const float *p, uint64_t pol, bool ok) {
    return ld_b1_if(p, pol, ok);
  }
  static __device__ __forceinline__ raw_t lds(const float *p) { return *p; }
  static __device__ __forceinline__ float get(const raw_t &r, int) { return r; }
};
// Sixteen bf16 values in one 32-byte load (ld.global.v8.b32, sm_100+): p is
// 32-byte aligned.
struct U8 {
  uint4 a, b;
};
template <> struct Dense<uint16_t, 16> {
  using raw_t = U8;
  static __device__ __forceinline__ raw_t load(const uint16_t *p, uint64_t pol) {
    U8 r;
    asm volatile("ld.global.nc.L2::cache_hint.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
                 : "=r"(r.a.x), "=r"(r.a.y), "=r"(r.a.z), "=r"(r.a.w), "=r"(r.b.x),
                   "=r"(r.b.y), "=r"(r.b.z), "=r"(r.b.w)
                 : "l"(p), "l"(pol));
    return r;
  }
  static __device__ __forceinline__ raw_t load_if(const uint16_t *p, uint64_t pol, bool ok) {
    U8 r;
    SEGTACO_PRED_LD("b32", ".v8", "{%0,%1,%2,%3,%4,%5,%6,%7}",
                    "mov.b32 %0, 0;\n\tmov.b32 %1, 0;\n\tmov.b32 %2, 0;\n\tmov.b32 %3, 0;\n\t"
                    "mov.b32 %4, 0;\n\tmov.b32 %5, 0;\n\tmov.b32 %6, 0;\n\tmov.b32 %7, 0;\n\t",
                    "%8", "%9", "%10", "=r"(r.a.x), "=r"(r.a.y), "=r"(r.a.z), "=r"(r.a.w), "=r"(r.b.x), "=r"(r.b.y),
                    "=r"(r.b.z), "=r"(r.b.w));
    return r;
  }
  static __device__ __forceinline__ raw_t lds(const uint16_t *p) {
    U8 r;
    r.a = *reinterpret_cast<const uint4 *>(p);
    r.b = *reinterpret_cast<const uint4 *>(p + 8);
    return r;
  }
  static __device__ __forceinline__ float get(const raw_t &r, int v) {
    const uint4 &h = v < 8 ? r.a : r.b;
    const int q = (v & 7) >> 1;
    const uint32_t w = q == 0 ? h.x : q == 1 ? h.y : q == 2 ? h.z : h.w;
    return (v & 1) ? bf16hi(w) : bf16lo(w);
  }
};
template <> struct Dense<uint16_t, 8> {
  using raw_t = uint4;
  static __device__ __forceinline__ raw_t load(const uint16_t *p, uint64_t pol) {
    return ld_u4<true>(p, pol);
  }
  static __device__ __forceinline__ raw_t load_if(const uint16_t *p, uint64_t pol, bool ok) {
    return ld_u4_if(p, pol, ok);
  }
  static __device__ __forceinline__ raw_t lds(const uint16_t *p) {
    return *reinterpret_cast<const uint4 *>(p);
  }
  static __device__ __forceinline__ float get(const raw_t &r, int v) {
    const uint32_t w = v < 2 ? r.x : v < 4 ? r.y : v < 6 ? r.z : r.w;
    return (v & 1) ? bf16hi(w) : bf16lo(w);
  }
};
template <> struct Dense<uint16_t, 4> {
  using raw_t = uint2;
  static __device__ __forceinline__ raw_t load(const uint16_t *p, uint64_t pol) {
    return ld_u2<true>(p, pol);
  }
  static __device__ __forceinline__ raw_t load_if(const uint16_t *p, uint64_t pol, bool ok) {
    return ld_u2_if(p, pol, ok);
  }
  static __device__ __forceinline__ raw_t lds(const uint16_t *p) {
    return *reinterpret_cast<const uint2 *>(p);
  }
  static __device__ __forceinline__ float get(const raw_t &r, int v) {
    const uint32_t w = v < 2 ? r.x : r.y;
    return (v & 1) ? bf16hi(w) : bf16lo(w);
  }
};
template <> struct Dense<uint16_t, 2> {
  using raw_t = uint32_t;
  static __device__ __forceinline__ raw_t load(const uint16_t *p, uint64_t pol) {
    return ld_u1<true>(p, pol);
  }
  static __device__ __forceinline__ raw_t load_if(const uint16_t *p, uint64_t pol, bool ok) {
    return ld_u1_if(p, pol, ok);
  }
  static __device__ __forceinline__ raw_t lds(const uint16_t *p) {
    return *reinterpret_cast<const uint32_t *>(p);
  }
  static __device__ __forceinline__ float get(const raw_t &r, int v) {
    return (v & 1) ? bf16hi(r) : bf16lo(r);
  }
};
template <> struct Dense<uint16_t, 1> {
  using raw_t = uint32_t;
  static __device__ __forceinline__ raw_t load(const uint16_t *p, uint64_t) {
    return (uint32_t)__ldg(reinterpret_cast<const unsigned short *>(p));
  }
  static __device__ __forceinline__ raw_t load_if(const uint16_t *p, uint64_t pol, bool ok) {
    return ld_h1_if(p, pol, ok);
  }
  static __device__ __forceinline__ raw_t lds(const uint16_t *p) {
    return (uint32_t)*p;
  }
  static __device__ __forceinline__ float get(const raw_t &r, int) { return bf16lo(r); }
};

// Compatibility form used by the SDDMM kernel: load and convert at once.
template <typename BT, int V, bool kHint> struct DenseLoad {
  static __device__ __forceinline__ void run(const BT *p, float (&o)[V], uint64_t pol) {
    const auto r = Dense<BT, V>::load(p, pol);
#pragma unroll
    for (int v = 0; v < V; ++v) o[v] = Dense<BT, V>::get(r, v);
  }
};

// Store V floats (streaming: C is written once and never re-read here).
template <int V> __device__ __forceinline__ void store_c(float *p, const float (&a)[V]) {
  if constexpr (V >= 8) {
#pragma unroll
    for (int k = 0; k < V; k += 4)
      __stcs(reinterpret_cast<float4 *>(p + k), make_float4(a[k], a[k + 1], a[k + 2], a[k + 3]));
  } else if constexpr (V == 4) {
    __stcs(reinterpret_cast<float4 *>(p), make_float4(a[0], a[1], a[2], a[3]));
  } else if constexpr (V == 2) {
    __stcs(reinterpret_cast<float2 *>(p), make_float2(a[0], a[1]));
  } else {
    __stcs(p, a[0]);
  }
}

// Vector reduction into global memory (red.global.add.v4.f32, sm_90+).
__device__ __forceinline__ void red_add4(float *p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1,%2,%3,%4};" ::"l"(p), "f"(a), "f"(b), "f"(c),
               "f"(d)
               : "memory");
}
__device__ __forceinline__ void red_add2(float *p, float a, float b) {
  asm volatile("red.global.add.v2.f32 [%0], {%1,%2};" ::"l"(p), "f"(a), "f"(b) : "memory");
}
template <int V> __device__ __forceinline__ void atomic_add_c(float *p, const float (&a)[V]) {
  if constexpr (V >= 8) {
#pragma unroll
    for (int k = 0; k < V; k += 4) red_add4(p + k, a[k], a[k + 1], a[k + 2], a[k + 3]);
  } else if constexpr (V == 4) {
    red_add4(p, a[0], a[1], a[2], a[3]);
  } else if constexpr (V == 2) {
    red_add2(p, a[0], a[1]);
  } else {
    atomicAdd(p, a[0]);
  }
}

// Lanes [g*G, g*G+G) of a warp form lane group g.
template <int G> __device__ __forceinline__ unsigned group_mask(int lane) {
  if constexpr (G == 32) {
    (void)lane;
    return 0xffffffffu;
  } else {
    return ((1u << G) - 1u) << ((lane / G) * G);
  }
}

__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }

// Merge-path split of diagonal d over {row ends} U {nonzeros}: x = number of
// row ends taken; row end x sorts before nonzero y when row_ptr[x+1] <= y.
__device__ __forceinline__ int merge_path_x(const int *__restrict__ row_ptr, int M, long long nnz,
                                            long long d) {
  long long lo = d - nnz;
  if (lo < 0) lo = 0;
  long long hi = d < M ? d : M;
  while (lo < hi) {
    long long pivot = (lo + hi) >> 1;
    if ((long long)__ldg(row_ptr + pivot + 1) <= d - pivot - 1)
      lo = pivot + 1;
    else
      hi = pivot;
  }
  return (int)lo;
}

// Merge-path edges by rows instead of by search.  Row end r is merge item
// e_r - 1 with e_r = row_ptr[r+1] + r + 1, so the split of diagonal d takes
// x(d) = #{r : e_r <= d} row ends -- exactly the row merge_path_x finds.
// Hence the chunk edges c with e_{r-1} <= c*D < e_r (e_{-1} = 0) all have
// x = r, and one thread per row can write them; a tail thread (r = M) writes
// the edges at or past the last row end.  Every edge is written by exactly one
// thread, with coalesced reads of row_ptr.
__device__ __forceinline__ long long ceil_div_pos(long long a, long long D, bool small) {
  if (small) return (long long)(((unsigned)a + (unsigned)D - 1u) / (unsigned)D);
  return (a + D - 1) / D;
}
// Stores the edges [c_lo, c_hi] of row r (0 <= r <= M), zeroing row r of C
// (N columns) once if it straddles one of them.
__device__ __forceinline__ void merge_path_store_row(const int *__restrict__ row_ptr, int M,
                                                     long long nnz, long long D, long long nchunks,
                                                     long long r, long long c_lo, long long c_hi,
                                                     int *__restrict__ px, int *__restrict__ py,
                                                     float *__restrict__ C, long long ldc, int N) {
  const long long total = (long long)M + nnz;
  if (c_hi > nchunks) c_hi = nchunks;
  if (c_lo > c_hi) return;
  for (long long c = c_lo; c <= c_hi; ++c) {
    long long d = c * D;
    if (d > total) d = total;
    px[c] = (int)r;
    py[c] = (int)(d - r);
  }
  if (C != nullptr && r < M) {
    long long dl = c_hi * D;
    if (dl > total) dl = total;
    if ((long long)__ldg(row_ptr + r) < dl - r) {  // y grows with c: test the last edge
      float *dst = C + r * ldc;
      int k = 0;
      if ((((uintptr_t)dst) & 15) == 0)
        for (; k + 4 <= N; k += 4) *reinterpret_cast<float4 *>(dst + k) = make_float4(0, 0, 0, 0);
      for (; k < N; ++k) dst[k] = 0.0f;
    }
  }
}

}  // namespace segtaco
