// spmm_kernels.cuh -- the segTACO SpMM schedules as one warp-uniform kernel.
//
// C = A * B, A CSR (M x K), B dense K x N row-major, C dense M x N row-major.
//
// Work layout.  A warp owns one unit of work and one column slab:
//   * unit  = a merge-path chunk of rows+nonzeros (element-balanced, eb_*) or a
//             block of R consecutive rows (row-balanced, rb_*);
//   * slab  = W = G*V dense columns (blockIdx.y), G lanes x V-wide vector loads
//             (16 B per lane for fp32 V=4 / bf16 V=8).
// The 32 lanes form P = 32/G slots of G lanes.  The warp walks the unit's
// nonzeros in storage order, P at a time (one per slot): slot s takes the s-th
// nonzero of each step and reads one W-column segment of that B row.  All
// control flow is warp-uniform: a step whose P nonzeros all lie in the current
// row is a plain multiply-add (the fast path); a step that reaches a row end
// takes the slow path, which folds the slots' partial sums with xor shuffles
// and writes the row.
//
// Schedules (segTACO's 2x2 space, gpu_kernels.cuh:11-93):
//   rb_sr  row blocks, P = 1 (G = 32): every lane sums its columns of a row
//          serially in storage order with fmaf (segTACO spmm_rb_sr.h:187-243)
//   rb_pr  row blocks, P > 1: the slots take interleaved nonzeros of a row and
//          a shuffle tree combines them (segTACO spmm_rb_pr.h:223-375)
//   eb_sr  merge-path chunks, P = 1 (segTACO spmm_eb_sr.h:153-423)
//   eb_pr  merge-path chunks, P > 1, segmented by row (segTACO
//          spmm_eb_pr.h:281-480)
//
// Element-balanced chunks come from the merge-path split (partition.cu).  A row
// whose nonzeros straddle a chunk edge is zeroed by the partition kernel and
// receives red.global.add from each chunk that holds part of it; every other
// row is written once with a plain store, so C needs no memset and atomics
// happen only at partition edges.
//
// Blocks of the grid are dispatched x-fastest, so the GPU finishes (roughly)
// slab 0 of all units before slab 1: only a K x W slab of B has to stay in L2.
#pragma once

#include <climits>

#include "common.cuh"

namespace segtaco {

template <typename BT> struct SpmmArgs {
  int M, K, N;
  long long nnz;
  const int *__restrict__ row_ptr;
  const int *__restrict__ col;
  const float *__restrict__ val;  // nullptr: every value is 1
  const BT *__restrict__ B;
  long long ldb;
  float *__restrict__ C;
  long long ldc;
  const int *__restrict__ part_x;  // eb: merge-path row coordinate of each chunk edge
  const int *__restrict__ part_y;  // eb: merge-path nonzero coordinate
  long long units;                 // number of warps' units (chunks or row blocks)
  int rows_per_unit;               // rb: rows per warp
  int l2_hints;                    // 1: gathered B rows evict_last in L2
};

template <int V> __device__ __forceinline__ void zero(float (&a)[V]) {
#pragma unroll
  for (int v = 0; v < V; ++v) a[v] = 0.0f;
}

__device__ __forceinline__ float ld_val(const float *__restrict__ val, int q) {
  return val ? ld_stream(val + q) : 1.0f;
}

// Sum the P slots' partial sums (lanes g, g+G, g+2G, ...) into every lane.
template <int G, int V> __device__ __forceinline__ void fold_slots(float (&r)[V]) {
#pragma unroll
  for (int o = G; o < 32; o <<= 1) {
#pragma unroll
    for (int v = 0; v < V; ++v) r[v] += __shfl_xor_sync(0xffffffffu, r[v], o);
  }
}

// 4 CTAs (32 warps) per SM: at most 64 registers; the bf16 x 8 variants need
// a few more for their 8 accumulators and run 3 CTAs per SM.
template <typename BT, int V, int G, bool ROWS>
__global__ void __launch_bounds__(kCta, V == 8 ? 3 : 4) spmm_seg_kernel(SpmmArgs<BT> a) {
  constexpr int P = 32 / G;          // slots = nonzeros per step
  constexpr int S = G;               // steps per batch of 32 nonzeros
  // Steps whose B loads are in flight together: 4 sixteen-byte loads or 8
  // narrower ones per lane (raw registers: 16 at most).
  constexpr int UL = V * (int)sizeof(BT) >= 16 ? 4 : 8;
  constexpr int U = S < UL ? S : UL;
  using D = Dense<BT, V>;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int slot = lane / G, gl = lane & (G - 1);
  const long long w = (long long)blockIdx.x * (kCta / 32) + threadIdx.x / 32;
  if (w >= a.units) return;  // whole warp leaves together
  const int M = a.M;
  const int col0 = blockIdx.y * (G * V) + gl * V;
  const bool active = col0 < a.N;
  const uint64_t pol = l2_policy(a.l2_hints);
  // Inactive lanes (past N) still load, from column 0, so that no address is
  // out of bounds; their results are never stored.
  const BT *Bc = a.B + (active ? col0 : 0);
  const unsigned ldb = (unsigned)a.ldb;

  int x0, x1, y0, y1;
  bool head_split = false;
  if (ROWS) {
    const long long r0 = w * a.rows_per_unit;
    x0 = (int)r0;
    x1 = (int)min(r0 + a.rows_per_unit, (long long)M);
    y0 = __ldg(a.row_ptr + x0);
    y1 = __ldg(a.row_ptr + x1);
  } else {
    x0 = __ldg(a.part_x + w);
    y0 = __ldg(a.part_y + w);
    x1 = __ldg(a.part_x + w + 1);
    y1 = __ldg(a.part_y + w + 1);
    head_split = x0 < M && __ldg(a.row_ptr + x0) < y0;
  }

  // Current row and its end; lane l holds the end of row wb + l.
  int cur = x0, wb = x0;
  int rw = (wb + lane < M) ? __ldg(a.row_ptr + wb + 1 + lane) : INT_MAX;
  int cend = __shfl_sync(FULL, rw, 0);
  float acc[V];
  zero<V>(acc);

  // Write row `cur` (the slots' sum) and move to the next row.
  auto flush = [&]() {
    fold_slots<G, V>(acc);
    if (slot == 0 && active) {
      float *dst = a.C + (long long)cur * a.ldc + col0;
      if (!ROWS && cur == x0 && head_split)
        atomic_add_c<V>(dst, acc);
      else
        store_c<V>(dst, acc);
    }
    zero<V>(acc);
    ++cur;
    if (cur - wb == 32) {
      wb = cur;
      rw = (wb + lane < M) ? __ldg(a.row_ptr + wb + 1 + lane) : INT_MAX;
    }
    cend = __shfl_sync(FULL, rw, cur - wb);
  };

  int nb = y1 - y0 < 32 ? y1 - y0 : 32;
  int mc = lane < nb ? ld_stream(a.col + y0 + lane) : 0;
  float mv = lane < nb ? ld_val(a.val, y0 + lane) : 0.0f;
  for (int p = y0; p < y1; p += 32) {
    // Indices of the next batch are loaded while this one is processed.
    const int pn = p + 32;
    const int nbn = y1 - pn < 32 ? y1 - pn : 32;
    const int mcn = lane < nbn ? ld_stream(a.col + pn + lane) : 0;
    const float mvn = lane < nbn ? ld_val(a.val, pn + lane) : 0.0f;
    if (nb == 32 && p + 32 <= cend) {
      // The whole batch lies inside row `cur`: multiply-adds only.
#pragma unroll
      for (int s0 = 0; s0 < S; s0 += U) {
        typename D::raw_t b[U];
        float vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int t = (s0 + u) * P + slot;
          const int j = __shfl_sync(FULL, mc, t);
          vv[u] = __shfl_sync(FULL, mv, t);
          b[u] = D::load(Bc + (size_t)(unsigned)j * ldb, pol);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
          for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], D::get(b[u], v), acc[v]);
        }
      }
      nb = nbn;
      mc = mcn;
      mv = mvn;
      continue;
    }
#pragma unroll
    for (int s0 = 0; s0 < S; s0 += U) {
      if (s0 * P >= nb) break;
      typename D::raw_t b[U];
      float vv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        // Slots past the batch get j = 0, v = 0: a harmless load of B row 0.
        const int t = (s0 + u) * P + slot;
        const int j = __shfl_sync(FULL, mc, t);
        vv[u] = __shfl_sync(FULL, mv, t);
        b[u] = D::load(Bc + (size_t)(unsigned)j * ldb, pol);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int s = s0 + u;
        if (s * P >= nb) break;
        const int qf = p + s * P;                                   // first nonzero of the step
        const int ql = qf + (nb - s * P < P ? nb - s * P : P) - 1;  // last one
        if (ql < cend) {
          if (qf + slot <= ql) {  // slots past the batch hold row 0 of B: skip them
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], D::get(b[u], v), acc[v]);
          }
        } else {
          // The step reaches the end of row `cur` (and maybe of later rows).
          const int q = qf + slot;
          bool pending = q <= ql;
          for (;;) {
            if (pending && q < cend) {
#pragma unroll
              for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], D::get(b[u], v), acc[v]);
              pending = false;
            }
            if (cend > ql) break;
            flush();
          }
        }
      }
    }
    nb = nbn;
    mc = mcn;
    mv = mvn;
  }
  // Rows that end after the last nonzero of the unit (or hold none of it).
  while (cur < x1) flush();
  if (!ROWS && cur < M) {
    // Row x1 continues into the next chunk: its partial sum goes out by reduction.
    const int start = __ldg(a.row_ptr + cur);
    if (y1 > (start > y0 ? start : y0)) {
      fold_slots<G, V>(acc);
      if (slot == 0 && active) atomic_add_c<V>(a.C + (long long)cur * a.ldc + col0, acc);
    }
  }
}

}  // namespace segtaco
