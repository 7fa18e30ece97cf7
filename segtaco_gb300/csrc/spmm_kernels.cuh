// spmm_kernels.cuh -- the four segTACO SpMM schedules, written for sm_103a.
//
// C = A * B, A CSR (M x K), B dense K x N row-major, C dense M x N row-major.
//
// Common layout of work (all four kernels):
//   * A lane group of G lanes owns a column slab of W = G*V dense columns; lane
//     gl of the group owns columns [slab*W + gl*V, +V) and loads them with one
//     V-wide vector load per nonzero (16 B for fp32 V=4 / bf16 V=8), so one
//     group reads one W-column segment of a B row per nonzero, coalesced.
//   * blockIdx.y walks the column slabs.  CTAs are dispatched x-fastest, so the
//     GPU sweeps slab 0 of every row before slab 1: the slab of B being gathered
//     (K x W) is what must stay in L2, not all of B.
//   * Index/value streams are loaded cooperatively (one nonzero per lane) and
//     broadcast with shuffles; up to 8 dense loads per lane are in flight
//     before the first multiply-add.
//
// Schedules (segTACO's 2x2 space, gpu_kernels.cuh:11-93):
//   rb_sr  row-balanced, sequential: one group per row, nonzeros summed in
//          storage order with fmaf.  (segTACO: spmm_rb_sr.h:187-243,351-535)
//   rb_pr  row-balanced, parallel: one warp per row, the P = 32/G groups take
//          interleaved nonzeros, then a shuffle tree combines them.
//          (segTACO: spmm_rb_pr.h:223-375,428-948)
//   eb_sr  element-balanced, sequential: one group per merge-path chunk of D
//          items (row ends + nonzeros), walked in merge order.
//          (segTACO: spmm_eb_sr.h:153-423,856-1096)
//   eb_pr  element-balanced, parallel: one warp per merge-path chunk; each step
//          gives one nonzero to each group and a segmented suffix scan across
//          the groups (keyed by row) reduces them; a running carry joins rows
//          that span steps.  (segTACO: spmm_eb_pr.h:281-480,482-779)
//
// Element-balanced chunks come from the merge-path split (partition.cu).  A row
// whose nonzeros straddle a chunk edge is zeroed by the partition kernel and
// receives red.global.add from each chunk that holds part of it; every other
// row is written once with a plain store.  So C needs no memset and atomics
// happen only at partition edges.
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
  long long units;                 // rb: rows per group/warp; eb: number of chunks
  int l2_hints;                    // 1: gathered B rows evict_last in L2
};

template <int V> __device__ __forceinline__ void zero(float (&a)[V]) {
#pragma unroll
  for (int v = 0; v < V; ++v) a[v] = 0.0f;
}

__device__ __forceinline__ float ld_val(const float *__restrict__ val, int q) {
  return val ? ld_stream(val + q) : 1.0f;
}

// ===========================================================================
// rb_sr
// ===========================================================================
template <typename BT, int V, int G>
__global__ void __launch_bounds__(kCta) spmm_rb_sr_kernel(SpmmArgs<BT> a) {
  constexpr int NB = G >= 8 ? G : 8;  // nonzeros per index batch
  constexpr int IPL = NB / G;         // index registers per lane
  constexpr int U = 8;                // dense loads in flight per lane
  const int lane = threadIdx.x & 31;
  const int gl = lane & (G - 1);
  const unsigned gmask = group_mask<G>(lane);
  const long long group = (long long)blockIdx.x * (kCta / G) + threadIdx.x / G;
  const int col0 = blockIdx.y * (G * V) + gl * V;
  const bool active = col0 < a.N;
  const uint64_t pol = l2_policy(a.l2_hints);
  const BT *Bc = a.B + col0;
  long long r = group * a.units;
  const long long r_end = min(r + a.units, (long long)a.M);
  for (; r < r_end; ++r) {
    const int p0 = __ldg(a.row_ptr + r), p1 = __ldg(a.row_ptr + r + 1);
    float acc[V];
    zero<V>(acc);
    for (int p = p0; p < p1; p += NB) {
      const int nb = imin(NB, p1 - p);
      int mc[IPL];
      float mv[IPL];
#pragma unroll
      for (int k = 0; k < IPL; ++k) {
        const int t = k * G + gl;
        mc[k] = t < nb ? ld_stream(a.col + p + t) : 0;
        mv[k] = t < nb ? ld_val(a.val, p + t) : 0.0f;
      }
#pragma unroll
      for (int t0 = 0; t0 < NB; t0 += U) {
        if (t0 >= nb) break;
        float b[U][V];
        float vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int t = t0 + u;
          const int j = __shfl_sync(gmask, mc[t / G], t % G, G);
          vv[u] = __shfl_sync(gmask, mv[t / G], t % G, G);
          if (t < nb && active)
            DenseLoad<BT, V, true>::run(Bc + (long long)j * a.ldb, b[u], pol);
          else
            zero<V>(b[u]);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (t0 + u < nb) {
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], b[u][v], acc[v]);
          }
        }
      }
    }
    if (active) store_c<V>(a.C + r * a.ldc + col0, acc);
  }
}

// ===========================================================================
// rb_pr
// ===========================================================================
template <typename BT, int V, int G>
__global__ void __launch_bounds__(kCta) spmm_rb_pr_kernel(SpmmArgs<BT> a) {
  constexpr int P = 32 / G;           // groups per warp = nonzeros combined in parallel
  constexpr int U = G < 8 ? G : 8;    // dense loads in flight per lane
  const int lane = threadIdx.x & 31;
  const int g = lane / G, gl = lane & (G - 1);
  const long long warp = (long long)blockIdx.x * (kCta / 32) + threadIdx.x / 32;
  const int col0 = blockIdx.y * (G * V) + gl * V;
  const bool active = col0 < a.N;
  const uint64_t pol = l2_policy(a.l2_hints);
  const BT *Bc = a.B + col0;
  long long r = warp * a.units;
  const long long r_end = min(r + a.units, (long long)a.M);
  for (; r < r_end; ++r) {
    const int p0 = __ldg(a.row_ptr + r), p1 = __ldg(a.row_ptr + r + 1);
    float acc[V];
    zero<V>(acc);
    for (int p = p0; p < p1; p += 32) {
      const int nb = imin(32, p1 - p);
      const int mc = lane < nb ? ld_stream(a.col + p + lane) : 0;
      const float mv = lane < nb ? ld_val(a.val, p + lane) : 0.0f;
      // group g takes nonzeros t = g + P*k, k = 0..G-1
#pragma unroll
      for (int k0 = 0; k0 < G; k0 += U) {
        if (P * k0 >= nb) break;
        float b[U][V];
        float vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int t = g + P * (k0 + u);
          const int j = __shfl_sync(0xffffffffu, mc, t);
          vv[u] = __shfl_sync(0xffffffffu, mv, t);
          if (t < nb && active)
            DenseLoad<BT, V, true>::run(Bc + (long long)j * a.ldb, b[u], pol);
          else
            zero<V>(b[u]);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
          for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], b[u][v], acc[v]);
        }
      }
    }
#pragma unroll
    for (int o = G; o < 32; o <<= 1) {
#pragma unroll
      for (int v = 0; v < V; ++v) acc[v] += __shfl_xor_sync(0xffffffffu, acc[v], o);
    }
    if (g == 0 && active) store_c<V>(a.C + r * a.ldc + col0, acc);
  }
}

// ===========================================================================
// eb_sr
// ===========================================================================
template <typename BT, int V, int G>
__global__ void __launch_bounds__(kCta) spmm_eb_sr_kernel(SpmmArgs<BT> a) {
  constexpr int NB = G >= 8 ? G : 8;
  constexpr int IPL = NB / G;
  constexpr int U = 8;
  const int lane = threadIdx.x & 31;
  const int gl = lane & (G - 1);
  const unsigned gmask = group_mask<G>(lane);
  const long long c = (long long)blockIdx.x * (kCta / G) + threadIdx.x / G;
  if (c >= a.units) return;  // whole group leaves together
  const int col0 = blockIdx.y * (G * V) + gl * V;
  const bool active = col0 < a.N;
  const uint64_t pol = l2_policy(a.l2_hints);
  const BT *Bc = a.B + col0;
  const int M = a.M;
  const int x0 = __ldg(a.part_x + c), y0 = __ldg(a.part_y + c);
  const int x1 = __ldg(a.part_x + c + 1), y1 = __ldg(a.part_y + c + 1);
  const bool head_split = x0 < M && __ldg(a.row_ptr + x0) < y0;

  // Window of row ends: lane gl holds row_ptr[wb + 1 + gl] (INT_MAX past row M-1).
  int row = x0, wb = x0;
  int rw = (wb + gl < M) ? __ldg(a.row_ptr + wb + 1 + gl) : INT_MAX;
  int rend = __shfl_sync(gmask, rw, 0, G);
  bool dirty = false;  // acc holds contributions of the current row
  float acc[V];
  zero<V>(acc);

  // Write the finished row `row` and step to the next one.
#define SEGTACO_EB_SR_FLUSH()                                                         \
  do {                                                                                \
    if (active) {                                                                     \
      float *dst = a.C + (long long)row * a.ldc + col0;                              \
      if (row == x0 && head_split) {                                                  \
        if (dirty) atomic_add_c<V>(dst, acc);                                         \
      } else {                                                                        \
        store_c<V>(dst, acc);                                                         \
      }                                                                               \
    }                                                                                 \
    zero<V>(acc);                                                                     \
    dirty = false;                                                                    \
    ++row;                                                                            \
    if (row - wb == G) {                                                              \
      wb = row;                                                                       \
      rw = (wb + gl < M) ? __ldg(a.row_ptr + wb + 1 + gl) : INT_MAX;                 \
    }                                                                                 \
    rend = __shfl_sync(gmask, rw, row - wb, G);                                       \
  } while (0)

  for (int p = y0; p < y1; p += NB) {
    const int nb = imin(NB, y1 - p);
    int mc[IPL];
    float mv[IPL];
#pragma unroll
    for (int k = 0; k < IPL; ++k) {
      const int t = k * G + gl;
      mc[k] = t < nb ? ld_stream(a.col + p + t) : 0;
      mv[k] = t < nb ? ld_val(a.val, p + t) : 0.0f;
    }
#pragma unroll
    for (int t0 = 0; t0 < NB; t0 += U) {
      if (t0 >= nb) break;
      float b[U][V];
      float vv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int t = t0 + u;
        const int j = __shfl_sync(gmask, mc[t / G], t % G, G);
        vv[u] = __shfl_sync(gmask, mv[t / G], t % G, G);
        if (t < nb && active)
          DenseLoad<BT, V, true>::run(Bc + (long long)j * a.ldb, b[u], pol);
        else
          zero<V>(b[u]);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (t0 + u < nb) {
          const int q = p + t0 + u;
          while (rend <= q) SEGTACO_EB_SR_FLUSH();
#pragma unroll
          for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], b[u][v], acc[v]);
          dirty = true;
        }
      }
    }
  }
  while (row < x1) SEGTACO_EB_SR_FLUSH();
#undef SEGTACO_EB_SR_FLUSH
  // Row x1 is unfinished in this chunk: its partial sum goes out by reduction.
  if (dirty && active && row < M) atomic_add_c<V>(a.C + (long long)row * a.ldc + col0, acc);
}

// ===========================================================================
// eb_pr
// ===========================================================================
// Row of nonzero q by bisection over row_ptr[lo..hi] (slow path, used when the
// 32-row window does not cover a batch, i.e. long runs of empty rows).
__device__ __forceinline__ int row_of(const int *__restrict__ row_ptr, int lo, int hi, int q) {
  // last r in [lo, hi] with row_ptr[r] <= q
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(row_ptr + mid) <= q)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

template <typename BT, int V, int G>
__global__ void __launch_bounds__(kCta) spmm_eb_pr_kernel(SpmmArgs<BT> a) {
  constexpr int P = 32 / G;          // nonzeros per step (one per group)
  constexpr int S = G;               // steps per batch of 32 nonzeros
  constexpr int U = S < 8 ? S : 8;   // steps whose dense loads are in flight together
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int g = lane / G, gl = lane & (G - 1);
  const long long c = (long long)blockIdx.x * (kCta / 32) + threadIdx.x / 32;
  if (c >= a.units) return;  // whole warp leaves together
  const int col0 = blockIdx.y * (G * V) + gl * V;
  const bool active = col0 < a.N;
  const uint64_t pol = l2_policy(a.l2_hints);
  const BT *Bc = a.B + col0;
  const int M = a.M;
  const int x0 = __ldg(a.part_x + c), y0 = __ldg(a.part_y + c);
  const int x1 = __ldg(a.part_x + c + 1), y1 = __ldg(a.part_y + c + 1);
  const bool head_split = x0 < M && __ldg(a.row_ptr + x0) < y0;

  // 1. Empty rows finished in this chunk are written as zeros.
  for (int r0 = x0; r0 < x1; r0 += 32) {
    const int r = r0 + lane;
    bool empty = false;
    if (r < x1) empty = __ldg(a.row_ptr + r) == __ldg(a.row_ptr + r + 1);
    unsigned em = __ballot_sync(FULL, empty);
    while (em) {
      const int src = __ffs(em) - 1;
      em &= em - 1;
      if (active) {
        float z[V];
        zero<V>(z);
        store_c<V>(a.C + (long long)(r0 + src) * a.ldc + col0, z);
      }
    }
  }

  // 2. Nonzeros.  Window: lane l holds the end of row wb + l.
  int wb = x0;
  int rw = (wb + lane < M) ? __ldg(a.row_ptr + wb + 1 + lane) : INT_MAX;
  int carry_row = -1;
  float carry[V];
  zero<V>(carry);
  for (int p = y0; p < y1; p += 32) {
    const int nb = imin(32, y1 - p);
    const int mc = lane < nb ? ld_stream(a.col + p + lane) : 0;
    const float mv = lane < nb ? ld_val(a.val, p + lane) : 0.0f;
    // Re-base the window on the row of nonzero p.
    for (;;) {
      const int adv = __popc(__ballot_sync(FULL, rw <= p));
      if (adv == 0) break;
      wb += adv;
      rw = (wb + lane < M) ? __ldg(a.row_ptr + wb + 1 + lane) : INT_MAX;
    }
    const bool covered = __shfl_sync(FULL, rw, 31) > p + nb - 1;
#pragma unroll
    for (int s0 = 0; s0 < S; s0 += U) {
      if (s0 * P >= nb) break;
      float b[U][V];
      float vv[U];
      int rq[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int t = (s0 + u) * P + g;  // this group's nonzero in step s0+u
        const int j = __shfl_sync(FULL, mc, t);
        vv[u] = __shfl_sync(FULL, mv, t);
        if (t < nb && active)
          DenseLoad<BT, V, true>::run(Bc + (long long)j * a.ldb, b[u], pol);
        else
          zero<V>(b[u]);
        int r = INT_MAX;
        if (covered) {
#pragma unroll
          for (int gg = 0; gg < P; ++gg) {
            const unsigned bal = __ballot_sync(FULL, rw <= p + (s0 + u) * P + gg);
            if (g == gg) r = wb + __popc(bal);
          }
        } else if (t < nb) {
          r = row_of(a.row_ptr, wb, x1 < M ? x1 : M - 1, p + t);
        }
        rq[u] = t < nb ? r : INT_MAX;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int s = s0 + u;
        if (s * P >= nb) break;
        const int row = rq[u];
        float prod[V];
#pragma unroll
        for (int v = 0; v < V; ++v) prod[v] = vv[u] * b[u][v];
        if (g == 0 && row == carry_row) {
#pragma unroll
          for (int v = 0; v < V; ++v) prod[v] += carry[v];
        }
        // Segmented suffix scan across groups: each segment head ends with the total.
#pragma unroll
        for (int d = 1; d < P; d <<= 1) {
          const int orow = __shfl_down_sync(FULL, row, d * G);
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const float o = __shfl_down_sync(FULL, prod[v], d * G);
            if (g + d < P && orow == row) prod[v] += o;
          }
        }
        const int prev = __shfl_up_sync(FULL, row, G);
        const bool is_head = row != INT_MAX && (g == 0 || prev != row);
        const int last_g = imin(P, nb - s * P) - 1;  // last group with a valid nonzero
        const int tail_row = __shfl_sync(FULL, row, last_g * G);
        const int q_last = p + s * P + last_g;
        bool tail_open;
        if (q_last + 1 < y1) {
          const int rend_tail = (covered && tail_row - wb < 32)
                                    ? __shfl_sync(FULL, rw, (tail_row - wb) & 31)
                                    : __ldg(a.row_ptr + tail_row + 1);
          tail_open = rend_tail > q_last + 1;
        } else {
          tail_open = tail_row == x1;  // row end of x1 belongs to the next chunk
        }
        if (is_head && !(row == tail_row && tail_open) && active) {
          float *dst = a.C + (long long)row * a.ldc + col0;
          if (row == x0 && head_split)
            atomic_add_c<V>(dst, prod);
          else
            store_c<V>(dst, prod);
        }
        // The head of the tail segment hands its total to group 0 as the carry.
        const unsigned heads = __ballot_sync(FULL, is_head && gl == 0);
        const int head_lane = 31 - __clz(heads);
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const float cv = __shfl_sync(FULL, prod[v], head_lane + gl);
          carry[v] = tail_open ? cv : 0.0f;
        }
        carry_row = tail_open ? tail_row : -1;
      }
    }
  }
  if (carry_row >= 0 && g == 0 && active)
    atomic_add_c<V>(a.C + (long long)carry_row * a.ldc + col0, carry);
}

}  // namespace segtaco
