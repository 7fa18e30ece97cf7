// spmm_kernels.cuh -- the segTACO SpMM schedules as one warp-uniform kernel.
//
// C = A * B, A CSR (M x K), B dense K x N row-major, C dense M x N row-major.
//
// Work layout.  A warp owns one unit of work and one column slab:
//   * unit  = a merge-path chunk of rows+nonzeros (element-balanced, eb_*) or a
//             block of R consecutive rows (row-balanced, rb_*);
//   * slab  = W = G*V dense columns (blockIdx.y), G lanes x V-wide vector loads
//             (16 B per lane for fp32 V=4 / bf16 V=8; 32 B, one
//             ld.global.v8, for fp32 V=8 / bf16 V=16 when B exceeds L2).
// The 32 lanes form P = 32/G slots of G lanes; a slot reads one W-column
// segment of one B row per step.  The warp walks the unit's rows in order and
// treats each row by its length (all control flow is warp-uniform):
//   * a row with >= 2P nonzeros (in this unit) is split over the slots: step k
//     gives slot s the nonzero k*P + s; batches of 32 nonzeros are aligned to
//     the row start, so the inner loop is multiply-adds only; at the row end
//     the slots' partial sums are folded with xor shuffles and slot 0 writes;
//   * a run of shorter rows is spread one row per slot (up to P rows whose
//     nonzeros fit one 32-nonzero batch); each slot sums its own row and
//     writes it, so short rows pay no fold.
// The next batch of column indices and values is always loaded (from the next
// row start) before the current one is used.
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
  int long_row;                    // rb: rows of >= long_row nonzeros are left to the
                                   // long-row CTAs or pieces (spmm_long.cu); 0: none
  // rb_pr: the first piece_cap warps of a row-block launch take the pieces of
  // the long rows, (row, first nonzero) pairs: piece_count[0] of rows of
  // several pieces from entry 0, piece_count[1] of one-piece rows from entry
  // piece_multi.  A piece of several stores its partial row (piece_ld floats)
  // and counts itself in piece_ctr[first piece of the row * slabs + slab]; the
  // last piece of a row sums the row's partials in piece order into C.
  // piece_parts > 1: the pieces run in a launch of their own (spmm_pieces_kernel),
  // pass p over the nonzeros whose columns lie in [p*Kp, (p+1)*Kp) (Kp = K /
  // piece_parts rounded up) of every piece, so that a pass gathers from that
  // range of B's rows only; each (piece, pass) leaves a partial row.
  const int2 *__restrict__ pieces;
  const int *__restrict__ piece_count;
  unsigned *piece_ctr;
  float *piece_part;
  long long piece_cap;
  long long piece_multi;
  long long piece_ld;
  int piece_len;
  int piece_parts;
  unsigned long long *piece_queue;  // the passes' work counter (cleared before the launch)
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

// Reduce-scatter form of fold_slots: at each xor level the lane keeps one half
// of its remaining values and trades the other half with its partner, so the
// P slots' sums end spread over the lanes (P = 8, V = 8: 7 shuffles instead of
// 24, one column per lane).  On return the lane holds the sums of its columns
// col0 + first .. col0 + first + R - 1 in r[0 .. R-1], R = fold_scatter_count.
// Where the values run out before the slots do (V < P), the last levels add
// whole values and only the lanes with a clear bit at those levels own the
// result (`owner`), so that each column is written once.
template <int G, int V> __host__ __device__ constexpr int fold_scatter_count() {
  int c = V;
  for (int o = G; o < 32; o <<= 1)
    if (c >= 2) c /= 2;
  return c;
}
template <int G, int V>
__device__ __forceinline__ int fold_slots_scatter(float (&r)[V], int lane, bool &owner) {
  int first = 0;
  int c = V;
  owner = true;
#pragma unroll
  for (int o = G; o < 32; o <<= 1) {
    const bool hi = (lane & o) != 0;
    if (c >= 2) {
      const int h = c / 2;
#pragma unroll
      for (int i = 0; i < V / 2; ++i) {
        if (i < h) {
          const float keep = hi ? r[i + h] : r[i];
          const float send = hi ? r[i] : r[i + h];
          r[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
      }
      if (hi) first += h;
      c = h;
    } else {
      r[0] += __shfl_xor_sync(0xffffffffu, r[0], o);
      if (hi) owner = false;
    }
  }
  return first;
}

// Store (or, at partition edges, add) R consecutive floats.
template <int R> __device__ __forceinline__ void put_c(float *p, const float *a, bool add) {
  if constexpr (R >= 4) {
#pragma unroll
    for (int k = 0; k < R; k += 4) {
      if (add)
        red_add4(p + k, a[k], a[k + 1], a[k + 2], a[k + 3]);
      else
        __stcs(reinterpret_cast<float4 *>(p + k), make_float4(a[k], a[k + 1], a[k + 2], a[k + 3]));
    }
  } else if constexpr (R == 2) {
    if (add)
      red_add2(p, a[0], a[1]);
    else
      __stcs(reinterpret_cast<float2 *>(p), make_float2(a[0], a[1]));
  } else {
    if (add)
      atomicAdd(p, a[0]);
    else
      __stcs(p, a[0]);
  }
}

// The end of a piece of a long row (rb_pr): its R sums of columns c0 .. c0+R-1
// (`mine`: this lane holds such columns) become the piece's partial row (in
// pass `pass` of piece_parts); the (piece, pass) of the row that counts
// itself last sums the row's partials in (piece, pass) order and stores them
// in C, so the result does not depend on which finishes first.  A row of one
// piece in one pass stores directly.  y0: the piece's first nonzero.
template <typename BT, int R>
__device__ __forceinline__ void finish_piece(const SpmmArgs<BT> &a, long long w, int row, int y0,
                                             int slab, int slabs, const float *acc, bool mine,
                                             int c0, int lane, int pass) {
  const int rs = __ldg(a.row_ptr + row), re = __ldg(a.row_ptr + row + 1);
  const int n = (re - rs + a.piece_len - 1) / a.piece_len;
  const int np = a.piece_parts;
  float *dst = a.C + (long long)row * a.ldc + c0;
  if (n == 1 && np == 1) {
    if (mine) put_c<R>(dst, acc, false);
    return;
  }
  const long long first = w - (y0 - rs) / a.piece_len;
  if (mine) {
    float *part = a.piece_part + (w * np + pass) * a.piece_ld + c0;
#pragma unroll
    for (int k = 0; k < R; ++k) __stcg(part + k, acc[k]);
  }
  __threadfence();
  __syncwarp();
  unsigned seen = 0;
  if (lane == 0) seen = atomicAdd(a.piece_ctr + first * slabs + slab, 1u);
  seen = __shfl_sync(0xffffffffu, seen, 0);
  if (seen != (unsigned)(n * np - 1)) return;
  __threadfence();
  // every piece of the row has counted itself: the counter is free again (a
  // later product may reuse the list)
  if (lane == 0) a.piece_ctr[first * slabs + slab] = 0u;
  if (mine) {
    float sum[R];
#pragma unroll
    for (int k = 0; k < R; ++k) sum[k] = 0.0f;
    for (long long q = first * np; q < (first + n) * np; ++q) {
      const float *part = a.piece_part + q * a.piece_ld + c0;
#pragma unroll
      for (int k = 0; k < R; ++k) sum[k] += __ldcg(part + k);
    }
    put_c<R>(dst, sum, false);
  }
}

// First position in [lo, hi) whose column is >= target (hi if none), searched
// by the whole warp: 32 probes per round narrow the range to one probe step.
// On a row whose columns are not sorted it still returns a position in [lo,
// hi], so the passes' ranges [b_p, b_p+1) still cover the piece exactly once.
__device__ __forceinline__ int warp_lower_bound(const int *__restrict__ col, int lo, int hi,
                                                long long target, int lane) {
  const unsigned FULL = 0xffffffffu;
  while (hi - lo > 32) {
    const long long step = (hi - lo + 31) / 32;
    const long long p = lo + lane * step;
    const bool ge = p >= hi || (long long)__ldg(col + p) >= target;
    const unsigned m = __ballot_sync(FULL, ge);
    if (m == 0u) {
      lo += (int)(31 * step + 1);  // every probe below target (p < hi for all lanes)
      continue;
    }
    const int f = __ffs(m) - 1;
    const long long nhi = lo + f * step;
    if (f > 0) lo = (int)(lo + (f - 1) * step + 1);
    hi = nhi < hi ? (int)nhi : hi;
  }
  const long long p = (long long)lo + lane;
  const bool ge = p < hi && (long long)__ldg(col + p) >= target;
  const unsigned m = __ballot_sync(FULL, ge);
  return m ? lo + __ffs(m) - 1 : hi;
}

// Rows [lo, lo + rows) of the current column slab of B staged in shared
// memory (W = G*V values per row): gathers of those rows read the copy.
template <typename BT> struct Window {
  const BT *base = nullptr;
  int lo = 0, rows = 0;
};

// Walk one unit (merge-path chunk or row block) `w` over column slab `slab`.
// The body of every SpMM kernel below (single problem or batched).
template <typename BT, int V, int G, bool ROWS, bool DEEP, bool WIN = false>
__device__ __forceinline__ void spmm_walk_unit(const SpmmArgs<BT> &a, long long w, int slab,
                                               int lane, Window<BT> win = Window<BT>()) {
  constexpr int P = 32 / G;                 // slots
  // Rows with >= LONG nonzeros are split over the slots (LONG <= 32, so a
  // short row always fits one batch).
  constexpr int LONG = P == 1 ? 0 : (2 * P < 32 ? 2 * P : 32);
  // B loads in flight per lane: 4 sixteen-byte or 8 narrower raw vectors.
  constexpr int UL = (V * (int)sizeof(BT) >= 16 && !DEEP) ? 4 : 8;
  constexpr int UB = G < UL ? G : UL;       // steps per sub-batch in a split row
  using D = Dense<BT, V>;
  const unsigned FULL = 0xffffffffu;
  const int slot = lane / G, gl = lane & (G - 1);
  const int M = a.M;
  const int col0 = slab * (G * V) + gl * V;
  const bool active = col0 < a.N;
  const uint64_t pol = l2_policy(a.l2_hints);
  // Inactive lanes (past N) still load, from column 0, so that no address is
  // out of bounds; their results are never stored.
  const BT *Bc = a.B + (active ? col0 : 0);
  const unsigned ldb = (unsigned)a.ldb;
  // B row slice j of this lane: from the staged window when it holds row j.
  auto gather = [&](int j) -> typename D::raw_t {
    if constexpr (WIN) {
      const unsigned d = (unsigned)(j - win.lo);
      if (d < (unsigned)win.rows) return D::lds(win.base + d * (G * V) + gl * V);
    }
    return D::load(Bc + (size_t)(unsigned)j * ldb, pol);
  };

  int x0, x1, y0, y1;
  bool head_split = false, tail_open = false;
  if (ROWS) {
    if (w < a.piece_cap) {
      // A piece of a long row: its nonzeros [y0, y1) walked like a merge-path
      // chunk inside one row, the sum left to finish_piece.
      if (w < a.piece_multi ? w >= (long long)__ldg(a.piece_count)
                            : w - a.piece_multi >= (long long)__ldg(a.piece_count + 1))
        return;
      const int2 pc = __ldg(a.pieces + w);
      x0 = x1 = pc.x;
      y0 = pc.y;
      y1 = min(pc.y + a.piece_len, __ldg(a.row_ptr + pc.x + 1));
      head_split = tail_open = true;
    } else {
      const long long r0 = (w - a.piece_cap) * a.rows_per_unit;
      x0 = (int)r0;
      x1 = (int)min(r0 + a.rows_per_unit, (long long)M);
      y0 = __ldg(a.row_ptr + x0);
      y1 = __ldg(a.row_ptr + x1);
    }
  } else {
    x0 = __ldg(a.part_x + w);
    y0 = __ldg(a.part_y + w);
    x1 = __ldg(a.part_x + w + 1);
    y1 = __ldg(a.part_y + w + 1);
    // Row x0 began in an earlier chunk; row x1 holds nonzeros here and ends in a later one.
    head_split = x0 < M && __ldg(a.row_ptr + x0) < y0;
    tail_open = x1 < M && __ldg(a.row_ptr + x1) < y1;
  }
  const int last = tail_open ? x1 : x1 - 1;  // rows of this unit: x0 .. last
  const bool piece = ROWS && tail_open;      // a piece of a long row (rb_pr)

  // Row ends: lane l holds the end of row wb + l (INT_MAX past the last row).
  int cur = x0, wb = x0;
  int rw = (wb + lane < M) ? __ldg(a.row_ptr + wb + 1 + lane) : INT_MAX;
  int cstart = y0;  // first nonzero of row `cur` inside this unit
  // Batch buffer: lane l holds nonzero cstart + l (0 / 0.0 past the unit).
  int mc = lane < y1 - cstart ? ld_stream(a.col + cstart + lane) : 0;
  float mv = lane < y1 - cstart ? ld_val(a.val, cstart + lane) : 0.0f;
  float acc[V];

  while (cur <= last) {
    if (cur - wb > 32 - P) {  // keep rows cur .. cur+P-1 inside the window
      wb = cur;
      rw = (wb + lane < M) ? __ldg(a.row_ptr + wb + 1 + lane) : INT_MAX;
    }
    const int rend = min(__shfl_sync(FULL, rw, cur - wb), y1);
    if constexpr (ROWS) {
      if (a.long_row > 0 && !piece && rend - cstart >= a.long_row) {
        // a long row: summed by the long-row CTAs; the batch buffer moves on
        cstart = rend;
        ++cur;
        mc = lane < y1 - cstart ? ld_stream(a.col + cstart + lane) : 0;
        mv = lane < y1 - cstart ? ld_val(a.val, cstart + lane) : 0.0f;
        continue;
      }
    }
    if (P == 1 || rend - cstart >= LONG || piece) {
      // ---- row `cur` split over the slots --------------------------------
      zero<V>(acc);
      int p0 = cstart;
      if constexpr (G == 1 && V * (int)sizeof(BT) <= 16) {
        // One lane per slot: lane l takes nonzeros p+l, p+l+32, ... of blocks
        // of 32*R directly (no shuffles), R gathers in flight, the next
        // block's indices loading meanwhile.
        constexpr int R = 4;
        if (rend - p0 >= 32 * R) {
          int jc[R];
          float vc[R];
#pragma unroll
          for (int b = 0; b < R; ++b) {
            jc[b] = ld_stream(a.col + p0 + lane + 32 * b);
            vc[b] = ld_val(a.val, p0 + lane + 32 * b);
          }
          while (p0 + 32 * R <= rend) {
            const int pn = p0 + 32 * R;
            const bool more = pn + 32 * R <= rend;
            int jn[R];
            float vn[R];
#pragma unroll
            for (int b = 0; b < R; ++b) {
              jn[b] = more ? ld_stream(a.col + pn + lane + 32 * b) : 0;
              vn[b] = more ? ld_val(a.val, pn + lane + 32 * b) : 0.0f;
            }
            typename D::raw_t bb[R];
#pragma unroll
            for (int b = 0; b < R; ++b) bb[b] = gather(jc[b]);
#pragma unroll
            for (int b = 0; b < R; ++b) {
#pragma unroll
              for (int v = 0; v < V; ++v) acc[v] = fmaf(vc[b], D::get(bb[b], v), acc[v]);
            }
#pragma unroll
            for (int b = 0; b < R; ++b) {
              jc[b] = jn[b];
              vc[b] = vn[b];
            }
            p0 = pn;
          }
          // the batch buffer restarts at p0
          mc = lane < y1 - p0 ? ld_stream(a.col + p0 + lane) : 0;
          mv = lane < y1 - p0 ? ld_val(a.val, p0 + lane) : 0.0f;
        }
      }
      for (int p = p0; p < rend; p += 32) {
        const int nb = rend - p < 32 ? rend - p : 32;
        const int nxt = p + 32 < rend ? p + 32 : rend;
        const int mcn = lane < y1 - nxt ? ld_stream(a.col + nxt + lane) : 0;
        const float mvn = lane < y1 - nxt ? ld_val(a.val, nxt + lane) : 0.0f;
        if (nb == 32) {
#pragma unroll
          for (int s0 = 0; s0 < G; s0 += UB) {
            typename D::raw_t b[UB];
            float vv[UB];
#pragma unroll
            for (int u = 0; u < UB; ++u) {
              const int t = (s0 + u) * P + slot;
              const int j = __shfl_sync(FULL, mc, t);
              vv[u] = __shfl_sync(FULL, mv, t);
              b[u] = gather(j);
            }
#pragma unroll
            for (int u = 0; u < UB; ++u) {
#pragma unroll
              for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], D::get(b[u], v), acc[v]);
            }
          }
        } else {
          for (int s0 = 0; s0 * P < nb; s0 += UB) {
            typename D::raw_t b[UB];
            float vv[UB];
#pragma unroll
            for (int u = 0; u < UB; ++u) {
              const int t = (s0 + u) * P + slot;
              const bool ok = t < nb;
              const int j = __shfl_sync(FULL, mc, ok ? t : 0);
              const float v = __shfl_sync(FULL, mv, ok ? t : 0);
              vv[u] = ok ? v : 0.0f;
              b[u] = gather(j);
            }
#pragma unroll
            for (int u = 0; u < UB; ++u) {
              if ((s0 + u) * P + slot < nb) {
#pragma unroll
                for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], D::get(b[u], v), acc[v]);
              }
            }
          }
        }
        mc = mcn;
        mv = mvn;
      }
      if constexpr (P > 1) {
        // the slots' sums, spread over the lanes: every lane writes its share
        bool owner;
        const int first = fold_slots_scatter<G, V>(acc, lane, owner);
        if (ROWS && piece) {
          finish_piece<BT, fold_scatter_count<G, V>()>(a, w, cur, y0, slab,
                                                       (a.N + G * V - 1) / (G * V), acc,
                                                       active && owner, col0 + first, lane, 0);
        } else if (active && owner) {
          const bool edge = (cur == x0 && head_split) || (cur == x1 && tail_open);
          constexpr int R = fold_scatter_count<G, V>();
          put_c<R>(a.C + (long long)cur * a.ldc + col0 + first, acc,
                                            edge);
        }
      } else if (ROWS && piece) {
        finish_piece<BT, V>(a, w, cur, y0, slab, (a.N + G * V - 1) / (G * V), acc, active, col0,
                            lane, 0);
      } else if (active) {
        float *dst = a.C + (long long)cur * a.ldc + col0;
        if ((cur == x0 && head_split) || (cur == x1 && tail_open))
          atomic_add_c<V>(dst, acc);
        else
          store_c<V>(dst, acc);
      }
      cstart = rend;
      ++cur;
    } else {
      // ---- short rows: slot s takes row cur + s -------------------------
      // Every lane takes part in every shuffle (r - wb <= 31 by the window rule).
      const int r = cur + slot;
      const int rw_r = __shfl_sync(FULL, rw, r - wb);
      const int rw_prev = __shfl_sync(FULL, rw, r - wb - 1 >= 0 ? r - wb - 1 : 0);
      const int e = r <= last ? min(rw_r, y1) : INT_MAX;
      const int prev_end = min(rw_prev, y1);
      const int sbeg = slot == 0 ? cstart : prev_end;
      const int len = e - sbeg;
      // Take the longest prefix of slots whose rows are short and fit the batch.
      const bool ok = r <= last && len < LONG && e - cstart <= 32;
      unsigned leaders = 0;
#pragma unroll
      for (int q = 0; q < P; ++q) leaders |= 1u << (q * G);
      const unsigned bad = ~__ballot_sync(FULL, ok) & leaders;
      int k = bad ? (__ffs(bad) - 1) / G : P;  // slot 0 always qualifies ...
      if (k < 1) k = 1;                        // ... and the walk must advance regardless
      const bool incl = slot < k;
      const int nxt = __shfl_sync(FULL, e, (k - 1) * G);
      const int mcn = lane < y1 - nxt ? ld_stream(a.col + nxt + lane) : 0;
      const float mvn = lane < y1 - nxt ? ld_val(a.val, nxt + lane) : 0.0f;
      const int mylen = incl ? len : 0;
      const int maxlen = (int)__reduce_max_sync(FULL, (unsigned)mylen);
      const int off = sbeg - cstart;
      zero<V>(acc);
      for (int k0 = 0; k0 < maxlen; k0 += UL) {
        typename D::raw_t b[UL];
        float vv[UL];
#pragma unroll
        for (int u = 0; u < UL; ++u) {
          const bool okk = k0 + u < mylen;
          const int t = okk ? off + k0 + u : 0;
          const int j = __shfl_sync(FULL, mc, t);
          const float v = __shfl_sync(FULL, mv, t);
          vv[u] = okk ? v : 0.0f;
          b[u] = gather(j);
        }
#pragma unroll
        for (int u = 0; u < UL; ++u) {
          if (k0 + u < mylen) {
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], D::get(b[u], v), acc[v]);
          }
        }
      }
      if (incl && active) {
        float *dst = a.C + (long long)r * a.ldc + col0;
        if ((r == x0 && head_split) || (r == x1 && tail_open)) {
          if (mylen > 0) atomic_add_c<V>(dst, acc);
        } else {
          store_c<V>(dst, acc);
        }
      }
      cur += k;
      cstart = nxt;
      mc = mcn;
      mv = mvn;
    }
  }
}

// Flat walk of one unit: the unit's nonzeros in batches of up to 32 (one per
// lane), each batch inside a window of 32 consecutive rows (lane i holds the
// end of row wb + i).  Slot s owns batch positions s*Q .. s*Q+Q-1 (Q = G) and
// sums them in order into `acc`, issuing all of its B loads of a sub-block (up
// to 8 per lane) before the first multiply-add, whatever the row lengths.  At
// a position that ends a row the slot writes its sum, except the first row end
// of slots s >= 1, whose row began in an earlier slot: that partial waits for
// a segmented scan over the slots (flag = the slot saw a row end, value = the
// slot's open sum), which also yields the carry of the row still open after
// the batch.  Slot 0 starts each batch from that carry, so with one slot
// (P = 1) every row is one sequential fmaf chain in storage order.  Empty rows
// of the unit are zeroed first, P rows at a time.
template <typename BT, int V, int G, bool ROWS>
__device__ __forceinline__ void spmm_flat_unit(const SpmmArgs<BT> &a, long long w, int slab,
                                               int lane) {
  constexpr int P = 32 / G;  // slots
  constexpr int Q = G;       // batch positions per slot
  constexpr int U = Q < 8 ? Q : 8;
  using D = Dense<BT, V>;
  const unsigned FULL = 0xffffffffu;
  const int slot = lane / G, gl = lane & (G - 1);
  const int M = a.M;
  const int col0 = slab * (G * V) + gl * V;
  const bool active = col0 < a.N;
  const uint64_t pol = l2_policy(a.l2_hints);
  const BT *Bc = a.B + (active ? col0 : 0);  // lanes past N load column 0, never store
  const unsigned ldb = (unsigned)a.ldb;

  int x0, x1, y0, y1, rp0;
  bool head_split = false, tail_open = false;
  if (ROWS) {
    const long long r0 = w * a.rows_per_unit;
    x0 = (int)r0;
    x1 = (int)min(r0 + a.rows_per_unit, (long long)M);
    y0 = rp0 = __ldg(a.row_ptr + x0);
    y1 = __ldg(a.row_ptr + x1);
  } else {
    x0 = __ldg(a.part_x + w);
    y0 = __ldg(a.part_y + w);
    x1 = __ldg(a.part_x + w + 1);
    y1 = __ldg(a.part_y + w + 1);
    rp0 = x0 < M ? __ldg(a.row_ptr + x0) : y0;
    head_split = rp0 < y0;
    tail_open = x1 < M && __ldg(a.row_ptr + x1) < y1;
  }
  const int last = tail_open ? x1 : x1 - 1;  // rows of this unit: x0 .. last
  // Window: lane i holds the end of row wb + i (INT_MAX past M).
  auto window = [&](int base) {
    return (base + lane < M) ? __ldg(a.row_ptr + base + 1 + lane) : INT_MAX;
  };
  int wb = x0;
  int rw = window(wb);
  int p0 = y0;
  int mc = lane < y1 - p0 ? ld_stream(a.col + p0 + lane) : 0;
  float mv = lane < y1 - p0 ? ld_val(a.val, p0 + lane) : 0.0f;
  float acc[V], head[V];
  zero<V>(acc);
  zero<V>(head);

  // ---- empty rows of the unit (row starts from the window) ----
  {
    int e = rw, before = rp0;
    for (int rb = x0; rb <= last; rb += 32) {
      if (rb != x0) e = window(rb);
      int sb = __shfl_up_sync(FULL, e, 1);
      if (lane == 0) sb = before;
      const bool empty = rb + lane <= last && e == sb;
      before = __shfl_sync(FULL, e, 31);
      unsigned m = __ballot_sync(FULL, empty);
      while (m) {  // slot s zeroes the s-th remaining empty row
        unsigned mm = m;
        int pos = -1;
#pragma unroll
        for (int q = 0; q < P; ++q) {
          const int b = __ffs(mm) - 1;
          if (q == slot) pos = b;
          mm &= mm - 1;
        }
        if (pos >= 0 && active) store_c<V>(a.C + (long long)(rb + pos) * a.ldc + col0, acc);
        m = mm;
      }
    }
  }

  // ---- nonzeros ----
  while (p0 < y1) {
    // The window must start at or before the row of p0 and contain it.
    int wend = __shfl_sync(FULL, rw, 31);
    while (wend <= p0) {  // every window row ends by p0: move on 32 rows
      wb += 32;
      rw = window(wb);
      wend = __shfl_sync(FULL, rw, 31);
    }
    // Batch: nonzeros p0 .. pe-1, all in rows of the window.
    int pe = p0 + 32;
    if (pe > y1) pe = y1;
    if (pe > wend) pe = wend;
    const int nb = pe - p0;
    const int mcn = lane < y1 - pe ? ld_stream(a.col + pe + lane) : 0;
    const float mvn = lane < y1 - pe ? ld_val(a.val, pe + lane) : 0.0f;
    // Window row of nonzero p0 + lane: the number of window rows ending <= it.
    const int p = p0 + lane;
    int rr = 0;
#pragma unroll
    for (int st = 16; st > 0; st >>= 1) {
      const int cand = __shfl_sync(FULL, rw, rr + st - 1);
      if (cand <= p) rr += st;
    }
    const int rend = __shfl_sync(FULL, rw, rr);
    // code: bit 0 = ends its row (valid positions only), bits 2.. = window row
    const int code = lane < nb ? (rr << 2) | (rend == p + 1 ? 1 : 0) : 0;

    if (slot != 0) zero<V>(acc);
    bool flushed = false;
    int hrow = 0;
    const int kend = nb < Q ? nb : Q;  // slot 0 holds the most valid positions
    // Sub-blocks of U positions, one after another (unrolling them would let
    // the compiler hoist every load of the batch and spill).
#pragma unroll 1
    for (int k0 = 0; k0 < kend; k0 += U) {
      typename D::raw_t b[U];
      // Positions past the batch (t >= nb) reload the batch's first B row
      // (a cache hit, no new traffic) and are never used.
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int t = slot * Q + k0 + u;
        const int j = __shfl_sync(FULL, mc, t < nb ? t : 0);
        b[u] = D::load(Bc + (size_t)(unsigned)j * ldb, pol);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int t = slot * Q + k0 + u;
        const float x = __shfl_sync(FULL, mv, t);
        const int cd = __shfl_sync(FULL, code, t);
        if (t < nb) {
#pragma unroll
          for (int v = 0; v < V; ++v) acc[v] = fmaf(x, D::get(b[u], v), acc[v]);
        }
        if (cd & 1) {
          const int row = wb + (cd >> 2);
          if (slot == 0 || flushed) {
            if (active) {
              float *dst = a.C + (long long)row * a.ldc + col0;
              if (!ROWS && ((row == x0 && head_split) || (row == x1 && tail_open)))
                atomic_add_c<V>(dst, acc);
              else
                store_c<V>(dst, acc);
            }
          } else {
#pragma unroll
            for (int v = 0; v < V; ++v) head[v] = acc[v];
            hrow = row;
          }
          flushed = true;
          zero<V>(acc);
        }
      }
    }
    if (P > 1) {
      // Inclusive segmented scan over slots: value = open sum, reset where a
      // slot saw a row end.
      float sc[V];
#pragma unroll
      for (int v = 0; v < V; ++v) sc[v] = acc[v];
      int f = flushed ? 1 : 0;
#pragma unroll
      for (int d = 1; d < P; d <<= 1) {
        const int fo = __shfl_up_sync(FULL, f, d * G);
        float o[V];
#pragma unroll
        for (int v = 0; v < V; ++v) o[v] = __shfl_up_sync(FULL, sc[v], d * G);
        if (slot >= d) {
          if (!f) {
#pragma unroll
            for (int v = 0; v < V; ++v) sc[v] += o[v];
          }
          f |= fo;
        }
      }
      // The first row end of slot s >= 1 closes the row open after slot s-1.
      float in[V];
#pragma unroll
      for (int v = 0; v < V; ++v) in[v] = __shfl_up_sync(FULL, sc[v], G);
      if (slot > 0 && flushed && active) {
#pragma unroll
        for (int v = 0; v < V; ++v) head[v] += in[v];
        float *dst = a.C + (long long)hrow * a.ldc + col0;
        if (!ROWS && ((hrow == x0 && head_split) || (hrow == x1 && tail_open)))
          atomic_add_c<V>(dst, head);
        else
          store_c<V>(dst, head);
      }
      // Carry of the row still open: the scan value of the last slot, to slot 0.
#pragma unroll
      for (int v = 0; v < V; ++v) acc[v] = __shfl_sync(FULL, sc[v], (P - 1) * G + gl);
    }
    p0 = pe;
    mc = mcn;
    mv = mvn;
  }
  // The row open at the unit's end continues in the next unit (tail_open).
  if (!ROWS && tail_open && slot == 0 && active)
    atomic_add_c<V>(a.C + (long long)x1 * a.ldc + col0, acc);
}

// Slot walk of merge-path chunks: slot s of warp w owns chunk w*P + s (its
// own row range and nonzero range) and walks it in merge order on its own --
// each step takes the slot's next nonzero, and a position at or past the end
// of the slot's current row first stores that row (and any empty rows after
// it).  A round trip issues U positions per slot (U * P per warp) whatever
// the row lengths, so short rows cost no more than long ones, and no fold is
// needed: each row of a chunk is one sequential fmaf chain in storage order
// (so it also serves the sequential schedule, eb_sr, on narrow slabs).  A row
// cut by a chunk edge is zeroed by the partition kernel and receives
// red.global.add from every chunk holding part of it.
//
// Per slot, row ends come from a window of G of them (lane g holds the end of
// row wr + g) and the next G, read one window ahead; the slot's U column
// indices and values of a round trip are one coalesced load by its lanes and
// reach the other lanes of the slot by shuffles of width G.
template <typename BT, int V, int G>
__device__ __forceinline__ void spmm_slot_unit(const SpmmArgs<BT> &a, long long w, int slab,
                                               int lane) {
  constexpr int P = 32 / G;  // slots (one chunk each)
  // Positions per slot per round trip: one per lane of the slot, at most 8
  // and at most 128 bytes of B in flight per lane.
  constexpr int UB_ = 128 / (V * (int)sizeof(BT)) < 1 ? 1 : 128 / (V * (int)sizeof(BT));
  constexpr int U = G < 8 ? (G < UB_ ? G : UB_) : (8 < UB_ ? 8 : UB_);
  using D = Dense<BT, V>;
  const unsigned FULL = 0xffffffffu;
  const int slot = lane / G, gl = lane & (G - 1);
  const unsigned smask = group_mask<G>(lane);
  const int M = a.M;
  const int col0 = slab * (G * V) + gl * V;
  const bool active = col0 < a.N;
  const uint64_t pol = l2_policy(a.l2_hints);
  const BT *Bc = a.B + (active ? col0 : 0);  // lanes past N load column 0, never store
  const unsigned ldb = (unsigned)a.ldb;

  const long long c = w * P + slot;
  const bool has = c < a.units;
  int x = 0, x1 = 0, y = 0, y1 = 0;
  if (has) {
    x = __ldg(a.part_x + c);
    y = __ldg(a.part_y + c);
    x1 = __ldg(a.part_x + c + 1);
    y1 = __ldg(a.part_y + c + 1);
  }
  // Row x began in an earlier chunk; row x1 holds nonzeros here and ends later.
  const bool head_split = has && x < M && __ldg(a.row_ptr + x) < y;
  const bool tail_open = has && x1 < M && __ldg(a.row_ptr + x1) < y1;
  auto rp = [&](long long i) -> int { return i <= M ? __ldg(a.row_ptr + i) : INT_MAX; };
  int wr = x;                            // lane gl: end of row wr + gl
  int rw_cur = has ? rp((long long)wr + 1 + gl) : INT_MAX;
  int rw_nxt = has ? rp((long long)wr + 1 + G + gl) : INT_MAX;
  // End of row r (r >= wr; the slot's lanes move together).
  auto row_end = [&](int r) -> int {
    while (r - wr >= G) {
      wr += G;
      rw_cur = rw_nxt;
      rw_nxt = rp((long long)wr + 1 + G + gl);
    }
    return __shfl_sync(smask, rw_cur, r - wr, G);
  };
  float acc[V];
  zero<V>(acc);
  auto flush = [&](int r) {
    if (active) {
      float *dst = a.C + (long long)r * a.ldc + col0;
      if ((r == x && head_split) || (r == x1 && tail_open))
        atomic_add_c<V>(dst, acc);
      else
        store_c<V>(dst, acc);
    }
    zero<V>(acc);
  };
  int row = x;
  int rend = has ? row_end(row) : INT_MAX;
  int p = y;
  for (;;) {
    const bool more = has && p < y1;
    if (!__any_sync(FULL, more)) break;
    // The slot's next U column indices and values (lane gl < U: position p + gl).
    const int q = p + gl;
    const bool okq = more && gl < U && q < y1;
    const int mc = okq ? ld_stream(a.col + q) : 0;
    const float mv = okq ? ld_val(a.val, q) : 0.0f;
    typename D::raw_t b[U];
    float vv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int j = __shfl_sync(FULL, mc, u, G);
      vv[u] = __shfl_sync(FULL, mv, u, G);
      b[u] = D::load(Bc + (size_t)(unsigned)j * ldb, pol);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int pos = p + u;
      if (more && pos < y1) {
        while (pos >= rend) {  // rows ending before this position (empty ones too)
          flush(row);
          ++row;
          rend = row_end(row);
        }
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], D::get(b[u], v), acc[v]);
      }
    }
    p += U;
  }
  if (has) {
    // Rows that end inside the chunk after its last nonzero (empty or not),
    // then the row still open at the chunk's end.
    while (row < x1) {
      flush(row);
      ++row;
    }
    if (tail_open) flush(x1);
  }
}

// Sequential walk of a merge-path chunk for 8-byte lanes (eb_sr with bf16 B
// over 128-column slabs, or fp32 over 64): the warp is one slot and walks the
// chunk's nonzeros in storage order, every column of a row one fmaf chain, as
// the flat walk does for 16-byte lanes.  Instead of two shuffles per gather
// (index and value), the chunk's indices and values are staged in shared
// memory by coalesced loads (kSeqStage at a time) and each step reads four of
// them with one broadcast 16-byte shared load per array, then issues U
// gathers before the first multiply-add.  Control flow is warp-uniform: row
// ends come from a window of 32 row ends in the lanes.  A row cut by a chunk
// edge is zeroed by the partition kernel and receives red.global.add from each
// chunk holding part of it.  Measured on GB300 (1M x 1M power law, N = 128):
// bf16 eb_sr 0.840 -> 0.819 ms against the row walk, fp32 at 64 columns 1.500
// -> 1.472 ms (the flat walk over 128 columns stays the fp32 default, 1.434
// ms).  With 4-byte lanes (one fp32 column per lane, 32-column slabs) it took
// 2.55 ms at 16 gathers in flight (32 spill): a gather then brings only 128
// bytes per warp, so the walk is bound by its per-position work.
constexpr int kSeqStage = 512;
template <typename BT, int V> __host__ __device__ constexpr int seq_loads() { return 8; }
template <typename BT, int V>
__device__ __forceinline__ void spmm_seq_unit(const SpmmArgs<BT> &a, long long w, int slab,
                                              int lane, int *__restrict__ cs,
                                              float *__restrict__ vs) {
  constexpr int U = seq_loads<BT, V>();
  using D = Dense<BT, V>;
  const unsigned FULL = 0xffffffffu;
  const int M = a.M;
  const int col0 = slab * (32 * V) + lane * V;
  const bool active = col0 < a.N;
  const uint64_t pol = l2_policy(a.l2_hints);
  const BT *Bc = a.B + (active ? col0 : 0);  // lanes past N load column 0, never store
  const unsigned ldb = (unsigned)a.ldb;

  const int x0 = __ldg(a.part_x + w), y0 = __ldg(a.part_y + w);
  const int x1 = __ldg(a.part_x + w + 1), y1 = __ldg(a.part_y + w + 1);
  // Row x0 began in an earlier chunk; row x1 holds nonzeros here and ends later.
  const bool head_split = x0 < M && __ldg(a.row_ptr + x0) < y0;
  const bool tail_open = x1 < M && __ldg(a.row_ptr + x1) < y1;
  int wb = x0;  // lane l: end of row wb + l
  int rw = wb + lane < M ? __ldg(a.row_ptr + wb + 1 + lane) : INT_MAX;
  auto row_end = [&](int r) -> int {
    while (r - wb >= 32) {
      wb += 32;
      rw = wb + lane < M ? __ldg(a.row_ptr + wb + 1 + lane) : INT_MAX;
    }
    return __shfl_sync(FULL, rw, r - wb);
  };
  float acc[V];
  zero<V>(acc);
  auto flush = [&](int r) {
    if (active) {
      float *dst = a.C + (long long)r * a.ldc + col0;
      if ((r == x0 && head_split) || (r == x1 && tail_open))
        atomic_add_c<V>(dst, acc);
      else
        store_c<V>(dst, acc);
    }
    zero<V>(acc);
  };
  int row = x0;
  int rend = row_end(row);  // INT_MAX past the last row
  int base = 0, lim = -1;  // staged nonzeros [base, lim), base a multiple of 4
  int p = y0;
  while (p < y1) {
    if (p >= lim) {
      __syncwarp();
      base = p & ~3;
      lim = min(base + kSeqStage, y1);
      for (int k = lane; k < lim - base; k += 32) {
        cs[k] = ld_stream(a.col + base + k);
        vs[k] = ld_val(a.val, base + k);
      }
      __syncwarp();
    }
    // Positions g .. g+U-1 of this step (g a multiple of 4); those in [p, end)
    // are this chunk's, the others load B row 0 (a cache hit) and are unused.
    const int g = p & ~3;
    const int end = min(g + U, lim);
    const int o = g - base;
    typename D::raw_t b[U];
#pragma unroll
    for (int j = 0; j < U / 4; ++j) {
      const int4 c4 = *reinterpret_cast<const int4 *>(cs + o + 4 * j);
      const int cc[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int pos = g + 4 * j + k;
        const int col = pos >= p && pos < end ? cc[k] : 0;
        b[4 * j + k] = D::load(Bc + (size_t)(unsigned)col * ldb, pol);
      }
    }
#pragma unroll
    for (int j = 0; j < U / 4; ++j) {
      const float4 v4 = *reinterpret_cast<const float4 *>(vs + o + 4 * j);
      const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int pos = g + 4 * j + k;
        if (pos >= p && pos < end) {
          while (pos >= rend) {  // rows ending before this position (empty ones too)
            flush(row);
            ++row;
            rend = row_end(row);
          }
#pragma unroll
          for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[k], D::get(b[4 * j + k], v), acc[v]);
        }
      }
    }
    p = end;
  }
  // Rows that end inside the chunk after its last nonzero (empty or not), then
  // the row still open at the chunk's end.
  while (row < x1) {
    flush(row);
    ++row;
  }
  if (tail_open) flush(x1);
}

// Walks of a unit: the row walk with 4 or 8 loads in flight per lane, the
// flat walk, the slot walk or the sequential walk over merge-path chunks
// (chosen by the planner, api.cu).
constexpr int kWalkRows = 0, kWalkRowsDeep = 1, kWalkFlat = 2, kWalkSlots = 3, kWalkSeq = 4;

// CTAs of the SpMM kernels: 4 warps each, so a CTA that finishes early frees
// its slot soon (warps of a CTA walk units of uneven cost).  32 warps per SM
// at most 64 registers, except the variants that need more (spmm_min_ctas).
constexpr int kSpmmCta = 128;
constexpr int kSpmmWarps = kSpmmCta / 32;
template <int V, int G, bool HEAVY> constexpr int spmm_min_ctas() {
  // 8-element lanes fit 64 registers only for G <= 4 (the autotuned W = 32
  // case; ptxas: fp32 V = 8, G = 4 spills 4 bytes, measured faster than 24
  // warps without the spill); wider groups, the flat walk with 8-element
  // lanes and the deep row walk take 24 warps.
  return ((HEAVY || (V == 8 && G > 4) || V == 16) ? 24 : 32) / kSpmmWarps;
}

// One pass of one piece of a long row (rb_pr, spmm_pieces_pass): the row's
// nonzeros [b_pass, b_pass+1) of the piece, split over the P = 32/G slots in
// batches of 32 (slot s takes batch positions s, s+P, ...), 4 sixteen-byte
// or wider loads (8 narrower ones) in flight per lane, the next batch's
// indices loading meanwhile; then the slots' sums folded and left to
// finish_piece.  The same arithmetic as the row walk's split path, without
// its row bookkeeping.
template <typename BT, int V, int G>
__device__ __forceinline__ void spmm_piece_unit(const SpmmArgs<BT> &a, long long w, int slab,
                                                int lane, int pass) {
  constexpr int P = 32 / G;
  constexpr int UL = V * (int)sizeof(BT) >= 16 ? 4 : 8;
  constexpr int UB = G < UL ? G : UL;  // steps of a batch in flight per lane
  using D = Dense<BT, V>;
  const unsigned FULL = 0xffffffffu;
  const int slot = lane / G, gl = lane & (G - 1);
  const int col0 = slab * (G * V) + gl * V;
  const bool active = col0 < a.N;
  const uint64_t pol = l2_policy(a.l2_hints);
  const BT *Bc = a.B + (active ? col0 : 0);  // lanes past N load column 0, never store
  const unsigned ldb = (unsigned)a.ldb;
  if (w < a.piece_multi ? w >= (long long)__ldg(a.piece_count)
                        : w - a.piece_multi >= (long long)__ldg(a.piece_count + 1))
    return;
  const int2 pc = __ldg(a.pieces + w);
  const int row = pc.x;
  int y0 = pc.y;
  int y1 = min(pc.y + a.piece_len, __ldg(a.row_ptr + row + 1));
  if (a.piece_parts > 1) {
    const long long Kp = ((long long)a.K + a.piece_parts - 1) / a.piece_parts;
    for (int q = 1; q <= pass; ++q) y0 = warp_lower_bound(a.col, y0, y1, q * Kp, lane);
    if (pass + 1 < a.piece_parts) y1 = warp_lower_bound(a.col, y0, y1, (pass + 1) * Kp, lane);
  }
  float acc[V];
  zero<V>(acc);
  int mc = lane < y1 - y0 ? ld_stream(a.col + y0 + lane) : 0;
  float mv = lane < y1 - y0 ? ld_val(a.val, y0 + lane) : 0.0f;
  for (int p = y0; p < y1; p += 32) {
    const int nb = y1 - p < 32 ? y1 - p : 32;
    const int nxt = p + 32;
    const int mcn = lane < y1 - nxt ? ld_stream(a.col + nxt + lane) : 0;
    const float mvn = lane < y1 - nxt ? ld_val(a.val, nxt + lane) : 0.0f;
#pragma unroll
    for (int s0 = 0; s0 < G; s0 += UB) {
      if (s0 * P >= nb) break;  // warp-uniform
      typename D::raw_t b[UB];
      float vv[UB];
#pragma unroll
      for (int u = 0; u < UB; ++u) {
        const int t = (s0 + u) * P + slot;
        const bool ok = t < nb;
        const int j = __shfl_sync(FULL, mc, ok ? t : 0);
        const float v = __shfl_sync(FULL, mv, ok ? t : 0);
        vv[u] = ok ? v : 0.0f;
        b[u] = D::load(Bc + (size_t)(unsigned)j * ldb, pol);
      }
#pragma unroll
      for (int u = 0; u < UB; ++u) {
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v] = fmaf(vv[u], D::get(b[u], v), acc[v]);
      }
    }
    mc = mcn;
    mv = mvn;
  }
  bool owner;
  const int first = fold_slots_scatter<G, V>(acc, lane, owner);
  finish_piece<BT, fold_scatter_count<G, V>()>(a, w, row, pc.y, slab,
                                               (a.N + G * V - 1) / (G * V), acc,
                                               active && owner, col0 + first, lane, pass);
}

// rb_pr's pieces in piece_parts passes (a launch of their own, before the row
// blocks): items (pass, slab, piece) in that order, each warp taking the next
// item from a counter, so that the grid works through one (pass, slab) at a
// time and its gathers stay within one range of B's rows of one slab (Kp x W
// elements) while it runs.
template <typename BT, int V, int G>
__device__ __forceinline__ void spmm_pieces_pass(const SpmmArgs<BT> &a, int lane) {
  const long long n0 = min((long long)__ldg(a.piece_count), a.piece_multi);
  const long long n1 = min((long long)__ldg(a.piece_count + 1), a.piece_cap - a.piece_multi);
  const long long total = n0 + n1;
  const long long slabs = (a.N + G * V - 1) / (G * V);
  const unsigned long long items = (unsigned long long)(total * slabs * a.piece_parts);
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(a.piece_queue, 1ull);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= items) return;
    const long long i = (long long)(t % (unsigned long long)total);
    const long long ps = (long long)(t / (unsigned long long)total);
    spmm_piece_unit<BT, V, G>(a, i < n0 ? i : a.piece_multi + (i - n0), (int)(ps % slabs), lane,
                              (int)(ps / slabs));
  }
}

// The pieces' passes as a kernel of their own: a persistent grid of
// spmm_min_ctas CTAs per multiprocessor (the row blocks' occupancy).
template <typename BT, int V, int G>
__global__ void __launch_bounds__(kSpmmCta, spmm_min_ctas<V, G, false>())
    spmm_pieces_kernel(SpmmArgs<BT> a) {
  spmm_pieces_pass<BT, V, G>(a, threadIdx.x & 31);
}

template <typename BT, int V, int G, bool ROWS, int WALK = kWalkRows>
__global__ void __launch_bounds__(kSpmmCta, spmm_min_ctas<V, G, WALK == kWalkRowsDeep ||
                                                                  (WALK == kWalkFlat && V == 8)>())
    spmm_seg_kernel(SpmmArgs<BT> a) {
  const long long w = (long long)blockIdx.x * kSpmmWarps + threadIdx.x / 32;
  if constexpr (WALK == kWalkSlots) {  // a.units chunks, 32 / G per warp
    if (w * (32 / G) >= a.units) return;
    spmm_slot_unit<BT, V, G>(a, w, blockIdx.y, threadIdx.x & 31);
    return;
  }
  if constexpr (WALK == kWalkSeq) {  // merge-path chunks, one per warp
    __shared__ __align__(16) int s_col[kSpmmWarps][kSeqStage + seq_loads<BT, V>()];
    __shared__ __align__(16) float s_val[kSpmmWarps][kSeqStage + seq_loads<BT, V>()];
    if (w >= a.units) return;
    const int wi = threadIdx.x / 32;
    spmm_seq_unit<BT, V>(a, w, blockIdx.y, threadIdx.x & 31, s_col[wi], s_val[wi]);
    return;
  }
  if (w >= a.units + a.piece_cap) return;  // whole warp leaves together
  if (WALK == kWalkFlat)
    spmm_flat_unit<BT, V, G, ROWS>(a, w, blockIdx.y, threadIdx.x & 31);
  else
    spmm_walk_unit<BT, V, G, ROWS, WALK == kWalkRowsDeep>(a, w, blockIdx.y, threadIdx.x & 31);
}

}  // namespace segtaco
