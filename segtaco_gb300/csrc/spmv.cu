// spmv.cu -- y = A x by merge path (the N = 1 form of the element-balanced
// schedule; segTACO's element-balanced SpMV is spmv_csr_gpu_taco.h:4-100).
//
// One CTA takes one merge-path tile of kTile = 256 x 8 items (row ends +
// nonzeros).  It stages the tile's row ends and its products a_p * x[col_p]
// in shared memory with coalesced loads (the x gathers hit L2: x is K floats),
// then every thread walks 8 merge items sequentially.  Rows that end inside a
// thread after its first row end are stored into shared row slots directly;
// the partials that cross thread boundaries are combined by a warp segmented
// scan, so a row spanning the tile costs one shared atomic per warp, not one
// per thread.  Rows wholly inside the tile are stored once to y; the two rows
// that straddle the tile edges were zeroed by the partition kernel and get a
// reduction.
#include <climits>

#include "common.cuh"
#include "internal.h"

namespace segtaco {

constexpr int kSpmvIpt = 8;
constexpr int kSpmvTile = kCta * kSpmvIpt;
// Shared slots are skewed by one word per 32: a warp whose lanes read items 8
// apart (the per-thread walk) then touches 32 different banks, and the
// coalesced staging writes stay conflict-free.
__device__ __forceinline__ int sk(int i) { return i + (i >> 5); }
constexpr int kSpmvSlots = kSpmvTile + kSpmvTile / 32 + 2;

__global__ void __launch_bounds__(kCta) spmv_kernel(int M, const int *__restrict__ row_ptr,
                                                   const int *__restrict__ col,
                                                   const float *__restrict__ val,
                                                   const float *__restrict__ x,
                                                   float *__restrict__ y,
                                                   const int *__restrict__ px,
                                                   const int *__restrict__ py, long long ntiles) {
  __shared__ int s_rend[kSpmvSlots];
  __shared__ float s_prod[kSpmvSlots];
  __shared__ float s_row[kSpmvSlots];
  const long long c = blockIdx.x;
  if (c >= ntiles) return;
  const int x0 = __ldg(px + c), y0 = __ldg(py + c);
  const int x1 = __ldg(px + c + 1), y1 = __ldg(py + c + 1);
  const int nrows = x1 - x0;  // row ends in this tile
  const int nnzs = y1 - y0;
  const int tid = threadIdx.x;

  // Stage row ends (relative to y0) for rows x0 .. x1 (x1 only as a sentinel).
  for (int i = tid; i <= nrows; i += kCta) {
    const int r = x0 + i;
    s_rend[sk(i)] = (r < M) ? __ldg(row_ptr + r + 1) - y0 : INT_MAX;
    s_row[sk(i)] = 0.0f;
  }
  // Stage products; issue all loads of a thread before using them.
  {
    int cj[kSpmvIpt];
    float cv[kSpmvIpt];
#pragma unroll
    for (int k = 0; k < kSpmvIpt; ++k) {
      const int i = k * kCta + tid;
      cj[k] = i < nnzs ? ld_stream(col + y0 + i) : 0;
      cv[k] = i < nnzs ? (val ? ld_stream(val + y0 + i) : 1.0f) : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < kSpmvIpt; ++k) {
      const int i = k * kCta + tid;
      if (i < nnzs) s_prod[sk(i)] = cv[k] * __ldg(x + cj[k]);
    }
  }
  __syncthreads();

  // Thread-level merge path inside the tile.
  const int total = nrows + nnzs;
  int d = tid * kSpmvIpt;
  if (d > total) d = total;
  int lo = d - nnzs < 0 ? 0 : d - nnzs, hi = d < nrows ? d : nrows;
  while (lo < hi) {
    const int pivot = (lo + hi) >> 1;
    if (s_rend[sk(pivot)] <= d - pivot - 1)
      lo = pivot + 1;
    else
      hi = pivot;
  }
  int tx = lo, ty = d - lo;
  const int dend = d + kSpmvIpt < total ? d + kSpmvIpt : total;
  // A row that ends inside this thread after its first row end began here too:
  // it is stored once.  The partial before the first row end (`first`, row
  // r0) and the one after the last (`run`, row tx) are shared with other
  // threads and combined by a warp segmented scan below.
  const int r0 = tx;
  float run = 0.0f, first = 0.0f;
  bool ended = false;
  for (int it = d; it < dend; ++it) {
    if (s_rend[sk(tx)] <= ty) {  // row end first on ties
      if (ended) {
        s_row[sk(tx)] = run;
      } else {
        first = run;
        ended = true;
      }
      run = 0.0f;
      ++tx;
    } else {
      run += s_prod[sk(ty)];
      ++ty;
    }
  }
  // Inclusive segmented scan over the warp's lanes of the open partials
  // (a lane that saw a row end starts a new segment).
  const unsigned FULL = 0xffffffffu;
  const int lane = tid & 31;
  float sc = run;
  int f = ended ? 1 : 0;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float v = __shfl_up_sync(FULL, sc, o);
    const int fo = __shfl_up_sync(FULL, f, o);
    if (lane >= o) {
      if (!f) sc += v;
      f |= fo;
    }
  }
  float in = __shfl_up_sync(FULL, sc, 1);
  if (lane == 0) in = 0.0f;
  // The first row end of a lane closes the row open after the lanes before it
  // (which may have begun in an earlier warp: atomic); the last lane carries
  // the warp's open partial to the row it stops in.
  if (ended) atomicAdd(&s_row[sk(r0)], first + in);
  if (lane == 31 && sc != 0.0f) atomicAdd(&s_row[sk(tx)], sc);
  __syncthreads();

  const bool head_split = x0 < M && __ldg(row_ptr + x0) < y0;
  for (int i = tid; i <= nrows; i += kCta) {
    const int r = x0 + i;
    if (r >= M) break;
    const float v = s_row[sk(i)];
    if (i == nrows) {
      // Row x1 is unfinished: add the partial only if this tile holds some of it.
      if (y1 > y0 && __ldg(row_ptr + r) < y1) atomicAdd(y + r, v);
    } else if (i == 0 && head_split) {
      atomicAdd(y + r, v);
    } else {
      y[r] = v;
    }
  }
}

int launch_spmv(int M, long long nnz, const int *row_ptr, const int *col, const float *val,
                const float *x, float *y, int *px, int *py, long long D, long long nchunks,
                cudaStream_t s) {
  (void)D;
  if (M == 0) return SEGTACO_OK;
  SEGTACO_TRY(launch_merge_path(row_ptr, M, nnz, kSpmvTile, nchunks, px, py, y, 1, 1, s));
  spmv_kernel<<<(unsigned)nchunks, kCta, 0, s>>>(M, row_ptr, col, val, x, y, px, py, nchunks);
  return check_launch("spmv_kernel");
}

long long spmv_tile_items() { return kSpmvTile; }

}  // namespace segtaco
