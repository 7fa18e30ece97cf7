// partition.cu -- partition arrays over row_ptr and CSR validation.
//
//   merge_path_kernel        merge-path split of {row ends} U {nonzeros}: a
//                            thread per row writes the chunk edges inside it;
//                            also zeroes the C rows that straddle a chunk edge
//                            (they are then accumulated with reductions).
//   block_starts_taco_kernel segTACO's block starts, taco_binarySearchBefore per
//                            block (gpu_library.h:185-240), bit-exact.
//   block_starts_canonical   last r with row_ptr[r] <= b*P (upper_bound - 1).
//   row_ids_kernel           row of every nonzero, the result of
//                            binary_search_segment_number (gpu_library.h:138-152).
//   validate_kernel          row_ptr monotone / bounds, 0 <= col < K.
#include <climits>

#include "common.cuh"
#include "internal.h"

namespace segtaco {

constexpr int kPartRows = 4;  // rows per partition thread

__global__ void merge_path_kernel(const int *__restrict__ row_ptr, int M, long long nnz,
                                  long long D, long long nchunks, int *__restrict__ px,
                                  int *__restrict__ py, float *__restrict__ C, long long ldc,
                                  int N) {
  // Row r owns the chunk edges that fall between row end r-1 and row end r
  // (merge_path_store_row); r = M is the tail.  A thread walks kPartRows
  // consecutive rows, its row_ptr loads independent of one another.
  const long long r0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kPartRows;
  if (r0 > M) return;
  const bool small = (long long)M + nnz + D < 0x7fffffffLL;
  long long e[kPartRows + 1];  // e[k] = e_{r0+k-1} = row_ptr[r0+k] + r0 + k (e_{-1} = 0)
#pragma unroll
  for (int k = 0; k <= kPartRows; ++k) {
    const long long r = r0 + k;
    e[k] = (r > 0 && r <= M) ? (long long)__ldg(row_ptr + r) + r : 0;
  }
  long long lo = ceil_div_pos(e[0], D, small);  // first edge at or past e_{r0-1}
#pragma unroll
  for (int k = 0; k < kPartRows; ++k) {
    const long long r = r0 + k;
    if (r < M) {
      const long long nxt = ceil_div_pos(e[k + 1], D, small);  // first edge past row r
      merge_path_store_row(row_ptr, M, nnz, D, nchunks, r, lo, nxt - 1, px, py, C, ldc, N);
      lo = nxt;
    } else if (r == M) {
      merge_path_store_row(row_ptr, M, nnz, D, nchunks, r, lo, nchunks, px, py, C, ldc, N);
    }
  }
}

// Same bisection as taco_binarySearchBefore (gpu_library.h:185-205).
__device__ __forceinline__ int taco_search_before(const int *__restrict__ array, int start, int end,
                                                  int target) {
  if (__ldg(array + end) <= target) return end;
  int lower = start, upper = end;
  while (upper - lower > 1) {
    const int mid = (upper + lower) / 2;
    const int v = __ldg(array + mid);
    if (v < target)
      lower = mid;
    else if (v > target)
      upper = mid;
    else
      return mid;
  }
  return lower;
}

__global__ void block_starts_taco_kernel(const int *__restrict__ row_ptr, int M, int P, long long nblk,
                                         int *__restrict__ out) {
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b > nblk) return;
  out[b] = taco_search_before(row_ptr, 0, M, (int)(b * P));
}

__global__ void block_starts_canonical_kernel(const int *__restrict__ row_ptr, int M, int P,
                                              long long nblk, int *__restrict__ out) {
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b > nblk) return;
  const long long t = b * P;
  int lo = 0, hi = M + 1;  // first index with row_ptr[idx] > t
  while (lo < hi) {
    const int mid = lo + ((hi - lo) >> 1);
    if ((long long)__ldg(row_ptr + mid) <= t)
      lo = mid + 1;
    else
      hi = mid;
  }
  int r = lo - 1;
  out[b] = r < 0 ? 0 : (r > M ? M : r);
}

// Row of every nonzero: a warp per row writes its run (coalesced).
__global__ void row_ids_kernel(const int *__restrict__ row_ptr, int M, int *__restrict__ out) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= M) return;
  const int p0 = __ldg(row_ptr + w), p1 = __ldg(row_ptr + w + 1);
  for (int p = p0 + lane; p < p1; p += 32) out[p] = (int)w;
}

// err[0] = first failing check code (0 = none), err[1] = an index that fails it.
__global__ void validate_kernel(const int *__restrict__ row_ptr, int M, int K, long long nnz,
                                const int *__restrict__ col, int *__restrict__ err) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    if (__ldg(row_ptr) != 0) {
      atomicCAS(err, 0, 1);
      err[1] = 0;
    }
    if ((long long)__ldg(row_ptr + M) != nnz) {
      atomicCAS(err, 0, 2);
      err[1] = M;
    }
  }
  if (i < M) {
    if (__ldg(row_ptr + i) > __ldg(row_ptr + i + 1)) {
      if (atomicCAS(err, 0, 3) == 0) err[1] = (int)i;
    }
  }
  if (i < nnz) {
    const int c = __ldg(col + i);
    if (c < 0 || c >= K) {
      if (atomicCAS(err, 0, 4) == 0) err[1] = (int)i;
    }
  }
}

static inline unsigned grid_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

int launch_merge_path(const int *row_ptr, int M, long long nnz, long long D, long long nchunks,
                      int *px, int *py, float *C, long long ldc, int N, cudaStream_t s) {
  const long long threads = ((long long)M + kPartRows) / kPartRows;  // rows 0 .. M
  merge_path_kernel<<<grid_for(threads, 256), 256, 0, s>>>(row_ptr, M, nnz, D, nchunks, px, py, C,
                                                           ldc, N);
  return check_launch("merge_path_kernel");
}

int launch_block_starts_taco(const int *row_ptr, int M, int P, long long nblk, int *out,
                             cudaStream_t s) {
  block_starts_taco_kernel<<<grid_for(nblk + 1, 256), 256, 0, s>>>(row_ptr, M, P, nblk, out);
  return check_launch("block_starts_taco_kernel");
}

int launch_block_starts_canonical(const int *row_ptr, int M, int P, long long nblk, int *out,
                                  cudaStream_t s) {
  block_starts_canonical_kernel<<<grid_for(nblk + 1, 256), 256, 0, s>>>(row_ptr, M, P, nblk, out);
  return check_launch("block_starts_canonical_kernel");
}

int launch_row_ids(const int *row_ptr, int M, int *out, cudaStream_t s) {
  if (M == 0) return SEGTACO_OK;
  row_ids_kernel<<<grid_for((long long)M * 32, 256), 256, 0, s>>>(row_ptr, M, out);
  return check_launch("row_ids_kernel");
}

int launch_validate(const int *row_ptr, int M, int K, long long nnz, const int *col, int *err,
                    cudaStream_t s) {
  long long n = nnz > M ? nnz : M;
  if (n < 1) n = 1;
  validate_kernel<<<grid_for(n, 256), 256, 0, s>>>(row_ptr, M, K, nnz, col, err);
  return check_launch("validate_kernel");
}

}  // namespace segtaco
