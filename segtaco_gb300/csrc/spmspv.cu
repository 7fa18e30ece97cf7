// spmspv.cu -- y = A x with a sparse x, pushed over the columns of A.
//
// segTACO's SpMSpV (spmspv_csr_gpu_taco.h:5-55; CPU reference
// spmspv_csr_gpu.h:9-32) stores A as the CSR of A^T and gives each stored x_j
// one thread that walks column j and adds A_ij * x_j into y[i] atomically.
// Here a warp takes one stored x_j (lanes stride the column, so long columns
// are split 32 ways and the row-index / value reads are coalesced), and y is
// cleared on the same stream first.
#include "common.cuh"
#include "internal.h"

namespace segtaco {

__global__ void __launch_bounds__(kCta) spmspv_kernel(const int *__restrict__ col_ptr,
                                                     const int *__restrict__ row_idx,
                                                     const float *__restrict__ val, int nx,
                                                     const int *__restrict__ x_idx,
                                                     const float *__restrict__ x_vals,
                                                     float *__restrict__ y) {
  const int lane = threadIdx.x & 31;
  const long long nwarps = (long long)gridDim.x * (kCta / 32);
  for (long long t = (long long)blockIdx.x * (kCta / 32) + threadIdx.x / 32; t < nx; t += nwarps) {
    const int j = __ldg(x_idx + t);
    const float xv = __ldg(x_vals + t);
    const int p0 = __ldg(col_ptr + j), p1 = __ldg(col_ptr + j + 1);
    for (int p = p0 + lane; p < p1; p += 32) {
      const float a = val ? ld_stream(val + p) : 1.0f;
      atomicAdd(y + ld_stream(row_idx + p), a * xv);
    }
  }
}

int launch_spmspv(int M, int K, const int *col_ptr, const int *row_idx, const float *val, int nx,
                  const int *x_idx, const float *x_vals, float *y, cudaStream_t s) {
  (void)K;
  if (M > 0) SEGTACO_TRY(check_cuda(cudaMemsetAsync(y, 0, (size_t)M * sizeof(float), s), "memset y"));
  if (nx <= 0) return SEGTACO_OK;
  long long warps = nx;
  long long blocks = (warps + (kCta / 32) - 1) / (kCta / 32);
  if (blocks > 152 * 64) blocks = 152 * 64;
  spmspv_kernel<<<(unsigned)blocks, kCta, 0, s>>>(col_ptr, row_idx, val, nx, x_idx, x_vals, y);
  return check_launch("spmspv_kernel");
}

}  // namespace segtaco
