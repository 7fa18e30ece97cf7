// vendor.cu -- cuSPARSE SpMM (CSR_ALG2, row-major B and C) on device operands.
//
// A comparator only: segTACO's verification reference and its "alg2" sweep
// column are cusparseSpMM with CUSPARSE_SPMM_CSR_ALG2 on row-major B and C
// (matrix_kernels/spmm_csr_gpu_cusparse.h:171-260).  The vendor library is
// called, never inspected.
#include <cusparse.h>

#include "internal.h"

using namespace segtaco;

extern "C" int segtaco_vendor_spmm(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                                   const int32_t *col, const float *vals, const float *B,
                                   int64_t ldb, float *C, int64_t ldc, int32_t N, void *stream) {
  if (M <= 0 || N <= 0) return SEGTACO_OK;
  if (!row_ptr || !C || (nnz > 0 && (!col || !vals || !B)))
    return set_error(SEGTACO_EINVAL, "segtaco_vendor_spmm: NULL operand");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cusparseHandle_t h = nullptr;
  cusparseSpMatDescr_t a = nullptr;
  cusparseDnMatDescr_t b = nullptr, c = nullptr;
  void *work = nullptr;
  size_t bytes = 0;
  int st = SEGTACO_OK;
  const float alpha = 1.0f, beta = 0.0f;
#define CS(x)                                                                   \
  do {                                                                          \
    cusparseStatus_t _c = (x);                                                  \
    if (_c != CUSPARSE_STATUS_SUCCESS && st == SEGTACO_OK)                      \
      st = set_error(SEGTACO_ECUDA, "%s: %s", #x, cusparseGetErrorString(_c)); \
  } while (0)
  CS(cusparseCreate(&h));
  if (st == SEGTACO_OK) CS(cusparseSetStream(h, s));
  CS(cusparseCreateCsr(&a, M, K, nnz, (void *)row_ptr, (void *)col, (void *)vals,
                       CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_BASE_ZERO,
                       CUDA_R_32F));
  CS(cusparseCreateDnMat(&b, K, N, ldb, (void *)B, CUDA_R_32F, CUSPARSE_ORDER_ROW));
  CS(cusparseCreateDnMat(&c, M, N, ldc, C, CUDA_R_32F, CUSPARSE_ORDER_ROW));
  CS(cusparseSpMM_bufferSize(h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE,
                             &alpha, a, b, &beta, c, CUDA_R_32F, CUSPARSE_SPMM_CSR_ALG2, &bytes));
  if (st == SEGTACO_OK && bytes) st = check_cuda(cudaMallocAsync(&work, bytes, s), "cudaMallocAsync");
  CS(cusparseSpMM(h, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, a,
                  b, &beta, c, CUDA_R_32F, CUSPARSE_SPMM_CSR_ALG2, work));
  if (work) cudaFreeAsync(work, s);
  if (a) cusparseDestroySpMat(a);
  if (b) cusparseDestroyDnMat(b);
  if (c) cusparseDestroyDnMat(c);
  if (h) cusparseDestroy(h);
#undef CS
  return st;
}
