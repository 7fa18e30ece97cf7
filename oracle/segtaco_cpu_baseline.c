/*
 * segtaco_cpu_baseline.c -- the timed CPU baseline for CSR SpMM / SpMV.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY: bench.py times it as the CPU
 * baseline (and as the reference arm); the product library never calls it.
 *
 * It is the reference's own CPU product for this path restated in C: Eigen
 * 3.4's row-major sparse x row-major dense kernel
 * (eigen-3.4.0/Eigen/src/SparseCore/SparseDenseProduct.h:109-146), i.e.
 *   - OpenMP over rows with schedule(dynamic, ceil(n / (4*threads)))  (:124-127)
 *   - per row: res_i = 0, then res_i += a_ip * B.row(j) in storage order (:141-146)
 * The inner loop over the dense row is left to the compiler to vectorise, as
 * Eigen's packet code does; this translation unit is compiled without
 * -ffp-contract=off, so a contracting compiler may fuse the multiply-add.
 */
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void orc_cpu_spmm_eigen_order(int32_t M, int32_t N, const int32_t *row_ptr,
                              const int32_t *col, const float *val, const float *B,
                              float *C, int32_t threads) {
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
  int64_t chunk = ((int64_t)M + threads * 4 - 1) / (threads * 4);
  if (chunk < 1) chunk = 1;
#pragma omp parallel for schedule(dynamic, chunk) num_threads(threads)
#endif
  for (int32_t i = 0; i < M; ++i) {
    float *restrict c = C + (int64_t)i * N;
    for (int32_t k = 0; k < N; ++k) c[k] = 0.0f;
    for (int32_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
      const float v = val[p];
      const float *restrict b = B + (int64_t)col[p] * N;
      for (int32_t k = 0; k < N; ++k) c[k] += v * b[k];
    }
  }
}

/* SpMV in the same order (SparseDenseProduct.h:60-66, column-per-column path). */
void orc_cpu_spmv_eigen_order(int32_t M, const int32_t *row_ptr, const int32_t *col,
                              const float *val, const float *x, float *y, int32_t threads) {
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
  int64_t chunk = ((int64_t)M + threads * 4 - 1) / (threads * 4);
  if (chunk < 1) chunk = 1;
#pragma omp parallel for schedule(dynamic, chunk) num_threads(threads)
#endif
  for (int32_t i = 0; i < M; ++i) {
    float tmp = 0.0f;
    for (int32_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) tmp += val[p] * x[col[p]];
    y[i] = tmp;
  }
}

int32_t orc_cpu_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
