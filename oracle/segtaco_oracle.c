/*
 * segtaco_oracle.c -- CPU oracle for the CSR SpMM / SpMV / SDDMM / SpMSpV hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, and only as the checker or the timed CPU baseline.
 *
 * It restates, in plain C, the reference algorithms of segTACO (paths are
 * relative to the segTACO source tree):
 *
 *   spmm_cpu_naive              matrix_experiments/spmm_csr_gpu.h:110-127
 *   Eigen row-major SpMM        eigen-3.4.0/Eigen/src/SparseCore/SparseDenseProduct.h:141-146
 *                               (the product behind ds.h:32-33's EigenCSR * EigenRowMajor)
 *   sddmm_csr_cpu_taco_ref      matrix_experiments/sddmm_csr_gpu.h:9-50
 *   spmspv_csr_cpu_taco_ref     matrix_experiments/spmspv_csr_gpu.h:9-32
 *   binary_search_segment_number gpu_library.h:138-152
 *   taco_binarySearchAfter      gpu_library.h:164-184
 *   taco_binarySearchBefore     gpu_library.h:185-205
 *   taco_binarySearchBeforeBlock gpu_library.h:206-215 (+ launcher :236-240)
 *
 * plus this project's own partition definitions (canonical start rows and the
 * merge-path split of rows+nonzeros), so that the device partition arrays can
 * be compared bit-exactly.
 *
 * Compiled with -ffp-contract=off so that a*b+c is a multiply then an add on
 * every host; the "fma" variants call fmaf() explicitly.  Results therefore
 * agree bit for bit between x86-64 and aarch64 hosts.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Searches over row_ptr                                                */
/* ------------------------------------------------------------------ */

/* Row that holds nonzero `e`: the smallest mid in [1, n_seg) with
 * seg_offsets[mid] > e, minus one (gpu_library.h:138-152).  For e >= nnz the
 * search runs off the end and returns n_seg - 1. */
int32_t orc_binary_search_segment_number(const int32_t *seg_offsets, int32_t n_seg,
                                         int32_t n_elem, int32_t elem_id) {
  (void)n_elem;
  int32_t lo = 1, hi = n_seg;
  while (lo < hi) {
    int32_t mid = (lo + hi) >> 1;
    if (seg_offsets[mid] <= elem_id)
      lo = mid + 1;
    else
      hi = mid;
  }
  return hi - 1;
}

/* Bisection that returns arrayEnd when array[arrayEnd] <= target, an exact
 * hit when one is met, else the last lower bound (gpu_library.h:185-205). */
int32_t orc_taco_search_before(const int32_t *array, int32_t start, int32_t end,
                               int32_t target) {
  if (array[end] <= target) return end;
  int32_t lower = start, upper = end;
  while (upper - lower > 1) {
    int32_t mid = (upper + lower) / 2;
    int32_t v = array[mid];
    if (v < target)
      lower = mid;
    else if (v > target)
      upper = mid;
    else
      return mid;
  }
  return lower;
}

/* Mirror image of the above (gpu_library.h:164-184). */
int32_t orc_taco_search_after(const int32_t *array, int32_t start, int32_t end,
                              int32_t target) {
  if (array[start] >= target) return start;
  int32_t lower = start, upper = end;
  while (upper - lower > 1) {
    int32_t mid = (upper + lower) / 2;
    int32_t v = array[mid];
    if (v < target)
      lower = mid;
    else if (v > target)
      upper = mid;
    else
      return mid;
  }
  return upper;
}

/* Reference partition array: out[b] = taco_binarySearchBefore(row_ptr, 0, M,
 * b*P) for b = 0..nblk (gpu_library.h:206-215,236-240). */
void orc_block_starts_taco(const int32_t *row_ptr, int32_t M, int32_t P, int32_t nblk,
                           int32_t *out) {
  for (int32_t b = 0; b <= nblk; ++b)
    out[b] = orc_taco_search_before(row_ptr, 0, M, (int32_t)((int64_t)b * P));
}

/* Canonical start row of each block: the last r in [0, M] with row_ptr[r] <=
 * b*P, i.e. upper_bound(row_ptr[0..M], b*P) - 1.  For b*P < nnz that is the one
 * non-empty row holding nonzero b*P; it satisfies the consumer contract
 * row_ptr[start[b]] <= b*P that the reference kernels rely on
 * (matrix_kernels/spmm_eb_sr.h:882-893). */
void orc_block_starts_canonical(const int32_t *row_ptr, int32_t M, int32_t P, int32_t nblk,
                                int32_t *out) {
  for (int32_t b = 0; b <= nblk; ++b) {
    int64_t t = (int64_t)b * P;
    int32_t lo = 0, hi = M + 1; /* first index with row_ptr[idx] > t */
    while (lo < hi) {
      int32_t mid = lo + ((hi - lo) >> 1);
      if ((int64_t)row_ptr[mid] <= t)
        lo = mid + 1;
      else
        hi = mid;
    }
    int32_t r = lo - 1;
    if (r < 0) r = 0;
    if (r > M) r = M;
    out[b] = r;
  }
}

/* Merge-path split of the merged sequence {row ends} U {nonzeros}.  Row end x
 * sorts before nonzero y when row_ptr[x+1] <= y.  Diagonal d is split into
 * (x, y), x + y = d, x = number of row ends taken.  Chunk c covers diagonals
 * [c*D, min((c+1)*D, M+nnz)); out_x / out_y have nchunks+1 entries. */
void orc_merge_path(const int32_t *row_ptr, int32_t M, int64_t nnz, int64_t D,
                    int64_t nchunks, int32_t *out_x, int32_t *out_y) {
  int64_t total = (int64_t)M + nnz;
  for (int64_t c = 0; c <= nchunks; ++c) {
    int64_t d = c * D;
    if (d > total) d = total;
    int64_t lo = d - nnz;
    if (lo < 0) lo = 0;
    int64_t hi = d < M ? d : M;
    while (lo < hi) {
      int64_t pivot = (lo + hi) >> 1;
      if ((int64_t)row_ptr[pivot + 1] <= d - pivot - 1)
        lo = pivot + 1;
      else
        hi = pivot;
    }
    out_x[c] = (int32_t)lo;
    out_y[c] = (int32_t)(d - lo);
  }
}

/* Row id of every nonzero (linear walk; the definition the searches must meet). */
void orc_row_ids(const int32_t *row_ptr, int32_t M, int32_t *out) {
  for (int32_t i = 0; i < M; ++i)
    for (int32_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) out[p] = i;
}

/* ------------------------------------------------------------------ */
/* SpMM                                                                */
/* ------------------------------------------------------------------ */

static inline float bf16_to_f32(uint16_t h) {
  uint32_t u = ((uint32_t)h) << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

/* C64 = A * B accumulated in double: the definition of spmm_cpu_naive
 * (matrix_experiments/spmm_csr_gpu.h:110-127) with a double accumulator.
 * vals == NULL means all ones (gpu_library.h:155-162).  b_bf16 != 0 means B
 * holds bf16 bit patterns (uint16), converted exactly to float first. */
void orc_spmm_f64(int32_t M, int32_t N, const int32_t *row_ptr, const int32_t *col,
                  const float *val, const void *B, int32_t ldb, int32_t b_bf16,
                  double *C, int32_t ldc) {
  const float *Bf = (const float *)B;
  const uint16_t *Bh = (const uint16_t *)B;
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t i = 0; i < M; ++i) {
    double *c = C + (int64_t)i * ldc;
    for (int32_t k = 0; k < N; ++k) c[k] = 0.0;
    for (int32_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
      double v = val ? (double)val[p] : 1.0;
      int64_t j = col[p];
      if (b_bf16) {
        const uint16_t *b = Bh + j * ldb;
        for (int32_t k = 0; k < N; ++k) c[k] += v * (double)bf16_to_f32(b[k]);
      } else {
        const float *b = Bf + j * ldb;
        for (int32_t k = 0; k < N; ++k) c[k] += v * (double)b[k];
      }
    }
  }
}

/* Error bound scale: S[i,k] = sum_p |a_ip| * |b_jk|.  Forward error of any
 * summation order is bounded by (len * u) * S, so |c - c64| / S is the
 * order-independent relative error used by the tests. */
void orc_spmm_absbound(int32_t M, int32_t N, const int32_t *row_ptr, const int32_t *col,
                       const float *val, const void *B, int32_t ldb, int32_t b_bf16,
                       double *S, int32_t lds) {
  const float *Bf = (const float *)B;
  const uint16_t *Bh = (const uint16_t *)B;
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t i = 0; i < M; ++i) {
    double *s = S + (int64_t)i * lds;
    for (int32_t k = 0; k < N; ++k) s[k] = 0.0;
    for (int32_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
      double v = fabs(val ? (double)val[p] : 1.0);
      int64_t j = col[p];
      if (b_bf16) {
        const uint16_t *b = Bh + j * ldb;
        for (int32_t k = 0; k < N; ++k) s[k] += v * fabs((double)bf16_to_f32(b[k]));
      } else {
        const float *b = Bf + j * ldb;
        for (int32_t k = 0; k < N; ++k) s[k] += v * fabs((double)b[k]);
      }
    }
  }
}

/* FP32 product in the Eigen row-major order: for each row, res_i starts at 0
 * and gets (alpha*a_ip) * rhs.row(j) added nonzero by nonzero in storage order
 * (SparseDenseProduct.h:141-146; alpha = 1).  use_fma selects a fused
 * multiply-add per step, which is what a contracting compiler emits. */
void orc_spmm_f32_rowseq(int32_t M, int32_t N, const int32_t *row_ptr, const int32_t *col,
                         const float *val, const float *B, int32_t ldb, float *C,
                         int32_t ldc, int32_t use_fma) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t i = 0; i < M; ++i) {
    float *c = C + (int64_t)i * ldc;
    for (int32_t k = 0; k < N; ++k) c[k] = 0.0f;
    for (int32_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
      float v = val ? val[p] : 1.0f;
      const float *b = B + (int64_t)col[p] * ldb;
      if (use_fma)
        for (int32_t k = 0; k < N; ++k) c[k] = fmaf(v, b[k], c[k]);
      else
        for (int32_t k = 0; k < N; ++k) c[k] = c[k] + v * b[k];
    }
  }
}

/* ------------------------------------------------------------------ */
/* SpMV, SDDMM, SpMSpV                                                 */
/* ------------------------------------------------------------------ */

/* y = A x in double (the operation of matrix_kernels/spmv_csr_gpu_taco.h:4-76). */
void orc_spmv_f64(int32_t M, const int32_t *row_ptr, const int32_t *col, const float *val,
                  const float *x, double *y) {
#pragma omp parallel for schedule(dynamic, 1024)
  for (int32_t i = 0; i < M; ++i) {
    double s = 0.0;
    for (int32_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p)
      s += (val ? (double)val[p] : 1.0) * (double)x[col[p]];
    y[i] = s;
  }
}

/* out[p] = a_p * sum_k X[i,k] * Y[j,k] for every nonzero p = (i, j), in double
 * (sddmm_csr_gpu.h:38-43 computes A_vals[jB] += (B_vals[jB]*C[i,k]) * D[j,k]).
 * x_bf16 != 0: X and Y hold bf16 bit patterns.  bound[p] (optional) receives
 * |a_p| * sum_k |X[i,k] Y[j,k]|. */
void orc_sddmm_f64(int32_t M, int32_t D, const int32_t *row_ptr, const int32_t *col,
                   const float *val, const void *X, const void *Y, int32_t ldx, int32_t ldy,
                   int32_t x_bf16, double *out, double *bound) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t i = 0; i < M; ++i) {
    for (int32_t p = row_ptr[i]; p < row_ptr[i + 1]; ++p) {
      int64_t j = col[p];
      double a = val ? (double)val[p] : 1.0;
      double s = 0.0, sb = 0.0;
      for (int32_t k = 0; k < D; ++k) {
        double xv, yv;
        if (x_bf16) {
          xv = bf16_to_f32(((const uint16_t *)X)[(int64_t)i * ldx + k]);
          yv = bf16_to_f32(((const uint16_t *)Y)[j * ldy + k]);
        } else {
          xv = ((const float *)X)[(int64_t)i * ldx + k];
          yv = ((const float *)Y)[j * ldy + k];
        }
        s += xv * yv;
        sb += fabs(xv * yv);
      }
      out[p] = a * s;
      if (bound) bound[p] = fabs(a) * sb;
    }
  }
}

/* y = A x with x sparse, pushed column by column over A stored as CSC (the CSR
 * of A^T, spmspv_csr_gpu.h:37-43): for each stored x_j, y[i] += A_ij * x_j
 * (spmspv_csr_gpu.h:24-31).  Double accumulation, x entries in storage order. */
void orc_spmspv_f64(int32_t M, const int32_t *col_ptr, const int32_t *row_idx,
                    const float *val, int32_t nx, const int32_t *x_idx, const float *x_val,
                    double *y, double *bound) {
  for (int32_t i = 0; i < M; ++i) {
    y[i] = 0.0;
    if (bound) bound[i] = 0.0;
  }
  for (int32_t t = 0; t < nx; ++t) {
    int32_t j = x_idx[t];
    double xv = x_val[t];
    for (int32_t p = col_ptr[j]; p < col_ptr[j + 1]; ++p) {
      double a = val ? (double)val[p] : 1.0;
      y[row_idx[p]] += a * xv;
      if (bound) bound[row_idx[p]] += fabs(a * xv);
    }
  }
}

/* ------------------------------------------------------------------ */
/* Comparison helpers                                                  */
/* ------------------------------------------------------------------ */

/* max_i |got_i - ref_i| / max(S_i, tiny): the bound-normalised error. */
double orc_max_bound_err_f32(int64_t n, const float *got, const double *ref, const double *S) {
  double worst = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    double s = S[i] > 1e-30 ? S[i] : 1e-30;
    double e = fabs((double)got[i] - ref[i]);
    if (S[i] == 0.0 && e == 0.0) continue;
    double r = e / s;
    if (r > worst || r != r) worst = r;
  }
  return worst;
}

/* max plain relative error over entries with |ref| > floor. */
double orc_max_rel_err_f32(int64_t n, const float *got, const double *ref, double floor_abs) {
  double worst = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    double a = fabs(ref[i]);
    if (a <= floor_abs) continue;
    double r = fabs((double)got[i] - ref[i]) / a;
    if (r > worst || r != r) worst = r;
  }
  return worst;
}

int32_t orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
