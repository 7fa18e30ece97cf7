/*
 * segtaco_taco.h -- segTACO's kernel-selection surface, served by libsegtaco.
 *
 * A segTACO driver (matrix_main.cpp -> matrix_experiments/spmm_csr_gpu.h)
 * calls kernels by name with host-side taco_tensor_t operands and reads the
 * GPU time of the last call from get_gpu_timer_result().  This header declares
 * the same names with the same C++ signatures as segTACO's gpu_kernels.cuh, so
 * that driver links against libsegtaco unchanged.  Each call behaves like the
 * segTACO wrapper it replaces (e.g. matrix_kernels/spmm_eb_sr.h:908-928):
 * A/B are copied host->device, the timed region (partition + kernel) runs on
 * the legacy default stream between two events, and C is copied back into
 * C->vals.  C is overwritten.  Device buffers are reused across calls (see
 * segtaco_taco_release) instead of being allocated and freed every call.
 * Errors are fail-stop (message on stderr, exit), as segTACO's gpuErrchk
 * (gpu_library.h:22-30); use segtaco_taco_call() for a status-returning form.
 *
 * The tuning suffix of each name selects a schedule and tuning hints (rows per
 * unit, nonzeros per unit, vector width); unlike the segTACO originals, every
 * name computes the full product for any N (segTACO's *_256_{g}_{c},
 * *_{Nnz}_{group} and *_taco/_512_64 variants only cover some columns, see
 * spmm_rb_sr.h:363, spmm_eb_sr.h:874, spmm_eb_pr.h:482-524, spmm_eb_sr.h:5-54).
 */
#ifndef SEGTACO_TACO_H
#define SEGTACO_TACO_H

/* The taco_tensor_t ABI (segTACO taco_tensor_t.h:4-15).  The layout must match
 * field for field, so it is declared under segTACO's own include guard: a
 * translation unit that includes segTACO's header first gets that definition,
 * and the two never coexist. */
#ifndef TACO_TENSOR_T_H
#define TACO_TENSOR_T_H
#include <stdint.h>
typedef enum { taco_mode_dense, taco_mode_sparse } taco_mode_t;
struct taco_tensor_t {
  int32_t order;             /* number of modes                          */
  int32_t *dimensions;       /* dimensions[0] rows, dimensions[1] columns */
  int32_t csize;             /* component size                           */
  int32_t *mode_ordering;    /* mode storage ordering                    */
  taco_mode_t *mode_types;   /* mode storage types                       */
  int32_t ***indices;        /* CSR: indices[1][0] = row_ptr, [1][1] = col */
  float *vals;               /* values                                   */
  int32_t vals_size;         /* values array size                        */
};
#endif

#ifdef __cplusplus
extern "C" {
#endif
/* Status-returning form for FFI callers: runs the named kernel (any name
 * declared below) and returns SEGTACO_OK or an error code; never exits. */
int segtaco_taco_call(const char *name, struct taco_tensor_t *out, struct taco_tensor_t *a,
                      struct taco_tensor_t *b, struct taco_tensor_t *c);
/* Milliseconds of the last timed region (same value as get_gpu_timer_result). */
float segtaco_taco_timer_ms(void);
/* Device copies of the operands are kept per operand role and grown on
 * demand across calls (segTACO allocates and frees them per call); this frees
 * them. */
void segtaco_taco_release(void);
/* Number of names segtaco_taco_call accepts, and the i-th of them. */
int segtaco_taco_num_names(void);
const char *segtaco_taco_name(int i);
#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
/* gpu_kernels.cuh:4 */
float get_gpu_timer_result();

/* Side operations, reference signatures (gpu_kernels.cuh:6-8,25-27; the
 * segTACO versions are commented out of its build). */
void spmv_csr_gpu_taco(taco_tensor_t *y, taco_tensor_t *A, taco_tensor_t *x);
void sddmm_csr_gpu_taco(taco_tensor_t *A, taco_tensor_t *B, taco_tensor_t *C, taco_tensor_t *D);
void sddmm_csr_gpu_warp(taco_tensor_t *A, taco_tensor_t *B, taco_tensor_t *C, taco_tensor_t *D);
void spmspv_csr_gpu_taco(taco_tensor_t *y, taco_tensor_t *A, taco_tensor_t *x);

/* SpMM, gpu_kernels.cuh:11-93 (in that order), plus the two names defined
 * but not declared there (spmm_rb_sr.h:334, spmm_eb_sr.h:834). */
#define SEGTACO_SPMM_DECL(name) void name(taco_tensor_t *C, taco_tensor_t *A, taco_tensor_t *B);
SEGTACO_SPMM_DECL(spmm_csr_gpu_taco)
SEGTACO_SPMM_DECL(spmm_csr_gpu_warp)
SEGTACO_SPMM_DECL(spmm_csr_gpu_cusparse)
SEGTACO_SPMM_DECL(spmm_csr_gpu_reduction)
SEGTACO_SPMM_DECL(spmm_csr_pr_eb)
SEGTACO_SPMM_DECL(spmm_csr_cusparse_row)
SEGTACO_SPMM_DECL(spmm_rb_sr_taco)
SEGTACO_SPMM_DECL(spmm_rb_sr)
SEGTACO_SPMM_DECL(spmm_rb_pr_taco)
SEGTACO_SPMM_DECL(spmm_rb_pr)
SEGTACO_SPMM_DECL(spmm_eb_sr_taco)
SEGTACO_SPMM_DECL(spmm_eb_sr)
SEGTACO_SPMM_DECL(spmm_eb_pr_taco)
SEGTACO_SPMM_DECL(spmm_eb_pr)
SEGTACO_SPMM_DECL(spmm_eb_sr_search)
SEGTACO_SPMM_DECL(spmm_eb_pr_search)
SEGTACO_SPMM_DECL(spmm_rb_sr_512_64)
SEGTACO_SPMM_DECL(spmm_eb_sr_512_64)
SEGTACO_SPMM_DECL(spmm_rb_pr_256)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_1_4_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_2_4_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_4_4_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_1_8_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_2_8_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_4_8_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_1_8_8)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_2_8_8)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_4_8_8)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_1_16_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_2_16_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_4_16_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_1_16_8)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_2_16_8)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_4_16_8)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_1_16_16)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_2_16_16)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_4_16_16)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_1_32_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_2_32_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_4_32_4)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_1_32_8)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_2_32_8)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_4_32_8)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_1_32_16)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_2_32_16)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_4_32_16)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_1_32_32)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_2_32_32)
SEGTACO_SPMM_DECL(spmm_rb_pr_256_4_32_32)
SEGTACO_SPMM_DECL(spmm_eb_pr_256_32)
SEGTACO_SPMM_DECL(spmm_eb_pr_256_16)
SEGTACO_SPMM_DECL(spmm_eb_pr_256_8)
SEGTACO_SPMM_DECL(spmm_eb_pr_256_4)
SEGTACO_SPMM_DECL(spmm_eb_pr_128_32)
SEGTACO_SPMM_DECL(spmm_eb_pr_128_16)
SEGTACO_SPMM_DECL(spmm_eb_pr_128_8)
SEGTACO_SPMM_DECL(spmm_eb_pr_128_4)
SEGTACO_SPMM_DECL(spmm_eb_pr_64_32)
SEGTACO_SPMM_DECL(spmm_eb_pr_64_16)
SEGTACO_SPMM_DECL(spmm_eb_pr_64_8)
SEGTACO_SPMM_DECL(spmm_eb_pr_64_4)
SEGTACO_SPMM_DECL(spmm_rb_sr_256_1_1)
SEGTACO_SPMM_DECL(spmm_rb_sr_256_1_2)
SEGTACO_SPMM_DECL(spmm_rb_sr_256_1_4)
SEGTACO_SPMM_DECL(spmm_rb_sr_256_2_1)
SEGTACO_SPMM_DECL(spmm_rb_sr_256_2_2)
SEGTACO_SPMM_DECL(spmm_rb_sr_256_2_4)
SEGTACO_SPMM_DECL(spmm_rb_sr_256_4_1)
SEGTACO_SPMM_DECL(spmm_rb_sr_256_4_2)
SEGTACO_SPMM_DECL(spmm_rb_sr_256_4_4)
SEGTACO_SPMM_DECL(spmm_eb_sr_256_4_1)
SEGTACO_SPMM_DECL(spmm_eb_sr_256_4_2)
SEGTACO_SPMM_DECL(spmm_eb_sr_256_4_4)
SEGTACO_SPMM_DECL(spmm_eb_sr_256_8_1)
SEGTACO_SPMM_DECL(spmm_eb_sr_256_8_2)
SEGTACO_SPMM_DECL(spmm_eb_sr_256_8_4)
SEGTACO_SPMM_DECL(spmm_eb_sr_256_16_1)
SEGTACO_SPMM_DECL(spmm_eb_sr_256_16_2)
SEGTACO_SPMM_DECL(spmm_eb_sr_256_16_4)
SEGTACO_SPMM_DECL(spmm_rb_sr_256_4)
SEGTACO_SPMM_DECL(spmm_eb_sr_256_4)
#undef SEGTACO_SPMM_DECL
#endif /* __cplusplus */

#endif /* SEGTACO_TACO_H */
