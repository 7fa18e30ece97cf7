/*
 * segtaco.h -- C ABI of the GB300 (sm_103a) CSR sparse kernels.
 *
 * This is the layer that every front end binds: the taco_tensor_t drop-in
 * (segtaco_taco.h), the Python bindings, and any cgo/JNI/ctypes caller.  All
 * arguments are plain C: device pointers, sizes, an opaque CUDA stream.  Every
 * entry point returns a status code (SEGTACO_OK == 0); nothing here exits the
 * process.  Calls are re-entrant: operands travel as arguments, never through
 * global device symbols (the segTACO kernels read theirs from __device__
 * globals, gpu_library.h:336-361,463-472, which makes them single-caller).
 *
 * Operand conventions (the segTACO taco_tensor_t CSR view, ds.h:411-458):
 *   A      CSR, M rows x K columns, int32 row_ptr[M+1] (row_ptr[0] == 0,
 *          row_ptr[M] == nnz), int32 col[nnz] sorted within a row is NOT
 *          required, float vals[nnz]; vals == NULL means every value is 1
 *          (gpu_library.h:155-162).
 *   B      dense K x N, row-major, leading dimension ldb (elements).
 *   C      dense M x N, row-major, leading dimension ldc; fully OVERWRITTEN
 *          (segTACO zeroes C inside its timed region, e.g. spmm_rb_sr.h:400).
 *   stream a cudaStream_t passed as void*; NULL = the legacy default stream.
 *
 * Scratch: entry points that need scratch memory take (workspace, bytes);
 * *_workspace_size() says how much.  workspace == NULL makes the library
 * allocate it stream-ordered (cudaMallocAsync/cudaFreeAsync) for that call.
 */
#ifndef SEGTACO_H
#define SEGTACO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define SEGTACO_OK 0
#define SEGTACO_EINVAL (-1)      /* bad argument / malformed CSR              */
#define SEGTACO_ECUDA (-2)       /* a CUDA runtime call failed                */
#define SEGTACO_ENOMEM (-3)      /* device allocation failed                  */
#define SEGTACO_ETIMEOUT (-4)    /* a bounded device wait gave up             */
#define SEGTACO_EUNSUPPORTED (-5)/* shape / dtype combination not supported   */
#define SEGTACO_ECANCELLED (-6)  /* request cancelled (serving loop)          */
#define SEGTACO_EBUSY (-7)       /* admission refused (capacity)              */

/* ---- schedules (segTACO's 2x2 space, gpu_kernels.cuh:11-93) ------------ */
#define SEGTACO_AUTO (-1)
#define SEGTACO_RB_SR 0 /* row-balanced, sequential reduction     (spmm_rb_sr.h) */
#define SEGTACO_RB_PR 1 /* row-balanced, parallel reduction       (spmm_rb_pr.h) */
#define SEGTACO_EB_SR 2 /* element-balanced, sequential reduction (spmm_eb_sr.h) */
#define SEGTACO_EB_PR 3 /* element-balanced, parallel reduction   (spmm_eb_pr.h) */

/* ---- dense operand types ------------------------------------------------ */
#define SEGTACO_F32 0
#define SEGTACO_BF16 1 /* bf16 bit patterns (uint16), FP32 accumulation */

/* ---- flags ---------------------------------------------------------------- */
#define SEGTACO_FLAG_L2_HINTS 1u  /* gathered B rows evict_last in L2               */
#define SEGTACO_FLAG_PARTITION_READY 2u /* workspace holds segtaco_spmm_partition()'s
                                           output for this A, C, N and config: skip it */
#define SEGTACO_FLAG_SMEM_RING 4u /* gather B rows into a shared-memory ring with
                                     cp.async (16-byte vectors only) instead of loading
                                     them into registers */
#define SEGTACO_FLAG_TMA_BULK 8u  /* with SMEM_RING: fill the ring with cp.async.bulk
                                     (TMA) copies rather than 16-byte cp.async copies */

/* Tuning knobs.  Zero in a field means "choose automatically". */
typedef struct segtaco_config {
  int32_t schedule;       /* SEGTACO_RB_SR .. SEGTACO_EB_PR, or SEGTACO_AUTO    */
  int32_t col_tile;       /* W: dense columns per CTA column slab (multiple of vec) */
  int32_t vec;            /* dense elements per lane per load: 1, 2, 4 (bf16: 8)  */
  int32_t rows_per_unit;  /* rb: rows handled by one lane group / warp            */
  int32_t items_per_unit; /* eb: merge-path items (rows + nonzeros) per unit      */
  uint32_t flags;         /* SEGTACO_FLAG_*                                        */
  int32_t depth;          /* dense loads in flight per lane (0 = automatic, 4 or 8) */
} segtaco_config;

/* Library identity and build checks. */
const char *segtaco_version(void);
/* Status word of the device kernels on the current device: SEGTACO_OK, or
 * SEGTACO_ETIMEOUT if a kernel gave up a bounded wait (its output is then
 * incomplete).  clear != 0 resets it.  Synchronises the device. */
int segtaco_device_status(int clear);
/* Human-readable text of the last error raised on this host thread. */
const char *segtaco_last_error(void);
/* 1 when a CUDA device is usable by this process, else 0 (never fails). */
int segtaco_device_available(void);

/* Fill *cfg with the automatic choice for this shape (host-side statistics
 * only: M, K, nnz, N, and optionally max/mean row length if known >= 0). */
int segtaco_autotune_heuristic(int32_t M, int32_t K, int64_t nnz, int32_t N, int32_t b_dtype,
                               int64_t max_row_len, segtaco_config *cfg);

/* ---- SpMM: C = A * B  (the segTACO hot path) --------------------------- */
int segtaco_spmm_workspace_size(int32_t M, int32_t K, int64_t nnz, int32_t N, int32_t b_dtype,
                                const segtaco_config *cfg, size_t *bytes);
int segtaco_spmm(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr, const int32_t *col,
                 const float *vals, const void *B, int32_t b_dtype, int64_t ldb, float *C,
                 int64_t ldc, int32_t N, const segtaco_config *cfg, void *workspace,
                 size_t workspace_bytes, void *stream);

/* segtaco_spmm without any allocation (no counterpart in segTACO).  For
 * callers that cannot call cudaMalloc -- a host framework whose allocator
 * owns the device memory, a serving loop with a memory budget fixed at
 * start-up, a caller that cannot take an allocation's device-wide sync -- the
 * element-balanced schedules' scratch (merge-path chunk coordinates) comes
 * from a fixed 2 MiB array in the library's device memory instead of a
 * workspace.  Limit: at most 262,143 merge-path chunks, i.e.
 * ceil((M + nnz) / items_per_unit) <= 262,143 (M + nnz <= ~134M at the default
 * 512 items); larger problems get SEGTACO_EINVAL.  The first call on each
 * device looks up the array's address (cudaGetSymbolAddress) and should come
 * before any stream capture.  All calls share the array: calls that overlap on
 * the GPU race on it.  SEGTACO_FLAG_PARTITION_READY is not accepted. */
int segtaco_spmm_noalloc(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                         const int32_t *col, const float *vals, const void *B, int32_t b_dtype,
                         int64_t ldb, float *C, int64_t ldc, int32_t N,
                         const segtaco_config *cfg, void *stream);

/* The first half of segtaco_spmm, for callers that time or overlap it: the
 * merge-path partition of A into `workspace` (element-balanced schedules) and
 * the zeroing of the C rows that straddle chunk edges.  A following
 * segtaco_spmm with SEGTACO_FLAG_PARTITION_READY, the same config, workspace,
 * A, C and N runs only the product kernel.  Must be repeated before every
 * product (the zeroing belongs to one product).  No-op for rb schedules.
 * workspace must be the caller's (not NULL). */
int segtaco_spmm_partition(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                           float *C, int64_t ldc, int32_t N, int32_t b_dtype,
                           const segtaco_config *cfg, void *workspace, size_t workspace_bytes,
                           void *stream);

/* cuSPARSE SpMM (CSR_ALG2, row-major) on the same operands: the vendor
 * comparator segTACO verifies against (spmm_csr_gpu_cusparse.h:171-260).
 * Not a hot path; creates and destroys a cuSPARSE handle per call. */
int segtaco_vendor_spmm(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                        const int32_t *col, const float *vals, const float *B, int64_t ldb,
                        float *C, int64_t ldc, int32_t N, void *stream);

/* ---- batched SpMM: many uneven products, one persistent launch per kernel
 * variant, optionally replayed as a CUDA graph --------------------------- */
typedef struct segtaco_spmm_problem {
  int32_t M, K, N, b_dtype;
  int64_t nnz;
  const int32_t *row_ptr, *col; /* device CSR of A                      */
  const float *vals;            /* NULL: all ones                       */
  const void *B;                /* K x N, row-major, leading dim ldb    */
  int64_t ldb;
  float *C;                     /* M x N, row-major, leading dim ldc    */
  int64_t ldc;
} segtaco_spmm_problem;
typedef struct segtaco_batch segtaco_batch;
/* Plans `count` problems.  configs == NULL: each problem's config comes from
 * segtaco_autotune_heuristic on its row-length statistics (computed on the
 * device; the call synchronises `stream`).  The operand pointers are baked
 * into the batch: later runs compute with whatever the buffers then hold. */
int segtaco_batch_create(int32_t count, const segtaco_spmm_problem *problems,
                         const segtaco_config *configs, void *stream, segtaco_batch **out);
/* Enqueue every product of the batch on `stream`. */
int segtaco_batch_run(segtaco_batch *batch, void *stream);
/* Same, through a CUDA graph captured on the first call and replayed after. */
int segtaco_batch_run_graph(segtaco_batch *batch, void *stream);
/* Kernel-variant groups, total work items, and (if configs != NULL, count
 * entries) the configuration chosen for each problem. */
int segtaco_batch_info(const segtaco_batch *batch, int32_t *groups, int64_t *items,
                       segtaco_config *configs);
int segtaco_batch_destroy(segtaco_batch *batch);
/* Row-length statistics of a device CSR (the autotuner's input):
 * stats[0] max row length, [1] empty rows, [2] rows >= 32, [3] nonzeros in
 * rows >= 32.  Synchronises `stream`. */
int segtaco_row_stats(int32_t M, const int32_t *row_ptr, int64_t *stats, void *stream);

/* ---- partition arrays (exported so they can be checked bit-exactly) ---- */
/* segTACO's block starts: out[b] = taco_binarySearchBefore(row_ptr, 0, M, b*P)
 * for b = 0..ceil(nnz/P)  (gpu_library.h:185-240).  out has ceil(nnz/P)+1 entries. */
int segtaco_block_starts_taco(int32_t M, int64_t nnz, const int32_t *row_ptr, int32_t P,
                              int32_t *out, void *stream);
/* Canonical block starts: out[b] = last r in [0, M] with row_ptr[r] <= b*P. */
int segtaco_block_starts_canonical(int32_t M, int64_t nnz, const int32_t *row_ptr, int32_t P,
                                   int32_t *out, void *stream);
/* Merge-path split of {row ends} U {nonzeros} into chunks of D items:
 * out_x[c], out_y[c] for c = 0..nchunks with nchunks = max(1, ceil((M+nnz)/D)). */
int segtaco_merge_path(int32_t M, int64_t nnz, const int32_t *row_ptr, int64_t D,
                       int32_t *out_x, int32_t *out_y, void *stream);
/* Row of every nonzero (binary_search_segment_number semantics, gpu_library.h:138-152). */
int segtaco_row_ids(int32_t M, int64_t nnz, const int32_t *row_ptr, int32_t *out, void *stream);
/* Checks row_ptr[0]==0, monotone, row_ptr[M]==nnz and 0 <= col < K on the
 * device; returns SEGTACO_EINVAL (with the first bad index in the message)
 * if the CSR is malformed.  Synchronises the stream. */
int segtaco_csr_validate(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                         const int32_t *col, void *stream);

/* ---- SpMV: y = A x  (merge-path, N = 1) ------------------------------- */
int segtaco_spmv_workspace_size(int32_t M, int64_t nnz, size_t *bytes);
int segtaco_spmv(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr, const int32_t *col,
                 const float *vals, const float *x, float *y, void *workspace,
                 size_t workspace_bytes, void *stream);

/* ---- SDDMM: out[p] = vals[p] * <X[i,:], Y[j,:]> for every nonzero p=(i,j)
 * X is M x D, Y is K x D, row-major (ldx, ldy), f32 or bf16 (x_dtype).
 * vals == NULL means 1 (the plain sampled product). ------------------------ */
int segtaco_sddmm(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr, const int32_t *col,
                  const float *vals, const void *X, const void *Y, int32_t x_dtype, int64_t ldx,
                  int64_t ldy, int32_t D, float *out, void *stream);

/* ---- SpMSpV: y = A x, x sparse (nx entries), A given as CSC
 * (col_ptr[K+1], row_idx[nnz], vals) -- the CSR of A^T that segTACO's
 * experiment builds (spmspv_csr_gpu.h:37-43).  y (M) is overwritten. ----- */
int segtaco_spmspv(int32_t M, int32_t K, int64_t nnz, const int32_t *col_ptr,
                   const int32_t *row_idx, const float *vals, int32_t nx, const int32_t *x_idx,
                   const float *x_vals, float *y, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SEGTACO_H */
