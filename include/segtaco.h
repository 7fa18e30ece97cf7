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
#define SEGTACO_FLAG_ROW_WALK 16u /* walk each unit row by row (the default except
                                     for eb_sr; depth 4 or 8 loads in flight)    */
#define SEGTACO_FLAG_FLAT_WALK 32u /* walk each unit in batches of 32 nonzeros
                                      across rows (the default for eb_sr with
                                      16-byte vectors)                           */
#define SEGTACO_FLAG_LONG_ROWS 64u /* rb schedules with nnz >= 1M: rows of at
                                      least items_per_unit nonzeros are taken
                                      out of the row blocks (see
                                      items_per_unit).  rb_sr: long-row CTAs on
                                      a side stream the library forks from the
                                      call's stream and joins before returning
                                      (created by the first such call on a
                                      host thread and device; a call captured
                                      into a graph before that runs both
                                      kernels on the call's stream).  rb_pr:
                                      pieces of 4096 nonzeros inside the
                                      row-block launch, no side stream;
                                      segtaco_autotune_heuristic sets it when
                                      the longest row reaches 512 nonzeros     */

#define SEGTACO_FLAG_SLOT_WALK 256u /* eb schedules: every slot of a warp walks its
                                      own merge-path chunk (items_per_unit items,
                                      0 = 64) in merge order, each row of a chunk
                                      one sequential chain; rows cut by chunk
                                      edges are combined by atomics */
#define SEGTACO_FLAG_WINDOW 128u /* rb schedules, matrices whose nonzeros lie
                                     near the diagonal (H = items_per_unit; 0 =
                                     32).  rb_pr with N >= 64 (a multiple of 16),
                                     C 16-byte aligned and ldc a multiple of 4:
                                     the band kernel -- 32-row blocks with B rows
                                     [i0 - H, i0 + 32 + H) of a 64-column slab in
                                     shared memory (one TMA tensor copy), the
                                     block's in-band nonzeros as a dense tile, 4 x
                                     4 register tiles, off-band nonzeros gathered;
                                     32 + 2H <= 256.  Otherwise each CTA of 4 *
                                     rows_per_unit rows stages B rows [i0 - H,
                                     i1 + H) of its slab and gathers rows inside
                                     that window from it (4 * rows_per_unit + 2H
                                     <= 256).  Needs B 16-byte aligned and ldb *
                                     element size a multiple of 16; otherwise
                                     ignored.  Not with LONG_ROWS.
                                     segtaco_autotune_heuristic reads the bit as
                                     "rows lie near the diagonal" and keeps it
                                     for rb_pr's band kernel                    */

/* Tuning knobs.  Zero in a field means "choose automatically". */
typedef struct segtaco_config {
  int32_t schedule;       /* SEGTACO_RB_SR .. SEGTACO_EB_PR, or SEGTACO_AUTO    */
  int32_t col_tile;       /* W: dense columns per CTA column slab (multiple of vec) */
  int32_t vec;            /* dense elements per lane per load: 1, 2, 4, 8 (bf16
                             also 16); 8 fp32 / 16 bf16 is one 32-byte load (B
                             32-byte aligned).  The planner narrows it to what
                             N, ldb and the pointers allow                     */
  int32_t rows_per_unit;  /* rb: rows handled by one lane group / warp            */
  int32_t items_per_unit; /* eb: merge-path items (rows + nonzeros) per unit
                             (0: 512, fewer for small products).
                             rb with SEGTACO_FLAG_LONG_ROWS and nnz >= 1M:
                             rows of at least this many nonzeros (0 = 2048
                             for rb_sr, 512 for rb_pr).
                             rb_sr: to long-row CTAs that stage B rows in
                             shared memory for the whole CTA, each column
                             still summed in storage order, beside the
                             row-block kernel.  rb_pr: split into pieces of
                             4096 nonzeros (2048 with k_parts > 1) that warps
                             of the row-block launch take over the same
                             column slabs; each piece's
                             partial row goes to the workspace and the last
                             piece of a row sums them in piece order, so the
                             result does not vary from run to run          */
  uint32_t flags;         /* SEGTACO_FLAG_*                                        */
  int32_t depth;          /* row walk: dense loads in flight per lane (0 = 4, 4, 8) */
  int32_t k_parts;        /* rb_pr pieces: passes over ranges of B's rows, 1 .. 8
                             (0: one).  With more than one the pieces (of
                             2048 nonzeros) run in a launch of their own
                             before the row blocks, pass p taking the
                             nonzeros of columns [p*Kp, (p+1)*Kp), Kp = K /
                             k_parts rounded up, so that a pass gathers from
                             that range of B only; columns sorted within each
                             row keep a pass inside its range (unsorted rows
                             stay correct, without that locality); every
                             (piece, pass) leaves a partial row, summed in
                             order.  Opt-in: the short rows then no longer
                             overlap the pieces                            */
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
 * only: M, K, nnz, N, and optionally max/mean row length if known >= 0).
 * On input, cfg->schedule may request a schedule (else SEGTACO_AUTO) and
 * cfg->flags & SEGTACO_FLAG_WINDOW says that most nonzeros lie within 32 of
 * the diagonal (segtaco_band_stats): row-block schedules then get the staged
 * B window.  Every other input field is ignored and overwritten. */
int segtaco_autotune_heuristic(int32_t M, int32_t K, int64_t nnz, int32_t N, int32_t b_dtype,
                               int64_t max_row_len, segtaco_config *cfg);

/* ---- SpMM: C = A * B  (the segTACO hot path) --------------------------- */
/* The plan segtaco_spmm would run for these arguments, as text: schedule,
 * kernel (rows, chunks, long_rows, window, tma_ring), lanes V x G, slab width
 * W, slabs, walk, window halo, rows per unit.  C is taken as dense (ldc = N,
 * aligned); B's alignment and ldb matter. */
int segtaco_spmm_plan_name(int32_t M, int32_t K, int64_t nnz, int32_t N, int32_t b_dtype,
                           const void *B, int64_t ldb, const segtaco_config *cfg, char *out,
                           size_t len);
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
 * element-balanced schedules' scratch (merge-path chunk coordinates) and
 * the row-block schedules' list of long rows come from a fixed 2 MiB array in
 * the library's device memory instead of a workspace (rb_pr's pieces, whose
 * partial rows do not fit there, give way to the long-row CTAs; a list of more
 * than 262,143 entries is not made: every row then stays in the row-block
 * kernel).
 * Limit: at most 262,143 merge-path chunks, i.e. ceil((M + nnz) /
 * items_per_unit) <= 262,143 (M + nnz <= ~134M at the default 512 items);
 * larger problems get SEGTACO_EINVAL.  The first call on each
 * device looks up the array's address (cudaGetSymbolAddress) and should come
 * before any stream capture; the address is kept for the process, so a
 * cudaDeviceReset of a device that served this call is not supported.  With
 * SEGTACO_FLAG_LONG_ROWS the long-row CTAs run on `stream` itself (no side
 * stream or events are created).  All calls share the array: calls that
 * overlap on the GPU race on it.  SEGTACO_FLAG_PARTITION_READY is not
 * accepted. */
int segtaco_spmm_noalloc(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                         const int32_t *col, const float *vals, const void *B, int32_t b_dtype,
                         int64_t ldb, float *C, int64_t ldc, int32_t N,
                         const segtaco_config *cfg, void *stream);

/* The first half of segtaco_spmm, for callers that time or overlap it: the
 * merge-path partition of A into `workspace` (element-balanced schedules) and
 * the zeroing of the C rows that straddle chunk edges.  A following
 * segtaco_spmm with SEGTACO_FLAG_PARTITION_READY, the same config, workspace,
 * A, C and N runs only the product kernel.  Must be repeated before every
 * product (the zeroing belongs to one product).  For rb schedules with
 * long rows (see items_per_unit) it lists the long rows (rb_sr) or their
 * pieces (rb_pr) instead, and that list may serve repeated products; no-op
 * for the other rb cases.  workspace must be the caller's (not NULL). */
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
/* Enqueue every product of the batch on `stream` (its kernel groups fork onto
 * the batch's own side streams and join `stream` before the run ends).  Runs
 * of one batch share its device buffers and side streams: issue them from one
 * host thread, one after another in stream order. */
int segtaco_batch_run(segtaco_batch *batch, void *stream);
/* Same, through a CUDA graph captured on the first call and replayed after. */
int segtaco_batch_run_graph(segtaco_batch *batch, void *stream);
/* Same as segtaco_batch_run, with problems released in order by a gate:
 * problem i may run once *gate > i.  `gate` is device memory or mapped host
 * memory that the caller raises while the launch runs.  Waits are bounded:
 * after `timeout_ns` (at most 60 s) without release the kernels record
 * SEGTACO_ETIMEOUT, read and cleared by segtaco_device_status(1), and end;
 * products of problems never released are then not written. */
int segtaco_batch_run_gated(segtaco_batch *batch, const int64_t *gate, int64_t timeout_ns,
                            void *stream);
/* Kernel-variant groups, total work items, and (if configs != NULL, count
 * entries) the configuration chosen for each problem. */
int segtaco_batch_info(const segtaco_batch *batch, int32_t *groups, int64_t *items,
                       segtaco_config *configs);
int segtaco_batch_destroy(segtaco_batch *batch);
/* ---- Serving loop (segtaco_server_*) -------------------------------------
 * A native scheduler thread admits SpMM and SDDMM requests as they arrive.
 * CSR operands stay resident in a device cache keyed by matrix id (LRU, capped
 * by bytes and by free HBM).  Whenever one of `slots` streams is idle, the
 * pending requests that fit (staging bytes, cache room) form the next batch:
 * their SpMMs run in one persistent batched launch, their SDDMMs beside it, and
 * copies of one batch overlap the kernels of the others.  Failures complete a
 * request with a status; nothing exits the process. */
#define SEGTACO_OP_SPMM 0
#define SEGTACO_OP_SDDMM 1

#define SEGTACO_SERVER_PER_CALL 1u    /* one request per batch through the plain
                                         segtaco_spmm path (per-call comparator)  */
#define SEGTACO_SERVER_FAKE_DEVICE 2u /* tests of the host logic only: host memory
                                         stands in for the device and no kernel
                                         runs, so outputs are NOT written         */

#define SEGTACO_REQ_DEVICE_DENSE 1u   /* dense operands and output are device
                                         pointers (no staging copies)             */

typedef struct segtaco_server_config {
  int32_t max_batch;      /* requests per batch (0: 64)                           */
  int32_t slots;          /* batches in flight, one stream each (0: 4); measured
                             on GB300 with the served stream of the bench: 4 x 64
                             beat 3 x 256, 6 x 32 and 8 x 16 overall             */
  int64_t cache_bytes;    /* device CSR cache cap (0: 120 GB), clamped to the
                             free HBM at creation minus reserve_bytes             */
  int64_t staging_bytes;  /* device bytes of staged dense operands in flight
                             (0: 8 GB)                                            */
  int64_t reserve_bytes;  /* HBM left free (0: 2 GB)                              */
  uint32_t flags;         /* SEGTACO_SERVER_*                                     */
  int32_t fail_alloc_at;  /* fault injection: the n-th device allocation
                             (1-based) fails with ENOMEM; 0 = never               */
  int32_t fake_delay_us;  /* FAKE_DEVICE: time a batch stays in flight            */
  int32_t reserved;
} segtaco_server_config;

typedef struct segtaco_request {
  int32_t op;       /* SEGTACO_OP_*                                               */
  int32_t dtype;    /* dense operand type (SEGTACO_F32 / SEGTACO_BF16)            */
  int64_t matrix;   /* id given to segtaco_server_add_matrix                      */
  int32_t N;        /* SpMM: columns of B and C; SDDMM: D                         */
  uint32_t flags;   /* SEGTACO_REQ_*                                              */
  const void *B;    /* SpMM: B, K x N; SDDMM: X, M x D (row-major, dense)         */
  const void *Y;    /* SDDMM: Y, K x D; unused for SpMM                           */
  float *out;       /* SpMM: C, M x N; SDDMM: nnz values                          */
} segtaco_request;

typedef struct segtaco_server_stats {
  int64_t submitted, completed, failed, cancelled, pending, in_flight;
  int64_t batches, cache_hits, cache_misses, evictions, cache_bytes;
  int64_t h2d_bytes, d2h_bytes;
  double p50_us, p99_us, max_us, mean_us; /* arrival -> completion, requests
                                             completed OK since the last reset   */
  double span_s;                          /* first arrival -> last completion     */
  double mean_batch;                      /* requests per batch                   */
} segtaco_server_stats;

typedef struct segtaco_server segtaco_server;
int segtaco_server_create(const segtaco_server_config *cfg, segtaco_server **out);
/* Registers host CSR arrays under `id` (checked here: row_ptr monotone from 0
 * to nnz, 0 <= col < K).  The arrays must stay valid while the server lives;
 * pinned host memory makes their uploads asynchronous.  vals NULL: all ones. */
int segtaco_server_add_matrix(segtaco_server *srv, int64_t id, int32_t M, int32_t K,
                              int64_t nnz, const int32_t *row_ptr, const int32_t *col,
                              const float *vals);
/* Queues a request; *ticket identifies it.  Requests naming an unknown matrix
 * or an unsupported shape are refused here with SEGTACO_EINVAL. */
int segtaco_server_submit(segtaco_server *srv, const segtaco_request *req, int64_t *ticket);
/* Open-loop arrivals: submits reqs[i] at arrival_us[i] microseconds after the
 * call starts (latency counts from that instant); returns once all are queued. */
int segtaco_server_replay(segtaco_server *srv, int32_t n, const segtaco_request *reqs,
                          const double *arrival_us, int64_t *tickets);
/* Waits up to timeout_ms (< 0: forever) for a request: SEGTACO_OK with its
 * final status in *status, or SEGTACO_ETIMEOUT if still running. */
int segtaco_server_wait(segtaco_server *srv, int64_t ticket, int32_t timeout_ms,
                        int32_t *status);
/* Waits until nothing is pending or in flight. */
int segtaco_server_drain(segtaco_server *srv, int32_t timeout_ms);
/* Cancels a request not yet admitted (SEGTACO_OK; it completes with
 * SEGTACO_ECANCELLED); SEGTACO_EBUSY once it is admitted or done. */
int segtaco_server_cancel(segtaco_server *srv, int64_t ticket);
int segtaco_server_get_stats(segtaco_server *srv, int32_t reset, segtaco_server_stats *out);
/* Stops the scheduler: pending requests complete with SEGTACO_ECANCELLED,
 * batches in flight finish first. */
int segtaco_server_destroy(segtaco_server *srv);

/* Diagnostic: n gathers of row_bytes-byte rows (16..512, a power of two) at
 * pseudo-random rows of buf (rows x row_bytes bytes, 16-byte aligned) by a
 * persistent grid of `blocks` CTAs of 256 threads (0: one full resident wave).  Timing it gives the
 * random-gather ceiling that bounds SpMM with scattered columns. */
int segtaco_probe_gather(const void *buf, int64_t rows, int32_t row_bytes, int64_t n,
                         uint32_t seed, float *sink, int32_t blocks, void *stream);

/* Diagnostic: `bytes` from src to dst by the SM-driven copy kernel the serving
 * loop uses (either side may be pinned host memory); `desc` is 64 bytes of
 * device scratch for the segment descriptor. */
int segtaco_probe_copy(void *dst, const void *src, int64_t bytes, void *desc, int32_t blocks,
                       void *stream);

/* ---- MatrixMarket ingest (host) ------------------------------------------ */
#define SEGTACO_MTX_SEGTACO_PATTERN 1u /* the CSR segTACO's read_mtx_file builds
                                          (symmetric files mirrored, sorted and
                                          deduplicated, then cut to the header's
                                          entry count; others sorted, duplicates
                                          kept); default: all symmetries mirrored,
                                          duplicates summed                     */
#define SEGTACO_MTX_VALUES_FILE 0      /* values from the file (pattern: 1)     */
#define SEGTACO_MTX_VALUES_SEGTACO 1   /* {0, 0.1, 0.2} like segTACO's
                                          fill_random, from a seeded generator  */
#define SEGTACO_MTX_VALUES_ONES 2

typedef struct segtaco_host_csr {
  int32_t M, K;
  int64_t nnz;
  int32_t *row_ptr, *col; /* malloc'd; free with segtaco_host_csr_free */
  float *vals;
} segtaco_host_csr;
/* Reads a MatrixMarket coordinate file into a host CSR (columns sorted within
 * rows).  Replaces segTACO's read_mtx_file + fill_random (ds.h:183-274). */
int segtaco_mtx_read(const char *path, uint32_t flags, int32_t values, uint64_t seed,
                     segtaco_host_csr *out);
void segtaco_host_csr_free(segtaco_host_csr *csr);

/* Row-length statistics of a device CSR (the autotuner's input):
 * stats[0] max row length, [1] empty rows, [2] rows >= 32, [3] nonzeros in
 * rows >= 32.  Synchronises `stream`. */
int segtaco_row_stats(int32_t M, const int32_t *row_ptr, int64_t *stats, void *stream);
/* Number of nonzeros of A (device CSR) within `halo` columns of the diagonal
 * (row i against column i*K/M), into *in_band (host).  Synchronises `stream`.
 * The autotuner's locality test for SEGTACO_FLAG_WINDOW. */
int segtaco_band_stats(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                       const int32_t *col, int32_t halo, int64_t *in_band, void *stream);

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

/* SDDMM kernels: element-balanced blocks of nonzeros, one per warp; the
 * fixed-shape kernel (each dot product split over `lanes` lanes with one or
 * two 32-byte, or up to four 16-byte, loads of X[i] and Y[j] per lane) where
 * D and the operands' alignment allow it, else the general kernel (V-wide
 * vectors, lanes covering D) -- segTACO's two schedules are the row-warp
 * sddmm_csr_gpu_warp and the element-balanced sddmm_csr_gpu_taco
 * (sddmm_csr_gpu_taco.h:46-68, 120-148). */
#define SEGTACO_SDDMM_AUTO 0
#define SEGTACO_SDDMM_FIXED 1
#define SEGTACO_SDDMM_GENERAL 2
#define SEGTACO_SDDMM_BAND 3 /* rows near the diagonal: 32-row blocks, the dense tile of
                                their dot products with the Y window of 96 rows around
                                the diagonal, off-band nonzeros from global memory;
                                D = 64, ldx and ldy multiples of 4, X and Y aligned to
                                4 elements (otherwise ignored) */
typedef struct segtaco_sddmm_config {
  int32_t kernel;     /* SEGTACO_SDDMM_AUTO / _FIXED / _GENERAL / _BAND             */
  int32_t block_nnz;  /* nonzeros per warp block, a power of two 32 .. 4096 (0: 256) */
  int32_t lanes;      /* lanes per dot product (0: from D; power of two); a count
                         the fixed kernel has no shape for (one 32-byte load per
                         lane, two from 4 lanes, or four 16-byte loads) is
                         ignored                                               */
  int32_t reserved;
} segtaco_sddmm_config;
/* The library's SDDMM configuration for this shape: the block size so that a
 * small problem still fills the GPU (at least two waves of warps); the kernel
 * family and the lanes per dot product follow from D, the element type and
 * the operands' alignment at launch.  cfg->kernel == SEGTACO_SDDMM_BAND on
 * entry reports that the nonzeros lie near the diagonal (segtaco_band_stats):
 * it is kept for D = 64.  max_row_len (< 0 if unknown) is accepted and not
 * used. */
int segtaco_sddmm_autotune(int32_t M, int32_t K, int64_t nnz, int32_t D, int32_t x_dtype,
                           int64_t max_row_len, segtaco_sddmm_config *cfg);
/* segtaco_sddmm with an explicit configuration (NULL: segtaco_sddmm_autotune
 * on the shape alone). */
int segtaco_sddmm_ex(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                     const int32_t *col, const float *vals, const void *X, const void *Y,
                     int32_t x_dtype, int64_t ldx, int64_t ldy, int32_t D, float *out,
                     const segtaco_sddmm_config *cfg, void *stream);

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
