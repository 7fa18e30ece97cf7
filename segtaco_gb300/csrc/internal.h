// internal.h -- host-side plumbing shared by the translation units of libsegtaco.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "segtaco.h"

namespace segtaco {

// Records a message for segtaco_last_error() and returns `code`.
int set_error(int code, const char *fmt, ...);
// cudaGetLastError() after a launch -> status (message names the kernel).
int check_launch(const char *what);
// A CUDA runtime result -> status.
int check_cuda(cudaError_t e, const char *what);

#define SEGTACO_TRY(expr)          \
  do {                             \
    int _st = (expr);              \
    if (_st != SEGTACO_OK) return _st; \
  } while (0)

// Scratch memory for one call: either the caller's buffer or a stream-ordered
// allocation released at the end of the call.
class Scratch {
 public:
  Scratch(void *user, size_t user_bytes, cudaStream_t s) : user_(user), cap_(user_bytes), s_(s) {}
  ~Scratch();
  // Carve `bytes` (256-byte aligned) out of the scratch; allocates when the
  // caller gave none.  Returns SEGTACO_OK or an error status.
  int reserve(size_t total_bytes);
  void *take(size_t bytes);

 private:
  void *user_;
  size_t cap_;
  cudaStream_t s_;
  void *owned_ = nullptr;
  char *base_ = nullptr;
  size_t used_ = 0, total_ = 0;
};

inline size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

// ---- launchers (partition.cu) ----
int launch_merge_path(const int *row_ptr, int M, long long nnz, long long D, long long nchunks,
                      int *px, int *py, float *C, long long ldc, int N, cudaStream_t s);
int launch_block_starts_taco(const int *row_ptr, int M, int P, long long nblk, int *out,
                             cudaStream_t s);
int launch_block_starts_canonical(const int *row_ptr, int M, int P, long long nblk, int *out,
                                  cudaStream_t s);
int launch_row_ids(const int *row_ptr, int M, int *out, cudaStream_t s);
int launch_validate(const int *row_ptr, int M, int K, long long nnz, const int *col, int *err,
                    cudaStream_t s);

// ---- SpMM kernel launch description (spmm_*.cu) ----
struct SpmmLaunch {
  int dtype;     // SEGTACO_F32 / SEGTACO_BF16
  int V, G;      // vector width (elements) and lanes per slot (P = 32/G slots)
  bool l2_hints;
  int M, K, N;
  long long nnz;
  const int *row_ptr, *col;
  const float *val;
  const void *B;
  long long ldb;
  float *C;
  long long ldc;
  const int *part_x, *part_y;  // chunks only
  long long units;             // warps: merge-path chunks or row blocks
  int rows_per_unit;           // row blocks only
  bool use_tma;                // gather B into a shared-memory ring (spmm_tma.cuh)
  bool bulk_copies;            // ... with cp.async.bulk (TMA) rather than cp.async
  bool deep;                   // row walk: 8 sixteen-byte loads in flight per lane
  int walk;                    // kWalkRows / kWalkRowsDeep / kWalkFlat (spmm_kernels.cuh)
  int long_row = 0;            // rb: rows of >= long_row nonzeros go to spmm_long.cu
  int carveout = -1;           // >= 0: preferred shared-memory carveout (%) of the launch
  bool no_fork = false;        // rb long rows: both kernels on the call's stream (no side
                               // stream or events are created)
  int window_halo = -1;        // >= 0: rb rows with B rows [i0 - halo, i1 + halo) of each
                               // row block staged by TMA (spmm_window.cu)
  int band_halo = -1;          // >= 0: rb_pr banded row blocks (spmm_band_kernel)
  // rb_pr long rows as pieces of piece_len nonzeros in the row-block launch
  // (spmm_long.cu): (row, first nonzero) pairs, their count, the list capacity.
  int piece_len = 0;
  const int *pieces = nullptr;
  const int *piece_count = nullptr;
  unsigned *piece_ctr = nullptr;  // per (first piece of a row, slab) counters
  float *piece_part = nullptr;    // partial rows, piece_ld floats per piece
  long long piece_cap = 0;        // list entries (both parts)
  long long piece_multi = 0;      // entries of the front part (rows of several pieces)
  long long piece_ld = 0;
  // > 1: the pieces run in a launch of their own before the row blocks, in
  // piece_parts passes over ranges of B's rows (spmm_pieces_pass)
  int piece_parts = 1;
  unsigned long long *piece_queue = nullptr;  // the passes' work counter (8-byte aligned)
};
// One launcher per (dense type, unit kind); each switches over (V, G).
int launch_spmm_f32_rows(const SpmmLaunch &L, cudaStream_t s);
int launch_spmm_f32_chunks(const SpmmLaunch &L, cudaStream_t s);
int launch_spmm_bf16_rows(const SpmmLaunch &L, cudaStream_t s);
int launch_spmm_bf16_chunks(const SpmmLaunch &L, cudaStream_t s);
// rb_pr's pieces in piece_parts passes (a persistent launch before the row
// blocks).
int launch_spmm_pieces_f32(const SpmmLaunch &L, cudaStream_t s);
int launch_spmm_pieces_bf16(const SpmmLaunch &L, cudaStream_t s);
// TMA variants: 16-byte lane vectors only (fp32 x 4, bf16 x 8), any G.
int launch_spmm_tma_f32(const SpmmLaunch &L, bool rows, cudaStream_t s);
int launch_spmm_tma_bf16(const SpmmLaunch &L, bool rows, cudaStream_t s);
// Device status word of the TMA kernels on the current device.
int tma_status_ptr(int **out);
// Row blocks with their B window staged in shared memory (rb only).
int launch_spmm_window(const SpmmLaunch &L, cudaStream_t s);
// Banded row blocks of rb_pr: 32 rows x 64 columns per CTA, the band of A as a
// dense tile, B's band window by TMA (spmm_window.cu).
int launch_spmm_band(const SpmmLaunch &L, cudaStream_t s);
bool window_variant_exists(int dtype, int V, int G);
int launch_band_stats(const int *row_ptr, const int *col, int M, int K, int halo,
                      unsigned long long *out, cudaStream_t s);

// Resolved plan of one SpMM call (api.cu).
struct SpmmPlan {
  int schedule, V, G, W, slabs;
  long long rows_per_unit;   // rb
  long long items_per_unit;  // eb (merge-path D)
  long long nchunks;         // eb
  bool l2_hints;
  bool use_tma;
  bool bulk_copies;
  bool deep;
  int walk;                  // kWalkRows / kWalkRowsDeep / kWalkFlat
  int long_row;              // rb: long-row threshold (0: every row in the row-block kernel)
  bool no_fork = false;      // rb long rows: no side stream (segtaco_spmm_noalloc)
  int window_halo = -1;      // rb: >= 0 stages each row block's B window (spmm_window.cu)
  int band_halo = -1;        // rb_pr: >= 0 banded row blocks with a dense band tile
  int piece_len = 0;         // rb_pr: long rows split into pieces of this many nonzeros
  int piece_parts = 1;       // rb_pr pieces: passes over ranges of B's rows (> 1: a launch
                             // of their own before the row blocks)
  long long px_entries;      // int32 entries of the first workspace array (eb: chunk-edge
                             // rows; rb long rows: the list of long rows)
  long long py_entries;      // ... of the second (eb: chunk-edge nonzeros; long rows: counters)
  size_t workspace;          // bytes
};
// `pieces` false: rb_pr long rows go to the long-row CTAs, as for rb_sr.
int plan_spmm(int M, int K, long long nnz, int N, int b_dtype, long long ldb, long long ldc,
              const void *B, const float *C, const segtaco_config *cfg, SpmmPlan *plan,
              bool pieces = true);
// Runs a planned SpMM with partition arrays already in `px/py` (eb) or none.
int run_spmm_planned(const SpmmPlan &plan, int M, int K, long long nnz, const int *row_ptr,
                     const int *col, const float *vals, const void *B, int b_dtype, long long ldb,
                     float *C, long long ldc, int N, int *px, int *py, cudaStream_t s,
                     bool partition_ready = false);

// ---- side ops (sddmm.cu, spmspv.cu; SpMV runs the SpMM kernel with N = 1) ----
// One SDDMM problem of a multi-problem launch (device array): block b of the
// launch with blk_begin <= b < blk_begin + ceil(nnz / sddmm_block_nnz()).
struct SddmmProblem {
  int M;
  long long nnz;
  const int *row_ptr, *col;
  const float *val;
  const void *X, *Y;
  long long ldx, ldy;
  float *out;
  const int *starts;  // block starts of row_ptr (sddmm_block_nnz() nonzeros each)
  long long blk_begin;
};
// Kernel shape of an SDDMM: family 0 = the general kernel (V-wide vectors),
// 1 = fp32 32-byte lanes, 2 = bf16 32-byte lanes, 3 = 16-byte lanes; problems
// of one non-zero family and (KI, G) can share a multi-problem launch.
struct SddmmShape {
  int family = 0, KI = 0, G = 0, V = 1;
};
SddmmShape sddmm_shape(int x_dtype, int D, long long ldx, long long ldy, const void *X,
                       const void *Y, int lanes = 0);
// One launch over `nprobs` problems of the fixed shape `sh` (device array
// `probs`, blocks 0 .. total_blocks - 1); their block starts must be ready.
int launch_sddmm_multi(const SddmmShape &sh, int x_dtype, const SddmmProblem *probs, int nprobs,
                       long long total_blocks, cudaStream_t s);
// `starts_ready`: `starts` already holds the block starts of this row_ptr (a
// cached matrix), so only the product is launched.
// SDDMM of a banded matrix (sddmm_band.cu): 32-row blocks, the dense tile of
// X-block x Y-window dot products, off-band nonzeros from global memory.  D =
// 64, ldx and ldy multiples of 4, X and Y aligned to 4 elements.
bool sddmm_band_applies(int x_dtype, int D, long long ldx, long long ldy, const void *X,
                        const void *Y);
int launch_sddmm_band(int M, int K, long long nnz, const int *row_ptr, const int *col,
                      const float *val, const void *X, const void *Y, int x_dtype, long long ldx,
                      long long ldy, int D, float *out, cudaStream_t s);
int launch_sddmm(int M, long long nnz, const int *row_ptr, const int *col, const float *val,
                 const void *X, const void *Y, int x_dtype, long long ldx, long long ldy, int D,
                 float *out, int *starts, int P, long long nblk, cudaStream_t s,
                 bool starts_ready = false, int lanes = 0,
                 int kernel = 0);
// ---- long rows of the row-block schedules (spmm_long.cu) ----
// Row-block products below this many nonzeros walk every row in the row-block
// kernel: the list pass and the fork would cost more than a long row there.
constexpr long long kLongRowsMinNnz = 1000000;
// Merge-path items per chunk of a product launched alone: 512 (a warp's
// chunk), halved down to 32 while the grid would hold fewer than 4,096
// chunks, so that small products still fill the 152 SMs.  Measured on GB300,
// 16,384 x 16,384 with 16 nonzeros per row, N = 32 (partition + product):
// eb_sr 0.0462 -> 0.0240 ms and eb_pr 0.0295 -> 0.0203 ms with 64 items.
inline long long default_chunk_items(long long M, long long nnz) {
  long long D = 512;
  while (D > 32 && (M + nnz) / D < 4096) D >>= 1;
  return D;
}
// Default long-row threshold (items_per_unit = 0).  Measured on GB300 (1M x 1M
// power law, N = 128, Zipf 1.8 / 1.922, rb_sr): 1024: 2.33 / 1.45 ms, 2048:
// 2.27 / 1.44, 4096: 2.23 / 1.46.
constexpr long long kLongRowDefault = 2048;
inline long long long_row_threshold(const segtaco_config &c) {
  return c.items_per_unit > 0 ? c.items_per_unit : kLongRowDefault;
}
// rb_pr splits every row of >= T nonzeros (default kPieceThreshold) into
// pieces of S = kPieceLen nonzeros.  Measured on GB300, 1M x 1M power law,
// N = 128, T = 512, 64 short rows per warp: S = 512 1.193 ms, 1024 1.159,
// 2048 1.129, 4096 1.114, 8192 1.120, 16384 1.367 (too few pieces to spread
// the longest rows); T = 256 / 1024 at S = 4096: 1.135 / 1.134 ms.  The
// 10M-nonzero Zipf 1.922 matrix: 0.689 ms at S = 4096, 0.769 at 8192.  Rows
// of more than S nonzeros (n = ceil(len / S) <= 2 len / S pieces each, at most
// 2 nnz / S in all) take the front of the piece list, each piece with a
// partial row and a counter per column slab; rows of T .. S nonzeros (at most
// nnz / T) are one piece each at the back and store directly.  The workspace,
// in int32 entries from the start of the first array: the (row, first
// nonzero) pairs, the counters, the partial rows (`ld` floats each, 256-byte
// aligned).
constexpr long long kPieceLen = 4096;
constexpr long long kPieceThreshold = 512;
// Pieces of the passes over ranges of B's rows (piece_parts > 1): shorter, so
// that each (pass, slab) holds enough of them for every warp of the grid
// (two passes: 512 1.318 ms, 1024 1.147, 2048 1.081, 4096 1.182).
constexpr long long kPassPieceLen = 2048;
//
// With R > 1 passes over ranges of B's rows (spmm_pieces_pass) every piece
// leaves R partial rows, one per pass, so every row (one-piece rows too) gets
// counters and R partial rows per piece: counters for all `cap` entries, the
// partial rows at (entry * R + pass).
struct PieceLayout {
  long long multi, cap, ld, ctr, part, entries;
};
inline PieceLayout piece_layout(long long nnz, long long T, long long S, int slabs, int W,
                                int parts = 1) {
  PieceLayout p;
  p.multi = 2 * nnz / S + 1;
  p.cap = p.multi + nnz / T + 1;
  p.ld = (long long)slabs * W;
  p.ctr = 2 * p.cap;
  const long long rows = parts > 1 ? p.cap : p.multi;  // entries with counters / partials
  p.part = (p.ctr + rows * slabs + 63) / 64 * 64;
  p.entries = p.part + rows * (parts > 1 ? parts : 1) * p.ld;
  return p;
}
// Passes over ranges of B's rows for rb_pr's pieces (segtaco_config.k_parts,
// at most 8; one by default).  Measured on GB300, 1M x 1M power law, N = 128:
// the long rows alone (4394 rows of >= 512 nonzeros, each range an SpMM of
// its own) take 0.567 ms in one pass, 0.423 in two, 0.426 in four; but the
// passes then run apart from the short rows, which in one pass fill the
// warps the pieces leave idle, and the whole product gains little or loses:
// rb_pr 1.098-1.118 ms in one pass, in two 1.081 (pieces of 2048), 1.147
// (1024), 1.182 (4096); the 10M-nonzero Zipf 1.922 matrix 0.683-0.691 ms in
// one pass, 0.739-0.850 in two.
constexpr int kMaxPieceParts = 8;
// The two parts of the long-row list for threshold T: rows of >= 8T nonzeros
// (at most nnz / 8T of them) and rows of T .. 8T-1 (at most nnz / T).
inline void long_list_caps(long long nnz, long long T, long long *hi, long long *lo) {
  *hi = nnz / (8 * T) + 1;
  *lo = nnz / T + 1;
}
// Lists the rows of >= long_row nonzeros into `list` (long_list_caps entries)
// and their counts into counters[0..1] (`counters`: 4 int32, cleared here).
int launch_long_rows_list(const int *row_ptr, int M, long long nnz, int long_row, int *list,
                          int *counters, cudaStream_t s);
// The long-row CTAs for the listed rows, on a side stream forked from `s`, and
// the row-block kernel `L` (L.long_row set: it skips those rows) on `s`.
int launch_spmm_long_rows(const SpmmLaunch &L, const int *list, int *counters, cudaStream_t s);
// rb_pr: lists every row of >= long_row nonzeros as pieces of piece_len
// nonzeros into `pieces` (piece_layout: the pairs, the counters of each row's
// first piece cleared here; with parts > 1 those of one-piece rows too),
// counting the front and back parts in count[0] and count[1] (cleared here).
int launch_long_pieces_list(const int *row_ptr, int M, long long nnz, int long_row, int piece_len,
                            int slabs, int W, int parts, int *pieces, int *count, cudaStream_t s);
// Multiprocessors of the current device (cached per device).
int device_sms();

int launch_spmspv(int M, int K, const int *col_ptr, const int *row_idx, const float *val, int nx,
                  const int *x_idx, const float *x_vals, float *y, cudaStream_t s);

}  // namespace segtaco
