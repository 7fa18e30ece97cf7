// api.cu -- the extern "C" entry points of include/segtaco.h, argument checks,
// scratch handling and the SpMM planner (schedule / slab width / vector width).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "internal.h"

namespace segtaco {

static thread_local std::string g_last_error;

int set_error(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return SEGTACO_OK;
  const int code = (e == cudaErrorMemoryAllocation) ? SEGTACO_ENOMEM : SEGTACO_ECUDA;
  return set_error(code, "%s: %s", what, cudaGetErrorString(e));
}

int check_launch(const char *what) { return check_cuda(cudaGetLastError(), what); }

Scratch::~Scratch() {
  if (owned_) cudaFreeAsync(owned_, s_);
}

int Scratch::reserve(size_t total) {
  total_ = total;
  used_ = 0;
  if (total == 0) return SEGTACO_OK;
  if (user_) {
    if (cap_ < total)
      return set_error(SEGTACO_EINVAL, "workspace too small: %zu bytes given, %zu needed", cap_,
                       total);
    if (((uintptr_t)user_) & 255)
      return set_error(SEGTACO_EINVAL, "workspace must be 256-byte aligned");
    base_ = static_cast<char *>(user_);
    return SEGTACO_OK;
  }
  SEGTACO_TRY(check_cuda(cudaMallocAsync(&owned_, total, s_), "cudaMallocAsync(workspace)"));
  base_ = static_cast<char *>(owned_);
  return SEGTACO_OK;
}

void *Scratch::take(size_t bytes) {
  void *p = base_ + used_;
  used_ += align256(bytes);
  return p;
}

// ---------------------------------------------------------------------------
// SpMM planner
// ---------------------------------------------------------------------------
static bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }


int plan_spmm(int M, int K, long long nnz, int N, int b_dtype, long long ldb, long long ldc,
              const void *B, const float *C, const segtaco_config *cfg, SpmmPlan *plan,
              bool pieces) {
  segtaco_config c{};
  c.schedule = SEGTACO_AUTO;
  if (cfg) c = *cfg;
  const int esz = b_dtype == SEGTACO_BF16 ? 2 : 4;
  // Vector width: the widest 16-byte-or-less load that N, the strides and the
  // base pointers allow, for both the B loads and the C stores.
  // fp32 also takes vec = 8 on request: one 32-byte load per lane.
  int V = c.vec > 0 ? c.vec : 16 / esz;
  if (V > (esz == 2 ? 16 : 8) || !is_pow2(V))
    return set_error(SEGTACO_EINVAL, "vec=%d not in {1,2,4,8} (bf16: up to 16)", c.vec);
  auto fits = [&](int v) {
    const int vc = v < 4 ? v : 4;           // C is stored in float4 pieces
    const int ab = v * esz;                  // one B load of v elements per lane
    return N % v == 0 && ldb % v == 0 && ((uintptr_t)B % ab) == 0 && ldc % vc == 0 &&
           ((uintptr_t)C % (vc * 4)) == 0;
  };
  while (V > 1 && !fits(V)) V >>= 1;
  int schedule = c.schedule;
  // Without row-length statistics the merge path is the safe default: its
  // work per unit is bounded whatever the row-length skew.
  if (schedule == SEGTACO_AUTO) schedule = SEGTACO_EB_PR;
  if (schedule < SEGTACO_RB_SR || schedule > SEGTACO_EB_PR)
    return set_error(SEGTACO_EINVAL, "unknown schedule %d", schedule);
  // The slot walk keeps every row of a chunk in one slot, in storage order,
  // so eb_sr may use several slots there; elsewhere a sequential schedule is
  // one slot of 32 lanes.
  const bool slot_walk = (c.flags & SEGTACO_FLAG_SLOT_WALK) &&
                         (schedule == SEGTACO_EB_SR || schedule == SEGTACO_EB_PR);
  const bool sequential = (schedule == SEGTACO_RB_SR || schedule == SEGTACO_EB_SR) && !slot_walk;
  // Slab width W = G*V columns.  Sequential schedules use one slot (G = 32);
  // parallel ones use P = 32/G >= 2 slots, by default a 128-byte B segment per
  // nonzero (32 fp32 / 64 bf16 columns).
  int G;
  // 16-element (32-byte bf16) lanes exist for G <= 4 only: the sequential
  // schedules (G = 32) take at most 8.
  if (sequential && V > 8) V = 8;
  if (sequential) {
    G = 32;
    if (c.col_tile > 0 && c.vec <= 0) {
      // A requested slab width picks the vector width (W = 32*V).
      while (V > 1 && 32 * V > c.col_tile) V >>= 1;
    }
    // No idle half-slab: N = 32 takes one column per lane, not 8 lanes of 4.
    if (c.vec <= 0)
      while (V > 1 && 32 * (V / 2) >= N) V >>= 1;
  } else {
    int W = c.col_tile > 0 ? c.col_tile : 128 / esz;
    if (V > 8 && W / V > 4) V = 8;  // 16-element lanes: G <= 4
    G = W / V;
    if (G < 1) G = 1;
    if (G > 16) G = 16;
    while (!is_pow2(G)) --G;
    while (G > 1 && (G / 2) * V >= N) G >>= 1;  // no idle half-slots
  }
  const int W = G * V;
  plan->schedule = schedule;
  plan->V = V;
  plan->G = G;
  plan->W = W;
  plan->slabs = (N + W - 1) / W;
  plan->l2_hints = (c.flags & SEGTACO_FLAG_L2_HINTS) != 0;
  // TMA bulk copies need 16-byte lane vectors and 16-byte aligned segments
  // (V == 16/esz already implies N, ldb and B are multiples / aligned).
  plan->use_tma = (c.flags & SEGTACO_FLAG_SMEM_RING) && V * esz == 16;
  plan->bulk_copies = (c.flags & SEGTACO_FLAG_TMA_BULK) != 0;
  if (c.depth != 0 && c.depth != 4 && c.depth != 8)
    return set_error(SEGTACO_EINVAL, "depth=%d not in {0, 4, 8}", c.depth);
  plan->deep = c.depth == 8;
  // Walk: the flat walk by default for eb_sr (one slot over merge-path chunks:
  // short rows share a batch of 32 nonzeros instead of a round trip each;
  // measured on GB300 1.44 vs 1.53 ms on the 1M x 1M power-law SpMM), the row
  // walk everywhere else (rb units are too small to amortise the flat walk's
  // per-unit setup, and with several slots its flush bookkeeping costs more
  // instructions than the row walk); the flags force either.  Walks other
  // than the 4-load row walk exist for sixteen-byte vectors only.
  const bool wide = V * esz == 16;
  if ((c.flags & SEGTACO_FLAG_ROW_WALK) && (c.flags & SEGTACO_FLAG_FLAT_WALK))
    return set_error(SEGTACO_EINVAL, "ROW_WALK and FLAT_WALK are exclusive");
  const bool flat = wide && ((c.flags & SEGTACO_FLAG_FLAT_WALK) ||
                             (schedule == SEGTACO_EB_SR && G == 32 &&
                              !(c.flags & SEGTACO_FLAG_ROW_WALK)));
  plan->walk = flat ? 2 : (plan->deep && wide ? 1 : 0);
  // The slot walk (every slot its own merge-path chunk) on request, for the
  // element-balanced schedules and the lane shapes it is compiled for.
  const bool eb = schedule == SEGTACO_EB_SR || schedule == SEGTACO_EB_PR;
  if ((c.flags & SEGTACO_FLAG_SLOT_WALK) && eb && !plan->use_tma) {
    const int k = V * 100 + G;
    const bool ok = esz == 4 ? (k == 804 || k == 408 || k == 808 || k == 404 || k == 416 ||
                                k == 101)
                             : (k == 1604 || k == 804 || k == 808);
    if (ok) plan->walk = 3;
  }
  // eb_sr with 8-byte lanes (bf16 over 128-column slabs, fp32 over 64): the
  // sequential walk with staged indices (spmm_seq_unit), unless a walk is
  // forced.
  if (schedule == SEGTACO_EB_SR && G == 32 && !plan->use_tma && plan->walk == 0 &&
      !(c.flags & (SEGTACO_FLAG_ROW_WALK | SEGTACO_FLAG_FLAT_WALK)) && V * esz == 8)
    plan->walk = 4;
  plan->rows_per_unit = c.rows_per_unit > 0 ? c.rows_per_unit : 1;
  plan->items_per_unit = 0;
  plan->nchunks = (M + plan->rows_per_unit - 1) / plan->rows_per_unit;  // rb: row blocks
  plan->workspace = 0;
  plan->long_row = 0;
  plan->piece_len = 0;
  plan->piece_parts = 1;
  plan->px_entries = plan->py_entries = 0;
  if (schedule == SEGTACO_EB_SR || schedule == SEGTACO_EB_PR) {
    // merge-path items per chunk: one chunk per warp (512, fewer for small
    // products), or per slot in the slot walk (64, so a warp still covers
    // about 512)
    long long D = c.items_per_unit > 0   ? c.items_per_unit
                  : plan->walk == 3 ? 64
                                    : default_chunk_items(M, nnz);
    if (D < 1) D = 1;
    const long long total = (long long)M + nnz;
    long long nch = (total + D - 1) / D;
    if (nch < 1) nch = 1;
    plan->items_per_unit = D;
    plan->nchunks = nch;
    plan->px_entries = plan->py_entries = nch + 1;
  } else if (nnz >= kLongRowsMinNnz && (c.flags & SEGTACO_FLAG_LONG_ROWS) &&
             plan->walk != 2 && !plan->use_tma) {
    const int epc = 16 / esz;
    if (schedule == SEGTACO_RB_PR && pieces) {
      // rb_pr: long rows as pieces of kPieceLen nonzeros in the row-block
      // launch (spmm_long.cu), over the same column slabs; rows from
      // kPieceThreshold nonzeros by default.
      long long T = c.items_per_unit > 0 ? c.items_per_unit : kPieceThreshold;
      if (T > nnz) T = nnz;
      plan->long_row = (int)T;
      // passes over ranges of B's rows (a launch of their own before the row
      // blocks) on request
      int parts = c.k_parts > 0 ? c.k_parts : 1;
      if (parts > kMaxPieceParts) parts = kMaxPieceParts;
      if (parts > K) parts = K > 0 ? K : 1;
      plan->piece_parts = parts;
      plan->piece_len = (int)(parts > 1 ? kPassPieceLen : kPieceLen);
      plan->px_entries = piece_layout(nnz, T, plan->piece_len, plan->slabs, W, parts).entries;
      plan->py_entries = 4;  // the count
    } else if (N % epc == 0 && ldb % epc == 0 && ((uintptr_t)B % 16) == 0) {
      // Long rows to CTAs of their own (spmm_long.cu): their ring copies
      // 16-byte chunks of B rows, so B, ldb and N must allow 16-byte pieces.
      long long T = long_row_threshold(c);
      if (T > nnz) T = nnz;
      long long hi, lo;
      long_list_caps(nnz, T, &hi, &lo);
      plan->long_row = (int)T;
      plan->px_entries = hi + lo;
      plan->py_entries = 4;  // the two parts' counts, 64-bit work queue
    }
  }
  plan->window_halo = -1;
  plan->band_halo = -1;
  if ((c.flags & SEGTACO_FLAG_WINDOW) && schedule == SEGTACO_RB_PR && plan->long_row == 0 &&
      !plan->use_tma && nnz > 0 && K > 0 && N >= 64 && N % 16 == 0 &&
      ((uintptr_t)B % 16) == 0 && (ldb * esz) % 16 == 0 && ((uintptr_t)C % 16) == 0 &&
      ldc % 4 == 0) {
    // rb_pr on a banded matrix: 32-row blocks with the band of A as a dense
    // tile and B's window of 32 + 2H rows by TMA (spmm_band_kernel).
    const long long H = c.items_per_unit > 0 ? c.items_per_unit : 32;
    if (32 + 2 * H <= 256) plan->band_halo = (int)H;
  }
  if ((c.flags & SEGTACO_FLAG_WINDOW) && plan->band_halo < 0 && plan->long_row == 0 &&
      !plan->use_tma && nnz > 0 && K > 0 &&
      (schedule == SEGTACO_RB_SR || schedule == SEGTACO_RB_PR) && plan->walk != 2) {
    // TMA needs B 16-byte aligned and its row pitch a multiple of 16 bytes;
    // the window's rows (4 per-warp row blocks plus two halos) fit one box.
    const long long H = c.items_per_unit > 0 ? c.items_per_unit : 32;
    const long long wrows = 4 * plan->rows_per_unit + 2 * H;
    if (((uintptr_t)B % 16) == 0 && (ldb * esz) % 16 == 0 && wrows <= 256 &&
        (size_t)wrows * W * esz <= 60 * 1024 && window_variant_exists(b_dtype, V, G))
      plan->window_halo = (int)H;
  }
  if (plan->px_entries)
    plan->workspace = align256((size_t)plan->px_entries * sizeof(int)) +
                      align256((size_t)plan->py_entries * sizeof(int));
  return SEGTACO_OK;
}

int run_spmm_planned(const SpmmPlan &plan, int M, int K, long long nnz, const int *row_ptr,
                     const int *col, const float *vals, const void *B, int b_dtype, long long ldb,
                     float *C, long long ldc, int N, int *px, int *py, cudaStream_t s,
                     bool partition_ready) {
  if (M == 0 || N == 0) return SEGTACO_OK;
  SpmmLaunch L;
  L.dtype = b_dtype;
  L.V = plan.V;
  L.G = plan.G;
  L.l2_hints = plan.l2_hints;
  L.M = M;
  L.K = K;
  L.N = N;
  L.nnz = nnz;
  L.row_ptr = row_ptr;
  L.col = col;
  L.val = vals;
  L.B = B;
  L.ldb = ldb;
  L.C = C;
  L.ldc = ldc;
  L.part_x = px;
  L.part_y = py;
  L.units = plan.nchunks;
  L.rows_per_unit = (int)plan.rows_per_unit;
  L.use_tma = plan.use_tma;
  L.bulk_copies = plan.bulk_copies;
  L.deep = plan.deep;
  L.walk = plan.walk;
  L.no_fork = plan.no_fork;
  L.window_halo = plan.window_halo;
  L.band_halo = plan.band_halo;
  const bool bf16 = b_dtype == SEGTACO_BF16;
  switch (plan.schedule) {
    case SEGTACO_RB_SR:
    case SEGTACO_RB_PR:
      if (L.use_tma) return bf16 ? launch_spmm_tma_bf16(L, true, s) : launch_spmm_tma_f32(L, true, s);
      if (plan.band_halo >= 0) return launch_spmm_band(L, s);
      if (plan.window_halo >= 0) return launch_spmm_window(L, s);
      if (plan.long_row > 0 && plan.piece_len > 0) {
        L.long_row = plan.long_row;
        if (!partition_ready)
          SEGTACO_TRY(launch_long_pieces_list(row_ptr, M, nnz, plan.long_row, plan.piece_len,
                                              plan.slabs, plan.W, plan.piece_parts, px, py, s));
        const PieceLayout pl = piece_layout(nnz, plan.long_row, plan.piece_len, plan.slabs,
                                            plan.W, plan.piece_parts);
        L.piece_len = plan.piece_len;
        L.pieces = px;
        L.piece_count = py;
        L.piece_ctr = reinterpret_cast<unsigned *>(px + pl.ctr);
        L.piece_part = reinterpret_cast<float *>(px + pl.part);
        L.piece_cap = pl.cap;
        L.piece_multi = pl.multi;
        L.piece_ld = pl.ld;
        L.piece_parts = plan.piece_parts;
        // count[2..3]: the passes' work counter (the count array is 256-byte aligned)
        L.piece_queue = reinterpret_cast<unsigned long long *>(py + 2);
        if (plan.piece_parts > 1) {
          // the pieces' passes, then the row blocks of the short rows alone
          SEGTACO_TRY(bf16 ? launch_spmm_pieces_bf16(L, s) : launch_spmm_pieces_f32(L, s));
          L.piece_len = 0;
          L.piece_cap = 0;
        }
        return bf16 ? launch_spmm_bf16_rows(L, s) : launch_spmm_f32_rows(L, s);
      }
      if (plan.long_row > 0) {
        L.long_row = plan.long_row;
        if (!partition_ready)
          SEGTACO_TRY(launch_long_rows_list(row_ptr, M, nnz, plan.long_row, px, py, s));
        return launch_spmm_long_rows(L, px, py, s);
      }
      return bf16 ? launch_spmm_bf16_rows(L, s) : launch_spmm_f32_rows(L, s);
    case SEGTACO_EB_SR:
    case SEGTACO_EB_PR:
      if (!partition_ready)
        SEGTACO_TRY(launch_merge_path(row_ptr, M, nnz, plan.items_per_unit, plan.nchunks, px, py,
                                      C, ldc, N, s));
      if (L.use_tma) return bf16 ? launch_spmm_tma_bf16(L, false, s) : launch_spmm_tma_f32(L, false, s);
      return bf16 ? launch_spmm_bf16_chunks(L, s) : launch_spmm_f32_chunks(L, s);
    default:
      return set_error(SEGTACO_EINVAL, "unknown schedule %d", plan.schedule);
  }
}

long long sddmm_block_nnz();

// Host-side checks of the CSR arguments; `need_col` is false for the calls
// that only read row_ptr (partitions, row ids).
static int check_csr_args(int M, int K, long long nnz, const int *row_ptr, const int *col,
                          bool need_col = true) {
  if (M < 0 || K < 0 || nnz < 0) return set_error(SEGTACO_EINVAL, "negative size");
  if (nnz > 0x7fffffffLL) return set_error(SEGTACO_EINVAL, "nnz exceeds int32 indices");
  if (M > 0 && row_ptr == nullptr) return set_error(SEGTACO_EINVAL, "row_ptr is NULL");
  if (need_col && nnz > 0 && col == nullptr) return set_error(SEGTACO_EINVAL, "col is NULL");
  return SEGTACO_OK;
}

}  // namespace segtaco

using namespace segtaco;

extern "C" {

const char *segtaco_version(void) { return "segtaco-gb300 0.1 (sm_103a)"; }

const char *segtaco_last_error(void) { return g_last_error.c_str(); }

int segtaco_device_available(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n > 0 ? 1 : 0;
}

int segtaco_autotune_heuristic(int32_t M, int32_t K, int64_t nnz, int32_t N, int32_t b_dtype,
                               int64_t max_row_len, segtaco_config *cfg) {
  if (!cfg) return set_error(SEGTACO_EINVAL, "cfg is NULL");
  const int requested = cfg->schedule;
  const bool banded = (cfg->flags & SEGTACO_FLAG_WINDOW) != 0;
  memset(cfg, 0, sizeof(*cfg));
  const double mean = M > 0 ? (double)nnz / M : 0.0;
  // Row-balanced when rows are short and even; merge path otherwise.
  const bool even = max_row_len >= 0 && mean > 0.0 && (double)max_row_len <= 4.0 * mean + 8.0;
  const int schedule = (requested >= SEGTACO_RB_SR && requested <= SEGTACO_EB_PR)
                           ? requested
                           : (even ? SEGTACO_RB_PR : SEGTACO_EB_PR);
  cfg->schedule = schedule;
  const int esz = b_dtype == SEGTACO_BF16 ? 2 : 4;
  const bool sequential = schedule == SEGTACO_RB_SR || schedule == SEGTACO_EB_SR;
  // Column slab: the B slab should stay in L2 (measured on GB300: 128-byte
  // segments for the parallel schedules; the sequential ones take 16-byte
  // vectors on all 32 lanes).  A B that fits L2 whole is one slab.
  const double bbytes = (double)K * N * esz;
  const bool skewed = mean > 0.0 && (double)max_row_len > 8.0 * mean;
  if (sequential) {
    // The narrowest lanes that still cover N in one slab (N = 32: one column
    // per lane, all 32 lanes busy; measured on GB300, 16,384^2 with 16
    // nonzeros per row, N = 32: 16-byte lanes left 24 of 32 lanes idle).
    int v = 16 / esz;
    while (v > 1 && 32 * (v / 2) >= N) v >>= 1;
    cfg->col_tile = 32 * v;
  } else
    cfg->col_tile = bbytes <= 48e6 ? (N <= 64 * 4 / esz ? N : 64 * 4 / esz) : 128 / esz;
  // Row-block schedules from 1M nonzeros whose longest row reaches the
  // long-row threshold hand those rows to CTAs of their own (spmm_long.cu;
  // without row statistics they stay in the row-block kernel: the long-row
  // launch costs its L1 carveout, banded 262,144 rows N = 64 rb_pr 0.344 ->
  // 0.435 ms).  rb_sr's row-block kernel then takes 128-column slabs also for
  // bf16 (8-byte lanes).  Measured on GB300, 1M x 1M power law, N = 128:
  // fp32 2.32 ms (64-column slabs: 2.45), bf16 2.29 ms (256: 2.52).
  const bool long_rows =
      (schedule == SEGTACO_RB_SR || schedule == SEGTACO_RB_PR) && nnz >= kLongRowsMinNnz &&
      max_row_len >= (schedule == SEGTACO_RB_PR ? kPieceThreshold : kLongRowDefault);
  if (schedule == SEGTACO_RB_SR && long_rows) cfg->col_tile = 128;
  // fp32 with B beyond L2 (32-column slabs): 8 columns per lane (one 32-byte
  // load, 4 lanes per 128-byte segment, 8 slots), so a warp step covers 8 rows
  // or 8 nonzeros instead of 4.  Measured on GB300: 1M x 1M power law (skewed
  // rows), N = 128, eb_pr 1.33 -> 1.15 ms, rb_pr 2.84 -> 2.49 ms; banded
  // 262,144 rows (even rows, 19M nonzeros), N = 64, rb_pr 0.368 -> 0.344 ms.
  // Even rows with few nonzeros keep 4 (the 256-matrix pool, products of at
  // most a few million nonzeros, 3.74 -> 3.87 ms with 8); with B in L2
  // (64-column slabs: 8 lanes per slot, 24 warps per SM) the pool lost more
  // (4.38 ms).
  if (!sequential && esz == 4 && bbytes > 48e6 && N % 8 == 0 && (skewed || nnz >= 4000000))
    cfg->vec = 8;
  // A B that fits L2 whole (up to ~96 MB) under a large product: one slab of
  // up to 64 columns (8 per lane, G = 8), so A is read once.  Measured on
  // GB300, banded 262,144 rows (19.1M nonzeros), N = 64, rb_pr: 0.248 ms
  // against 0.323 ms with two 32-column slabs.
  if (!sequential && esz == 4 && bbytes > 48e6 && bbytes <= 96e6 && nnz >= 4000000 &&
      N % 8 == 0 && !skewed)
    cfg->col_tile = N < 64 ? N : 64;
  // bf16 likewise: 16 columns per lane (one 32-byte load) on 64-column slabs.
  // Measured on GB300: 1M x 1M power law, N = 128, eb_pr 0.996 -> 0.823 ms;
  // with B in L2 (banded, N = 64) 8 stays faster (0.224 vs 0.235 ms).
  if (!sequential && esz == 2 && bbytes > 48e6 && N % 16 == 0 && (skewed || nnz >= 4000000))
    cfg->vec = 16;
  // eb: merge-path items per chunk; rb: the long-row threshold.
  cfg->items_per_unit = (schedule == SEGTACO_RB_SR || schedule == SEGTACO_RB_PR)
                            ? (int)kLongRowDefault
                            : (int)default_chunk_items(M, nnz);
  cfg->rows_per_unit = schedule == SEGTACO_RB_PR || schedule == SEGTACO_RB_SR ? 4 : 1;
  // rb_sr walks its rows one after another in one slot: fewer rows per warp
  // while the rows are few.  Measured on GB300, 16,384 x 16,384 with 16
  // nonzeros per row, N = 32: 0.0174 ms with 4 rows, 0.0154 with 2.
  if (schedule == SEGTACO_RB_SR)
    while (cfg->rows_per_unit > 1 && M / cfg->rows_per_unit < 8192) cfg->rows_per_unit >>= 1;
  cfg->depth = (schedule == SEGTACO_RB_SR || schedule == SEGTACO_RB_PR) ? 8 : 4;
  cfg->flags = long_rows ? SEGTACO_FLAG_LONG_ROWS : 0;
  // rb_pr's long rows as pieces of the row-block launch (rows of >= 512
  // nonzeros, pieces of 4096); the rows left are short, so a warp takes 64 of
  // them to fill its slots (32 while that leaves fewer than 8192 warps).
  // Measured on GB300, 1M x 1M power law, N = 128: 1.69 ms with the long-row
  // CTAs (threshold 2048, 4 rows per warp), 1.58 with pieces of 512, 1.22
  // with 32 rows per warp (2 rows: 2.01); pieces of 4096: 1.119 ms with 32
  // rows, 1.114 with 64 (the 10M-nonzero Zipf 1.922 matrix 0.697 / 0.689).
  // Rows of ~73 nonzeros (banded, N = 64) keep 4: 0.251 ms against 0.266
  // with 16.
  if (schedule == SEGTACO_RB_PR && long_rows) {
    cfg->items_per_unit = (int)kPieceThreshold;
    if (mean < 32.0) cfg->rows_per_unit = M / 64 >= 8192 ? 64 : 32;
  }
  // fp32 B beyond L2 under skewed rows: the gathered B rows evict_last in L2
  // (A and C stream with evict-first loads and stores).  Measured on GB300,
  // 1M x 1M power law, N = 128, three alternations: eb_pr 1.128 -> 1.110 ms,
  // rb_pr (pieces, 32 rows per warp) 1.219 -> 1.201; rb_sr unchanged (1.683
  // / 1.687).
  if (!sequential && esz == 4 && bbytes > 48e6 && skewed) cfg->flags |= SEGTACO_FLAG_L2_HINTS;
  // Rows known to lie near the diagonal (the caller's segtaco_band_stats):
  // rb_pr takes the band kernel (32-row blocks, the band of A as a dense tile,
  // B's window by TMA, 4 x 4 register tiles; spmm_window.cu) with a halo of
  // 32.  Measured on GB300, banded-plus-random 262,144 rows (half band 32, 8
  // off-band nonzeros per row): fp32 N = 64 0.2465 -> 0.2325 ms, bf16 B
  // 0.2323 -> 0.1725 ms, fp32 N = 128 0.650 -> 0.455 ms (halo 16: 0.61 ms,
  // 48: 0.29 ms at fp32 N = 64).  The staged window for the row-block walk
  // (still one gathered B slice per nonzero, from shared memory instead of
  // L1) measured slower than the plain row blocks (0.373 vs 0.248 ms) and is
  // not chosen; rb_sr keeps the plain row blocks.
  if (banded && schedule == SEGTACO_RB_PR && !long_rows && N >= 64 && N % 16 == 0) {
    cfg->flags |= SEGTACO_FLAG_WINDOW;
    cfg->items_per_unit = 32;
  }
  return SEGTACO_OK;
}

int segtaco_spmm_plan_name(int32_t M, int32_t K, int64_t nnz, int32_t N, int32_t b_dtype,
                           const void *B, int64_t ldb, const segtaco_config *cfg, char *out,
                           size_t len) {
  if (!out || len == 0) return set_error(SEGTACO_EINVAL, "out is NULL");
  SpmmPlan plan;
  SEGTACO_TRY(plan_spmm(M, K, nnz, N, b_dtype, ldb, N, B, nullptr, cfg, &plan));
  static const char *sched[] = {"rb_sr", "rb_pr", "eb_sr", "eb_pr"};
  const char *kernel = plan.use_tma         ? "tma_ring"
                       : plan.band_halo >= 0   ? "band"
                       : plan.window_halo >= 0 ? "window"
                       : plan.long_row > 0 ? (plan.piece_len > 0 ? "pieces" : "long_rows")
                       : (plan.schedule >= SEGTACO_EB_SR) ? "chunks" : "rows";
  snprintf(out, len, "%s %s V=%d G=%d W=%d slabs=%d walk=%d halo=%d rows_per_unit=%lld parts=%d",
           sched[plan.schedule], kernel, plan.V, plan.G, plan.W, plan.slabs, plan.walk,
           plan.band_halo >= 0 ? plan.band_halo : plan.window_halo,
           (long long)plan.rows_per_unit, plan.piece_len > 0 ? plan.piece_parts : 1);
  return SEGTACO_OK;
}

int segtaco_spmm_workspace_size(int32_t M, int32_t K, int64_t nnz, int32_t N, int32_t b_dtype,
                                const segtaco_config *cfg, size_t *bytes) {
  if (!bytes) return set_error(SEGTACO_EINVAL, "bytes is NULL");
  SpmmPlan plan;
  // Alignment does not change the workspace: plan with aligned stand-ins.
  SEGTACO_TRY(plan_spmm(M, K, nnz, N, b_dtype, N, N, nullptr, nullptr, cfg, &plan));
  *bytes = plan.workspace;
  return SEGTACO_OK;
}

int segtaco_spmm(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr, const int32_t *col,
                 const float *vals, const void *B, int32_t b_dtype, int64_t ldb, float *C,
                 int64_t ldc, int32_t N, const segtaco_config *cfg, void *workspace,
                 size_t workspace_bytes, void *stream) {
  SEGTACO_TRY(check_csr_args(M, K, nnz, row_ptr, col));
  if (N < 0) return set_error(SEGTACO_EINVAL, "negative N");
  if (b_dtype != SEGTACO_F32 && b_dtype != SEGTACO_BF16)
    return set_error(SEGTACO_EINVAL, "unknown dense dtype %d", b_dtype);
  if (M == 0 || N == 0) return SEGTACO_OK;
  if (C == nullptr) return set_error(SEGTACO_EINVAL, "C is NULL");
  if (nnz > 0 && B == nullptr) return set_error(SEGTACO_EINVAL, "B is NULL");
  if (ldb < N || ldc < N) return set_error(SEGTACO_EINVAL, "ldb/ldc smaller than N");
  SpmmPlan plan;
  SEGTACO_TRY(plan_spmm(M, K, nnz, N, b_dtype, ldb, ldc, B, C, cfg, &plan));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch scratch(workspace, workspace_bytes, s);
  SEGTACO_TRY(scratch.reserve(plan.workspace));
  int *px = nullptr, *py = nullptr;
  if (plan.workspace) {
    px = static_cast<int *>(scratch.take(plan.px_entries * sizeof(int)));
    py = static_cast<int *>(scratch.take(plan.py_entries * sizeof(int)));
  }
  const bool ready = cfg && (cfg->flags & SEGTACO_FLAG_PARTITION_READY);
  if (ready && plan.workspace && !workspace)
    return set_error(SEGTACO_EINVAL, "PARTITION_READY needs the caller's workspace");
  return run_spmm_planned(plan, M, K, nnz, row_ptr, col, vals, B, b_dtype, ldb, C, ldc, N, px, py,
                          s, ready);
}

int segtaco_spmm_partition(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr, float *C,
                           int64_t ldc, int32_t N, int32_t b_dtype, const segtaco_config *cfg,
                           void *workspace, size_t workspace_bytes, void *stream) {
  SEGTACO_TRY(check_csr_args(M, K, nnz, row_ptr, nullptr, false));
  if (M == 0 || N == 0) return SEGTACO_OK;
  if (C == nullptr || ldc < N) return set_error(SEGTACO_EINVAL, "C is NULL or ldc < N");
  SpmmPlan plan;
  SEGTACO_TRY(plan_spmm(M, K, nnz, N, b_dtype, N, ldc, nullptr, C, cfg, &plan));
  if (!plan.workspace) return SEGTACO_OK;
  if (!workspace) return set_error(SEGTACO_EINVAL, "segtaco_spmm_partition needs a workspace");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch scratch(workspace, workspace_bytes, s);
  SEGTACO_TRY(scratch.reserve(plan.workspace));
  int *px = static_cast<int *>(scratch.take(plan.px_entries * sizeof(int)));
  int *py = static_cast<int *>(scratch.take(plan.py_entries * sizeof(int)));
  if (plan.long_row > 0 && plan.piece_len > 0)
    return launch_long_pieces_list(row_ptr, M, nnz, plan.long_row, plan.piece_len, plan.slabs,
                                   plan.W, plan.piece_parts, px, py, s);
  if (plan.long_row > 0) return launch_long_rows_list(row_ptr, M, nnz, plan.long_row, px, py, s);
  return launch_merge_path(row_ptr, M, nnz, plan.items_per_unit, plan.nchunks, px, py, C, ldc, N,
                           s);
}

int segtaco_block_starts_taco(int32_t M, int64_t nnz, const int32_t *row_ptr, int32_t P,
                              int32_t *out, void *stream) {
  SEGTACO_TRY(check_csr_args(M, 0, nnz, row_ptr, nullptr, false));
  if (P <= 0 || out == nullptr) return set_error(SEGTACO_EINVAL, "P must be > 0, out non-NULL");
  const long long nblk = (nnz + P - 1) / P;
  return launch_block_starts_taco(row_ptr, M, P, nblk, out, static_cast<cudaStream_t>(stream));
}

int segtaco_block_starts_canonical(int32_t M, int64_t nnz, const int32_t *row_ptr, int32_t P,
                                   int32_t *out, void *stream) {
  SEGTACO_TRY(check_csr_args(M, 0, nnz, row_ptr, nullptr, false));
  if (P <= 0 || out == nullptr) return set_error(SEGTACO_EINVAL, "P must be > 0, out non-NULL");
  const long long nblk = (nnz + P - 1) / P;
  return launch_block_starts_canonical(row_ptr, M, P, nblk, out,
                                       static_cast<cudaStream_t>(stream));
}

int segtaco_merge_path(int32_t M, int64_t nnz, const int32_t *row_ptr, int64_t D, int32_t *out_x,
                       int32_t *out_y, void *stream) {
  SEGTACO_TRY(check_csr_args(M, 0, nnz, row_ptr, nullptr, false));
  if (D <= 0 || !out_x || !out_y) return set_error(SEGTACO_EINVAL, "D must be > 0, outputs non-NULL");
  long long nch = ((long long)M + nnz + D - 1) / D;
  if (nch < 1) nch = 1;
  return launch_merge_path(row_ptr, M, nnz, D, nch, out_x, out_y, nullptr, 0, 0,
                           static_cast<cudaStream_t>(stream));
}

int segtaco_row_ids(int32_t M, int64_t nnz, const int32_t *row_ptr, int32_t *out, void *stream) {
  SEGTACO_TRY(check_csr_args(M, 0, nnz, row_ptr, nullptr, false));
  if (nnz > 0 && out == nullptr) return set_error(SEGTACO_EINVAL, "out is NULL");
  return launch_row_ids(row_ptr, M, out, static_cast<cudaStream_t>(stream));
}

int segtaco_csr_validate(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                         const int32_t *col, void *stream) {
  SEGTACO_TRY(check_csr_args(M, K, nnz, row_ptr, col));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch scratch(nullptr, 0, s);
  SEGTACO_TRY(scratch.reserve(256));
  int *err = static_cast<int *>(scratch.take(2 * sizeof(int)));
  SEGTACO_TRY(check_cuda(cudaMemsetAsync(err, 0, 2 * sizeof(int), s), "memset"));
  SEGTACO_TRY(launch_validate(row_ptr, M, K, nnz, col, err, s));
  int h[2] = {0, 0};
  SEGTACO_TRY(check_cuda(cudaMemcpyAsync(h, err, sizeof(h), cudaMemcpyDeviceToHost, s), "copy"));
  SEGTACO_TRY(check_cuda(cudaStreamSynchronize(s), "sync"));
  static const char *what[] = {"", "row_ptr[0] != 0", "row_ptr[M] != nnz",
                               "row_ptr decreases at row", "col out of [0, K) at nonzero"};
  if (h[0] != 0) return set_error(SEGTACO_EINVAL, "malformed CSR: %s %d", what[h[0] & 7], h[1]);
  return SEGTACO_OK;
}

// SpMV is the N = 1 point of the SpMM segment kernel: eb_pr with one lane per
// slot (32 nonzeros or short rows per warp step) over 512-item merge-path
// chunks.  Measured on GB300 (1M x 1M power-law, 20.6M nonzeros): 0.140 ms,
// against 0.222 ms for a dedicated merge-path tile kernel staging products in
// shared memory.
static segtaco_config spmv_config() {
  segtaco_config c = {};
  c.schedule = SEGTACO_EB_PR;
  c.col_tile = 1;
  c.vec = 1;
  c.items_per_unit = 512;
  return c;
}

int segtaco_spmv_workspace_size(int32_t M, int64_t nnz, size_t *bytes) {
  if (!bytes) return set_error(SEGTACO_EINVAL, "bytes is NULL");
  if (M < 0 || nnz < 0) return set_error(SEGTACO_EINVAL, "negative size");
  const segtaco_config c = spmv_config();
  SpmmPlan plan;
  SEGTACO_TRY(plan_spmm(M, 1, nnz, 1, SEGTACO_F32, 1, 1, nullptr, nullptr, &c, &plan));
  *bytes = plan.workspace;
  return SEGTACO_OK;
}

int segtaco_spmv(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr, const int32_t *col,
                 const float *vals, const float *x, float *y, void *workspace,
                 size_t workspace_bytes, void *stream) {
  SEGTACO_TRY(check_csr_args(M, K, nnz, row_ptr, col));
  if (M == 0) return SEGTACO_OK;
  if (y == nullptr || (nnz > 0 && x == nullptr)) return set_error(SEGTACO_EINVAL, "x/y is NULL");
  const segtaco_config c = spmv_config();
  SpmmPlan plan;
  SEGTACO_TRY(plan_spmm(M, K, nnz, 1, SEGTACO_F32, 1, 1, x, y, &c, &plan));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch scratch(workspace, workspace_bytes, s);
  SEGTACO_TRY(scratch.reserve(plan.workspace));
  int *px = nullptr, *py = nullptr;
  if (plan.workspace) {
    px = static_cast<int *>(scratch.take(plan.px_entries * sizeof(int)));
    py = static_cast<int *>(scratch.take(plan.py_entries * sizeof(int)));
  }
  return run_spmm_planned(plan, M, K, nnz, row_ptr, col, vals, x, SEGTACO_F32, 1, y, 1, 1, px, py,
                          s);
}

int segtaco_sddmm_autotune(int32_t M, int32_t K, int64_t nnz, int32_t D, int32_t x_dtype,
                           int64_t max_row_len, segtaco_sddmm_config *cfg) {
  if (!cfg) return set_error(SEGTACO_EINVAL, "cfg is NULL");
  if (M < 0 || K < 0 || nnz < 0 || D < 0) return set_error(SEGTACO_EINVAL, "negative size");
  const bool banded = cfg->kernel == SEGTACO_SDDMM_BAND;
  memset(cfg, 0, sizeof(*cfg));
  cfg->kernel = SEGTACO_SDDMM_AUTO;
  // Rows known to lie near the diagonal: the band kernel (sddmm_band.cu).
  // Measured on GB300, banded-plus-random 262,144 rows, D = 64: fp32 0.330 ->
  // 0.245 ms, bf16 factors 0.303 -> 0.224 ms.
  if (banded && D == 64) cfg->kernel = SEGTACO_SDDMM_BAND;
  (void)x_dtype;
  // Blocks of 256 nonzeros per warp; smaller for small problems, so that the
  // launch still holds two waves of warps (152 SMs x 32 warps).
  const long long two_waves = 2LL * 152 * 32;
  int blk = 256;
  while (blk > 32 && (nnz + blk - 1) / blk < two_waves) blk >>= 1;
  cfg->block_nnz = blk;
  cfg->lanes = 0;  // from D (sddmm_shape)
  (void)max_row_len;
  (void)K;
  return SEGTACO_OK;
}

int segtaco_sddmm_ex(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                     const int32_t *col, const float *vals, const void *X, const void *Y,
                     int32_t x_dtype, int64_t ldx, int64_t ldy, int32_t D, float *out,
                     const segtaco_sddmm_config *cfg, void *stream) {
  SEGTACO_TRY(check_csr_args(M, K, nnz, row_ptr, col));
  if (x_dtype != SEGTACO_F32 && x_dtype != SEGTACO_BF16)
    return set_error(SEGTACO_EINVAL, "unknown dense dtype %d", x_dtype);
  if (nnz == 0) return SEGTACO_OK;
  if (D < 0 || ldx < D || ldy < D) return set_error(SEGTACO_EINVAL, "bad D/ldx/ldy");
  if (!X || !Y || !out) return set_error(SEGTACO_EINVAL, "X/Y/out is NULL");
  segtaco_sddmm_config c;
  if (cfg)
    c = *cfg;
  else
    SEGTACO_TRY(segtaco_sddmm_autotune(M, K, nnz, D, x_dtype, -1, &c));
  const long long P = c.block_nnz > 0 ? c.block_nnz : sddmm_block_nnz();
  if (P < 32 || P > 4096 || (P & (P - 1)))
    return set_error(SEGTACO_EINVAL, "block_nnz=%lld not a power of two in [32, 4096]", P);
  if (c.lanes < 0 || c.lanes > 32 || (c.lanes & (c.lanes - 1)))
    return set_error(SEGTACO_EINVAL, "lanes=%d not 0 or a power of two up to 32", c.lanes);
  if (c.kernel < SEGTACO_SDDMM_AUTO || c.kernel > SEGTACO_SDDMM_BAND)
    return set_error(SEGTACO_EINVAL, "unknown SDDMM kernel %d", c.kernel);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (c.kernel == SEGTACO_SDDMM_BAND && sddmm_band_applies(x_dtype, D, ldx, ldy, X, Y))
    return launch_sddmm_band(M, K, nnz, row_ptr, col, vals, X, Y, x_dtype, ldx, ldy, D, out, s);
  if (c.kernel == SEGTACO_SDDMM_BAND) c.kernel = SEGTACO_SDDMM_AUTO;
  const long long nblk = (nnz + P - 1) / P;
  Scratch scratch(nullptr, 0, s);
  SEGTACO_TRY(scratch.reserve(align256((size_t)(nblk + 1) * sizeof(int))));
  int *starts = static_cast<int *>(scratch.take((nblk + 1) * sizeof(int)));
  return launch_sddmm(M, nnz, row_ptr, col, vals, X, Y, x_dtype, ldx, ldy, D, out, starts, (int)P,
                      nblk, s, false, c.lanes, c.kernel);
}

int segtaco_sddmm(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr, const int32_t *col,
                  const float *vals, const void *X, const void *Y, int32_t x_dtype, int64_t ldx,
                  int64_t ldy, int32_t D, float *out, void *stream) {
  return segtaco_sddmm_ex(M, K, nnz, row_ptr, col, vals, X, Y, x_dtype, ldx, ldy, D, out, nullptr,
                          stream);
}

int segtaco_spmspv(int32_t M, int32_t K, int64_t nnz, const int32_t *col_ptr,
                   const int32_t *row_idx, const float *vals, int32_t nx, const int32_t *x_idx,
                   const float *x_vals, float *y, void *stream) {
  SEGTACO_TRY(check_csr_args(K, M, nnz, col_ptr, row_idx));
  if (nx < 0) return set_error(SEGTACO_EINVAL, "negative nx");
  if (M > 0 && y == nullptr) return set_error(SEGTACO_EINVAL, "y is NULL");
  if (nx > 0 && (!x_idx || !x_vals)) return set_error(SEGTACO_EINVAL, "x is NULL");
  return launch_spmspv(M, K, col_ptr, row_idx, vals, nx, x_idx, x_vals, y,
                       static_cast<cudaStream_t>(stream));
}

}  // extern "C"
