// noalloc.cu -- segtaco_spmm_noalloc: the SpMM entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc: a host framework whose allocator owns
// and has already reserved the device memory, a serving loop that fixes its
// memory budget at start-up and must not allocate afterwards, or a caller that
// cannot afford the device-wide synchronisation an allocation may bring.  For
// them this entry point takes the scratch of the element-balanced schedules
// (the merge-path chunk coordinates) from a fixed array compiled into the
// library, instead of from a caller workspace or cudaMallocAsync.
//
// The array lives in device memory of every GPU that loads the library, for
// as long as the process runs (2 MiB).  Host code cannot hand the symbol
// itself to a kernel (on the host it only names a stand-in), so on the first
// call on each device this file looks up the array's device address with
// cudaGetSymbolAddress, with that device current, and caches it per device.
// That first call on a device should therefore come before any stream capture.
// The cached address belongs to the device's primary context: after
// cudaDeviceReset the module may load elsewhere, so resetting a device that
// has served this entry point is not supported.  Besides the look-up, the
// first call of a kernel variant may set its shared-memory attribute
// (cudaFuncSetAttribute, the rb long-row CTAs); nothing else is created: the
// long-row CTAs and the row-block kernel both run on the caller's stream.
//
// All calls share the one array: calls whose work overlaps on the GPU (on
// different streams, or from different host threads without ordering) race on
// it and must not be issued.  Nothing needs clearing between calls: the
// partition kernel writes every coordinate that the product kernel then reads.
#include <mutex>

#include "internal.h"

namespace segtaco {
namespace {

constexpr int kMaxDevices = 64;
// Two int32 arrays (chunk-edge rows, chunk-edge nonzeros) of this many entries.
constexpr long long kNoallocEntries = 262144;

static __device__ __align__(256) int g_noalloc_scratch[2 * kNoallocEntries];

std::mutex g_setup_mu;
int *g_scratch_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
int scratch_for_current_device(int **out) {
  int dev = -1;
  SEGTACO_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(SEGTACO_EUNSUPPORTED, "segtaco_spmm_noalloc: device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void *p = nullptr;
    SEGTACO_TRY(check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                           "cudaGetSymbolAddress(g_noalloc_scratch)"));
    g_scratch_ptr[dev] = static_cast<int *>(p);
  }
  *out = g_scratch_ptr[dev];
  return SEGTACO_OK;
}

}  // namespace
}  // namespace segtaco

using namespace segtaco;

extern "C" int segtaco_spmm_noalloc(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                                    const int32_t *col, const float *vals, const void *B,
                                    int32_t b_dtype, int64_t ldb, float *C, int64_t ldc, int32_t N,
                                    const segtaco_config *cfg, void *stream) {
  if (M < 0 || K < 0 || nnz < 0 || N < 0)
    return set_error(SEGTACO_EINVAL, "segtaco_spmm_noalloc: negative size");
  if (nnz > 0x7fffffffLL) return set_error(SEGTACO_EINVAL, "nnz exceeds int32 indices");
  if (b_dtype != SEGTACO_F32 && b_dtype != SEGTACO_BF16)
    return set_error(SEGTACO_EINVAL, "unknown dense dtype %d", b_dtype);
  if (M == 0 || N == 0) return SEGTACO_OK;
  if (!row_ptr || (nnz > 0 && (!col || !B)) || !C)
    return set_error(SEGTACO_EINVAL, "segtaco_spmm_noalloc: NULL operand");
  if (ldb < N || ldc < N) return set_error(SEGTACO_EINVAL, "ldb/ldc smaller than N");
  if (cfg && (cfg->flags & SEGTACO_FLAG_PARTITION_READY))
    return set_error(SEGTACO_EINVAL,
                     "segtaco_spmm_noalloc: PARTITION_READY is not supported (shared scratch)");
  SpmmPlan plan;
  SEGTACO_TRY(plan_spmm(M, K, nnz, N, b_dtype, ldb, ldc, B, C, cfg, &plan));
  if (plan.piece_len > 0 && plan.px_entries > kNoallocEntries)
    // rb_pr pieces whose partial rows would not fit: the long-row CTAs
    SEGTACO_TRY(plan_spmm(M, K, nnz, N, b_dtype, ldb, ldc, B, C, cfg, &plan, false));
  plan.no_fork = true;  // rb long rows: no side stream or events, both kernels on `stream`
  if (plan.long_row > 0 && plan.px_entries > kNoallocEntries) {
    // the long-row list would not fit: every row in the row-block kernel
    plan.long_row = 0;
    plan.piece_len = 0;
    plan.px_entries = plan.py_entries = 0;
    plan.workspace = 0;
  }
  int *px = nullptr, *py = nullptr;
  if (plan.workspace) {
    if (plan.px_entries > kNoallocEntries)
      return set_error(SEGTACO_EINVAL,
                       "segtaco_spmm_noalloc: %lld merge-path chunks exceed the fixed scratch of "
                       "%lld chunks (2 MiB); raise items_per_unit or use segtaco_spmm",
                       plan.nchunks, kNoallocEntries - 1);
    int *base = nullptr;
    SEGTACO_TRY(scratch_for_current_device(&base));
    px = base;
    py = base + kNoallocEntries;
  }
  return run_spmm_planned(plan, M, K, nnz, row_ptr, col, vals, B, b_dtype, ldb, C, ldc, N, px, py,
                          static_cast<cudaStream_t>(stream));
}
