// spmm_window.cu -- row-block SpMM with the reused B rows staged by TMA.
//
// For matrices whose nonzeros cluster around the diagonal (banded, block
// diagonal, meshes), the rows of a row block gather B rows from a short range
// around the block: rows i0 .. i1-1 touch B rows near [i0 - H, i1 + H).  Each
// 128-thread CTA here owns a block of 4 * rows_per_unit rows and one column
// slab; one thread brings the window B[i0 - H .. i1 + H) x slab into shared
// memory with a single cp.async.bulk.tensor.2d copy (a tensor map over B,
// box = window rows x slab columns; rows outside [0, K) are zero-filled by the
// copy engine), completing on an mbarrier.  Then the four warps walk their row
// blocks exactly as the row-block kernel does (spmm_walk_unit), except that a
// gather of a B row inside the window reads the shared copy; rows outside it
// (the off-band nonzeros) are still gathered from global memory.  So every
// in-band B row crosses L2 once per row block instead of once per nonzero.
//
// The wait is bounded: after kWindowSpin polls the CTA records SEGTACO_ETIMEOUT
// in the device status word (segtaco_device_status), waits once more, bounded,
// for its copy, and leaves its rows unwritten.
//
// Same results as the row-block kernel: the walk, its summation order and its
// stores are unchanged, only where a B value is read from.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <mutex>

#include "spmm_launch.cuh"

namespace segtaco {
namespace {

constexpr long long kWindowSpin = 1LL << 22;

__device__ __forceinline__ uint32_t sm_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool window_wait(uint32_t bar) {
  for (long long i = 0; i < kWindowSpin; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(0)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Most gathers come from shared memory here, so fewer resident warps hide
// the latency: 16 warps per SM, whose registers hold the walk and both
// gather paths without spilling.
template <typename BT, int V, int G> constexpr int window_min_ctas() {
  return 16 / kSpmmWarps;
}

template <typename BT, int V, int G>
__global__ void __launch_bounds__(kSpmmCta, window_min_ctas<BT, V, G>())
    spmm_window_kernel(SpmmArgs<BT> a, const __grid_constant__ CUtensorMap tm, int halo,
                       int *status) {
  constexpr int W = G * V;
  extern __shared__ __align__(128) unsigned char smem[];
  const long long rows_blk = (long long)kSpmmWarps * a.rows_per_unit;
  const int wrows = (int)(rows_blk + 2 * halo);
  BT *win = reinterpret_cast<BT *>(smem);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + (((size_t)wrows * W * sizeof(BT) + 15) & ~size_t(15)));
  const int wlo = (int)((long long)blockIdx.x * rows_blk - halo);
  const uint32_t b = sm_u32(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t bytes = (uint32_t)((size_t)wrows * W * sizeof(BT));
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes)
                 : "memory");
    // x = the slab's first column (a multiple of W: 16-byte aligned), y = the
    // window's first row (negative at the top edge: zero-filled)
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cta.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(sm_u32(win)),
        "l"(&tm), "r"((int)(blockIdx.y * W)), "r"(wlo), "r"(b)
        : "memory");
  }
  if (!window_wait(b)) {
    if (threadIdx.x == 0) atomicExch(status, SEGTACO_ETIMEOUT);
    window_wait(b);  // the copy may still land: wait for it once more, bounded
    return;
  }
  const long long w = (long long)blockIdx.x * kSpmmWarps + threadIdx.x / 32;
  if (w >= a.units) return;
  Window<BT> wv;
  wv.base = win;
  wv.lo = wlo;
  wv.rows = wrows;
  spmm_walk_unit<BT, V, G, true, false, true>(a, w, blockIdx.y, threadIdx.x & 31, wv);
}

// ---------------------------------------------------------------------------
// Banded row blocks for rb_pr (SEGTACO_FLAG_WINDOW with a parallel reduction).
//
// On a banded matrix the plain row blocks deliver each nonzero's 64-column B
// slice to registers (256 bytes for 64 multiply-adds), and that load/store
// data pipe is their bound; the window kernel above only moves the same bytes
// from shared memory instead of L1.  Here B values are reused from registers:
// a CTA owns kBandRows = 32 consecutive rows and a slab of 64 columns, brings
// the band window B[jw0 .. jw0 + win) x slab (win = 32 + 2H rows around the
// diagonal, column i0 * K / M of its first row) into shared memory with one
// TMA tensor copy, and scatters its rows' in-window nonzeros into a dense
// tile At[win][32] (row pitch kBandPitch = 36 floats: 16-byte aligned, and
// the scatter's consecutive columns of one row spread over 8 banks).  Thread
// (rb, cb) then keeps rows 4rb .. 4rb+3 x columns 4cb .. 4cb+3 in registers
// and, for every window row j, reads At[j][4rb .. 4rb+3] and B[j][4cb ..
// 4cb+3] (two 16-byte shared loads) for 16 multiply-adds: 2 bytes to
// registers per multiply-add.  The tile holds zeros where a row has no
// nonzero (win steps per row instead of ~2H + 1 nonzeros), and the summation
// order within a row differs from the storage order, which the parallel
// reduction allows; duplicate entries of a row add up in the tile.
//
// The scatter reads the block's nonzeros (contiguous in A) coalesced, finding
// each one's row among the 33 staged row starts; off-band nonzeros (outside
// the window) go to a per-row list of kBandList entries, and each thread
// gathers its 4 columns of them from global memory, 8 at a time (a row with
// more walks its nonzeros in global memory instead).  The TMA wait is bounded
// as in the window kernel (SEGTACO_ETIMEOUT, rows left unwritten).
constexpr int kBandRows = 32;
constexpr int kBandCols = 64;
constexpr int kBandList = 16;
constexpr int kBandPitch = 36;

// Four consecutive B values as floats: from shared memory, or from global
// memory through the read-only path.
template <typename BT> __device__ __forceinline__ float4 band_b4(const BT *p) {
  if constexpr (sizeof(BT) == 4) {
    return *reinterpret_cast<const float4 *>(p);
  } else {
    const uint2 x = *reinterpret_cast<const uint2 *>(p);
    return make_float4(bf16lo(x.x), bf16hi(x.x), bf16lo(x.y), bf16hi(x.y));
  }
}
template <typename BT> __device__ __forceinline__ float4 band_b4_global(const BT *p) {
  if constexpr (sizeof(BT) == 4) {
    return __ldg(reinterpret_cast<const float4 *>(p));
  } else {
    const uint2 x = __ldg(reinterpret_cast<const uint2 *>(p));
    return make_float4(bf16lo(x.x), bf16hi(x.x), bf16lo(x.y), bf16hi(x.y));
  }
}
__device__ __forceinline__ void band_fma4(float (&acc)[4], float x, const float4 &b) {
  acc[0] = fmaf(x, b.x, acc[0]);
  acc[1] = fmaf(x, b.y, acc[1]);
  acc[2] = fmaf(x, b.z, acc[2]);
  acc[3] = fmaf(x, b.w, acc[3]);
}

// Shared-memory layout of a band CTA (byte offsets; win = window rows).
struct BandSmem {
  size_t at, rp, cnt, lcol, lval, bar, bytes;
};
template <typename BT> __host__ __device__ inline BandSmem band_smem(int win) {
  BandSmem m;
  size_t o = ((size_t)win * kBandCols * sizeof(BT) + 127) & ~size_t(127);  // B window first
  m.at = o;
  o += (size_t)win * kBandPitch * 4;
  m.rp = o;
  o += (kBandRows + 1) * 4;
  m.cnt = o;
  o += kBandRows * 4;
  m.lcol = o;
  o += kBandRows * kBandList * 4;
  m.lval = o;
  o += kBandRows * kBandList * 4;
  m.bar = (o + 7) & ~size_t(7);
  m.bytes = m.bar + 8;
  return m;
}

template <typename BT>
__global__ void __launch_bounds__(kSpmmCta)
    spmm_band_kernel(SpmmArgs<BT> a, const __grid_constant__ CUtensorMap tm, int halo,
                     int *status) {
  const int win = kBandRows + 2 * halo;
  const BandSmem L = band_smem<BT>(win);
  extern __shared__ __align__(128) unsigned char smem[];
  BT *bw = reinterpret_cast<BT *>(smem);  // [win][kBandCols]
  float *at = reinterpret_cast<float *>(smem + L.at);  // [win][kBandPitch]
  int *rp = reinterpret_cast<int *>(smem + L.rp);
  int *cnt = reinterpret_cast<int *>(smem + L.cnt);
  int *lcol = reinterpret_cast<int *>(smem + L.lcol);
  float *lval = reinterpret_cast<float *>(smem + L.lval);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L.bar);
  const int t = threadIdx.x;
  const int M = a.M;
  const int i0 = blockIdx.x * kBandRows;
  const int jw0 = (int)((long long)i0 * a.K / M) - halo;
  const uint32_t b = sm_u32(bar);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int e = t; e < win * kBandPitch / 4; e += kSpmmCta)
    reinterpret_cast<float4 *>(at)[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (t <= kBandRows) rp[t] = __ldg(a.row_ptr + min(i0 + t, M));
  if (t < kBandRows) cnt[t] = 0;
  __syncthreads();
  if (t == 0) {
    const uint32_t bytes = (uint32_t)((size_t)win * kBandCols * sizeof(BT));
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes)
                 : "memory");
    // x = the slab's first column (a multiple of 64 elements), y = the
    // window's first row (negative at the top edge: zero-filled)
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cta.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(sm_u32(bw)),
        "l"(&tm), "r"((int)(blockIdx.y * kBandCols)), "r"(jw0), "r"(b)
        : "memory");
  }
  // Scatter the block's nonzeros rp[0] .. rp[32]-1, eight per thread per pass
  // (loads first, then the row searches and shared-memory updates).
  constexpr int SQ = 8;
  const int k_end = rp[kBandRows];
  for (int k0 = rp[0] + t; k0 < k_end; k0 += SQ * kSpmmCta) {
    int cj[SQ];
    float cv[SQ];
#pragma unroll
    for (int q = 0; q < SQ; ++q) {
      const int k = k0 + q * kSpmmCta;
      cj[q] = k < k_end ? __ldg(a.col + k) : 0;
      cv[q] = k < k_end ? ld_val(a.val, k) : 0.0f;
    }
#pragma unroll
    for (int q = 0; q < SQ; ++q) {
      const int k = k0 + q * kSpmmCta;
      if (k < k_end) {
        int r = 0;  // the last row whose start is <= k
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (r + step <= kBandRows - 1 && rp[r + step] <= k) r += step;
        const unsigned d = (unsigned)(cj[q] - jw0);
        if (d < (unsigned)win) {
          atomicAdd(at + d * kBandPitch + r, cv[q]);
        } else {
          const int slot = atomicAdd(cnt + r, 1);
          if (slot < kBandList) {
            lcol[r * kBandList + slot] = cj[q];
            lval[r * kBandList + slot] = cv[q];
          }
        }
      }
    }
  }
  __syncthreads();
  if (!window_wait(b)) {
    if (t == 0) atomicExch(status, SEGTACO_ETIMEOUT);
    window_wait(b);  // the copy may still land: wait for it once more, bounded
    return;
  }
  const int rb = t >> 4, cb = t & 15;
  const int c0 = blockIdx.y * kBandCols + 4 * cb;  // this thread's first column
  if (c0 >= a.N) return;                           // N is a multiple of 16
  float acc[4][4];
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.0f;
  // The first off-band gathers of row 4rb, issued before the tile product so
  // that their latency hides behind it.
  const int n0 = cnt[4 * rb];
  const int pre = n0 <= kBandList ? min(n0, 8) : 0;
  float4 g0[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    // slots past the row's list gather B row 0 (in bounds) and are not used
    const int j = e < pre ? lcol[4 * rb * kBandList + e] : 0;
    g0[e] = band_b4_global<BT>(a.B + (size_t)(unsigned)j * a.ldb + c0);
  }
  const float *acol = at + 4 * rb;
  const BT *bcol = bw + 4 * cb;
#pragma unroll 4
  for (int j = 0; j < win; ++j) {
    const float4 x = *reinterpret_cast<const float4 *>(acol + j * kBandPitch);
    const float4 bv = band_b4<BT>(bcol + j * kBandCols);
    band_fma4(acc[0], x.x, bv);
    band_fma4(acc[1], x.y, bv);
    band_fma4(acc[2], x.z, bv);
    band_fma4(acc[3], x.w, bv);
  }
  // Off-band nonzeros of the thread's four rows, from global memory.
#pragma unroll
  for (int e = 0; e < 8; ++e)
    if (e < pre) band_fma4(acc[0], lval[4 * rb * kBandList + e], g0[e]);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = 4 * rb + q;
    const int n = cnt[r];
    if (n <= kBandList) {
      for (int e0 = q == 0 ? pre : 0; e0 < n; e0 += 8) {
        float4 g[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int ee = e0 + e < n ? e0 + e : e0;
          g[e] = band_b4_global<BT>(a.B + (size_t)(unsigned)lcol[r * kBandList + ee] * a.ldb + c0);
        }
#pragma unroll
        for (int e = 0; e < 8; ++e)
          if (e0 + e < n) band_fma4(acc[q], lval[r * kBandList + e0 + e], g[e]);
      }
    } else {
      // more off-band nonzeros than the list holds: walk the row
      for (int k = rp[r]; k < rp[r + 1]; ++k) {
        const int j = __ldg(a.col + k);
        if ((unsigned)(j - jw0) >= (unsigned)win)
          band_fma4(acc[q], ld_val(a.val, k),
                    band_b4_global<BT>(a.B + (size_t)(unsigned)j * a.ldb + c0));
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = i0 + 4 * rb + q;
    if (i < M)
      __stcs(reinterpret_cast<float4 *>(a.C + (long long)i * a.ldc + c0),
             make_float4(acc[q][0], acc[q][1], acc[q][2], acc[q][3]));
  }
}

// cuTensorMapEncodeTiled from the driver, looked up once.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

template <typename BT, int V, int G> int launch_window_variant(const SpmmLaunch &L, cudaStream_t s) {
  constexpr int W = G * V;
  const long long rows_blk = (long long)kSpmmWarps * L.rows_per_unit;
  const long long wrows = rows_blk + 2LL * L.window_halo;
  if (wrows > 256)
    return set_error(SEGTACO_EINVAL, "window of %lld rows (4*rows_per_unit + 2*halo) > 256",
                     wrows);
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return set_error(SEGTACO_EUNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  CUtensorMap tm;
  const cuuint64_t dims[2] = {(cuuint64_t)L.N, (cuuint64_t)L.K};
  const cuuint64_t strides[1] = {(cuuint64_t)L.ldb * sizeof(BT)};
  const cuuint32_t box[2] = {(cuuint32_t)W, (cuuint32_t)wrows};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = enc(&tm, sizeof(BT) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                               : CU_TENSOR_MAP_DATA_TYPE_UINT16,
                         2, const_cast<void *>(L.B), dims, strides, box, es,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return set_error(SEGTACO_EINVAL, "window: tensor map of B rejected (CUresult %d)", (int)r);
  const size_t bytes = (((size_t)wrows * W * sizeof(BT) + 15) & ~size_t(15)) + 16;
  auto kern = spmm_window_kernel<BT, V, G>;
  // The shared-memory opt-in, once per device.
  static std::atomic<unsigned long long> opted{0};
  int dev = 0;
  SEGTACO_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(opted.load() & bit)) {
    SEGTACO_TRY(check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)(64 * 1024)),
                           "cudaFuncSetAttribute(spmm_window_kernel)"));
    opted.fetch_or(bit);
  }
  if (bytes > 64 * 1024) return set_error(SEGTACO_EINVAL, "window of %zu bytes > 64 KB", bytes);
  int *status = nullptr;
  SEGTACO_TRY(tma_status_ptr(&status));
  const SpmmArgs<BT> a = make_spmm_args<BT>(L);
  const dim3 grid = spmm_grid(L);
  kern<<<grid, kSpmmCta, bytes, s>>>(a, tm, L.window_halo, status);
  return check_launch("spmm_window_kernel");
}

template <typename BT> int launch_window(const SpmmLaunch &L, cudaStream_t s) {
  switch (L.V * 100 + L.G) {
#define SEGTACO_WINDOW_CASE(V, G) \
  case V * 100 + G:               \
    return launch_window_variant<BT, V, G>(L, s);
    SEGTACO_WINDOW_CASE(8, 4)
    SEGTACO_WINDOW_CASE(4, 8)
    SEGTACO_WINDOW_CASE(8, 8)
    SEGTACO_WINDOW_CASE(4, 16)
    SEGTACO_WINDOW_CASE(8, 16)
    SEGTACO_WINDOW_CASE(1, 32)
    SEGTACO_WINDOW_CASE(2, 32)
#undef SEGTACO_WINDOW_CASE
    default:
      break;
  }
  if constexpr (sizeof(BT) == 2) {
    if (L.V == 16 && L.G == 4) return launch_window_variant<BT, 16, 4>(L, s);
  }
  return set_error(SEGTACO_EUNSUPPORTED, "window: no variant V=%d G=%d", L.V, L.G);
}

template <typename BT> int launch_band_typed(const SpmmLaunch &L, cudaStream_t s) {
  const int win = kBandRows + 2 * L.band_halo;
  if (L.band_halo < 0 || win > 256)
    return set_error(SEGTACO_EINVAL, "band window of %d rows (32 + 2*halo) > 256", win);
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return set_error(SEGTACO_EUNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  CUtensorMap tm;
  const cuuint64_t dims[2] = {(cuuint64_t)L.N, (cuuint64_t)L.K};
  const cuuint64_t strides[1] = {(cuuint64_t)L.ldb * sizeof(BT)};
  const cuuint32_t box[2] = {(cuuint32_t)kBandCols, (cuuint32_t)win};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = enc(&tm, sizeof(BT) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                               : CU_TENSOR_MAP_DATA_TYPE_UINT16,
                         2, const_cast<void *>(L.B), dims, strides, box, es,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return set_error(SEGTACO_EINVAL, "band: tensor map of B rejected (CUresult %d)", (int)r);
  const size_t bytes = band_smem<BT>(win).bytes;
  auto kern = spmm_band_kernel<BT>;
  static std::atomic<unsigned long long> opted{0};
  int dev = 0;
  SEGTACO_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(opted.load() & bit)) {
    SEGTACO_TRY(check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)(200 * 1024)),
                           "cudaFuncSetAttribute(spmm_band_kernel)"));
    opted.fetch_or(bit);
  }
  if (bytes > 200 * 1024) return set_error(SEGTACO_EINVAL, "band tiles of %zu bytes > 200 KB", bytes);
  int *status = nullptr;
  SEGTACO_TRY(tma_status_ptr(&status));
  const SpmmArgs<BT> a = make_spmm_args<BT>(L);
  const dim3 grid((unsigned)((L.M + kBandRows - 1) / kBandRows),
                  (unsigned)((L.N + kBandCols - 1) / kBandCols), 1);
  kern<<<grid, kSpmmCta, bytes, s>>>(a, tm, L.band_halo, status);
  return check_launch("spmm_band_kernel");
}

// Nonzeros within `halo` of the diagonal (row i scaled to column i*K/M).
// A warp per 32 consecutive rows: lane l reads the bounds of row r0 + l, then
// the warp walks each of the 32 rows with its lanes striding the row's
// nonzeros (coalesced; a row of 50,000 nonzeros costs its warp ~1,600 steps
// instead of one thread 50,000).
__global__ void band_stats_kernel(const int *__restrict__ row_ptr, const int *__restrict__ col,
                                  int M, int K, int halo, unsigned long long *out) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  unsigned long long n = 0;
  const long long warps = (long long)gridDim.x * (blockDim.x / 32);
  for (long long r0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / 32 * 32; r0 < M;
       r0 += warps * 32) {
    const long long rl = r0 + lane;
    const int b = rl < M ? __ldg(row_ptr + rl) : 0;
    const int e = rl < M ? __ldg(row_ptr + rl + 1) : 0;
    for (int i = 0; i < 32; ++i) {
      const int bi = __shfl_sync(FULL, b, i), ei = __shfl_sync(FULL, e, i);
      const long long d = (r0 + i) * (long long)K / M;
      for (int p = bi + lane; p < ei; p += 32) {
        const long long c = __ldg(col + p);
        n += (c >= d - halo && c <= d + halo) ? 1 : 0;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(out, n);
}

}  // namespace

int launch_band_stats(const int *row_ptr, const int *col, int M, int K, int halo,
                      unsigned long long *out, cudaStream_t s) {
  SEGTACO_TRY(check_cuda(cudaMemsetAsync(out, 0, sizeof(unsigned long long), s), "memset"));
  if (M <= 0) return SEGTACO_OK;
  long long blocks = (M + 255) / 256;  // 8 warps of 32 rows per block
  if (blocks > 4096) blocks = 4096;
  band_stats_kernel<<<(unsigned)blocks, 256, 0, s>>>(row_ptr, col, M, K, halo, out);
  return check_launch("band_stats_kernel");
}

bool window_variant_exists(int dtype, int V, int G) {
  const int k = V * 100 + G;
  if (k == 804 || k == 408 || k == 808 || k == 416 || k == 816 || k == 132 || k == 232)
    return true;
  return dtype == SEGTACO_BF16 && k == 1604;
}

int launch_spmm_window(const SpmmLaunch &L, cudaStream_t s) {
  return L.dtype == SEGTACO_BF16 ? launch_window<uint16_t>(L, s) : launch_window<float>(L, s);
}

int launch_spmm_band(const SpmmLaunch &L, cudaStream_t s) {
  return L.dtype == SEGTACO_BF16 ? launch_band_typed<uint16_t>(L, s)
                                 : launch_band_typed<float>(L, s);
}

}  // namespace segtaco

using namespace segtaco;

extern "C" int segtaco_band_stats(int32_t M, int32_t K, int64_t nnz, const int32_t *row_ptr,
                                  const int32_t *col, int32_t halo, int64_t *in_band,
                                  void *stream) {
  if (M < 0 || K < 0 || nnz < 0 || halo < 0 || !in_band)
    return set_error(SEGTACO_EINVAL, "segtaco_band_stats: bad arguments");
  *in_band = 0;
  if (M == 0 || nnz == 0) return SEGTACO_OK;
  if (!row_ptr || !col) return set_error(SEGTACO_EINVAL, "segtaco_band_stats: NULL CSR");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch scratch(nullptr, 0, s);
  SEGTACO_TRY(scratch.reserve(256));
  auto *d = static_cast<unsigned long long *>(scratch.take(sizeof(unsigned long long)));
  SEGTACO_TRY(launch_band_stats(row_ptr, col, M, K, halo, d, s));
  unsigned long long h = 0;
  SEGTACO_TRY(check_cuda(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s), "copy"));
  SEGTACO_TRY(check_cuda(cudaStreamSynchronize(s), "sync"));
  *in_band = (int64_t)h;
  return SEGTACO_OK;
}
