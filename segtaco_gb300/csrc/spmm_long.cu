// spmm_long.cu -- the long rows of the row-balanced SpMM schedules (rb_sr, rb_pr).
//
// In rb_sr every column of a row is one fmaf chain in storage order
// (segTACO spmm_rb_sr.h:187-243: one thread sums a row serially), so the
// row-block kernel walks a row with one warp per column slab, and that warp's
// B loads in flight (8 per lane) bound it: a 48,000-nonzero row of a
// power-law matrix takes ~3.6 ms at one DRAM round trip per 8 nonzeros while
// the rest of the product is done long before.  Here the rows of at least
// `long_row` nonzeros get a CTA per slab of 128 columns: all 128 threads copy
// the B row segments of the next stages of 64 nonzeros into a shared-memory
// ring with cp.async (3 stages, 192 B rows in flight per CTA), and thread t
// sums column t of the slab from the ring in storage order -- the same fmaf
// chain, so the result is bit-identical to the one-warp walk.  The row-block
// kernel skips those rows (SpmmArgs::long_row) and runs beside this one on the
// caller's stream; this kernel runs on a side stream forked from it and
// joined before the call returns (also inside a CUDA graph capture).
//
// Work list: long_rows_list_kernel appends every row of >= 8 * long_row
// nonzeros to the front part of `list` and every other row of >= long_row to
// the back part (long_list_caps gives both capacities) and counts them in
// counters[0] / counters[1]; the long-row CTAs take (row, slab) items, front
// part first (the longest rows start first), from the 64-bit queue
// counters[2..3], which is cleared on the side stream before each launch.
// Measured on GB300 (1M x 1M power law, Zipf 1.8, N = 128): rb_sr 3.94 ms
// with every row in the row-block kernel; 2.34 ms with long rows of >= 4096
// nonzeros here at 3 x 32 rows in flight (alone: 1.38 ms, held up by the
// longest row; the row-block kernel alone 1.21 ms); 2.23 ms at 3 x 64.
// Slabs of 32 columns (4 CTAs per row of N = 128, 7 x 64 rows in flight)
// took 2.79 ms: the gathers of B (512 MB, beyond L2) make this kernel
// DRAM-bound, and narrower slabs only re-read the row's indices.
//
// rb_pr splits a row over the lanes of one warp (segTACO spmm_rb_pr.h:223-375)
// and meets the same tail.  Its long rows become pieces of kPieceLen nonzeros
// that warps of the row-block launch itself take (spmm_walk_unit), over the
// same 32-column slabs as the short rows, so both share the slab's L2 working
// set: long_pieces_list_kernel lists them, each piece stores its partial row
// in the workspace and the last piece of a row (a counter per row and slab)
// sums the partial rows in piece order, so the result is the same from run to
// run.  Measured on GB300 (1M x 1M power law, N = 128): 1.69 ms with the
// long-row CTAs, 1.58 with pieces of 512 at 4 short rows per warp, 1.20 at
// 32, 1.114 with pieces of 4096 at 64.  The CTAs (each warp summing a
// quarter of every stage, the four partials folded at the end) remain for the
// allocation-free entry point where its fixed scratch cannot hold the partial
// rows.
#include <algorithm>
#include <atomic>

#include "spmm_launch.cuh"

namespace segtaco {
namespace {

constexpr int kLongCta = 128;   // threads of a long-row CTA
constexpr int kLongStage = 64;  // nonzeros per ring stage
constexpr int kLongRing = 4;    // stages in the ring (all but one in flight)
// The long-row CTAs launch at the device's highest priority and the row-block
// kernel beside them asks for the whole unified L1 as shared memory (it uses
// none): otherwise its CTAs fill the SMs first, under a carveout too small for
// a 132 KB ring, and the long rows wait for its last wave.  Measured on GB300
// (1M x 1M power law, N = 128, rb_sr / rb_pr): 2.01 / 2.11 ms without either,
// 1.95 / 2.01 with the priority, 2.17 / 2.22 with the carveout, 1.69 / 1.70
// with both (bf16 B: 1.25 / 1.36 -> 0.93 / 1.06).
constexpr int kRowBlockCarveout = 100;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async_16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_4(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ float to_f32(float x) { return x; }
__device__ __forceinline__ float to_f32(uint16_t x) { return bf16lo(x); }

// CPL consecutive dense values of a ring row as floats, in one shared load.
template <typename BT, int CPL>
__device__ __forceinline__ void lds_cols(const BT *p, float (&o)[CPL]) {
  constexpr int BYTES = CPL * (int)sizeof(BT);
  uint32_t w[BYTES >= 4 ? BYTES / 4 : 1];
  if constexpr (BYTES == 16) {
    const uint4 x = *reinterpret_cast<const uint4 *>(p);
    w[0] = x.x, w[1] = x.y, w[2] = x.z, w[3] = x.w;
  } else if constexpr (BYTES == 8) {
    const uint2 x = *reinterpret_cast<const uint2 *>(p);
    w[0] = x.x, w[1] = x.y;
  } else if constexpr (BYTES == 4) {
    w[0] = *reinterpret_cast<const uint32_t *>(p);
  } else {
    w[0] = *reinterpret_cast<const uint16_t *>(p);
  }
#pragma unroll
  for (int v = 0; v < CPL; ++v) {
    if constexpr (sizeof(BT) == 4)
      o[v] = __uint_as_float(w[v]);
    else
      o[v] = (v & 1) ? bf16hi(w[v >> 1]) : bf16lo(w[v >> 1]);
  }
}

__global__ void long_rows_list_kernel(const int *__restrict__ row_ptr, int M, int long_row,
                                      int *__restrict__ list, long long cap_hi,
                                      long long cap_lo, int *counters) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= M) return;
  const int len = __ldg(row_ptr + r + 1) - __ldg(row_ptr + r);
  if (len < long_row) return;
  if ((long long)len >= 8LL * long_row) {
    const int i = atomicAdd(counters, 1);
    if (i < cap_hi) list[i] = (int)r;
  } else {
    const int i = atomicAdd(counters + 1, 1);
    if (i < cap_lo) list[cap_hi + i] = (int)r;
  }
}

// rb_pr: thread per row; a row of >= long_row nonzeros appends its pieces of
// piece_len nonzeros: several (consecutive entries of the front part, the
// counters of its first piece cleared, one per column slab) or one (the back
// part, from entry `multi`; its counters cleared too when the pieces run in
// several passes, `all_ctr`).
__global__ void long_pieces_list_kernel(const int *__restrict__ row_ptr, int M, int long_row,
                                        int piece_len, int2 *__restrict__ pieces,
                                        long long multi, long long cap,
                                        unsigned *__restrict__ ctr, int slabs, int *count,
                                        bool all_ctr) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= M) return;
  const int b = __ldg(row_ptr + r);
  const int len = __ldg(row_ptr + r + 1) - b;
  if (len < long_row) return;
  const int n = (len + piece_len - 1) / piece_len;
  if (n == 1) {
    const long long i = multi + atomicAdd(count + 1, 1);
    if (i < cap) {
      pieces[i] = make_int2((int)r, b);
      if (all_ctr)
        for (int sl = 0; sl < slabs; ++sl) ctr[i * slabs + sl] = 0u;
    }
    return;
  }
  const long long i = atomicAdd(count, n);
  for (int k = 0; k < n && i + k < multi; ++k) pieces[i + k] = make_int2((int)r, b + k * piece_len);
  if (i < multi)
    for (int sl = 0; sl < slabs; ++sl) ctr[i * slabs + sl] = 0u;
}

// One CTA per (column slab of W columns, long row) item at a time; every
// thread copies: a row segment is CH = W / EPC sixteen-byte chunks, RP = 128 /
// CH rows per pass of the CTA.  Sequential (rb_sr): thread t sums column
// slab*W + t (t < W) over the whole row in storage order.  Parallel (PR,
// rb_pr): warp w sums rows w*16 .. w*16+15 of every stage of 64, lane l
// columns l*W/32 .. (l+1)*W/32-1 (one shared load), and the four warps'
// partial sums are folded as (w0 + w1) + (w2 + w3) at the row's end.
template <typename BT, int W, bool PR>
__global__ void __launch_bounds__(kLongCta)
    spmm_long_rows_kernel(SpmmArgs<BT> a, const int *__restrict__ list, long long cap_hi,
                          long long cap_lo, int *counters, int slabs) {
  constexpr int EPC = 16 / (int)sizeof(BT);
  constexpr int CH = W / EPC;
  constexpr int RP = kLongCta / CH;
  constexpr int RPT = kLongStage / RP;  // rows a thread copies per stage
  static_assert(CH <= kLongCta && kLongCta % CH == 0 && kLongStage % RP == 0, "ring layout");
  extern __shared__ __align__(128) unsigned char smem[];
  BT *ring = reinterpret_cast<BT *>(smem);  // [kLongRing][kLongStage][W]
  float *vring = reinterpret_cast<float *>(smem + sizeof(BT) * kLongRing * kLongStage * W);
  __shared__ long long item_s;

  const int t = threadIdx.x;
  const int c = t % CH, rr = t / CH;
  const long long n_hi = min((long long)counters[0], cap_hi);
  const long long n_lo = min((long long)counters[1], cap_lo);
  const long long items = (n_hi + n_lo) * slabs;
  unsigned long long *queue = reinterpret_cast<unsigned long long *>(counters + 2);
  const size_t ldb = (size_t)a.ldb;

  for (;;) {
    if (t == 0) item_s = (long long)atomicAdd(queue, 1ull);
    __syncthreads();
    const long long item = item_s;
    __syncthreads();  // everyone has read item_s before it is rewritten
    if (item >= items) break;
    // Front part (the longest rows) row by row with all their slabs; the
    // back part slab by slab, so that its CTAs share one slab of B at a time.
    long long li;
    int slab;
    if (item < n_hi * slabs) {
      li = item / slabs;
      slab = (int)(item - li * slabs);
    } else {
      const long long it = item - n_hi * slabs;  // n_lo > 0 here
      slab = (int)(it / n_lo);
      li = n_hi + (it - (long long)slab * n_lo);
    }
    const int r = __ldg(list + (li < n_hi ? li : cap_hi + (li - n_hi)));
    const int pb = __ldg(a.row_ptr + r), pe = __ldg(a.row_ptr + r + 1);
    const int col0 = slab * W;
    // This thread's chunk: columns col0 + c*EPC .. +EPC-1, all < N or all >= N
    // (N is a multiple of EPC).
    const bool chunk_in = col0 + c * EPC < a.N;
    const BT *Bc = a.B + col0 + c * EPC;
    const int nst = (pe - pb + kLongStage - 1) / kLongStage;

    int jn[RPT];  // column indices of the rows this thread copies next
    auto load_cols = [&](int st) {
      const int base = pb + st * kLongStage;
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        const int p = base + rr + RP * i;
        jn[i] = p < pe ? ld_stream(a.col + p) : -1;
      }
    };
    auto issue = [&](int st) {
      const int slot = st % kLongRing;
      BT *dst = ring + (size_t)slot * kLongStage * W + c * EPC;
#pragma unroll
      for (int i = 0; i < RPT; ++i) {
        if (jn[i] >= 0 && chunk_in)
          cp_async_16(dst + (rr + RP * i) * W, Bc + (size_t)(unsigned)jn[i] * ldb);
      }
      if (t < kLongStage) {
        const int p = pb + st * kLongStage + t;
        if (p < pe) {
          if (a.val)
            cp_async_4(vring + slot * kLongStage + t, a.val + p);
          else
            vring[slot * kLongStage + t] = 1.0f;
        }
      }
    };

#pragma unroll
    for (int st = 0; st < kLongRing - 1; ++st) {
      if (st < nst) {
        load_cols(st);
        issue(st);
      }
      cp_async_commit();
    }
    if (kLongRing - 1 < nst) load_cols(kLongRing - 1);

    constexpr int CPL = W / 32;             // PR: columns per lane
    constexpr int RW = kLongStage / 4;      // PR: rows of a stage per warp
    const int warp = t >> 5, lane = t & 31;
    float acc = 0.0f;
    float pacc[CPL];
#pragma unroll
    for (int v = 0; v < CPL; ++v) pacc[v] = 0.0f;
    for (int st = 0; st < nst; ++st) {
      cp_async_wait<kLongRing - 2>();  // stage st has landed (this thread's copies) ...
      __syncthreads();                 // ... and every thread's; slot st-1 is free
      const int sn = st + kLongRing - 1;
      if (sn < nst) issue(sn);
      cp_async_commit();
      if (sn + 1 < nst) load_cols(sn + 1);
      if constexpr (PR) {
        const int slot = st % kLongRing;
        const BT *src = ring + (size_t)slot * kLongStage * W + lane * CPL;
        const float *vs = vring + slot * kLongStage;
        const int cnt = min(kLongStage, pe - (pb + st * kLongStage));
        const int iend = min(warp * RW + RW, cnt);
#pragma unroll 4
        for (int i = warp * RW; i < iend; ++i) {
          float b[CPL];
          lds_cols<BT, CPL>(src + i * W, b);
          const float v = vs[i];
#pragma unroll
          for (int u = 0; u < CPL; ++u) pacc[u] = fmaf(v, b[u], pacc[u]);
        }
      } else if (t < W) {
        const int slot = st % kLongRing;
        const BT *src = ring + (size_t)slot * kLongStage * W + t;
        const float *vs = vring + slot * kLongStage;
        const int cnt = min(kLongStage, pe - (pb + st * kLongStage));
        if (cnt == kLongStage) {
#pragma unroll 8
          for (int i = 0; i < kLongStage; ++i) acc = fmaf(vs[i], to_f32(src[i * W]), acc);
        } else {
          for (int i = 0; i < cnt; ++i) acc = fmaf(vs[i], to_f32(src[i * W]), acc);
        }
      }
    }
    if constexpr (PR) {
      // Fold the warps' partial sums through the (drained) ring.
      float *part = reinterpret_cast<float *>(smem);  // [4][W]
      __syncthreads();
#pragma unroll
      for (int u = 0; u < CPL; ++u) part[warp * W + lane * CPL + u] = pacc[u];
      __syncthreads();
      if (t < W)
        acc = (part[t] + part[W + t]) + (part[2 * W + t] + part[3 * W + t]);
    }
    if (t < W && col0 + t < a.N) a.C[(long long)r * a.ldc + col0 + t] = acc;
  }
}

template <typename BT, int W> constexpr size_t long_smem_bytes() {
  return sizeof(BT) * kLongRing * kLongStage * W + sizeof(float) * kLongRing * kLongStage;
}

template <typename BT, int W, bool PR>
int launch_long_kernel(const SpmmArgs<BT> &a, const int *list, int *counters, int sms,
                       cudaStream_t s) {
  long long cap_hi, cap_lo;
  long_list_caps(a.nnz, a.long_row, &cap_hi, &cap_lo);
  constexpr size_t bytes = long_smem_bytes<BT, W>();
  // The shared-memory opt-in, once per device (so a later graph capture of
  // the call makes no attribute call).
  static std::atomic<unsigned long long> opted{0};
  int dev = 0;
  SEGTACO_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(opted.load() & bit)) {
    SEGTACO_TRY(check_cuda(cudaFuncSetAttribute(spmm_long_rows_kernel<BT, W, PR>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)bytes),
                           "cudaFuncSetAttribute(spmm_long_rows_kernel)"));
    opted.fetch_or(bit);
  }
  const int slabs = (a.N + W - 1) / W;
  // Persistent CTAs: as many as fit beside the row-block kernel, at most two
  // per SM and at most one per item.
  const long long per_sm = bytes <= 100 * 1024 ? 2 : 1;
  const long long g = std::min<long long>(sms * per_sm, (cap_hi + cap_lo) * (long long)slabs);
  int least = 0, greatest = 0;
  SEGTACO_TRY(check_cuda(cudaDeviceGetStreamPriorityRange(&least, &greatest),
                         "cudaDeviceGetStreamPriorityRange"));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)std::max<long long>(g, 1));
  cfg.blockDim = dim3(kLongCta);
  cfg.dynamicSmemBytes = bytes;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePriority;
  attr[0].val.priority = greatest;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return check_cuda(cudaLaunchKernelEx(&cfg, spmm_long_rows_kernel<BT, W, PR>, a, list, cap_hi,
                                       cap_lo, counters, slabs),
                    "cudaLaunchKernelEx(spmm_long_rows_kernel)");
}

template <typename BT>
int launch_long_typed(const SpmmLaunch &L, const int *list, int *counters, int sms,
                      cudaStream_t s) {
  const SpmmArgs<BT> a = make_spmm_args<BT>(L);
  // Slabs of 128 columns (one per row at N <= 128); 32 or 64 for narrower N.
  // rb_sr plans one slot of 32 lanes (G = 32), rb_pr several.
  if (L.G == 32) {
    // The row-block kernel's slab width (its B working set) where narrower.
    const int W = L.V * L.G;
    if (L.N <= 32 || W <= 32) return launch_long_kernel<BT, 32, false>(a, list, counters, sms, s);
    if (L.N <= 64 || W <= 64) return launch_long_kernel<BT, 64, false>(a, list, counters, sms, s);
    return launch_long_kernel<BT, 128, false>(a, list, counters, sms, s);
  }
  if (L.N <= 32) return launch_long_kernel<BT, 32, true>(a, list, counters, sms, s);
  if (L.N <= 64) return launch_long_kernel<BT, 64, true>(a, list, counters, sms, s);
  return launch_long_kernel<BT, 128, true>(a, list, counters, sms, s);
}

// Side stream and events of one host thread on one device, kept for the
// thread's lifetime and destroyed when the thread exits (a thread pool that
// retires threads does not pile them up).  At process exit the CUDA runtime
// may already be unloaded; the destroy calls then fail and are ignored.
struct LongFork {
  cudaStream_t side = nullptr;
  cudaEvent_t start = nullptr, done = nullptr;
};
constexpr int kForkDevices = 64;
struct LongForks {
  LongFork dev[kForkDevices];
  ~LongForks() {
    for (LongFork &f : dev) {
      if (f.side) cudaStreamDestroy(f.side);
      if (f.start) cudaEventDestroy(f.start);
      if (f.done) cudaEventDestroy(f.done);
    }
    cudaGetLastError();
  }
};
thread_local LongForks t_forks;

// The fork of this thread on the current device, created on first use (not
// while `s` is being captured: then the caller runs both kernels on `s`).
LongFork *long_fork(cudaStream_t s) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (dev < 0 || dev >= kForkDevices) return nullptr;
  LongFork &t_fork = t_forks.dev[dev];
  if (t_fork.side) return &t_fork;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (cs != cudaStreamCaptureStatusNone) return nullptr;
  LongFork f;
  if (cudaStreamCreateWithFlags(&f.side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&f.start, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    if (f.side) cudaStreamDestroy(f.side);
    if (f.start) cudaEventDestroy(f.start);
    return nullptr;
  }
  t_fork = f;
  return &t_fork;
}

}  // namespace

int device_sms() {
  static std::atomic<int> counts[kForkDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kForkDevices) {
    cudaGetLastError();
    return 148;
  }
  int n = counts[dev].load(std::memory_order_relaxed);
  if (n < 1) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
      cudaGetLastError();
      n = 148;
    }
    counts[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

int launch_long_rows_list(const int *row_ptr, int M, long long nnz, int long_row, int *list,
                          int *counters, cudaStream_t s) {
  long long cap_hi, cap_lo;
  long_list_caps(nnz, long_row, &cap_hi, &cap_lo);
  SEGTACO_TRY(check_cuda(cudaMemsetAsync(counters, 0, 4 * sizeof(int), s), "cudaMemsetAsync"));
  if (M <= 0) return SEGTACO_OK;
  long_rows_list_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(row_ptr, M, long_row, list,
                                                                    cap_hi, cap_lo, counters);
  return check_launch("long_rows_list_kernel");
}

int launch_long_pieces_list(const int *row_ptr, int M, long long nnz, int long_row, int piece_len,
                            int slabs, int W, int parts, int *pieces, int *count, cudaStream_t s) {
  SEGTACO_TRY(check_cuda(cudaMemsetAsync(count, 0, 2 * sizeof(int), s), "cudaMemsetAsync"));
  if (M <= 0) return SEGTACO_OK;
  const PieceLayout pl = piece_layout(nnz, long_row, piece_len, slabs, W, parts);
  long_pieces_list_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(
      row_ptr, M, long_row, piece_len, reinterpret_cast<int2 *>(pieces), pl.multi, pl.cap,
      reinterpret_cast<unsigned *>(pieces + pl.ctr), slabs, count, parts > 1);
  return check_launch("long_pieces_list_kernel");
}

int launch_spmm_long_rows(const SpmmLaunch &L, const int *list, int *counters, cudaStream_t s) {
  const bool bf16 = L.dtype == SEGTACO_BF16;
  const int sms = device_sms();
  // The work queue is cleared before the fork, so that the long-row kernel is
  // the side stream's first operation and reaches the GPU before the
  // row-block kernel.
  SEGTACO_TRY(check_cuda(cudaMemsetAsync(counters + 2, 0, sizeof(unsigned long long), s),
                         "cudaMemsetAsync"));
  // segtaco_spmm_noalloc creates no side stream: both kernels go to `s`.
  LongFork *f = L.no_fork ? nullptr : long_fork(s);
  cudaStream_t ls = f ? f->side : s;
  if (f) {
    SEGTACO_TRY(check_cuda(cudaEventRecord(f->start, s), "cudaEventRecord"));
    SEGTACO_TRY(check_cuda(cudaStreamWaitEvent(f->side, f->start, 0), "cudaStreamWaitEvent"));
  }
  int st = bf16 ? launch_long_typed<uint16_t>(L, list, counters, sms, ls)
                : launch_long_typed<float>(L, list, counters, sms, ls);
  // The row-block kernel on the caller's stream (beside the side stream's
  // long-row CTAs when forked).
  SpmmLaunch R = L;
  R.carveout = kRowBlockCarveout;
  if (st == SEGTACO_OK) st = bf16 ? launch_spmm_bf16_rows(R, s) : launch_spmm_f32_rows(R, s);
  // Join the side stream whatever happened, so that a capture stays whole.
  if (f) {
    const int j1 = check_cuda(cudaEventRecord(f->done, f->side), "cudaEventRecord");
    const int j2 = check_cuda(cudaStreamWaitEvent(s, f->done, 0), "cudaStreamWaitEvent");
    if (st == SEGTACO_OK) st = j1 != SEGTACO_OK ? j1 : j2;
  }
  return st;
}

}  // namespace segtaco
