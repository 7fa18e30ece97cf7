// sddmm.cu -- out[p] = vals[p] * <X[i,:], Y[j,:]> for every nonzero p = (i, j).
//
// segTACO's SDDMM (sddmm_csr_gpu_taco.h:5-150, CPU reference sddmm_csr_gpu.h:9-50)
// is element-balanced: nonzero blocks with start rows from
// taco_binarySearchBeforeBlock.  Here a warp takes a block of kSddmmBlock
// nonzeros whose start row is the canonical block start; a group of G lanes
// computes one dot product with V-wide loads of X[i] and Y[j] (one 16-byte load
// per lane for D = 64 fp32 or D = 64 bf16), reduces it with xor shuffles, and
// the 32 results of a batch leave in one coalesced store.  The loads of U = 4
// steps (4P nonzeros) are issued before their multiply-adds.  X[i] is re-read
// for every nonzero of row i but stays in L1.
#include <climits>

#include "common.cuh"
#include "internal.h"

namespace segtaco {

constexpr int kSddmmBlock = 256;  // nonzeros per warp

template <typename XT, int V, int G, int U = (V == 8 ? 1 : 4)>
__global__ void __launch_bounds__(kCta, 3) sddmm_kernel(int M, long long nnz,
                                                    const int *__restrict__ row_ptr,
                                                    const int *__restrict__ col,
                                                    const float *__restrict__ val,
                                                    const XT *__restrict__ X,
                                                    const XT *__restrict__ Y, long long ldx,
                                                    long long ldy, int D, float *__restrict__ out,
                                                    const int *__restrict__ starts,
                                                    long long nblk, int blk) {
  constexpr int P = 32 / G;  // nonzeros per step
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int g = lane / G, gl = lane & (G - 1);
  const long long w = (long long)blockIdx.x * (kCta / 32) + threadIdx.x / 32;
  if (w >= nblk) return;
  const long long pb = w * blk;
  const long long pe = pb + blk < nnz ? pb + blk : nnz;
  int wb = __ldg(starts + w);  // row of nonzero pb
  int rw = (wb + lane < M) ? __ldg(row_ptr + wb + 1 + lane) : INT_MAX;
  for (long long p = pb; p < pe; p += 32) {
    const int nb = (int)(pe - p < 32 ? pe - p : 32);
    const int mc = lane < nb ? ld_stream(col + p + lane) : 0;
    const float mv = lane < nb ? (val ? ld_stream(val + p + lane) : 1.0f) : 0.0f;
    for (;;) {
      const int adv = __popc(__ballot_sync(FULL, (long long)rw <= p));
      if (adv == 0) break;
      wb += adv;
      rw = (wb + lane < M) ? __ldg(row_ptr + wb + 1 + lane) : INT_MAX;
    }
    const bool covered = (long long)__shfl_sync(FULL, rw, 31) > p + nb - 1;
    float res = 0.0f;
    const int nsteps = (nb + P - 1) / P;
    // Steps of P nonzeros, U at a time: every load of the U steps is issued
    // before the first multiply-add.
    for (int s0 = 0; s0 < nsteps; s0 += U) {
      int rows[U], js[U];
      bool ok[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int s = s0 + u;
        const int t = s * P + g;
        ok[u] = s < nsteps && t < nb;
        js[u] = __shfl_sync(FULL, mc, t & 31);
        int row = wb;
        if (covered) {
#pragma unroll
          for (int gg = 0; gg < P; ++gg) {
            const unsigned bal = __ballot_sync(FULL, (long long)rw <= p + s * P + gg);
            if (g == gg) row = wb + __popc(bal);
          }
        } else if (ok[u]) {
          int lo = wb, hi = M - 1;
          const long long q = p + t;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((long long)__ldg(row_ptr + mid) <= q)
              lo = mid;
            else
              hi = mid - 1;
          }
          row = lo;
        }
        rows[u] = row;
      }
      float acc[U];
#pragma unroll
      for (int u = 0; u < U; ++u) acc[u] = 0.0f;
      for (int k = gl * V; k < D; k += G * V) {
        float xa[U][V], ya[U][V];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (ok[u]) {
            DenseLoad<XT, V, false>::run(X + (long long)rows[u] * ldx + k, xa[u], 0);
            DenseLoad<XT, V, false>::run(Y + (long long)js[u] * ldy + k, ya[u], 0);
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (ok[u]) {
#pragma unroll
            for (int v = 0; v < V; ++v) acc[u] = fmaf(xa[u][v], ya[u][v], acc[u]);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        float a = acc[u];
#pragma unroll
        for (int o = 1; o < G; o <<= 1) a += __shfl_xor_sync(FULL, a, o);
        // Nonzero t of step s was reduced by group t - s*P; lane t keeps it.
        const int s = s0 + u;
        const float r = __shfl_sync(FULL, a, ((lane - s * P) & (P - 1)) * G);
        if (lane / P == s) res = r;
      }
    }
    if (lane < nb) out[p + lane] = mv * res;
  }
}

// Sixteen-byte vectors and D = G*V*KI: G lanes per dot product, each lane
// KI vector loads of X[i] and of Y[j] (KI = 4 whenever D allows), so one step
// covers P = 32/G nonzeros and its reduction takes only log2(G) shuffles.  The
// row of every nonzero of a batch is found once (a search of the 32-row
// window, or of row_ptr when the batch leaves it) and passed by one shuffle
// per step.  A group keeps its slice of X[i] in registers until its row
// changes.  Raw vectors stay in registers until their multiply-adds.
template <typename XT, int V, int G, int KI>
__device__ __forceinline__ void sddmm_fixed_block(
    int M, long long nnz, const int *__restrict__ row_ptr, const int *__restrict__ col,
    const float *__restrict__ val, const XT *__restrict__ X, const XT *__restrict__ Y,
    long long ldx, long long ldy, float *__restrict__ out, const int *__restrict__ starts,
    long long w, int blk) {
  constexpr int P = 32 / G;
  using Dv = Dense<XT, V>;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int g = lane / G, gl = lane & (G - 1);
  const uint64_t pol = l2_policy_evict_normal();
  const long long pb = w * blk;
  const long long pe = pb + blk < nnz ? pb + blk : nnz;
  int wb = __ldg(starts + w);  // row of nonzero pb
  int rw = (wb + lane < M) ? __ldg(row_ptr + wb + 1 + lane) : INT_MAX;
  // The group's slice of X[xrow] stays in registers while its nonzeros stay in
  // that row (consecutive nonzeros of a row go to the same group's steps).
  typename Dv::raw_t xa[KI];
  int xrow = -1;
  for (long long p = pb; p < pe; p += 32) {
    const int nb = (int)(pe - p < 32 ? pe - p : 32);
    const int mc = lane < nb ? ld_stream(col + p + lane) : 0;
    const float mv = lane < nb ? (val ? ld_stream(val + p + lane) : 1.0f) : 0.0f;
    for (;;) {
      const int adv = __popc(__ballot_sync(FULL, (long long)rw <= p));
      if (adv == 0) break;
      wb += adv;
      rw = (wb + lane < M) ? __ldg(row_ptr + wb + 1 + lane) : INT_MAX;
    }
    // Row of nonzero p + lane.
    const long long q = p + lane;
    int myrow;
    if ((long long)__shfl_sync(FULL, rw, 31) > p + nb - 1) {  // the window holds the batch
      int rr = 0;
#pragma unroll
      for (int st = 16; st > 0; st >>= 1)
        if ((long long)__shfl_sync(FULL, rw, rr + st - 1) <= q) rr += st;
      myrow = wb + rr;
    } else {
      int lo = wb, hi = M - 1;
      if (lane < nb) {
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if ((long long)__ldg(row_ptr + mid) <= q)
            lo = mid;
          else
            hi = mid - 1;
        }
      }
      myrow = lo;
    }
    float res = 0.0f;
    const int nsteps = (nb + P - 1) / P;
    for (int s = 0; s < nsteps; ++s) {
      const int t = s * P + g;
      const int j = __shfl_sync(FULL, mc, t & 31);
      const int row = __shfl_sync(FULL, myrow, t & 31);
      float acc = 0.0f;
      if (t < nb) {
        if (row != xrow) {  // a new row for this group: its slice of X[i]
          const XT *xr = X + (long long)row * ldx + gl * V;
#pragma unroll
          for (int k = 0; k < KI; ++k) xa[k] = Dv::load(xr + k * G * V, pol);
          xrow = row;
        }
        const XT *yr = Y + (long long)j * ldy + gl * V;
        typename Dv::raw_t ya[KI];
#pragma unroll
        for (int k = 0; k < KI; ++k) ya[k] = Dv::load(yr + k * G * V, pol);
#pragma unroll
        for (int k = 0; k < KI; ++k) {
#pragma unroll
          for (int v = 0; v < V; ++v) acc = fmaf(Dv::get(xa[k], v), Dv::get(ya[k], v), acc);
        }
      }
#pragma unroll
      for (int o = 1; o < G; o <<= 1) acc += __shfl_xor_sync(FULL, acc, o);
      const float r = __shfl_sync(FULL, acc, ((lane - s * P) & (P - 1)) * G);
      if (lane / P == s) res = r;
    }
    if (lane < nb) out[p + lane] = mv * res;
  }
}

template <typename XT, int V, int G, int KI>
__global__ void __launch_bounds__(kCta, 4) sddmm_fixed_kernel(
    int M, long long nnz, const int *__restrict__ row_ptr, const int *__restrict__ col,
    const float *__restrict__ val, const XT *__restrict__ X, const XT *__restrict__ Y,
    long long ldx, long long ldy, float *__restrict__ out, const int *__restrict__ starts,
    long long nblk, int blk) {
  const long long w = (long long)blockIdx.x * (kCta / 32) + threadIdx.x / 32;
  if (w >= nblk) return;  // whole warp leaves together
  sddmm_fixed_block<XT, V, G, KI>(M, nnz, row_ptr, col, val, X, Y, ldx, ldy, out, starts, w,
                                  blk);
}

// Several problems of one shape in one launch: warp w takes block
// w - blk_begin[p] of the last problem p with blk_begin[p] <= w.
template <typename XT, int V, int G, int KI>
__global__ void __launch_bounds__(kCta, 4) sddmm_fixed_multi_kernel(
    const SddmmProblem *__restrict__ probs, int nprobs, long long total) {
  const long long w = (long long)blockIdx.x * (kCta / 32) + threadIdx.x / 32;
  if (w >= total) return;  // whole warp leaves together
  int lo = 0, hi = nprobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].blk_begin <= w)
      lo = mid;
    else
      hi = mid - 1;
  }
  const SddmmProblem &a = probs[lo];
  sddmm_fixed_block<XT, V, G, KI>(a.M, a.nnz, a.row_ptr, a.col, a.val,
                                  static_cast<const XT *>(a.X), static_cast<const XT *>(a.Y),
                                  a.ldx, a.ldy, a.out, a.starts, w - a.blk_begin, kSddmmBlock);
}

// Fixed shapes (KI, G) of each family, for both launches.
#define SEGTACO_SDDMM_SHAPES32(X_) \
  X_(1, 1) X_(1, 2) X_(1, 4) X_(2, 4) X_(2, 8) X_(2, 16) X_(1, 8) X_(1, 16) X_(1, 32)
#define SEGTACO_SDDMM_SHAPES16(X_) \
  X_(1, 1) X_(2, 1) X_(4, 1) X_(4, 2) X_(4, 4) X_(4, 8) X_(4, 16) X_(4, 32)

// Fixed shape of an SDDMM (shared by the single and the multi-problem launch):
// family 1 = fp32 32-byte lanes (V = 8), 2 = bf16 32-byte lanes (V = 16),
// 3 = 16-byte lanes (V = 16 / element size), 0 = the general kernel.
SddmmShape sddmm_shape(int x_dtype, int D, long long ldx, long long ldy, const void *X,
                       const void *Y, int lanes) {
  SddmmShape sh;
  const int esz = x_dtype == SEGTACO_BF16 ? 2 : 4;
  const uintptr_t al = (uintptr_t)X | (uintptr_t)Y;
  int V = 16 / esz;
  while (V > 1 && (D % V != 0 || ldx % V != 0 || ldy % V != 0 || (al % (V * esz)) != 0)) V >>= 1;
  sh.V = V;
  // 32-byte lanes (one ld.global.v8), G >= 4 lanes reading whole 128-byte lines
  // of a row per load instruction (16-byte lanes read each line of Y in two
  // halves, and the kernel is bound by the L1 data pipe); KI <= 2 loads per
  // lane keep the variants within 64 registers.
  const int w32 = 32 / esz;
  if (V * esz == 16 && D % w32 == 0 && ldx % w32 == 0 && ldy % w32 == 0 && (al % 32) == 0) {
    const int T = D / w32;
    if (T >= 1 && T <= 32 && (T & (T - 1)) == 0) {
      sh.family = esz == 4 ? 1 : 2;
      sh.G = T < 4 ? T : (T / 2 > 4 ? T / 2 : 4);
      // A requested lane count with one load per lane, or two from 4 lanes
      // (the compiled shapes); other requests keep the default.
      if (lanes > 0 && (lanes & (lanes - 1)) == 0 && T % lanes == 0 &&
          (T / lanes == 1 || (T / lanes == 2 && lanes >= 4)))
        sh.G = lanes;
      sh.KI = T / sh.G;
      return sh;
    }
  }
  // Sixteen-byte vectors with D / V a power of two up to 128 (KI <= 4 loads).
  if (V * esz == 16 && D % V == 0) {
    const int T = D / V;
    if (T >= 1 && T <= 128 && (T & (T - 1)) == 0) {
      sh.family = 3;
      sh.KI = T < 4 ? T : 4;
      // A requested lane count with four loads per lane (the compiled
      // shapes); other requests keep the default.
      if (lanes > 0 && (lanes & (lanes - 1)) == 0 && T >= 4 && T % lanes == 0 && T / lanes == 4)
        sh.KI = 4;
      sh.G = T / sh.KI;
    }
  }
  return sh;
}

namespace {
// Switch over the family's shapes, each case launching CASE_(XT, V, KI, G).
#define SEGTACO_SDDMM_SWITCH(sh, x_dtype)                                                  \
  switch ((sh).family * 10000 + (sh).KI * 100 + (sh).G) {                                \
    SEGTACO_SDDMM_SHAPES32(SEGTACO_SDDMM_F1) SEGTACO_SDDMM_SHAPES32(SEGTACO_SDDMM_F2)     \
    default:                                                                             \
      if ((sh).family == 3 && (x_dtype) == SEGTACO_BF16) {                               \
        switch ((sh).KI * 100 + (sh).G) {                                                \
          SEGTACO_SDDMM_SHAPES16(SEGTACO_SDDMM_F3B)                                      \
          default: return set_error(SEGTACO_EUNSUPPORTED, "sddmm: no fixed shape");      \
        }                                                                                \
      } else if ((sh).family == 3) {                                                     \
        switch ((sh).KI * 100 + (sh).G) {                                                \
          SEGTACO_SDDMM_SHAPES16(SEGTACO_SDDMM_F3F)                                      \
          default: return set_error(SEGTACO_EUNSUPPORTED, "sddmm: no fixed shape");      \
        }                                                                                \
      } else {                                                                           \
        return set_error(SEGTACO_EUNSUPPORTED, "sddmm: no fixed shape");                 \
      }                                                                                  \
  }
#define SEGTACO_SDDMM_F1(KI_, G_) \
  case 10000 + KI_ * 100 + G_: CASE_(float, 8, KI_, G_) break;
#define SEGTACO_SDDMM_F2(KI_, G_) \
  case 20000 + KI_ * 100 + G_: CASE_(uint16_t, 16, KI_, G_) break;
#define SEGTACO_SDDMM_F3B(KI_, G_) \
  case KI_ * 100 + G_: CASE_(uint16_t, 8, KI_, G_) break;
#define SEGTACO_SDDMM_F3F(KI_, G_) \
  case KI_ * 100 + G_: CASE_(float, 4, KI_, G_) break;

int launch_fixed_single(const SddmmShape &sh, int x_dtype, dim3 grid, int M, long long nnz,
                        const int *row_ptr, const int *col, const float *val, const void *X,
                        const void *Y, long long ldx, long long ldy, float *out, const int *starts,
                        long long nblk, int blk, cudaStream_t s) {
#define CASE_(XT, V, KI, G)                                                                \
  sddmm_fixed_kernel<XT, V, G, KI><<<grid, kCta, 0, s>>>(M, nnz, row_ptr, col, val,       \
                                                         static_cast<const XT *>(X),      \
                                                         static_cast<const XT *>(Y), ldx, \
                                                         ldy, out, starts, nblk, blk);
  SEGTACO_SDDMM_SWITCH(sh, x_dtype)
#undef CASE_
  return check_launch("sddmm_fixed_kernel");
}

int launch_fixed_multi(const SddmmShape &sh, int x_dtype, dim3 grid, const SddmmProblem *probs,
                       int nprobs, long long total, cudaStream_t s) {
#define CASE_(XT, V, KI, G) \
  sddmm_fixed_multi_kernel<XT, V, G, KI><<<grid, kCta, 0, s>>>(probs, nprobs, total);
  SEGTACO_SDDMM_SWITCH(sh, x_dtype)
#undef CASE_
  return check_launch("sddmm_fixed_multi_kernel");
}

}  // namespace

#define SEGTACO_SDDMM_CASE(XT, V, G)                                                          \
  case V * 100 + G:                                                                           \
    sddmm_kernel<XT, V, G><<<grid, kCta, 0, s>>>(M, nnz, row_ptr, col, val,                   \
                                                 static_cast<const XT *>(X),                  \
                                                 static_cast<const XT *>(Y), ldx, ldy, D, out, \
                                                 starts, nblk, P);                            \
    break;

int launch_sddmm(int M, long long nnz, const int *row_ptr, const int *col, const float *val,
                 const void *X, const void *Y, int x_dtype, long long ldx, long long ldy, int D,
                 float *out, int *starts, int P, long long nblk, cudaStream_t s,
                 bool starts_ready, int lanes, int kernel) {
  if (nnz == 0) return SEGTACO_OK;
  if (!starts_ready)
    SEGTACO_TRY(launch_block_starts_canonical(row_ptr, M, P, nblk, starts, s));
  const dim3 grid((unsigned)((nblk + (kCta / 32) - 1) / (kCta / 32)));
  // The fixed-shape kernel where D and the operands allow it (unless the
  // general one is asked for); the general kernel (V-wide vectors, G lanes
  // covering D) otherwise.
  const SddmmShape sh = sddmm_shape(x_dtype, D, ldx, ldy, X, Y, lanes);
  if (sh.family != 0 && kernel != SEGTACO_SDDMM_GENERAL)
    return launch_fixed_single(sh, x_dtype, grid, M, nnz, row_ptr, col, val, X, Y, ldx, ldy, out,
                               starts, nblk, P, s);
  const int V = sh.V;
  // Lanes per dot product: enough to cover D in one pass, at most 32.
  int G = 1;
  while (G < 32 && G * V < D) G <<= 1;
  if (x_dtype == SEGTACO_BF16) {
    switch (V * 100 + G) {
      SEGTACO_SDDMM_CASE(uint16_t, 8, 1) SEGTACO_SDDMM_CASE(uint16_t, 8, 2)
      SEGTACO_SDDMM_CASE(uint16_t, 8, 4) SEGTACO_SDDMM_CASE(uint16_t, 8, 8)
      SEGTACO_SDDMM_CASE(uint16_t, 8, 16) SEGTACO_SDDMM_CASE(uint16_t, 8, 32)
      SEGTACO_SDDMM_CASE(uint16_t, 4, 1) SEGTACO_SDDMM_CASE(uint16_t, 4, 2)
      SEGTACO_SDDMM_CASE(uint16_t, 4, 4) SEGTACO_SDDMM_CASE(uint16_t, 4, 8)
      SEGTACO_SDDMM_CASE(uint16_t, 4, 16) SEGTACO_SDDMM_CASE(uint16_t, 4, 32)
      SEGTACO_SDDMM_CASE(uint16_t, 2, 1) SEGTACO_SDDMM_CASE(uint16_t, 2, 2)
      SEGTACO_SDDMM_CASE(uint16_t, 2, 4) SEGTACO_SDDMM_CASE(uint16_t, 2, 8)
      SEGTACO_SDDMM_CASE(uint16_t, 2, 16) SEGTACO_SDDMM_CASE(uint16_t, 2, 32)
      SEGTACO_SDDMM_CASE(uint16_t, 1, 1) SEGTACO_SDDMM_CASE(uint16_t, 1, 2)
      SEGTACO_SDDMM_CASE(uint16_t, 1, 4) SEGTACO_SDDMM_CASE(uint16_t, 1, 8)
      SEGTACO_SDDMM_CASE(uint16_t, 1, 16) SEGTACO_SDDMM_CASE(uint16_t, 1, 32)
      default:
        return set_error(SEGTACO_EUNSUPPORTED, "sddmm: no bf16 variant V=%d G=%d", V, G);
    }
  } else {
    switch (V * 100 + G) {
      SEGTACO_SDDMM_CASE(float, 4, 1) SEGTACO_SDDMM_CASE(float, 4, 2)
      SEGTACO_SDDMM_CASE(float, 4, 4) SEGTACO_SDDMM_CASE(float, 4, 8)
      SEGTACO_SDDMM_CASE(float, 4, 16) SEGTACO_SDDMM_CASE(float, 4, 32)
      SEGTACO_SDDMM_CASE(float, 2, 1) SEGTACO_SDDMM_CASE(float, 2, 2)
      SEGTACO_SDDMM_CASE(float, 2, 4) SEGTACO_SDDMM_CASE(float, 2, 8)
      SEGTACO_SDDMM_CASE(float, 2, 16) SEGTACO_SDDMM_CASE(float, 2, 32)
      SEGTACO_SDDMM_CASE(float, 1, 1) SEGTACO_SDDMM_CASE(float, 1, 2)
      SEGTACO_SDDMM_CASE(float, 1, 4) SEGTACO_SDDMM_CASE(float, 1, 8)
      SEGTACO_SDDMM_CASE(float, 1, 16) SEGTACO_SDDMM_CASE(float, 1, 32)
      default:
        return set_error(SEGTACO_EUNSUPPORTED, "sddmm: no f32 variant V=%d G=%d", V, G);
    }
  }
  return check_launch("sddmm_kernel");
}

int launch_sddmm_multi(const SddmmShape &sh, int x_dtype, const SddmmProblem *probs, int nprobs,
                      long long total_blocks, cudaStream_t s) {
  if (total_blocks <= 0 || nprobs <= 0) return SEGTACO_OK;
  if (sh.family == 0) return set_error(SEGTACO_EUNSUPPORTED, "sddmm: no fixed shape to batch");
  const dim3 grid((unsigned)((total_blocks + (kCta / 32) - 1) / (kCta / 32)));
  return launch_fixed_multi(sh, x_dtype, grid, probs, nprobs, total_blocks, s);
}

long long sddmm_block_nnz() { return kSddmmBlock; }

}  // namespace segtaco
