// sddmm_band.cu -- SDDMM on banded matrices: out[k] = val[k] * <X[i], Y[j]> for
// the nonzeros (i, j) of A that lie near the diagonal.
//
// The warp-block SDDMM kernels (sddmm.cu) gather Y[j] once per nonzero (256
// bytes for D = 64 fp32) and keep X[i] in registers while a row lasts; on a
// banded matrix those gathers hit L1 and the load/store data pipe bounds them.
// Rows i and i + 1 share almost all of their band, so here a CTA owns 32
// consecutive rows and computes every dot product of its band at once: it
// stages the rows' X block (32 x D) and the Y window of 32 + 2 kSbHalo rows
// around the diagonal (column i0 * K / M of its first row) in shared memory,
// both transposed (d-major), and each thread forms a 4 x 6 block of the dense
// tile <X[4rb + q], Y[jw0 + 6cb + c]> with 4 shared loads per step of d for
// 24 multiply-adds.  The tile then goes to shared memory and every nonzero of
// the block reads its dot product there.  Nonzeros outside the window (off
// band) are listed (kSbList per block) and then computed by 16 lanes each, 4
// elements per lane from a row-major copy of the X block and Y[j] in global
// memory, summed by shuffles; beyond the list a thread computes the dot
// product alone.  The tile holds dot products for window positions without a
// nonzero too (96 per row instead of ~2 kSbHalo + 1).
#include "common.cuh"
#include "internal.h"

namespace segtaco {
namespace {

constexpr int kSbRows = 32;                     // rows per CTA
constexpr int kSbHalo = 32;                     // window rows on either side
constexpr int kSbWin = kSbRows + 2 * kSbHalo;  // 96 window rows
constexpr int kSbD = 64;                        // dot-product length
// Pitches (floats) of the transposed X block and Y window: 16-byte rows for X
// (a thread reads its 4 rows with one 16-byte load), 8-byte rows for Y whose
// 6-column reads of 16 threads cover 32 distinct banks.
constexpr int kSbXP = kSbRows + 4;
constexpr int kSbYP = kSbWin + 2;
constexpr int kSbCta = 128;
constexpr int kSbList = 512;  // off-band nonzeros listed per block
constexpr int kSbXR = kSbD + 4;  // pitch of the row-major X copy (floats)

// Four consecutive X or Y values as floats (fp32: 16 bytes; bf16: 8 bytes).
template <typename XT> __device__ __forceinline__ float4 sb_ld4(const XT *p) {
  if constexpr (sizeof(XT) == 4) {
    return __ldg(reinterpret_cast<const float4 *>(p));
  } else {
    const uint2 x = __ldg(reinterpret_cast<const uint2 *>(p));
    return make_float4(bf16lo(x.x), bf16hi(x.x), bf16lo(x.y), bf16hi(x.y));
  }
}

template <typename XT>
__global__ void __launch_bounds__(kSbCta, 6)  // 34.4 KB of shared memory: six per SM
    sddmm_band_kernel(int M, int K, const int *__restrict__ row_ptr, const int *__restrict__ col,
                      const float *__restrict__ val, const XT *__restrict__ X,
                      const XT *__restrict__ Y, long long ldx, long long ldy,
                      float *__restrict__ out) {
  __shared__ __align__(16) float xt[kSbD * kSbXP];  // xt[d][r]
  __shared__ __align__(16) float yt[kSbD * kSbYP];  // yt[d][jr]; later the tile [r][jr]
  __shared__ int rp[kSbRows + 1];
  __shared__ int lcount;
  // Off-band nonzeros (k, row, column, value bits), in the X block's space once
  // the tile product no longer reads it.
  static_assert(kSbList * 4 <= kSbD * kSbXP, "the list fits the transposed X block");
  int4 *lst = reinterpret_cast<int4 *>(xt);
  const int t = threadIdx.x;
  const int i0 = blockIdx.x * kSbRows;
  const int jw0 = (int)((long long)i0 * K / M) - kSbHalo;
  // X block and Y window, transposed; rows outside [0, M) / [0, K) are zeros.
  // Every thread loads its 4 X and 12 Y vectors, four at a time, before it
  // stores them.
  static_assert(kSbRows * (kSbD / 4) == 4 * kSbCta && kSbWin * (kSbD / 4) == 12 * kSbCta,
                "staging shape");
  constexpr int kSv = 8;  // vectors in flight per thread
#pragma unroll
  for (int pass = 0; pass < 16 / kSv; ++pass) {
    float4 v[kSv];
#pragma unroll
    for (int u = 0; u < kSv; ++u) {
      const int e = t + (pass * kSv + u) * kSbCta;  // 0 .. 511: X, 512 .. 2047: Y
      if (e < kSbRows * (kSbD / 4)) {
        const int i = i0 + e / (kSbD / 4);
        v[u] = i < M ? sb_ld4<XT>(X + (size_t)i * ldx + 4 * (e % (kSbD / 4)))
                     : make_float4(0, 0, 0, 0);
      } else {
        const int e2 = e - kSbRows * (kSbD / 4);
        const int j = jw0 + e2 / (kSbD / 4);
        v[u] = j >= 0 && j < K ? sb_ld4<XT>(Y + (size_t)j * ldy + 4 * (e2 % (kSbD / 4)))
                               : make_float4(0, 0, 0, 0);
      }
    }
#pragma unroll
    for (int u = 0; u < kSv; ++u) {
      const int e = t + (pass * kSv + u) * kSbCta;
      float *dst;
      int pitch, col, q;
      if (e < kSbRows * (kSbD / 4)) {
        dst = xt, pitch = kSbXP, col = e / (kSbD / 4), q = e % (kSbD / 4);
      } else {
        const int e2 = e - kSbRows * (kSbD / 4);
        dst = yt, pitch = kSbYP, col = e2 / (kSbD / 4), q = e2 % (kSbD / 4);
      }
      dst[(4 * q + 0) * pitch + col] = v[u].x;
      dst[(4 * q + 1) * pitch + col] = v[u].y;
      dst[(4 * q + 2) * pitch + col] = v[u].z;
      dst[(4 * q + 3) * pitch + col] = v[u].w;
    }
  }
  if (t <= kSbRows) rp[t] = __ldg(row_ptr + min(i0 + t, M));
  if (t == 0) lcount = 0;
  __syncthreads();
  // The dense tile: rows 4rb .. 4rb+3 x window rows 6cb .. 6cb+5.
  const int rb = t >> 4, cb = t & 15;
  float acc[4][6];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[q][c] = 0.0f;
#pragma unroll 4
  for (int d = 0; d < kSbD; ++d) {
    const float4 x4 = *reinterpret_cast<const float4 *>(xt + d * kSbXP + 4 * rb);
    const float x[4] = {x4.x, x4.y, x4.z, x4.w};
    float y[6];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 y2 = *reinterpret_cast<const float2 *>(yt + d * kSbYP + 6 * cb + 2 * c);
      y[2 * c] = y2.x;
      y[2 * c + 1] = y2.y;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int c = 0; c < 6; ++c) acc[q][c] = fmaf(x[q], y[c], acc[q][c]);
  }
  __syncthreads();  // every thread is done with yt
  float *tile = yt;  // tile[r][jr], pitch kSbYP
  float *xr = yt + kSbRows * kSbYP;  // X block row-major, pitch kSbXR (after the tile)
  static_assert(kSbRows * kSbYP + kSbRows * kSbXR <= kSbD * kSbYP, "tile and X copy fit");
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int c = 0; c < 6; ++c) tile[(4 * rb + q) * kSbYP + 6 * cb + c] = acc[q][c];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int e = t + u * kSbCta;  // 0 .. 511: row e / 16, elements 4 (e % 16) ..
    const int i = i0 + e / (kSbD / 4);
    const float4 x = i < M ? sb_ld4<XT>(X + (size_t)i * ldx + 4 * (e % (kSbD / 4)))
                           : make_float4(0, 0, 0, 0);
    *reinterpret_cast<float4 *>(xr + (e / (kSbD / 4)) * kSbXR + 4 * (e % (kSbD / 4))) = x;
  }
  __syncthreads();
  // The block's nonzeros, coalesced, eight per thread per pass.
  constexpr int SQ = 8;
  const int k_end = rp[kSbRows];
  for (int k0 = rp[0] + t; k0 < k_end; k0 += SQ * kSbCta) {
    int cj[SQ];
    float cv[SQ];
#pragma unroll
    for (int u = 0; u < SQ; ++u) {
      const int k = k0 + u * kSbCta;
      cj[u] = k < k_end ? __ldg(col + k) : 0;
      cv[u] = k < k_end ? (val ? __ldg(val + k) : 1.0f) : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < SQ; ++u) {
      const int k = k0 + u * kSbCta;
      if (k < k_end) {
        int r = 0;  // the last row whose start is <= k
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (r + step <= kSbRows - 1 && rp[r + step] <= k) r += step;
        const unsigned dj = (unsigned)(cj[u] - jw0);
        if (dj < (unsigned)kSbWin) {
          out[k] = cv[u] * tile[r * kSbYP + dj];
        } else {
          const int slot = atomicAdd(&lcount, 1);
          if (slot < kSbList) {
            lst[slot] = make_int4(k, r, cj[u], __float_as_int(cv[u]));
          } else {
            // past the list: the dot product by this thread alone
            const XT *yr = Y + (size_t)(unsigned)cj[u] * ldy;
            float s = 0.0f;
#pragma unroll 4
            for (int q = 0; q < kSbD / 4; ++q) {
              const float4 y = sb_ld4<XT>(yr + 4 * q);
              const float4 x = *reinterpret_cast<const float4 *>(xr + r * kSbXR + 4 * q);
              s = fmaf(x.x, y.x, s);
              s = fmaf(x.y, y.y, s);
              s = fmaf(x.z, y.z, s);
              s = fmaf(x.w, y.w, s);
            }
            out[k] = cv[u] * s;
          }
        }
      }
    }
  }
  __syncthreads();
  // Listed off-band nonzeros: 16 lanes each (lane l: elements 4l .. 4l+3); a
  // warp takes two per step, four steps with their gathers in flight at once,
  // and every lane of it takes part in the shuffles.
  const int n = min(lcount, kSbList);
  const int w = t >> 5, hw = (t >> 4) & 1, l = t & 15;
  constexpr int kSteps = 4, kStride = kSbCta / 16;  // 8 entries per step over the CTA
  for (int e0 = 2 * w; e0 < n; e0 += kSteps * kStride) {
    int4 it[kSteps];
    float4 y[kSteps];
#pragma unroll
    for (int u = 0; u < kSteps; ++u) {
      const int e = e0 + u * kStride + hw;
      it[u] = lst[e < n ? e : e0];  // past the list: entry e0 again, not stored
      y[u] = sb_ld4<XT>(Y + (size_t)(unsigned)it[u].z * ldy + 4 * l);
    }
#pragma unroll
    for (int u = 0; u < kSteps; ++u) {
      const float4 x = *reinterpret_cast<const float4 *>(xr + it[u].y * kSbXR + 4 * l);
      float s = x.x * y[u].x;
      s = fmaf(x.y, y[u].y, s);
      s = fmaf(x.z, y[u].z, s);
      s = fmaf(x.w, y[u].w, s);
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, 16);
      if (e0 + u * kStride + hw < n && l == 0) out[it[u].x] = __int_as_float(it[u].w) * s;
    }
  }
}

}  // namespace

bool sddmm_band_applies(int x_dtype, int D, long long ldx, long long ldy, const void *X,
                        const void *Y) {
  const int esz = x_dtype == SEGTACO_BF16 ? 2 : 4;
  const uintptr_t al = (uintptr_t)X | (uintptr_t)Y;
  return D == kSbD && ldx % 4 == 0 && ldy % 4 == 0 && (al % (4 * esz)) == 0;
}

int launch_sddmm_band(int M, int K, long long nnz, const int *row_ptr, const int *col,
                      const float *val, const void *X, const void *Y, int x_dtype, long long ldx,
                      long long ldy, int D, float *out, cudaStream_t s) {
  if (nnz == 0 || M == 0) return SEGTACO_OK;
  if (!sddmm_band_applies(x_dtype, D, ldx, ldy, X, Y))
    return set_error(SEGTACO_EINVAL,
                     "sddmm band kernel: needs D = 64, ldx and ldy multiples of 4 and X, Y "
                     "aligned to 4 elements");
  const dim3 grid((unsigned)((M + kSbRows - 1) / kSbRows));
  if (x_dtype == SEGTACO_BF16)
    sddmm_band_kernel<uint16_t><<<grid, kSbCta, 0, s>>>(
        M, K, row_ptr, col, val, static_cast<const uint16_t *>(X),
        static_cast<const uint16_t *>(Y), ldx, ldy, out);
  else
    sddmm_band_kernel<float><<<grid, kSbCta, 0, s>>>(M, K, row_ptr, col, val,
                                                     static_cast<const float *>(X),
                                                     static_cast<const float *>(Y), ldx, ldy, out);
  return check_launch("sddmm_band_kernel");
}

}  // namespace segtaco
