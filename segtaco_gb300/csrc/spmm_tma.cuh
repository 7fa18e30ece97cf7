// spmm_tma.cuh -- the SpMM segment kernel with B gathered by TMA bulk copies.
//
// Same work layout and row walk as spmm_seg_kernel (spmm_kernels.cuh): a warp
// owns one unit (merge-path chunk or row block) and one W-column slab; its 32
// lanes form P = 32/G slots; long rows are split over the slots, runs of short
// rows go one row per slot.  What differs is how the B row segments arrive:
//
//   * Producer.  The unit's nonzeros are cut into rounds of 32 positions; the
//     W-column segment of B row col[q] lands in slot (q - y0) mod 32*RR of a
//     per-warp shared-memory ring of RR rounds.  Two copy engines:
//       BULK = true : lane l issues one cp.async.bulk (TMA) copy of segment l;
//                     lane 0 arms the round's mbarrier with the byte count
//                     (mbarrier.arrive.expect_tx) and the copies complete on it;
//       BULK = false: the lanes issue the round's 32*G 16-byte pieces as
//                     cp.async.cg copies (G each) and every lane arrives on the
//                     round's mbarrier when its copies have landed
//                     (cp.async.mbarrier.arrive.noinc).
//     Up to RR rounds (RR*32 segments) are in flight per warp, none of them in
//     registers.  Small bulk copies are limited by the TMA request rate, so the
//     cp.async engine is the default for these 64-512 byte segments.
//   * Consumer.  Before it reads nonzero q the warp waits (mbarrier
//     try_wait.parity) for q's round; then each lane reads its V columns of the
//     segment with one ld.shared.v4 and does V multiply-adds.  A round's ring
//     slot is refilled (next round) once the walk has passed all of it.
//
// Every wait is bounded: after kSpinLimit polls the kernel records
// SEGTACO_ETIMEOUT in a device status word, waits (again bounded) for its own
// copies still in flight, and returns.  segtaco_device_status() reads and
// clears the word.
#pragma once

#include <climits>

#include "spmm_kernels.cuh"

namespace segtaco {

constexpr int kTmaWarps = 4;                  // warps per CTA
constexpr long long kSpinLimit = 1LL << 24;   // polls of one mbarrier before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait: true when the phase with `parity` completed.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long i = 0; i < kSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t bar, uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1], %2, [%3], %4;" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar), "l"(pol)
      : "memory");
}
// 16-byte asynchronous copy global -> shared through the load/store unit.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint64_t pol) {
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(dst),
               "l"(src), "l"(pol)
               : "memory");
}
// Arrive on `bar` once all of this thread's earlier cp.async copies have landed.
__device__ __forceinline__ void cp_async_arrive(uint32_t bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Raw 16-byte read of lane data from the ring.
__device__ __forceinline__ uint4 lds128(const unsigned char *p) {
  return *reinterpret_cast<const uint4 *>(p);
}
template <typename BT> struct Vec16;
template <> struct Vec16<float> {  // 4 floats
  static constexpr int V = 4;
  static __device__ __forceinline__ float get(const uint4 &r, int v) {
    const uint32_t w = v == 0 ? r.x : v == 1 ? r.y : v == 2 ? r.z : r.w;
    return __uint_as_float(w);
  }
};
template <> struct Vec16<uint16_t> {  // 8 bf16
  static constexpr int V = 8;
  static __device__ __forceinline__ float get(const uint4 &r, int v) {
    const uint32_t w = v < 2 ? r.x : v < 4 ? r.y : v < 6 ? r.z : r.w;
    return (v & 1) ? bf16hi(w) : bf16lo(w);
  }
};

struct TmaExtra {
  int *status;  // device status word (SEGTACO_ETIMEOUT on a timed-out wait)
};

// Dynamic shared memory of one CTA for (BT, G, RR).
template <typename BT, int G, int RR> constexpr int tma_smem_bytes() {
  return kTmaWarps * (RR * 32 * G * 16 + RR * 8);
}

// Ring depth: 16 KB of segments per warp, at least two rounds (a 32-position
// window of the walk can straddle two rounds).
template <int G> constexpr int tma_ring_rounds() { return 32 / G >= 2 ? 32 / G : 2; }

template <typename BT, int G, bool ROWS, int RR, bool BULK>
__global__ void __launch_bounds__(kTmaWarps * 32)
    spmm_tma_kernel(SpmmArgs<BT> a, TmaExtra ex) {
  static_assert(RR >= 2, "a window can straddle two rounds");
  using VT = Vec16<BT>;
  constexpr int V = VT::V;
  constexpr int P = 32 / G;
  constexpr int LONG = P == 1 ? 0 : (2 * P < 32 ? 2 * P : 32);
  constexpr int SEG = G * 16;       // bytes of one nonzero's slab segment
  constexpr int ROUND = 32 * SEG;   // bytes of one round (32 segments)
  constexpr int RING = RR * 32;     // nonzero positions in the ring
  const unsigned FULL = 0xffffffffu;
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x / 32;
  const int slot = lane / G, gl = lane & (G - 1);
  unsigned char *ring = smem + wib * (RR * ROUND);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kTmaWarps * RR * ROUND) + wib * RR;
  const long long w = (long long)blockIdx.x * kTmaWarps + wib;
  if (w >= a.units) return;  // whole warp leaves; barriers are per warp
  const int M = a.M;
  const int slab0 = blockIdx.y * (G * V);  // first column of the slab
  const int col0 = slab0 + gl * V;
  const bool active = col0 < a.N;
  const int slab_w = a.N - slab0 < G * V ? a.N - slab0 : G * V;
  const uint32_t seg_bytes = (uint32_t)slab_w * (uint32_t)sizeof(BT);  // multiple of 16 (host)
  const uint64_t pol = l2_policy(a.l2_hints);
  const BT *Bs = a.B + slab0;
  const unsigned ldb = (unsigned)a.ldb;

  int x0, x1, y0, y1;
  bool head_split = false, tail_open = false;
  if (ROWS) {
    const long long r0 = w * a.rows_per_unit;
    x0 = (int)r0;
    x1 = (int)min(r0 + a.rows_per_unit, (long long)M);
    y0 = __ldg(a.row_ptr + x0);
    y1 = __ldg(a.row_ptr + x1);
  } else {
    x0 = __ldg(a.part_x + w);
    y0 = __ldg(a.part_y + w);
    x1 = __ldg(a.part_x + w + 1);
    y1 = __ldg(a.part_y + w + 1);
    head_split = x0 < M && __ldg(a.row_ptr + x0) < y0;
    tail_open = x1 < M && __ldg(a.row_ptr + x1) < y1;
  }
  const int last = tail_open ? x1 : x1 - 1;
  const int rounds = (y1 - y0 + 31) / 32;

  if (lane == 0) {
#pragma unroll
    for (int b = 0; b < RR; ++b) mbar_init(smem_u32(&bars[b]), BULK ? 1 : 32);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();

  // ---- producer ----------------------------------------------------------
  int issued = 0;  // rounds issued
  // Column indices of the next round to issue, loaded one round ahead.
  int pj = 0, pj_round = -1;
  auto load_cols = [&](int rnd) {
    const int q0 = y0 + rnd * 32;
    pj = lane < y1 - q0 ? ld_stream(a.col + q0 + lane) : 0;
    pj_round = rnd;
  };
  auto issue = [&](int rnd) {
    const int q0 = y0 + rnd * 32;
    const int n = y1 - q0 < 32 ? y1 - q0 : 32;
    const int rs = rnd % RR;
    const uint32_t bar = smem_u32(&bars[rs]);
    if (pj_round != rnd) load_cols(rnd);
    const int j = pj;
    __syncwarp();
    fence_proxy_async_smem();  // earlier reads of this ring slot before the async writes
    if (BULK) {
      if (lane == 0) mbar_expect_tx(bar, (uint32_t)n * seg_bytes);
      __syncwarp();
      if (lane < n)
        bulk_g2s(smem_u32(ring + rs * ROUND + lane * SEG), Bs + (size_t)(unsigned)j * ldb,
                 seg_bytes, bar, pol);
    } else {
      // Lane l copies 16-byte piece c = l % G of positions l/G, l/G + P, ...
      const int c = lane & (G - 1);
      const bool piece_ok = (uint32_t)c * 16u < seg_bytes;  // last slab may be narrower
      const uint32_t dst0 = smem_u32(ring + rs * ROUND + c * 16);
#pragma unroll
      for (int k = 0; k < G; ++k) {
        const int i = lane / G + k * P;
        const int ji = __shfl_sync(FULL, j, i);
        if (i < n && piece_ok)
          cp_async16(dst0 + i * SEG, Bs + (size_t)(unsigned)ji * ldb + c * (16 / sizeof(BT)), pol);
      }
      cp_async_arrive(bar);
    }
    if (rnd + 1 < rounds) load_cols(rnd + 1);
  };
  int waited = 0;  // rounds known complete
  bool failed = false;
  // Wait until every round holding positions < `upto` is complete.
  auto need = [&](int upto) {
    const int last_round = (upto - y0 + 31) / 32;  // rounds [0, last_round) must be done
    while (!failed && waited < last_round) {
      const uint32_t bar = smem_u32(&bars[waited % RR]);
      if (!mbar_wait(bar, (uint32_t)((waited / RR) & 1))) failed = true;
      else ++waited;
    }
  };
  // Refill: rounds wholly below position `pos` are consumed.
  auto refill = [&](int pos) {
    const int done = (pos - y0) / 32;
    while (issued < rounds && issued < done + RR) issue(issued++);
  };
  refill(y0);

  int cur = x0, wb = x0;
  int rw = (wb + lane < M) ? __ldg(a.row_ptr + wb + 1 + lane) : INT_MAX;
  int cstart = y0;
  float mv = lane < y1 - cstart ? ld_val(a.val, cstart + lane) : 0.0f;
  float acc[V];

  // Position q sits at ring offset (q - y0) mod RING; since a round is 32
  // consecutive segments, its bytes start at offset * SEG.
  const unsigned char *lane_ring = ring + gl * 16;

  while (cur <= last && !failed) {
    if (cur - wb > 32 - P) {
      wb = cur;
      rw = (wb + lane < M) ? __ldg(a.row_ptr + wb + 1 + lane) : INT_MAX;
    }
    const int rend = min(__shfl_sync(FULL, rw, cur - wb), y1);
    if (P == 1 || rend - cstart >= LONG) {
      zero<V>(acc);
      for (int p = cstart; p < rend && !failed; p += 32) {
        const int nb = rend - p < 32 ? rend - p : 32;
        const int nxt = p + 32 < rend ? p + 32 : rend;
        const float mvn = lane < y1 - nxt ? ld_val(a.val, nxt + lane) : 0.0f;
        need(p + nb);
        if (failed) break;
        const int base = (p - y0) & (RING - 1);
#pragma unroll 4
        for (int s = 0; s * P < nb; ++s) {
          const int t = s * P + slot;
          const bool ok = t < nb;
          const float v = __shfl_sync(FULL, mv, ok ? t : 0);
          if (ok) {
            const uint4 r = lds128(lane_ring + ((base + t) & (RING - 1)) * SEG);
#pragma unroll
            for (int e = 0; e < V; ++e) acc[e] = fmaf(v, VT::get(r, e), acc[e]);
          }
        }
        mv = mvn;
        refill(nxt);
      }
      fold_slots<G, V>(acc);
      if (slot == 0 && active && !failed) {
        float *dst = a.C + (long long)cur * a.ldc + col0;
        if (!ROWS && ((cur == x0 && head_split) || (cur == x1 && tail_open)))
          atomic_add_c<V>(dst, acc);
        else
          store_c<V>(dst, acc);
      }
      cstart = rend;
      ++cur;
    } else {
      const int r = cur + slot;
      const int rw_r = __shfl_sync(FULL, rw, r - wb);
      const int rw_prev = __shfl_sync(FULL, rw, r - wb - 1 >= 0 ? r - wb - 1 : 0);
      const int e = r <= last ? min(rw_r, y1) : INT_MAX;
      const int prev_end = min(rw_prev, y1);
      const int sbeg = slot == 0 ? cstart : prev_end;
      const int len = e - sbeg;
      const bool ok = r <= last && len < LONG && e - cstart <= 32;
      unsigned leaders = 0;
#pragma unroll
      for (int q = 0; q < P; ++q) leaders |= 1u << (q * G);
      const unsigned bad = ~__ballot_sync(FULL, ok) & leaders;
      int k = bad ? (__ffs(bad) - 1) / G : P;
      if (k < 1) k = 1;
      const bool incl = slot < k;
      const int nxt = __shfl_sync(FULL, e, (k - 1) * G);
      const float mvn = lane < y1 - nxt ? ld_val(a.val, nxt + lane) : 0.0f;
      const int mylen = incl ? len : 0;
      const int maxlen = (int)__reduce_max_sync(FULL, (unsigned)mylen);
      const int off = sbeg - cstart;
      need(nxt);
      zero<V>(acc);
      if (!failed) {
        const int base = (sbeg - y0) & (RING - 1);
        for (int kk = 0; kk < maxlen; ++kk) {
          const bool okk = kk < mylen;
          const float v = __shfl_sync(FULL, mv, okk ? off + kk : 0);
          if (okk) {
            const uint4 rr = lds128(lane_ring + ((base + kk) & (RING - 1)) * SEG);
#pragma unroll
            for (int q = 0; q < V; ++q) acc[q] = fmaf(v, VT::get(rr, q), acc[q]);
          }
        }
        if (incl && active) {
          float *dst = a.C + (long long)r * a.ldc + col0;
          if (!ROWS && ((r == x0 && head_split) || (r == x1 && tail_open))) {
            if (mylen > 0) atomic_add_c<V>(dst, acc);
          } else {
            store_c<V>(dst, acc);
          }
        }
      }
      cur += k;
      cstart = nxt;
      mv = mvn;
      refill(nxt);
    }
  }
  if (failed) {
    if (lane == 0) atomicCAS(ex.status, 0, SEGTACO_ETIMEOUT);
    // Wait (bounded) for this warp's copies still in flight before leaving.
    for (int rnd = waited; rnd < issued; ++rnd)
      if (!mbar_wait(smem_u32(&bars[rnd % RR]), (uint32_t)((rnd / RR) & 1))) break;
  }
}

}  // namespace segtaco
