// spmm_launch.cuh -- shared body of the SpMM launchers.  Each spmm_<dtype>_<unit>.cu
// instantiates spmm_seg_kernel for one dense type and one unit kind (row blocks
// or merge-path chunks) over every (vector width V, lanes per slot G) pair, so
// the variants compile in parallel translation units.
#pragma once

#include "internal.h"
#include "spmm_kernels.cuh"

namespace segtaco {

template <typename BT> inline SpmmArgs<BT> make_spmm_args(const SpmmLaunch &L) {
  SpmmArgs<BT> a;
  a.M = L.M;
  a.K = L.K;
  a.N = L.N;
  a.nnz = L.nnz;
  a.row_ptr = L.row_ptr;
  a.col = L.col;
  a.val = L.val;
  a.B = static_cast<const BT *>(L.B);
  a.ldb = L.ldb;
  a.C = L.C;
  a.ldc = L.ldc;
  a.part_x = L.part_x;
  a.part_y = L.part_y;
  a.units = L.units;
  a.rows_per_unit = L.rows_per_unit;
  a.l2_hints = L.l2_hints ? 1 : 0;
  a.long_row = L.long_row;
  a.pieces = reinterpret_cast<const int2 *>(L.pieces);
  a.piece_count = L.piece_count;
  a.piece_ctr = L.piece_ctr;
  a.piece_part = L.piece_part;
  a.piece_cap = L.piece_len > 0 ? L.piece_cap : 0;
  a.piece_multi = L.piece_multi;
  a.piece_ld = L.piece_ld;
  a.piece_len = L.piece_len;
  a.piece_parts = L.piece_parts > 1 ? L.piece_parts : 1;
  a.piece_queue = L.piece_queue;
  return a;
}

// A launch of one SpMM kernel variant; carveout >= 0 asks for that percentage
// of the SM's unified L1 / shared memory as shared memory for this launch
// (the row-block kernel beside the long-row CTAs, spmm_long.cu).
template <typename BT>
inline void launch_seg(void (*kern)(SpmmArgs<BT>), dim3 grid, cudaStream_t s,
                       const SpmmArgs<BT> &a, int carveout) {
  if (carveout < 0) {
    kern<<<grid, kSpmmCta, 0, s>>>(a);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(kSpmmCta);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePreferredSharedMemoryCarveout;
  attr[0].val.sharedMemCarveout = (unsigned)carveout;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, a);  // errors surface in the caller's check_launch
}

// One warp per unit (x), one column slab per blockIdx.y; the slot walk packs
// 32 / G units (one per slot) into a warp.
inline dim3 spmm_grid(const SpmmLaunch &L) {
  const long long W = (long long)L.V * L.G;
  const unsigned slabs = (unsigned)((L.N + W - 1) / W);
  const long long per_warp = L.walk == kWalkSlots ? 32 / L.G : 1;
  const long long units = L.units + (L.piece_len > 0 ? L.piece_cap : 0);
  const long long warps = (units + per_warp - 1) / per_warp;
  long long x = (warps + kSpmmWarps - 1) / kSpmmWarps;
  if (x < 1) x = 1;
  return dim3((unsigned)x, slabs, 1);
}

}  // namespace segtaco

#define SEGTACO_VG_COMMON(X, R) \
  X(1, 1, R) X(1, 2, R) X(1, 4, R) X(1, 8, R) X(1, 16, R) X(1, 32, R) \
  X(2, 1, R) X(2, 2, R) X(2, 4, R) X(2, 8, R) X(2, 16, R) X(2, 32, R) \
  X(4, 1, R) X(4, 2, R) X(4, 4, R) X(4, 8, R) X(4, 16, R) X(4, 32, R) \
  X(8, 1, R) X(8, 2, R) X(8, 4, R) X(8, 8, R) X(8, 16, R) X(8, 32, R)
#define SEGTACO_VG_F32(X, R) SEGTACO_VG_COMMON(X, R)
#define SEGTACO_VG_BF16(X, R) SEGTACO_VG_COMMON(X, R) X(16, 1, R) X(16, 2, R) X(16, 4, R)

// Sixteen-byte-vector variants of the other walks: the row walk with 8 loads
// in flight per lane (kWalkRowsDeep) and the flat walk (kWalkFlat).
#define SEGTACO_WALK_CASE(BT, G, R, WALK)                                              \
  case G:                                                                              \
    launch_seg(spmm_seg_kernel<BT, 16 / sizeof(BT), G, R, WALK>, grid, s, a, L.carveout); \
    break;
#define SEGTACO_WALK_CASES(BT, R, WALK)                                                 \
  SEGTACO_WALK_CASE(BT, 1, R, WALK) SEGTACO_WALK_CASE(BT, 2, R, WALK)                   \
  SEGTACO_WALK_CASE(BT, 4, R, WALK) SEGTACO_WALK_CASE(BT, 8, R, WALK)                   \
  SEGTACO_WALK_CASE(BT, 16, R, WALK) SEGTACO_WALK_CASE(BT, 32, R, WALK)

// Slot-walk variants (merge-path chunks only).
#define SEGTACO_SLOT_CASE(BT, V, G)                                                      \
  case V * 100 + G:                                                                      \
    launch_seg(spmm_seg_kernel<BT, V, G, false, kWalkSlots>, grid, s, a, L.carveout);    \
    break;
#define SEGTACO_SLOT_CASES_F32(BT)                                                       \
  SEGTACO_SLOT_CASE(BT, 8, 4) SEGTACO_SLOT_CASE(BT, 4, 8) SEGTACO_SLOT_CASE(BT, 8, 8)    \
  SEGTACO_SLOT_CASE(BT, 4, 4) SEGTACO_SLOT_CASE(BT, 4, 16) SEGTACO_SLOT_CASE(BT, 1, 1)
#define SEGTACO_SLOT_CASES_BF16(BT)                                                      \
  SEGTACO_SLOT_CASE(BT, 16, 4) SEGTACO_SLOT_CASE(BT, 8, 4) SEGTACO_SLOT_CASE(BT, 8, 8)
#define SEGTACO_SLOT_CASES(BT)                                                           \
  if constexpr (sizeof(BT) == 4) {                                                       \
    switch (L.V * 100 + L.G) {                                                           \
      SEGTACO_SLOT_CASES_F32(BT)                                                         \
      default:                                                                           \
        return set_error(SEGTACO_EUNSUPPORTED, "slot walk: no variant V=%d G=%d", L.V, L.G); \
    }                                                                                    \
  } else {                                                                               \
    switch (L.V * 100 + L.G) {                                                           \
      SEGTACO_SLOT_CASES_BF16(BT)                                                        \
      default:                                                                           \
        return set_error(SEGTACO_EUNSUPPORTED, "slot walk: no variant V=%d G=%d", L.V, L.G); \
    }                                                                                    \
  }

// Sequential-walk variants (merge-path chunks, one 32-lane slot): 8-byte lanes.
#define SEGTACO_SEQ_CASE(BT, V)                                                          \
  case V:                                                                                \
    launch_seg(spmm_seg_kernel<BT, V, 32, false, kWalkSeq>, grid, s, a, L.carveout);     \
    break;
#define SEGTACO_SEQ_CASES(BT)                                                            \
  if constexpr (sizeof(BT) == 4) {                                                       \
    switch (L.V) {                                                                       \
      SEGTACO_SEQ_CASE(BT, 2)                                                            \
      default:                                                                           \
        return set_error(SEGTACO_EUNSUPPORTED, "sequential walk: no variant V=%d", L.V); \
    }                                                                                    \
  } else {                                                                               \
    switch (L.V) {                                                                       \
      SEGTACO_SEQ_CASE(BT, 4)                                                            \
      default:                                                                           \
        return set_error(SEGTACO_EUNSUPPORTED, "sequential walk: no variant V=%d", L.V); \
    }                                                                                    \
  }

// Defines int NAME(const SpmmLaunch&, cudaStream_t) for one (dtype, unit kind).
#define SEGTACO_DEFINE_SPMM_LAUNCHER(NAME, BT, VG_LIST, ROWS)                             \
  namespace segtaco {                                                                     \
  int NAME(const SpmmLaunch &L, cudaStream_t s) {                                         \
    const SpmmArgs<BT> a = make_spmm_args<BT>(L);                                         \
    const dim3 grid = spmm_grid(L);                                                       \
    if constexpr (!ROWS) {                                                                \
      if (L.walk == kWalkSlots) {                                                         \
        SEGTACO_SLOT_CASES(BT)                                                            \
        return check_launch(#NAME);                                                       \
      }                                                                                   \
      if (L.walk == kWalkSeq) {                                                           \
        SEGTACO_SEQ_CASES(BT)                                                             \
        return check_launch(#NAME);                                                       \
      }                                                                                   \
    }                                                                                     \
    if (L.walk != kWalkRows && L.V * (int)sizeof(BT) == 16) {                            \
      if (L.walk == kWalkRowsDeep) {                                                      \
        switch (L.G) {                                                                    \
          SEGTACO_WALK_CASES(BT, ROWS, kWalkRowsDeep)                                     \
          default:                                                                        \
            return set_error(SEGTACO_EUNSUPPORTED, #NAME ": no deep walk G=%d", L.G);      \
        }                                                                                 \
      } else {                                                                            \
        switch (L.G) {                                                                    \
          SEGTACO_WALK_CASES(BT, ROWS, kWalkFlat)                                         \
          default:                                                                        \
            return set_error(SEGTACO_EUNSUPPORTED, #NAME ": no flat walk G=%d", L.G);      \
        }                                                                                 \
      }                                                                                   \
      return check_launch(#NAME);                                                         \
    }                                                                                     \
    switch (L.V * 100 + L.G) {                                                            \
      VG_LIST(SEGTACO_SPMM_CASE, ROWS)                                                    \
      default:                                                                            \
        return set_error(SEGTACO_EUNSUPPORTED, #NAME ": no variant V=%d G=%d", L.V, L.G);  \
    }                                                                                     \
    return check_launch(#NAME);                                                           \
  }                                                                                       \
  }

// The pieces' launcher of one dense type (spmm_<dtype>_pieces.cu): the row
// walk's (V, G) pairs with at least two slots.
#define SEGTACO_PIECES_CASE(BT, V, G)                                                    \
  case V * 100 + G:                                                                      \
    spmm_pieces_kernel<BT, V, G>                                                         \
        <<<spmm_min_ctas<V, G, false>() * device_sms(), kSpmmCta, 0, s>>>(a);            \
    break;
#define SEGTACO_PIECES_VG(X, BT)                                                         \
  X(BT, 1, 1) X(BT, 1, 2) X(BT, 1, 4) X(BT, 1, 8) X(BT, 1, 16)                           \
  X(BT, 2, 1) X(BT, 2, 2) X(BT, 2, 4) X(BT, 2, 8) X(BT, 2, 16)                           \
  X(BT, 4, 1) X(BT, 4, 2) X(BT, 4, 4) X(BT, 4, 8) X(BT, 4, 16)                           \
  X(BT, 8, 1) X(BT, 8, 2) X(BT, 8, 4) X(BT, 8, 8) X(BT, 8, 16)
#define SEGTACO_DEFINE_PIECES_LAUNCHER(NAME, BT, EXTRA)                                  \
  namespace segtaco {                                                                    \
  int NAME(const SpmmLaunch &L, cudaStream_t s) {                                        \
    const SpmmArgs<BT> a = make_spmm_args<BT>(L);                                        \
    SEGTACO_TRY(check_cuda(cudaMemsetAsync(L.piece_queue, 0, sizeof(unsigned long long), s), \
                           "cudaMemsetAsync"));                                          \
    switch (L.V * 100 + L.G) {                                                           \
      SEGTACO_PIECES_VG(SEGTACO_PIECES_CASE, BT)                                         \
      EXTRA                                                                              \
      default:                                                                           \
        return set_error(SEGTACO_EUNSUPPORTED, #NAME ": no variant V=%d G=%d", L.V, L.G); \
    }                                                                                    \
    return check_launch(#NAME);                                                          \
  }                                                                                      \
  }
