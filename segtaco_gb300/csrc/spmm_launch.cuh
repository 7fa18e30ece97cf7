// spmm_launch.cuh -- shared body of the per-(schedule, dtype) SpMM launchers.
// Each spmm_<schedule>_<dtype>.cu instantiates one schedule for one dense type
// over every (vector width V, lanes per group G) pair, so the kernel variants
// compile in parallel translation units.
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
  a.l2_hints = L.l2_hints ? 1 : 0;
  return a;
}

// Grid of one SpMM launch: x over rows / chunks, y over column slabs.
inline dim3 spmm_grid(const SpmmLaunch &L) {
  const long long W = (long long)L.V * L.G;
  const unsigned slabs = (unsigned)((L.N + W - 1) / W);
  long long x = 1;
  switch (L.schedule) {
    case SEGTACO_RB_SR: {
      const long long groups = (L.M + L.units - 1) / L.units;
      x = (groups + (kCta / L.G) - 1) / (kCta / L.G);
      break;
    }
    case SEGTACO_RB_PR: {
      const long long warps = (L.M + L.units - 1) / L.units;
      x = (warps + (kCta / 32) - 1) / (kCta / 32);
      break;
    }
    case SEGTACO_EB_SR:
      x = (L.units + (kCta / L.G) - 1) / (kCta / L.G);
      break;
    default:
      x = (L.units + (kCta / 32) - 1) / (kCta / 32);
      break;
  }
  if (x < 1) x = 1;
  return dim3((unsigned)x, slabs, 1);
}

}  // namespace segtaco

#define SEGTACO_VG_F32(X) \
  X(1, 1) X(1, 2) X(1, 4) X(1, 8) X(1, 16) X(1, 32) \
  X(2, 1) X(2, 2) X(2, 4) X(2, 8) X(2, 16) X(2, 32) \
  X(4, 1) X(4, 2) X(4, 4) X(4, 8) X(4, 16) X(4, 32)
#define SEGTACO_VG_BF16(X) \
  X(1, 1) X(1, 2) X(1, 4) X(1, 8) X(1, 16) X(1, 32) \
  X(2, 1) X(2, 2) X(2, 4) X(2, 8) X(2, 16) X(2, 32) \
  X(4, 1) X(4, 2) X(4, 4) X(4, 8) X(4, 16) X(4, 32) \
  X(8, 1) X(8, 2) X(8, 4) X(8, 8) X(8, 16) X(8, 32)

// Defines int NAME(const SpmmLaunch&, cudaStream_t) for KERNEL over BT.
#define SEGTACO_DEFINE_SPMM_LAUNCHER(NAME, KERNEL, BT, VG_LIST)                          \
  namespace segtaco {                                                                    \
  int NAME(const SpmmLaunch &L, cudaStream_t s) {                                        \
    const SpmmArgs<BT> a = make_spmm_args<BT>(L);                                        \
    const dim3 grid = spmm_grid(L);                                                      \
    switch (L.V * 100 + L.G) {                                                           \
      VG_LIST(SEGTACO_SPMM_CASE_##KERNEL)                                                \
      default:                                                                           \
        return set_error(SEGTACO_EUNSUPPORTED, #NAME ": no variant V=%d G=%d", L.V, L.G); \
    }                                                                                    \
    return check_launch(#KERNEL);                                                        \
  }                                                                                      \
  }
