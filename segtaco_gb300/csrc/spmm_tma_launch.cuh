// spmm_tma_launch.cuh -- shared body of the TMA SpMM launchers.
#pragma once

#include "internal.h"
#include "spmm_launch.cuh"
#include "spmm_tma.cuh"

namespace segtaco {

template <typename BT, int G, bool ROWS, bool BULK>
int launch_tma_variant(const SpmmLaunch &L, cudaStream_t s) {
  constexpr int RR = tma_ring_rounds<G>();
  constexpr int smem = tma_smem_bytes<BT, G, RR>();
  auto kern = spmm_tma_kernel<BT, G, ROWS, RR, BULK>;
  static bool configured = false;  // one attribute call per variant and process
  if (!configured) {
    SEGTACO_TRY(check_cuda(
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
        "cudaFuncSetAttribute(spmm_tma_kernel)"));
    configured = true;
  }
  TmaExtra ex;
  SEGTACO_TRY(tma_status_ptr(&ex.status));
  const long long W = (long long)G * (16 / (long long)sizeof(BT));
  const unsigned slabs = (unsigned)((L.N + W - 1) / W);
  long long x = (L.units + kTmaWarps - 1) / kTmaWarps;
  if (x < 1) x = 1;
  kern<<<dim3((unsigned)x, slabs, 1), kTmaWarps * 32, smem, s>>>(make_spmm_args<BT>(L), ex);
  return check_launch("spmm_tma_kernel");
}

template <typename BT> int launch_tma(const SpmmLaunch &L, bool rows, cudaStream_t s) {
  switch (L.G * 4 + (rows ? 2 : 0) + (L.bulk_copies ? 1 : 0)) {
#define SEGTACO_TMA_CASE(G)                                  \
  case G * 4 + 3:                                            \
    return launch_tma_variant<BT, G, true, true>(L, s);      \
  case G * 4 + 2:                                            \
    return launch_tma_variant<BT, G, true, false>(L, s);     \
  case G * 4 + 1:                                            \
    return launch_tma_variant<BT, G, false, true>(L, s);     \
  case G * 4:                                                \
    return launch_tma_variant<BT, G, false, false>(L, s);
    SEGTACO_TMA_CASE(1)
    SEGTACO_TMA_CASE(2)
    SEGTACO_TMA_CASE(4)
    SEGTACO_TMA_CASE(8)
    SEGTACO_TMA_CASE(16)
    SEGTACO_TMA_CASE(32)
#undef SEGTACO_TMA_CASE
    default:
      return set_error(SEGTACO_EUNSUPPORTED, "spmm_tma: no variant G=%d", L.G);
  }
}

}  // namespace segtaco
