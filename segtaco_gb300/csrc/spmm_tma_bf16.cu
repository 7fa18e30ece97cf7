// spmm_tma_bf16.cu -- TMA SpMM launcher for bf16 B.
#include "spmm_tma_launch.cuh"

namespace segtaco {
int launch_spmm_tma_bf16(const SpmmLaunch &L, bool rows, cudaStream_t s) {
  return launch_tma<uint16_t>(L, rows, s);
}
}  // namespace segtaco
