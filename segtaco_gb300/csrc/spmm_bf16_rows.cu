// spmm_bf16_rows.cu -- SpMM launcher: dense operand bf16, units = rows.
#include "spmm_launch.cuh"

#define SEGTACO_SPMM_CASE(V, G, R)                                   \
  case V * 100 + G:                                                  \
    launch_seg(spmm_seg_kernel<uint16_t, V, G, R>, grid, s, a, L.carveout);   \
    break;

SEGTACO_DEFINE_SPMM_LAUNCHER(launch_spmm_bf16_rows, uint16_t, SEGTACO_VG_BF16, true)
