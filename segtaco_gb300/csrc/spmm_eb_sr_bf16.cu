// spmm_eb_sr_bf16.cu -- eb_sr SpMM launcher, dense operand bf16.
#include "spmm_launch.cuh"

#define SEGTACO_SPMM_CASE_spmm_eb_sr_kernel(V, G)                   \
  case V * 100 + G:                                                  \
    spmm_eb_sr_kernel<uint16_t, V, G><<<grid, kCta, 0, s>>>(a); \
    break;

SEGTACO_DEFINE_SPMM_LAUNCHER(launch_spmm_eb_sr_bf16, spmm_eb_sr_kernel, uint16_t, SEGTACO_VG_BF16)
