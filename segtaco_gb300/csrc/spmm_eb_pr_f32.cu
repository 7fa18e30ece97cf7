// spmm_eb_pr_f32.cu -- eb_pr SpMM launcher, dense operand f32.
#include "spmm_launch.cuh"

#define SEGTACO_SPMM_CASE_spmm_eb_pr_kernel(V, G)                   \
  case V * 100 + G:                                                  \
    spmm_eb_pr_kernel<float, V, G><<<grid, kCta, 0, s>>>(a); \
    break;

SEGTACO_DEFINE_SPMM_LAUNCHER(launch_spmm_eb_pr_f32, spmm_eb_pr_kernel, float, SEGTACO_VG_F32)
