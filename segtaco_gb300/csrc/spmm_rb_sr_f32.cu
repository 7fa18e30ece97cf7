// spmm_rb_sr_f32.cu -- rb_sr SpMM launcher, dense operand f32.
#include "spmm_launch.cuh"

#define SEGTACO_SPMM_CASE_spmm_rb_sr_kernel(V, G)                   \
  case V * 100 + G:                                                  \
    spmm_rb_sr_kernel<float, V, G><<<grid, kCta, 0, s>>>(a); \
    break;

SEGTACO_DEFINE_SPMM_LAUNCHER(launch_spmm_rb_sr_f32, spmm_rb_sr_kernel, float, SEGTACO_VG_F32)
