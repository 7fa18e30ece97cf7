// spmm_f32_chunks.cu -- SpMM launcher: dense operand f32, units = chunks.
#include "spmm_launch.cuh"

#define SEGTACO_SPMM_CASE(V, G, R)                                   \
  case V * 100 + G:                                                  \
    launch_seg(spmm_seg_kernel<float, V, G, R>, grid, s, a, L.carveout);   \
    break;

SEGTACO_DEFINE_SPMM_LAUNCHER(launch_spmm_f32_chunks, float, SEGTACO_VG_F32, false)
