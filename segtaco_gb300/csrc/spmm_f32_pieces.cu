// spmm_f32_pieces.cu -- rb_pr's long-row pieces in passes over ranges of B's
// rows (spmm_pieces_kernel), dense operand f32.
#include "spmm_launch.cuh"

SEGTACO_DEFINE_PIECES_LAUNCHER(launch_spmm_pieces_f32, float, )
