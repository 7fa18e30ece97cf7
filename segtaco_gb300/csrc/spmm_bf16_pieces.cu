// spmm_bf16_pieces.cu -- rb_pr's long-row pieces in passes over ranges of B's
// rows (spmm_pieces_kernel), dense operand bf16.
#include "spmm_launch.cuh"

SEGTACO_DEFINE_PIECES_LAUNCHER(launch_spmm_pieces_bf16, uint16_t,
                               SEGTACO_PIECES_CASE(uint16_t, 16, 1)
                                   SEGTACO_PIECES_CASE(uint16_t, 16, 2)
                                       SEGTACO_PIECES_CASE(uint16_t, 16, 4))
