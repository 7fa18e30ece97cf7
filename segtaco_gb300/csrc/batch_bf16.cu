// batch_bf16.cu -- persistent batched SpMM launchers, dense operand bf16.
#include "batch.cuh"
#include "internal.h"
#include "spmm_launch.cuh"

namespace segtaco {

#define SEGTACO_BATCH_CASE(V, G, R)                                                        \
  case V * 100 + G:                                                                        \
    spmm_batch_kernel<uint16_t, V, G, R><<<g.grid, kSpmmCta, 0, s>>>(                            \
        static_cast<const BatchProblem<uint16_t> *>(g.probs), g.item_begin, g.nprobs,         \
        g.total_items, g.queue, g.gate);                                                           \
    break;
#define SEGTACO_BATCH_OCC(V, G, R)                                                         \
  case V * 100 + G:                                                                        \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, spmm_batch_kernel<uint16_t, V, G, R>, \
                                                      kSpmmCta, 0);                            \
    break;

int launch_batch_bf16(const BatchGroupLaunch &g, cudaStream_t s) {
  if (g.rows) {
    switch (g.V * 100 + g.G) {
      SEGTACO_VG_BF16(SEGTACO_BATCH_CASE, true)
      default:
        return set_error(SEGTACO_EUNSUPPORTED, "batch: no variant V=%d G=%d", g.V, g.G);
    }
  } else {
    switch (g.V * 100 + g.G) {
      SEGTACO_VG_BF16(SEGTACO_BATCH_CASE, false)
      default:
        return set_error(SEGTACO_EUNSUPPORTED, "batch: no variant V=%d G=%d", g.V, g.G);
    }
  }
  return check_launch("spmm_batch_kernel");
}

int batch_blocks_per_sm_bf16(int V, int G, bool rows, int *out) {
  cudaError_t e = cudaErrorInvalidValue;
  if (rows) {
    switch (V * 100 + G) { SEGTACO_VG_BF16(SEGTACO_BATCH_OCC, true) default: break; }
  } else {
    switch (V * 100 + G) { SEGTACO_VG_BF16(SEGTACO_BATCH_OCC, false) default: break; }
  }
  return check_cuda(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor(batch)");
}

}  // namespace segtaco
