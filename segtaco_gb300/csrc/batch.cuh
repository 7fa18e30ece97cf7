// batch.cuh -- many SpMMs of uneven shapes in one persistent launch per variant.
//
// Every problem of a batch is planned like a single segtaco_spmm (schedule,
// vector width V, lanes per slot G, units of work).  Problems that share a
// kernel variant (dense type, V, G, unit kind) form a group.  For each group
// one persistent kernel is launched, sized to fill the GPU; its warps take
// work items from a global atomic queue.  An item is (problem, slab, unit):
// items of a problem are numbered slab-major, so one problem's slab sweeps
// stay together, and problems follow each other in order.
//
// The merge-path partitions of all element-balanced problems are computed by
// one launch (a thread per chunk edge across every problem), which also zeroes
// the rows that straddle chunk edges.
#pragma once

#include "spmm_kernels.cuh"

namespace segtaco {

template <typename BT> struct BatchProblem {
  SpmmArgs<BT> a;        // the problem, exactly as a single launch sees it
  long long item_begin;  // first queue item of this problem within its group
  int slabs;
};

// Queue item -> problem: last p with begin[p] <= item (begin[0] == 0).
__device__ __forceinline__ int find_problem(const long long *__restrict__ begin, int n,
                                            long long item) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (begin[mid] <= item)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Problems' item_begin values are staged in shared memory when they fit.
constexpr int kBatchSmemProblems = 1024;

template <typename BT, int V, int G, bool ROWS>
__global__ void __launch_bounds__(kCta, V == 8 ? 3 : 4)
    spmm_batch_kernel(const BatchProblem<BT> *__restrict__ probs,
                      const long long *__restrict__ item_begin, int nprobs,
                      long long total_items, unsigned long long *__restrict__ queue) {
  __shared__ long long s_begin[kBatchSmemProblems];
  const bool staged = nprobs <= kBatchSmemProblems;
  if (staged)
    for (int i = threadIdx.x; i < nprobs; i += blockDim.x) s_begin[i] = item_begin[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long item = 0;
    if (lane == 0) item = atomicAdd(queue, 1ULL);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= (unsigned long long)total_items) break;  // whole warp leaves together
    const int p = find_problem(staged ? s_begin : item_begin, nprobs, (long long)item);
    const BatchProblem<BT> &bp = probs[p];
    const long long local = (long long)item - bp.item_begin;
    const long long units = bp.a.units;
    const int slab = (int)(local / units);
    const long long w = local - (long long)slab * units;
    spmm_walk_unit<BT, V, G, ROWS, false>(bp.a, w, slab, lane);
  }
}

// One thread per chunk edge over every element-balanced problem of the batch.
struct BatchPartition {
  const int *row_ptr;
  int M;
  long long nnz;
  long long D;        // merge-path items per chunk
  long long nchunks;
  int *px, *py;       // nchunks + 1 entries each
  float *C;           // rows straddling an edge are zeroed (N columns, ldc)
  long long ldc;
  int N;
  long long edge_begin;  // first global edge index of this problem
};

// One persistent launch of a group (host side).
struct BatchGroupLaunch {
  int V, G;
  bool rows;
  const void *probs;  // BatchProblem<BT>[nprobs] in device memory
  const long long *item_begin;
  int nprobs;
  long long total_items;
  unsigned long long *queue;
  int grid;
};
int launch_batch_f32(const BatchGroupLaunch &g, cudaStream_t s);
int launch_batch_bf16(const BatchGroupLaunch &g, cudaStream_t s);
int batch_blocks_per_sm_f32(int V, int G, bool rows, int *out);
int batch_blocks_per_sm_bf16(int V, int G, bool rows, int *out);

}  // namespace segtaco
