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

#include <vector>

#include "internal.h"
#include "spmm_kernels.cuh"

namespace segtaco {

template <typename BT> struct BatchProblem {
  SpmmArgs<BT> a;        // the problem, exactly as a single launch sees it
  long long item_begin;  // first queue item of this problem within its group
  int slabs;
  int index;             // position in the batch (the gate releases problems in this order)
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Gate: problems with index < *gate may run.  A warp that draws an item of a
// problem not yet released polls the gate (lane 0, with backoff) until it is,
// until `timeout_ns` of %globaltimer time have passed, or until another warp
// has recorded a failure in *status.  On timeout it records SEGTACO_ETIMEOUT in
// *status and the warp leaves; every other waiting warp then leaves at its next
// poll, so the launch always ends within about one timeout.
struct BatchGate {
  const volatile long long *gate;  // device or mapped host memory; nullptr: no gate
  long long timeout_ns;
  int *status;
};

constexpr long long kGatePollLimit = 1LL << 26;

__device__ __forceinline__ bool batch_gate_wait(const BatchGate &g, int index, int lane) {
  int ok = 1;
  if (lane == 0 && *g.gate <= (long long)index) {
    const unsigned long long t0 = globaltimer_ns();
    for (long long polls = 0;; ++polls) {
      if (*g.gate > (long long)index) break;
      // The poll count is a backstop in case the timer does not advance.
      if (*reinterpret_cast<volatile int *>(g.status) != 0 || polls >= kGatePollLimit ||
          globaltimer_ns() - t0 > (unsigned long long)g.timeout_ns) {
        atomicCAS(g.status, 0, SEGTACO_ETIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(1000);
    }
  }
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

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
__global__ void __launch_bounds__(kSpmmCta, spmm_min_ctas<V, G, false>())
    spmm_batch_kernel(const BatchProblem<BT> *__restrict__ probs,
                      const long long *__restrict__ item_begin, int nprobs,
                      long long total_items, unsigned long long *__restrict__ queue,
                      BatchGate gate) {
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
    if (gate.gate != nullptr && !batch_gate_wait(gate, bp.index, lane)) break;
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
  long long row_begin;   // first global partition thread of this problem (M + 1 each)
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
  BatchGate gate;
};
// Host-side layout of a batch's descriptor buffer (one device allocation):
// partitions, per-group problem descriptors and item offsets, queue counters.
struct BatchLayout {
  struct Group {
    int dtype, V, G;
    bool rows;
    std::vector<int> members;  // problem indices
    long long total_items = 0;
    size_t off_probs = 0, off_begin = 0;
    int grid = 0;
  };
  std::vector<Group> groups;
  std::vector<size_t> off_px, off_py;
  std::vector<char> has_part;
  size_t off_parts = 0, off_queues = 0, bytes = 0;
  int nparts = 0;
  long long total_edges = 0;
  long long total_rows = 0;  // partition threads: M + 1 per element-balanced problem
};
// Groups the problems by kernel variant and lays out the buffer (pure host).
void batch_layout(const segtaco_spmm_problem *probs, const SpmmPlan *plans, int count,
                  BatchLayout *L);
// Writes the descriptor image for a buffer at device address `dbase` into
// `img` (L->bytes, zero-filled by the caller) and sizes each group's grid.
int batch_image(const segtaco_spmm_problem *probs, const SpmmPlan *plans, int count,
                BatchLayout *L, char *dbase, char *img, int device);
// Side streams over which the groups of one run are spread (optional): the
// groups are independent persistent launches, so a later group's CTAs take the
// SMs that an earlier group's tail leaves idle.  `join` holds one event per
// group.
struct BatchFork {
  int n = 0;
  cudaStream_t side[4] = {};
  cudaEvent_t start = nullptr;
  std::vector<cudaEvent_t> join;
};
// Enqueues one run: queue reset, merge-path partitions, one launch per group.
// `gate` (optional) holds back problems until the host releases them (its
// runs stay on `s`).
int batch_enqueue(const BatchLayout &L, char *dbase, cudaStream_t s,
                  const BatchGate *gate = nullptr, const BatchFork *fork = nullptr);

// Shape/pointer checks of one problem (pure host).
int check_batch_problem(const segtaco_spmm_problem &p, int index);
// Checks and plans one problem: the caller's config, or the heuristic on
// `max_row_len`; the ring and partition-ready flags are cleared and the depth
// reset (batch kernels keep four loads in flight).  `used` gets the config.
int plan_batch_problem(const segtaco_spmm_problem &p, const segtaco_config *cfg,
                       long long max_row_len, int index, segtaco_config *used, SpmmPlan *plan);

int launch_batch_f32(const BatchGroupLaunch &g, cudaStream_t s);
int launch_batch_bf16(const BatchGroupLaunch &g, cudaStream_t s);
int batch_blocks_per_sm_f32(int V, int G, bool rows, int *out);
int batch_blocks_per_sm_bf16(int V, int G, bool rows, int *out);

}  // namespace segtaco
