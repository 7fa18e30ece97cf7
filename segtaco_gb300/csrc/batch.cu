// batch.cu -- segtaco_batch_*: plan, run (optionally through a CUDA graph) and
// free a batch of SpMMs of uneven shapes.  Kernels: batch.cuh.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "batch.cuh"
#include "internal.h"

namespace segtaco {

// ---------------------------------------------------------------------------
// Row-length statistics (the autotuner's input), one launch per problem.
// ---------------------------------------------------------------------------
// stats[0] = max row length, stats[1] = empty rows, stats[2] = rows >= 32,
// stats[3] = nonzeros in rows >= 32.
__global__ void row_stats_kernel(const int *__restrict__ row_ptr, int M,
                                 unsigned long long *__restrict__ stats) {
  unsigned long long mx = 0, empty = 0, longr = 0, longnz = 0;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < M;
       r += (long long)gridDim.x * blockDim.x) {
    const unsigned long long len = (unsigned long long)(__ldg(row_ptr + r + 1) - __ldg(row_ptr + r));
    mx = len > mx ? len : mx;
    empty += len == 0;
    if (len >= 32) {
      ++longr;
      longnz += len;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long m2 = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = m2 > mx ? m2 : mx;
    empty += __shfl_xor_sync(0xffffffffu, empty, o);
    longr += __shfl_xor_sync(0xffffffffu, longr, o);
    longnz += __shfl_xor_sync(0xffffffffu, longnz, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(stats + 0, mx);
    atomicAdd(stats + 1, empty);
    atomicAdd(stats + 2, longr);
    atomicAdd(stats + 3, longnz);
  }
}

int launch_row_stats(const int *row_ptr, int M, unsigned long long *stats, cudaStream_t s) {
  if (M <= 0) return SEGTACO_OK;
  long long blocks = (M + 255) / 256;
  if (blocks > 1024) blocks = 1024;
  row_stats_kernel<<<(unsigned)blocks, 256, 0, s>>>(row_ptr, M, stats);
  return check_launch("row_stats_kernel");
}

// ---------------------------------------------------------------------------
// Batched merge-path partition.
// ---------------------------------------------------------------------------
constexpr int kBatchPartRows = 4;  // rows per partition thread

__global__ void batch_partition_kernel(const BatchPartition *__restrict__ parts, int nparts,
                                       long long total_rows) {
  // Global rows t over every problem, M + 1 each (the last is the problem's
  // tail); row t writes the chunk edges inside it (merge_path_store_row).  A
  // thread walks kBatchPartRows consecutive rows, possibly across problems.
  // The block's first problem comes from one search; a thread whose rows lie
  // in one problem loads their row_ptr entries together, before any store.
  __shared__ int s_part;
  const long long tb = (long long)blockIdx.x * blockDim.x * kBatchPartRows;
  if (threadIdx.x == 0) {
    int lo = 0, hi = nparts - 1;  // last part with row_begin <= tb
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (parts[mid].row_begin <= tb)
        lo = mid;
      else
        hi = mid - 1;
    }
    s_part = lo;
  }
  __syncthreads();
  const long long t0 = tb + (long long)threadIdx.x * kBatchPartRows;
  if (t0 >= total_rows) return;
  int lo = s_part;
  while (lo + 1 < nparts && parts[lo + 1].row_begin <= t0) ++lo;
  {
    const BatchPartition bp = parts[lo];
    const long long r0 = t0 - bp.row_begin;
    if (r0 + kBatchPartRows - 1 <= bp.M) {
      // rows r0 .. r0+3 all in this problem: e[k] = e_{r0+k-1} = row_ptr[r0+k] + r0 + k
      const bool small = (long long)bp.M + bp.nnz + bp.D < 0x7fffffffLL;
      long long e[kBatchPartRows + 1];
#pragma unroll
      for (int k = 0; k <= kBatchPartRows; ++k) {
        const long long r = r0 + k;
        e[k] = (r > 0 && r <= bp.M) ? (long long)__ldg(bp.row_ptr + r) + r : 0;
      }
      long long c_lo = ceil_div_pos(e[0], bp.D, small);
#pragma unroll
      for (int k = 0; k < kBatchPartRows; ++k) {
        const long long r = r0 + k;
        if (r < bp.M) {
          const long long nxt = ceil_div_pos(e[k + 1], bp.D, small);
          merge_path_store_row(bp.row_ptr, bp.M, bp.nnz, bp.D, bp.nchunks, r, c_lo, nxt - 1,
                               bp.px, bp.py, bp.C, bp.ldc, bp.N);
          c_lo = nxt;
        } else {
          merge_path_store_row(bp.row_ptr, bp.M, bp.nnz, bp.D, bp.nchunks, r, c_lo, bp.nchunks,
                               bp.px, bp.py, bp.C, bp.ldc, bp.N);
        }
      }
      return;
    }
  }
  for (int k = 0; k < kBatchPartRows; ++k) {
    const long long t = t0 + k;
    if (t >= total_rows) break;
    while (lo + 1 < nparts && parts[lo + 1].row_begin <= t) ++lo;
    const BatchPartition &bp = parts[lo];
    const long long r = t - bp.row_begin;
    const bool small = (long long)bp.M + bp.nnz + bp.D < 0x7fffffffLL;
    const long long e_prev = r > 0 ? (long long)__ldg(bp.row_ptr + r) + r : 0;
    const long long c_lo = ceil_div_pos(e_prev, bp.D, small);
    if (r < bp.M) {
      const long long e_r = (long long)__ldg(bp.row_ptr + r + 1) + r + 1;
      merge_path_store_row(bp.row_ptr, bp.M, bp.nnz, bp.D, bp.nchunks, r, c_lo,
                           ceil_div_pos(e_r, bp.D, small) - 1, bp.px, bp.py, bp.C, bp.ldc, bp.N);
    } else {
      merge_path_store_row(bp.row_ptr, bp.M, bp.nnz, bp.D, bp.nchunks, r, c_lo, bp.nchunks, bp.px,
                           bp.py, bp.C, bp.ldc, bp.N);
    }
  }
}

// ---------------------------------------------------------------------------
// Descriptor layout, image and enqueue.
// ---------------------------------------------------------------------------
namespace {

template <typename BT>
void fill_problem(BatchProblem<BT> &bp, const segtaco_spmm_problem &p, const SpmmPlan &plan,
                  int *px, int *py, long long item_begin, int index) {
  memset(&bp, 0, sizeof(bp));
  SpmmArgs<BT> &a = bp.a;
  a.M = p.M;
  a.K = p.K;
  a.N = p.N;
  a.nnz = p.nnz;
  a.row_ptr = p.row_ptr;
  a.col = p.col;
  a.val = p.vals;
  a.B = static_cast<const BT *>(p.B);
  a.ldb = p.ldb;
  a.C = p.C;
  a.ldc = p.ldc;
  a.part_x = px;
  a.part_y = py;
  a.units = plan.nchunks;
  a.rows_per_unit = (int)plan.rows_per_unit;
  a.l2_hints = plan.l2_hints ? 1 : 0;
  bp.item_begin = item_begin;
  bp.slabs = plan.slabs;
  bp.index = index;
}

// Resident CTAs per SM of each batch kernel variant, per device (queried once).
int blocks_per_sm(int device, int dtype, int V, int G, bool rows, int *out) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, bool>, int> cache;
  const auto key = std::make_tuple(device, dtype, V, G, rows);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      *out = it->second;
      return SEGTACO_OK;
    }
  }
  int n = 0;
  SEGTACO_TRY(dtype == SEGTACO_BF16 ? batch_blocks_per_sm_bf16(V, G, rows, &n)
                                    : batch_blocks_per_sm_f32(V, G, rows, &n));
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = n;
  *out = n;
  return SEGTACO_OK;
}

int sm_count(int device) {
  static std::mutex mu;
  static std::map<int, int> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(device);
  if (it != cache.end()) return it->second;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) sms = 1;
  cache[device] = sms;
  return sms;
}

}  // namespace

void batch_layout(const segtaco_spmm_problem *probs, const SpmmPlan *plans, int count,
                  BatchLayout *L) {
  *L = BatchLayout();
  std::map<std::tuple<int, int, int, bool>, int> gidx;
  for (int i = 0; i < count; ++i) {
    const auto &p = probs[i];
    if (p.M == 0 || p.N == 0) continue;
    const auto &pl = plans[i];
    const bool rows = pl.schedule == SEGTACO_RB_SR || pl.schedule == SEGTACO_RB_PR;
    const auto key = std::make_tuple(p.b_dtype, pl.V, pl.G, rows);
    auto it = gidx.find(key);
    if (it == gidx.end()) {
      it = gidx.emplace(key, (int)L->groups.size()).first;
      BatchLayout::Group g;
      g.dtype = p.b_dtype;
      g.V = pl.V;
      g.G = pl.G;
      g.rows = rows;
      L->groups.push_back(g);
    }
    L->groups[it->second].members.push_back(i);
  }
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += align256(bytes);
    return o;
  };
  L->off_px.assign(count, 0);
  L->off_py.assign(count, 0);
  L->has_part.assign(count, 0);
  for (int i = 0; i < count; ++i) {
    const auto &pl = plans[i];
    const bool eb = pl.schedule == SEGTACO_EB_SR || pl.schedule == SEGTACO_EB_PR;
    if (eb && probs[i].M > 0 && probs[i].N > 0) {
      L->has_part[i] = 1;
      L->off_px[i] = take((pl.nchunks + 1) * sizeof(int));
      L->off_py[i] = take((pl.nchunks + 1) * sizeof(int));
      ++L->nparts;
    }
  }
  L->off_parts = take(std::max(1, L->nparts) * sizeof(BatchPartition));
  for (auto &g : L->groups) {
    g.off_probs = take(g.members.size() * sizeof(BatchProblem<float>));
    g.off_begin = take(g.members.size() * sizeof(long long));
  }
  L->off_queues = take(std::max<size_t>(1, L->groups.size()) * sizeof(unsigned long long));
  L->bytes = off;
}

int batch_image(const segtaco_spmm_problem *probs, const SpmmPlan *plans, int count,
                BatchLayout *L, char *dbase, char *img, int device) {
  std::vector<BatchPartition> parts;
  long long edges = 0, prow = 0;
  for (int i = 0; i < count; ++i) {
    if (!L->has_part[i]) continue;
    const auto &p = probs[i];
    const auto &pl = plans[i];
    BatchPartition bp;
    bp.row_ptr = p.row_ptr;
    bp.M = p.M;
    bp.nnz = p.nnz;
    bp.D = pl.items_per_unit;
    bp.nchunks = pl.nchunks;
    bp.px = reinterpret_cast<int *>(dbase + L->off_px[i]);
    bp.py = reinterpret_cast<int *>(dbase + L->off_py[i]);
    bp.C = p.C;
    bp.ldc = p.ldc;
    bp.N = p.N;
    bp.edge_begin = edges;
    edges += pl.nchunks + 1;
    bp.row_begin = prow;
    prow += (long long)p.M + 1;
    parts.push_back(bp);
  }
  L->total_edges = edges;
  L->total_rows = prow;
  if (!parts.empty())
    memcpy(img + L->off_parts, parts.data(), parts.size() * sizeof(BatchPartition));
  const int sms = sm_count(device);
  for (auto &g : L->groups) {
    long long item = 0;
    std::vector<long long> begin;
    begin.reserve(g.members.size());
    for (size_t k = 0; k < g.members.size(); ++k) {
      const int i = g.members[k];
      const auto &pl = plans[i];
      int *px = L->has_part[i] ? reinterpret_cast<int *>(dbase + L->off_px[i]) : nullptr;
      int *py = L->has_part[i] ? reinterpret_cast<int *>(dbase + L->off_py[i]) : nullptr;
      begin.push_back(item);
      if (g.dtype == SEGTACO_BF16) {
        BatchProblem<uint16_t> bp;
        fill_problem(bp, probs[i], pl, px, py, item, i);
        memcpy(img + g.off_probs + k * sizeof(bp), &bp, sizeof(bp));
      } else {
        BatchProblem<float> bp;
        fill_problem(bp, probs[i], pl, px, py, item, i);
        memcpy(img + g.off_probs + k * sizeof(bp), &bp, sizeof(bp));
      }
      item += pl.nchunks * (long long)pl.slabs;
    }
    g.total_items = item;
    memcpy(img + g.off_begin, begin.data(), begin.size() * sizeof(long long));
    // Persistent grid: every SM full, never more CTAs than the items need.
    int per_sm = 0;
    SEGTACO_TRY(blocks_per_sm(device, g.dtype, g.V, g.G, g.rows, &per_sm));
    const long long need = (item + kSpmmWarps - 1) / kSpmmWarps;
    long long grid = (long long)std::max(1, per_sm) * std::max(1, sms);
    if (grid > need) grid = std::max(1LL, need);
    g.grid = (int)grid;
  }
  return SEGTACO_OK;
}

int batch_enqueue(const BatchLayout &L, char *dbase, cudaStream_t s, const BatchGate *gate,
                  const BatchFork *fork) {
  if (!L.groups.empty())
    SEGTACO_TRY(check_cuda(cudaMemsetAsync(dbase + L.off_queues, 0,
                                           L.groups.size() * sizeof(unsigned long long), s),
                           "memset queues"));
  if (L.total_rows > 0) {
    const long long per_block = 256LL * kBatchPartRows;
    const long long blocks = (L.total_rows + per_block - 1) / per_block;
    batch_partition_kernel<<<(unsigned)blocks, 256, 0, s>>>(
        reinterpret_cast<const BatchPartition *>(dbase + L.off_parts), L.nparts, L.total_rows);
    SEGTACO_TRY(check_launch("batch_partition_kernel"));
  }
  const bool forked = fork && fork->n > 0 && !gate && L.groups.size() > 1 &&
                      fork->join.size() >= L.groups.size();
  if (forked) SEGTACO_TRY(check_cuda(cudaEventRecord(fork->start, s), "cudaEventRecord"));
  std::vector<char> joined(L.groups.size(), 0);
  int next_side = 0;
  for (size_t gi = 0; gi < L.groups.size(); ++gi) {
    const auto &g = L.groups[gi];
    if (g.total_items == 0) continue;
    cudaStream_t gs = s;
    if (forked && gi > 0) {
      gs = fork->side[next_side++ % fork->n];
      SEGTACO_TRY(check_cuda(cudaStreamWaitEvent(gs, fork->start, 0), "cudaStreamWaitEvent"));
    }
    BatchGroupLaunch G;
    G.V = g.V;
    G.G = g.G;
    G.rows = g.rows;
    G.probs = dbase + g.off_probs;
    G.item_begin = reinterpret_cast<const long long *>(dbase + g.off_begin);
    G.nprobs = (int)g.members.size();
    G.total_items = g.total_items;
    G.queue = reinterpret_cast<unsigned long long *>(dbase + L.off_queues) + gi;
    G.grid = g.grid;
    G.gate = gate ? *gate : BatchGate{nullptr, 0, nullptr};
    SEGTACO_TRY(g.dtype == SEGTACO_BF16 ? launch_batch_bf16(G, gs) : launch_batch_f32(G, gs));
    if (gs != s) {
      SEGTACO_TRY(check_cuda(cudaEventRecord(fork->join[gi], gs), "cudaEventRecord"));
      joined[gi] = 1;
    }
  }
  for (size_t gi = 0; gi < L.groups.size(); ++gi)
    if (joined[gi])
      SEGTACO_TRY(check_cuda(cudaStreamWaitEvent(s, fork->join[gi], 0), "cudaStreamWaitEvent"));
  return SEGTACO_OK;
}

// Validates a problem and resolves its plan: the caller's config, or the
// heuristic on `max_row_len`.  Ring and partition-ready flags are cleared and
// the depth reset (batch kernels keep four loads in flight).
int check_batch_problem(const segtaco_spmm_problem &p, int index) {
  if (p.M < 0 || p.K < 0 || p.N < 0 || p.nnz < 0 || p.nnz > 0x7fffffffLL ||
      (p.M > 0 && !p.row_ptr) || (p.nnz > 0 && (!p.col || !p.B)) ||
      (p.M > 0 && p.N > 0 && !p.C) || p.ldb < p.N || p.ldc < p.N ||
      (p.b_dtype != SEGTACO_F32 && p.b_dtype != SEGTACO_BF16))
    return set_error(SEGTACO_EINVAL, "batch: problem %d is malformed", index);
  return SEGTACO_OK;
}

int plan_batch_problem(const segtaco_spmm_problem &p, const segtaco_config *cfg,
                       long long max_row_len, int index, segtaco_config *used, SpmmPlan *plan) {
  SEGTACO_TRY(check_batch_problem(p, index));
  segtaco_config c;
  if (cfg) {
    c = *cfg;
  } else {
    c.schedule = SEGTACO_AUTO;
    segtaco_autotune_heuristic(p.M, p.K, p.nnz, p.N, p.b_dtype, max_row_len, &c);
    // The batch fills the GPU with many problems: no problem needs the small
    // chunks and row blocks that make one small product fill it alone.
    if (c.schedule == SEGTACO_RB_SR || c.schedule == SEGTACO_RB_PR) c.rows_per_unit = 4;
  }
  if ((c.schedule == SEGTACO_EB_SR || c.schedule == SEGTACO_EB_PR) &&
      (!cfg || c.items_per_unit <= 0))
    c.items_per_unit = 512;
  c.depth = 0;
  c.flags &= ~(SEGTACO_FLAG_SMEM_RING | SEGTACO_FLAG_TMA_BULK | SEGTACO_FLAG_PARTITION_READY);
  // The persistent kernel walks every row of its items (no long-row CTAs).
  c.flags &= ~SEGTACO_FLAG_LONG_ROWS;
  *used = c;
  return plan_spmm(p.M, p.K, p.nnz, p.N, p.b_dtype, p.ldb, p.ldc, p.B, p.C, &c, plan);
}

}  // namespace segtaco

using namespace segtaco;

struct segtaco_batch {
  std::vector<segtaco_spmm_problem> problems;
  std::vector<SpmmPlan> plans;
  std::vector<segtaco_config> configs;
  BatchLayout layout;
  char *dmem = nullptr;
  cudaGraphExec_t graph = nullptr;
  int device = -1;
  BatchFork fork;  // created on the first run with more than one group
};

namespace {
// Side streams and events of a batch's fork (non-blocking streams, events
// without timing), created once.
int ensure_fork(segtaco_batch *b) {
  const size_t ng = b->layout.groups.size();
  if (ng < 2 || b->fork.n > 0) return SEGTACO_OK;
  BatchFork &f = b->fork;
  const int n = (int)std::min<size_t>(ng - 1, 4);
  SEGTACO_TRY(check_cuda(cudaEventCreateWithFlags(&f.start, cudaEventDisableTiming), "event"));
  f.join.assign(ng, nullptr);
  for (size_t i = 0; i < ng; ++i)
    SEGTACO_TRY(check_cuda(cudaEventCreateWithFlags(&f.join[i], cudaEventDisableTiming), "event"));
  for (int i = 0; i < n; ++i)
    SEGTACO_TRY(check_cuda(cudaStreamCreateWithFlags(&f.side[i], cudaStreamNonBlocking), "stream"));
  f.n = n;
  return SEGTACO_OK;
}
void destroy_fork(BatchFork &f) {
  for (int i = 0; i < 4; ++i)
    if (f.side[i]) cudaStreamDestroy(f.side[i]);
  for (cudaEvent_t e : f.join)
    if (e) cudaEventDestroy(e);
  if (f.start) cudaEventDestroy(f.start);
  f = BatchFork{};
}
}  // namespace

extern "C" {

int segtaco_row_stats(int32_t M, const int32_t *row_ptr, int64_t *stats, void *stream) {
  if (M < 0 || (M > 0 && !row_ptr) || !stats) return set_error(SEGTACO_EINVAL, "bad arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Scratch scratch(nullptr, 0, s);
  SEGTACO_TRY(scratch.reserve(256));
  auto *d = static_cast<unsigned long long *>(scratch.take(4 * sizeof(unsigned long long)));
  SEGTACO_TRY(check_cuda(cudaMemsetAsync(d, 0, 4 * sizeof(unsigned long long), s), "memset"));
  SEGTACO_TRY(launch_row_stats(row_ptr, M, d, s));
  unsigned long long h[4];
  SEGTACO_TRY(check_cuda(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s), "copy"));
  SEGTACO_TRY(check_cuda(cudaStreamSynchronize(s), "sync"));
  for (int i = 0; i < 4; ++i) stats[i] = (int64_t)h[i];
  return SEGTACO_OK;
}

int segtaco_batch_create(int32_t count, const segtaco_spmm_problem *problems,
                         const segtaco_config *configs, void *stream, segtaco_batch **out) {
  if (!out || count < 0 || (count > 0 && !problems))
    return set_error(SEGTACO_EINVAL, "segtaco_batch_create: bad arguments");
  *out = nullptr;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  auto *b = new segtaco_batch();
  auto fail = [&](int st) {
    segtaco_batch_destroy(b);
    return st;
  };
  b->problems.assign(problems, problems + count);
  b->configs.resize(count);
  b->plans.resize(count);
  // Validate every problem before any device work.
  for (int i = 0; i < count; ++i) {
    const int st = check_batch_problem(b->problems[i], i);
    if (st != SEGTACO_OK) return fail(st);
  }
  cudaGetDevice(&b->device);
  for (int i = 0; i < count; ++i) {
    const auto &p = b->problems[i];
    int64_t stats[4] = {0, 0, 0, 0};
    if (!configs && p.M > 0) {
      const int st = segtaco_row_stats(p.M, p.row_ptr, stats, stream);
      if (st != SEGTACO_OK) return fail(st);
    }
    const int st = plan_batch_problem(p, configs ? &configs[i] : nullptr, stats[0], i,
                                      &b->configs[i], &b->plans[i]);
    if (st != SEGTACO_OK) return fail(st);
  }
  batch_layout(b->problems.data(), b->plans.data(), count, &b->layout);
  {
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&b->dmem), b->layout.bytes);
    if (e != cudaSuccess) return fail(check_cuda(e, "cudaMalloc(batch)"));
  }
  std::vector<char> himg(b->layout.bytes, 0);
  {
    const int st = batch_image(b->problems.data(), b->plans.data(), count, &b->layout, b->dmem,
                               himg.data(), b->device);
    if (st != SEGTACO_OK) return fail(st);
  }
  {
    const int st = check_cuda(cudaMemcpyAsync(b->dmem, himg.data(), b->layout.bytes,
                                              cudaMemcpyHostToDevice, s),
                              "upload batch descriptors");
    if (st != SEGTACO_OK) return fail(st);
    const int st2 = check_cuda(cudaStreamSynchronize(s), "sync");
    if (st2 != SEGTACO_OK) return fail(st2);
  }
  *out = b;
  return SEGTACO_OK;
}

int segtaco_batch_run(segtaco_batch *b, void *stream) {
  if (!b) return set_error(SEGTACO_EINVAL, "batch is NULL");
  SEGTACO_TRY(ensure_fork(b));
  return batch_enqueue(b->layout, b->dmem, static_cast<cudaStream_t>(stream), nullptr, &b->fork);
}

int segtaco_batch_run_graph(segtaco_batch *b, void *stream) {
  if (!b) return set_error(SEGTACO_EINVAL, "batch is NULL");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!b->graph) {
    SEGTACO_TRY(ensure_fork(b));  // side streams join the capture through events
    // Capture on a private stream so the caller's stream may be the legacy one.
    cudaStream_t cs;
    SEGTACO_TRY(check_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "stream"));
    cudaGraph_t graph = nullptr;
    int st = check_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture");
    if (st == SEGTACO_OK) {
      const int est = batch_enqueue(b->layout, b->dmem, cs, nullptr, &b->fork);
      const int cst = check_cuda(cudaStreamEndCapture(cs, &graph), "end capture");
      st = est != SEGTACO_OK ? est : cst;
    }
    if (st == SEGTACO_OK)
      st = check_cuda(cudaGraphInstantiate(&b->graph, graph, 0), "cudaGraphInstantiate");
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    SEGTACO_TRY(st);
  }
  return check_cuda(cudaGraphLaunch(b->graph, s), "cudaGraphLaunch");
}

int segtaco_batch_run_gated(segtaco_batch *b, const int64_t *gate, int64_t timeout_ns,
                            void *stream) {
  if (!b || !gate) return set_error(SEGTACO_EINVAL, "batch or gate is NULL");
  if (timeout_ns <= 0 || timeout_ns > 60LL * 1000000000LL)
    return set_error(SEGTACO_EINVAL, "gate timeout must be in (0, 60 s]");
  BatchGate g;
  g.gate = reinterpret_cast<const volatile long long *>(gate);
  g.timeout_ns = timeout_ns;
  SEGTACO_TRY(tma_status_ptr(&g.status));
  return batch_enqueue(b->layout, b->dmem, static_cast<cudaStream_t>(stream), &g);
}

int segtaco_batch_info(const segtaco_batch *b, int32_t *groups, int64_t *items,
                       segtaco_config *configs) {
  if (!b) return set_error(SEGTACO_EINVAL, "batch is NULL");
  if (groups) *groups = (int32_t)b->layout.groups.size();
  if (items) {
    long long t = 0;
    for (const auto &g : b->layout.groups) t += g.total_items;
    *items = t;
  }
  if (configs)
    for (size_t i = 0; i < b->configs.size(); ++i) configs[i] = b->configs[i];
  return SEGTACO_OK;
}

int segtaco_batch_destroy(segtaco_batch *b) {
  if (!b) return SEGTACO_OK;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  destroy_fork(b->fork);
  if (b->dmem) cudaFree(b->dmem);
  delete b;
  return SEGTACO_OK;
}

}  // extern "C"
