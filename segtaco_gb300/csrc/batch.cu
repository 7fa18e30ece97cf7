// batch.cu -- segtaco_batch_*: plan, run (optionally through a CUDA graph) and
// free a batch of SpMMs of uneven shapes.  Kernels: batch.cuh.
#include <algorithm>
#include <cstring>
#include <map>
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
__global__ void batch_partition_kernel(const BatchPartition *__restrict__ parts, int nparts,
                                       long long total_edges) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_edges) return;
  int lo = 0, hi = nparts - 1;  // last part with edge_begin <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (parts[mid].edge_begin <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  const BatchPartition &bp = parts[lo];
  const long long c = t - bp.edge_begin;
  long long d = c * bp.D;
  const long long total = (long long)bp.M + bp.nnz;
  if (d > total) d = total;
  const int x = merge_path_x(bp.row_ptr, bp.M, bp.nnz, d);
  const int y = (int)(d - x);
  bp.px[c] = x;
  bp.py[c] = y;
  if (x < bp.M && __ldg(bp.row_ptr + x) < y) {
    float *dst = bp.C + (long long)x * bp.ldc;
    int k = 0;
    if ((((uintptr_t)dst) & 15) == 0)
      for (; k + 4 <= bp.N; k += 4) *reinterpret_cast<float4 *>(dst + k) = make_float4(0, 0, 0, 0);
    for (; k < bp.N; ++k) dst[k] = 0.0f;
  }
}

}  // namespace segtaco

using namespace segtaco;

struct segtaco_batch {
  struct Group {
    int dtype, V, G;
    bool rows;
    std::vector<int> members;
    long long total_items = 0;
    size_t off_probs = 0, off_begin = 0;  // offsets into the device buffer
    int grid = 0;
  };
  std::vector<segtaco_spmm_problem> problems;
  std::vector<SpmmPlan> plans;
  std::vector<segtaco_config> configs;
  std::vector<Group> groups;
  char *dmem = nullptr;
  size_t dbytes = 0;
  size_t off_parts = 0, off_queues = 0;
  int nparts = 0;
  long long total_edges = 0;
  cudaGraphExec_t graph = nullptr;
  int device = -1;
};

namespace {

int enqueue(segtaco_batch *b, cudaStream_t s) {
  if (!b->groups.empty())
    SEGTACO_TRY(check_cuda(cudaMemsetAsync(b->dmem + b->off_queues, 0,
                                           b->groups.size() * sizeof(unsigned long long), s),
                           "memset queues"));
  if (b->total_edges > 0) {
    const long long blocks = (b->total_edges + 255) / 256;
    batch_partition_kernel<<<(unsigned)blocks, 256, 0, s>>>(
        reinterpret_cast<const BatchPartition *>(b->dmem + b->off_parts), b->nparts,
        b->total_edges);
    SEGTACO_TRY(check_launch("batch_partition_kernel"));
  }
  for (size_t gi = 0; gi < b->groups.size(); ++gi) {
    const auto &g = b->groups[gi];
    if (g.total_items == 0) continue;
    BatchGroupLaunch L;
    L.V = g.V;
    L.G = g.G;
    L.rows = g.rows;
    L.probs = b->dmem + g.off_probs;
    L.item_begin = reinterpret_cast<const long long *>(b->dmem + g.off_begin);
    L.nprobs = (int)g.members.size();
    L.total_items = g.total_items;
    L.queue = reinterpret_cast<unsigned long long *>(b->dmem + b->off_queues) + gi;
    L.grid = g.grid;
    SEGTACO_TRY(g.dtype == SEGTACO_BF16 ? launch_batch_bf16(L, s) : launch_batch_f32(L, s));
  }
  return SEGTACO_OK;
}

template <typename BT>
void fill_problem(BatchProblem<BT> &bp, const segtaco_spmm_problem &p, const SpmmPlan &plan,
                  int *px, int *py, long long item_begin) {
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
  cudaGetDevice(&b->device);
  b->problems.assign(problems, problems + count);
  b->configs.resize(count);
  b->plans.resize(count);
  // ---- configs: the caller's, or the heuristic on device row statistics ----
  std::vector<int64_t> stats(4 * (size_t)count, 0);
  if (!configs) {
    for (int i = 0; i < count; ++i) {
      const auto &p = b->problems[i];
      if (p.M > 0) {
        const int st = segtaco_row_stats(p.M, p.row_ptr, &stats[4 * (size_t)i], stream);
        if (st != SEGTACO_OK) return fail(st);
      }
    }
  }
  for (int i = 0; i < count; ++i) {
    const auto &p = b->problems[i];
    if (p.M < 0 || p.K < 0 || p.N < 0 || p.nnz < 0 || p.nnz > 0x7fffffffLL ||
        (p.M > 0 && !p.row_ptr) ||
        (p.nnz > 0 && (!p.col || !p.B)) || (p.M > 0 && p.N > 0 && !p.C) || p.ldb < p.N ||
        p.ldc < p.N || (p.b_dtype != SEGTACO_F32 && p.b_dtype != SEGTACO_BF16))
      return fail(set_error(SEGTACO_EINVAL, "segtaco_batch_create: problem %d is malformed", i));
    segtaco_config c;
    if (configs) {
      c = configs[i];
    } else {
      c.schedule = SEGTACO_AUTO;
      segtaco_autotune_heuristic(p.M, p.K, p.nnz, p.N, p.b_dtype, stats[4 * (size_t)i], &c);
    }
    c.depth = 0;                          // batch kernels keep 4 loads in flight
    c.flags &= ~(SEGTACO_FLAG_SMEM_RING | SEGTACO_FLAG_TMA_BULK | SEGTACO_FLAG_PARTITION_READY);
    b->configs[i] = c;
    const int st = plan_spmm(p.M, p.K, p.nnz, p.N, p.b_dtype, p.ldb, p.ldc, p.B, p.C, &c,
                             &b->plans[i]);
    if (st != SEGTACO_OK) return fail(st);
  }
  // ---- groups by kernel variant ----
  std::map<std::tuple<int, int, int, bool>, int> gidx;
  for (int i = 0; i < count; ++i) {
    const auto &p = b->problems[i];
    if (p.M == 0 || p.N == 0) continue;
    const auto &pl = b->plans[i];
    const bool rows = pl.schedule == SEGTACO_RB_SR || pl.schedule == SEGTACO_RB_PR;
    const auto key = std::make_tuple(p.b_dtype, pl.V, pl.G, rows);
    auto it = gidx.find(key);
    if (it == gidx.end()) {
      it = gidx.emplace(key, (int)b->groups.size()).first;
      segtaco_batch::Group g;
      g.dtype = p.b_dtype;
      g.V = pl.V;
      g.G = pl.G;
      g.rows = rows;
      b->groups.push_back(g);
    }
    b->groups[it->second].members.push_back(i);
  }
  // ---- device buffer layout ----
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += align256(bytes);
    return o;
  };
  std::vector<size_t> off_px(count, 0), off_py(count, 0);
  std::vector<char> has_part(count, 0);
  for (int i = 0; i < count; ++i) {
    const auto &pl = b->plans[i];
    const bool eb = pl.schedule == SEGTACO_EB_SR || pl.schedule == SEGTACO_EB_PR;
    if (eb && b->problems[i].M > 0 && b->problems[i].N > 0) {
      has_part[i] = 1;
      off_px[i] = take((pl.nchunks + 1) * sizeof(int));
      off_py[i] = take((pl.nchunks + 1) * sizeof(int));
      ++b->nparts;
    }
  }
  b->off_parts = take(std::max(1, b->nparts) * sizeof(BatchPartition));
  for (auto &g : b->groups) {
    g.off_probs = take(g.members.size() * sizeof(BatchProblem<float>));
    g.off_begin = take(g.members.size() * sizeof(long long));
  }
  b->off_queues = take(std::max<size_t>(1, b->groups.size()) * sizeof(unsigned long long));
  b->dbytes = off;
  {
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&b->dmem), b->dbytes);
    if (e != cudaSuccess) return fail(check_cuda(e, "cudaMalloc(batch)"));
  }
  // ---- host images of the descriptors ----
  std::vector<char> himg(b->dbytes, 0);
  std::vector<BatchPartition> parts;
  long long edges = 0;
  for (int i = 0; i < count; ++i) {
    if (!has_part[i]) continue;
    const auto &p = b->problems[i];
    const auto &pl = b->plans[i];
    BatchPartition bp;
    bp.row_ptr = p.row_ptr;
    bp.M = p.M;
    bp.nnz = p.nnz;
    bp.D = pl.items_per_unit;
    bp.nchunks = pl.nchunks;
    bp.px = reinterpret_cast<int *>(b->dmem + off_px[i]);
    bp.py = reinterpret_cast<int *>(b->dmem + off_py[i]);
    bp.C = p.C;
    bp.ldc = p.ldc;
    bp.N = p.N;
    bp.edge_begin = edges;
    edges += pl.nchunks + 1;
    parts.push_back(bp);
  }
  b->total_edges = edges;
  if (!parts.empty())
    memcpy(himg.data() + b->off_parts, parts.data(), parts.size() * sizeof(BatchPartition));
  for (auto &g : b->groups) {
    long long item = 0;
    std::vector<long long> begin;
    for (size_t k = 0; k < g.members.size(); ++k) {
      const int i = g.members[k];
      const auto &pl = b->plans[i];
      int *px = has_part[i] ? reinterpret_cast<int *>(b->dmem + off_px[i]) : nullptr;
      int *py = has_part[i] ? reinterpret_cast<int *>(b->dmem + off_py[i]) : nullptr;
      begin.push_back(item);
      if (g.dtype == SEGTACO_BF16) {
        BatchProblem<uint16_t> bp;
        fill_problem(bp, b->problems[i], pl, px, py, item);
        memcpy(himg.data() + g.off_probs + k * sizeof(bp), &bp, sizeof(bp));
      } else {
        BatchProblem<float> bp;
        fill_problem(bp, b->problems[i], pl, px, py, item);
        memcpy(himg.data() + g.off_probs + k * sizeof(bp), &bp, sizeof(bp));
      }
      item += pl.nchunks * (long long)pl.slabs;
    }
    g.total_items = item;
    memcpy(himg.data() + g.off_begin, begin.data(), begin.size() * sizeof(long long));
    // Persistent grid: every SM full, never more CTAs than items need.
    int per_sm = 0, sms = 0;
    const int st = g.dtype == SEGTACO_BF16 ? batch_blocks_per_sm_bf16(g.V, g.G, g.rows, &per_sm)
                                           : batch_blocks_per_sm_f32(g.V, g.G, g.rows, &per_sm);
    if (st != SEGTACO_OK) return fail(st);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    const long long need = (item + (kCta / 32) - 1) / (kCta / 32);
    long long grid = (long long)std::max(1, per_sm) * std::max(1, sms);
    if (grid > need) grid = std::max(1LL, need);
    g.grid = (int)grid;
  }
  {
    const int st = check_cuda(cudaMemcpyAsync(b->dmem, himg.data(), b->dbytes,
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
  return enqueue(b, static_cast<cudaStream_t>(stream));
}

int segtaco_batch_run_graph(segtaco_batch *b, void *stream) {
  if (!b) return set_error(SEGTACO_EINVAL, "batch is NULL");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!b->graph) {
    // Capture on a private stream so the caller's stream may be the legacy one.
    cudaStream_t cs;
    SEGTACO_TRY(check_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "stream"));
    cudaGraph_t graph = nullptr;
    int st = check_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture");
    if (st == SEGTACO_OK) {
      const int est = enqueue(b, cs);
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

int segtaco_batch_info(const segtaco_batch *b, int32_t *groups, int64_t *items,
                       segtaco_config *configs) {
  if (!b) return set_error(SEGTACO_EINVAL, "batch is NULL");
  if (groups) *groups = (int32_t)b->groups.size();
  if (items) {
    long long t = 0;
    for (const auto &g : b->groups) t += g.total_items;
    *items = t;
  }
  if (configs)
    for (size_t i = 0; i < b->configs.size(); ++i) configs[i] = b->configs[i];
  return SEGTACO_OK;
}

int segtaco_batch_destroy(segtaco_batch *b) {
  if (!b) return SEGTACO_OK;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->dmem) cudaFree(b->dmem);
  delete b;
  return SEGTACO_OK;
}

}  // extern "C"
