// server.cu -- segtaco_server_*: the serving loop.
//
// One scheduler thread owns the device side: the CSR cache, the streams
// ("slots") and every CUDA call.  Client threads only queue requests and wait
// on tickets.  The scheduler repeats:
//   1. completions: a slot whose batch has finished completes its requests,
//      releases their staging bytes and unpins their matrices;
//   2. admission: when a slot is idle, pending requests are taken in arrival
//      order while they fit -- staging bytes under the cap, and their matrix
//      resident or admissible (LRU eviction of unpinned entries until the cap
//      holds) -- up to max_batch;
//   3. launch on that slot's stream: uploads of newly admitted matrices, copies
//      of the dense operands into staging buffers, one persistent batched
//      launch for the SpMMs (batch.cu), one launch per SDDMM, copies of the
//      results back, then an event.
// With several slots, one batch's copies overlap another batch's kernels, and
// requests that arrive meanwhile join the next idle slot's batch.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <list>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.cuh"
#include "internal.h"

namespace segtaco {
long long sddmm_block_nnz();
}

using namespace segtaco;

namespace {

using Clock = std::chrono::steady_clock;

double now_us() {
  return std::chrono::duration<double, std::micro>(Clock::now().time_since_epoch()).count();
}

enum ReqState { kPending, kAdmitted, kDone };

struct Matrix {
  int64_t id = 0;
  int M = 0, K = 0;
  long long nnz = 0;
  const int *h_rp = nullptr, *h_col = nullptr;
  const float *h_val = nullptr;
  long long max_row = 0;
  size_t bytes = 0, off_col = 0, off_val = 0;
  size_t off_starts = 0;  // SDDMM block starts of row_ptr, computed at upload
  // Residency: touched by the scheduler thread only.
  char *dmem = nullptr;
  bool resident = false;
  bool upload_failed = false;
  int pins = 0;
  cudaEvent_t ready = nullptr;
  std::list<Matrix *>::iterator lru;
  bool in_lru = false;
};

struct Req {
  segtaco_request r{};
  int64_t ticket = 0;
  Matrix *m = nullptr;
  double t_arrival = 0, t_done = 0;
  int status = SEGTACO_OK;
  ReqState state = kPending;
  size_t in_bytes = 0, out_bytes = 0, scratch_bytes = 0;
  // Device bytes this request holds while admitted: staged inputs and output
  // (none for device-resident operands) plus kernel scratch.
  size_t staged() const { return align256(in_bytes) + align256(out_bytes) + scratch_bytes; }
  segtaco_config cfg{};
  SpmmPlan plan{};
  char *dbuf = nullptr;
};

struct Slot {
  cudaStream_t s = nullptr;
  cudaEvent_t done = nullptr;
  bool busy = false;
  std::vector<Req *> reqs;
  std::vector<Matrix *> mats;
  size_t staged = 0;
  char *ddesc = nullptr;
  size_t ddesc_cap = 0;
  char *hdesc = nullptr;
  size_t hdesc_cap = 0;
  double fake_ready_at = 0;
};

size_t esize(int dtype) { return dtype == SEGTACO_BF16 ? 2 : 4; }

}  // namespace

struct segtaco_server {
  segtaco_server_config cfg{};
  bool fake = false, per_call = false;
  int device = 0;
  cudaMemPool_t pool = nullptr;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Req *> pending;
  std::vector<std::unique_ptr<Req>> reqs;  // index = ticket
  std::unordered_map<int64_t, std::unique_ptr<Matrix>> mats;
  bool stopping = false;
  std::thread worker;

  // Scheduler-owned.
  std::list<Matrix *> lru;  // front = most recently used
  size_t cache_used = 0, cache_cap = 0, staged = 0;
  std::vector<Slot> slots;
  long long allocs = 0;

  // Counters (under mu).
  int64_t n_submitted = 0, n_completed = 0, n_failed = 0, n_cancelled = 0, n_in_flight = 0;
  int64_t n_batches = 0, n_batched_reqs = 0, hits = 0, misses = 0, evictions = 0;
  int64_t h2d = 0, d2h = 0, cache_now = 0;
  std::vector<double> lat;
  double first_arrival = -1, last_done = 0;

  // ---- device primitives (fake: host memory, no copies, no kernels) ----
  int dev_alloc(void **p, size_t bytes, cudaStream_t s) {
    ++allocs;
    if (cfg.fail_alloc_at > 0 && allocs == cfg.fail_alloc_at)
      return set_error(SEGTACO_ENOMEM, "server: injected allocation failure (allocation %lld)",
                       allocs);
    if (fake) {
      *p = aligned_alloc(256, align256(std::max<size_t>(bytes, 1)));
      return *p ? SEGTACO_OK : set_error(SEGTACO_ENOMEM, "server: host allocation failed");
    }
    const cudaError_t e = cudaMallocFromPoolAsync(p, std::max<size_t>(bytes, 1), pool, s);
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      return set_error(SEGTACO_ENOMEM, "server: device allocation of %zu bytes failed", bytes);
    }
    return check_cuda(e, "cudaMallocFromPoolAsync");
  }
  void dev_free(void *p, cudaStream_t s) {
    if (!p) return;
    if (fake)
      free(p);
    else
      cudaFreeAsync(p, s);
  }
  int copy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
    if (fake || bytes == 0) return SEGTACO_OK;
    return check_cuda(cudaMemcpyAsync(dst, src, bytes, kind, s), "server copy");
  }

  // ---- scheduler ----
  void loop();
  bool slot_finished(Slot &sl);
  void complete(Slot &sl, double t);  // under mu
  void select(std::vector<Req *> &take, std::vector<Matrix *> &evict,
              std::vector<Matrix *> &upload);  // under mu
  void launch(Slot &sl, std::vector<Req *> &take, std::vector<Matrix *> &evict,
              std::vector<Matrix *> &upload);
  void fail_locked(Req *q, int status) {
    q->status = status;
    q->state = kDone;
    q->t_done = now_us();
    ++n_failed;
    cv_done.notify_all();
  }
  int submit_at(const segtaco_request &r, double t_arrival, int64_t *ticket);
};

namespace {

void lru_touch(segtaco_server *S, Matrix *m) {
  if (m->in_lru) S->lru.erase(m->lru);
  S->lru.push_front(m);
  m->lru = S->lru.begin();
  m->in_lru = true;
}

void lru_remove(segtaco_server *S, Matrix *m) {
  if (m->in_lru) S->lru.erase(m->lru);
  m->in_lru = false;
}

}  // namespace

bool segtaco_server::slot_finished(Slot &sl) {
  if (fake) return now_us() >= sl.fake_ready_at;
  const cudaError_t e = cudaEventQuery(sl.done);
  if (e == cudaErrorNotReady) return false;
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(SEGTACO_ECUDA, "server: batch failed: %s", cudaGetErrorString(e));
    for (Req *q : sl.reqs)
      if (q->status == SEGTACO_OK) q->status = SEGTACO_ECUDA;
  }
  return true;
}

void segtaco_server::complete(Slot &sl, double t) {
  for (Req *q : sl.reqs) {
    q->t_done = t;
    q->state = kDone;
    if (q->status == SEGTACO_OK) {
      ++n_completed;
      lat.push_back(t - q->t_arrival);
      last_done = t;
    } else {
      ++n_failed;
    }
  }
  n_in_flight -= (int64_t)sl.reqs.size();
  staged -= sl.staged;
  for (Matrix *m : sl.mats) --m->pins;
  sl.reqs.clear();
  sl.mats.clear();
  sl.staged = 0;
  sl.busy = false;
  cache_now = (int64_t)cache_used;
  cv_done.notify_all();
}

void segtaco_server::select(std::vector<Req *> &take, std::vector<Matrix *> &evict,
                            std::vector<Matrix *> &upload) {
  const size_t max_batch = per_call ? 1 : (size_t)cfg.max_batch;
  for (auto it = pending.begin(); it != pending.end() && take.size() < max_batch;) {
    Req *q = *it;
    Matrix *m = q->m;
    const size_t need = q->staged();
    if (need > (size_t)cfg.staging_bytes) {
      set_error(SEGTACO_ENOMEM, "server: request %lld needs %zu staging bytes, cap %lld",
                (long long)q->ticket, need, (long long)cfg.staging_bytes);
      fail_locked(q, SEGTACO_ENOMEM);
      it = pending.erase(it);
      continue;
    }
    if (staged + need > (size_t)cfg.staging_bytes) break;  // wait for staging to drain
    if (!m->resident) {
      if (m->bytes > cache_cap) {
        set_error(SEGTACO_ENOMEM, "server: matrix %lld (%zu bytes) exceeds the cache cap %zu",
                  (long long)m->id, m->bytes, cache_cap);
        fail_locked(q, SEGTACO_ENOMEM);
        it = pending.erase(it);
        continue;
      }
      // Evict least recently used unpinned entries until the matrix fits.
      auto v = lru.end();
      while (cache_used + m->bytes > cache_cap && v != lru.begin()) {
        --v;
        Matrix *victim = *v;
        if (victim->pins > 0) continue;
        auto next = v;
        ++next;
        lru.erase(v);
        victim->in_lru = false;
        victim->resident = false;
        cache_used -= victim->bytes;
        evict.push_back(victim);
        ++evictions;
        v = next;
      }
      if (cache_used + m->bytes > cache_cap) break;  // wait for pinned entries to drain
      cache_used += m->bytes;
      m->resident = true;
      m->upload_failed = false;
      upload.push_back(m);
      ++misses;
    } else {
      ++hits;
    }
    ++m->pins;
    lru_touch(this, m);
    staged += need;
    q->state = kAdmitted;
    take.push_back(q);
    it = pending.erase(it);
  }
  cache_now = (int64_t)cache_used;
}

void segtaco_server::launch(Slot &sl, std::vector<Req *> &take, std::vector<Matrix *> &evict,
                            std::vector<Matrix *> &upload) {
  cudaStream_t s = sl.s;
  int64_t up = 0, down = 0;
  for (Matrix *v : evict) {
    dev_free(v->dmem, s);
    v->dmem = nullptr;
  }
  for (Matrix *m : upload) {
    void *p = nullptr;
    if (dev_alloc(&p, m->bytes, s) != SEGTACO_OK) {
      m->upload_failed = true;
      continue;
    }
    m->dmem = static_cast<char *>(p);
    if (reinterpret_cast<uintptr_t>(p) & 255) {
      set_error(SEGTACO_EUNSUPPORTED, "server: cache entry not 256-byte aligned");
      m->upload_failed = true;
      continue;
    }
    int st = copy(m->dmem, m->h_rp, (size_t)(m->M + 1) * 4, cudaMemcpyHostToDevice, s);
    if (st == SEGTACO_OK && m->nnz)
      st = copy(m->dmem + m->off_col, m->h_col, (size_t)m->nnz * 4, cudaMemcpyHostToDevice, s);
    if (st == SEGTACO_OK && m->nnz && m->h_val)
      st = copy(m->dmem + m->off_val, m->h_val, (size_t)m->nnz * 4, cudaMemcpyHostToDevice, s);
    // The SDDMM block starts depend only on row_ptr: computed once here, so a
    // resident matrix's SDDMM requests launch the product alone.
    if (st == SEGTACO_OK && m->nnz && !fake) {
      const long long P = sddmm_block_nnz();
      st = launch_block_starts_canonical(reinterpret_cast<const int *>(m->dmem), m->M, (int)P,
                                         (m->nnz + P - 1) / P,
                                         reinterpret_cast<int *>(m->dmem + m->off_starts), s);
    }
    if (!fake) {
      if (!m->ready) cudaEventCreateWithFlags(&m->ready, cudaEventDisableTiming);
      cudaEventRecord(m->ready, s);
    }
    if (st != SEGTACO_OK) m->upload_failed = true;
    up += (int64_t)m->bytes;
  }
  std::vector<segtaco_spmm_problem> probs;
  std::vector<SpmmPlan> plans;
  std::vector<Req *> spmm_reqs;
  // SDDMM requests of one fixed kernel shape and dtype share one launch.
  struct SddmmGroup {
    SddmmShape sh;
    int dtype = 0;
    std::vector<SddmmProblem> probs;
    std::vector<Req *> reqs;
  };
  std::vector<SddmmGroup> sddmm_groups;
  std::vector<Matrix *> waited;
  for (Req *q : take) {
    Matrix *m = q->m;
    sl.mats.push_back(m);
    if (m->upload_failed) {
      q->status = SEGTACO_ENOMEM;
      continue;
    }
    if (!fake && m->ready &&
        std::find(upload.begin(), upload.end(), m) == upload.end() &&
        std::find(waited.begin(), waited.end(), m) == waited.end()) {
      cudaStreamWaitEvent(s, m->ready, 0);  // uploaded by another slot's batch
      waited.push_back(m);
    }
    const bool on_device = q->r.flags & SEGTACO_REQ_DEVICE_DENSE;
    const void *Bd = q->r.B, *Yd = q->r.Y;
    float *outd = q->r.out;
    char *scratch = nullptr;
    if (!on_device) {
      void *p = nullptr;
      if (dev_alloc(&p, q->staged(), s) != SEGTACO_OK) {
        q->status = SEGTACO_ENOMEM;
        continue;
      }
      q->dbuf = static_cast<char *>(p);
      if (reinterpret_cast<uintptr_t>(p) & 255) {  // plans assume 256-byte staging bases
        q->status = set_error(SEGTACO_EUNSUPPORTED, "server: staging buffer not 256-byte aligned");
        continue;
      }
      const size_t es = esize(q->r.dtype);
      const size_t out_off = align256(q->in_bytes);
      scratch = q->dbuf + out_off + align256(q->out_bytes);
      int st;
      if (q->r.op == SEGTACO_OP_SPMM) {
        st = copy(q->dbuf, q->r.B, q->in_bytes, cudaMemcpyHostToDevice, s);
        Bd = q->dbuf;
      } else {
        const size_t xb = (size_t)m->M * q->r.N * es;
        st = copy(q->dbuf, q->r.B, xb, cudaMemcpyHostToDevice, s);
        if (st == SEGTACO_OK)
          st = copy(q->dbuf + align256(xb), q->r.Y, q->in_bytes - align256(xb),
                    cudaMemcpyHostToDevice, s);
        Bd = q->dbuf;
        Yd = q->dbuf + align256(xb);
      }
      outd = reinterpret_cast<float *>(q->dbuf + out_off);
      if (st != SEGTACO_OK) {
        q->status = st;
        continue;
      }
      up += (int64_t)q->in_bytes;
    } else if (q->scratch_bytes) {
      void *p = nullptr;
      if (dev_alloc(&p, q->scratch_bytes, s) != SEGTACO_OK) {
        q->status = SEGTACO_ENOMEM;
        continue;
      }
      q->dbuf = static_cast<char *>(p);
      scratch = q->dbuf;
    }
    const int *rp = reinterpret_cast<const int *>(m->dmem);
    const int *col = reinterpret_cast<const int *>(m->dmem + m->off_col);
    const float *val = m->h_val ? reinterpret_cast<const float *>(m->dmem + m->off_val) : nullptr;
    if (q->r.op == SEGTACO_OP_SPMM) {
      segtaco_spmm_problem p;
      p.M = m->M;
      p.K = m->K;
      p.N = q->r.N;
      p.b_dtype = q->r.dtype;
      p.nnz = m->nnz;
      p.row_ptr = rp;
      p.col = col;
      p.vals = val;
      p.B = Bd;
      p.ldb = q->r.N;
      p.C = outd;
      p.ldc = q->r.N;
      if (per_call) {
        if (fake) continue;
        int *px = reinterpret_cast<int *>(scratch);
        int *py = px ? px + (q->plan.nchunks + 1) : nullptr;
        const int st = run_spmm_planned(q->plan, p.M, p.K, p.nnz, rp, col, val, Bd, p.b_dtype,
                                        p.ldb, outd, p.ldc, p.N, px, py, s);
        if (st != SEGTACO_OK) q->status = st;
      } else {
        probs.push_back(p);
        plans.push_back(q->plan);
        spmm_reqs.push_back(q);
      }
    } else if (!fake && m->nnz > 0) {
      const long long P = sddmm_block_nnz();
      const long long nblk = (m->nnz + P - 1) / P;
      const int *starts = reinterpret_cast<const int *>(m->dmem + m->off_starts);
      const SddmmShape sh = sddmm_shape(q->r.dtype, q->r.N, q->r.N, q->r.N, Bd, Yd);
      if (per_call || sh.family == 0) {
        const int st = launch_sddmm(m->M, m->nnz, rp, col, val, Bd, Yd, q->r.dtype, q->r.N,
                                    q->r.N, q->r.N, outd, const_cast<int *>(starts), (int)P,
                                    nblk, s, /*starts_ready=*/true);
        if (st != SEGTACO_OK) q->status = st;
      } else {
        SddmmGroup *g = nullptr;
        for (SddmmGroup &x : sddmm_groups)
          if (x.dtype == q->r.dtype && x.sh.family == sh.family && x.sh.KI == sh.KI &&
              x.sh.G == sh.G)
            g = &x;
        if (!g) {
          sddmm_groups.emplace_back();
          g = &sddmm_groups.back();
          g->sh = sh;
          g->dtype = q->r.dtype;
        }
        SddmmProblem sp;
        sp.M = m->M;
        sp.nnz = m->nnz;
        sp.row_ptr = rp;
        sp.col = col;
        sp.val = val;
        sp.X = Bd;
        sp.Y = Yd;
        sp.ldx = q->r.N;
        sp.ldy = q->r.N;
        sp.out = outd;
        sp.starts = starts;
        sp.blk_begin = 0;
        g->probs.push_back(sp);
        g->reqs.push_back(q);
      }
    }
  }
  // One launch per SDDMM group; its descriptors in stream-ordered device memory
  // freed on the same stream after the launch.
  for (SddmmGroup &g : sddmm_groups) {
    const long long P = sddmm_block_nnz();
    long long total = 0;
    for (SddmmProblem &sp : g.probs) {
      sp.blk_begin = total;
      total += (sp.nnz + P - 1) / P;
    }
    int st = SEGTACO_OK;
    if (g.probs.size() == 1) {
      const SddmmProblem &sp = g.probs[0];
      st = launch_sddmm(sp.M, sp.nnz, sp.row_ptr, sp.col, sp.val, sp.X, sp.Y, g.dtype,
                        sp.ldx, sp.ldy, (int)sp.ldx, sp.out, const_cast<int *>(sp.starts), (int)P,
                        total, s, /*starts_ready=*/true);
    } else {
      const size_t bytes = g.probs.size() * sizeof(SddmmProblem);
      void *d = nullptr;
      st = dev_alloc(&d, bytes, s);
      if (st == SEGTACO_OK) st = copy(d, g.probs.data(), bytes, cudaMemcpyHostToDevice, s);
      if (st == SEGTACO_OK)
        st = launch_sddmm_multi(g.sh, g.dtype, static_cast<const SddmmProblem *>(d),
                                (int)g.probs.size(), total, s);
      if (d) dev_free(d, s);
    }
    if (st != SEGTACO_OK)
      for (Req *q : g.reqs) q->status = st;
  }
  if (!probs.empty() && !fake) {
    BatchLayout L;
    batch_layout(probs.data(), plans.data(), (int)probs.size(), &L);
    int st = SEGTACO_OK;
    if (L.bytes > sl.hdesc_cap) {
      if (sl.hdesc) cudaFreeHost(sl.hdesc);
      sl.hdesc = nullptr;
      sl.hdesc_cap = 0;
      const size_t cap = std::max(L.bytes * 2, (size_t)1 << 20);
      st = check_cuda(cudaMallocHost(reinterpret_cast<void **>(&sl.hdesc), cap), "cudaMallocHost");
      if (st == SEGTACO_OK) sl.hdesc_cap = cap;
    }
    if (st == SEGTACO_OK && L.bytes > sl.ddesc_cap) {
      dev_free(sl.ddesc, s);
      sl.ddesc = nullptr;
      sl.ddesc_cap = 0;
      const size_t cap = std::max(L.bytes * 2, (size_t)1 << 20);
      void *p = nullptr;
      st = dev_alloc(&p, cap, s);
      if (st == SEGTACO_OK) {
        sl.ddesc = static_cast<char *>(p);
        sl.ddesc_cap = cap;
      }
    }
    if (st == SEGTACO_OK) {
      memset(sl.hdesc, 0, L.bytes);
      st = batch_image(probs.data(), plans.data(), (int)probs.size(), &L, sl.ddesc, sl.hdesc,
                       device);
    }
    if (st == SEGTACO_OK)
      st = copy(sl.ddesc, sl.hdesc, L.bytes, cudaMemcpyHostToDevice, s);
    if (st == SEGTACO_OK) st = batch_enqueue(L, sl.ddesc, s);
    if (st != SEGTACO_OK)
      for (Req *q : spmm_reqs) q->status = st;
  }
  for (Req *q : take) {
    if (q->dbuf && !(q->r.flags & SEGTACO_REQ_DEVICE_DENSE) && q->status == SEGTACO_OK) {
      const int st = copy(q->r.out, q->dbuf + align256(q->in_bytes), q->out_bytes,
                          cudaMemcpyDeviceToHost, s);
      if (st != SEGTACO_OK) q->status = st;
      down += (int64_t)q->out_bytes;
    }
    dev_free(q->dbuf, s);
    q->dbuf = nullptr;
  }
  if (fake) {
    sl.fake_ready_at = now_us() + cfg.fake_delay_us;
  } else if (cudaEventRecord(sl.done, s) != cudaSuccess) {
    cudaGetLastError();
    for (Req *q : take)
      if (q->status == SEGTACO_OK) q->status = SEGTACO_ECUDA;
    cudaStreamSynchronize(s);
  }
  // Matrices whose upload failed leave the cache again.
  for (Matrix *m : upload)
    if (m->upload_failed && m->resident) {
      m->resident = false;
      lru_remove(this, m);
      cache_used -= m->bytes;
      dev_free(m->dmem, s);
      m->dmem = nullptr;
    }
  std::lock_guard<std::mutex> lk(mu);
  h2d += up;
  d2h += down;
}

void segtaco_server::loop() {
  if (!fake) cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    bool progress = false, busy = false;
    for (auto &sl : slots) {
      if (!sl.busy) continue;
      lk.unlock();
      const bool fin = slot_finished(sl);
      lk.lock();
      if (fin) {
        complete(sl, now_us());
        progress = true;
      } else {
        busy = true;
      }
    }
    if (stopping && pending.empty() && !busy) break;
    Slot *idle = nullptr;
    for (auto &sl : slots)
      if (!sl.busy) {
        idle = &sl;
        break;
      }
    if (idle && !pending.empty()) {
      std::vector<Req *> take;
      std::vector<Matrix *> evict, upload;
      const int64_t failed_before = n_failed;
      select(take, evict, upload);
      if (n_failed != failed_before) progress = true;
      if (!take.empty()) {
        idle->busy = true;
        idle->reqs = take;
        size_t st = 0;
        for (Req *q : take) st += q->staged();
        idle->staged = st;
        n_in_flight += (int64_t)take.size();
        ++n_batches;
        n_batched_reqs += (int64_t)take.size();
        lk.unlock();
        launch(*idle, take, evict, upload);
        lk.lock();
        progress = true;
        busy = true;
      }
    }
    if (!progress) {
      if (busy) {
        lk.unlock();
        for (int i = 0; i < 64; ++i) std::this_thread::yield();
        lk.lock();
      } else {
        cv_work.wait_for(lk, std::chrono::milliseconds(5));
      }
    }
  }
}

int segtaco_server::submit_at(const segtaco_request &r, double t_arrival, int64_t *ticket) {
  if (r.op != SEGTACO_OP_SPMM && r.op != SEGTACO_OP_SDDMM)
    return set_error(SEGTACO_EINVAL, "server: unknown op %d", r.op);
  if (r.dtype != SEGTACO_F32 && r.dtype != SEGTACO_BF16)
    return set_error(SEGTACO_EINVAL, "server: unknown dense dtype %d", r.dtype);
  if (r.N <= 0 || r.N > (1 << 16)) return set_error(SEGTACO_EINVAL, "server: N = %d", r.N);
  auto q = std::make_unique<Req>();
  q->r = r;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = mats.find(r.matrix);
    if (it == mats.end())
      return set_error(SEGTACO_EINVAL, "server: unknown matrix id %lld", (long long)r.matrix);
    q->m = it->second.get();
  }
  Matrix *m = q->m;
  const size_t es = esize(r.dtype);
  const bool on_device = r.flags & SEGTACO_REQ_DEVICE_DENSE;
  if (r.op == SEGTACO_OP_SPMM) {
    if ((m->nnz > 0 && !r.B) || (m->M > 0 && !r.out))
      return set_error(SEGTACO_EINVAL, "server: B or out is NULL");
    q->in_bytes = (size_t)m->K * r.N * es;
    q->out_bytes = (size_t)m->M * r.N * 4;
    segtaco_spmm_problem p{};
    p.M = m->M;
    p.K = m->K;
    p.N = r.N;
    p.b_dtype = r.dtype;
    p.nnz = m->nnz;
    p.row_ptr = reinterpret_cast<const int *>(256);  // stand-ins with the alignment of
    p.col = reinterpret_cast<const int *>(256);      // the staging buffers (256 bytes)
    p.B = on_device ? r.B : reinterpret_cast<const void *>(256);
    p.ldb = r.N;
    p.C = on_device ? r.out : reinterpret_cast<float *>(256);
    p.ldc = r.N;
    segtaco_config *cfg = nullptr;
    const int st = plan_batch_problem(p, cfg, m->max_row, 0, &q->cfg, &q->plan);
    if (st != SEGTACO_OK) return st;
    if (per_call) q->scratch_bytes = align256((size_t)(q->plan.nchunks + 1) * 8);
  } else {
    if (m->nnz > 0 && (!r.B || !r.Y || !r.out))
      return set_error(SEGTACO_EINVAL, "server: X, Y or out is NULL");
    q->in_bytes = align256((size_t)m->M * r.N * es) + (size_t)m->K * r.N * es;
    q->out_bytes = (size_t)m->nnz * 4;
    q->scratch_bytes = 0;  // block starts live with the cached matrix
  }
  if (on_device) {
    q->in_bytes = 0;  // nothing staged: staged() counts only scratch
    q->out_bytes = 0;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (stopping) return set_error(SEGTACO_ECANCELLED, "server: shutting down");
  q->ticket = (int64_t)reqs.size();
  q->t_arrival = t_arrival;
  if (first_arrival < 0 || t_arrival < first_arrival) first_arrival = t_arrival;
  pending.push_back(q.get());
  *ticket = q->ticket;
  reqs.push_back(std::move(q));
  ++n_submitted;
  cv_work.notify_one();
  return SEGTACO_OK;
}

extern "C" {

int segtaco_server_create(const segtaco_server_config *cfg, segtaco_server **out) {
  if (!out) return set_error(SEGTACO_EINVAL, "server: out is NULL");
  *out = nullptr;
  auto S = std::make_unique<segtaco_server>();
  if (cfg) S->cfg = *cfg;
  auto &c = S->cfg;
  if (c.max_batch < 0 || c.slots < 0 || c.cache_bytes < 0 || c.staging_bytes < 0 ||
      c.reserve_bytes < 0 || c.fail_alloc_at < 0 || c.fake_delay_us < 0)
    return set_error(SEGTACO_EINVAL, "server: negative configuration value");
  if (c.max_batch == 0) c.max_batch = 64;
  if (c.slots == 0) c.slots = 4;
  if (c.slots > 16) c.slots = 16;
  if (c.cache_bytes == 0) c.cache_bytes = 120LL << 30;
  if (c.staging_bytes == 0) c.staging_bytes = 8LL << 30;
  if (c.reserve_bytes == 0) c.reserve_bytes = 2LL << 30;
  S->fake = c.flags & SEGTACO_SERVER_FAKE_DEVICE;
  S->per_call = c.flags & SEGTACO_SERVER_PER_CALL;
  S->cache_cap = (size_t)c.cache_bytes;
  S->slots.resize(c.slots);
  if (!S->fake) {
    SEGTACO_TRY(check_cuda(cudaGetDevice(&S->device), "cudaGetDevice"));
    size_t free_b = 0, total_b = 0;
    SEGTACO_TRY(check_cuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo"));
    const long long room = (long long)free_b - c.reserve_bytes - c.staging_bytes;
    if (room <= 0) return set_error(SEGTACO_ENOMEM, "server: no free HBM for a cache");
    S->cache_cap = std::min(S->cache_cap, (size_t)room);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = S->device;
    SEGTACO_TRY(check_cuda(cudaMemPoolCreate(&S->pool, &props), "cudaMemPoolCreate"));
    uint64_t keep = ~0ULL;
    cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    for (auto &sl : S->slots) {
      SEGTACO_TRY(check_cuda(cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking), "stream"));
      SEGTACO_TRY(check_cuda(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming), "event"));
    }
  }
  segtaco_server *raw = S.release();
  raw->worker = std::thread([raw] { raw->loop(); });
  *out = raw;
  return SEGTACO_OK;
}

int segtaco_server_add_matrix(segtaco_server *S, int64_t id, int32_t M, int32_t K, int64_t nnz,
                              const int32_t *row_ptr, const int32_t *col, const float *vals) {
  if (!S) return set_error(SEGTACO_EINVAL, "server is NULL");
  if (M < 0 || K < 0 || nnz < 0 || nnz > 0x7fffffffLL || !row_ptr || (nnz > 0 && !col))
    return set_error(SEGTACO_EINVAL, "server: bad CSR arguments for matrix %lld", (long long)id);
  if (row_ptr[0] != 0 || row_ptr[M] != nnz)
    return set_error(SEGTACO_EINVAL, "server: matrix %lld: row_ptr must run from 0 to nnz",
                     (long long)id);
  long long max_row = 0;
  for (int i = 0; i < M; ++i) {
    const long long len = (long long)row_ptr[i + 1] - row_ptr[i];
    if (len < 0)
      return set_error(SEGTACO_EINVAL, "server: matrix %lld: row_ptr decreases at row %d",
                       (long long)id, i);
    max_row = std::max(max_row, len);
  }
  for (long long p = 0; p < nnz; ++p)
    if (col[p] < 0 || col[p] >= K)
      return set_error(SEGTACO_EINVAL, "server: matrix %lld: column %d out of range at %lld",
                       (long long)id, col[p], p);
  auto m = std::make_unique<Matrix>();
  m->id = id;
  m->M = M;
  m->K = K;
  m->nnz = nnz;
  m->h_rp = row_ptr;
  m->h_col = col;
  m->h_val = vals;
  m->max_row = max_row;
  m->off_col = align256((size_t)(M + 1) * 4);
  m->off_val = m->off_col + align256((size_t)nnz * 4);
  m->off_starts = m->off_val + (vals ? align256((size_t)nnz * 4) : 0);
  {
    const long long P = sddmm_block_nnz();
    m->bytes = m->off_starts + align256((size_t)((nnz + P - 1) / P + 1) * 4);
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->mats.count(id)) return set_error(SEGTACO_EINVAL, "server: matrix id %lld exists", (long long)id);
  S->mats.emplace(id, std::move(m));
  return SEGTACO_OK;
}

int segtaco_server_submit(segtaco_server *S, const segtaco_request *req, int64_t *ticket) {
  if (!S || !req || !ticket) return set_error(SEGTACO_EINVAL, "server: NULL argument");
  return S->submit_at(*req, now_us(), ticket);
}

int segtaco_server_replay(segtaco_server *S, int32_t n, const segtaco_request *reqs,
                          const double *arrival_us, int64_t *tickets) {
  if (!S || n < 0 || (n > 0 && (!reqs || !arrival_us || !tickets)))
    return set_error(SEGTACO_EINVAL, "server: bad replay arguments");
  const double t0 = now_us();
  int first_error = SEGTACO_OK;
  for (int i = 0; i < n; ++i) {
    const double target = t0 + arrival_us[i];
    for (;;) {
      const double left = target - now_us();
      if (left <= 0) break;
      if (left > 300)
        std::this_thread::sleep_for(std::chrono::microseconds((long long)(left - 200)));
      else
        std::this_thread::yield();
    }
    const int st = S->submit_at(reqs[i], target, &tickets[i]);
    if (st != SEGTACO_OK) {
      tickets[i] = -1;
      if (first_error == SEGTACO_OK) first_error = st;
    }
  }
  return first_error;
}

int segtaco_server_wait(segtaco_server *S, int64_t ticket, int32_t timeout_ms, int32_t *status) {
  if (!S) return set_error(SEGTACO_EINVAL, "server is NULL");
  std::unique_lock<std::mutex> lk(S->mu);
  if (ticket < 0 || ticket >= (int64_t)S->reqs.size())
    return set_error(SEGTACO_EINVAL, "server: unknown ticket %lld", (long long)ticket);
  Req *q = S->reqs[ticket].get();
  auto done = [&] { return q->state == kDone; };
  if (timeout_ms < 0)
    S->cv_done.wait(lk, done);
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done))
    return SEGTACO_ETIMEOUT;
  if (status) *status = q->status;
  return SEGTACO_OK;
}

int segtaco_server_drain(segtaco_server *S, int32_t timeout_ms) {
  if (!S) return set_error(SEGTACO_EINVAL, "server is NULL");
  std::unique_lock<std::mutex> lk(S->mu);
  auto idle = [&] { return S->pending.empty() && S->n_in_flight == 0; };
  if (timeout_ms < 0)
    S->cv_done.wait(lk, idle);
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), idle))
    return set_error(SEGTACO_ETIMEOUT, "server: drain timed out");
  return SEGTACO_OK;
}

int segtaco_server_cancel(segtaco_server *S, int64_t ticket) {
  if (!S) return set_error(SEGTACO_EINVAL, "server is NULL");
  std::lock_guard<std::mutex> lk(S->mu);
  if (ticket < 0 || ticket >= (int64_t)S->reqs.size())
    return set_error(SEGTACO_EINVAL, "server: unknown ticket %lld", (long long)ticket);
  Req *q = S->reqs[ticket].get();
  if (q->state != kPending) return SEGTACO_EBUSY;
  S->pending.erase(std::find(S->pending.begin(), S->pending.end(), q));
  q->status = SEGTACO_ECANCELLED;
  q->state = kDone;
  q->t_done = now_us();
  ++S->n_cancelled;
  S->cv_done.notify_all();
  return SEGTACO_OK;
}

int segtaco_server_get_stats(segtaco_server *S, int32_t reset, segtaco_server_stats *out) {
  if (!S || !out) return set_error(SEGTACO_EINVAL, "server: NULL argument");
  std::lock_guard<std::mutex> lk(S->mu);
  segtaco_server_stats st{};
  st.submitted = S->n_submitted;
  st.completed = S->n_completed;
  st.failed = S->n_failed;
  st.cancelled = S->n_cancelled;
  st.pending = (int64_t)S->pending.size();
  st.in_flight = S->n_in_flight;
  st.batches = S->n_batches;
  st.cache_hits = S->hits;
  st.cache_misses = S->misses;
  st.evictions = S->evictions;
  st.cache_bytes = S->cache_now;
  st.h2d_bytes = S->h2d;
  st.d2h_bytes = S->d2h;
  st.mean_batch = S->n_batches ? (double)S->n_batched_reqs / S->n_batches : 0.0;
  if (!S->lat.empty()) {
    std::vector<double> v = S->lat;
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
      const size_t i = (size_t)std::min<double>(v.size() - 1, std::ceil(p * v.size()) - 1);
      return v[i];
    };
    st.p50_us = pct(0.50);
    st.p99_us = pct(0.99);
    st.max_us = v.back();
    double sum = 0;
    for (double x : v) sum += x;
    st.mean_us = sum / v.size();
    st.span_s = (S->last_done - S->first_arrival) * 1e-6;
  }
  *out = st;
  if (reset) {
    S->lat.clear();
    S->n_submitted = S->n_completed = S->n_failed = S->n_cancelled = 0;
    S->n_batches = S->n_batched_reqs = S->hits = S->misses = S->evictions = 0;
    S->h2d = S->d2h = 0;
    S->first_arrival = -1;
    S->last_done = 0;
  }
  return SEGTACO_OK;
}

int segtaco_server_destroy(segtaco_server *S) {
  if (!S) return SEGTACO_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    for (Req *q : S->pending) {
      q->status = SEGTACO_ECANCELLED;
      q->state = kDone;
      ++S->n_cancelled;
    }
    S->pending.clear();
    S->stopping = true;
    S->cv_work.notify_all();
    S->cv_done.notify_all();
  }
  if (S->worker.joinable()) S->worker.join();
  if (!S->fake) {
    for (auto &sl : S->slots) {
      if (sl.s) cudaStreamSynchronize(sl.s);
      if (sl.ddesc) cudaFreeAsync(sl.ddesc, sl.s);
      if (sl.hdesc) cudaFreeHost(sl.hdesc);
    }
    for (auto &kv : S->mats) {
      Matrix *m = kv.second.get();
      if (m->dmem) cudaFreeAsync(m->dmem, S->slots[0].s);
      if (m->ready) cudaEventDestroy(m->ready);
    }
    for (auto &sl : S->slots) {
      if (sl.s) {
        cudaStreamSynchronize(sl.s);
        cudaStreamDestroy(sl.s);
      }
      if (sl.done) cudaEventDestroy(sl.done);
    }
    if (S->pool) cudaMemPoolDestroy(S->pool);
  } else {
    for (auto &sl : S->slots) free(sl.ddesc);
    for (auto &kv : S->mats) free(kv.second->dmem);
  }
  delete S;
  return SEGTACO_OK;
}

}  // extern "C"
