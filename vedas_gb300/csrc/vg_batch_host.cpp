// Batched multi-query execution.
//
// Every query keeps the reference's own plan and job semantics (the host
// mirror in compat/).  Queries advance in waves, one job per query per wave,
// so each query still runs its jobs strictly in plan order (its bounds and
// empty intervals flow from job to job exactly as in QueryPlan::execute).
// Within a wave the device work of all queries is issued together: one
// segmented stable sort for every index swap and implicit join re-sort, one
// copy launch and one unique launch for every select, and one count / scan /
// write chain for every join.  The host phases of a wave (index lookups,
// bounds, empty intervals, relation bookkeeping) run on a thread pool.
#include "vg_batch_host.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>

#include <sched.h>

#include "vg_batch.h"
#include "vg_pool.h"

namespace vg {

namespace {

using Clock = std::chrono::steady_clock;

double since(Clock::time_point t0) {
  return std::chrono::duration<double>(Clock::now() - t0).count();
}

// Persistent host workers for the per-query phases of a wave.  run() hands
// out indices through one atomic counter; the calling thread works too.  A
// wave has several parallel phases a few hundred microseconds apart, so
// idle workers poll for the next phase for a while (kSpin polls) before they
// sleep on the condition variable, and the caller polls for the loop's
// completion the same way: a sleeping thread takes tens of microseconds to
// wake, which would add up over the hundreds of phases of a batch.  A loop is
// complete when all of its items have run; workers busy with queued work
// (post) join it late or not at all, and it does not wait for them.
//
// There is one process-wide pool over all host threads, and one smaller pool
// per wave engine of a batch: the engines' parallel phases run at the same
// time on disjoint threads (engine_pools, UseEnginePool), while planning uses
// them all.
class WorkerPool {
 public:
  // The calling thread's pool: its engine's pool on an engine thread, else
  // the process-wide one.
  static WorkerPool& get() {
    WorkerPool* p = current();
    return p ? *p : global();
  }
  static WorkerPool& global() {
    static WorkerPool pool(host_threads());
    return pool;
  }
  static WorkerPool*& current() {
    static thread_local WorkerPool* p = nullptr;
    return p;
  }
  // VG_HOST_THREADS sets the number of host threads of the process-wide pool,
  // the calling thread included (default: the CPUs this process may run on,
  // at most 32).
  static unsigned host_threads() {
    unsigned total = std::thread::hardware_concurrency();
    cpu_set_t set;
    CPU_ZERO(&set);
    if (sched_getaffinity(0, sizeof(set), &set) == 0 && CPU_COUNT(&set) > 0)
      total = static_cast<unsigned>(CPU_COUNT(&set));
    if (const char* e = std::getenv("VG_HOST_THREADS")) {
      const long v = std::strtol(e, nullptr, 10);
      if (v >= 1) total = static_cast<unsigned>(v);
    }
    return std::max(1u, std::min(total, 32u));
  }
  // threads: the calling thread and threads - 1 workers.
  explicit WorkerPool(unsigned threads) {
    for (unsigned t = 1; t < threads; ++t) workers_.emplace_back([this] { loop(); });
  }
  WorkerPool(const WorkerPool&) = delete;
  WorkerPool& operator=(const WorkerPool&) = delete;

  void run(size_t n, const std::function<void(size_t)>& f0) {
    if (n < 64 || workers_.empty()) {   // small loops run on the caller alone
      for (size_t i = 0; i < n; ++i) f0(i);
      return;
    }
    // the items run with the caller's stream and deferred frees
    const ThreadExec ex = tl_exec;
    const bool carry = ex.stream != nullptr || ex.defer != nullptr;
    const std::function<void(size_t)> wrapped = [&](size_t i) {
      ThreadExecScope sc(ex);
      f0(i);
    };
    const std::function<void(size_t)>& f = carry ? wrapped : f0;
    std::lock_guard<std::mutex> serial(run_mu_);  // one parallel loop at a time
    // No worker is inside a loop here (the last one closed with active_ at 0),
    // so the loop's state can be written before it is opened.
    fn_ = &f;
    n_ = n;
    next_.store(0);
    done_.store(0);
    open_.store(true);
    {
      std::lock_guard<std::mutex> lk(mu_);
      gen_.fetch_add(1);
    }
    cv_.notify_all();
    drain(f, n);
    // The loop ends when every item has run.  Workers that are still busy
    // with queued work never joined it, and nothing waits for them.
    for (int i = 0; i < kSpin && done_.load() != n; ++i) {
    }
    if (done_.load() != n) {
      std::unique_lock<std::mutex> lk(mu_);
      done_cv_.wait(lk, [&] { return done_.load() == n; });
    }
    // Close it, then wait for the workers inside to leave (they find no more
    // items).  A worker that joins after the close sees it closed and leaves
    // without touching the loop's state.
    open_.store(false);
    while (active_.load() != 0) std::this_thread::yield();
    fn_ = nullptr;
    std::exception_ptr e;
    {
      std::lock_guard<std::mutex> lk(err_mu_);
      e = err_;
      err_ = nullptr;
    }
    if (e) std::rethrow_exception(e);
  }

  // Work that no caller waits for.  Idle workers run it between parallel
  // loops; a pool without workers runs it at once on the caller.
  void post(void (*fn)(void*), void* arg) {
    if (workers_.empty()) {
      run_task({fn, arg});
      return;
    }
    {
      std::lock_guard<std::mutex> lk(bg_mu_);
      bg_.push_back({fn, arg});
      bg_n_.fetch_add(1, std::memory_order_release);
    }
    {
      std::lock_guard<std::mutex> lk(mu_);   // a worker about to sleep sees bg_n_ or this notify
    }
    cv_.notify_one();
  }

  // Runs the queued work on the caller and waits for the work that workers
  // are running; the first error a task raised is rethrown here.
  void drain() {
    while (run_one()) {
    }
    while (bg_running_.load(std::memory_order_acquire) != 0) std::this_thread::yield();
    std::string msg;
    {
      std::lock_guard<std::mutex> lk(bg_mu_);
      msg.swap(bg_err_);
    }
    if (!msg.empty()) throw Error(VG_ERR_INVALID, "background release: " + msg);
  }

  ~WorkerPool() {
    stop_.store(true);
    {
      std::lock_guard<std::mutex> lk(mu_);
      gen_.fetch_add(1, std::memory_order_release);
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }

 private:
  static constexpr int kSpin = 1 << 16;

  // Items are taken a few at a time: one shared counter hit per item would
  // make the counter's cache line the bottleneck of short items.  The first
  // exception an item throws is kept and rethrown by run() on the caller.
  void drain(const std::function<void(size_t)>& f, size_t n) {
    const size_t parts = workers_.size() + 1;
    size_t chunk = n / (parts * 8);
    chunk = chunk < 1 ? 1 : (chunk > 16 ? 16 : chunk);
    for (size_t b = next_.fetch_add(chunk); b < n; b = next_.fetch_add(chunk)) {
      const size_t e = b + chunk < n ? b + chunk : n;
      for (size_t i = b; i < e; ++i) {
        try {
          f(i);
        } catch (...) {
          std::lock_guard<std::mutex> lk(err_mu_);
          if (!err_) err_ = std::current_exception();
        }
      }
      if (done_.fetch_add(e - b) + (e - b) == n) {
        std::lock_guard<std::mutex> lk(mu_);
        done_cv_.notify_all();
      }
    }
  }

  struct Task {
    void (*fn)(void*);
    void* arg;
  };

  void run_task(Task t) {
    try {
      t.fn(t.arg);
    } catch (const std::exception& e) {
      std::lock_guard<std::mutex> lk(bg_mu_);
      if (bg_err_.empty()) bg_err_ = e.what();
    } catch (...) {
      std::lock_guard<std::mutex> lk(bg_mu_);
      if (bg_err_.empty()) bg_err_ = "unknown exception";
    }
  }

  // Takes and runs one queued task; false when none is queued.
  bool run_one() {
    if (bg_n_.load(std::memory_order_acquire) == 0) return false;
    Task t;
    {
      std::lock_guard<std::mutex> lk(bg_mu_);
      if (bg_.empty()) return false;
      t = bg_.front();
      bg_.pop_front();
      bg_running_.fetch_add(1, std::memory_order_acq_rel);
      bg_n_.fetch_sub(1, std::memory_order_release);
    }
    run_task(t);
    bg_running_.fetch_sub(1, std::memory_order_acq_rel);
    return true;
  }

  void loop() {
    uint64_t seen = 0;
    while (true) {
      uint64_t g = gen_.load(std::memory_order_acquire);
      for (int i = 0; g == seen && i < kSpin; ++i) {
        if (bg_n_.load(std::memory_order_relaxed) != 0 && run_one()) i = 0;
        g = gen_.load(std::memory_order_acquire);
      }
      if (g == seen) {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] {
          return gen_.load(std::memory_order_acquire) != seen || bg_n_.load(std::memory_order_acquire) != 0;
        });
        g = gen_.load(std::memory_order_acquire);
        if (g == seen) continue;   // woken for queued work: run it from the polling loop
      }
      seen = g;
      if (stop_.load()) return;
      // join the loop only while it is open (see run)
      active_.fetch_add(1);
      if (open_.load() && gen_.load() == g) drain(*fn_, n_);
      active_.fetch_sub(1);
    }
  }

  std::vector<std::thread> workers_;
  std::mutex mu_, run_mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(size_t)>* fn_ = nullptr;   // with n_: read by workers only while open_
  size_t n_ = 0;
  std::atomic<size_t> next_{0};
  std::atomic<size_t> done_{0};     // items of the open loop that have run
  std::atomic<size_t> active_{0};   // workers inside the open loop
  std::atomic<bool> open_{false};
  std::atomic<uint64_t> gen_{0};
  std::atomic<bool> stop_{false};
  std::mutex err_mu_;
  std::exception_ptr err_;
  // queued work (post / drain)
  std::mutex bg_mu_;
  std::deque<Task> bg_;
  std::string bg_err_;
  std::atomic<size_t> bg_n_{0}, bg_running_{0};
};

// The pools of the wave engines of a batch (batch_engines() of them), each
// over an equal share of the host threads, the engine's own thread included;
// made on first use.  With one engine, the engine uses the process-wide pool.
std::atomic<bool> g_engine_pools_made{false};

std::vector<std::unique_ptr<WorkerPool>>& engine_pools() {
  static std::vector<std::unique_ptr<WorkerPool>> v = [] {
    std::vector<std::unique_ptr<WorkerPool>> p;
    const size_t ne = batch_engines();
    const unsigned share = std::max<unsigned>(1, WorkerPool::host_threads() / static_cast<unsigned>(ne));
    if (ne > 1)
      for (size_t e = 0; e < ne; ++e) p.emplace_back(new WorkerPool(share));
    g_engine_pools_made.store(true);
    return p;
  }();
  return v;
}

// Makes engine e's pool the calling thread's pool for its lifetime.
class UseEnginePool {
 public:
  explicit UseEnginePool(size_t e) : prev_(WorkerPool::current()) {
    auto& p = engine_pools();
    if (e < p.size()) WorkerPool::current() = p[e].get();
  }
  ~UseEnginePool() { WorkerPool::current() = prev_; }

 private:
  WorkerPool* prev_;
};

template <typename F>
void pfor(size_t n, F&& f) {
  std::function<void(size_t)> fn = f;
  WorkerPool::get().run(n, fn);
}

template <typename F>
bool guarded(BatchQuery* q, F&& f) {
  try {
    f();
    return true;
  } catch (const Error& e) {
    q->status = e.status;
    q->error = e.what();
  } catch (const std::exception& e) {
    q->status = VG_ERR_INVALID;
    q->error = e.what();
  }
  return false;
}

// Estimated HBM of a query's relations: every pattern's selected rows times
// its variables, in uint32 cells, three times over (the relation, a re-sort's
// key and value buffers).
uint64_t estimate_bytes(vedas::VedasStorage* st, vedas::SparqlQuery& sq) {
  uint64_t est = 0;
  for (size_t i = 0; i < sq.getPatternNum(); ++i) {
    vedas::TriplePattern* tp = sq.getPatternPtr(i);
    uint64_t rows = tp->estimate_rows;
    if (sq.getPatternNum() == 1) {
      auto r = vedas::QueryExecutor::findL2OffsetFromL1(st->getPredicateIndexValues(),
                                                        st->getPredicateIndexOffsets(), tp->getPredicateId(),
                                                        st->getTripleSize());
      rows = r.second >= r.first ? r.second - r.first : 0;
    }
    est += rows * std::max<size_t>(tp->getVariableNum(), 1) * 4 * 3;
  }
  return est + 4096;
}

}  // namespace

void prepare_mirrors(vedas::VedasStorage* storage) { storage->prepareMirrors(); }

void plan_query(Ctx& ctx, vedas::VedasStorage* storage, const char* text, PlannedQuery& pq) {
  guarded(pq.out, [&] {
    pq.ex = std::make_unique<vedas::QueryExecutor>(storage, &ctx);
    pq.sq = std::make_unique<vedas::SparqlQuery>(text, storage->resolver());
    std::set<std::string> sel = pq.sq->getSelectedVariables();
    pq.plan = std::make_unique<vedas::QueryPlan>(sel);
    pq.ex->plan(*pq.sq, *pq.plan);
    pq.plan->beginExecution();
    pq.ex->exe_log.reserve(2 * pq.plan->jobNum() + 2);
    pq.ex->log_text = false;   // batch logs are read as numbers (vg_batch_log)
    pq.est_bytes = estimate_bytes(storage, *pq.sq);
  });
}

BatchResult::~BatchResult() {
  // results, headers and logs of thousands of queries
  auto release = [&](size_t i) {
    BatchQuery& q = queries[i];
    if (ctx) rel_free(*ctx, q.rel);
    std::vector<std::string>().swap(q.headers);
    std::vector<vedas::ExecuteLogRecord>().swap(q.log);
    std::string().swap(q.error);
  };
  if (serial) {
    for (size_t i = 0; i < queries.size(); ++i) release(i);
  } else {
    pfor(queries.size(), release);
  }
}

WaveEngine::WaveEngine(Ctx& ctx, int key_bits) : ctx_(ctx), key_bits_(key_bits) {
  VG_CUDA(cudaEventCreateWithFlags(&ev_a_, cudaEventDisableTiming | cudaEventBlockingSync));
  VG_CUDA(cudaEventCreateWithFlags(&ev_b_, cudaEventDisableTiming | cudaEventBlockingSync));
}

void WaveEngine::use_own_stream() {
  if (own_stream_) return;
  VG_CUDA(cudaStreamCreateWithFlags(&own_stream_, cudaStreamNonBlocking));
  // the engine's work starts after everything already on the context's stream
  cudaEvent_t ev;
  VG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  VG_CUDA(cudaEventRecord(ev, ctx_.stream.main));
  VG_CUDA(cudaStreamWaitEvent(own_stream_, ev, 0));
  cudaEventDestroy(ev);
}

ThreadExec WaveEngine::exec() { return ThreadExec{own_stream_, nullptr}; }

// While a stage enqueues device work, the blocks it frees (scratch of the
// launches just enqueued) may still be read on the engine's stream: those
// frees are held back.  Elsewhere in a stage every block freed was last used
// by work the stage has already waited for, and goes back at once.
ThreadExec WaveEngine::enqueue_exec() { return ThreadExec{own_stream_, own_stream_ ? &defer_ : nullptr}; }

void WaveEngine::finish_stream() {
  if (!own_stream_) return;
  VG_CUDA(cudaStreamSynchronize(own_stream_));
  ctx_.flush(defer_);
}

namespace {
// Waits for a stage's event: polls briefly (most stages are nearly done
// when asked), then sleeps in the CUDA driver so that a waiting engine thread
// leaves its core to the host workers.
void wait_event(cudaEvent_t ev) {
  for (int i = 0; i < 100; ++i) {
    const cudaError_t e = cudaEventQuery(ev);
    if (e == cudaSuccess) return;
    if (e != cudaErrorNotReady) VG_CUDA(e);
  }
  VG_CUDA(cudaEventSynchronize(ev));
}
}  // namespace

WaveEngine::~WaveEngine() {
  bury();
  if (own_stream_) cudaStreamSynchronize(own_stream_);
  else if (a_pending_ || b_pending_) cudaStreamSynchronize(ctx_.stream.main);
  {
    ThreadExecScope sc(exec());   // the stream is idle: frees go back at once
    for (auto& r : jouts_) rel_free(ctx_, r);
    if (jb_.lo || jb_.offs || jb_.d_totals) jb_.release(ctx_);
    if (d_bump_) ctx_.free(d_bump_);
  }
  ctx_.flush(defer_);   // the stream is idle: every held-back free is safe now
  // the region goes back to the arena when its last output is freed
  if (region_) ctx_.arena.region_close(region_);
  if (own_stream_) cudaStreamDestroy(own_stream_);
  if (ev_a_) cudaEventDestroy(ev_a_);
  if (ev_b_) cudaEventDestroy(ev_b_);
}

void WaveEngine::use_region(size_t bytes) {
  if (region_ || bytes == 0) return;
  region_ = ctx_.arena.region_open(bytes);
  if (!region_) return;
  d_bump_ = ctx_.alloc<uint64_t>(1);
  VG_CUDA(cudaMemsetAsync(d_bump_, 0, sizeof(uint64_t), ctx_.stream));
  region_bump_ = 0;
}

void WaveEngine::add(PlannedQuery* pq) { active_.push_back(pq); }

void WaveEngine::bury() {
  release_later(graveyard_);
  graveyard_.clear();
}

void WaveEngine::reset() {
  cudaStreamSynchronize(ctx_.stream);
  a_pending_ = b_pending_ = false;
  bury();
  for (auto& r : jouts_) rel_free(ctx_, r);
  jouts_.clear();
  jb_ = JoinBatch();
  active_.clear();
  run_.clear();
  items_.clear();
  final_.clear();
  fin_seg_.clear();
  fin_res_.clear();
  next_is_a_ = true;
}

void WaveEngine::step(std::vector<PlannedQuery*>& completed) {
  ThreadExecScope sc(exec());
  if (next_is_a_) stage_a(completed);
  else stage_b(completed);
  next_is_a_ = !next_is_a_;
}

void WaveEngine::retire_failed(PlannedQuery* q, std::vector<PlannedQuery*>& completed) {
  if (q->ex) q->out->log = std::move(q->ex->exe_log);
  q->plan.reset();
  completed.push_back(q);
}

// Host finishing of every job of the wave in flight (its device results are
// in: stage B's event has passed).
void WaveEngine::finish_wave() {
  auto t0 = Clock::now();
  const uint32_t* jfl = nullptr;
  if (!joins_.empty()) {
    const uint64_t* hb = h_b_.data();
    if (placed_wave_) {
      // placed joins' first/last came with stage A; the others' with stage B
      const uint32_t* fb = reinterpret_cast<const uint32_t*>(hb + off_fl_);
      for (size_t m = 0; m < joins_.size(); ++m)
        if (!placed_[m]) {
          jfl_[2 * m] = fb[2 * m];
          jfl_[2 * m + 1] = fb[2 * m + 1];
        }
      jfl = jfl_.data();
    } else {
      jfl = reinterpret_cast<const uint32_t*>(hb + off_fl_);
    }
    const uint32_t* c0 = reinterpret_cast<const uint32_t*>(hb + off_jc0_);
    uint64_t off = 0;
    for (size_t m : jsmall_) {
      Item& it = items_[joins_[m]];
      const uint64_t n = jouts_[m].nrows;
      it.c0.assign(c0 + off, c0 + off + n);
      it.has_c0 = true;
      off += n;
    }
  }
  pfor(items_.size(), [&](size_t k) {
    Item& it = items_[k];
    BatchQuery* out = run_[k]->out;
    if (it.kind == Item::kSwap) {
      guarded(out, [&] { it.xj->finish(it.has_c0 ? &it.c0 : nullptr); });
    } else if (it.kind == Item::kJoin) {
      const size_t m = static_cast<size_t>(it.join);
      if (!guarded(out, [&] {
            it.jj->finish(it.jw, jouts_[m], jfl[2 * m], jfl[2 * m + 1], it.has_c0 ? &it.c0 : nullptr);
          }))
        rel_free(ctx_, jouts_[m]);
    }
  });
  jouts_.clear();
  joins_.clear();
  jsmall_.clear();
  for (PlannedQuery* q : run_) {
    ++q->next;
    active_.push_back(q);   // sorted into "next job" or "finished" by the next stage A
  }
  run_.clear();
  items_.clear();
  prof.finish_s += since(t0);
}

void WaveEngine::stage_a(std::vector<PlannedQuery*>& completed) {
  Trace tr{'A', 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (tracing) tr.t0 = since(trace_origin);
  if (b_pending_) {
    auto t0 = Clock::now();
    wait_event(ev_b_);
    b_pending_ = false;
    prof.device_s += since(t0);
  }
  // everything enqueued on the engine's stream so far is done (waited for
  // now, or in stage B with nothing enqueued since): held-back frees are safe
  if (own_stream_) ctx_.flush(defer_);
  if (tracing) tr.t_wait = since(trace_origin);
  {
    auto tf = Clock::now();
    if (!run_.empty()) finish_wave();
    tr.h_finish = since(tf);
  }

  // queries with a next job run it; the others finish (or have failed)
  std::vector<PlannedQuery*> done;
  for (PlannedQuery* q : active_) {
    if (q->out->status != VG_OK || !q->plan || q->next >= q->plan->jobNum()) done.push_back(q);
    else run_.push_back(q);
  }
  active_.clear();

  auto t0 = Clock::now();
  items_.assign(run_.size(), Item());
  const size_t nrun = run_.size();
  if (nrun > 0) {
    ++waves_;
    pfor(nrun, [&](size_t k) {
      PlannedQuery* q = run_[k];
      vedas::QueryJob* job = q->plan->getJob(q->next);
      Item& it = items_[k];
      guarded(q->out, [&] {
        if (auto* sj = dynamic_cast<vedas::SelectQueryJob*>(job)) {
          sj->prepare(it.sw);
          it.kind = Item::kSelect;
        } else if (auto* j = dynamic_cast<vedas::JoinQueryJob*>(job)) {
          j->prepare(it.jw);
          it.jj = j;
          it.kind = it.jw.empty ? Item::kNone : Item::kJoin;
        } else if (auto* x = dynamic_cast<vedas::IndexSwapJob*>(job)) {
          it.xj = x;
          it.xir = x->prepare();
          it.kind = Item::kSwap;
        } else {
          job->startJob(0);  // transfer: a pass-through on one device
        }
      });
      if (q->out->status != VG_OK) it.kind = Item::kNone;
    });
  }
  prof.prepare_s += since(t0);
  tr.h_prepare = since(t0);

  // projection of the queries that finished; failed ones go back at once
  t0 = Clock::now();
  std::vector<PlannedQuery*> fin;
  for (PlannedQuery* q : done) {
    if (q->out->status != VG_OK || !q->plan) retire_failed(q, completed);
    else fin.push_back(q);
  }
  std::vector<SegRows> seg(fin.size());
  std::vector<vedas::FullRelationIR*> res(fin.size(), nullptr);
  pfor(fin.size(), [&](size_t k) {
    PlannedQuery* q = fin[k];
    guarded(q->out, [&] {
      vedas::FullRelationIR* r = q->plan->project();
      SegRows& sr = seg[k];
      sr.ncols = static_cast<uint32_t>(r->getColumnNum());
      sr.n = r->size();
      for (uint32_t c = 0; c < sr.ncols; ++c) {
        sr.in[c] = r->getRelationRawPointer(c);
        sr.out[c] = ctx_.alloc<uint32_t>(sr.n);
      }
      res[k] = r;
    });
  });
  for (size_t k = 0; k < fin.size(); ++k) {
    if (res[k]) {
      final_.push_back(fin[k]);
      fin_seg_.push_back(seg[k]);
      fin_res_.push_back(res[k]);
    } else {
      retire_failed(fin[k], completed);
    }
  }
  prof.final_s += since(t0);
  tr.h_final = since(t0);

  // device half 1
  ThreadExecScope enqueue_scope(enqueue_exec());
  t0 = Clock::now();
  std::vector<Rel*> to_sort;
  std::vector<const Rel*> swap_rels;
  swap_small_.clear();
  joins_.clear();
  std::vector<CopyPiece> pieces;
  std::vector<const Rel*> jl, jr;
  for (size_t k = 0; k < items_.size(); ++k) {
    Item& it = items_[k];
    if (it.kind == Item::kJoin) {
      if (it.jw.sortL) to_sort.push_back(&it.jw.lir->rel());
      if (it.jw.sortR) to_sort.push_back(&it.jw.rir->rel());
      it.join = static_cast<int64_t>(joins_.size());
      joins_.push_back(k);
      jl.push_back(&it.jw.lir->rel());
      jr.push_back(&it.jw.rir->rel());
    } else if (it.kind == Item::kSwap) {
      to_sort.push_back(&it.xir->rel());
      if (it.xir->size() > 2 && it.xir->size() < 100) {
        swap_small_.push_back(k);
        swap_rels.push_back(&it.xir->rel());
      }
    } else if (it.kind == Item::kSelect) {
      pieces.insert(pieces.end(), it.sw.pieces.begin(), it.sw.pieces.end());
    }
  }
  const size_t c0_words = (col0_words(swap_rels) + 1) / 2;
  // joins placed on the device: the small outputs whose column 0 the host
  // scans get staging slots
  placed_wave_ = region_ != nullptr && !jl.empty();
  uint32_t nslots = 0;
  if (placed_wave_) {
    c0_slot_.assign(jl.size(), -1);
    for (size_t m = 0; m < joins_.size(); ++m)
      if (!items_[joins_[m]].jj->isLastJoinForVar()) c0_slot_[m] = static_cast<int32_t>(nslots++);
  }
  off_tot_ = 0;
  off_fin_ = off_tot_ + jl.size();
  off_err_ = off_fin_ + fin_seg_.size();
  off_c0_ = off_err_ + 1;
  off_fla_ = off_c0_ + c0_words;
  off_bump_ = off_fla_ + (placed_wave_ ? jl.size() : 0);
  off_c0a_ = off_bump_ + 1;
  const size_t c0a_words = placed_wave_ ? (static_cast<size_t>(nslots) * kSmallC0Words + 1) / 2 : 0;
  uint64_t* ha = h_a_.reserve(off_c0a_ + c0a_words + 1);
  bool any = false;
  auto tp = Clock::now();
  if (!to_sort.empty()) {
    batched_sort_by_first(ctx_, to_sort, key_bits_);
    any = true;
  }
  tr.h_sort = since(tp);
  if (!swap_rels.empty()) {
    batched_col0_enqueue(ctx_, swap_rels, reinterpret_cast<uint32_t*>(ha + off_c0_));
    any = true;
  }
  tp = Clock::now();
  if (!pieces.empty()) {
    batched_copy(ctx_, pieces);
    any = true;
  }
  tr.h_copy = since(tp);
  tp = Clock::now();
  if (!jl.empty()) {
    batched_join_count(ctx_, jl, jr, jb_, ha + off_tot_);
    // the device error record comes back with the totals: a look-back that
    // gave up leaves the offsets wrong, and stage B must then not write
    VG_CUDA(cudaMemcpyAsync(ha + off_err_, ctx_.d_err, sizeof(DeviceErrors), cudaMemcpyDeviceToHost,
                            ctx_.stream));
    if (placed_wave_)
      batched_join_place_write(ctx_, jb_, region_, d_bump_, c0_slot_, nslots,
                               reinterpret_cast<uint32_t*>(ha + off_fla_), reinterpret_cast<uint32_t*>(ha + off_c0a_),
                               ha + off_bump_);
    any = true;
  }
  tr.h_join = since(tp);
  tp = Clock::now();
  if (!fin_seg_.empty()) {
    batched_unique_enqueue(ctx_, fin_seg_, ha + off_fin_);
    any = true;
  }
  tr.h_unique = since(tp);
  if (any) {
    VG_CUDA(cudaEventRecord(ev_a_, ctx_.stream));
    a_pending_ = true;
  }
  prof.device_s += since(t0);
  if (tracing) {
    tr.t_end = since(trace_origin);
    tr.items = static_cast<uint32_t>(items_.size());
    tr.joins = static_cast<uint32_t>(jl.size());
    tr.sorted_rels = static_cast<uint32_t>(to_sort.size());
    for (const Rel* r : jl) tr.join_left_rows += r->nrows;
    trace.push_back(tr);
  }
}

void WaveEngine::stage_b(std::vector<PlannedQuery*>& completed) {
  if (!a_pending_) return;
  Trace tr{'B', 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (tracing) tr.t0 = since(trace_origin);
  auto t0 = Clock::now();
  wait_event(ev_a_);
  a_pending_ = false;
  prof.device_s += since(t0);
  if (own_stream_) ctx_.flush(defer_);
  if (tracing) tr.t_wait = since(trace_origin);
  const uint64_t* ha = h_a_.data();

  // staged columns of the wave in flight
  {
    const uint32_t* c0 = reinterpret_cast<const uint32_t*>(ha + off_c0_);
    uint64_t off = 0;
    for (size_t k : swap_small_) {
      Item& it = items_[k];
      const uint64_t n = it.xir->size();
      it.c0.assign(c0 + off, c0 + off + n);
      it.has_c0 = true;
      off += n;
    }
  }

  // queries that finished: results handed back
  t0 = Clock::now();
  if (!final_.empty()) {
    const uint64_t* kept = ha + off_fin_;
    note_unique_writes(ctx_, fin_seg_, kept);
    pfor(final_.size(), [&](size_t k) {
      PlannedQuery* q = final_[k];
      BatchQuery* out = q->out;
      vedas::FullRelationIR* r = fin_res_[k];
      for (size_t c = 0; c < r->getColumnNum(); ++c) out->headers.push_back(r->getHeader(c));
      Rel in = r->release();
      rel_free(ctx_, in);
      Rel o;
      o.ncols = fin_seg_[k].ncols;
      o.nrows = kept[k];
      for (uint32_t c = 0; c < o.ncols; ++c) {
        o.cols[c] = fin_seg_[k].out[c];
        ctx_.arena.shrink(o.cols[c], o.nrows * sizeof(uint32_t));
      }
      out->rel = o;
      if (q->ex) out->log = std::move(q->ex->exe_log);
    });
    // the plans (jobs, intermediate relations, host state) of finished
    // queries are destroyed by idle host workers
    for (PlannedQuery* q : final_) graveyard_.push_back(std::move(q->plan));
    bury();
    for (PlannedQuery* q : final_) completed.push_back(q);
    if (host_) {
      std::vector<BatchQuery*> outs;
      for (PlannedQuery* q : final_) outs.push_back(q->out);
      host_->add(outs);   // on the download stream, after an event on the engine's
    }
    final_.clear();
    fin_seg_.clear();
    fin_res_.clear();
  }
  prof.final_s += since(t0);

  // device half 2: join outputs
  ThreadExecScope enqueue_scope(enqueue_exec());
  t0 = Clock::now();
  if (!joins_.empty() && placed_wave_) {
    DeviceErrors he;
    std::memcpy(&he, ha + off_err_, sizeof(he));
    if (he.timeout) ctx_.raise_device_errors(he);
    const uint64_t* tot = ha + off_tot_;
    const size_t J = joins_.size();
    int64_t blocks = 0;
    const uint64_t nb = place_outputs_on_host(jb_, tot, region_, region_bump_, jouts_, placed_, blocks);
    if (nb != ha[off_bump_]) fail(VG_ERR_CUDA, "join output placement differs between device and host");
    region_bump_ = nb;
    ctx_.arena.region_adopt(region_, blocks);
    const uint32_t* fla = reinterpret_cast<const uint32_t*>(ha + off_fla_);
    const uint32_t* c0a = reinterpret_cast<const uint32_t*>(ha + off_c0a_);
    jfl_.assign(2 * J, 0);
    std::vector<size_t> fb_small;
    bool fallback = false;
    double wbytes = 0;
    for (size_t m = 0; m < J; ++m) {
      if (tot[m] > 0xFFFFFFFFull) fail(VG_ERR_OVERFLOW, "join output exceeds 2^32 rows");
      const uint32_t ncols = jb_.l[m]->ncols + jb_.r[m]->ncols - 1;
      if (placed_[m]) {
        wbytes += 4.0 * tot[m] * (2.0 * ncols - 1);
        jfl_[2 * m] = fla[2 * m];
        jfl_[2 * m + 1] = fla[2 * m + 1];
        if (c0_slot_[m] >= 0 && tot[m] > 2 && tot[m] < kSmallC0Words) {
          Item& it = items_[joins_[m]];
          const uint32_t* src = c0a + static_cast<size_t>(c0_slot_[m]) * kSmallC0Words;
          it.c0.assign(src, src + tot[m]);
          it.has_c0 = true;
        }
      } else if (tot[m] == 0) {
        jouts_[m] = rel_alloc(ctx_, ncols, 0);
        placed_[m] = 1;                     // nothing to write
      } else {
        fallback = true;
        if (c0_slot_[m] >= 0 && tot[m] > 2 && tot[m] < kSmallC0Words) fb_small.push_back(m);
      }
    }
    ctx_.add_bytes("join_write", wbytes);
    if (!fallback) {
      jb_.release(ctx_);
      jsmall_.clear();
    } else {
      // outputs that did not fit the region: allocated and written after this round trip
      uint64_t small_rows = 0;
      for (size_t m : fb_small) small_rows += tot[m];
      off_fl_ = 0;
      off_jc0_ = (2 * J + 1) / 2;
      uint64_t* hb = h_b_.reserve(off_jc0_ + (small_rows + 1) / 2 + 1);
      batched_join_write(ctx_, jb_, tot, jouts_, reinterpret_cast<uint32_t*>(hb + off_fl_), placed_.data());
      std::vector<const Rel*> small;
      for (size_t m : fb_small) small.push_back(&jouts_[m]);
      batched_col0_enqueue(ctx_, small, reinterpret_cast<uint32_t*>(hb + off_jc0_));
      jsmall_ = std::move(fb_small);
      VG_CUDA(cudaEventRecord(ev_b_, ctx_.stream));
      b_pending_ = true;
    }
    if (tracing) {
      tr.joins = static_cast<uint32_t>(J);
      for (size_t m = 0; m < J; ++m) tr.join_out_rows += tot[m];
    }
  } else if (!joins_.empty()) {
    DeviceErrors he;
    std::memcpy(&he, ha + off_err_, sizeof(he));
    if (he.timeout) ctx_.raise_device_errors(he);
    const uint64_t* tot = ha + off_tot_;
    std::vector<const Rel*> small;
    std::vector<size_t> who;
    for (size_t m = 0; m < joins_.size(); ++m) {
      Item& it = items_[joins_[m]];
      if (!it.jj->isLastJoinForVar() && tot[m] > 2 && tot[m] < 100) who.push_back(m);
    }
    const size_t J = joins_.size();
    uint64_t small_rows = 0;
    for (size_t m : who) small_rows += tot[m];
    off_fl_ = 0;
    off_jc0_ = (2 * J + 1) / 2;
    uint64_t* hb = h_b_.reserve(off_jc0_ + (small_rows + 1) / 2 + 1);
    batched_join_write(ctx_, jb_, tot, jouts_, reinterpret_cast<uint32_t*>(hb + off_fl_));
    for (size_t m : who) small.push_back(&jouts_[m]);
    batched_col0_enqueue(ctx_, small, reinterpret_cast<uint32_t*>(hb + off_jc0_));
    jsmall_ = std::move(who);
    VG_CUDA(cudaEventRecord(ev_b_, ctx_.stream));
    b_pending_ = true;
    if (tracing) {
      tr.joins = static_cast<uint32_t>(J);
      for (size_t m = 0; m < J; ++m) tr.join_out_rows += tot[m];
    }
  } else {
    jsmall_.clear();
  }
  prof.device_s += since(t0);
  if (tracing) {
    tr.t_end = since(trace_origin);
    tr.items = static_cast<uint32_t>(items_.size());
    trace.push_back(tr);
  }
}

HostResults::~HostResults() {
  // a destructor reports nothing: an error of the copies (a context already
  // failed) has been raised by the batch itself; the chunks are kept out of
  // the pool then, since a copy into them may not have ended
  bool ok = true;
  try {
    finish();
  } catch (const std::exception&) {
    ok = false;
  }
  if (ok)
    for (Chunk& c : chunks_) ctx_.give_pinned(c.p, c.cap);
}

void HostResults::retire_stages(bool all) {
  // a staging block is freed once the main stream is ordered after its copy
  // (a no-op wait when the copy is already done)
  std::vector<Pending> keep;
  for (Pending& p : pending_) {
    if (!all && cudaEventQuery(p.done) != cudaSuccess) {
      keep.push_back(p);
      continue;
    }
    VG_CUDA(cudaStreamWaitEvent(ctx_.stream, p.done, 0));
    for (void* b : p.scratch) ctx_.free(b);
    cudaEventDestroy(p.done);
  }
  pending_.swap(keep);
}

bool HostResults::add(const std::vector<BatchQuery*>& qs) {
  std::lock_guard<std::mutex> lk(mu_);
  retire_stages(false);
  uint64_t words = 0;
  for (const BatchQuery* q : qs) words += q->rel.nrows * q->rel.ncols;
  if (words == 0) return false;
  const size_t bytes = words * sizeof(uint32_t);
  const size_t span = (bytes + 255) / 256 * 256;   // what the chunk gives up (the next start stays aligned)
  if (chunks_.empty() || chunks_.back().used + span > chunks_.back().cap) {
    size_t got = 0;
    void* p = ctx_.take_pinned(std::max<size_t>(span, size_t{256} << 20), &got);
    chunks_.push_back({static_cast<char*>(p), got, 0});
  }
  Chunk& ch = chunks_.back();
  uint32_t* host = reinterpret_cast<uint32_t*>(ch.p + ch.used);
  std::vector<CopyPiece> pieces;
  uint64_t off = 0;
  for (BatchQuery* q : qs)
    for (uint32_t c = 0; c < q->rel.ncols; ++c) {
      pieces.push_back({q->rel.cols[c], host + off, q->rel.nrows});
      q->host[c] = host + off;
      off += q->rel.nrows;
    }
  // the copy kernel runs on the download stream after the results are
  // complete on the calling thread's stream; its scratch is freed once it is done
  cudaEvent_t ready, done;
  VG_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  VG_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
  VG_CUDA(cudaEventRecord(ready, ctx_.stream));
  cudaStream_t dl = ctx_.dl_stream();
  VG_CUDA(cudaStreamWaitEvent(dl, ready, 0));
  DeferredFrees scratch;
  {
    ThreadExecScope sc(ThreadExec{dl, &scratch});
    batched_copy(ctx_, pieces);
    VG_CUDA(cudaEventRecord(done, dl));
  }
  cudaEventDestroy(ready);
  pending_.push_back({std::move(scratch.blocks), done});
  ch.used += span;
  bytes_ += bytes;
  return true;
}

void HostResults::finish() {
  std::lock_guard<std::mutex> lk(mu_);
  if (ctx_.dl_stream_) VG_CUDA(cudaStreamSynchronize(ctx_.dl_stream_));
  retire_stages(true);
}

void run_batch(Ctx& ctx, vedas::VedasStorage* storage, const char* const* texts, size_t n, BatchResult& out,
               bool to_host) {
  auto t_all = Clock::now();
  out.ctx = &ctx;
  out.queries.clear();
  out.queries.resize(n);
  prepare_mirrors(storage);
  std::vector<PlannedQuery> pq(n);
  auto t0 = Clock::now();
  pfor(n, [&](size_t i) {
    pq[i].out = &out.queries[i];
    plan_query(ctx, storage, texts[i] ? texts[i] : "", pq[i]);
  });
  const double plan_s = since(t0);
  // engines take turns on the stream: while the device runs one engine's
  // half-wave, the host runs the others' stages.  Each engine runs on its own
  // host thread with its own share of the worker threads, so the engines'
  // parallel phases run at the same time.
  const int kb = key_bits_for(storage);
  const size_t ne = batch_engines();
  std::vector<std::unique_ptr<WaveEngine>> eng;
  for (size_t e = 0; e < ne; ++e) eng.push_back(std::make_unique<WaveEngine>(ctx, kb));
  if (to_host) {
    out.host = std::make_unique<HostResults>(ctx);
    for (auto& e : eng) e->set_host_results(out.host.get());
  }
  // each engine places its join outputs on the device, in a region of its
  // own, and (VG_ENGINE_STREAMS, default on) issues its work on a stream of
  // its own, so that the engines' kernels overlap on the device
  const size_t region_bytes = join_region_bytes(ctx, ne);
  const bool own_streams = engine_streams();
  for (auto& e : eng) {
    e->use_region(region_bytes);
    if (own_streams) e->use_own_stream();
  }
  const char* trace_path = std::getenv("VG_WAVE_TRACE");
  for (auto& e : eng) {
    e->tracing = trace_path != nullptr;
    e->trace_origin = t_all;
  }
  // Queries are dealt in batch order.  (Dealing by cost, so that every
  // engine got the same mix of long and short job lists, was measured slower
  // on the 4096-query batch: 27.3 ms against 22.7 ms per batch, since every
  // engine then ran the longest chain of waves, each wave with few queries.)
  for (size_t i = 0; i < pq.size(); ++i) eng[i % ne]->add(&pq[i]);
  std::vector<std::exception_ptr> err(ne);
  auto drive = [&](size_t e) {
    UseEnginePool use(e);
    std::vector<PlannedQuery*> done;
    try {
      while (eng[e]->active() > 0) eng[e]->step(done);
    } catch (...) {
      err[e] = std::current_exception();
    }
  };
  std::vector<std::thread> th;
  for (size_t e = 1; e < ne; ++e) th.emplace_back(drive, e);
  drive(0);
  for (auto& t : th) t.join();
  // the results are read on the context's stream: the engines' streams finish first
  for (auto& e : eng) e->finish_stream();
  for (auto& e : err)
    if (e) std::rethrow_exception(e);
  out.waves = 0;
  out.prof = BatchProfile();
  for (auto& e : eng) {
    out.waves = std::max(out.waves, e->waves());
    out.prof.prepare_s += e->prof.prepare_s;
    out.prof.device_s += e->prof.device_s;
    out.prof.finish_s += e->prof.finish_s;
    out.prof.final_s += e->prof.final_s;
  }
  out.prof.plan_s = plan_s;
  if (trace_path) {
    // one line per stage: engine stage t0 t_wait t_end items joins sorted_rels join_left_rows
    // join_out_rows, then host seconds: finish prepare final sort copy join unique
    if (FILE* f = std::fopen(trace_path, "a")) {
      std::fprintf(f, "# batch of %zu queries, planned in %.6f s\n", n, plan_s);
      for (size_t e = 0; e < eng.size(); ++e)
        for (const auto& t : eng[e]->trace)
          std::fprintf(f, "%zu %c %.6f %.6f %.6f %u %u %u %llu %llu %.6f %.6f %.6f %.6f %.6f %.6f %.6f\n", e, t.stage,
                       t.t0, t.t_wait, t.t_end, t.items, t.joins, t.sorted_rels,
                       static_cast<unsigned long long>(t.join_left_rows), static_cast<unsigned long long>(t.join_out_rows),
                       t.h_finish, t.h_prepare, t.h_final, t.h_sort, t.h_copy, t.h_join, t.h_unique);
      std::fclose(f);
    }
  }
  if (out.host) out.host->finish();
  ctx.check_device_errors();
  // plans, parsed queries and executors (bounds, empty intervals, logs) are
  // destroyed by idle host workers
  for (auto& e : eng) e->bury();
  release_later(pq);
  out.prof.total_s = since(t_all);
}

void parallel_for(size_t n, const std::function<void(size_t)>& f) { WorkerPool::get().run(n, f); }

void run_on_engine_pool(size_t e, const std::function<void()>& f) {
  UseEnginePool use(e);
  f();
}

size_t join_region_bytes(const Ctx& ctx, size_t engines) {
  // VG_JOIN_REGION_MB per engine (default 4096; 0 turns device-side placement
  // off), at most an eighth of the arena shared by the engines
  long mb = 4096;
  if (const char* e = std::getenv("VG_JOIN_REGION_MB")) mb = std::strtol(e, nullptr, 10);
  if (mb <= 0) return 0;
  const size_t want = static_cast<size_t>(mb) << 20;
  const size_t cap = ctx.arena.capacity() / (8 * std::max<size_t>(engines, 1));
  return std::min(want, cap);
}

bool engine_streams() {
  const char* e = std::getenv("VG_ENGINE_STREAMS");
  return !(e && std::strtol(e, nullptr, 10) == 0);
}

size_t batch_engines() {
  static const size_t n = [] {
    long v = 4;
    if (const char* e = std::getenv("VG_BATCH_ENGINES")) v = std::strtol(e, nullptr, 10);
    return static_cast<size_t>(std::min(8L, std::max(1L, v)));
  }();
  return n;
}

size_t serve_engines() {
  static const size_t n = [] {
    long v = 1;
    if (const char* e = std::getenv("VG_SERVE_ENGINES")) v = std::strtol(e, nullptr, 10);
    return static_cast<size_t>(std::min(8L, std::max(1L, v)));
  }();
  return n;
}

void post_background(void (*fn)(void*), void* arg) { WorkerPool::get().post(fn, arg); }

void drain_background() {
  // the queued releases free blocks whose last use is done: to the arena at once
  ThreadExecScope sc(ThreadExec{tl_exec.stream, nullptr});
  WorkerPool::global().drain();
  if (g_engine_pools_made.load())
    for (auto& p : engine_pools()) p->drain();
}

namespace {
const bool kReclaimHook = (set_arena_reclaim(&drain_background), true);

// Groups of this many queries' host state per queued task.
constexpr size_t kReleaseGroup = 16;

template <typename T>
void release_groups(std::vector<T>& v) {
  for (size_t b = 0; b < v.size(); b += kReleaseGroup) {
    const size_t e = std::min(v.size(), b + kReleaseGroup);
    auto* grp = new std::vector<T>();
    grp->reserve(e - b);
    for (size_t i = b; i < e; ++i) grp->push_back(std::move(v[i]));
    post_background([](void* p) { delete static_cast<std::vector<T>*>(p); }, grp);
  }
  v.clear();
}
}  // namespace

void release_later(std::vector<std::unique_ptr<vedas::QueryPlan>>& plans) { release_groups(plans); }

// The whole vector is handed over at once; queued tasks release ranges of
// it (a query's plan first, since its jobs point at the executor, then the
// parsed query and the executor) and the last one deletes it.
void release_later(std::vector<PlannedQuery>& pq) {
  if (pq.empty()) return;
  struct Held {
    std::vector<PlannedQuery> v;
    std::atomic<size_t> left{0};
  };
  struct Range {
    Held* h;
    size_t b, e;
  };
  constexpr size_t kRange = 64;
  auto* h = new Held;
  h->v = std::move(pq);
  pq.clear();
  const size_t n = h->v.size(), groups = (n + kRange - 1) / kRange;
  h->left.store(groups);
  for (size_t b = 0; b < n; b += kRange) {
    post_background(
        [](void* p) {
          std::unique_ptr<Range> r(static_cast<Range*>(p));
          for (size_t i = r->b; i < r->e; ++i) {
            PlannedQuery& q = r->h->v[i];
            q.plan.reset();
            q.ex.reset();
            q.sq.reset();
          }
          if (r->h->left.fetch_sub(1, std::memory_order_acq_rel) == 1) delete r->h;
        },
        new Range{h, b, std::min(n, b + kRange)});
  }
}

uint64_t selfcheck_pools(unsigned pools, unsigned threads, unsigned loops) {
  // one caller thread per pool, as the wave engines use theirs
  std::atomic<uint64_t> bad{0}, posted{0}, ran{0};
  std::vector<std::thread> callers;
  for (unsigned k = 0; k < pools; ++k)
    callers.emplace_back([&, k] {
      WorkerPool pool(threads);
      uint64_t x = 0x9E3779B97F4A7C15ull * (k + 1);
      for (unsigned it = 0; it < loops; ++it) {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        const size_t n = 1 + x % 4000;
        std::vector<std::atomic<uint32_t>> hit(n);
        for (auto& h : hit) h.store(0);
        pool.run(n, [&](size_t i) { hit[i].fetch_add(1); });
        for (auto& h : hit) bad += h.load() != 1;
        if (it % 3 == 0) {   // queued work that the loops must not wait for
          ++posted;
          pool.post([](void* a) { static_cast<std::atomic<uint64_t>*>(a)->fetch_add(1); }, &ran);
        }
      }
      pool.drain();
    });
  for (auto& t : callers) t.join();
  return bad.load() + (posted.load() - ran.load());
}

int key_bits_for(vedas::VedasStorage* storage) {
  const uint32_t m = storage->index().max_id;
  int b = 1;
  while (b < 32 && (uint64_t{1} << b) <= m) ++b;
  return b;
}

}  // namespace vg
