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
#include <cstdlib>
#include <functional>
#include <mutex>
#include <thread>

#include "vg_batch.h"

namespace vg {

namespace {

using Clock = std::chrono::steady_clock;

double since(Clock::time_point t0) {
  return std::chrono::duration<double>(Clock::now() - t0).count();
}

// Persistent host workers for the per-query phases of a wave.  run() hands
// out indices through one atomic counter; the calling thread works too.
class WorkerPool {
 public:
  static WorkerPool& get() {
    static WorkerPool pool;
    return pool;
  }

  void run(size_t n, const std::function<void(size_t)>& f) {
    std::lock_guard<std::mutex> serial(run_mu_);  // one parallel loop at a time
    if (n < 64 || workers_.empty()) {
      for (size_t i = 0; i < n; ++i) f(i);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn_ = &f;
      n_ = n;
      next_.store(0);
      busy_ = workers_.size();
      ++gen_;
    }
    cv_.notify_all();
    drain(f, n);
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return busy_ == 0; });
    fn_ = nullptr;
  }

  ~WorkerPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }

 private:
  // VG_HOST_THREADS sets the number of host threads of a parallel phase,
  // the calling thread included (default: the hardware threads, at most 32).
  WorkerPool() {
    unsigned total = std::thread::hardware_concurrency();
    if (const char* e = std::getenv("VG_HOST_THREADS")) {
      const long v = std::strtol(e, nullptr, 10);
      if (v >= 1) total = static_cast<unsigned>(v);
    }
    const unsigned nt = total > 1 ? std::min<unsigned>(total - 1, 31) : 0;
    for (unsigned t = 0; t < nt; ++t) workers_.emplace_back([this] { loop(); });
  }

  void drain(const std::function<void(size_t)>& f, size_t n) {
    for (size_t i = next_.fetch_add(1); i < n; i = next_.fetch_add(1)) f(i);
  }

  void loop() {
    uint64_t seen = 0;
    while (true) {
      const std::function<void(size_t)>* f;
      size_t n;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
        f = fn_;
        n = n_;
      }
      if (f) drain(*f, n);
      std::lock_guard<std::mutex> lk(mu_);
      if (--busy_ == 0) done_cv_.notify_all();
    }
  }

  std::vector<std::thread> workers_;
  std::mutex mu_, run_mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(size_t)>* fn_ = nullptr;
  size_t n_ = 0;
  std::atomic<size_t> next_{0};
  size_t busy_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
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

void prepare_mirrors(vedas::VedasStorage* storage) {
  storage->getPredicateIndexValues();
  storage->getPredicateIndexOffsets();
  storage->getPredicateSubjectIndexValues();
  storage->getPredicateSubjectIndexOffsets();
  storage->getPredicateObjectIndexValues();
  storage->getPredicateObjectIndexOffsets();
  storage->getPSdata();
  storage->getPOdata();
  storage->getPSOdata();
  storage->getPOSdata();
}

void plan_query(Ctx& ctx, vedas::VedasStorage* storage, const std::string& text, PlannedQuery& pq) {
  guarded(pq.out, [&] {
    pq.ex = std::make_unique<vedas::QueryExecutor>(storage, &ctx);
    pq.sq = std::make_unique<vedas::SparqlQuery>(text.c_str());
    std::set<std::string> sel = pq.sq->getSelectedVariables();
    pq.plan = std::make_unique<vedas::QueryPlan>(sel);
    pq.ex->plan(*pq.sq, *pq.plan);
    pq.plan->beginExecution();
    pq.est_bytes = estimate_bytes(storage, *pq.sq);
  });
}

BatchResult::~BatchResult() {
  if (ctx)
    for (auto& q : queries) rel_free(*ctx, q.rel);
}

void WaveEngine::add(PlannedQuery* pq) { active_.push_back(pq); }

void WaveEngine::wave(std::vector<PlannedQuery*>& completed) {
  // Queries that failed while planning, or have no job left, finish now.
  std::vector<PlannedQuery*> run, done;
  for (PlannedQuery* q : active_) {
    if (q->out->status != VG_OK || !q->plan || q->next >= q->plan->jobNum()) done.push_back(q);
    else run.push_back(q);
  }
  if (!run.empty()) {
    ++waves_;
    enum Kind { kNone, kSelect, kJoin, kSwap };
    struct Item {
      Kind kind = kNone;
      vedas::SelectWork sw;
      vedas::JoinQueryJob* jj = nullptr;
      vedas::JoinWork jw;
      vedas::IndexSwapJob* xj = nullptr;
      vedas::FullRelationIR* xir = nullptr;
    };
    std::vector<Item> items(run.size());
    auto t0 = Clock::now();
    pfor(run.size(), [&](size_t k) {
      PlannedQuery* q = run[k];
      vedas::QueryJob* job = q->plan->getJob(q->next);
      Item& it = items[k];
      guarded(q->out, [&] {
        if (auto* s = dynamic_cast<vedas::SelectQueryJob*>(job)) {
          s->prepare(it.sw);
          it.kind = kSelect;
        } else if (auto* j = dynamic_cast<vedas::JoinQueryJob*>(job)) {
          j->prepare(it.jw);
          it.jj = j;
          it.kind = it.jw.empty ? kNone : kJoin;
        } else if (auto* x = dynamic_cast<vedas::IndexSwapJob*>(job)) {
          it.xj = x;
          it.xir = x->prepare();
          it.kind = kSwap;
        } else {
          job->startJob(0);  // transfer: a pass-through on one device
        }
      });
      if (q->out->status != VG_OK) it.kind = kNone;
    });
    prof.prepare_s += since(t0);

    // 1. every stable re-sort by column 0 of this wave in one segmented sort
    t0 = Clock::now();
    std::vector<Rel*> to_sort;
    for (auto& it : items) {
      if (it.kind == kJoin) {
        if (it.jw.sortL) to_sort.push_back(&it.jw.lir->rel());
        if (it.jw.sortR) to_sort.push_back(&it.jw.rir->rel());
      } else if (it.kind == kSwap) {
        to_sort.push_back(&it.xir->rel());
      }
    }
    batched_sort_by_first(ctx_, to_sort);

    // 2. empty-interval scans of swapped relations need column 0 of the small ones
    std::vector<std::vector<uint32_t>> swap_c0;
    std::vector<const std::vector<uint32_t>*> swap_c0_of(items.size(), nullptr);
    {
      std::vector<const Rel*> small;
      std::vector<size_t> who;
      for (size_t k = 0; k < items.size(); ++k)
        if (items[k].kind == kSwap && items[k].xir->size() > 2 && items[k].xir->size() < 100) {
          small.push_back(&items[k].xir->rel());
          who.push_back(k);
        }
      batched_col0(ctx_, small, swap_c0);
      for (size_t m = 0; m < who.size(); ++m) swap_c0_of[who[m]] = &swap_c0[m];
    }

    // 3. selects: all copies in one launch, all unique compactions in one
    std::vector<uint64_t> kept_of(items.size(), 0);
    {
      std::vector<CopyPiece> pieces;
      std::vector<SegRows> useg;
      std::vector<size_t> uwho;
      for (size_t k = 0; k < items.size(); ++k) {
        if (items[k].kind != kSelect) continue;
        auto& w = items[k].sw;
        if (w.unique) {
          SegRows s;
          s.ncols = 1;
          s.n = w.uniq_n;
          s.in[0] = w.uniq_src;
          s.out[0] = w.ir->getRelationRawPointer(0);
          useg.push_back(s);
          uwho.push_back(k);
        } else {
          pieces.insert(pieces.end(), w.pieces.begin(), w.pieces.end());
        }
      }
      batched_copy(ctx_, pieces);
      std::vector<uint64_t> kept = batched_unique(ctx_, useg);
      for (size_t m = 0; m < uwho.size(); ++m) kept_of[uwho[m]] = kept[m];
    }

    // 4. joins: one count / scan / write chain for all of them
    std::vector<size_t> jwho;
    std::vector<Rel> jouts;
    std::vector<uint32_t> jfl;
    std::vector<std::vector<uint32_t>> join_c0;
    std::vector<const std::vector<uint32_t>*> join_c0_of(items.size(), nullptr);
    {
      std::vector<const Rel*> L, R;
      for (size_t k = 0; k < items.size(); ++k)
        if (items[k].kind == kJoin) {
          L.push_back(&items[k].jw.lir->rel());
          R.push_back(&items[k].jw.rir->rel());
          jwho.push_back(k);
        }
      batched_join(ctx_, L, R, jouts, jfl);
      std::vector<const Rel*> small;
      std::vector<size_t> who;
      for (size_t m = 0; m < jwho.size(); ++m)
        if (!items[jwho[m]].jj->isLastJoinForVar() && jouts[m].nrows > 2 && jouts[m].nrows < 100) {
          small.push_back(&jouts[m]);
          who.push_back(jwho[m]);
        }
      batched_col0(ctx_, small, join_c0);
      for (size_t m = 0; m < who.size(); ++m) join_c0_of[who[m]] = &join_c0[m];
    }
    prof.device_s += since(t0);

    // 5. host finishing of every job of the wave
    t0 = Clock::now();
    std::vector<size_t> jpos(items.size(), 0);
    for (size_t m = 0; m < jwho.size(); ++m) jpos[jwho[m]] = m;
    pfor(items.size(), [&](size_t k) {
      Item& it = items[k];
      BatchQuery* out = run[k]->out;
      if (it.kind == kSwap) {
        guarded(out, [&] { it.xj->finish(swap_c0_of[k]); });
      } else if (it.kind == kSelect) {
        if (it.sw.unique) vedas::SelectQueryJob::finishUnique(it.sw, kept_of[k]);
      } else if (it.kind == kJoin) {
        const size_t m = jpos[k];
        if (!guarded(out, [&] { it.jj->finish(it.jw, jouts[m], jfl[2 * m], jfl[2 * m + 1], join_c0_of[k]); }))
          rel_free(ctx_, jouts[m]);
      }
    });
    for (PlannedQuery* q : run) {
      ++q->next;
      if (q->out->status != VG_OK || q->next >= q->plan->jobNum()) done.push_back(q);
    }
    prof.finish_s += since(t0);
  }
  if (!done.empty()) {
    auto t0 = Clock::now();
    finalize(done, completed);
    prof.final_s += since(t0);
  }
  for (PlannedQuery* q : done) q->retired = true;
  std::vector<PlannedQuery*> still;
  for (PlannedQuery* q : active_)
    if (!q->retired) still.push_back(q);
  active_.swap(still);
}

// Projection and the final adjacent-unique pass (QueryPlan::execute, after
// its job loop) of every query that just finished, in one batched launch.
void WaveEngine::finalize(std::vector<PlannedQuery*>& done, std::vector<PlannedQuery*>& completed) {
  // 1. projection and output buffers, per query on the host pool
  std::vector<SegRows> seg(done.size());
  std::vector<vedas::FullRelationIR*> res(done.size(), nullptr);
  pfor(done.size(), [&](size_t k) {
    PlannedQuery* q = done[k];
    BatchQuery* out = q->out;
    if (out->status != VG_OK || !q->plan) return;
    guarded(out, [&] {
      vedas::FullRelationIR* r = q->plan->project();
      SegRows& s = seg[k];
      s.ncols = static_cast<uint32_t>(r->getColumnNum());
      s.n = r->size();
      for (uint32_t c = 0; c < s.ncols; ++c) {
        s.in[c] = r->getRelationRawPointer(c);
        s.out[c] = ctx_.alloc<uint32_t>(s.n);
      }
      res[k] = r;
    });
  });
  // 2. one batched adjacent-unique pass over all of them
  std::vector<SegRows> fin;
  std::vector<size_t> who;
  for (size_t k = 0; k < done.size(); ++k)
    if (res[k]) {
      fin.push_back(seg[k]);
      who.push_back(k);
    }
  std::vector<uint64_t> kept = batched_unique(ctx_, fin);
  std::vector<uint64_t> kept_of(done.size(), 0);
  for (size_t m = 0; m < who.size(); ++m) kept_of[who[m]] = kept[m];
  // 3. results handed over, intermediates freed, per query on the host pool
  pfor(done.size(), [&](size_t k) {
    PlannedQuery* q = done[k];
    BatchQuery* out = q->out;
    if (vedas::FullRelationIR* r = res[k]) {
      for (size_t c = 0; c < r->getColumnNum(); ++c) out->headers.push_back(r->getHeader(c));
      Rel in = r->release();
      rel_free(ctx_, in);
      Rel o;
      o.ncols = seg[k].ncols;
      o.nrows = kept_of[k];
      for (uint32_t c = 0; c < o.ncols; ++c) {
        o.cols[c] = seg[k].out[c];
        ctx_.arena.shrink(o.cols[c], o.nrows * sizeof(uint32_t));
      }
      out->rel = o;
    }
    if (q->ex) out->log = std::move(q->ex->exe_log);
    q->plan.reset();  // frees every intermediate relation of the query
  });
  for (PlannedQuery* q : done) completed.push_back(q);
}

void run_batch(Ctx& ctx, vedas::VedasStorage* storage, const std::vector<std::string>& texts, BatchResult& out) {
  auto t_all = Clock::now();
  out.ctx = &ctx;
  out.queries.clear();
  out.queries.resize(texts.size());
  prepare_mirrors(storage);
  std::vector<PlannedQuery> pq(texts.size());
  auto t0 = Clock::now();
  pfor(texts.size(), [&](size_t i) {
    pq[i].out = &out.queries[i];
    plan_query(ctx, storage, texts[i], pq[i]);
  });
  WaveEngine eng(ctx);
  eng.prof.plan_s = since(t0);
  for (auto& q : pq) eng.add(&q);
  std::vector<PlannedQuery*> completed;
  while (eng.active() > 0) eng.wave(completed);
  out.waves = eng.waves();
  out.prof = eng.prof;
  ctx.check_device_errors();
  out.prof.total_s = since(t_all);
}

}  // namespace vg
