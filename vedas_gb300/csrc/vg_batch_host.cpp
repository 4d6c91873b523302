// Batched multi-query execution.
//
// Every query keeps the reference's own plan and job semantics (the host
// mirror in compat/).  Queries advance in waves, one job per query per wave,
// so each query still sees its jobs strictly in plan order (its bounds and
// empty intervals flow from job to job exactly as in QueryPlan::execute).
// Within a wave the device work of all queries is issued together: one
// segmented stable sort for every index swap and implicit join re-sort, one
// copy launch and one unique launch for every select, and one count / scan /
// write chain for every join.  Host planning of the queries runs on a thread
// pool.
#include "vg_batch_host.h"

#include <algorithm>
#include <atomic>
#include <thread>

#include "vg_batch.h"

namespace vg {

namespace {

template <typename F>
void parallel_for(size_t n, F&& f) {
  unsigned hw = std::thread::hardware_concurrency();
  unsigned nt = hw ? std::min<unsigned>(hw, 32) : 4;
  if (n < 64 || nt <= 1) {
    for (size_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&] {
      for (size_t i = next.fetch_add(1); i < n; i = next.fetch_add(1)) f(i);
    });
  for (auto& t : th) t.join();
}

template <typename F>
bool guarded(BatchQuery& q, F&& f) {
  try {
    f();
    return true;
  } catch (const Error& e) {
    q.status = e.status;
    q.error = e.what();
  } catch (const std::exception& e) {
    q.status = VG_ERR_INVALID;
    q.error = e.what();
  }
  return false;
}

}  // namespace

BatchResult::~BatchResult() {
  if (ctx)
    for (auto& q : queries) rel_free(*ctx, q.rel);
}

void run_batch(Ctx& ctx, vedas::VedasStorage* storage, const std::vector<std::string>& texts, BatchResult& out) {
  out.ctx = &ctx;
  out.queries.clear();
  out.queries.resize(texts.size());
  // Host mirrors are created lazily; make them all before planning in parallel.
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

  std::vector<std::unique_ptr<vedas::QueryExecutor>> ex(texts.size());
  std::vector<std::unique_ptr<vedas::SparqlQuery>> sq(texts.size());
  std::vector<std::unique_ptr<vedas::QueryPlan>> plan(texts.size());
  std::vector<size_t> next(texts.size(), 0);

  // Planning (pre-scan, QueryGraph, job list) is host-only: run it in parallel.
  parallel_for(texts.size(), [&](size_t i) {
    BatchQuery& q = out.queries[i];
    guarded(q, [&] {
      ex[i] = std::make_unique<vedas::QueryExecutor>(storage, &ctx);
      sq[i] = std::make_unique<vedas::SparqlQuery>(texts[i].c_str());
      std::set<std::string> sel = sq[i]->getSelectedVariables();
      plan[i] = std::make_unique<vedas::QueryPlan>(sel);
      ex[i]->plan(*sq[i], *plan[i]);
      plan[i]->beginExecution();
    });
  });

  out.waves = 0;
  while (true) {
    std::vector<size_t> active;
    for (size_t i = 0; i < texts.size(); ++i)
      if (out.queries[i].status == VG_OK && plan[i] && next[i] < plan[i]->jobNum()) active.push_back(i);
    if (active.empty()) break;
    ++out.waves;

    struct SelectItem { size_t q; vedas::SelectWork w; };
    struct JoinItem { size_t q; vedas::JoinQueryJob* job; vedas::JoinWork w; };
    struct SwapItem { size_t q; vedas::IndexSwapJob* job; vedas::FullRelationIR* ir; };
    std::vector<SelectItem> sels;
    std::vector<JoinItem> joins;
    std::vector<SwapItem> swaps;
    for (size_t i : active) {
      vedas::QueryJob* job = plan[i]->getJob(next[i]);
      BatchQuery& q = out.queries[i];
      guarded(q, [&] {
        if (auto* s = dynamic_cast<vedas::SelectQueryJob*>(job)) {
          SelectItem it{i, {}};
          s->prepare(it.w);
          sels.push_back(std::move(it));
        } else if (auto* j = dynamic_cast<vedas::JoinQueryJob*>(job)) {
          JoinItem it{i, j, {}};
          j->prepare(it.w);
          if (!it.w.empty) joins.push_back(it);
        } else if (auto* w = dynamic_cast<vedas::IndexSwapJob*>(job)) {
          swaps.push_back({i, w, w->prepare()});
        } else {
          job->startJob(0);  // transfer: a pass-through on one device
        }
      });
    }

    // 1. every stable re-sort by column 0 of this wave in one segmented sort
    std::vector<Rel*> to_sort;
    for (auto& it : joins) {
      if (it.w.sortL) to_sort.push_back(&it.w.lir->rel());
      if (it.w.sortR) to_sort.push_back(&it.w.rir->rel());
    }
    for (auto& it : swaps) to_sort.push_back(&it.ir->rel());
    batched_sort_by_first(ctx, to_sort);

    // 2. index swaps: empty-interval scans need column 0 of small relations
    {
      std::vector<const Rel*> small;
      std::vector<size_t> who;
      for (size_t k = 0; k < swaps.size(); ++k)
        if (swaps[k].ir->size() > 2 && swaps[k].ir->size() < 100) {
          small.push_back(&swaps[k].ir->rel());
          who.push_back(k);
        }
      std::vector<std::vector<uint32_t>> c0;
      batched_col0(ctx, small, c0);
      std::vector<const std::vector<uint32_t>*> per(swaps.size(), nullptr);
      for (size_t m = 0; m < who.size(); ++m) per[who[m]] = &c0[m];
      for (size_t k = 0; k < swaps.size(); ++k)
        guarded(out.queries[swaps[k].q], [&] { swaps[k].job->finish(per[k]); });
    }

    // 3. selects: all copies in one launch, all unique compactions in one
    {
      std::vector<CopyPiece> pieces;
      std::vector<SegRows> useg;
      std::vector<size_t> uwho;
      for (size_t k = 0; k < sels.size(); ++k) {
        auto& w = sels[k].w;
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
      batched_copy(ctx, pieces);
      std::vector<uint64_t> kept = batched_unique(ctx, useg);
      for (size_t m = 0; m < uwho.size(); ++m) vedas::SelectQueryJob::finishUnique(sels[uwho[m]].w, kept[m]);
    }

    // 4. joins: one count / scan / write chain for all of them
    if (!joins.empty()) {
      std::vector<const Rel*> L, R;
      for (auto& it : joins) {
        L.push_back(&it.w.lir->rel());
        R.push_back(&it.w.rir->rel());
      }
      std::vector<Rel> outs;
      std::vector<uint32_t> fl;
      batched_join(ctx, L, R, outs, fl);
      std::vector<const Rel*> small;
      std::vector<size_t> who;
      for (size_t k = 0; k < joins.size(); ++k)
        if (!joins[k].job->isLastJoinForVar() && outs[k].nrows > 2 && outs[k].nrows < 100) {
          small.push_back(&outs[k]);
          who.push_back(k);
        }
      std::vector<std::vector<uint32_t>> c0;
      batched_col0(ctx, small, c0);
      std::vector<const std::vector<uint32_t>*> per(joins.size(), nullptr);
      for (size_t m = 0; m < who.size(); ++m) per[who[m]] = &c0[m];
      for (size_t k = 0; k < joins.size(); ++k) {
        BatchQuery& q = out.queries[joins[k].q];
        if (!guarded(q, [&] { joins[k].job->finish(joins[k].w, outs[k], fl[2 * k], fl[2 * k + 1], per[k]); }))
          rel_free(ctx, outs[k]);
      }
    }
    for (size_t i : active) ++next[i];
  }

  // Projection and the final adjacent-unique pass of every query at once.
  std::vector<SegRows> fin;
  std::vector<size_t> fwho;
  std::vector<vedas::FullRelationIR*> fres;
  for (size_t i = 0; i < texts.size(); ++i) {
    BatchQuery& q = out.queries[i];
    if (q.status != VG_OK || !plan[i]) continue;
    guarded(q, [&] {
      vedas::FullRelationIR* res = plan[i]->project();
      SegRows s;
      s.ncols = static_cast<uint32_t>(res->getColumnNum());
      s.n = res->size();
      for (uint32_t c = 0; c < s.ncols; ++c) {
        s.in[c] = res->getRelationRawPointer(c);
        s.out[c] = ctx.alloc<uint32_t>(s.n);
      }
      fin.push_back(s);
      fwho.push_back(i);
      fres.push_back(res);
    });
  }
  std::vector<uint64_t> kept = batched_unique(ctx, fin);
  for (size_t m = 0; m < fwho.size(); ++m) {
    BatchQuery& q = out.queries[fwho[m]];
    vedas::FullRelationIR* res = fres[m];
    for (size_t c = 0; c < res->getColumnNum(); ++c) q.headers.push_back(res->getHeader(c));
    Rel r = res->release();
    rel_free(ctx, r);
    Rel o;
    o.ncols = fin[m].ncols;
    o.nrows = kept[m];
    for (uint32_t c = 0; c < o.ncols; ++c) {
      o.cols[c] = fin[m].out[c];
      ctx.arena.shrink(o.cols[c], o.nrows * sizeof(uint32_t));
    }
    q.rel = o;
    q.log = ex[fwho[m]]->exe_log;
  }
  for (size_t i = 0; i < texts.size(); ++i) {
    BatchQuery& q = out.queries[i];
    if (q.status != VG_OK && ex[i]) q.log = ex[i]->exe_log;
  }
  plan.clear();  // frees every intermediate relation
  ctx.check_device_errors();
}

}  // namespace vg
