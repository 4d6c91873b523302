// Serving loop: continuous batching over wave engines.
//
// Clients submit query text from any thread; the query is planned on the
// caller's thread (host work only) and queued.  Each of the server's wave
// engines (VG_SERVE_ENGINES, default 1) has a worker thread, a stream and a
// join-output region of its own.  Before each of its waves a worker admits
// queued queries into its engine, first come first served, while the sum of
// the estimated relation bytes of every query in flight and the bytes of
// finished results not yet released stays within the budget (with nothing
// in flight anywhere the head of the queue is admitted whenever its own
// estimate fits, so a client holding results cannot stall the queue for
// good); then it runs one wave for everything its engine holds, so queries
// that arrived while others were on the GPU join them at the next wave
// boundary and share its batched launches.  The engines' waves overlap on
// the device as in a batch.  A queue limit, when set, refuses the queries
// that waited longer than it before admission, and new ones while the head
// of the queue has waited half of it (load shedding: under overload the
// admitted ones keep their latency).  Finished queries release
// their reservation and wake their waiters.  Results are read on a separate
// stream, so a download does not wait for any engine's next wave.
#pragma once

#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "vg_batch_host.h"

namespace vg {
namespace {
using Clock = std::chrono::steady_clock;
}

struct ServeItem {
  uint64_t ticket = 0;
  PlannedQuery pq;
  BatchQuery q;
  Clock::time_point t_submit, t_admit, t_done;
  uint64_t held = 0;   // device bytes of the finished result until release
  size_t engine = 0;   // the engine that runs it
  bool done = false;
};

class Server {
 public:
  Server(Ctx& ctx, vedas::VedasStorage* st, uint64_t budget) : ctx_(ctx), st_(st), budget_(budget) {
    prepare_mirrors(st_);
    VG_CUDA(cudaStreamCreateWithFlags(&dl_stream_, cudaStreamNonBlocking));
    const size_t ne = serve_engines();
    const size_t region = join_region_bytes(ctx_, ne);
    const bool streams = engine_streams();
    for (size_t e = 0; e < ne; ++e) {
      eng_.push_back(std::make_unique<WaveEngine>(ctx_, key_bits_for(st_)));
      if (region) eng_.back()->use_region(region);
      if (streams) eng_.back()->use_own_stream();
    }
    // one engine works with the process-wide pool; several split the host
    // threads as a batch's engines do
    for (size_t e = 0; e < ne; ++e)
      workers_.emplace_back([this, e, ne] {
        if (ne > 1) run_on_engine_pool(e, [&] { loop(e); });
        else loop(e);
      });
  }

  ~Server() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_work_.notify_all();
    for (auto& w : workers_)
      if (w.joinable()) w.join();
    for (auto& e : eng_) e->finish_stream();
    eng_.clear();
    for (auto& kv : items_) rel_free(ctx_, kv.second->q.rel);
    if (dl_stream_) cudaStreamDestroy(dl_stream_);
  }

  uint64_t submit(const char* text) {
    uint64_t t = 0;
    submit_many(&text, 1, &t);
    return t;
  }

  // Plans n queries (host only; on the worker pool when there are many,
  // otherwise on the caller's thread) and queues them in order.  With a
  // queue limit, queries that arrive while the head of the queue has already
  // waited half the limit are refused at once, without planning: under
  // overload the planning of queries that would be shed costs the host time
  // the admitted ones need.
  void submit_many(const char* const* texts, size_t n, uint64_t* tickets) {
    std::vector<std::unique_ptr<ServeItem>> its(n);
    const auto now = Clock::now();
    for (size_t i = 0; i < n; ++i) {
      its[i] = std::make_unique<ServeItem>();
      its[i]->t_submit = now;
      its[i]->pq.out = &its[i]->q;
    }
    bool overloaded = false;
    {
      std::lock_guard<std::mutex> lk(mu_);
      shed_locked(now);
      overloaded = queue_limit_s_ > 0 && !queue_.empty() &&
                   std::chrono::duration<double>(now - queue_.front()->t_submit).count() > 0.5 * queue_limit_s_;
    }
    if (overloaded) {
      for (size_t i = 0; i < n; ++i) {
        its[i]->q.status = VG_ERR_REJECTED;
        its[i]->q.error = "the serving queue is past half its limit";
      }
    } else {
      parallel_for(n, [&](size_t i) { plan_query(ctx_, st_, texts[i] ? texts[i] : "", its[i]->pq); });
    }
    std::lock_guard<std::mutex> lk(mu_);
    for (size_t i = 0; i < n; ++i) {
      ServeItem* raw = its[i].get();
      raw->ticket = ++next_ticket_;
      tickets[i] = raw->ticket;
      ++submitted_;
      items_[raw->ticket] = std::move(its[i]);
      if (raw->q.status == VG_OK && raw->pq.est_bytes > budget_) {
        raw->q.status = VG_ERR_REJECTED;
        raw->q.error = "estimated relation bytes exceed the serving budget";
      }
      if (raw->q.status != VG_OK) {
        finish_locked(raw);
        ++rejected_;
      } else {
        queue_.push_back(raw);
      }
    }
    cv_work_.notify_all();
  }

  bool wait(uint64_t ticket, double timeout_s) {
    std::unique_lock<std::mutex> lk(mu_);
    ServeItem* it = find_locked(ticket);
    auto pred = [&] { return it->done; };
    if (timeout_s < 0) {
      cv_done_.wait(lk, pred);
      return true;
    }
    return cv_done_.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
  }

  ServeItem* get(uint64_t ticket) {
    std::lock_guard<std::mutex> lk(mu_);
    return find_locked(ticket);
  }

  void download(uint64_t ticket, uint32_t col, uint32_t* host) {
    ServeItem* it = get(ticket);
    if (!it->done || col >= it->q.rel.ncols) fail(VG_ERR_INVALID, "result not ready or no such column");
    const uint64_t n = it->q.rel.nrows;
    if (n) {
      VG_CUDA(cudaMemcpyAsync(host, it->q.rel.cols[col], n * 4, cudaMemcpyDeviceToHost, dl_stream_));
      VG_CUDA(cudaStreamSynchronize(dl_stream_));
    }
  }

  void release(uint64_t ticket) {
    std::unique_ptr<ServeItem> it;
    {
      std::lock_guard<std::mutex> lk(mu_);
      auto f = items_.find(ticket);
      if (f == items_.end()) fail(VG_ERR_INVALID, "unknown ticket");
      if (!f->second->done) fail(VG_ERR_INVALID, "query still running");
      it = std::move(f->second);
      items_.erase(f);
      held_ -= it->held;
    }
    rel_free(ctx_, it->q.rel);
    cv_work_.notify_all();   // admission may have waited for these bytes
  }

  // Queries that waited longer than `seconds` in the queue are refused
  // (VG_ERR_REJECTED) instead of admitted; 0 turns the limit off.
  void set_queue_limit(double seconds) {
    std::lock_guard<std::mutex> lk(mu_);
    queue_limit_s_ = seconds > 0 ? seconds : 0.0;
  }

  void stats(uint64_t out[6]) {
    std::lock_guard<std::mutex> lk(mu_);
    out[0] = submitted_;
    out[1] = completed_;
    out[2] = rejected_;
    uint64_t w = 0;
    for (auto& e : eng_) w += e->waves();
    out[3] = w;
    out[4] = reserved_;
    out[5] = peak_inflight_;
  }

  vg_status worker_status() {
    std::lock_guard<std::mutex> lk(mu_);
    return worker_status_;
  }

 private:
  Ctx& ctx_;
  vedas::VedasStorage* st_;
  uint64_t budget_;
  std::vector<std::unique_ptr<WaveEngine>> eng_;
  cudaStream_t dl_stream_ = nullptr;
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
  std::deque<ServeItem*> queue_;
  std::unordered_map<uint64_t, std::unique_ptr<ServeItem>> items_;
  std::unordered_map<PlannedQuery*, ServeItem*> inflight_;
  uint64_t next_ticket_ = 0, submitted_ = 0, completed_ = 0, rejected_ = 0, reserved_ = 0, peak_inflight_ = 0;
  uint64_t held_ = 0;   // bytes of finished results not yet released
  double queue_limit_s_ = 0.0;
  bool stop_ = false;
  vg_status worker_status_ = VG_OK;

  static uint64_t result_bytes(const Rel& r) { return 4ull * r.nrows * r.ncols; }

  ServeItem* find_locked(uint64_t ticket) {
    auto f = items_.find(ticket);
    if (f == items_.end()) fail(VG_ERR_INVALID, "unknown ticket");
    return f->second.get();
  }

  void finish_locked(ServeItem* it) {
    it->done = true;
    it->t_done = Clock::now();
    cv_done_.notify_all();
  }

  // Refuses queued queries past the queue limit (from the head: the queue
  // is in arrival order).
  void shed_locked(Clock::time_point now) {
    if (queue_limit_s_ <= 0) return;
    while (!queue_.empty() &&
           std::chrono::duration<double>(now - queue_.front()->t_submit).count() > queue_limit_s_) {
      ServeItem* it = queue_.front();
      queue_.pop_front();
      it->q.status = VG_ERR_REJECTED;
      it->q.error = "waited longer than the serving queue limit";
      ++rejected_;
      finish_locked(it);
    }
  }

  bool head_fits_locked() const {
    if (queue_.empty()) return false;
    return reserved_ + held_ + queue_.front()->pq.est_bytes <= budget_ || reserved_ == 0;
  }

  void loop(size_t e) {
    WaveEngine& eng = *eng_[e];
    while (true) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_work_.wait(lk, [&] {
          shed_locked(Clock::now());
          return stop_ || eng.active() > 0 || head_fits_locked();
        });
        if (stop_ && eng.active() == 0) return;
        // admission at the engine's wave boundary, first come first served
        while (head_fits_locked()) {
          ServeItem* it = queue_.front();
          queue_.pop_front();
          reserved_ += it->pq.est_bytes;
          it->t_admit = Clock::now();
          it->engine = e;
          inflight_[&it->pq] = it;
          eng.add(&it->pq);
        }
        if (inflight_.size() > peak_inflight_) peak_inflight_ = inflight_.size();
      }
      if (eng.active() == 0) continue;
      std::vector<PlannedQuery*> completed;
      try {
        eng.wave(completed);
        if (eng.active() == 0) eng.bury();   // idle: free finished queries' intermediates now
      } catch (const Error& err) {
        // a device-level failure ends every query in flight on this engine with its status
        try {
          eng.finish_stream();
        } catch (const Error&) {
          // the context itself failed: the status below says so
        }
        std::lock_guard<std::mutex> lk(mu_);
        worker_status_ = err.status;
        completed.clear();
        for (auto& kv : inflight_)
          if (kv.second->engine == e) {
            kv.second->q.status = err.status;
            kv.second->q.error = err.what();
            completed.push_back(kv.first);
          }
        for (PlannedQuery* pq : completed) pq->plan.reset();
        eng.reset();
      }
      std::lock_guard<std::mutex> lk(mu_);
      for (PlannedQuery* pq : completed) {
        auto f = inflight_.find(pq);
        if (f == inflight_.end()) continue;
        ServeItem* it = f->second;
        inflight_.erase(f);
        reserved_ -= it->pq.est_bytes;
        it->held = it->q.status == VG_OK ? result_bytes(it->q.rel) : 0;
        held_ += it->held;
        ++completed_;
        finish_locked(it);
      }
      if (!completed.empty()) cv_work_.notify_all();   // reservations went back
    }
  }
};

}  // namespace vg
