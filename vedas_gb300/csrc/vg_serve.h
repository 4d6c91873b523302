// Serving loop: continuous batching over the wave engine.
//
// Clients submit query text from any thread; the query is planned on the
// caller's thread (host work only) and queued.  One worker thread owns the
// device: before every wave it admits queued queries, first come first
// served, while the sum of their estimated relation bytes and the bytes of
// finished results not yet released stays within the budget (with nothing in
// flight the head of the queue is admitted whenever its own estimate fits, so
// a client holding results cannot stall the queue for good); then it runs one
// wave for everything in flight, so queries that
// arrived while others were on the GPU join them at the next wave boundary
// and their work shares the same batched launches.  Finished queries release
// their reservation and wake their waiters.  Results are read on a separate
// stream, so a download does not wait for the worker's next wave.
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
  bool done = false;
};

class Server {
 public:
  Server(Ctx& ctx, vedas::VedasStorage* st, uint64_t budget)
      : ctx_(ctx), st_(st), budget_(budget), eng_(ctx, key_bits_for(st)) {
    prepare_mirrors(st_);
    VG_CUDA(cudaStreamCreateWithFlags(&dl_stream_, cudaStreamNonBlocking));
    worker_ = std::thread([this] { loop(); });
  }

  ~Server() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_work_.notify_all();
    if (worker_.joinable()) worker_.join();
    for (auto& kv : items_) rel_free(ctx_, kv.second->q.rel);
    if (dl_stream_) cudaStreamDestroy(dl_stream_);
  }

  uint64_t submit(const char* text) {
    uint64_t t = 0;
    submit_many(&text, 1, &t);
    return t;
  }

  // Plans n queries (host only; on the worker pool when there are many,
  // otherwise on the caller's thread) and queues them in order.
  void submit_many(const char* const* texts, size_t n, uint64_t* tickets) {
    std::vector<std::unique_ptr<ServeItem>> its(n);
    const auto now = Clock::now();
    for (size_t i = 0; i < n; ++i) {
      its[i] = std::make_unique<ServeItem>();
      its[i]->t_submit = now;
      its[i]->pq.out = &its[i]->q;
    }
    parallel_for(n, [&](size_t i) { plan_query(ctx_, st_, texts[i] ? texts[i] : "", its[i]->pq); });
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

  void stats(uint64_t out[6]) {
    std::lock_guard<std::mutex> lk(mu_);
    out[0] = submitted_;
    out[1] = completed_;
    out[2] = rejected_;
    out[3] = eng_.waves();
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
  WaveEngine eng_;
  cudaStream_t dl_stream_ = nullptr;
  std::thread worker_;
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
  std::deque<ServeItem*> queue_;
  std::unordered_map<uint64_t, std::unique_ptr<ServeItem>> items_;
  std::unordered_map<PlannedQuery*, ServeItem*> inflight_;
  uint64_t next_ticket_ = 0, submitted_ = 0, completed_ = 0, rejected_ = 0, reserved_ = 0, peak_inflight_ = 0;
  uint64_t held_ = 0;   // bytes of finished results not yet released
  bool stop_ = false;
  vg_status worker_status_ = VG_OK;

  ServeItem* find_locked(uint64_t ticket) {
    auto f = items_.find(ticket);
    if (f == items_.end()) fail(VG_ERR_INVALID, "unknown ticket");
    return f->second.get();
  }

  static uint64_t result_bytes(const Rel& r) { return 4ull * r.nrows * r.ncols; }

  void finish_locked(ServeItem* it) {
    it->done = true;
    it->t_done = Clock::now();
    cv_done_.notify_all();
  }

  void loop() {
    while (true) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_work_.wait(lk, [&] { return stop_ || !queue_.empty() || eng_.active() > 0; });
        if (stop_ && eng_.active() == 0) return;
        // admission at the wave boundary, first come first served
        while (!queue_.empty() && (reserved_ + held_ + queue_.front()->pq.est_bytes <= budget_ ||
                                   (eng_.active() == 0 && reserved_ == 0))) {
          ServeItem* it = queue_.front();
          queue_.pop_front();
          reserved_ += it->pq.est_bytes;
          it->t_admit = Clock::now();
          inflight_[&it->pq] = it;
          eng_.add(&it->pq);
        }
        if (eng_.active() > peak_inflight_) peak_inflight_ = eng_.active();
      }
      if (eng_.active() == 0) continue;
      std::vector<PlannedQuery*> completed;
      try {
        eng_.wave(completed);
        if (eng_.active() == 0) eng_.bury();   // idle: free finished queries' intermediates now
      } catch (const Error& e) {
        // a device-level failure ends every query in flight with its status
        std::lock_guard<std::mutex> lk(mu_);
        worker_status_ = e.status;
        for (auto& kv : inflight_) {
          kv.second->q.status = e.status;
          kv.second->q.error = e.what();
        }
        std::vector<PlannedQuery*> all;
        for (auto& kv : inflight_) all.push_back(kv.first);
        completed = all;
        for (PlannedQuery* pq : all) pq->plan.reset();
        eng_.reset();
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
    }
  }
};

}  // namespace vg
