#pragma once

#include <chrono>
#include <memory>
#include <string>
#include <vector>

#include "compat/vedas_compat.h"
#include "vg_relops.h"

namespace vg {

struct BatchQuery {
  vg_status status = VG_OK;
  std::string error;
  std::vector<std::string> headers;
  Rel rel;
  std::vector<vedas::ExecuteLogRecord> log;
};

// Seconds spent in each part of a batched run.
struct BatchProfile {
  double plan_s = 0, prepare_s = 0, device_s = 0, finish_s = 0, final_s = 0, total_s = 0;
};

// One query in flight: the reference's plan and how far it has run.
struct PlannedQuery {
  std::unique_ptr<vedas::QueryExecutor> ex;
  std::unique_ptr<vedas::SparqlQuery> sq;
  std::unique_ptr<vedas::QueryPlan> plan;
  size_t next = 0;
  uint64_t est_bytes = 0;   // estimated HBM for its relations (admission)
  BatchQuery* out = nullptr;
  bool retired = false;     // handed back by the wave engine
};

// Plans one query on the host (thread-safe across queries once the storage's
// host mirrors exist: see prepare_mirrors).  Errors go to pq.out.
void plan_query(Ctx& ctx, vedas::VedasStorage* storage, const std::string& text, PlannedQuery& pq);
void prepare_mirrors(vedas::VedasStorage* storage);

// Advances every added query by one job per wave; the device work of a wave
// is issued as batched launches.  Queries that finish (or fail) are projected,
// de-duplicated in one batched pass, have their intermediates freed and are
// handed back.
class WaveEngine {
 public:
  explicit WaveEngine(Ctx& ctx) : ctx_(ctx) {}
  void add(PlannedQuery* pq);
  size_t active() const { return active_.size(); }
  // Forgets every query in flight (after a device-level failure).
  void reset() { active_.clear(); }
  void wave(std::vector<PlannedQuery*>& completed);
  uint32_t waves() const { return waves_; }
  BatchProfile prof;

 private:
  Ctx& ctx_;
  std::vector<PlannedQuery*> active_;
  uint32_t waves_ = 0;
  void finalize(std::vector<PlannedQuery*>& done, std::vector<PlannedQuery*>& completed);
};

struct BatchResult {
  Ctx* ctx = nullptr;
  std::vector<BatchQuery> queries;
  uint32_t waves = 0;
  BatchProfile prof;
  ~BatchResult();
};

// Runs every query to completion together; per-query failures are recorded
// in their BatchQuery and do not stop the others.
void run_batch(Ctx& ctx, vedas::VedasStorage* storage, const std::vector<std::string>& texts,
               BatchResult& out);

}  // namespace vg
