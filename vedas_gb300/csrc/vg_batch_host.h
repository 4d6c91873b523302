#pragma once

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

struct BatchResult {
  Ctx* ctx = nullptr;
  std::vector<BatchQuery> queries;
  uint32_t waves = 0;
  ~BatchResult();
};

// Runs every query to completion together; per-query failures are recorded
// in their BatchQuery and do not stop the others.
void run_batch(Ctx& ctx, vedas::VedasStorage* storage, const std::vector<std::string>& texts,
               BatchResult& out);

}  // namespace vg
