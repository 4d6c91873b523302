// The C-ABI (include/vedas_gb300.h): status codes at the boundary, no
// exceptions across it.
#include <chrono>
#include <cstring>
#include <memory>
#include <string>

#include "compat/vedas_compat.h"
#include "vg_batch.h"
#include "vg_batch_host.h"
#include "vg_ingest.h"
#include "vg_selfcheck.h"
#include "vg_ctx.h"
#include "vg_serve.h"
#include "vg_index.h"
#include "vg_relops.h"

struct vg_ctx {
  vg::Ctx c;
};

struct vg_index {
  vg_ctx* ctx = nullptr;
  std::unique_ptr<vedas::VedasStorage> st;
  std::unique_ptr<vg::DictResolver> resolver;   // set by vg_index_set_dict
};

struct vg_batch {
  vg::BatchResult r;
};

struct vg_dict {
  vg::Dict d;
};

struct vg_server {
  std::unique_ptr<vg::Server> srv;
};

struct vg_result {
  vg_ctx* ctx = nullptr;
  vg::Rel rel;
  std::vector<std::string> headers;
  std::vector<vedas::ExecuteLogRecord> log;
  ~vg_result() {
    if (ctx) vg::rel_free(ctx->c, rel);
  }
};

namespace {

thread_local std::string g_last_error;

template <typename F>
vg_status guard(F&& f) {
  try {
    f();
    return VG_OK;
  } catch (const vg::Error& e) {
    g_last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return VG_ERR_OOM;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return VG_ERR_INVALID;
  }
}

vg::Rel to_rel(const vg_ir* ir) {
  vg::Rel r;
  r.ncols = ir->ncols;
  r.nrows = ir->nrows;
  for (uint32_t c = 0; c < ir->ncols && c < VG_MAX_COLS; ++c) r.cols[c] = ir->cols[c];
  return r;
}

void from_rel(const vg::Rel& r, vg_ir* ir) {
  std::memset(ir, 0, sizeof(*ir));
  ir->ncols = r.ncols;
  ir->nrows = r.nrows;
  for (uint32_t c = 0; c < r.ncols; ++c) ir->cols[c] = r.cols[c];
}

void check_ir(const vg_ir* ir) {
  if (!ir || ir->ncols == 0 || ir->ncols > VG_MAX_COLS) vg::fail(VG_ERR_INVALID, "bad relation");
}

}  // namespace

extern "C" {

const char* vg_status_string(vg_status s) {
  switch (s) {
    case VG_OK: return "ok";
    case VG_ERR_INVALID: return "invalid argument";
    case VG_ERR_OOM: return "out of memory";
    case VG_ERR_CUDA: return "CUDA error";
    case VG_ERR_TIMEOUT: return "bounded device wait expired";
    case VG_ERR_UNSUPPORTED: return "unsupported input";
    case VG_ERR_PARSE: return "query parse error";
    case VG_ERR_OVERFLOW: return "size limit exceeded";
    case VG_ERR_REJECTED: return "admission rejected";
  }
  return "unknown status";
}

const char* vg_last_error(void) { return g_last_error.c_str(); }

vg_status vg_ctx_create(int device, size_t arena_bytes, vg_ctx** out) {
  if (!out) return VG_ERR_INVALID;
  *out = nullptr;
  auto h = std::make_unique<vg_ctx>();
  vg_status st = guard([&] {
    vg::Ctx& c = h->c;
    c.device = device;
    VG_CUDA(cudaSetDevice(device));
    VG_CUDA(cudaStreamCreateWithFlags(&c.stream.main, cudaStreamNonBlocking));
    VG_CUDA(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, device));
    if (arena_bytes == 0) {
      size_t fr = 0, tot = 0;
      VG_CUDA(cudaMemGetInfo(&fr, &tot));
      arena_bytes = fr / 10 * 9;
    }
    c.arena.init(arena_bytes);
    VG_CUDA(cudaMalloc(&c.d_err, sizeof(vg::DeviceErrors)));
    VG_CUDA(cudaMemset(c.d_err, 0, sizeof(vg::DeviceErrors)));
    VG_CUDA(cudaMallocHost(&c.h_small, vg::Ctx::kSmallWords * sizeof(uint64_t)));
  });
  if (st != VG_OK) {
    vg_ctx_destroy(h.release());
    return st;
  }
  *out = h.release();
  return VG_OK;
}

vg_status vg_ctx_destroy(vg_ctx* ctx) {
  if (!ctx) return VG_OK;
  vg::Ctx& c = ctx->c;
  // queued releases of finished queries free into this context's arena
  guard([] { vg::drain_background(); });
  if (c.stream.main) cudaStreamSynchronize(c.stream.main);
  c.release_dl_stream();
  c.release_pinned();
  c.release_upload_ring();
  c.arena.release();
  if (c.d_err) cudaFree(c.d_err);
  if (c.h_small) cudaFreeHost(c.h_small);
  if (c.stream.main) cudaStreamDestroy(c.stream.main);
  delete ctx;
  return VG_OK;
}

vg_status vg_ctx_memory(vg_ctx* ctx, size_t* used, size_t* peak, size_t* capacity) {
  if (!ctx) return VG_ERR_INVALID;
  const vg_status st = guard([] { vg::drain_background(); });
  if (st != VG_OK) return st;
  if (used) *used = ctx->c.arena.used();
  if (peak) *peak = ctx->c.arena.peak();
  if (capacity) *capacity = ctx->c.arena.capacity();
  return VG_OK;
}

vg_status vg_ctx_sync(vg_ctx* ctx) {
  if (!ctx) return VG_ERR_INVALID;
  return guard([&] { ctx->c.sync(); });
}

void* vg_ctx_stream(vg_ctx* ctx) { return ctx ? static_cast<void*>(ctx->c.stream.main) : nullptr; }

vg_status vg_stats_reset(vg_ctx* ctx, int timing) {
  if (!ctx) return VG_ERR_INVALID;
  return guard([&] {
    ctx->c.reset_stats();
    ctx->c.timing = timing != 0;
  });
}

uint32_t vg_stats_count(vg_ctx* ctx) { return ctx ? static_cast<uint32_t>(ctx->c.kstats.size()) : 0; }

uint64_t vg_stats_launches(vg_ctx* ctx) { return ctx ? ctx->c.launches : 0; }

vg_status vg_stats_get(vg_ctx* ctx, uint32_t i, const char** name, uint64_t* launches, double* bytes,
                       double* ms) {
  if (!ctx || i >= ctx->c.kstats.size()) return VG_ERR_INVALID;
  return guard([&] {
    ctx->c.collect_timing();
    auto it = ctx->c.kstats.begin();
    std::advance(it, i);
    if (name) *name = it->first.c_str();
    if (launches) *launches = it->second.launches;
    if (bytes) *bytes = it->second.bytes;
    if (ms) *ms = it->second.ms;
  });
}

vg_status vg_index_build(vg_ctx* ctx, const uint32_t* s, const uint32_t* p, const uint32_t* o, uint64_t n,
                         int full_index, int inputs_on_device, vg_index** out) {
  if (!ctx || !out || (n && (!s || !p || !o))) return VG_ERR_INVALID;
  *out = nullptr;
  auto h = std::make_unique<vg_index>();
  h->ctx = ctx;
  vg_status st = guard([&] {
    h->st = std::make_unique<vedas::VedasStorage>(&ctx->c, s, p, o, n, inputs_on_device != 0, full_index != 0);
    ctx->c.check_device_errors();
  });
  if (st == VG_OK) *out = h.release();
  return st;
}

vg_status vg_index_free(vg_index* ix) {
  if (!ix) return VG_OK;
  vg_status st = guard([&] {
    vg::drain_background();
    ix->ctx->c.sync();
    ix->st.reset();
  });
  delete ix;
  return st;
}

vg_status vg_index_array(vg_index* ix, const char* name, const uint32_t** dev, const uint32_t** host,
                         uint64_t* len) {
  if (!ix || !name) return VG_ERR_INVALID;
  return guard([&] {
    vg::Index& I = ix->st->index();
    if (!I.dev.count(name)) vg::fail(VG_ERR_INVALID, std::string("no index array ") + name);
    const vg::DevArray& d = I.get(name);
    if (dev) *dev = d.ptr;
    if (len) *len = d.len;
    if (host) *host = I.host_array(name).data();
  });
}

vg_status vg_index_write(vg_index* ix, const char* path) {
  if (!ix || !path) return VG_ERR_INVALID;
  return guard([&] { ix->st->write(path); });
}

vg_status vg_index_open(vg_ctx* ctx, const char* path, int full_index, vg_index** out) {
  if (!ctx || !path || !out) return VG_ERR_INVALID;
  *out = nullptr;
  auto h = std::make_unique<vg_index>();
  h->ctx = ctx;
  vg_status st = guard([&] { h->st = std::make_unique<vedas::VedasStorage>(&ctx->c, path, full_index != 0); });
  if (st == VG_OK) *out = h.release();
  return st;
}

vg_status vg_ir_alloc(vg_ctx* ctx, uint32_t ncols, uint64_t nrows, vg_ir* out) {
  if (!ctx || !out || ncols == 0 || ncols > VG_MAX_COLS) return VG_ERR_INVALID;
  return guard([&] { from_rel(vg::rel_alloc(ctx->c, ncols, nrows), out); });
}

vg_status vg_ir_free(vg_ctx* ctx, vg_ir* ir) {
  if (!ctx || !ir) return VG_ERR_INVALID;
  return guard([&] {
    vg::Rel r = to_rel(ir);
    vg::rel_free(ctx->c, r);
    std::memset(ir, 0, sizeof(*ir));
  });
}

vg_status vg_ir_upload(vg_ctx* ctx, vg_ir* ir, uint32_t col, const uint32_t* host, uint64_t n) {
  if (!ctx || !ir || col >= ir->ncols || n > ir->nrows || (n && !host)) return VG_ERR_INVALID;
  return guard([&] {
    if (n) VG_CUDA(cudaMemcpyAsync(ir->cols[col], host, n * 4, cudaMemcpyHostToDevice, ctx->c.stream));
    ctx->c.sync();
  });
}

vg_status vg_ir_download(vg_ctx* ctx, const vg_ir* ir, uint32_t col, uint32_t* host) {
  if (!ctx || !ir || col >= ir->ncols || (ir->nrows && !host)) return VG_ERR_INVALID;
  return guard([&] { vg::download(ctx->c, ir->cols[col], ir->nrows, host); });
}

vg_status vg_select(vg_ctx* ctx, vg_index* ix, const vg_select_desc* d, vg_ir* out, uint32_t bu[3]) {
  if (!ctx || !ix || !d || !out || d->kind < 1 || d->kind > 3) return VG_ERR_INVALID;
  return guard([&] {
    vedas::QueryExecutor ex(ix->st.get(), &ctx->c);
    const std::string v0 = "?v0", v1 = "?v1";
    if (d->has_bound) ex.variables_bound[v0] = {d->bound_lo, d->bound_hi};
    if (d->eif[0] || d->eif[1] || d->eif[2] || d->eif[3])
      ex.empty_interval_dict.updateBound(v0, d->eif[0], d->eif[1], d->eif[2], d->eif[3]);
    std::unique_ptr<vedas::SelectQueryJob> job;
    if (d->kind == 3)
      job.reset(new vedas::SelectQueryJob(&ex, d->index_pos != 0, v0, v1, d->pred, d->second_used != 0));
    else
      job.reset(new vedas::SelectQueryJob(&ex, d->kind == 1, v0, d->pred, d->constant));
    job->startJob(0);
    auto* ir = dynamic_cast<vedas::FullRelationIR*>(job->getIR());
    vg::Rel r = ir->release();
    vg::rel_own(ctx->c, r);   // the caller owns (and frees) every column
    from_rel(r, out);
    if (bu) {
      bu[2] = 0;
      if (d->has_bound && d->kind != 3) {
        bu[0] = ex.variables_bound[v0].first;
        bu[1] = ex.variables_bound[v0].second;
        bu[2] = 1;
      }
    }
    ctx->c.sync();
  });
}

vg_status vg_join(vg_ctx* ctx, const vg_ir* l, const vg_ir* r, vg_ir* out, uint32_t first_last[2]) {
  if (!ctx || !out) return VG_ERR_INVALID;
  return guard([&] {
    check_ir(l);
    check_ir(r);
    vg::Rel o;
    vg::join(ctx->c, to_rel(l), to_rel(r), false, o);
    from_rel(o, out);
    if (first_last && o.nrows > 0) {
      VG_CUDA(cudaMemcpyAsync(&first_last[0], o.cols[0], 4, cudaMemcpyDeviceToHost, ctx->c.stream));
      VG_CUDA(cudaMemcpyAsync(&first_last[1], o.cols[0] + o.nrows - 1, 4, cudaMemcpyDeviceToHost, ctx->c.stream));
    }
    ctx->c.check_device_errors();
  });
}

vg_status vg_join2(vg_ctx* ctx, const vg_ir* l, const vg_ir* r, vg_ir* out) {
  if (!ctx || !out) return VG_ERR_INVALID;
  return guard([&] {
    check_ir(l);
    check_ir(r);
    vg::Rel o;
    vg::join(ctx->c, to_rel(l), to_rel(r), true, o);
    from_rel(o, out);
    ctx->c.check_device_errors();
  });
}

vg_status vg_swap(vg_ctx* ctx, vg_ir* ir, uint32_t col) {
  if (!ctx || !ir || col >= ir->ncols) return VG_ERR_INVALID;
  return guard([&] {
    vg::Rel r = to_rel(ir);
    std::swap(r.cols[0], r.cols[col]);
    vg::sort_by_first(ctx->c, r);
    from_rel(r, ir);
    ctx->c.check_device_errors();
  });
}

vg_status vg_sort_rows(vg_ctx* ctx, vg_ir* ir) {
  if (!ctx || !ir) return VG_ERR_INVALID;
  return guard([&] {
    check_ir(ir);
    vg::Rel r = to_rel(ir);
    vg::sort_rows(ctx->c, r);
    from_rel(r, ir);
    ctx->c.check_device_errors();
  });
}

vg_status vg_unique(vg_ctx* ctx, vg_ir* ir) {
  if (!ctx || !ir) return VG_ERR_INVALID;
  return guard([&] {
    check_ir(ir);
    vg::Rel r = to_rel(ir);
    vg::unique_in_place(ctx->c, r);
    from_rel(r, ir);
  });
}

vg_status vg_eif_scan(vg_ctx* ctx, const vg_ir* ir, uint64_t out4[4]) {
  if (!ctx || !ir || !out4 || ir->ncols == 0 || ir->nrows <= 2 || ir->nrows >= 100) return VG_ERR_INVALID;
  return guard([&] {
    std::vector<uint32_t> c0(ir->nrows);
    vg::download(ctx->c, ir->cols[0], ir->nrows, c0.data());
    size_t b[4];
    vedas::QueryExecutor::eifBounds(c0.data(), c0.size(), b);
    for (int i = 0; i < 4; ++i) out4[i] = b[i];
  });
}

vg_status vg_query(vg_ctx* ctx, vg_index* ix, const char* sparql, vg_result** out) {
  if (!ctx || !ix || !sparql || !out) return VG_ERR_INVALID;
  *out = nullptr;
  auto res = std::make_unique<vg_result>();
  vg_status st = guard([&] {
    vedas::QueryExecutor ex(ix->st.get(), &ctx->c);
    vedas::SparqlQuery sq(sparql, ix->st->resolver());
    std::set<std::string> sel = sq.getSelectedVariables();
    vedas::QueryPlan plan(sel);
    ex.plan(sq, plan);
    vedas::SparqlResult sr;
    plan.execute(sr);
    vedas::FullRelationIR* ir = sr.getResultIR();
    for (size_t c = 0; c < ir->getColumnNum(); ++c) res->headers.push_back(ir->getHeader(c));
    res->rel = ir->release();
    vg::rel_own(ctx->c, res->rel);   // a result never refers to index memory
    res->ctx = ctx;
    res->log = ex.exe_log;
    ctx->c.check_device_errors();
  });
  if (st == VG_OK) *out = res.release();
  return st;
}

uint32_t vg_result_ncols(const vg_result* r) { return r ? static_cast<uint32_t>(r->headers.size()) : 0; }
uint64_t vg_result_nrows(const vg_result* r) { return r ? r->rel.nrows : 0; }
const char* vg_result_header(const vg_result* r, uint32_t c) {
  return (r && c < r->headers.size()) ? r->headers[c].c_str() : nullptr;
}
const uint32_t* vg_result_column_device(const vg_result* r, uint32_t c) {
  return (r && c < r->rel.ncols) ? r->rel.cols[c] : nullptr;
}
vg_status vg_result_download(const vg_result* r, uint32_t c, uint32_t* host) {
  if (!r || c >= r->rel.ncols) return VG_ERR_INVALID;
  return guard([&] { vg::download(r->ctx->c, r->rel.cols[c], r->rel.nrows, host); });
}
uint32_t vg_result_nlog(const vg_result* r) { return r ? static_cast<uint32_t>(r->log.size()) : 0; }
void vg_result_log(const vg_result* r, uint32_t i, uint32_t* op, uint64_t* p1, uint64_t* p2, uint64_t* p3) {
  if (!r || i >= r->log.size()) return;
  const auto& l = r->log[i];
  if (op) *op = static_cast<uint32_t>(l.op);
  if (p1) *p1 = l.param1;
  if (p2) *p2 = l.param2;
  if (p3) *p3 = l.param3;
}
vg_status vg_result_free(vg_result* r) {
  delete r;
  return VG_OK;
}

namespace {
// name -> (field, smallest value, largest value, value list: 0 for a range)
struct TuneKnob {
  const char* name;
  uint32_t vg::TuneParams::*field;
  uint32_t lo, hi;
};
const TuneKnob kKnobs[] = {
    {"sort_items", &vg::TuneParams::sort_items, 8, 16},
    {"sort_lookback", &vg::TuneParams::sort_lookback, 1, 4},
    {"join_small_rows", &vg::TuneParams::join_small_rows, 0, 256},
    {"write_small_rows", &vg::TuneParams::write_small_rows, 0, 4096},
    {"unique_small_rows", &vg::TuneParams::unique_small_rows, 0, 256},
    {"write_blocks_per_sm", &vg::TuneParams::write_blocks_per_sm, 1, 8},
};
const TuneKnob* find_knob(const char* name) {
  if (!name) return nullptr;
  for (const TuneKnob& k : kKnobs)
    if (std::strcmp(k.name, name) == 0) return &k;
  return nullptr;
}
}  // namespace

vg_status vg_tune_set(vg_ctx* ctx, const char* name, int64_t value) {
  const TuneKnob* k = find_knob(name);
  if (!ctx || !k || value < static_cast<int64_t>(k->lo) || value > static_cast<int64_t>(k->hi)) return VG_ERR_INVALID;
  if (k->field == &vg::TuneParams::sort_items && value != 8 && value != 12 && value != 16) return VG_ERR_INVALID;
  if (k->field == &vg::TuneParams::sort_lookback && value != 1 && value != 4) return VG_ERR_INVALID;
  ctx->c.tune.*(k->field) = static_cast<uint32_t>(value);
  return VG_OK;
}

vg_status vg_tune_get(vg_ctx* ctx, const char* name, int64_t* value) {
  const TuneKnob* k = find_knob(name);
  if (!ctx || !k || !value) return VG_ERR_INVALID;
  *value = ctx->c.tune.*(k->field);
  return VG_OK;
}

vg_status vg_query_loop(vg_ctx* ctx, vg_index* ix, const char* const* queries, uint32_t nq, double* seconds,
                        uint64_t* rows, vg_status* status) {
  if (!ctx || !ix || (nq && !queries)) return VG_ERR_INVALID;
  for (uint32_t i = 0; i < nq; ++i) {
    const auto t0 = std::chrono::steady_clock::now();
    vg_result* r = nullptr;
    const vg_status st = queries[i] ? vg_query(ctx, ix, queries[i], &r) : VG_ERR_INVALID;
    const uint64_t n = r ? r->rel.nrows : 0;
    if (r) vg_result_free(r);
    if (seconds) seconds[i] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rows) rows[i] = n;
    if (status) status[i] = st;
  }
  return VG_OK;
}

namespace {
int describe(vedas::PlanTreeNode* n, vedas::SparqlQuery& sq, std::string& out, int& counter) {
  if (!n) return -1;
  int a = -1, b = -1;
  if (n->child1) a = describe(n->child1, sq, out, counter);
  if (n->child2) b = describe(n->child2, sq, out, counter);
  if (n->op == vedas::UPLOAD) {
    std::string idx = "-";
    if (n->tp->getVariableNum() == 2) idx = (n->tp->getSubject() == n->var) ? "PSO" : "POS";
    out += "U" + std::to_string(n->tp->getId()) + ":" + idx + ";";
  } else if (n->op == vedas::JOIN) {
    out += "J" + std::to_string(a) + "," + std::to_string(b) + ":" + n->var + ":" + (n->reuseVar ? "0" : "1") + ";";
  } else {
    out += "W" + std::to_string(a) + ":" + n->var + ";";
  }
  return counter++;
}
}  // namespace

vg_status vg_plan_describe(const char* sparql, const uint64_t* est, uint32_t n, char* buf, size_t cap) {
  if (!sparql || !buf || (n && !est)) return VG_ERR_INVALID;
  return guard([&] {
    vedas::SparqlQuery sq(sparql);
    for (uint32_t i = 0; i < n && i < sq.getPatternNum(); ++i) sq.getPatternPtr(i)->estimate_rows = est[i];
    vedas::QueryGraph qg(&sq);
    vedas::PlanTreeNode* root = qg.generateQueryPlan();
    std::string s;
    int counter = 0;
    describe(root, sq, s, counter);
    if (s.size() + 1 > cap) vg::fail(VG_ERR_OVERFLOW, "plan text exceeds the buffer");
    std::memcpy(buf, s.c_str(), s.size() + 1);
  });
}

vg_status vg_eid_sequence(const uint64_t* quads, uint32_t n, uint64_t out4[4]) {
  if ((n && !quads) || !out4 || n == 0) return VG_ERR_INVALID;
  return guard([&] {
    vedas::EmptyIntervalDict d;
    for (uint32_t i = 0; i < n; ++i)
      d.updateBound("?x", quads[4 * i], quads[4 * i + 1], quads[4 * i + 2], quads[4 * i + 3]);
    vedas::VAR_BOUND v = d.getBound("?x");
    out4[0] = std::get<0>(v);
    out4[1] = std::get<1>(v);
    out4[2] = std::get<2>(v);
    out4[3] = std::get<3>(v);
  });
}

namespace {
vg_status batch_run(vg_ctx* ctx, vg_index* ix, const char* const* queries, uint32_t nq, bool to_host,
                    vg_batch** out) {
  if (!ctx || !ix || !out || (nq && !queries)) return VG_ERR_INVALID;
  *out = nullptr;
  auto b = std::make_unique<vg_batch>();
  vg_status st = guard([&] { vg::run_batch(ctx->c, ix->st.get(), queries, nq, b->r, to_host); });
  if (st == VG_OK) *out = b.release();
  return st;
}
}  // namespace

vg_status vg_batch_run(vg_ctx* ctx, vg_index* ix, const char* const* queries, uint32_t nq, vg_batch** out) {
  return batch_run(ctx, ix, queries, nq, false, out);
}

vg_status vg_batch_run_host(vg_ctx* ctx, vg_index* ix, const char* const* queries, uint32_t nq, vg_batch** out) {
  return batch_run(ctx, ix, queries, nq, true, out);
}

const uint32_t* vg_batch_host_column(const vg_batch* b, uint32_t q, uint32_t c) {
  if (!b || !b->r.host || q >= b->r.queries.size() || c >= b->r.queries[q].rel.ncols) return nullptr;
  return b->r.queries[q].host[c];
}

uint32_t vg_batch_size(const vg_batch* b) { return b ? static_cast<uint32_t>(b->r.queries.size()) : 0; }
uint32_t vg_batch_waves(const vg_batch* b) { return b ? b->r.waves : 0; }
vg_status vg_batch_profile(const vg_batch* b, double out6[6]) {
  if (!b || !out6) return VG_ERR_INVALID;
  const vg::BatchProfile& p = b->r.prof;
  out6[0] = p.plan_s;
  out6[1] = p.prepare_s;
  out6[2] = p.device_s;
  out6[3] = p.finish_s;
  out6[4] = p.final_s;
  out6[5] = p.total_s;
  return VG_OK;
}
vg_status vg_batch_query_status(const vg_batch* b, uint32_t q) {
  return (b && q < b->r.queries.size()) ? b->r.queries[q].status : VG_ERR_INVALID;
}
const char* vg_batch_query_error(const vg_batch* b, uint32_t q) {
  return (b && q < b->r.queries.size()) ? b->r.queries[q].error.c_str() : "";
}
uint32_t vg_batch_ncols(const vg_batch* b, uint32_t q) {
  return (b && q < b->r.queries.size()) ? static_cast<uint32_t>(b->r.queries[q].headers.size()) : 0;
}
uint64_t vg_batch_nrows(const vg_batch* b, uint32_t q) {
  return (b && q < b->r.queries.size()) ? b->r.queries[q].rel.nrows : 0;
}
vg_status vg_batch_rows(const vg_batch* b, uint64_t* nrows) {
  if (!b || (!nrows && !b->r.queries.empty())) return VG_ERR_INVALID;
  for (size_t q = 0; q < b->r.queries.size(); ++q) nrows[q] = b->r.queries[q].rel.nrows;
  return VG_OK;
}
const char* vg_batch_header(const vg_batch* b, uint32_t q, uint32_t c) {
  if (!b || q >= b->r.queries.size() || c >= b->r.queries[q].headers.size()) return nullptr;
  return b->r.queries[q].headers[c].c_str();
}
const uint32_t* vg_batch_column_device(const vg_batch* b, uint32_t q, uint32_t c) {
  if (!b || q >= b->r.queries.size() || c >= b->r.queries[q].rel.ncols) return nullptr;
  return b->r.queries[q].rel.cols[c];
}
vg_status vg_batch_download(const vg_batch* b, uint32_t q, uint32_t c, uint32_t* host) {
  if (!b || q >= b->r.queries.size() || c >= b->r.queries[q].rel.ncols) return VG_ERR_INVALID;
  return guard([&] {
    const vg::Rel& r = b->r.queries[q].rel;
    vg::download(*b->r.ctx, r.cols[c], r.nrows, host);
  });
}
uint64_t vg_batch_result_words(const vg_batch* b) {
  if (!b) return 0;
  uint64_t w = 0;
  for (const auto& q : b->r.queries) w += q.rel.nrows * q.rel.ncols;
  return w;
}

vg_status vg_batch_download_all(const vg_batch* b, uint32_t* host) {
  if (!b) return VG_ERR_INVALID;
  return guard([&] {
    vg::Ctx& ctx = *b->r.ctx;
    const uint64_t words = vg_batch_result_words(b);
    if (words == 0) return;
    if (!host) vg::fail(VG_ERR_INVALID, "null host buffer");
    vg::Scratch<uint32_t> stage(ctx, words);
    std::vector<vg::CopyPiece> pieces;
    uint64_t off = 0;
    for (const auto& q : b->r.queries)
      for (uint32_t c = 0; c < q.rel.ncols; ++c) {
        pieces.push_back({q.rel.cols[c], stage.get() + off, q.rel.nrows});
        off += q.rel.nrows;
      }
    vg::batched_copy(ctx, pieces);
    VG_CUDA(cudaMemcpyAsync(host, stage.get(), words * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
  });
}

uint32_t vg_batch_nlog(const vg_batch* b, uint32_t q) {
  return (b && q < b->r.queries.size()) ? static_cast<uint32_t>(b->r.queries[q].log.size()) : 0;
}
void vg_batch_log(const vg_batch* b, uint32_t q, uint32_t i, uint32_t* op, uint64_t* p1, uint64_t* p2,
                  uint64_t* p3) {
  if (!b || q >= b->r.queries.size() || i >= b->r.queries[q].log.size()) return;
  const auto& l = b->r.queries[q].log[i];
  if (op) *op = static_cast<uint32_t>(l.op);
  if (p1) *p1 = l.param1;
  if (p2) *p2 = l.param2;
  if (p3) *p3 = l.param3;
}
vg_status vg_batch_free(vg_batch* b) {
  if (!b) return VG_OK;
  // released by an idle host worker; the context drains such releases before
  // it is destroyed, before its memory statistics are read, and before its
  // arena reports that it is out of memory
  b->r.serial = true;
  return guard([&] {
    // the page-locked result copies go back to the context's pool at once,
    // so that the next batch reuses them instead of pinning new memory
    b->r.host.reset();
    vg::post_background([](void* p) { delete static_cast<vg_batch*>(p); }, b);
  });
}

vg_status vg_ingest_ntriples(vg_ctx* ctx, const char* text, uint64_t len, int literal_dict, uint32_t** s,
                             uint32_t** p, uint32_t** o, uint64_t* n, vg_dict** dict) {
  if (!ctx || (len && !text) || !s || !p || !o || !n || !dict) return VG_ERR_INVALID;
  *s = *p = *o = nullptr;
  *n = 0;
  *dict = nullptr;
  auto d = std::make_unique<vg_dict>();
  vg::Ingested in;
  vg_status st = guard([&] {
    vg::ingest_ntriples(ctx->c, text, len, literal_dict != 0, in);
    d->d = std::move(in.dict);
  });
  if (st != VG_OK) {
    if (in.s) ctx->c.free(in.s);
    if (in.p) ctx->c.free(in.p);
    if (in.o) ctx->c.free(in.o);
    return st;
  }
  *s = in.s;
  *p = in.p;
  *o = in.o;
  *n = in.n;
  *dict = d.release();
  return VG_OK;
}

vg_status vg_ingest_free(vg_ctx* ctx, uint32_t* s, uint32_t* p, uint32_t* o) {
  if (!ctx) return VG_ERR_INVALID;
  return guard([&] {
    ctx->c.free(s);
    ctx->c.free(p);
    ctx->c.free(o);
  });
}

uint64_t vg_dict_size(const vg_dict* d, int kind) {
  if (!d) return 0;
  return kind == 0 ? d->d.so.size() : kind == 1 ? d->d.p.size() : kind == 2 ? d->d.l.size() : 0;
}

const char* vg_dict_term(const vg_dict* d, int kind, uint32_t id) {
  if (!d) return nullptr;
  const std::string* t = d->d.term(kind, id);
  return t ? t->c_str() : nullptr;
}

uint32_t vg_dict_lookup(vg_dict* d, int kind, const char* term) {
  if (!d || !term) return 0;
  return d->d.lookup(kind, term);
}

vg_status vg_dict_write(const vg_dict* d, const char* path) {
  if (!d || !path) return VG_ERR_INVALID;
  return guard([&] { vg::write_vdd(d->d, path); });
}

vg_status vg_dict_open(const char* path, vg_dict** out) {
  if (!path || !out) return VG_ERR_INVALID;
  *out = nullptr;
  auto d = std::make_unique<vg_dict>();
  vg_status st = guard([&] { vg::read_vdd(path, d->d); });
  if (st == VG_OK) *out = d.release();
  return st;
}

namespace {
vg_status decode_into(const vg::Dict& d, const std::vector<const uint32_t*>& cols, uint64_t nrows, char* buf,
                      size_t cap, size_t* needed) {
  const std::string text = vg::decode_rows(d, cols, nrows);
  if (needed) *needed = text.size() + 1;
  if (!buf || cap < text.size() + 1) return VG_ERR_OVERFLOW;
  std::memcpy(buf, text.c_str(), text.size() + 1);
  return VG_OK;
}

// The result columns of a relation in host memory.
std::vector<std::vector<uint32_t>> host_columns(vg::Ctx& ctx, const vg::Rel& r) {
  std::vector<std::vector<uint32_t>> h(r.ncols);
  for (uint32_t c = 0; c < r.ncols; ++c) {
    h[c].resize(r.nrows);
    if (r.nrows)
      VG_CUDA(cudaMemcpyAsync(h[c].data(), r.cols[c], r.nrows * 4, cudaMemcpyDeviceToHost, ctx.stream));
  }
  ctx.sync();
  return h;
}
}  // namespace

vg_status vg_result_decode(const vg_result* r, const vg_dict* d, char* buf, size_t cap, size_t* needed) {
  if (!r || !d) return VG_ERR_INVALID;
  vg_status st = VG_OK;
  vg_status g = guard([&] {
    auto h = host_columns(r->ctx->c, r->rel);
    std::vector<const uint32_t*> cols;
    for (auto& v : h) cols.push_back(v.data());
    st = decode_into(d->d, cols, r->rel.nrows, buf, cap, needed);
  });
  return g != VG_OK ? g : st;
}

vg_status vg_batch_decode(const vg_batch* b, uint32_t q, const vg_dict* d, char* buf, size_t cap, size_t* needed) {
  if (!b || !d || q >= b->r.queries.size()) return VG_ERR_INVALID;
  const vg::BatchQuery& bq = b->r.queries[q];
  if (bq.status != VG_OK) return bq.status;
  vg_status st = VG_OK;
  vg_status g = guard([&] {
    std::vector<std::vector<uint32_t>> h;
    std::vector<const uint32_t*> cols;
    if (b->r.host && (bq.rel.nrows == 0 || bq.host[0])) {
      for (uint32_t c = 0; c < bq.rel.ncols; ++c) cols.push_back(bq.host[c]);   // copies made during the batch
    } else {
      h = host_columns(*b->r.ctx, bq.rel);
      for (auto& v : h) cols.push_back(v.data());
    }
    st = decode_into(d->d, cols, bq.rel.nrows, buf, cap, needed);
  });
  return g != VG_OK ? g : st;
}

vg_status vg_index_set_dict(vg_index* ix, const vg_dict* d) {
  if (!ix) return VG_ERR_INVALID;
  return guard([&] {
    ix->st->setResolver(nullptr);
    ix->resolver.reset();
    if (d) {
      ix->resolver = std::make_unique<vg::DictResolver>(&d->d);
      ix->st->setResolver(ix->resolver.get());
    }
  });
}

vg_status vg_dict_free(vg_dict* d) {
  delete d;
  return VG_OK;
}

void vg_ingest_set_hash_bits(int bits) { vg::set_ingest_hash_bits(bits); }

vg_status vg_selfcheck_bounded_wait(vg_ctx* ctx, int which) {
  if (!ctx || which < 0 || which > 1) return VG_ERR_INVALID;
  return guard([&] { vg::selfcheck_bounded_wait(ctx->c, which); });
}

vg_status vg_selfcheck_l2_lookup(uint32_t seed, uint32_t graphs, uint32_t lookups, uint64_t* mismatches) {
  if (!mismatches) return VG_ERR_INVALID;
  return guard([&] { *mismatches = vedas::selfcheck_l2_lookup(seed, graphs, lookups); });
}

vg_status vg_selfcheck_pools(uint32_t pools, uint32_t threads, uint32_t loops, uint64_t* errors) {
  if (!errors || pools == 0 || pools > 16 || threads == 0 || threads > 32) return VG_ERR_INVALID;
  return guard([&] { *errors = vg::selfcheck_pools(pools, threads, loops); });
}

vg_status vg_serve_start(vg_ctx* ctx, vg_index* ix, size_t budget_bytes, vg_server** out) {
  if (!ctx || !ix || !out) return VG_ERR_INVALID;
  *out = nullptr;
  auto s = std::make_unique<vg_server>();
  vg_status st = guard([&] { s->srv = std::make_unique<vg::Server>(ctx->c, ix->st.get(), budget_bytes); });
  if (st == VG_OK) *out = s.release();
  return st;
}

vg_status vg_serve_submit(vg_server* s, const char* sparql, uint64_t* ticket) {
  if (!s || !sparql || !ticket) return VG_ERR_INVALID;
  return guard([&] { *ticket = s->srv->submit(sparql); });
}

vg_status vg_serve_submit_many(vg_server* s, const char* const* sparql, uint32_t n, uint64_t* tickets) {
  if (!s || (n && (!sparql || !tickets))) return VG_ERR_INVALID;
  return guard([&] { s->srv->submit_many(sparql, n, tickets); });
}

vg_status vg_serve_wait(vg_server* s, uint64_t ticket, double timeout_s, int* done) {
  if (!s || !done) return VG_ERR_INVALID;
  return guard([&] { *done = s->srv->wait(ticket, timeout_s) ? 1 : 0; });
}

vg_status vg_serve_query_status(vg_server* s, uint64_t ticket) {
  if (!s) return VG_ERR_INVALID;
  vg_status qs = VG_OK;
  vg_status st = guard([&] {
    vg::ServeItem* it = s->srv->get(ticket);
    if (!it->done) vg::fail(VG_ERR_INVALID, "query still running");
    qs = it->q.status;
    if (qs != VG_OK) g_last_error = it->q.error;
  });
  return st != VG_OK ? st : qs;
}

uint32_t vg_serve_ncols(vg_server* s, uint64_t ticket) {
  uint32_t n = 0;
  if (s) guard([&] { n = static_cast<uint32_t>(s->srv->get(ticket)->q.headers.size()); });
  return n;
}

uint64_t vg_serve_nrows(vg_server* s, uint64_t ticket) {
  uint64_t n = 0;
  if (s) guard([&] { n = s->srv->get(ticket)->q.rel.nrows; });
  return n;
}

const char* vg_serve_header(vg_server* s, uint64_t ticket, uint32_t c) {
  const char* h = nullptr;
  if (s)
    guard([&] {
      vg::ServeItem* it = s->srv->get(ticket);
      if (c < it->q.headers.size()) h = it->q.headers[c].c_str();
    });
  return h;
}

vg_status vg_serve_download(vg_server* s, uint64_t ticket, uint32_t c, uint32_t* host) {
  if (!s) return VG_ERR_INVALID;
  return guard([&] { s->srv->download(ticket, c, host); });
}

vg_status vg_serve_latency(vg_server* s, uint64_t ticket, double* queued_s, double* total_s) {
  if (!s) return VG_ERR_INVALID;
  return guard([&] {
    vg::ServeItem* it = s->srv->get(ticket);
    if (!it->done) vg::fail(VG_ERR_INVALID, "query still running");
    const bool admitted = it->t_admit.time_since_epoch().count() != 0;
    if (queued_s)
      *queued_s = admitted ? std::chrono::duration<double>(it->t_admit - it->t_submit).count() : 0.0;
    if (total_s) *total_s = std::chrono::duration<double>(it->t_done - it->t_submit).count();
  });
}

vg_status vg_serve_release(vg_server* s, uint64_t ticket) {
  if (!s) return VG_ERR_INVALID;
  return guard([&] { s->srv->release(ticket); });
}

vg_status vg_serve_set_queue_limit(vg_server* s, double seconds) {
  if (!s || !(seconds >= 0)) return VG_ERR_INVALID;
  return guard([&] { s->srv->set_queue_limit(seconds); });
}

vg_status vg_serve_stats(vg_server* s, uint64_t out6[6]) {
  if (!s || !out6) return VG_ERR_INVALID;
  return guard([&] { s->srv->stats(out6); });
}

vg_status vg_serve_stop(vg_server* s) {
  if (!s) return VG_OK;
  vg_status st = guard([&] { s->srv.reset(); });
  delete s;
  return st;
}

}  // extern "C"
