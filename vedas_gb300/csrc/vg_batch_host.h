#pragma once

#include <chrono>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "compat/vedas_compat.h"
#include "vg_batch.h"
#include "vg_pool.h"
#include "vg_relops.h"

namespace vg {

struct BatchQuery {
  vg_status status = VG_OK;
  std::string error;
  std::vector<std::string> headers;
  Rel rel;
  std::vector<vedas::ExecuteLogRecord> log;
  const uint32_t* host[VG_MAX_COLS] = {nullptr};   // page-locked copies (HostResults)
};

// Page-locked host copies of finished queries' results, made while the batch
// runs: each time queries finish, one copy kernel on a second stream packs
// their columns straight into page-locked host memory (which kernels address
// directly under unified addressing), so the transfers overlap the rest of
// the batch and need no device staging.  Chunks of page-locked memory come
// from the context's pool and go back to it with the HostResults.
class HostResults {
 public:
  explicit HostResults(Ctx& ctx) : ctx_(ctx) {}
  ~HostResults();
  HostResults(const HostResults&) = delete;
  HostResults& operator=(const HostResults&) = delete;
  // Enqueues the copies of these queries' result columns on the download
  // stream, after the work already on the calling thread's stream; false
  // when there was nothing to copy.
  bool add(const std::vector<BatchQuery*>& qs);
  // Waits for every copy.
  void finish();
  uint64_t bytes() const { return bytes_; }

 private:
  struct Chunk {
    char* p;
    size_t cap, used;
  };
  struct Pending {
    std::vector<void*> scratch;   // device blocks of the copy, freed once it is done
    cudaEvent_t done;
  };
  Ctx& ctx_;
  std::mutex mu_;   // add() is called by both engines of a batch
  std::vector<Chunk> chunks_;
  std::vector<Pending> pending_;
  uint64_t bytes_ = 0;
  void retire_stages(bool all);
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
};

// Plans one query on the host (thread-safe across queries once the storage's
// host mirrors exist: see prepare_mirrors).  Errors go to pq.out.
void plan_query(Ctx& ctx, vedas::VedasStorage* storage, const char* text, PlannedQuery& pq);
// Destroys the host state of finished queries (plans with their jobs and
// intermediate relations, parsed queries, executors) on idle host workers
// (post_background); the vectors are left empty.  Device memory goes back to
// the arena when a worker gets to it: drain_background() waits for that.
void release_later(std::vector<std::unique_ptr<vedas::QueryPlan>>& plans);
void release_later(std::vector<PlannedQuery>& pq);
// Wave engines of one run_batch, each on its own host thread with its own
// share of the host worker threads (VG_BATCH_ENGINES, 1..8; default 4).
size_t batch_engines();
// Wave engines of a server (VG_SERVE_ENGINES, 1-8, default 1).
size_t serve_engines();
// Runs f on the calling thread with engine e's share of the host threads as
// the pool of its parallel loops (as a batch's engine thread e does).
void run_on_engine_pool(size_t e, const std::function<void()>& f);
// Bytes of the region in which each of `engines` wave engines places its join
// outputs on the device (0: no region).
size_t join_region_bytes(const Ctx& ctx, size_t engines);
// Whether the wave engines of a batch run on streams of their own
// (VG_ENGINE_STREAMS=0 puts them all on the context's stream).
bool engine_streams();
void prepare_mirrors(vedas::VedasStorage* storage);

// Advances every added query by one job per wave; the device work of a wave
// is issued as batched launches.  A wave has two stages:
//  A: finish the previous wave's jobs on the host, prepare every query's next
//     job, and enqueue the first device half (sorts, select copies, join
//     counts and scans, and the final compaction of queries that just
//     finished);
//  B: wait for that half, hand finished queries back, allocate the join
//     outputs and enqueue the join writes.
// Nothing else waits on the device.  Several engines on one stream, each
// driven by its own host thread with its own worker pool, keep the device
// busy with one engine's work while the host runs the others' stages.
class WaveEngine {
 public:
  // key_bits bounds every relation value (< 2^key_bits), so the segmented
  // sorts run without a host round trip; 0 when unknown.
  explicit WaveEngine(Ctx& ctx, int key_bits = 0);
  ~WaveEngine();
  WaveEngine(const WaveEngine&) = delete;
  WaveEngine& operator=(const WaveEngine&) = delete;
  void add(PlannedQuery* pq);
  // Queries added and not yet handed back (waiting, in flight or finishing).
  size_t active() const { return active_.size() + run_.size() + final_.size(); }
  // Forgets every query in flight (after a device-level failure).
  void reset();
  // Stage A then stage B.
  void wave(std::vector<PlannedQuery*>& completed) {
    stage_a(completed);
    stage_b(completed);
  }
  // The next stage (A and B alternate).
  void step(std::vector<PlannedQuery*>& completed);
  // Copies each finished query's result to the host as it finishes.
  void set_host_results(HostResults* h) { host_ = h; }
  // Places the join outputs of every wave on the device, in a region of
  // `bytes` of the arena (when one is free), so that a wave's join write
  // follows its count without a host round trip; outputs that do not fit
  // are written after one, as without a region.
  void use_region(size_t bytes);
  // Issues the engine's work on a stream of its own (after everything on the
  // context's stream), with its frees held back until its stream has passed
  // the blocks' last use.  finish_stream waits for that stream.
  void use_own_stream();
  void finish_stream();
  // Destroys the plans of handed-back queries that are still pending.
  void bury();
  uint32_t waves() const { return waves_; }
  BatchProfile prof;

  // Per-stage timeline, kept when tracing is on (VG_WAVE_TRACE names a file
  // that run_batch appends it to): seconds since the batch started at the
  // stage's start, after its wait for the device, and at its end, with the
  // stage's work.
  struct Trace {
    char stage;              // 'A' or 'B'
    double t0, t_wait, t_end;
    uint32_t items, joins, sorted_rels;
    uint64_t join_left_rows, join_out_rows;
    // host seconds of the stage's parts (stage A): finishing the previous
    // wave, preparing the next jobs, projections, and enqueueing the sorts,
    // the select copies, the joins and the final compaction
    double h_finish, h_prepare, h_final, h_sort, h_copy, h_join, h_unique;
  };
  bool tracing = false;
  std::chrono::steady_clock::time_point trace_origin;
  std::vector<Trace> trace;

  // Host state of one job of the wave in flight.
  struct Item {
    enum Kind { kNone, kSelect, kJoin, kSwap } kind = kNone;
    vedas::SelectWork sw;
    vedas::JoinQueryJob* jj = nullptr;
    vedas::JoinWork jw;
    vedas::IndexSwapJob* xj = nullptr;
    vedas::FullRelationIR* xir = nullptr;
    int64_t join = -1;                  // index among the wave's joins
    std::vector<uint32_t> c0;           // staged column 0 (small swapped relations, small join outputs)
    bool has_c0 = false;
  };

 private:
  void stage_a(std::vector<PlannedQuery*>& completed);
  void stage_b(std::vector<PlannedQuery*>& completed);
  void finish_wave();
  void retire_failed(PlannedQuery* q, std::vector<PlannedQuery*>& completed);

  Ctx& ctx_;
  int key_bits_ = 0;
  HostResults* host_ = nullptr;
  uint32_t waves_ = 0;
  bool next_is_a_ = true;
  std::vector<PlannedQuery*> active_;   // queries waiting for their next job
  // the wave in flight
  std::vector<PlannedQuery*> run_;
  std::vector<Item> items_;
  std::vector<size_t> swap_small_;      // items whose swapped relation stages column 0
  std::vector<size_t> joins_;           // items with a join, in batch order
  std::vector<size_t> jsmall_;          // joins (by batch index) whose small output stages column 0
  JoinBatch jb_;
  std::vector<Rel> jouts_;
  // queries whose last job finished: compacted in stage A, handed back in stage B
  std::vector<PlannedQuery*> final_;
  std::vector<std::unique_ptr<vedas::QueryPlan>> graveyard_;   // handed to release_later by bury()
  std::vector<SegRows> fin_seg_;
  std::vector<vedas::FullRelationIR*> fin_res_;
  // device -> host results of each stage and the events that mark them
  PinnedWords h_a_{ctx_}, h_b_{ctx_};
  size_t off_tot_ = 0, off_fin_ = 0, off_c0_ = 0, off_err_ = 0;   // words into h_a_
  size_t off_fla_ = 0, off_bump_ = 0, off_c0a_ = 0;               // words into h_a_ (placed joins)
  size_t off_fl_ = 0, off_jc0_ = 0;                               // words into h_b_
  // the engine's own stream and its held-back frees (use_own_stream)
  cudaStream_t own_stream_ = nullptr;
  DeferredFrees defer_;
  ThreadExec exec();           // the engine's stream, frees at once
  ThreadExec enqueue_exec();   // the engine's stream, frees held back
  // device-side placement of join outputs (use_region)
  Arena::Region* region_ = nullptr;
  uint64_t* d_bump_ = nullptr;     // device: region bytes handed out
  uint64_t region_bump_ = 0;       // the same on the host, as of the last wave read back
  bool placed_wave_ = false;       // the wave in flight placed its joins on the device
  std::vector<int32_t> c0_slot_;   // per join of the wave: its small column-0 slot, or -1
  std::vector<uint8_t> placed_;    // per join: written by the device-side placement
  std::vector<uint32_t> jfl_;      // per join: first and last key of the output
  cudaEvent_t ev_a_ = nullptr, ev_b_ = nullptr;
  bool a_pending_ = false, b_pending_ = false;
};

struct BatchResult {
  Ctx* ctx = nullptr;
  std::vector<BatchQuery> queries;
  uint32_t waves = 0;
  BatchProfile prof;
  std::unique_ptr<HostResults> host;   // with run_batch(..., to_host)
  // Releases results, headers and logs on the worker pool (one thread when
  // serial: a queued release runs on one idle worker).
  bool serial = false;
  ~BatchResult();
};

// Bits that hold every id of the storage's index (for WaveEngine's key_bits).
int key_bits_for(vedas::VedasStorage* storage);

// Host-only self-check of the worker pools: `pools` caller threads, each
// with its own pool of `threads` threads, run `loops` parallel loops of
// random sizes and queue work between them.  Returns the number of items
// that did not run exactly once plus queued tasks that never ran (0 when
// correct).
uint64_t selfcheck_pools(unsigned pools, unsigned threads, unsigned loops);

// Runs every query to completion together; per-query failures are recorded
// in their BatchQuery and do not stop the others.
// With to_host, every result is also copied to page-locked host memory
// while the batch runs (BatchQuery::host).  texts[i] is query i's text (a
// null pointer reads as an empty query); the texts are read during the call.
void run_batch(Ctx& ctx, vedas::VedasStorage* storage, const char* const* texts, size_t n, BatchResult& out,
               bool to_host = false);

}  // namespace vg
