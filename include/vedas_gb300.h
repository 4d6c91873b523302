/* VEDAS GB300 query-execution core: C-ABI.
 *
 * Every entry point returns a vg_status and never throws.  Pointers are plain
 * host or device pointers as documented per call; sizes are element counts.
 * A vg_ctx owns one CUDA device, one stream and one HBM arena; calls on the
 * same context must not overlap (one host thread per context), matching the
 * reference's one-host-thread-per-GPU execution.
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the reference project).
 */
#ifndef VEDAS_GB300_H
#define VEDAS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum vg_status {
  VG_OK = 0,
  VG_ERR_INVALID = 1,      /* bad argument */
  VG_ERR_OOM = 2,          /* arena or host allocation failed */
  VG_ERR_CUDA = 3,         /* CUDA runtime error */
  VG_ERR_TIMEOUT = 4,      /* a bounded device wait expired */
  VG_ERR_UNSUPPORTED = 5,  /* input outside what this core implements */
  VG_ERR_PARSE = 6,        /* query text not understood */
  VG_ERR_OVERFLOW = 7,     /* an output exceeded its reservation or a size limit */
  VG_ERR_REJECTED = 8      /* serving: admission refused (memory budget) */
} vg_status;

/* Human-readable text of a status, and of the last error on this thread. */
const char* vg_status_string(vg_status s);
const char* vg_last_error(void);

/* ---- context ----------------------------------------------------------- */
typedef struct vg_ctx vg_ctx;

/* Creates a context on `device` with an HBM arena of `arena_bytes`
 * (0 = 90% of the device's free memory).  Replaces the per-column
 * thrust::device_vector allocations of FullRelationIR
 * (src/FullRelationIR.cu:19-31) with one up-front slab. */
vg_status vg_ctx_create(int device, size_t arena_bytes, vg_ctx** out);
/* Waits for the context's queued releases, then frees the context.  Indexes,
 * results, batches and servers made on it must be freed before. */
vg_status vg_ctx_destroy(vg_ctx* ctx);
/* Arena accounting: bytes in use, peak, capacity. */
vg_status vg_ctx_memory(vg_ctx* ctx, size_t* used, size_t* peak, size_t* capacity);
/* Blocks until all work queued on the context's stream is done. */
vg_status vg_ctx_sync(vg_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work after the core's. */
void* vg_ctx_stream(vg_ctx* ctx);

/* Kernel accounting (no reference counterpart; the reference has only
 * host-side chrono timers, src/QueryExecutor.h:60-77).  vg_stats_reset clears
 * the counters and turns per-launch CUDA-event timing on or off; the query
 * calls count every kernel launch with the algorithmic bytes it moves.
 * vg_stats_get synchronizes and reports kernel i of vg_stats_count. */
vg_status vg_stats_reset(vg_ctx* ctx, int timing);
uint32_t vg_stats_count(vg_ctx* ctx);
uint64_t vg_stats_launches(vg_ctx* ctx);
vg_status vg_stats_get(vg_ctx* ctx, uint32_t i, const char** name, uint64_t* launches, double* bytes,
                       double* ms);

/* Launch parameters of the context's kernels (no reference counterpart: the
 * reference's tile and block sizes are ModernGPU's and Thrust's built-in
 * ones).  Choices change speed only, never results:
 *   sort_items           radix-sort keys per thread, 8 or 16 (tile 2048 / 4096)
 *   join_small_rows      joins with at most this many left rows are counted
 *                        one per warp (0..256)
 *   write_small_rows     join outputs with at most this many rows (of joins
 *                        with at most 256 left rows) are written one per warp
 *                        (0..4096)
 *   unique_small_rows    final compactions of at most this many rows run one
 *                        per warp (0..256)
 *   write_blocks_per_sm  blocks per SM of a batched join write whose size is
 *                        only known on the device (1..8)
 * vedas_gb300.tune picks them from timed trials per GPU and workload shape.
 * VG_ERR_INVALID for an unknown name or a value out of range. */
vg_status vg_tune_set(vg_ctx* ctx, const char* name, int64_t value);
vg_status vg_tune_get(vg_ctx* ctx, const char* name, int64_t* value);

/* ---- index build (hot path a) ----------------------------------------- */
typedef struct vg_index vg_index;

/* Builds the permutation indexes from n dictionary-encoded triples.
 * Replaces VedasStorage::VedasStorage(RdfData&, bool preload, bool fullIndex)
 * (src/VedasStorage.cu:25-73; createIndex1Level :270-289, createIndex
 * :306-358).  s, p, o are HOST pointers when inputs_on_device == 0, device
 * pointers otherwise.  The index stays resident in HBM; host mirrors of the
 * arrays are made on first request (vg_index_array with a host pointer). */
vg_status vg_index_build(vg_ctx* ctx, const uint32_t* s, const uint32_t* p, const uint32_t* o,
                         uint64_t n, int full_index, int inputs_on_device, vg_index** out);
vg_status vg_index_free(vg_index* ix);
/* One array of the reference layout, by the VedasStorage member name:
 * p_idx_values, p_idx_offsets, ps_s_idx_values, ps_idx_offsets,
 * po_o_idx_values, po_idx_offsets, ps_data, po_data, pso_data, pos_data and,
 * with the full index, s_idx_values, s_idx_offsets, sp_p_idx_values,
 * sp_idx_offsets, so_o_idx_values, so_idx_offsets, o_idx_values,
 * o_idx_offsets, os_data, op_p_idx_values, op_idx_offsets, spo_data,
 * sop_data, ops_data, osp_data.  Replaces the VedasStorage getters
 * (src/VedasStorage.h:14-59).  `dev` receives the HBM copy; `host`, if
 * non-null, receives a host mirror (copied on first use). */
vg_status vg_index_array(vg_index* ix, const char* name, const uint32_t** dev,
                         const uint32_t** host, uint64_t* len);
/* Binary .vds file in the reference's layout: VedasStorage::write / open
 * (src/VedasStorage.cu:459-516). */
vg_status vg_index_write(vg_index* ix, const char* path);
vg_status vg_index_open(vg_ctx* ctx, const char* path, int full_index, vg_index** out);

/* ---- relations (FullRelationIR) ---------------------------------------- */
#define VG_MAX_COLS 9 /* FullRelationIR::sort supports up to 9 columns (src/FullRelationIR.cu:218-335) */

/* A relation of `ncols` uint32 device columns with `nrows` rows, column-major
 * (FullRelationIR, src/FullRelationIR.h:10-47).  Column memory comes from the
 * context arena. */
typedef struct vg_ir {
  uint32_t ncols;
  uint64_t nrows;
  uint32_t* cols[VG_MAX_COLS];
} vg_ir;

vg_status vg_ir_alloc(vg_ctx* ctx, uint32_t ncols, uint64_t nrows, vg_ir* out);
vg_status vg_ir_free(vg_ctx* ctx, vg_ir* ir);
/* Host <-> device column copies (FullRelationIR::setRelation,
 * src/FullRelationIR.cu:578-592, and the D2H of SparqlResult::printResult). */
vg_status vg_ir_upload(vg_ctx* ctx, vg_ir* ir, uint32_t col, const uint32_t* host, uint64_t n);
vg_status vg_ir_download(vg_ctx* ctx, const vg_ir* ir, uint32_t col, uint32_t* host);

/* ---- hot-path jobs ------------------------------------------------------ */

/* Select (hot path b): one triple pattern against the partial index.
 * Replaces SelectQueryJob::startJob (src/SelectQueryJob.cu:86-270).
 *  kind 1: one variable, subject (?s p o) -> POS index, output [?s]
 *  kind 2: one variable, object  (s p ?o) -> PSO index, output [?o]
 *  kind 3: two variables (?s p ?o), level-2 data ps_data / pso_data
 *          (index PSO) or po_data / pos_data (index POS)
 * bound_lo/hi: the variables_bound entry of the first output variable
 * (has_bound = 0 for none); eif[4]: its EmptyIntervalDict entry
 * (lb1, ub1, lb2, ub2).  second_used = 0 keeps only column 0, adjacent-unique.
 * On return out_bound_update[0..1] holds the (lo, hi) the reference passes
 * to updateBoundDict for one-variable selects (flag in out_bound_update[2]). */
typedef struct vg_select_desc {
  int kind;          /* 1, 2 or 3 */
  int index_pos;     /* kind 3: 0 = PSO, 1 = POS */
  uint32_t pred;     /* predicate id */
  uint32_t constant; /* kinds 1/2: the bound object / subject */
  int has_bound;
  uint32_t bound_lo, bound_hi;
  uint64_t eif[4];
  int second_used;
} vg_select_desc;
vg_status vg_select(vg_ctx* ctx, vg_index* ix, const vg_select_desc* d, vg_ir* out,
                    uint32_t out_bound_update[3]);

/* Join (hot path c): sorted inner join of l and r on column 0 of each (both
 * sorted ascending by column 0).  Output rows are ordered by left row, then
 * right row: column 0 = key, then l's columns 1.., then r's columns 1..
 * Replaces the inner join and gather of JoinQueryJob::join
 * (src/JoinQueryJob.cu:262-380; mgpu::inner_join semantics).
 * first_last receives out column 0's first and last value when rows > 0. */
vg_status vg_join(vg_ctx* ctx, const vg_ir* l, const vg_ir* r, vg_ir* out,
                  uint32_t first_last[2]);
/* The join above for callers that cannot allocate device memory: it takes
 * no vg_ctx and allocates nothing (no cudaMalloc, cudaFree or allocating
 * library call).  This entry point has no counterpart in the reference.
 * Hosts that have divided all HBM among their own pools, or serving threads
 * that may only launch work, cannot give the core an arena; this variant
 * keeps its scratch in a fixed file-scope device array instead, which caps
 * l_rows at 2,097,152 (larger inputs return VG_ERR_OVERFLOW) and costs about
 * 32 MiB on every GPU that loads the library, until the process exits.
 * Columns are device pointers, column 0 of each side its sorted join key;
 * out_cols are l_ncols + r_ncols - 1 caller-allocated device buffers of
 * out_capacity rows.  *out_rows receives the result row count; when it
 * exceeds out_capacity nothing is written and VG_ERR_OVERFLOW is returned.
 * Runs on `stream` (a cudaStream_t, 0 = default) and returns after the join
 * finished.  The first call on each device looks up the scratch address
 * (make it before any stream capture).  All calls share the scratch: calls
 * that overlap on the GPU race.  Errors are described by
 * vg_noalloc_last_error(). */
vg_status vg_join_noalloc(const uint32_t* const* l_cols, uint32_t l_ncols, uint64_t l_rows,
                          const uint32_t* const* r_cols, uint32_t r_ncols, uint64_t r_rows,
                          uint32_t* const* out_cols, uint64_t out_capacity, uint64_t* out_rows,
                          void* stream);
const char* vg_noalloc_last_error(void);

/* Two-variable join: keys are (column 0, column 1) of each side, both
 * sorted lexicographically by them; output column 0..1 = keys, then the
 * rest of l, then the rest of r (src/JoinQueryJob.cu:181-225, :360-377). */
vg_status vg_join2(vg_ctx* ctx, const vg_ir* l, const vg_ir* r, vg_ir* out);

/* Index swap (hot path d): stable re-sort of the relation by column `col`,
 * which becomes column 0 (swapColumn(0, col) + sortByFirstColumn;
 * src/IndexSwapJob.cu:28-63, src/FullRelationIR.cu:594-727).  In place. */
vg_status vg_swap(vg_ctx* ctx, vg_ir* ir, uint32_t col);
/* Full lexicographic sort over all columns (FullRelationIR::sort,
 * src/FullRelationIR.cu:218-336).  In place. */
vg_status vg_sort_rows(vg_ctx* ctx, vg_ir* ir);
/* Adjacent duplicate-row removal (FullRelationIR::removeDuplicate,
 * src/FullRelationIR.cu:338-522).  In place; nrows is updated. */
vg_status vg_unique(vg_ctx* ctx, vg_ir* ir);
/* Empty-interval scan of column 0 for relations with 2 < nrows < 100
 * (src/JoinQueryJob.cu:398-433, src/IndexSwapJob.cu:81-118): out4 receives
 * the four bounds passed to EmptyIntervalDict::updateBound. */
vg_status vg_eif_scan(vg_ctx* ctx, const vg_ir* ir, uint64_t out4[4]);

/* ---- whole queries ------------------------------------------------------ */
typedef struct vg_result vg_result;

/* Runs one SPARQL basic-graph-pattern query through the reference's planning
 * and job semantics on the device.  Replaces QueryExecutor::query
 * (src/QueryExecutor.cu:294-431) + QueryPlan::execute (src/QueryPlan.cu:114-257).
 * Query text: SELECT * | ?v ... WHERE { s p o . ... } with constants written
 * as <ID> or "ID". */
vg_status vg_query(vg_ctx* ctx, vg_index* ix, const char* sparql, vg_result** out);
uint32_t vg_result_ncols(const vg_result* r);
uint64_t vg_result_nrows(const vg_result* r);
const char* vg_result_header(const vg_result* r, uint32_t c);
/* Device pointer of a result column, and a D2H copy of it. */
const uint32_t* vg_result_column_device(const vg_result* r, uint32_t c);
vg_status vg_result_download(const vg_result* r, uint32_t c, uint32_t* host);
/* Execution log (QueryExecutor::exe_log, src/vedas.h:87-103): op 0 JOIN,
 * 1 UPLOAD, 2 SWAP with its three size parameters. */
uint32_t vg_result_nlog(const vg_result* r);
void vg_result_log(const vg_result* r, uint32_t i, uint32_t* op, uint64_t* p1, uint64_t* p2,
                   uint64_t* p3);
vg_status vg_result_free(vg_result* r);
/* The reference's one-query-at-a-time benchmark loop (vdBench,
 * src/VedasBench.cu:144-176) in C: for each query in order, vg_query then
 * vg_result_free, timed per query on the host clock.  seconds[i], rows[i]
 * and status[i] (each optional, nq entries) receive query i's wall time,
 * result rows and status; the call itself fails only on bad arguments. */
vg_status vg_query_loop(vg_ctx* ctx, vg_index* ix, const char* const* queries, uint32_t nq, double* seconds,
                        uint64_t* rows, vg_status* status);

/* ---- host planning logic (no device needed) ----------------------------- */
/* The job list QueryGraph::generateQueryPlan (src/QueryGraph.cu:64-74) and
 * QueryExecutor::postorderTraversal (src/QueryExecutor.cu:106-135) produce
 * for `sparql` when its patterns have the given estimate_rows, written to
 * buf as "U<pattern>:<PSO|POS|->;" selects, "J<left job>,<right job>:<var>:
 * <last join for var>;" joins and "W<job>:<var>;" index swaps. */
vg_status vg_plan_describe(const char* sparql, const uint64_t* estimate_rows, uint32_t npatterns, char* buf,
                           size_t cap);
/* EmptyIntervalDict::updateBound (src/EmptyIntervalDict.cu:33-106) applied
 * n times to one variable (quads: n x (lb1, ub1, lb2, ub2)); out4 receives
 * the variable's final entry. */
vg_status vg_eid_sequence(const uint64_t* quads, uint32_t n, uint64_t out4[4]);

/* ---- batched execution -------------------------------------------------- */
typedef struct vg_batch vg_batch;

/* Runs nq queries together.  Each query follows exactly the job sequence and
 * semantics of vg_query (QueryExecutor::query + QueryPlan::execute); queries
 * advance one job per wave and every wave's sorts, selects and joins run as
 * batched launches.  Replaces the reference's one-query-at-a-time loop
 * (vdBench, src/VedasBench.cu:144-176).  A query the core refuses gets its
 * own status; the others complete. */
vg_status vg_batch_run(vg_ctx* ctx, vg_index* ix, const char* const* queries, uint32_t nq,
                       vg_batch** out);
/* vg_batch_run, and every query's result columns are also copied to
 * page-locked host memory owned by the batch as the query finishes, on a
 * second stream, so the transfers overlap the rest of the batch.  The copies
 * are complete when the call returns; vg_batch_host_column gives them (valid
 * until vg_batch_free; vg_batch_nrows(b, q) words; NULL for a failed query).
 * The reference has no batched execution; this is the batch counterpart of
 * reading a SparqlResult on the host (src/SparqlResult.cu). */
vg_status vg_batch_run_host(vg_ctx* ctx, vg_index* ix, const char* const* queries, uint32_t nq,
                            vg_batch** out);
const uint32_t* vg_batch_host_column(const vg_batch* b, uint32_t q, uint32_t c);
uint32_t vg_batch_size(const vg_batch* b);
uint32_t vg_batch_waves(const vg_batch* b);
/* Seconds spent: out6 = {host planning, host job preparation, batched device
 * work (with its waits), host job completion, final de-duplication, total}. */
vg_status vg_batch_profile(const vg_batch* b, double out6[6]);
vg_status vg_batch_query_status(const vg_batch* b, uint32_t q);
const char* vg_batch_query_error(const vg_batch* b, uint32_t q);
uint32_t vg_batch_ncols(const vg_batch* b, uint32_t q);
uint64_t vg_batch_nrows(const vg_batch* b, uint32_t q);
/* Row counts of every query at once: nrows[q] for q < vg_batch_size(b). */
vg_status vg_batch_rows(const vg_batch* b, uint64_t* nrows);
const char* vg_batch_header(const vg_batch* b, uint32_t q, uint32_t c);
const uint32_t* vg_batch_column_device(const vg_batch* b, uint32_t q, uint32_t c);
vg_status vg_batch_download(const vg_batch* b, uint32_t q, uint32_t c, uint32_t* host);
/* All result columns of the batch in one device-to-host copy: query by
 * query, column by column, nrows words each; `host` holds
 * vg_batch_result_words(b) uint32 words (pinned memory is fastest). */
uint64_t vg_batch_result_words(const vg_batch* b);
vg_status vg_batch_download_all(const vg_batch* b, uint32_t* host);
uint32_t vg_batch_nlog(const vg_batch* b, uint32_t q);
void vg_batch_log(const vg_batch* b, uint32_t q, uint32_t i, uint32_t* op, uint64_t* p1, uint64_t* p2,
                  uint64_t* p3);
/* Releases the batch and its results.  The release runs on an idle host
 * worker after the call returns; vg_ctx_memory, vg_ctx_destroy, vg_index_free
 * and an allocation that would not fit otherwise wait for it. */
vg_status vg_batch_free(vg_batch* b);

/* ---- ingest (N-Triples) -------------------------------------------------- */
typedef struct vg_dict vg_dict;

/* Parses len bytes of N-Triples text (host memory) on the device and assigns
 * ids in order of first appearance, as the reference's loader does with
 * Raptor (load_rdf, src/loader.cu:19-93): subjects and non-literal objects
 * share one dictionary (ids from 1), predicates have their own (ids from 1),
 * literal objects a third (ids from 50,000,000) when literal_dict is set and
 * share the first otherwise.  On success *s, *p, *o are device columns of *n
 * ids (pass them to vg_index_build with inputs_on_device = 1; free them with
 * vg_ingest_free) and *dict the dictionaries.  A malformed statement gives
 * VG_ERR_PARSE with its line number in vg_last_error(). */
vg_status vg_ingest_ntriples(vg_ctx* ctx, const char* text, uint64_t len, int literal_dict, uint32_t** s,
                             uint32_t** p, uint32_t** o, uint64_t* n, vg_dict** dict);
vg_status vg_ingest_free(vg_ctx* ctx, uint32_t* s, uint32_t* p, uint32_t* o);
/* Dictionary kinds: 0 subject/object, 1 predicate, 2 literal. */
uint64_t vg_dict_size(const vg_dict* d, int kind);
/* The term of an id (its N-Triples text), NULL when unknown; valid until
 * vg_dict_free. */
const char* vg_dict_term(const vg_dict* d, int kind, uint32_t id);
/* The id of a term, 0 when absent (the query front end's IRI lookup). */
uint32_t vg_dict_lookup(vg_dict* d, int kind, const char* term);
/* The reference's .vdd text (VedasBuild save_dict, src/VedasBuild.cu:145-160),
 * written in id order; vg_dict_open reads entries in any order. */
vg_status vg_dict_write(const vg_dict* d, const char* path);
vg_status vg_dict_open(const char* path, vg_dict** out);
vg_status vg_dict_free(vg_dict* d);
/* Makes the queries on ix (vg_query, vg_batch_*, vg_serve_*) take constant
 * terms as text, mapped through d as the reference's TriplePattern does
 * (src/TriplePattern.cu:11-49): <iri> among subjects/objects or predicates by
 * position, a quoted object among literals (language tag and datatype
 * dropped, as Rasqal's value is), an absent term as id 0.  The ids are copied
 * into ix, so d may be freed afterwards; NULL restores numeric <ID>
 * constants. */
vg_status vg_index_set_dict(vg_index* ix, const vg_dict* d);
/* A result's rows as text (SparqlResult::printResult, src/SparqlResult.cu:
 * 42-123, without the table frame): one line per row, tab-separated terms,
 * each id decoded through the literal dictionary when it is in use and the
 * id is a literal id, through the subject/object dictionary otherwise;
 * unknown ids print as "?<id>".  *needed receives the size with the final
 * NUL; VG_ERR_OVERFLOW when cap is smaller (call again with a larger buf). */
vg_status vg_result_decode(const vg_result* r, const vg_dict* d, char* buf, size_t cap, size_t* needed);
/* The same for query q of a batch (from its host copies when the batch was
 * run with vg_batch_run_host). */
vg_status vg_batch_decode(const vg_batch* b, uint32_t q, const vg_dict* d, char* buf, size_t cap, size_t* needed);
/* Test hook, no reference counterpart: hash bits used to group terms (63
 * by default); fewer force hash collisions, which ingest resolves exactly. */
void vg_ingest_set_hash_bits(int bits);

/* ---- self-check ----------------------------------------------------------- */
/* No reference counterpart: runs one device wait that can never be satisfied
 * (which 0: a look-back status word nobody publishes; 1: an mbarrier that
 * expects bytes no copy delivers).  The wait gives up after about a second
 * and the call returns VG_ERR_TIMEOUT; the context stays usable. */
vg_status vg_selfcheck_bounded_wait(vg_ctx* ctx, int which);

/* No reference counterpart, no device use: `pools` threads, each with its own
 * host worker pool of `threads` threads (as the batch's wave engines have),
 * run `loops` parallel loops of random sizes and queue background work
 * between them.  *errors = items that did not run exactly once plus queued
 * tasks that never ran. */
vg_status vg_selfcheck_pools(uint32_t pools, uint32_t threads, uint32_t loops, uint64_t* errors);

/* No reference counterpart, no device use: on `graphs` random level-1/level-2
 * index arrays, `lookups` random (predicate, key) lookups through the
 * per-predicate level-2 range table, and searches of level-2 data ranges
 * through their sampled fences, give what the reference's searches give
 * (src/QueryExecutor.cu:596-646, src/SelectQueryJob.cu:74-86,
 * src/EmptyIntervalDict.cu:108-170), out-of-bounds cases included.
 * *mismatches = lookups that differ. */
vg_status vg_selfcheck_l2_lookup(uint32_t seed, uint32_t graphs, uint32_t lookups, uint64_t* mismatches);

/* ---- serving (continuous batching) -------------------------------------- */
typedef struct vg_server vg_server;

/* Starts a serving loop on the context: VG_SERVE_ENGINES wave engines
 * (default 1), each with a worker thread and a stream of its own.
 * Submitted queries are planned on the caller's thread, then admitted first
 * come first served at the engines' wave boundaries while the estimated
 * relation bytes of the queries in flight plus the bytes of finished results
 * not yet released stay within `budget_bytes`; admitted queries share the
 * batched launches of their engine's waves until they finish.  Replaces
 * vdQuery's REPL loop (src/VedasQuery.cu:136-205), which runs one query at a
 * time.  Only vg_serve_* calls may use the context while the server runs. */
vg_status vg_serve_start(vg_ctx* ctx, vg_index* ix, size_t budget_bytes, vg_server** out);
/* Queues one query; `ticket` identifies it.  A query whose estimate alone
 * exceeds the budget finishes at once with VG_ERR_REJECTED. */
vg_status vg_serve_submit(vg_server* s, const char* sparql, uint64_t* ticket);
/* Submits n queries at once (planned in parallel, queued in order);
 * tickets[i] is the ticket of sparql[i]. */
vg_status vg_serve_submit_many(vg_server* s, const char* const* sparql, uint32_t n, uint64_t* tickets);
/* Waits up to timeout_s seconds (< 0: forever); *done = 1 when finished. */
vg_status vg_serve_wait(vg_server* s, uint64_t ticket, double timeout_s, int* done);
/* The finished query's own status, and its result (as for vg_result_*). */
vg_status vg_serve_query_status(vg_server* s, uint64_t ticket);
uint32_t vg_serve_ncols(vg_server* s, uint64_t ticket);
uint64_t vg_serve_nrows(vg_server* s, uint64_t ticket);
const char* vg_serve_header(vg_server* s, uint64_t ticket, uint32_t c);
vg_status vg_serve_download(vg_server* s, uint64_t ticket, uint32_t c, uint32_t* host);
/* Seconds from submission to admission and to completion. */
vg_status vg_serve_latency(vg_server* s, uint64_t ticket, double* queued_s, double* total_s);
/* Frees a finished query's result. */
vg_status vg_serve_release(vg_server* s, uint64_t ticket);
/* Load shedding (no reference counterpart): queries that waited more than
 * `seconds` in the queue finish with VG_ERR_REJECTED instead of being
 * admitted, and queries submitted while the head of the queue has waited
 * half of it are refused at once, unplanned; 0 (the default) admits every
 * query however long it waited. */
vg_status vg_serve_set_queue_limit(vg_server* s, double seconds);
/* out6 = {submitted, completed, rejected, waves, reserved bytes, peak queries in flight}. */
vg_status vg_serve_stats(vg_server* s, uint64_t out6[6]);
/* Lets the queries in flight finish, then stops the worker. */
vg_status vg_serve_stop(vg_server* s);

#ifdef __cplusplus
}
#endif

#endif /* VEDAS_GB300_H */
