/* CPU oracle for the VEDAS query-execution path (TEST INFRASTRUCTURE ONLY).
 *
 * A restatement, in this project's own C++, of the reference's index build
 * and query path (VedasStorage, QueryExecutor pre-scan and plan, Select /
 * Join / IndexSwap jobs, EmptyIntervalDict, final projection and adjacent
 * dedup).  It is used only by tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg, as the checker; the product never links it.
 *
 * Parity pin: its outputs are checked against golden vectors produced by the
 * reference's own sources compiled for the host (oracle/_ref, see
 * oracle/Makefile and tests/golden/make_golden.py).
 *
 * Status codes: 0 ok; 1 bad query text; 2 the reference would take an
 * undefined-behaviour or assert-abort path on this input (see the message);
 * 3 other error.
 */
#ifndef VEDAS_ORACLE_H
#define VEDAS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vo_index vo_index;
typedef struct vo_result vo_result;

vo_index* vo_index_build(const uint32_t* s, const uint32_t* p, const uint32_t* o, uint64_t n,
                         int full_index);
void vo_index_free(vo_index* ix);
/* Named arrays of the reference layout (p_idx_values, ps_data, ...). */
int vo_index_array(const vo_index* ix, const char* name, const uint32_t** data, uint64_t* len);

vo_result* vo_query(vo_index* ix, const char* text);
int vo_result_status(const vo_result* r);
const char* vo_result_error(const vo_result* r);
uint32_t vo_result_ncols(const vo_result* r);
const char* vo_result_header(const vo_result* r, uint32_t c);
uint64_t vo_result_nrows(const vo_result* r);
const uint32_t* vo_result_column(const vo_result* r, uint32_t c);
uint32_t vo_result_nlog(const vo_result* r);
void vo_result_log(const vo_result* r, uint32_t i, uint32_t* op, uint64_t* p1, uint64_t* p2,
                   uint64_t* p3, const char** text);
void vo_result_free(vo_result* r);

/* Host logic: the plan for given per-pattern estimates, as a post-order job
 * list "U<tp>:<index>;", "J<l>,<r>:<var>:<last>;", "W<child>:<var>;"; and the
 * empty-interval entry after n updateBound calls (quads = n x 4 values). */
int vo_plan_describe(const char* text, const uint64_t* est, uint32_t n, char* buf, uint64_t cap);
int vo_eid_sequence(const uint64_t* quads, uint32_t n, uint64_t* out4);

/* Job-level checkers used by the kernel parity tests. */
/* Stable sort of rows by column 0 (FullRelationIR::sortByFirstColumn). */
void vo_sort_by_first(uint32_t** cols, uint32_t ncols, uint64_t nrows);
/* Inner join of two sorted key columns: pair count, then pairs (i ascending,
 * then j ascending) when out_l/out_r are non-null. */
uint64_t vo_inner_join(const uint32_t* a, uint64_t na, const uint32_t* b, uint64_t nb,
                       uint64_t* out_l, uint64_t* out_r);

/* N-Triples ingest (src/loader.cu:19-53): 0 on success with malloc'd id
 * columns and '\n'-joined dictionary terms in id order (subject/object,
 * predicate, literal); otherwise the 1-based number of the first malformed
 * line.  Free every output with vo_free.  Parity unpinned (Raptor absent). */
uint64_t vo_ingest_ntriples(const char* text, uint64_t len, int literal_dict, uint64_t* n_out, uint32_t** s,
                            uint32_t** p, uint32_t** o, char** so_terms, char** p_terms, char** l_terms);
void vo_free(void* ptr);

#ifdef __cplusplus
}
#endif

#endif
