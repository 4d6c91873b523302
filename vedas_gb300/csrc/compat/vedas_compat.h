// Host-side mirror of the reference's query-execution interfaces, on top of
// the GB300 kernels.  Class and method names, argument meaning and job
// semantics follow the reference (paths relative to the reference project):
//   VedasStorage        src/VedasStorage.h:8-132
//   FullRelationIR      src/FullRelationIR.h:10-47
//   EmptyIntervalDict   src/EmptyIntervalDict.h:6-23
//   TriplePattern       src/TriplePattern.h:7-36
//   SparqlQuery         src/SparqlQuery.h:10-47 (structured-text front end)
//   SparqlResult        src/SparqlResult.h:9-25
//   QueryJob & jobs     src/QueryJob.h, SelectQueryJob.h, JoinQueryJob.h,
//                       IndexSwapJob.h, TransferJob.h
//   QueryPlan           src/QueryPlan.h:15-49 (single-GPU execution)
//   QueryGraph          src/QueryGraph.h:14-47
//   QueryExecutor       src/QueryExecutor.h:39-123
// Relations live in HBM (arena spans) instead of thrust::device_vector, the
// index is resident in HBM, and the host keeps mirrors of the index arrays
// for the host-side binary searches the reference performs.
#pragma once

#include "vg_fence.h"

#include <cstdint>
#include <array>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <tuple>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

#include "../vg_ctx.h"
#include "../vg_index.h"
#include "../vg_relops.h"

namespace vedas {

typedef uint32_t TYPEID;
typedef std::vector<TYPEID> TYPEID_HOST_VEC;
typedef std::tuple<size_t, size_t, size_t, size_t> VAR_BOUND;
typedef std::map<std::string, std::pair<TYPEID, TYPEID>> BoundDict;

enum ExecuteLogRecordOp { JOIN_OP, UPLOAD_OP, SWAP_OP };
struct ExecuteLogRecord {
  int deviceId;
  ExecuteLogRecordOp op;
  size_t param1, param2, param3;
  std::string paramstr;
  ExecuteLogRecord(int d, ExecuteLogRecordOp o, std::string s, size_t p1, size_t p2 = 0, size_t p3 = 0)
      : deviceId(d), op(o), param1(p1), param2(p2), param3(p3), paramstr(std::move(s)) {}
};

class IR {
 public:
  virtual ~IR() = default;
};

// Maps the text of a constant query term to its dictionary id (the
// reference's TriplePattern constructor, src/TriplePattern.cu:11-49): pos 0
// subject, 1 predicate, 2 object.  Absent terms give 0, as the reference's
// map lookups do.  Must be callable from many threads at once.
class TermResolver {
 public:
  virtual ~TermResolver() = default;
  virtual TYPEID resolve(int pos, const std::string& term) const = 0;
};

class VedasStorage {
 public:
  // Builds the index on the device from host or device columns.
  VedasStorage(vg::Ctx* ctx, const TYPEID* s, const TYPEID* p, const TYPEID* o, size_t n,
               bool inputs_on_device, bool fullIndex);
  // Opens a .vds file written by write() (src/VedasStorage.cu:459-484).
  VedasStorage(vg::Ctx* ctx, const char* fname, bool fullIndex);
  ~VedasStorage();

  size_t getTripleSize() const { return ix_.n; }
  bool isFullIndex() const { return ix_.full; }
  // Host mirrors (the reference's getters return host vectors).
  TYPEID_HOST_VEC* getPredicateIndexValues() { return h(kPIdxV); }
  TYPEID_HOST_VEC* getPredicateIndexOffsets() { return h(kPIdxO); }
  TYPEID_HOST_VEC* getPredicateSubjectIndexValues() { return h(kPSIdxV); }
  TYPEID_HOST_VEC* getPredicateSubjectIndexOffsets() { return h(kPSIdxO); }
  TYPEID_HOST_VEC* getPredicateObjectIndexValues() { return h(kPOIdxV); }
  TYPEID_HOST_VEC* getPredicateObjectIndexOffsets() { return h(kPOIdxO); }
  TYPEID_HOST_VEC* getPSdata() { return h(kPS); }
  TYPEID_HOST_VEC* getPOdata() { return h(kPO); }
  TYPEID_HOST_VEC* getPSOdata() { return h(kPSO); }
  TYPEID_HOST_VEC* getPOSdata() { return h(kPOS); }
  TYPEID_HOST_VEC* getSOPdata() { return h(kSOP); }
  // Makes every host mirror above (downloading on first use) and the level-2
  // range tables below; after it the getters may be called from many threads
  // at once.
  void prepareMirrors();
  // Level-2 range of every predicate, for the predicate-subject (po = false)
  // or predicate-object (po = true) index: entry s is the first level-2 entry
  // whose offset is not below the predicate index offset s (the last entry
  // uses the triple count), i.e. findDataOffsetFromL2's two searches of the
  // level-2 offsets done once per predicate.  Empty before prepareMirrors().
  const std::vector<size_t>& l2RangeOfL1(bool po) const { return l2r_[po ? 1 : 0]; }
  // Every 64th key of the level-2 data (ps_data for po = false, po_data for
  // po = true), for fenced_bound; empty before prepareMirrors().
  const std::vector<uint32_t>& l2Fences(bool po) const { return fence_[po ? 1 : 0]; }
  // Device copies (resident).
  const TYPEID* dev(const char* name) const { return ix_.get(name).ptr; }
  const TYPEID* devPSdata() const { return d_[kPS]; }
  const TYPEID* devPOdata() const { return d_[kPO]; }
  const TYPEID* devPSOdata() const { return d_[kPSO]; }
  const TYPEID* devPOSdata() const { return d_[kPOS]; }
  const TYPEID* devPSIdxValues() const { return d_[kPSIdxV]; }
  const TYPEID* devPOIdxValues() const { return d_[kPOIdxV]; }
  uint64_t len(const char* name) const { return ix_.get(name).len; }
  vg::Index& index() { return ix_; }
  // Dictionary for constant terms written as text (IRIs, literals) in the
  // queries run on this storage; null: constants are numeric ids.
  const TermResolver* resolver() const { return resolver_; }
  void setResolver(const TermResolver* r) { resolver_ = r; }
  void write(const char* fname);

 private:
  enum Mirror { kPIdxV, kPIdxO, kPSIdxV, kPSIdxO, kPOIdxV, kPOIdxO, kPS, kPO, kPSO, kPOS, kSOP, kMirrors };
  static const char* const kMirrorName[kMirrors];
  vg::Index ix_;
  const TermResolver* resolver_ = nullptr;
  TYPEID_HOST_VEC* mirror_[kMirrors] = {};
  const TYPEID* d_[kMirrors] = {};
  std::vector<size_t> l2r_[2];
  std::vector<uint32_t> fence_[2];
  std::once_flag mirrors_once_;
  void cacheDevice();   // the device arrays' addresses (set at construction)
  TYPEID_HOST_VEC* h(Mirror m) {
    if (!mirror_[m]) mirror_[m] = const_cast<TYPEID_HOST_VEC*>(&ix_.host_array(kMirrorName[m]));
    return mirror_[m];
  }
};

class FullRelationIR : public IR {
 public:
  FullRelationIR(vg::Ctx* ctx, size_t columnNum, size_t relationSize);
  // A relation whose columns are views of index slices (not copied); see
  // vg::Rel::borrowed.
  FullRelationIR(vg::Ctx* ctx, size_t columnNum, size_t relationSize, const TYPEID* const* views);
  ~FullRelationIR() override;
  void sort();
  void removeDuplicate();
  TYPEID* getRelationRawPointer(size_t i) { return r_.cols[i]; }
  size_t getColumnNum() const { return headers.size(); }
  size_t getColumnId(const std::string& var) const;
  void setHeader(size_t i, const std::string& h, bool is_predicate);
  std::string getHeader(size_t i) const { return headers[i]; }
  std::string getHeaders(const std::string& delimitor) const;
  bool getIsPredicate(size_t i) const { return is_predicates[i]; }
  void sortByFirstColumn();
  void swapColumn(size_t i, size_t j);
  void removeColumn(size_t i);
  void removeColumn(size_t i, const std::string& maintain_var);
  // removeColumn(i, maintain_var) without its re-sort; true when the caller
  // must still sort by column 0 (i == 0).
  bool removeColumnDeferSort(size_t i, const std::string& maintain_var);
  size_t size() const { return r_.ncols == 0 ? 0 : r_.nrows; }
  vg::Rel& rel() { return r_; }
  vg::Ctx* ctx() const { return ctx_; }
  // Replaces the columns by `r` (takes ownership), keeping headers.
  void adopt(vg::Rel& r);
  // Hands the columns to the caller; the relation keeps its headers only.
  vg::Rel release();

 private:
  vg::Ctx* ctx_;
  vg::Rel r_;
  // per column (at most VG_MAX_COLS): kept in place, no allocation
  std::array<bool, VG_MAX_COLS> is_predicates{};
  std::vector<std::string> headers;
  // Variable -> column.  A relation has at most nine columns, so a short
  // list searched in order replaces the reference's hash map.  Entries are
  // assigned and found as in a map and never removed: the reference's map
  // also keeps a removed column's stale index.
  struct VarColumns {
    std::vector<std::pair<std::string, size_t>> v;
    const size_t* find(const std::string& k) const {
      for (const auto& e : v)
        if (e.first == k) return &e.second;
      return nullptr;
    }
    size_t& operator[](const std::string& k) {
      for (auto& e : v)
        if (e.first == k) return e.second;
      v.emplace_back(k, 0);
      return v.back().second;
    }
  } var_column_map;
};

class EmptyIntervalDict {
 public:
  VAR_BOUND getBound(const std::string& var) const { return dict.at(var); }
  void updateBound(const std::string& var, size_t lb1, size_t ub1, size_t lb2, size_t ub2);
  // The pieces of data[start, end) outside the two empty intervals of var
  // (offsets relative to the start of `data`).
  void getUploadRelationData(const std::string& var, const TYPEID* data, size_t start, size_t end,
                             size_t& relationSize, std::vector<std::pair<size_t, size_t>>& uploadIntervals,
                             std::vector<size_t>& offsets,
                             const std::vector<uint32_t>* fences = nullptr);
  size_t emptySize(const std::string& var);
  bool hasBoundFor(const std::string& var) const { return dict.count(var) > 0; }

 private:
  std::unordered_map<std::string, VAR_BOUND> dict;
};

class TriplePattern {
 public:
  // Constants are <ID> / "ID" numbers, or any term text when a resolver maps
  // them through the dictionaries.
  TriplePattern(size_t id, const std::string& s, const std::string& p, const std::string& o,
                const TermResolver* resolver = nullptr);
  size_t getId() const { return id; }
  TYPEID getSubjectId() const { return ids[0]; }
  TYPEID getPredicateId() const { return ids[1]; }
  TYPEID getObjectId() const { return ids[2]; }
  std::string getSubject() const { return names[0]; }
  std::string getPredicate() const { return names[1]; }
  std::string getObject() const { return names[2]; }
  size_t getVariableNum() const { return isVar[0] + isVar[1] + isVar[2]; }
  size_t getVariableBitmap() const { return isVar[0] * 4 + isVar[1] * 2 + isVar[2]; }
  bool subjectIsVariable() const { return isVar[0]; }
  bool predicateIsVariable() const { return isVar[1]; }
  bool objectIsVariable() const { return isVar[2]; }
  bool hasVariable(const std::string& v) const;
  size_t estimate_rows = 0;

 private:
  size_t id;
  std::string names[3];
  TYPEID ids[3] = {0, 0, 0};
  bool isVar[3] = {false, false, false};
};

// SPARQL basic-graph-pattern front end (the reference parses with Rasqal,
// src/SparqlQuery.cu:29-124): SELECT * | ?v.. WHERE { t t t . ... } with
// constants written as <ID> or "ID".
class SparqlQuery {
 public:
  explicit SparqlQuery(const char* q, const TermResolver* resolver = nullptr);
  size_t getPatternNum() const { return patterns.size(); }
  TriplePattern* getPatternPtr(size_t i) { return &patterns[i]; }
  std::map<std::string, int>& getVarCountMap() { return vars_count; }
  std::set<std::string> getSelectedVariables() const { return selected_variables; }
  int boundedNum = 0;

 private:
  std::vector<TriplePattern> patterns;
  std::set<std::string> selected_variables;
  std::map<std::string, int> vars_count;
};

class SparqlResult {
 public:
  void setResult(IR* ir);
  FullRelationIR* getResultIR() { return resultIR; }

 private:
  FullRelationIR* resultIR = nullptr;
};

class QueryExecutor;

class QueryJob {
 public:
  virtual ~QueryJob() = default;
  virtual IR* getIR() = 0;
  virtual int startJob(int gpuId) = 0;
  virtual std::string jobTypeName() const = 0;
  int getGpuId() const { return gpuId; }

 protected:
  int gpuId = 0;
  IR* intermediateResult = nullptr;
};

// Device work a select needs once its host-side lookups are done: copies of
// index slices into the new relation.
struct SelectWork {
  FullRelationIR* ir = nullptr;
  std::vector<vg::CopyPiece> pieces;
};

// Host state of a join between its phases: operands (possibly swapped),
// which operand still needs its stable re-sort by the join column, and the
// output once built.
struct JoinWork {
  FullRelationIR* lir = nullptr;
  FullRelationIR* rir = nullptr;
  bool sortL = false, sortR = false;
  size_t new_col_num = 0;
  bool empty = false;     // an operand is empty: output decided on the host
};

class SelectQueryJob : public QueryJob {
 public:
  // two variables (src/SelectQueryJob.h:14-19)
  SelectQueryJob(QueryExecutor* ex, bool pos_index, std::string v1, std::string v2, TYPEID id1,
                 bool is_second_var_used);
  // one variable (src/SelectQueryJob.h:20-24): subject_var selects POS
  SelectQueryJob(QueryExecutor* ex, bool subject_var, std::string v1, TYPEID id1, TYPEID id2);
  ~SelectQueryJob() override;
  int startJob(int gpuId) override;
  IR* getIR() override { return intermediateResult; }
  std::string jobTypeName() const override { return "Upload Job"; }
  // Host part: index lookups, bounds, empty intervals; allocates the
  // relation and describes the copies that fill it.
  void prepare(SelectWork& w);

 private:
  QueryExecutor* ex;
  bool pos_index = false;     // 2-var: POS vs PSO; 1-var: subject variable
  std::string variables[2];
  size_t variable_num;
  TYPEID dataid[2] = {0, 0};
  bool is_second_var_used = true;
};

class JoinQueryJob : public QueryJob {
 public:
  JoinQueryJob(QueryExecutor* ex, QueryJob* leftJob, QueryJob* rightJob, std::string joinVariable,
               bool lastJoinForVar = true);
  // The reference never frees join results; here the job owns its relation.
  ~JoinQueryJob() override { delete intermediateResult; }
  int startJob(int gpuId) override;
  IR* getIR() override { return intermediateResult; }
  std::string jobTypeName() const override { return "Join Job"; }
  void setQueryVarCounter(std::map<std::string, size_t>* c) { query_variable_counter = c; }
  std::string getJoinVariable() const { return joinVariable; }
  IR* join(FullRelationIR* lir, FullRelationIR* rir);
  // Phase 1 (host): operand swap, column pruning and implicit index swaps
  // (their re-sorts are left to the caller: w.sortL / w.sortR).
  void prepare(JoinWork& w);
  // Phase 3 (after the join kernels): output relation, log, bound update and
  // the empty-interval scan.  `col0` holds output column 0 when
  // 2 < rows < 100 (else unused); first/last its first and last value.
  void finish(JoinWork& w, vg::Rel& joined, TYPEID first, TYPEID last, const std::vector<TYPEID>* col0);
  bool isLastJoinForVar() const { return lastJoinForVar; }
  QueryJob* left() const { return leftJob; }
  QueryJob* right() const { return rightJob; }

 private:
  void setHeaders(JoinWork& w, FullRelationIR* out);
  QueryExecutor* ex;
  QueryJob* leftJob;
  QueryJob* rightJob;
  std::string joinVariable;
  bool lastJoinForVar;
  std::map<std::string, size_t>* query_variable_counter = nullptr;
};

class IndexSwapJob : public QueryJob {
 public:
  IndexSwapJob(QueryExecutor* ex, QueryJob* beforeJob, std::string swapVar);
  int startJob(int gpuId) override;
  IR* getIR() override { return intermediateResult; }
  std::string jobTypeName() const override { return "Index Swap Job"; }
  // Phase 1 (host): moves the swap column to position 0; the relation then
  // needs its stable re-sort by column 0.
  FullRelationIR* prepare();
  // Phase 2 (after the sort): log and the empty-interval scan (`col0` holds
  // column 0 when 2 < rows < 100).
  void finish(const std::vector<TYPEID>* col0);

 private:
  size_t swapped_col = 0;
  QueryExecutor* ex;
  QueryJob* beforeJob;
  std::string swapVar;
};

// Single-GPU build: the relation already lives on the executing device, so
// the transfer is a pass-through (src/TransferJob.cu:28-39 moves it by P2P).
class TransferJob : public QueryJob {
 public:
  TransferJob(size_t src_thread_id, size_t dest_thread_id, int src_gpu_id, int dest_gpu_id,
              QueryJob* job);
  int startJob(int gpuId) override;
  IR* getIR() override { return intermediateResult; }
  std::string jobTypeName() const override { return "Transfer Job"; }

 private:
  QueryJob* job;
  int src_gpu_id, dest_gpu_id;
};

class QueryPlan {
 public:
  explicit QueryPlan(std::set<std::string>& select_variable_set);
  ~QueryPlan();
  void pushJob(QueryJob* job);
  QueryJob* getJob(size_t i) { return jobs[i]; }
  size_t jobNum() const { return jobs.size(); }
  // Runs the jobs in order, projects and removes adjacent duplicates.
  void execute(SparqlResult& sparqlResult);
  // The pieces of execute() for callers that run the jobs themselves:
  // counters before the first job, projection of the final relation after
  // the last (the adjacent-unique step is left to the caller).
  void beginExecution();
  FullRelationIR* project();

 private:
  std::map<std::string, size_t> query_variable_counter;
  std::vector<QueryJob*> jobs;
  std::vector<std::string> select_variables;
};

enum PlanOperation { UPLOAD, JOIN, INDEXSWAP };
struct PlanTreeNode {
  PlanOperation op;
  PlanTreeNode* child1 = nullptr;
  PlanTreeNode* child2 = nullptr;
  bool reuseVar = false;
  TriplePattern* tp = nullptr;
  std::string var;
};

struct GraphEdge {
  std::string id, indexVar1, indexVar2;
  std::set<std::string> vars;
  TriplePattern* tp = nullptr;
  size_t estimateCardinality = 0;
  PlanTreeNode* treeNode = nullptr;
  bool hasVariable(const std::string& v) const { return vars.count(v) > 0; }
};

class QueryGraph {
 public:
  explicit QueryGraph(SparqlQuery* q);
  PlanTreeNode* generateQueryPlan();

 private:
  std::unordered_map<std::string, std::vector<std::pair<std::string, GraphEdge*>>> adjacencyList;
  std::vector<std::unique_ptr<GraphEdge>> edges;
  std::vector<std::unique_ptr<PlanTreeNode>> nodes;
  void addEdge(const std::string& a, const std::string& b, GraphEdge* e);
  bool edgeExist(const std::string& a, const std::string& b);
  void mergeEdge(const std::string end1, const std::string end2);
  std::tuple<size_t, size_t, std::string> sameMaxDegAndTotalCard(
      std::vector<std::pair<std::string, GraphEdge*>>& links);
  std::pair<std::string, std::string> findBestStarNode();
  PlanTreeNode* generateJoinPlanForNode(const std::string& vertex, const std::string& joinVar);
  PlanTreeNode* newNode(PlanOperation op);
};

class QueryExecutor {
 public:
  QueryExecutor(VedasStorage* storage, vg::Ctx* ctx);
  // Plans and runs one query (src/QueryExecutor.cu:294-431).
  void query(SparqlQuery& sq, SparqlResult& sr);
  // The job list the reference would run (for batching); the plan keeps it.
  void plan(SparqlQuery& sq, QueryPlan& plan);

  static void updateBoundDict(BoundDict* bound, const std::string& variable, TYPEID lowerBound,
                              TYPEID upperBound);
  static std::pair<size_t, size_t> findL2OffsetFromL1(const TYPEID_HOST_VEC* l1v, const TYPEID_HOST_VEC* l1o,
                                                      TYPEID id1, size_t n);
  static std::pair<size_t, size_t> findDataOffsetFromL2(const TYPEID_HOST_VEC* l2v,
                                                        const TYPEID_HOST_VEC* l2o, TYPEID lo, TYPEID hi,
                                                        TYPEID id2);
  static std::pair<size_t, size_t> findDataOffsetFromL2(const TYPEID_HOST_VEC* l2_data, size_t lo,
                                                        size_t hi, TYPEID id2);
  // findL2OffsetFromL1(l1v, l1o, id1, n) followed by the five-argument
  // findDataOffsetFromL2 on the predicate-subject (po = false) or
  // predicate-object index, with the level-2 offset searches read from the
  // storage's per-predicate table; the same result (and the same errors).
  static std::pair<size_t, size_t> findDataOffsetForKey(VedasStorage* st, bool po, TYPEID id1, TYPEID id2,
                                                        size_t n);
  // The same on plain arrays: l2r is l2RangesOfL1(l1o, l2o, n).
  static std::pair<size_t, size_t> findDataOffsetForKey(const TYPEID_HOST_VEC* l1v, const TYPEID_HOST_VEC* l1o,
                                                        const TYPEID_HOST_VEC* l2v, const TYPEID_HOST_VEC* l2o,
                                                        const std::vector<size_t>& l2r, TYPEID id1, TYPEID id2,
                                                        size_t n);
  // Entry s: lower_bound(l2o, l1o[s]); the last entry: lower_bound(l2o, n).
  static std::vector<size_t> l2RangesOfL1(const TYPEID_HOST_VEC& l1o, const TYPEID_HOST_VEC& l2o, size_t n);

  // Execution log of the current query (QueryExecutor::exe_log).
  std::vector<ExecuteLogRecord> exe_log;
  // Whether log records carry the reference's text (relation headers); the
  // batched engine turns it off, its logs are read as numbers only.
  bool log_text = true;
  static bool ENABLE_UPDATE_BOUND_AFTER_JOIN;

  VedasStorage* storage;
  vg::Ctx* ctx;
  BoundDict variables_bound;
  EmptyIntervalDict empty_interval_dict;
  std::set<std::string> selected_variables;
  std::unordered_set<std::string> join_vars;

  // Empty-interval scan of a relation's column 0 (2 < size < 100).
  void eifScan(FullRelationIR* ir, const std::string& var);
  // The four bounds that scan passes to EmptyIntervalDict::updateBound.
  static void eifBounds(const TYPEID* c0, size_t n, size_t out[4]);

 private:
  void createVariableBound(SparqlQuery& sq);
  void squeezeQueryBound1Var(TriplePattern* p);
  void squeezeQueryBound2Var(TriplePattern* p);
  int postorderTraversal(QueryPlan& plan, PlanTreeNode* root, SparqlQuery& sq);
  SelectQueryJob* createSelectQueryJob(TriplePattern* p, const std::string& index_used);
};

// A condition on which the reference itself would read out of bounds or trip
// an assert; the core refuses the query instead (VG_ERR_UNSUPPORTED).
struct ReferenceUB : vg::Error {
  explicit ReferenceUB(const std::string& m) : vg::Error(VG_ERR_UNSUPPORTED, m) {}
};

// Host-only self-check of the index lookups: on random level-1/level-2
// arrays, QueryExecutor::findDataOffsetForKey (per-predicate table, upper
// bound searched forward) and the data-form findDataOffsetFromL2 give what the
// reference's searches give (src/QueryExecutor.cu:596-646: std::lower_bound
// and std::upper_bound over the whole ranges), errors included.  Returns the
// number of lookups that differ.
uint64_t selfcheck_l2_lookup(uint32_t seed, uint32_t graphs, uint32_t lookups);

}  // namespace vedas
