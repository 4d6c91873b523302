// Reference-as-oracle driver (test infrastructure only; never shipped).
//
// Links the VEDAS reference's own src/*.cu files, compiled unmodified with g++
// against Thrust's OpenMP backend and the host shims in oracle/refshim/, and
// runs them on this project's synthetic inputs:
//
//   vedas_ref index <graph.bin> <out.bin> [full]
//       VedasStorage(RdfData&, preload=false, fullIndex) (src/VedasStorage.cu:25-73)
//       then dumps every index array through the VedasStorage getters.
//   vedas_ref time <graph.bin> <queries.txt> <reps>
//       Wall seconds of each timed pass of QueryExecutor::query over the
//       queries (the CPU-baseline calibration of the restatement).
//   vedas_ref vds-write <graph.bin> <out.vds> [full]
//       VedasStorage(RdfData&, ...) then VedasStorage::write: the reference's
//       own .vds file of the graph.
//   vedas_ref query <graph.bin> <queries.txt> <out.bin> [first_query] [full]
//       For each query line: SparqlQuery + QueryExecutor::query, as vdQuery's
//       REPL does (src/VedasQuery.cu:136-205), with ENABLE_UPDATE_BOUND_AFTER_JOIN
//       true (src/VedasQuery.cu:37).  Results are appended and flushed per
//       query so that a reference abort (its asserts are live) loses only the
//       query that aborted.
//
// Graph file: "VGRAPH1\0", u64 n, u32 s[n], u32 p[n], u32 o[n].
// Query text: SELECT * | ?v.. WHERE { t t t . ... } with constants written as
// <ID> (subject/predicate/object IDs) or "ID" (literal object IDs).
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <memory>

#include "EmptyIntervalDict.h"
#include "PlanTreeNode.h"
#include "QueryExecutor.h"
#include "QueryGraph.h"
#include "RdfData.h"
#include "SparqlQuery.h"
#include "SparqlResult.h"
#include "VedasStorage.h"

namespace {

bool read_graph(const char* path, TYPEID_HOST_VEC& s, TYPEID_HOST_VEC& p, TYPEID_HOST_VEC& o) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  char magic[8];
  in.read(magic, 8);
  if (std::memcmp(magic, "VGRAPH1", 7) != 0) return false;
  uint64_t n = 0;
  in.read(reinterpret_cast<char*>(&n), 8);
  s.resize(n);
  p.resize(n);
  o.resize(n);
  in.read(reinterpret_cast<char*>(s.data()), n * 4);
  in.read(reinterpret_cast<char*>(p.data()), n * 4);
  in.read(reinterpret_cast<char*>(o.data()), n * 4);
  return static_cast<bool>(in);
}

void put_u32(std::ofstream& out, uint32_t v) { out.write(reinterpret_cast<const char*>(&v), 4); }
void put_u64(std::ofstream& out, uint64_t v) { out.write(reinterpret_cast<const char*>(&v), 8); }
void put_str(std::ofstream& out, const std::string& s) {
  put_u32(out, static_cast<uint32_t>(s.size()));
  out.write(s.data(), static_cast<std::streamsize>(s.size()));
}
void put_arr(std::ofstream& out, const std::string& name, const TYPEID_HOST_VEC* v) {
  put_str(out, name);
  put_u64(out, v->size());
  if (!v->empty()) out.write(reinterpret_cast<const char*>(v->data()), v->size() * 4);
}

// Every constant of a query line, registered in the dictionaries under the
// exact key TriplePattern's constructor looks up (src/TriplePattern.cu:62-82).
void register_constants(const std::string& q, DICTTYPE& so, DICTTYPE& p, DICTTYPE& l) {
  for (size_t i = 0; i < q.size(); ++i) {
    char c = q[i];
    if (c != '<' && c != '"') continue;
    char close = (c == '<') ? '>' : '"';
    size_t e = q.find(close, i + 1);
    if (e == std::string::npos) break;
    std::string body = q.substr(i + 1, e - i - 1);
    TYPEID id = static_cast<TYPEID>(std::strtoul(body.c_str(), nullptr, 10));
    std::string key = std::string(1, c) + body + std::string(1, close);
    if (c == '<') {
      so[key] = id;
      p[key] = id;
    } else {
      l[key] = id;
    }
    i = e;
  }
}

int do_index(const char* graph, const char* outp, bool full) {
  TYPEID_HOST_VEC s, p, o;
  if (!read_graph(graph, s, p, o)) return 2;
  RdfData rdf(s, p, o);
  VedasStorage st(rdf, false, full);
  std::ofstream out(outp, std::ios::binary);
  put_arr(out, "p_idx_values", st.getPredicateIndexValues());
  put_arr(out, "p_idx_offsets", st.getPredicateIndexOffsets());
  put_arr(out, "ps_s_idx_values", st.getPredicateSubjectIndexValues());
  put_arr(out, "ps_idx_offsets", st.getPredicateSubjectIndexOffsets());
  put_arr(out, "po_o_idx_values", st.getPredicateObjectIndexValues());
  put_arr(out, "po_idx_offsets", st.getPredicateObjectIndexOffsets());
  put_arr(out, "ps_data", st.getPSdata());
  put_arr(out, "po_data", st.getPOdata());
  put_arr(out, "pso_data", st.getPSOdata());
  put_arr(out, "pos_data", st.getPOSdata());
  if (full) {
    put_arr(out, "s_idx_values", st.getSubjectIndexValues());
    put_arr(out, "s_idx_offsets", st.getSubjectIndexOffsets());
    put_arr(out, "sp_p_idx_values", st.getSubjectPredicateIndexValues());
    put_arr(out, "sp_idx_offsets", st.getSubjectPredicateIndexOffsets());
    put_arr(out, "so_o_idx_values", st.getSubjectObjectIndexValues());
    put_arr(out, "so_idx_offsets", st.getSubjectObjectIndexOffsets());
    put_arr(out, "o_idx_values", st.getObjectIndexValues());
    put_arr(out, "o_idx_offsets", st.getObjectIndexOffsets());
    put_arr(out, "os_data", st.getOSdata());
    put_arr(out, "op_p_idx_values", st.getObjectPredicateIndexValues());
    put_arr(out, "op_idx_offsets", st.getObjectPredicateIndexOffsets());
    put_arr(out, "spo_data", st.getSPOdata());
    put_arr(out, "sop_data", st.getSOPdata());
    put_arr(out, "ops_data", st.getOPSdata());
    put_arr(out, "osp_data", st.getOSPdata());
  }
  put_str(out, "");
  return out ? 0 : 3;
}

// The reference's own .vds file of a graph: VedasStorage(RdfData&, ...) then
// VedasStorage::write (src/VedasStorage.cu:486-516).
int do_vds_write(const char* graph, const char* outp, bool full) {
  TYPEID_HOST_VEC s, p, o;
  if (!read_graph(graph, s, p, o)) return 2;
  RdfData rdf(s, p, o);
  VedasStorage st(rdf, false, full);
  st.write(outp);
  return 0;
}

int do_query(const char* graph, const char* qpath, const char* outp, size_t first, bool full) {
  TYPEID_HOST_VEC s, p, o;
  if (!read_graph(graph, s, p, o)) return 2;
  RdfData rdf(s, p, o);
  VedasStorage st(rdf, false, full);

  std::vector<std::string> lines;
  {
    std::ifstream qin(qpath);
    std::string line;
    while (std::getline(qin, line))
      if (!line.empty()) lines.push_back(line);
  }
  std::ofstream out(outp, std::ios::binary | std::ios::app);
  std::vector<int> gpu_ids{0};
  ExecutionWorker worker(gpu_ids);
  mgpu::standard_context_t context(false);
  QueryExecutor::ENABLE_UPDATE_BOUND_AFTER_JOIN = true;
  QueryExecutor::ENABLE_FULL_INDEX = full;
  QueryExecutor::ENABLE_LITERAL_DICT = false;
  QueryExecutor::ENABLE_BOUND_DICT_AFTER_JOIN = false;

  for (size_t qi = first; qi < lines.size(); ++qi) {
    DICTTYPE so_map, p_map, l_map;
    register_constants(lines[qi], so_map, p_map, l_map);
    QueryExecutor::initTime();
    SparqlQuery sq(lines[qi].c_str(), so_map, p_map, l_map);
    SparqlResult sr;
    QueryExecutor qe(&st, &worker, &context);
    qe.query(sq, sr);

    std::vector<std::string> headers = sr.getHeaderVariables();
    std::vector<std::vector<TYPEID>> cols = sr.get();
    put_u32(out, static_cast<uint32_t>(qi));
    put_u32(out, headers.empty() ? 1u : 0u);
    put_u32(out, static_cast<uint32_t>(headers.size()));
    uint64_t nrows = cols.empty() ? 0 : cols[0].size();
    put_u64(out, nrows);
    for (size_t c = 0; c < headers.size(); ++c) {
      put_str(out, headers[c]);
      out.write(reinterpret_cast<const char*>(cols[c].data()), nrows * 4);
    }
    // execution log: (op, p1, p2, p3, text) per job, src/vedas.h:87-103
    put_u32(out, static_cast<uint32_t>(QueryExecutor::exe_log.size()));
    for (const ExecuteLogRecord& r : QueryExecutor::exe_log) {
      put_u32(out, static_cast<uint32_t>(r.op));
      put_u64(out, r.param1);
      put_u64(out, r.param2);
      put_u64(out, r.param3);
      put_str(out, r.paramstr);
    }
    out.flush();
  }
  return 0;
}

// Wall time of the reference's query path over a query file, as vdBench
// times it (src/VedasBench.cu:144-176: one QueryExecutor::query per query,
// in order, after the index is built): one untimed pass, then `reps` timed
// passes; prints "TIME <pass> <seconds> <result rows>" per timed pass to
// stderr (the reference's own messages go to stdout).
int do_time(const char* graph, const char* qpath, int reps) {
  TYPEID_HOST_VEC s, p, o;
  if (!read_graph(graph, s, p, o)) return 2;
  RdfData rdf(s, p, o);
  VedasStorage st(rdf, false, false);
  std::vector<std::string> lines;
  {
    std::ifstream qin(qpath);
    std::string line;
    while (std::getline(qin, line))
      if (!line.empty()) lines.push_back(line);
  }
  std::vector<int> gpu_ids{0};
  ExecutionWorker worker(gpu_ids);
  mgpu::standard_context_t context(false);
  QueryExecutor::ENABLE_UPDATE_BOUND_AFTER_JOIN = true;
  QueryExecutor::ENABLE_FULL_INDEX = false;
  QueryExecutor::ENABLE_LITERAL_DICT = false;
  QueryExecutor::ENABLE_BOUND_DICT_AFTER_JOIN = false;
  std::vector<DICTTYPE> so(lines.size()), pm(lines.size()), lm(lines.size());
  for (size_t qi = 0; qi < lines.size(); ++qi) register_constants(lines[qi], so[qi], pm[qi], lm[qi]);
  for (int pass = -1; pass < reps; ++pass) {
    uint64_t rows = 0;
    auto t0 = std::chrono::steady_clock::now();
    for (size_t qi = 0; qi < lines.size(); ++qi) {
      QueryExecutor::initTime();
      SparqlQuery sq(lines[qi].c_str(), so[qi], pm[qi], lm[qi]);
      SparqlResult sr;
      QueryExecutor qe(&st, &worker, &context);
      qe.query(sq, sr);
      std::vector<std::vector<TYPEID>> cols = sr.get();
      rows += cols.empty() ? 0 : cols[0].size();
    }
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (pass >= 0) std::fprintf(stderr, "TIME %d %.6f %llu\n", pass, sec, static_cast<unsigned long long>(rows));
  }
  return 0;
}

// Plan of one query line "<e0> <e1> ... | <query>" with the given per-pattern
// estimate_rows, through the reference's QueryGraph::generateQueryPlan
// (src/QueryGraph.cu:64-74), printed in the post-order that
// QueryExecutor::postorderTraversal emits jobs (src/QueryExecutor.cu:106-135).
int plan_node(PlanTreeNode* n, std::string& out, int& counter) {
  if (!n) return -1;
  int a = -1, b = -1;
  if (n->child1) a = plan_node(n->child1, out, counter);
  if (n->child2) b = plan_node(n->child2, out, counter);
  if (n->op == UPLOAD) {
    std::string idx = "-";
    if (n->tp->getVariableNum() == 2) idx = (n->tp->getSubject() == n->var) ? "PSO" : "POS";
    out += "U" + std::to_string(n->tp->getId()) + ":" + idx + ";";
  } else if (n->op == JOIN) {
    out += "J" + std::to_string(a) + "," + std::to_string(b) + ":" + n->var + ":" +
           (n->reuseVar ? "0" : "1") + ";";
  } else {
    out += "W" + std::to_string(a) + ":" + n->var + ";";
  }
  return counter++;
}

int do_plan(const char* qpath, const char* outp) {
  std::ifstream qin(qpath);
  std::ofstream out(outp);
  std::string line;
  while (std::getline(qin, line)) {
    if (line.empty()) continue;
    size_t bar = line.find('|');
    std::istringstream es(line.substr(0, bar));
    std::vector<size_t> est;
    size_t e;
    while (es >> e) est.push_back(e);
    std::string q = line.substr(bar + 1);
    DICTTYPE so_map, p_map, l_map;
    register_constants(q, so_map, p_map, l_map);
    SparqlQuery sq(q.c_str(), so_map, p_map, l_map);
    for (size_t i = 0; i < sq.getPatternNum() && i < est.size(); ++i) sq.getPatternPtr(i)->estimate_rows = est[i];
    QueryGraph qg(&sq, nullptr);
    PlanTreeNode* root = qg.generateQueryPlan();
    std::string s;
    int counter = 0;
    plan_node(root, s, counter);
    out << s << "\n";
  }
  return 0;
}

// EmptyIntervalDict sequences: lines "update lb1 ub1 lb2 ub2", "get" and
// "reset" on one variable; every "get" prints the bound tuple.
int do_eid(const char* inp, const char* outp) {
  std::ifstream in(inp);
  std::ofstream out(outp);
  std::unique_ptr<EmptyIntervalDict> d(new EmptyIntervalDict());
  std::string op;
  while (in >> op) {
    if (op == "reset") {
      d.reset(new EmptyIntervalDict());
    } else if (op == "update") {
      size_t a, b, c, e;
      in >> a >> b >> c >> e;
      d->updateBound("?x", a, b, c, e);
    } else if (op == "get") {
      VAR_BOUND v = d->getBound("?x");
      out << std::get<0>(v) << " " << std::get<1>(v) << " " << std::get<2>(v) << " " << std::get<3>(v) << "\n";
    }
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc >= 4 && std::string(argv[1]) == "plan") return do_plan(argv[2], argv[3]);
  if (argc >= 4 && std::string(argv[1]) == "eid") return do_eid(argv[2], argv[3]);
  if (argc >= 4 && std::string(argv[1]) == "index") {
    bool full = argc >= 5 && std::string(argv[4]) == "full";
    return do_index(argv[2], argv[3], full);
  }
  if (argc >= 5 && std::string(argv[1]) == "time") return do_time(argv[2], argv[3], std::atoi(argv[4]));
  if (argc >= 4 && std::string(argv[1]) == "vds-write") {
    bool full = argc >= 5 && std::string(argv[4]) == "full";
    return do_vds_write(argv[2], argv[3], full);
  }
  if (argc >= 5 && std::string(argv[1]) == "query") {
    size_t first = argc >= 6 ? std::strtoull(argv[5], nullptr, 10) : 0;
    bool full = argc >= 7 && std::string(argv[6]) == "full";
    return do_query(argv[2], argv[3], argv[4], first, full);
  }
  std::fprintf(stderr, "usage: vedas_ref index|query ...\n");
  return 1;
}
