// CPU oracle for the VEDAS query-execution path -- TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain C++ on host vectors, what the reference does
// on its GPU path, so that the CUDA implementation can be checked against it
// on the same inputs.  Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg load it; the product never does.  Its own parity pin is the
// golden vectors produced by the reference's unmodified sources built for the
// host (oracle/_ref).
//
// Every function names the reference code it follows (paths relative to the
// reference project).  Where the reference would read out of bounds or trip a
// live assert, the oracle raises OracleUB (status 2) instead of inventing a
// value, except for the pre-scan reads documented at the call site whose
// value is provably overwritten.
#include "oracle.h"

#include <omp.h>

#include <algorithm>
#include <climits>
#include <functional>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <parallel/algorithm>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

namespace {

using ID = uint32_t;
using Vec = std::vector<ID>;

struct OracleUB : std::runtime_error {
  explicit OracleUB(const std::string& m) : std::runtime_error(m) {}
};
struct OracleParse : std::runtime_error {
  explicit OracleParse(const std::string& m) : std::runtime_error(m) {}
};

// ---------------------------------------------------------------------------
// Index (src/VedasStorage.cu:25-73, createIndex1Level :270-289, createIndex
// :306-358).  Every permutation is a full-key lexicographic sort of the
// triples, so the result is independent of sort stability.
// ---------------------------------------------------------------------------
struct Index {
  bool full = false;
  std::map<std::string, Vec> arr;
  Vec& a(const char* n) { return arr[n]; }
  const Vec& get(const char* n) const {
    auto it = arr.find(n);
    static const Vec empty;
    return it == arr.end() ? empty : it->second;
  }
};

struct Triple {
  ID k0, k1, k2;
};

// Sorts the triples by (k0, k1, k2).
void sort_triples(std::vector<Triple>& t) {
  __gnu_parallel::sort(t.begin(), t.end(), [](const Triple& x, const Triple& y) {
    if (x.k0 != y.k0) return x.k0 < y.k0;
    if (x.k1 != y.k1) return x.k1 < y.k1;
    return x.k2 < y.k2;
  });
}

// reduce_by_key over the first key with constant 1, then exclusive scan:
// distinct values and the row where each run starts (VedasStorage.cu:280-287).
void level1(const std::vector<Triple>& t, Vec& values, Vec& offsets) {
  values.clear();
  offsets.clear();
  for (size_t i = 0; i < t.size(); ++i)
    if (i == 0 || t[i].k0 != t[i - 1].k0) {
      values.push_back(t[i].k0);
      offsets.push_back(static_cast<ID>(i));
    }
}

// reduce_by_key over (k0, k1): second key of each run and its start row
// (VedasStorage.cu:342-355; offsets are 32-bit there).
void level2(const std::vector<Triple>& t, Vec& values2, Vec& offsets2) {
  values2.clear();
  offsets2.clear();
  for (size_t i = 0; i < t.size(); ++i)
    if (i == 0 || t[i].k0 != t[i - 1].k0 || t[i].k1 != t[i - 1].k1) {
      values2.push_back(t[i].k1);
      offsets2.push_back(static_cast<ID>(i));
    }
}

void column(const std::vector<Triple>& t, int which, Vec& out) {
  out.resize(t.size());
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < static_cast<long long>(t.size()); ++i)
    out[i] = which == 0 ? t[i].k0 : (which == 1 ? t[i].k1 : t[i].k2);
}

std::unique_ptr<Index> build_index(const ID* s, const ID* p, const ID* o, uint64_t n, bool full) {
  auto ix = std::make_unique<Index>();
  ix->full = full;
  std::vector<Triple> t(n);
  // PSO (VedasStorage.cu:41-44): sort (p,s,o); L1 over p; ps_data = s, pso_data = o;
  // L2 over (p,s).
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < static_cast<long long>(n); ++i) t[i] = {p[i], s[i], o[i]};
  sort_triples(t);
  level1(t, ix->a("p_idx_values"), ix->a("p_idx_offsets"));
  column(t, 1, ix->a("ps_data"));
  column(t, 2, ix->a("pso_data"));
  level2(t, ix->a("ps_s_idx_values"), ix->a("ps_idx_offsets"));
  // POS (VedasStorage.cu:45-48): sort (p,o,s); L1 kept from PSO; po_data = o,
  // pos_data = s; L2 over (p,o).
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < static_cast<long long>(n); ++i) t[i] = {p[i], o[i], s[i]};
  sort_triples(t);
  column(t, 1, ix->a("po_data"));
  column(t, 2, ix->a("pos_data"));
  level2(t, ix->a("po_o_idx_values"), ix->a("po_idx_offsets"));
  if (full) {
    // SPO / SOP (VedasStorage.cu:59-62): the subject L1 is never filled (its
    // code is commented out at VedasStorage.cu:319-339), so s_idx_* stay empty.
    ix->a("s_idx_values");
    ix->a("s_idx_offsets");
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < static_cast<long long>(n); ++i) t[i] = {s[i], p[i], o[i]};
    sort_triples(t);
    column(t, 2, ix->a("spo_data"));
    level2(t, ix->a("sp_p_idx_values"), ix->a("sp_idx_offsets"));
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < static_cast<long long>(n); ++i) t[i] = {s[i], o[i], p[i]};
    sort_triples(t);
    column(t, 2, ix->a("sop_data"));
    level2(t, ix->a("so_o_idx_values"), ix->a("so_idx_offsets"));
    // OS / OPS (VedasStorage.cu:65-69): L1 over o from the (o,s,p) order.
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < static_cast<long long>(n); ++i) t[i] = {o[i], s[i], p[i]};
    sort_triples(t);
    level1(t, ix->a("o_idx_values"), ix->a("o_idx_offsets"));
    column(t, 1, ix->a("os_data"));
    column(t, 2, ix->a("osp_data"));
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < static_cast<long long>(n); ++i) t[i] = {o[i], p[i], s[i]};
    sort_triples(t);
    column(t, 2, ix->a("ops_data"));
    level2(t, ix->a("op_p_idx_values"), ix->a("op_idx_offsets"));
  }
  return ix;
}

// ---------------------------------------------------------------------------
// Query text (the SPARQL basic-graph-pattern subset) -> patterns.
// Pattern fields follow TriplePattern (src/TriplePattern.cu:49-88).
// ---------------------------------------------------------------------------
struct Pattern {
  bool var[3] = {false, false, false};
  std::string name[3];
  ID id[3] = {0, 0, 0};
  size_t estimate_rows = 0;
  size_t nvars() const { return var[0] + var[1] + var[2]; }
  size_t bitmap() const { return var[0] * 4 + var[1] * 2 + var[2]; }
  bool has_var(const std::string& v) const {
    for (int k = 0; k < 3; ++k)
      if (var[k] && name[k] == v) return true;
    return false;
  }
};

struct Query {
  std::vector<Pattern> patterns;
  std::map<std::string, int> vars_count;   // SparqlQuery.cu:65-67
  std::set<std::string> selected;          // SparqlQuery.cu:76-81
};

Query parse_query(const std::string& text) {
  Query q;
  std::vector<std::string> toks;
  for (size_t i = 0; i < text.size();) {
    char c = text[i];
    if (std::isspace(static_cast<unsigned char>(c))) {
      ++i;
      continue;
    }
    size_t b = i;
    if (c == '<') {
      size_t e = text.find('>', i);
      if (e == std::string::npos) throw OracleParse("unterminated <");
      i = e + 1;
    } else if (c == '"') {
      size_t e = text.find('"', i + 1);
      if (e == std::string::npos) throw OracleParse("unterminated \"");
      i = e + 1;
    } else if (c == '{' || c == '}' || c == '.' || c == '*') {
      ++i;
    } else {
      while (i < text.size() && !std::isspace(static_cast<unsigned char>(text[i])) &&
             text[i] != '{' && text[i] != '}' && text[i] != '.')
        ++i;
    }
    toks.push_back(text.substr(b, i - b));
  }
  size_t k = 0;
  bool star = false;
  std::vector<std::string> proj, order;
  auto note = [&](const std::string& v) {
    if (std::find(order.begin(), order.end(), v) == order.end()) order.push_back(v);
  };
  for (; k < toks.size() && toks[k] != "{"; ++k) {
    std::string up = toks[k];
    for (auto& ch : up) ch = static_cast<char>(std::toupper(static_cast<unsigned char>(ch)));
    if (up == "SELECT" || up == "WHERE" || up == "DISTINCT") continue;
    if (toks[k] == "*") star = true;
    else if (toks[k][0] == '?') {
      proj.push_back(toks[k]);
      note(toks[k]);
    } else
      throw OracleParse("unexpected token " + toks[k]);
  }
  if (k == toks.size()) throw OracleParse("missing {");
  ++k;
  std::vector<std::string> t3;
  for (; k < toks.size() && toks[k] != "}"; ++k) {
    if (toks[k] == ".") continue;
    t3.push_back(toks[k]);
    if (t3.size() == 3) {
      Pattern p;
      for (int j = 0; j < 3; ++j) {
        const std::string& t = t3[j];
        if (t[0] == '?') {
          p.var[j] = true;
          p.name[j] = t;
          note(t);
        } else if (t[0] == '<' || t[0] == '"') {
          p.id[j] = static_cast<ID>(std::strtoul(t.substr(1, t.size() - 2).c_str(), nullptr, 10));
        } else {
          throw OracleParse("bad term " + t);
        }
      }
      for (int j = 0; j < 3; ++j)
        if (p.var[j]) q.vars_count[p.name[j]] += 1;
      q.patterns.push_back(p);
      t3.clear();
    }
  }
  if (!t3.empty()) throw OracleParse("incomplete triple");
  if (q.patterns.empty()) throw OracleParse("no triple patterns");
  if (star)
    for (auto& v : order) q.selected.insert(v);
  else
    for (auto& v : proj) q.selected.insert(v);
  return q;
}

// ---------------------------------------------------------------------------
// Relation (src/FullRelationIR.h:10-47): column-major, headers, column map.
// ---------------------------------------------------------------------------
struct Relation {
  std::vector<Vec> col;
  std::vector<std::string> head;
  std::unordered_map<std::string, size_t> colmap;

  Relation() = default;
  Relation(size_t ncols, size_t nrows) : col(ncols, Vec(nrows)), head(ncols) {}
  size_t rows() const { return col.empty() ? 0 : col[0].size(); }
  size_t ncols() const { return head.size(); }
  void set_header(size_t i, const std::string& h) {  // FullRelationIR.cu:556-560
    head[i] = h;
    colmap[h] = i;
  }
  size_t column_of(const std::string& v) const {  // FullRelationIR.cu:533-536
    auto it = colmap.find(v);
    if (it == colmap.end()) throw OracleUB("getColumnId assert: no column " + v);
    return it->second;
  }
  void swap_columns(size_t i, size_t j) {  // FullRelationIR.cu:715-727
    if (i == j) return;
    std::swap(col[i], col[j]);
    std::swap(head[i], head[j]);
    colmap[head[i]] = i;
    colmap[head[j]] = j;
  }
  void remove_column(size_t i) {  // FullRelationIR.cu:729-736
    col.erase(col.begin() + static_cast<long>(i));
    head.erase(head.begin() + static_cast<long>(i));
    for (size_t k = i; k < head.size(); ++k) colmap[head[k]] = k;
  }
  void remove_column(size_t i, const std::string& keep) {  // FullRelationIR.cu:738-745
    remove_column(i);
    if (i == 0) {
      swap_columns(0, column_of(keep));
      sort_by_first();
    }
  }
  // Key-only sort by column 0 carrying the other columns; Thrust's comparison
  // sort (FullRelationIR.cu:594-713) is a stable merge sort, so equal keys
  // keep their order.  One column: plain sort (FullRelationIR.cu:598).
  void sort_by_first() {
    size_t n = rows();
    if (ncols() == 1) {
      __gnu_parallel::sort(col[0].begin(), col[0].end());
      return;
    }
    std::vector<uint64_t> kv(n);
#pragma omp parallel for schedule(static)
    for (long long r = 0; r < static_cast<long long>(n); ++r)
      kv[r] = (static_cast<uint64_t>(col[0][r]) << 32) | static_cast<uint64_t>(r);
    // (key, original row) is a total order equal to a stable sort by key.
    __gnu_parallel::sort(kv.begin(), kv.end());
    for (auto& c : col) {
      Vec out(n);
#pragma omp parallel for schedule(static)
      for (long long r = 0; r < static_cast<long long>(n); ++r) out[r] = c[kv[r] & 0xFFFFFFFFu];
      c.swap(out);
    }
  }
  // Full lexicographic sort over all columns (FullRelationIR.cu:218-336).
  void sort_all() {
    size_t n = rows(), k = ncols();
    if (k <= 1) return;  // case 1 is a no-op in the reference
    std::vector<uint64_t> perm(n);
    for (size_t r = 0; r < n; ++r) perm[r] = r;
    __gnu_parallel::stable_sort(perm.begin(), perm.end(), [&](uint64_t a, uint64_t b) {
      for (size_t c = 0; c < k; ++c)
        if (col[c][a] != col[c][b]) return col[c][a] < col[c][b];
      return false;
    });
    for (auto& c : col) {
      Vec out(n);
      for (size_t r = 0; r < n; ++r) out[r] = c[perm[r]];
      c.swap(out);
    }
  }
  // Adjacent duplicate removal over all columns (FullRelationIR.cu:338-522).
  void remove_duplicates() {
    size_t n = rows(), k = ncols();
    if (n == 0) return;
    size_t w = 1;
    for (size_t r = 1; r < n; ++r) {
      bool same = true;
      for (size_t c = 0; c < k && same; ++c) same = col[c][r] == col[c][w - 1];
      if (!same) {
        for (size_t c = 0; c < k; ++c) col[c][w] = col[c][r];
        ++w;
      }
    }
    for (auto& c : col) c.resize(w);
  }
};

// ---------------------------------------------------------------------------
// Bounds and empty-interval dictionary.
// ---------------------------------------------------------------------------
using BoundMap = std::map<std::string, std::pair<ID, ID>>;

// QueryExecutor::updateBoundDict (src/QueryExecutor.cu:583-594).
void update_bound(BoundMap& bound, const std::string& v, ID lo, ID hi) {
  auto cur = bound[v];
  if (hi < cur.first || lo > cur.second) lo = hi = 0;
  ID nmin = (lo == 0) ? 0 : std::max(cur.first, lo);
  ID nmax = std::min(cur.second, hi);
  bound[v] = {nmin, nmax};
}

using Quad = std::tuple<size_t, size_t, size_t, size_t>;

struct EmptyIntervals {
  std::unordered_map<std::string, Quad> dict;

  // EmptyIntervalDict::updateBound (src/EmptyIntervalDict.cu:33-106), with
  // its merge rule as written: an overlapping pair takes the later interval's
  // end (not the max), and with more than two intervals left the two longest
  // by (end - start) in size_t arithmetic are kept.
  void update(const std::string& v, size_t lb1, size_t ub1, size_t lb2, size_t ub2) {
    auto it = dict.find(v);
    if (it == dict.end()) {
      dict[v] = Quad(lb1, ub1, lb2, ub2);
      return;
    }
    Quad old = it->second;
    std::vector<std::pair<size_t, size_t>> iv = {{std::get<0>(old), std::get<1>(old)},
                                                 {std::get<2>(old), std::get<3>(old)},
                                                 {lb1, ub1},
                                                 {lb2, ub2}};
    std::sort(iv.begin(), iv.end());
    for (size_t pi = iv.size() - 1; pi >= 1; --pi) {
      if (iv[pi].first <= iv[pi - 1].second) {
        iv[pi - 1].second = iv[pi].second;
        iv.erase(iv.begin() + static_cast<long>(pi));
      }
    }
    if (iv.size() == 1) {
      dict[v] = Quad(0, 0, iv[0].first, iv[0].second);
    } else if (iv.size() == 2) {
      dict[v] = Quad(iv[0].first, iv[0].second, iv[1].first, iv[1].second);
    } else {
      size_t best = 0, second = 0, bi = 0, si = 0;
      for (size_t i = 0; i < iv.size(); ++i) {
        size_t d = iv[i].second - iv[i].first;
        if (d > best) {
          second = best;
          si = bi;
          best = d;
          bi = i;
        } else if (d > second) {
          second = d;
          si = i;
        }
      }
      if (bi > si)
        dict[v] = Quad(iv[si].first, iv[si].second, iv[bi].first, iv[bi].second);
      else
        dict[v] = Quad(iv[bi].first, iv[bi].second, iv[si].first, iv[si].second);
    }
  }

  // EmptyIntervalDict::getUploadRelationData (src/EmptyIntervalDict.cu:108-170):
  // the slice [start, end) of `data` minus the two empty intervals of `v`, as
  // (source begin, source end, destination offset) pieces.
  struct Piece {
    size_t b, e, dst;
  };
  std::vector<Piece> pieces(const std::string& v, const Vec& data, size_t start, size_t end,
                            size_t& total) {
    Quad q = dict[v];  // operator[]: an unknown variable gets (0,0,0,0)
    size_t lb1 = std::get<0>(q), ub1 = std::get<1>(q), lb2 = std::get<2>(q), ub2 = std::get<3>(q);
    if (!(lb1 == 0 || ub1 == 0 || lb1 != ub1) || !(lb2 == 0 || ub2 == 0 || lb2 != ub2))
      throw OracleUB("EmptyIntervalDict assert: degenerate interval for " + v);
    const ID* base = data.data();
    auto lb = [&](size_t x) {
      return static_cast<size_t>(std::lower_bound(base + start, base + end, x,
                                                  [](ID a, size_t b) { return a < b; }) - base);
    };
    auto ub = [&](size_t x) {
      return static_cast<size_t>(std::upper_bound(base + start, base + end, x,
                                                  [](size_t a, ID b) { return a < b; }) - base);
    };
    std::vector<Piece> out;
    if (ub2 == 0 && ub1 == 0) {
      out.push_back({start, end, 0});
      total = end - start;
    } else if (ub1 == 0) {
      size_t o1 = lb(lb2), o2 = ub(ub2);
      out.push_back({start, o1, 0});
      out.push_back({o2, end, o1 - start});
      total = (o1 - start) + (end - o2);
    } else {
      size_t o1 = lb(lb1), o2 = ub(ub1), o3 = lb(lb2), o4 = ub(ub2);
      out.push_back({start, o1, 0});
      if (o2 != o3) {
        if (o2 > o3) throw OracleUB("EmptyIntervalDict: negative-length upload piece for " + v);
        out.push_back({o2, o3, o1 - start});
      }
      if (o4 > end) throw OracleUB("EmptyIntervalDict: piece past the slice");
      size_t mid = (o2 != o3) ? (o3 - o2) : 0;
      out.push_back({o4, end, (o1 - start) + mid});
      total = (o1 - start) + mid + (end - o4);
    }
    return out;
  }
};

// ---------------------------------------------------------------------------
// Index lookups (src/QueryExecutor.cu:596-646).
// ---------------------------------------------------------------------------
std::pair<size_t, size_t> l1_range(const Vec& l1v, const Vec& l1o, ID id, size_t n) {
  if (l1v.empty()) return {0, 0};
  size_t s = std::lower_bound(l1v.begin(), l1v.end(), id) - l1v.begin();
  if (s >= l1o.size()) throw OracleUB("findL2OffsetFromL1 reads past the L1 index");
  size_t e = s + 1;
  size_t lo = l1o[s];
  size_t hi = (e == l1o.size()) ? n : l1o[e];
  return {lo, hi};
}

std::pair<size_t, size_t> l2_range_index(const Vec& l2v, const Vec& l2o, ID lo, ID hi, ID id2) {
  if (l2o.empty()) return {0, 0};
  size_t b = std::lower_bound(l2o.begin(), l2o.end(), lo) - l2o.begin();
  size_t e = std::lower_bound(l2o.begin(), l2o.end(), hi) - l2o.begin();
  size_t s2 = std::lower_bound(l2v.begin() + b, l2v.begin() + e, id2) - l2v.begin();
  size_t e2 = std::upper_bound(l2v.begin() + b, l2v.begin() + e, id2) - l2v.begin();
  if (s2 >= l2o.size() || e2 >= l2o.size())
    throw OracleUB("findDataOffsetFromL2 (index form) reads past the L2 offsets");
  return {l2o[s2], l2o[e2]};
}

std::pair<size_t, size_t> l2_range_data(const Vec& d, size_t lo, size_t hi, ID id2) {
  size_t s = std::lower_bound(d.begin() + lo, d.begin() + hi, id2) - d.begin();
  size_t e = std::upper_bound(d.begin() + lo, d.begin() + hi, id2) - d.begin();
  return {s, e};
}

// ---------------------------------------------------------------------------
// Plan tree (src/PlanTreeNode.h) and planner (src/QueryGraph.cu).  The
// planner's tie-breaks follow std::unordered_map iteration order, so the same
// container types receive the same operations in the same order.
// ---------------------------------------------------------------------------
enum class Op { Upload, Join, Swap };
struct PlanNode {
  Op op;
  PlanNode* c1 = nullptr;
  PlanNode* c2 = nullptr;
  bool reuse = false;
  int tp = -1;
  std::string var;
};

struct Edge {
  std::string id, iv1, iv2;
  std::set<std::string> vars;
  int tp = -1;
  size_t card = 0;
  PlanNode* node = nullptr;
  bool has(const std::string& v) const { return vars.count(v) > 0; }
};

struct Planner {
  using Link = std::pair<std::string, Edge*>;
  std::unordered_map<std::string, std::vector<Link>> adj;
  std::vector<std::unique_ptr<Edge>> edges;
  std::vector<std::unique_ptr<PlanNode>>& nodes;

  Planner(const Query& q, std::vector<std::unique_ptr<PlanNode>>& pool) : nodes(pool) {
    // QueryGraph::QueryGraph (src/QueryGraph.cu:38-62) and GraphEdge (:20-32)
    for (size_t i = 0; i < q.patterns.size(); ++i) {
      const Pattern& tp = q.patterns[i];
      std::string s = tp.var[0] ? tp.name[0] : std::to_string(tp.id[0]);
      std::string o = tp.var[2] ? tp.name[2] : std::to_string(tp.id[2]);
      auto e = std::make_unique<Edge>();
      e->id = std::to_string(tp.id[1]);
      if (s[0] == '?') {
        e->vars.insert(s);
        e->iv1 = s;
      }
      if (o[0] == '?') {
        e->vars.insert(o);
        if (e->iv1.empty()) e->iv1 = o;
        else e->iv2 = o;
      }
      e->tp = static_cast<int>(i);
      e->card = tp.estimate_rows * tp.nvars();
      add_edge(s, o, e.get());
      edges.push_back(std::move(e));
    }
  }
  PlanNode* node(Op op) {
    nodes.push_back(std::make_unique<PlanNode>());
    nodes.back()->op = op;
    return nodes.back().get();
  }
  void add_edge(const std::string& a, const std::string& b, Edge* e) {
    adj[a].push_back({b, e});
    adj[b].push_back({a, e});
  }
  bool edge_exists(const std::string& a, const std::string& b) {
    for (auto& l : adj[a])
      if (l.first == b) return true;
    return false;
  }
  // QueryGraph::mergeEdge (src/QueryGraph.cu:97-117)
  void merge(const std::string end1, const std::string end2) {  // by value: the callers pass elements of a list this mutates
    for (auto l : adj[end2]) {
      // a self-loop: the reference would erase from the list it walks
      if (l.first == end2) throw OracleUB("planner: merging a variable joined to itself");
      if (!edge_exists(end1, l.first)) add_edge(end1, l.first, l.second);
      auto& other = adj[l.first];
      for (auto it = other.rbegin(); it != other.rend(); ++it) {
        if (it->first == end2) {
          other.erase(--(it.base()));
          break;
        }
      }
    }
    adj.erase(end2);
  }
  // QueryGraph::sameMaxDegAndTotalCard (src/QueryGraph.cu:126-154)
  std::tuple<size_t, size_t, std::string> best_var(const std::vector<Link>& links) {
    std::unordered_map<std::string, size_t> cnt, card;
    for (auto l : links) {
      for (auto v : l.second->vars) {
        if (cnt.count(v)) {
          cnt[v] += 1;
          card[v] += l.second->card;
        } else {
          cnt[v] = 1;
          card[v] = l.second->card;
        }
      }
    }
    size_t md = 0, mc = 0;
    std::string bv;
    for (auto c : cnt) {
      size_t est = card[c.first];
      if (c.second > md || (c.second == md && est < mc)) {
        md = c.second;
        mc = est;
        bv = c.first;
      }
    }
    return {md, mc, bv};
  }
  // QueryGraph::findBestStarNode (src/QueryGraph.cu:156-176)
  std::pair<std::string, std::string> best_star() {
    std::string bn, bj;
    size_t md = 0, mc = 0;
    for (auto nd : adj) {
      auto t = best_var(nd.second);
      size_t deg = std::get<0>(t), est = std::get<1>(t);
      if (deg > md || (deg == md && est < mc)) {
        md = deg;
        bn = nd.first;
        mc = est;
        bj = std::get<2>(t);
      }
    }
    return {bn, bj};
  }
  // QueryGraph::generateJoinPlanForNode (src/QueryGraph.cu:214-278)
  PlanNode* star(const std::string& vertex, const std::string& jv) {
    auto& L = adj[vertex];
    std::sort(L.begin(), L.end(),
              [](const Link& a, const Link& b) { return a.second->card < b.second->card; });
    size_t first = 0;
    while (first < L.size() && !L[first].second->has(jv)) ++first;
    if (first == L.size()) throw OracleUB("planner: no edge holds the join variable");
    size_t last = 0;
    for (size_t i = first; i < L.size(); ++i)
      if (L[i].second->has(jv)) last = i;
    for (size_t i = first; i < L.size(); ++i) {
      if (!L[i].second->has(jv)) continue;
      if (!L[i].second->node) {
        PlanNode* u = node(Op::Upload);
        u->tp = L[i].second->tp;
        u->var = jv;
        L[i].second->node = u;
      }
      if (i > first) {
        Edge* e1 = L[first].second;
        Edge* e2 = L[i].second;
        if (e1->iv1 != jv && e1->iv2 != jv) {
          PlanNode* s = node(Op::Swap);
          s->c1 = e1->node;
          s->var = jv;
          e1->node = s;
          e1->iv1 = jv;
          e1->iv2 = "";
        }
        if (e2->iv1 != jv && e2->iv2 != jv) {
          PlanNode* s = node(Op::Swap);
          s->c1 = e2->node;
          s->var = jv;
          e2->node = s;
        }
        PlanNode* j = node(Op::Join);
        j->c1 = e1->node;
        j->c2 = e2->node;
        j->var = jv;
        j->reuse = (i != last);
        e1->node = j;
        double sigma = 0.000001;
        if (e1->card < 1000 && e2->card < 1000) sigma = 0.001;
        else if (e1->card < 1000 || e2->card < 1000) sigma = 0.0001;
        e1->card *= std::ceil(e2->card * sigma);
        for (auto v : e2->vars) e1->vars.insert(v);
      }
    }
    // a merge can remove entries of this very list (two patterns between the
    // same two variables): the reference then reads past its end
    // (src/QueryGraph.cu:268-274), or erases the list itself (self-loop)
    for (int i = static_cast<int>(L.size()) - 1; i > static_cast<int>(first); --i) {
      if (static_cast<size_t>(i) >= L.size()) throw OracleUB("planner: a merge removed edges of its own star");
      if (!L[i].second->has(jv)) continue;
      if (L[i].first == vertex) throw OracleUB("planner: a star merges its own vertex");
      merge(L[first].first, L[i].first);
    }
    if (first >= L.size()) throw OracleUB("planner: a merge removed edges of its own star");
    L[first].second->iv1 = jv;
    L[first].second->iv2 = "";
    return L[first].second->node;
  }
  // QueryGraph::generateQueryPlan (src/QueryGraph.cu:64-74)
  PlanNode* plan() {
    PlanNode* root = nullptr;
    int guard = 0;
    while (adj.size() > 2) {
      if (++guard > 64) throw OracleUB("planner does not terminate on this query graph");
      auto st = best_star();
      root = star(st.first, st.second);
    }
    return root;
  }
};

// ---------------------------------------------------------------------------
// Jobs and execution (src/QueryExecutor.cu:106-135, :294-431; QueryPlan.cu).
// ---------------------------------------------------------------------------
struct LogRec {
  uint32_t op;  // 0 JOIN, 1 UPLOAD, 2 SWAP (src/vedas.h:87)
  uint64_t p1, p2, p3;
  std::string text;
};

std::string headers_joined(const Relation& r) {
  std::string s;
  for (auto& h : r.head) s += h;
  return s;
}

struct Job {
  enum Kind { Select, Join, Swap } kind;
  int tp = -1;            // select
  std::string index;      // select: "" | "PSO" | "POS"
  int left = -1, right = -1;
  std::string var;        // join / swap variable
  bool last_for_var = true;
  std::shared_ptr<Relation> ir;
};

struct Executor {
  const Index& ix;
  Query& q;
  BoundMap bound;
  EmptyIntervals eid;
  std::unordered_set<std::string> join_vars;
  std::map<std::string, size_t> counter;
  std::vector<Job> jobs;
  std::vector<LogRec> log;

  Executor(const Index& i, Query& qq) : ix(i), q(qq) {}

  size_t n() const { return ix.get("pso_data").size(); }

  // --- pre-scan: createVariableBound (QueryExecutor.cu:441-479) ---
  void prescan() {
    for (auto& c : q.vars_count)
      if (c.second > 1) {
        join_vars.insert(c.first);
        bound[c.first] = {0u, 0xFFFFFFFFu};
      }
    bool zero = false;
    for (auto& tp : q.patterns) {
      if (tp.nvars() == 1) squeeze1(tp);
      else if (tp.nvars() == 2) squeeze2(tp);
      zero = zero || tp.estimate_rows == 0;
    }
    if (zero)
      for (auto& jv : join_vars) bound[jv] = {0u, 0u};
  }

  // squeezeQueryBound1Var + updateDataBound (QueryExecutor.cu:527-581, :649-678),
  // partial index: the first lookup uses an S/O level-1 index, which is empty
  // without the full index, so only the predicate-index lookup runs.
  void squeeze1(Pattern& tp) {
    if (tp.var[1]) throw OracleUB("predicate variable needs the full index");
    const Vec& l1v = ix.get("p_idx_values");
    const Vec& l1o = ix.get("p_idx_offsets");
    const Vec& l2d = tp.var[0] ? ix.get("po_data") : ix.get("ps_data");
    const Vec& data = tp.var[0] ? ix.get("pos_data") : ix.get("pso_data");
    const std::string& v = tp.var[0] ? tp.name[0] : tp.name[2];
    ID id2 = tp.var[0] ? tp.id[2] : tp.id[0];
    if (l1v.empty()) return;
    auto r1 = l1_range(l1v, l1o, tp.id[1], data.size());
    auto r2 = l2_range_data(l2d, r1.first, r1.second, id2);
    tp.estimate_rows = r2.second - r2.first;
    // With an empty range the reference reads data[first] and data[second-1]
    // (one before the range, or before the array when second == 0); the
    // estimate is 0, so the pre-scan later overwrites every join bound with
    // (0,0) and the value read has no effect.  0 stands in for it here.
    ID lo = r2.first < data.size() ? data[r2.first] : 0;
    ID hi = r2.second >= 1 ? data[r2.second - 1] : 0;
    if (bound.count(v)) update_bound(bound, v, lo, hi);
  }

  // squeezeQueryBound2Var + updateL2Bound (QueryExecutor.cu:680-765), bitmap 5.
  // The level-1 lookup is passed the SOP array's size as n, which is 0 without
  // the full index, so the last predicate's range ends at 0.
  void squeeze2(Pattern& tp) {
    if (tp.bitmap() != 5) throw OracleUB("two-variable pattern needs the full index");
    size_t data_size = 0;  // getSOPdata()->size(): empty without the full index
    auto r1 = l1_range(ix.get("p_idx_values"), ix.get("p_idx_offsets"), tp.id[1], data_size);
    auto l2bound = [&](const std::string& v, const Vec& l2d) {
      size_t s = r1.first, e = r1.second;
      tp.estimate_rows = (e == 0) ? 0 : e - s;
      if (bound.count(v)) {
        // e == 0 reads l2d[-1] in the reference; the estimate is then 0 and
        // the value is overwritten by the zero-result rule (see squeeze1).
        ID lo = s < l2d.size() ? l2d[s] : 0;
        ID hi = (e >= 1 && e - 1 < l2d.size()) ? l2d[e - 1] : 0;
        update_bound(bound, v, lo, hi);
      }
    };
    if (join_vars.count(tp.name[2])) l2bound(tp.name[2], ix.get("po_data"));
    if (join_vars.count(tp.name[0])) l2bound(tp.name[0], ix.get("ps_data"));
  }

  // --- SelectQueryJob::startJob (src/SelectQueryJob.cu:86-270) ---
  std::shared_ptr<Relation> run_select(const Job& j) {
    const Pattern& tp = q.patterns[static_cast<size_t>(j.tp)];
    const Vec& l1v = ix.get("p_idx_values");
    const Vec& l1o = ix.get("p_idx_offsets");
    if (tp.nvars() == 1) {
      // create1VarSelectQueryJob (QueryExecutor.cu:781-860), partial index
      if (tp.var[1]) throw OracleUB("predicate variable needs the full index");
      bool subj = tp.var[0];
      const Vec& l2v = subj ? ix.get("po_o_idx_values") : ix.get("ps_s_idx_values");
      const Vec& l2o = subj ? ix.get("po_idx_offsets") : ix.get("ps_idx_offsets");
      const Vec& data = subj ? ix.get("pos_data") : ix.get("pso_data");
      const std::string& v = subj ? tp.name[0] : tp.name[2];
      ID id2 = subj ? tp.id[2] : tp.id[0];
      auto r1 = l1_range(l1v, l1o, tp.id[1], data.size());
      auto r2 = l2_range_index(l2v, l2o, static_cast<ID>(r1.first), static_cast<ID>(r1.second), id2);
      if (r2.first > r2.second) r2.second = r2.first;
      size_t rows = r2.second - r2.first;
      auto ir = std::make_shared<Relation>(1, rows);
      ir->set_header(0, v);
      std::copy(data.begin() + r2.first, data.begin() + r2.second, ir->col[0].begin());
      log.push_back({1, rows, 1, 0, headers_joined(*ir)});
      if (bound.count(v)) {
        if (rows == 0) update_bound(bound, v, 0, 0);
        else update_bound(bound, v, data[r2.first], data[r2.second - 1]);
      }
      return ir;
    }
    if (tp.bitmap() != 5) throw OracleUB("two-variable pattern needs the full index");
    // create2VarSelectQueryJob case 5 (QueryExecutor.cu:904-934)
    bool pos = (j.index == "POS");
    const Vec& l2d = pos ? ix.get("po_data") : ix.get("ps_data");
    const Vec& data = pos ? ix.get("pos_data") : ix.get("pso_data");
    std::string v0 = pos ? tp.name[2] : tp.name[0];
    std::string v1 = pos ? tp.name[0] : tp.name[2];
    bool second_used = q.selected.count(v1) > 0 || bound.count(v1) > 0;
    auto r1 = l1_range(l1v, l1o, tp.id[1], data.size());
    size_t b0 = r1.first, e0 = r1.second;
    if (e0 == 0 || b0 >= l2d.size() || e0 > l2d.size())
      throw OracleUB("select reads outside the level-2 data");
    ID cur_min = l2d[b0], cur_max = l2d[e0 - 1];
    size_t first = b0, second = e0;
    if (bound.count(v0)) {
      auto bd = bound[v0];
      if (bd.first > cur_min)
        first = std::lower_bound(l2d.begin() + b0, l2d.begin() + e0, bd.first) - l2d.begin();
      if (bd.second < cur_max)
        second = std::upper_bound(l2d.begin() + b0, l2d.begin() + e0, bd.second) - l2d.begin();
    }
    size_t ds = first, de = second;
    if (ds > de) de = ds;
    if (!second_used) {
      if (first > second) throw OracleUB("select row count underflows");
      size_t row = second - first;
      auto ir = std::make_shared<Relation>(1, row);
      ir->set_header(0, v0);
      if (row > 0) {
        std::copy(l2d.begin() + first, l2d.begin() + second, ir->col[0].begin());
        ir->remove_duplicates();
      }
      log.push_back({1, row, 1, 0, headers_joined(*ir)});
      return ir;
    }
    size_t total = 0;
    auto pcs = eid.pieces(v0, l2d, ds, de, total);
    auto ir = std::make_shared<Relation>(2, total);
    ir->set_header(0, v0);
    ir->set_header(1, v1);
    log.push_back({1, total, 2, 0, headers_joined(*ir)});
    for (auto& pc : pcs) {
      if (pc.e < pc.b) throw OracleUB("negative upload piece");
      std::copy(l2d.begin() + pc.b, l2d.begin() + pc.e, ir->col[0].begin() + pc.dst);
      std::copy(data.begin() + pc.b, data.begin() + pc.e, ir->col[1].begin() + pc.dst);
    }
    return ir;
  }

  // Empty-interval scan over column 0 (JoinQueryJob.cu:398-433 and
  // IndexSwapJob.cu:81-118): the largest gap's neighbourhood of at most six
  // values, then the two largest gaps with the reference's >=/> rule and
  // zero-initialised gap bounds, updated with 32-bit wrapping arithmetic.
  void eif_scan(const Vec& c0, const std::string& var) {
    size_t n = c0.size();
    size_t pos = 0;
    ID best = 0;
    for (size_t k = 0; k + 1 < n; ++k) {
      ID d = c0[k + 1] - c0[k];
      if (k == 0 || d > best) {
        best = d;
        pos = k;
      }
    }
    size_t sc = pos >= 2 ? pos - 2 : 0;
    size_t ec = std::min(pos + 4, n);
    ID v[6];
    size_t sz = ec - sc;
    for (size_t i = 0; i < sz; ++i) v[i] = c0[sc + i];
    ID b[4] = {0, 0, 0, 0};
    size_t m1 = 0, m2 = 0;
    for (size_t i = 1; i < sz; ++i) {
      ID d = v[i] - v[i - 1];
      if (d >= m1) {
        m2 = m1;
        b[0] = b[2];
        b[1] = b[3];
        m1 = d;
        b[2] = v[i - 1];
        b[3] = v[i];
      } else if (d > m2) {
        m2 = d;
        b[0] = v[i - 1];
        b[1] = v[i];
      }
    }
    if (b[2] < b[0]) {
      std::swap(b[0], b[2]);
      std::swap(b[1], b[3]);
    }
    eid.update(var, static_cast<ID>(b[0] + 1u), static_cast<ID>(b[1] - 1u),
               static_cast<ID>(b[2] + 1u), static_cast<ID>(b[3] - 1u));
  }

  // --- JoinQueryJob::join (src/JoinQueryJob.cu:125-453) ---
  std::shared_ptr<Relation> run_join(const Job& j) {
    std::shared_ptr<Relation> L = jobs[static_cast<size_t>(j.left)].ir;
    std::shared_ptr<Relation> R = jobs[static_cast<size_t>(j.right)].ir;
    if (L->rows() > R->rows()) std::swap(L, R);
    std::vector<std::string> jvs;
    {
      std::string cur;
      for (char c : j.var) {
        if (c == ',') {
          if (!cur.empty()) jvs.push_back(cur);
          cur.clear();
        } else
          cur += c;
      }
      if (!cur.empty()) jvs.push_back(cur);
    }
    if (jvs.size() != 1) throw OracleUB("multi-variable join is not emitted by the planner");
    const std::string& jv = jvs[0];
    size_t ncol = L->ncols() + R->ncols() - 1;
    for (int i = static_cast<int>(L->ncols()) - 1; i >= 0; --i)
      if (counter[L->head[static_cast<size_t>(i)]] == 0 && L->head[static_cast<size_t>(i)] != jv) {
        L->remove_column(static_cast<size_t>(i), jv);
        ncol -= 1;
      }
    for (int i = static_cast<int>(R->ncols()) - 1; i >= 0; --i)
      if (counter[R->head[static_cast<size_t>(i)]] == 0 && R->head[static_cast<size_t>(i)] != jv) {
        R->remove_column(static_cast<size_t>(i), jv);
        ncol -= 1;
      }
    counter[jv] -= 1;
    size_t lj = L->column_of(jv), rj = R->column_of(jv);
    if (lj != 0) {
      L->swap_columns(0, lj);
      L->sort_by_first();
      log.push_back({2, L->rows(), L->ncols(), 0, ""});
    }
    if (rj != 0) {
      R->swap_columns(0, rj);
      R->sort_by_first();
      log.push_back({2, R->rows(), R->ncols(), 0, ""});
    }
    size_t ls = L->ncols(), rs = R->ncols();
    auto header_out = [&](Relation& out) {
      size_t h = 0;
      out.set_header(h++, L->head[0]);
      for (size_t i = 1; i < ls; ++i) out.set_header(h++, L->head[i]);
      for (size_t i = 1; i < rs; ++i) out.set_header(h++, R->head[i]);
    };
    if (L->rows() == 0 || R->rows() == 0) {
      auto out = std::make_shared<Relation>(ncol, 0);
      header_out(*out);
      log.push_back({0, L->rows(), R->rows(), 0, headers_joined(*L) + " x " + headers_joined(*R)});
      return out;
    }
    const Vec& a = L->col[0];
    const Vec& b = R->col[0];
    size_t na = a.size();
    std::vector<size_t> lo(na), cnt(na + 1);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < static_cast<long long>(na); ++i) {
      lo[i] = std::lower_bound(b.begin(), b.end(), a[i]) - b.begin();
      cnt[i] = (std::upper_bound(b.begin(), b.end(), a[i]) - b.begin()) - lo[i];
    }
    size_t total = 0;
    for (size_t i = 0; i < na; ++i) {
      size_t c = cnt[i];
      cnt[i] = total;
      total += c;
    }
    cnt[na] = total;
    if (total > static_cast<size_t>(INT_MAX)) throw OracleUB("join output exceeds int indices");
    auto out = std::make_shared<Relation>(ncol, total);
    header_out(*out);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < static_cast<long long>(na); ++i) {
      size_t k = cnt[i];
      for (size_t jj = lo[i]; k < cnt[i + 1]; ++jj, ++k) {
        size_t c = 0;
        out->col[c++][k] = a[i];
        for (size_t x = 1; x < ls; ++x) out->col[c++][k] = L->col[x][i];
        for (size_t x = 1; x < rs; ++x) out->col[c++][k] = R->col[x][jj];
      }
    }
    log.push_back({0, L->rows(), R->rows(), total, headers_joined(*L) + " x " + headers_joined(*R)});
    // ENABLE_UPDATE_BOUND_AFTER_JOIN (true in vdQuery, src/VedasQuery.cu:37)
    if (total > 0) {
      update_bound(bound, j.var, out->col[0][0], out->col[0][total - 1]);
      if (!j.last_for_var && total > 2 && total < 100) eif_scan(out->col[0], j.var);
    } else {
      update_bound(bound, j.var, 0, 0);
    }
    return out;
  }

  // --- IndexSwapJob::startJob (src/IndexSwapJob.cu:28-95) ---
  std::shared_ptr<Relation> run_swap(const Job& j) {
    std::shared_ptr<Relation> ir = jobs[static_cast<size_t>(j.left)].ir;
    size_t c = ir->column_of(j.var);
    ir->swap_columns(0, c);
    ir->sort_by_first();
    log.push_back({2, ir->rows(), ir->ncols(), 0, ir->head[0] + " <-> " + ir->head[c]});
    if (ir->rows() > 2 && ir->rows() < 100) eif_scan(ir->col[0], ir->head[0]);
    return ir;
  }

  // QueryExecutor::postorderTraversal (src/QueryExecutor.cu:106-135)
  int emit(PlanNode* nd) {
    if (!nd) return -1;
    int j1 = -1, j2 = -1;
    if (nd->c1) j1 = emit(nd->c1);
    if (nd->c2) j2 = emit(nd->c2);
    Job jb;
    switch (nd->op) {
      case Op::Upload: {
        jb.kind = Job::Select;
        jb.tp = nd->tp;
        const Pattern& tp = q.patterns[static_cast<size_t>(nd->tp)];
        if (tp.nvars() == 2) jb.index = (tp.var[0] && tp.name[0] == nd->var) ? "PSO" : "POS";
        else if (tp.nvars() != 1) throw OracleUB("three-variable pattern");
        break;
      }
      case Op::Join:
        jb.kind = Job::Join;
        jb.left = j1;
        jb.right = j2;
        jb.var = nd->var;
        jb.last_for_var = !nd->reuse;
        counter[nd->var] += 1;  // QueryPlan::pushJob (src/QueryPlan.cu:34-43)
        break;
      case Op::Swap:
        jb.kind = Job::Swap;
        jb.left = j1;
        jb.var = nd->var;
        break;
    }
    jobs.push_back(jb);
    return static_cast<int>(jobs.size()) - 1;
  }

  std::shared_ptr<Relation> run() {
    if (q.patterns.size() == 1) {
      // single pattern: one select with the default index (QueryExecutor.cu:305-312)
      const Pattern& tp = q.patterns[0];
      if (tp.nvars() == 3 || tp.nvars() == 0) throw OracleUB("unsupported single pattern");
      Job jb;
      jb.kind = Job::Select;
      jb.tp = 0;
      jobs.push_back(jb);
    } else {
      prescan();
      std::vector<std::unique_ptr<PlanNode>> pool;
      Planner pl(q, pool);
      PlanNode* root = pl.plan();
      if (!root) throw OracleUB("planner produced no plan (query graph has <= 2 vertices)");
      emit(root);
    }
    // QueryPlan::execute, single GPU (src/QueryPlan.cu:114-257)
    for (auto& sv : q.selected) counter[sv] = ULONG_MAX;
    for (auto& jb : jobs) {
      if (jb.kind == Job::Select) jb.ir = run_select(jb);
      else if (jb.kind == Job::Join) jb.ir = run_join(jb);
      else jb.ir = run_swap(jb);
    }
    std::shared_ptr<Relation> res = jobs.back().ir;
    for (int i = static_cast<int>(res->ncols()) - 1; i >= 1; --i)
      if (counter[res->head[static_cast<size_t>(i)]] == 0) res->remove_column(static_cast<size_t>(i));
    res->remove_duplicates();
    return res;
  }
};

}  // namespace

struct vo_index {
  std::unique_ptr<Index> ix;
};

struct vo_result {
  int status = 0;
  std::string error;
  std::shared_ptr<Relation> rel;
  std::vector<LogRec> log;
};

extern "C" {

vo_index* vo_index_build(const uint32_t* s, const uint32_t* p, const uint32_t* o, uint64_t n,
                         int full_index) {
  auto* h = new vo_index();
  h->ix = build_index(s, p, o, n, full_index != 0);
  return h;
}

void vo_index_free(vo_index* ix) { delete ix; }

int vo_index_array(const vo_index* h, const char* name, const uint32_t** data, uint64_t* len) {
  auto it = h->ix->arr.find(name);
  if (it == h->ix->arr.end()) return 1;
  *data = it->second.data();
  *len = it->second.size();
  return 0;
}

vo_result* vo_query(vo_index* h, const char* text) {
  auto* r = new vo_result();
  try {
    if (h->ix->full) throw std::runtime_error("queries are restated for the partial index only");
    Query q = parse_query(text);
    Executor ex(*h->ix, q);
    r->rel = ex.run();
    r->log = ex.log;
  } catch (const OracleParse& e) {
    r->status = 1;
    r->error = e.what();
  } catch (const OracleUB& e) {
    r->status = 2;
    r->error = e.what();
  } catch (const std::exception& e) {
    r->status = 3;
    r->error = e.what();
  }
  return r;
}

int vo_result_status(const vo_result* r) { return r->status; }
const char* vo_result_error(const vo_result* r) { return r->error.c_str(); }
uint32_t vo_result_ncols(const vo_result* r) {
  return r->rel ? static_cast<uint32_t>(r->rel->ncols()) : 0;
}
const char* vo_result_header(const vo_result* r, uint32_t c) { return r->rel->head[c].c_str(); }
uint64_t vo_result_nrows(const vo_result* r) { return r->rel ? r->rel->rows() : 0; }
const uint32_t* vo_result_column(const vo_result* r, uint32_t c) { return r->rel->col[c].data(); }
uint32_t vo_result_nlog(const vo_result* r) { return static_cast<uint32_t>(r->log.size()); }
void vo_result_log(const vo_result* r, uint32_t i, uint32_t* op, uint64_t* p1, uint64_t* p2,
                   uint64_t* p3, const char** text) {
  const LogRec& l = r->log[i];
  *op = l.op;
  *p1 = l.p1;
  *p2 = l.p2;
  *p3 = l.p3;
  *text = l.text.c_str();
}
void vo_result_free(vo_result* r) { delete r; }

// Plan description (post-order job list) for given per-pattern estimates:
// "U<tp>:<index>;" selects, "J<l>,<r>:<var>:<last>;" joins, "W<child>:<var>;" swaps.
int vo_plan_describe(const char* text, const uint64_t* est, uint32_t n, char* buf, uint64_t cap) {
  try {
    Query q = parse_query(text);
    for (uint32_t i = 0; i < n && i < q.patterns.size(); ++i) q.patterns[i].estimate_rows = est[i];
    std::vector<std::unique_ptr<PlanNode>> pool;
    Planner pl(q, pool);
    PlanNode* root = pl.plan();
    std::string s;
    int counter = 0;
    std::function<int(PlanNode*)> walk = [&](PlanNode* nd) -> int {
      if (!nd) return -1;
      int a = -1, b = -1;
      if (nd->c1) a = walk(nd->c1);
      if (nd->c2) b = walk(nd->c2);
      if (nd->op == Op::Upload) {
        const Pattern& tp = q.patterns[static_cast<size_t>(nd->tp)];
        std::string idx = "-";
        if (tp.nvars() == 2) idx = (tp.var[0] && tp.name[0] == nd->var) ? "PSO" : "POS";
        s += "U" + std::to_string(nd->tp) + ":" + idx + ";";
      } else if (nd->op == Op::Join) {
        s += "J" + std::to_string(a) + "," + std::to_string(b) + ":" + nd->var + ":" + (nd->reuse ? "0" : "1") + ";";
      } else {
        s += "W" + std::to_string(a) + ":" + nd->var + ";";
      }
      return counter++;
    };
    walk(root);
    if (s.size() + 1 > cap) return 3;
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return 0;
  } catch (const OracleParse&) {
    return 1;
  } catch (const OracleUB&) {
    return 2;
  }
}

// updateBound applied n times to one variable; out4 = the final entry.
int vo_eid_sequence(const uint64_t* quads, uint32_t n, uint64_t* out4) {
  EmptyIntervals e;
  for (uint32_t i = 0; i < n; ++i)
    e.update("?x", quads[4 * i], quads[4 * i + 1], quads[4 * i + 2], quads[4 * i + 3]);
  if (!e.dict.count("?x")) return 1;
  Quad qd = e.dict["?x"];
  out4[0] = std::get<0>(qd);
  out4[1] = std::get<1>(qd);
  out4[2] = std::get<2>(qd);
  out4[3] = std::get<3>(qd);
  return 0;
}

void vo_sort_by_first(uint32_t** cols, uint32_t ncols, uint64_t nrows) {
  Relation rel;
  rel.col.resize(ncols);
  rel.head.resize(ncols);
  for (uint32_t c = 0; c < ncols; ++c) rel.col[c].assign(cols[c], cols[c] + nrows);
  rel.sort_by_first();
  for (uint32_t c = 0; c < ncols; ++c) std::copy(rel.col[c].begin(), rel.col[c].end(), cols[c]);
}

uint64_t vo_inner_join(const uint32_t* a, uint64_t na, const uint32_t* b, uint64_t nb,
                       uint64_t* out_l, uint64_t* out_r) {
  uint64_t k = 0;
  for (uint64_t i = 0; i < na; ++i) {
    uint64_t lo = std::lower_bound(b, b + nb, a[i]) - b;
    uint64_t hi = std::upper_bound(b, b + nb, a[i]) - b;
    for (uint64_t j = lo; j < hi; ++j, ++k) {
      if (out_l) out_l[k] = i;
      if (out_r) out_r[k] = j;
    }
  }
  return k;
}

}  // extern "C"
