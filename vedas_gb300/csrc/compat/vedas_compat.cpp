// Host-side mirror of the reference's query path driving the GB300 kernels.
// Job semantics follow the reference files named at each function.
#include "vedas_compat.h"

#include <algorithm>
#include <cctype>
#include <climits>
#include <cmath>
#include <cstdlib>

namespace vedas {

bool QueryExecutor::ENABLE_UPDATE_BOUND_AFTER_JOIN = true;  // vdQuery default (src/VedasQuery.cu:37)

// ---------------------------------------------------------------------------
// VedasStorage
// ---------------------------------------------------------------------------
VedasStorage::VedasStorage(vg::Ctx* ctx, const TYPEID* s, const TYPEID* p, const TYPEID* o, size_t n,
                           bool inputs_on_device, bool fullIndex) {
  if (inputs_on_device) {
    vg::build_index(*ctx, s, p, o, n, fullIndex, ix_);
    cacheDevice();
    return;
  }
  vg::Scratch<uint32_t> ds(*ctx, n), dp(*ctx, n), dobj(*ctx, n);
  if (n) {
    VG_CUDA(cudaMemcpyAsync(ds.get(), s, n * 4, cudaMemcpyHostToDevice, ctx->stream));
    VG_CUDA(cudaMemcpyAsync(dp.get(), p, n * 4, cudaMemcpyHostToDevice, ctx->stream));
    VG_CUDA(cudaMemcpyAsync(dobj.get(), o, n * 4, cudaMemcpyHostToDevice, ctx->stream));
  }
  vg::build_index(*ctx, ds.get(), dp.get(), dobj.get(), n, fullIndex, ix_);
  cacheDevice();
  ctx->sync();
}

VedasStorage::VedasStorage(vg::Ctx* ctx, const char* fname, bool fullIndex) {
  vg::open_vds(*ctx, fname, fullIndex, ix_);
  cacheDevice();
}

void VedasStorage::cacheDevice() {
  for (int m = 0; m < kMirrors; ++m) d_[m] = ix_.get(kMirrorName[m]).ptr;
}

VedasStorage::~VedasStorage() { ix_.release(); }

void VedasStorage::write(const char* fname) { vg::write_vds(ix_, fname); }

const char* const VedasStorage::kMirrorName[VedasStorage::kMirrors] = {
    "p_idx_values", "p_idx_offsets", "ps_s_idx_values", "ps_idx_offsets", "po_o_idx_values", "po_idx_offsets",
    "ps_data",      "po_data",       "pso_data",        "pos_data",       "sop_data"};

void VedasStorage::prepareMirrors() {
  std::call_once(mirrors_once_, [this] {
    for (int m = 0; m < kMirrors; ++m) h(static_cast<Mirror>(m));
    for (int po = 0; po < 2; ++po) {
      l2r_[po] = QueryExecutor::l2RangesOfL1(*mirror_[kPIdxO], *mirror_[po ? kPOIdxO : kPSIdxO], ix_.n);
      const TYPEID_HOST_VEC& d = *mirror_[po ? kPO : kPS];
      fence_[po] = make_fences(d.data(), d.size());
    }
  });
}

// ---------------------------------------------------------------------------
// FullRelationIR (src/FullRelationIR.cu)
// ---------------------------------------------------------------------------
FullRelationIR::FullRelationIR(vg::Ctx* ctx, size_t columnNum, size_t relationSize) : ctx_(ctx) {
  r_ = vg::rel_alloc(*ctx, static_cast<uint32_t>(columnNum), relationSize);
  headers.resize(columnNum);
  var_column_map.v.reserve(columnNum + 1);
}

FullRelationIR::FullRelationIR(vg::Ctx* ctx, size_t columnNum, size_t relationSize, const TYPEID* const* views)
    : ctx_(ctx) {
  if (columnNum > VG_MAX_COLS) throw vg::Error(VG_ERR_UNSUPPORTED, "more than 9 columns");
  r_.ncols = static_cast<uint32_t>(columnNum);
  r_.nrows = relationSize;
  for (size_t c = 0; c < columnNum; ++c) r_.cols[c] = const_cast<TYPEID*>(views[c]);
  r_.borrowed = (1u << columnNum) - 1u;
  headers.resize(columnNum);
  var_column_map.v.reserve(columnNum + 1);
}

FullRelationIR::~FullRelationIR() { vg::rel_free(*ctx_, r_); }

void FullRelationIR::adopt(vg::Rel& r) {
  vg::rel_free(*ctx_, r_);
  r_ = r;
  r = vg::Rel();
}

vg::Rel FullRelationIR::release() {
  vg::Rel r = r_;
  r_ = vg::Rel();
  return r;
}

size_t FullRelationIR::getColumnId(const std::string& var) const {
  const size_t* c = var_column_map.find(var);
  if (!c) throw ReferenceUB("getColumnId: no column for " + var);
  return *c;
}

void FullRelationIR::setHeader(size_t i, const std::string& h, bool is_predicate) {
  headers[i] = h;
  var_column_map[h] = i;
  is_predicates[i] = is_predicate;
}

std::string FullRelationIR::getHeaders(const std::string& d) const {
  if (headers.empty()) return "";
  std::string s = headers[0];
  for (size_t i = 1; i < headers.size(); ++i) s += d + headers[i];
  return s;
}

void FullRelationIR::sort() { vg::sort_rows(*ctx_, r_); }
void FullRelationIR::removeDuplicate() { vg::unique_in_place(*ctx_, r_); }
void FullRelationIR::sortByFirstColumn() { vg::sort_by_first(*ctx_, r_); }

void FullRelationIR::swapColumn(size_t i, size_t j) {  // src/FullRelationIR.cu:715-727
  if (i == j) return;
  std::swap(r_.cols[i], r_.cols[j]);
  const uint32_t bi = r_.borrowed >> i & 1u, bj = r_.borrowed >> j & 1u;
  r_.borrowed = (r_.borrowed & ~((1u << i) | (1u << j))) | (bi << j) | (bj << i);
  bool t = is_predicates[i];
  is_predicates[i] = is_predicates[j];
  is_predicates[j] = t;
  std::swap(headers[i], headers[j]);
  var_column_map[headers[i]] = i;
  var_column_map[headers[j]] = j;
}

void FullRelationIR::removeColumn(size_t i) {  // src/FullRelationIR.cu:729-736
  vg::rel_drop_col(*ctx_, r_, static_cast<uint32_t>(i));
  // columns above i move down one place, with their ownership bits
  const uint32_t low = r_.borrowed & ((1u << i) - 1u);
  r_.borrowed = low | ((r_.borrowed >> (i + 1)) << i);
  for (size_t k = i; k + 1 < r_.ncols; ++k) r_.cols[k] = r_.cols[k + 1];
  r_.cols[r_.ncols - 1] = nullptr;
  r_.ncols -= 1;
  for (size_t k = i; k + 1 < VG_MAX_COLS; ++k) is_predicates[k] = is_predicates[k + 1];
  is_predicates[VG_MAX_COLS - 1] = false;
  headers.erase(headers.begin() + static_cast<long>(i));
  for (size_t k = i; k < headers.size(); ++k) var_column_map[headers[k]] = k;
}

void FullRelationIR::removeColumn(size_t i, const std::string& maintain_var) {  // :738-745
  if (removeColumnDeferSort(i, maintain_var)) sortByFirstColumn();
}

bool FullRelationIR::removeColumnDeferSort(size_t i, const std::string& maintain_var) {
  removeColumn(i);
  if (i != 0) return false;
  swapColumn(0, getColumnId(maintain_var));
  return true;
}

// ---------------------------------------------------------------------------
// EmptyIntervalDict (src/EmptyIntervalDict.cu)
// ---------------------------------------------------------------------------
size_t EmptyIntervalDict::emptySize(const std::string& var) {
  auto& t = dict[var];
  return (std::get<1>(t) - std::get<0>(t)) + (std::get<3>(t) - std::get<2>(t));
}

// Merge rule as written at src/EmptyIntervalDict.cu:33-106: overlapping
// neighbours take the later interval's end; with more than two intervals the
// two with the largest (end - start) in size_t arithmetic are kept.
void EmptyIntervalDict::updateBound(const std::string& var, size_t lb1, size_t ub1, size_t lb2, size_t ub2) {
  if (!hasBoundFor(var)) {
    dict[var] = std::make_tuple(lb1, ub1, lb2, ub2);
    return;
  }
  const VAR_BOUND old = dict.at(var);
  std::vector<std::pair<size_t, size_t>> iv;
  iv.push_back({std::get<0>(old), std::get<1>(old)});
  iv.push_back({std::get<2>(old), std::get<3>(old)});
  iv.push_back({lb1, ub1});
  iv.push_back({lb2, ub2});
  std::sort(iv.begin(), iv.end());
  for (size_t p = iv.size() - 1; p >= 1; --p) {
    if (iv[p].first <= iv[p - 1].second) {
      iv[p - 1].second = iv[p].second;
      iv.erase(iv.begin() + static_cast<long>(p));
    }
  }
  if (iv.size() == 1) {
    dict[var] = std::make_tuple(size_t(0), size_t(0), iv[0].first, iv[0].second);
  } else if (iv.size() == 2) {
    dict[var] = std::make_tuple(iv[0].first, iv[0].second, iv[1].first, iv[1].second);
  } else {
    size_t maxD = 0, secD = 0, maxI = 0, secI = 0;
    for (size_t i = 0; i < iv.size(); ++i) {
      size_t d = iv[i].second - iv[i].first;
      if (d > maxD) {
        secD = maxD;
        secI = maxI;
        maxD = d;
        maxI = i;
      } else if (d > secD) {
        secD = d;
        secI = i;
      }
    }
    if (maxI > secI)
      dict[var] = std::make_tuple(iv[secI].first, iv[secI].second, iv[maxI].first, iv[maxI].second);
    else
      dict[var] = std::make_tuple(iv[maxI].first, iv[maxI].second, iv[secI].first, iv[secI].second);
  }
}

// src/EmptyIntervalDict.cu:108-170 with absolute offsets into `data`.
void EmptyIntervalDict::getUploadRelationData(const std::string& var, const TYPEID* data, size_t start,
                                              size_t end, size_t& relationSize,
                                              std::vector<std::pair<size_t, size_t>>& up,
                                              std::vector<size_t>& offsets, const std::vector<uint32_t>* fences) {
  up.clear();
  offsets.clear();
  VAR_BOUND& t = dict[var];
  const size_t lb1 = std::get<0>(t), ub1 = std::get<1>(t), lb2 = std::get<2>(t), ub2 = std::get<3>(t);
  if (!(lb1 == 0 || ub1 == 0 || lb1 != ub1) || !(lb2 == 0 || ub2 == 0 || lb2 != ub2))
    throw ReferenceUB("EmptyIntervalDict assert: degenerate interval for " + var);
  // bounds of 64-bit values over 32-bit keys, searched through the fences when given
  auto lb = [&](size_t v) {
    if (fences) return fenced_bound(data, *fences, start, end, v, false);
    return static_cast<size_t>(
        std::lower_bound(data + start, data + end, v, [](TYPEID a, size_t b) { return a < b; }) - data);
  };
  auto ub = [&](size_t v) {
    if (fences) return fenced_bound(data, *fences, start, end, v, true);
    return static_cast<size_t>(
        std::upper_bound(data + start, data + end, v, [](size_t a, TYPEID b) { return a < b; }) - data);
  };
  if (ub2 == 0 && ub1 == 0) {
    up.push_back({start, end});
    offsets.push_back(0);
    relationSize = end - start;
  } else if (ub1 == 0) {
    const size_t o1 = lb(lb2), o2 = ub(ub2);
    up.push_back({start, o1});
    offsets.push_back(0);
    up.push_back({o2, end});
    offsets.push_back(o1 - start);
    relationSize = (o1 - start) + (end - o2);
  } else {
    const size_t o1 = lb(lb1), o2 = ub(ub1), o3 = lb(lb2), o4 = ub(ub2);
    up.push_back({start, o1});
    offsets.push_back(0);
    size_t mid = 0;
    if (o2 != o3) {
      if (o2 > o3) throw ReferenceUB("EmptyIntervalDict: negative-length upload interval for " + var);
      up.push_back({o2, o3});
      offsets.push_back(o1 - start);
      mid = o3 - o2;
    }
    if (o4 > end) throw ReferenceUB("EmptyIntervalDict: upload interval past the slice");
    up.push_back({o4, end});
    offsets.push_back((o1 - start) + mid);
    relationSize = (o1 - start) + mid + (end - o4);
  }
}

// ---------------------------------------------------------------------------
// TriplePattern / SparqlQuery / SparqlResult
// ---------------------------------------------------------------------------
static bool parse_id(const std::string& t, TYPEID& id) {
  if (t.size() < 3) return false;
  if (!((t.front() == '<' && t.back() == '>') || (t.front() == '"' && t.back() == '"'))) return false;
  std::string body = t.substr(1, t.size() - 2);
  if (body.empty()) return false;
  for (char c : body)
    if (!std::isdigit(static_cast<unsigned char>(c))) return false;
  unsigned long long v = std::strtoull(body.c_str(), nullptr, 10);
  if (v > 0xFFFFFFFFull) return false;
  id = static_cast<TYPEID>(v);
  return true;
}

TriplePattern::TriplePattern(size_t id_, const std::string& s, const std::string& p, const std::string& o,
                             const TermResolver* resolver)
    : id(id_) {
  const std::string* t[3] = {&s, &p, &o};
  for (int k = 0; k < 3; ++k) {
    isVar[k] = !t[k]->empty() && (*t[k])[0] == '?';
    if (isVar[k]) names[k] = *t[k];
    else if (resolver) ids[k] = resolver->resolve(k, *t[k]);
    else if (!parse_id(*t[k], ids[k])) throw vg::Error(VG_ERR_PARSE, "bad constant term " + *t[k]);
  }
}

bool TriplePattern::hasVariable(const std::string& v) const {
  for (int k = 0; k < 3; ++k)
    if (isVar[k] && names[k] == v) return true;
  return false;
}

SparqlQuery::SparqlQuery(const char* q, const TermResolver* resolver) {
  std::string text(q);
  std::vector<std::string> toks;
  for (size_t i = 0; i < text.size();) {
    const char c = text[i];
    if (std::isspace(static_cast<unsigned char>(c))) {
      ++i;
      continue;
    }
    const size_t b = i;
    if (c == '<' || c == '"') {
      const size_t e = text.find(c == '<' ? '>' : '"', i + 1);
      if (e == std::string::npos) throw vg::Error(VG_ERR_PARSE, "unterminated term");
      i = e + 1;
      if (c == '"' && i < text.size() && text[i] == '@') {   // language tag
        ++i;
        while (i < text.size() && (std::isalnum(static_cast<unsigned char>(text[i])) || text[i] == '-')) ++i;
      } else if (c == '"' && i + 1 < text.size() && text[i] == '^' && text[i + 1] == '^') {   // datatype
        const size_t d = text.find('>', i + 2);
        if (d == std::string::npos) throw vg::Error(VG_ERR_PARSE, "unterminated datatype");
        i = d + 1;
      }
    } else if (c == '{' || c == '}' || c == '.' || c == '*') {
      ++i;
    } else {
      while (i < text.size() && !std::isspace(static_cast<unsigned char>(text[i])) && text[i] != '{' &&
             text[i] != '}' && text[i] != '.')
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
      throw vg::Error(VG_ERR_PARSE, "unexpected token " + toks[k]);
  }
  if (k == toks.size()) throw vg::Error(VG_ERR_PARSE, "missing {");
  ++k;
  std::vector<std::string> t3;
  for (; k < toks.size() && toks[k] != "}"; ++k) {
    if (toks[k] == ".") continue;
    t3.push_back(toks[k]);
    if (t3.size() == 3) {
      TriplePattern tp(patterns.size(), t3[0], t3[1], t3[2], resolver);
      for (int j = 0; j < 3; ++j)
        if (t3[j][0] == '?') note(t3[j]);
      if (tp.subjectIsVariable()) vars_count[tp.getSubject()] += 1;  // src/SparqlQuery.cu:65-67
      if (tp.predicateIsVariable()) vars_count[tp.getPredicate()] += 1;
      if (tp.objectIsVariable()) vars_count[tp.getObject()] += 1;
      if (tp.getVariableNum() == 1) boundedNum++;
      patterns.push_back(tp);
      t3.clear();
    }
  }
  if (!t3.empty()) throw vg::Error(VG_ERR_PARSE, "incomplete triple pattern");
  if (patterns.empty()) throw vg::Error(VG_ERR_PARSE, "no triple patterns");
  if (star)
    for (auto& v : order) selected_variables.insert(v);
  else
    for (auto& v : proj) selected_variables.insert(v);
}

void SparqlResult::setResult(IR* ir) {
  resultIR = dynamic_cast<FullRelationIR*>(ir);
  if (!resultIR) throw vg::Error(VG_ERR_INVALID, "result is not a FullRelationIR");
}

// ---------------------------------------------------------------------------
// QueryExecutor index lookups (src/QueryExecutor.cu:583-646)
// ---------------------------------------------------------------------------
void QueryExecutor::updateBoundDict(BoundDict* bound, const std::string& variable, TYPEID lo, TYPEID hi) {
  auto vb = (*bound)[variable];
  if ((hi < vb.first) || (lo > vb.second)) lo = hi = 0;
  TYPEID nmin = (lo == 0) ? 0 : std::max(vb.first, lo);
  TYPEID nmax = std::min(vb.second, hi);
  (*bound)[variable] = std::make_pair(nmin, nmax);
}

std::pair<size_t, size_t> QueryExecutor::findL2OffsetFromL1(const TYPEID_HOST_VEC* l1v,
                                                            const TYPEID_HOST_VEC* l1o, TYPEID id1,
                                                            size_t n) {
  if (l1v->empty()) return {0, 0};
  const size_t s = std::lower_bound(l1v->begin(), l1v->end(), id1) - l1v->begin();
  if (s >= l1o->size()) throw ReferenceUB("findL2OffsetFromL1 reads past the level-1 index");
  const size_t e = s + 1;
  return {(*l1o)[s], (e == l1o->size()) ? n : (*l1o)[e]};
}

// std::upper_bound(a + from, a + hi, key), searched from the front: steps of
// 1, 2, 4, ... and a binary search inside the last one.  An upper bound just
// after the lower bound of the same key (a run of equal keys) takes a few
// reads in cache instead of a second search over the whole range.
static size_t upper_from(const TYPEID* a, size_t from, size_t hi, TYPEID key) {
  size_t lo = from, step = 1;
  while (lo < hi && !(key < a[lo])) {
    const size_t nx = lo + step;
    if (nx >= hi || key < a[nx]) return static_cast<size_t>(std::upper_bound(a + lo + 1, a + std::min(nx, hi), key) - a);
    lo = nx;
    step <<= 1;
  }
  return lo;
}

std::pair<size_t, size_t> QueryExecutor::findDataOffsetFromL2(const TYPEID_HOST_VEC* l2v,
                                                              const TYPEID_HOST_VEC* l2o, TYPEID lo,
                                                              TYPEID hi, TYPEID id2) {
  if (l2o->empty()) return {0, 0};
  const size_t b = std::lower_bound(l2o->begin(), l2o->end(), lo) - l2o->begin();
  const size_t e = std::lower_bound(l2o->begin(), l2o->end(), hi) - l2o->begin();
  const size_t s2 = std::lower_bound(l2v->begin() + b, l2v->begin() + e, id2) - l2v->begin();
  const size_t e2 = upper_from(l2v->data(), s2, e, id2);
  if (s2 >= l2o->size() || e2 >= l2o->size())
    throw ReferenceUB("findDataOffsetFromL2 reads past the level-2 offsets");
  return {(*l2o)[s2], (*l2o)[e2]};
}

std::pair<size_t, size_t> QueryExecutor::findDataOffsetFromL2(const TYPEID_HOST_VEC* d, size_t lo, size_t hi,
                                                              TYPEID id2) {
  const size_t s = std::lower_bound(d->begin() + lo, d->begin() + hi, id2) - d->begin();
  return {s, upper_from(d->data(), s, hi, id2)};
}

std::vector<size_t> QueryExecutor::l2RangesOfL1(const TYPEID_HOST_VEC& l1o, const TYPEID_HOST_VEC& l2o,
                                                size_t n) {
  std::vector<size_t> r(l1o.size() + 1);
  for (size_t s = 0; s <= l1o.size(); ++s) {
    const TYPEID v = s < l1o.size() ? l1o[s] : static_cast<TYPEID>(n);
    r[s] = static_cast<size_t>(std::lower_bound(l2o.begin(), l2o.end(), v) - l2o.begin());
  }
  return r;
}

std::pair<size_t, size_t> QueryExecutor::findDataOffsetForKey(VedasStorage* st, bool po, TYPEID id1, TYPEID id2,
                                                              size_t n) {
  TYPEID_HOST_VEC* l1v = st->getPredicateIndexValues();
  TYPEID_HOST_VEC* l1o = st->getPredicateIndexOffsets();
  TYPEID_HOST_VEC* l2v = po ? st->getPredicateObjectIndexValues() : st->getPredicateSubjectIndexValues();
  TYPEID_HOST_VEC* l2o = po ? st->getPredicateObjectIndexOffsets() : st->getPredicateSubjectIndexOffsets();
  if (n != st->getTripleSize()) {   // the table is made for the triple count
    auto r1 = findL2OffsetFromL1(l1v, l1o, id1, n);
    return findDataOffsetFromL2(l2v, l2o, static_cast<TYPEID>(r1.first), static_cast<TYPEID>(r1.second), id2);
  }
  return findDataOffsetForKey(l1v, l1o, l2v, l2o, st->l2RangeOfL1(po), id1, id2, n);
}

std::pair<size_t, size_t> QueryExecutor::findDataOffsetForKey(const TYPEID_HOST_VEC* l1v, const TYPEID_HOST_VEC* l1o,
                                                              const TYPEID_HOST_VEC* l2v, const TYPEID_HOST_VEC* l2o,
                                                              const std::vector<size_t>& r, TYPEID id1, TYPEID id2,
                                                              size_t n) {
  if (l1v->empty() || l2o->empty() || r.size() != l1o->size() + 1) {
    auto r1 = findL2OffsetFromL1(l1v, l1o, id1, n);
    return findDataOffsetFromL2(l2v, l2o, static_cast<TYPEID>(r1.first), static_cast<TYPEID>(r1.second), id2);
  }
  const size_t s = std::lower_bound(l1v->begin(), l1v->end(), id1) - l1v->begin();
  if (s >= l1o->size()) throw ReferenceUB("findL2OffsetFromL1 reads past the level-1 index");
  // lower_bound(l2o, l1o[s]) and lower_bound(l2o, l1o[s + 1] or n)
  const size_t b = r[s], e = r[s + 1];
  const size_t s2 = std::lower_bound(l2v->begin() + b, l2v->begin() + e, id2) - l2v->begin();
  const size_t e2 = upper_from(l2v->data(), s2, e, id2);
  if (s2 >= l2o->size() || e2 >= l2o->size())
    throw ReferenceUB("findDataOffsetFromL2 reads past the level-2 offsets");
  return {(*l2o)[s2], (*l2o)[e2]};
}

QueryExecutor::QueryExecutor(VedasStorage* s, vg::Ctx* c) : storage(s), ctx(c) {}

// createVariableBound (src/QueryExecutor.cu:441-479)
void QueryExecutor::createVariableBound(SparqlQuery& sq) {
  join_vars.clear();
  for (auto& c : sq.getVarCountMap())
    if (c.second > 1) {
      join_vars.insert(c.first);
      variables_bound[c.first] = std::make_pair(TYPEID(0), TYPEID(0xFFFFFFFFu));
    }
  bool zero = false;
  for (size_t i = 0; i < sq.getPatternNum(); ++i) {
    TriplePattern* p = sq.getPatternPtr(i);
    if (p->getVariableNum() == 1) squeezeQueryBound1Var(p);
    else if (p->getVariableNum() == 2) squeezeQueryBound2Var(p);
    zero = zero || p->estimate_rows == 0;
  }
  if (zero)
    for (const std::string& jv : join_vars) variables_bound[jv] = std::make_pair(TYPEID(0), TYPEID(0));
}

// squeezeQueryBound1Var + updateDataBound (src/QueryExecutor.cu:527-581,
// :649-678).  Without the full index the S/O level-1 lookup finds an empty
// index and returns, so only the predicate-index lookup runs.
void QueryExecutor::squeezeQueryBound1Var(TriplePattern* p) {
  if (p->predicateIsVariable()) throw vg::Error(VG_ERR_UNSUPPORTED, "predicate variables need the full index");
  const bool subj = p->subjectIsVariable();
  TYPEID_HOST_VEC* l1v = storage->getPredicateIndexValues();
  TYPEID_HOST_VEC* l1o = storage->getPredicateIndexOffsets();
  TYPEID_HOST_VEC* l2d = subj ? storage->getPOdata() : storage->getPSdata();
  TYPEID_HOST_VEC* data = subj ? storage->getPOSdata() : storage->getPSOdata();
  const std::string v = subj ? p->getSubject() : p->getObject();
  const TYPEID id2 = subj ? p->getObjectId() : p->getSubjectId();
  if (l1v->empty()) return;
  auto r1 = findL2OffsetFromL1(l1v, l1o, p->getPredicateId(), data->size());
  auto r2 = findDataOffsetFromL2(l2d, r1.first, r1.second, id2);
  p->estimate_rows = r2.second - r2.first;
  // An empty range makes the reference read one element before it; the
  // estimate is then 0 and the zero-result rule overwrites every join bound,
  // so the value read cannot matter.
  const TYPEID lo = r2.first < data->size() ? (*data)[r2.first] : 0;
  const TYPEID hi = r2.second >= 1 ? (*data)[r2.second - 1] : 0;
  if (variables_bound.count(v) > 0) updateBoundDict(&variables_bound, v, lo, hi);
}

// squeezeQueryBound2Var + updateL2Bound (src/QueryExecutor.cu:680-765),
// bitmap 5 (?s p ?o).  The level-1 lookup is given getSOPdata()->size(),
// which is 0 without the full index: the last predicate's range ends at 0.
void QueryExecutor::squeezeQueryBound2Var(TriplePattern* p) {
  if (p->getVariableBitmap() != 5) throw vg::Error(VG_ERR_UNSUPPORTED, "pattern needs the full index");
  const size_t data_size = storage->isFullIndex() ? storage->getTripleSize() : 0;
  auto r1 = findL2OffsetFromL1(storage->getPredicateIndexValues(), storage->getPredicateIndexOffsets(),
                               p->getPredicateId(), data_size);
  auto l2bound = [&](const std::string& var, TYPEID_HOST_VEC* l2d) {
    const size_t s = r1.first, e = r1.second;
    p->estimate_rows = (e == 0) ? 0 : e - s;
    if (variables_bound.count(var) > 0) {
      const TYPEID lo = s < l2d->size() ? (*l2d)[s] : 0;
      const TYPEID hi = (e >= 1 && e - 1 < l2d->size()) ? (*l2d)[e - 1] : 0;
      updateBoundDict(&variables_bound, var, lo, hi);
    }
  };
  if (join_vars.count(p->getObject())) l2bound(p->getObject(), storage->getPOdata());
  if (join_vars.count(p->getSubject())) l2bound(p->getSubject(), storage->getPSdata());
}

// create1VarSelectQueryJob / create2VarSelectQueryJob, partial index
// (src/QueryExecutor.cu:781-971).
SelectQueryJob* QueryExecutor::createSelectQueryJob(TriplePattern* p, const std::string& index_used) {
  if (p->getVariableNum() == 1) {
    if (p->predicateIsVariable()) throw vg::Error(VG_ERR_UNSUPPORTED, "predicate variables need the full index");
    if (p->subjectIsVariable())
      return new SelectQueryJob(this, true, p->getSubject(), p->getPredicateId(), p->getObjectId());
    return new SelectQueryJob(this, false, p->getObject(), p->getPredicateId(), p->getSubjectId());
  }
  if (p->getVariableNum() != 2 || p->getVariableBitmap() != 5)
    throw vg::Error(VG_ERR_UNSUPPORTED, "pattern shape needs the full index");
  if (index_used == "POS") {
    const bool used = selected_variables.count(p->getSubject()) > 0 || variables_bound.count(p->getSubject()) > 0;
    return new SelectQueryJob(this, true, p->getObject(), p->getSubject(), p->getPredicateId(), used);
  }
  const bool used = selected_variables.count(p->getObject()) > 0 || variables_bound.count(p->getObject()) > 0;
  return new SelectQueryJob(this, false, p->getSubject(), p->getObject(), p->getPredicateId(), used);
}

// postorderTraversal (src/QueryExecutor.cu:106-135)
int QueryExecutor::postorderTraversal(QueryPlan& plan, PlanTreeNode* root, SparqlQuery& sq) {
  if (root == nullptr) return -1;
  int j1 = -1, j2 = -1;
  if (root->child1) j1 = postorderTraversal(plan, root->child1, sq);
  if (root->child2) j2 = postorderTraversal(plan, root->child2, sq);
  switch (root->op) {
    case UPLOAD:
      if (root->tp->getVariableNum() == 1) plan.pushJob(createSelectQueryJob(root->tp, ""));
      else if (root->tp->getVariableNum() == 2)
        plan.pushJob(createSelectQueryJob(root->tp, root->tp->getSubject() == root->var ? "PSO" : "POS"));
      else
        throw vg::Error(VG_ERR_UNSUPPORTED, "three-variable pattern");
      break;
    case JOIN:
      plan.pushJob(new JoinQueryJob(this, plan.getJob(j1), plan.getJob(j2), root->var, !root->reuseVar));
      break;
    case INDEXSWAP:
      plan.pushJob(new IndexSwapJob(this, plan.getJob(j1), root->var));
      break;
  }
  return static_cast<int>(plan.jobNum()) - 1;
}

void QueryExecutor::plan(SparqlQuery& sq, QueryPlan& plan) {
  if (storage->isFullIndex()) throw vg::Error(VG_ERR_UNSUPPORTED, "queries run on the partial index");
  selected_variables = sq.getSelectedVariables();
  if (sq.getPatternNum() == 1) {  // src/QueryExecutor.cu:305-312
    plan.pushJob(createSelectQueryJob(sq.getPatternPtr(0), ""));
    return;
  }
  createVariableBound(sq);
  QueryGraph qg(&sq);
  PlanTreeNode* root = qg.generateQueryPlan();
  if (!root) throw ReferenceUB("the planner emits no plan for a query graph of two vertices");
  postorderTraversal(plan, root, sq);
}

void QueryExecutor::query(SparqlQuery& sq, SparqlResult& sr) {
  std::set<std::string> sel = sq.getSelectedVariables();
  QueryPlan qp(sel);
  plan(sq, qp);
  qp.execute(sr);
}

// Empty-interval scan (src/JoinQueryJob.cu:398-433, src/IndexSwapJob.cu:81-118).
void QueryExecutor::eifBounds(const TYPEID* c0, size_t n, size_t out[4]) {
  size_t pos = 0;
  TYPEID best = 0;
  for (size_t k = 0; k + 1 < n; ++k) {
    const TYPEID d = c0[k + 1] - c0[k];
    if (k == 0 || d > best) {  // thrust::max_element: first maximum
      best = d;
      pos = k;
    }
  }
  const size_t sc = pos >= 2 ? pos - 2 : 0;
  const size_t ec = std::min(pos + 4, n);
  TYPEID v[6];
  const size_t sz = ec - sc;
  for (size_t i = 0; i < sz; ++i) v[i] = c0[sc + i];
  TYPEID b[4] = {0, 0, 0, 0};
  size_t firstMax = 0, secondMax = 0;
  for (size_t i = 1; i < sz; ++i) {
    const TYPEID d = v[i] - v[i - 1];
    if (d >= firstMax) {
      secondMax = firstMax;
      b[0] = b[2];
      b[1] = b[3];
      firstMax = d;
      b[2] = v[i - 1];
      b[3] = v[i];
    } else if (d > secondMax) {
      secondMax = d;
      b[0] = v[i - 1];
      b[1] = v[i];
    }
  }
  if (b[2] < b[0]) {
    std::swap(b[0], b[2]);
    std::swap(b[1], b[3]);
  }
  // 32-bit arithmetic as in the reference: b - 1 wraps when b == 0
  out[0] = static_cast<TYPEID>(b[0] + 1u);
  out[1] = static_cast<TYPEID>(b[1] - 1u);
  out[2] = static_cast<TYPEID>(b[2] + 1u);
  out[3] = static_cast<TYPEID>(b[3] - 1u);
}

void QueryExecutor::eifScan(FullRelationIR* ir, const std::string& var) {
  const size_t n = ir->size();
  std::vector<TYPEID> c0(n);
  vg::download(*ctx, ir->getRelationRawPointer(0), n, c0.data());
  size_t b[4];
  eifBounds(c0.data(), n, b);
  empty_interval_dict.updateBound(var, b[0], b[1], b[2], b[3]);
}

// ---------------------------------------------------------------------------
// SelectQueryJob (src/SelectQueryJob.cu:86-270)
// ---------------------------------------------------------------------------
SelectQueryJob::SelectQueryJob(QueryExecutor* e, bool pos, std::string v1, std::string v2, TYPEID id1,
                               bool used)
    : ex(e), pos_index(pos), variable_num(2), is_second_var_used(used) {
  variables[0] = std::move(v1);
  variables[1] = std::move(v2);
  dataid[0] = id1;
}

SelectQueryJob::SelectQueryJob(QueryExecutor* e, bool subject_var, std::string v1, TYPEID id1, TYPEID id2)
    : ex(e), pos_index(subject_var), variable_num(1) {
  variables[0] = std::move(v1);
  dataid[0] = id1;
  dataid[1] = id2;
}

SelectQueryJob::~SelectQueryJob() { delete intermediateResult; }

int SelectQueryJob::startJob(int gpu) {
  gpuId = gpu;
  SelectWork w;
  prepare(w);
  if (!w.pieces.empty()) vg::multi_copy(*ex->ctx, w.pieces.data(), static_cast<int>(w.pieces.size()));
  return 0;
}

void SelectQueryJob::prepare(SelectWork& w) {
  VedasStorage* st = ex->storage;
  vg::Ctx* ctx = ex->ctx;
  TYPEID_HOST_VEC* l1v = st->getPredicateIndexValues();
  TYPEID_HOST_VEC* l1o = st->getPredicateIndexOffsets();
  if (variable_num == 1) {
    const bool subj = pos_index;
    TYPEID_HOST_VEC* data = subj ? st->getPOSdata() : st->getPSOdata();
    const TYPEID* ddata = subj ? st->devPOSdata() : st->devPSOdata();
    auto r2 = QueryExecutor::findDataOffsetForKey(st, subj, dataid[0], dataid[1], data->size());
    if (r2.first > r2.second) r2.second = r2.first;
    const size_t rows = r2.second - r2.first;
    // the uploaded slice is read, never written: the relation views it
    const TYPEID* view[1] = {ddata + r2.first};
    auto* ir = rows ? new FullRelationIR(ctx, 1, rows, view) : new FullRelationIR(ctx, 1, 0);
    ir->setHeader(0, variables[0], false);
    intermediateResult = ir;
    w.ir = ir;
    ex->exe_log.push_back(
        ExecuteLogRecord(gpuId, UPLOAD_OP, ex->log_text ? ir->getHeaders("") : std::string(), rows, 1));
    if (ex->variables_bound.count(variables[0]) > 0) {
      if (rows == 0) QueryExecutor::updateBoundDict(&ex->variables_bound, variables[0], 0, 0);
      else
        QueryExecutor::updateBoundDict(&ex->variables_bound, variables[0], (*data)[r2.first],
                                       (*data)[r2.second - 1]);
    }
    return;
  }
  // two variables: level-2 data ps_data (PSO) or po_data (POS)
  TYPEID_HOST_VEC* l2d = pos_index ? st->getPOdata() : st->getPSdata();
  const TYPEID* dl2d = pos_index ? st->devPOdata() : st->devPSdata();
  const TYPEID* ddata = pos_index ? st->devPOSdata() : st->devPSOdata();
  auto r1 = QueryExecutor::findL2OffsetFromL1(l1v, l1o, dataid[0], st->getTripleSize());
  const size_t b0 = r1.first, e0 = r1.second;
  if (e0 == 0 || b0 >= l2d->size() || e0 > l2d->size())
    throw ReferenceUB("select reads outside the level-2 data");
  const TYPEID cur_min = (*l2d)[b0], cur_max = (*l2d)[e0 - 1];
  size_t first = b0, second = e0;
  if (ex->variables_bound.count(variables[0]) > 0) {
    auto bd = ex->variables_bound[variables[0]];
    const std::vector<uint32_t>& fences = st->l2Fences(pos_index);
    if (bd.first > cur_min) first = fenced_bound(l2d->data(), fences, b0, e0, bd.first, false);
    if (bd.second < cur_max) second = fenced_bound(l2d->data(), fences, b0, e0, bd.second, true);
  }
  size_t ds = first, de = second;
  if (ds > de) de = ds;
  if (!is_second_var_used) {
    if (first > second) throw ReferenceUB("select row count underflows");
    const size_t row = second - first;
    // The reference uploads l2d[first, second) and removes adjacent
    // duplicates (src/SelectQueryJob.cu:151-166).  first and second are
    // boundaries of runs of equal keys (the
    // predicate's range, narrowed by a lower and an upper bound on the key),
    // so the distinct keys are exactly the level-2 index keys of the runs
    // that start in [first, second): a contiguous slice of the level-2 values.
    TYPEID_HOST_VEC* l2o = pos_index ? st->getPredicateObjectIndexOffsets() : st->getPredicateSubjectIndexOffsets();
    const TYPEID* dl2v = pos_index ? st->devPOIdxValues() : st->devPSIdxValues();
    // first and second lie in the predicate's data range, so their positions
    // among the level-2 offsets lie in the predicate's level-2 range
    auto l2lo = l2o->begin(), l2hi = l2o->end();
    const std::vector<size_t>& l2r = st->l2RangeOfL1(pos_index);
    if (l2r.size() == l1o->size() + 1) {
      const size_t s1 = std::lower_bound(l1v->begin(), l1v->end(), dataid[0]) - l1v->begin();
      l2lo = l2o->begin() + l2r[s1];
      l2hi = l2o->begin() + l2r[s1 + 1];
    }
    const size_t ra = static_cast<size_t>(std::lower_bound(l2lo, l2hi, first) - l2o->begin());
    const size_t rb = static_cast<size_t>(std::lower_bound(l2lo, l2hi, second) - l2o->begin());
    if (row > 0 && (ra >= l2o->size() || (*l2o)[ra] != first || rb < ra))
      throw vg::Error(VG_ERR_INVALID, "select range does not start a level-2 run");
    const size_t kept = row > 0 ? rb - ra : 0;
    const TYPEID* view[1] = {dl2v + ra};
    auto* ir = kept ? new FullRelationIR(ctx, 1, kept, view) : new FullRelationIR(ctx, 1, 0);
    ir->setHeader(0, variables[0], false);
    intermediateResult = ir;
    w.ir = ir;
    ex->exe_log.push_back(
        ExecuteLogRecord(gpuId, UPLOAD_OP, ex->log_text ? ir->getHeaders("") : std::string(), row, 1));
    return;
  }
  size_t total = 0;
  std::vector<std::pair<size_t, size_t>> up;
  std::vector<size_t> offs;
  ex->empty_interval_dict.getUploadRelationData(variables[0], l2d->data(), ds, de, total, up, offs,
                                                &st->l2Fences(pos_index));
  // one whole interval: the relation views the two index slices
  if (up.size() == 1 && offs[0] == 0 && up[0].second >= up[0].first && up[0].second - up[0].first == total &&
      total > 0) {
    const TYPEID* view[2] = {dl2d + up[0].first, ddata + up[0].first};
    auto* ir = new FullRelationIR(ctx, 2, total, view);
    ir->setHeader(0, variables[0], false);
    ir->setHeader(1, variables[1], false);
    intermediateResult = ir;
    w.ir = ir;
    ex->exe_log.push_back(
        ExecuteLogRecord(gpuId, UPLOAD_OP, ex->log_text ? ir->getHeaders("") : std::string(), total, 2));
    return;
  }
  auto* ir = new FullRelationIR(ctx, 2, total);
  ir->setHeader(0, variables[0], false);
  ir->setHeader(1, variables[1], false);
  intermediateResult = ir;
  w.ir = ir;
  ex->exe_log.push_back(
      ExecuteLogRecord(gpuId, UPLOAD_OP, ex->log_text ? ir->getHeaders("") : std::string(), total, 2));
  for (size_t i = 0; i < up.size(); ++i) {
    if (up[i].second < up[i].first) throw ReferenceUB("negative upload interval");
    const size_t len = up[i].second - up[i].first;
    if (offs[i] + len > total) throw ReferenceUB("upload interval past the relation");
    if (!len) continue;
    w.pieces.push_back({dl2d + up[i].first, ir->getRelationRawPointer(0) + offs[i], len});
    w.pieces.push_back({ddata + up[i].first, ir->getRelationRawPointer(1) + offs[i], len});
  }
}

// ---------------------------------------------------------------------------
// JoinQueryJob (src/JoinQueryJob.cu:44-453)
// ---------------------------------------------------------------------------
JoinQueryJob::JoinQueryJob(QueryExecutor* e, QueryJob* l, QueryJob* r, std::string jv, bool last)
    : ex(e), leftJob(l), rightJob(r), joinVariable(std::move(jv)), lastJoinForVar(last) {}

int JoinQueryJob::startJob(int gpu) {
  gpuId = gpu;
  auto* l = dynamic_cast<FullRelationIR*>(leftJob->getIR());
  auto* r = dynamic_cast<FullRelationIR*>(rightJob->getIR());
  if (!l || !r) throw vg::Error(VG_ERR_INVALID, "join operands are not relations");
  intermediateResult = join(l, r);
  return 0;
}

IR* JoinQueryJob::join(FullRelationIR* lir, FullRelationIR* rir) {
  (void)lir;
  (void)rir;
  JoinWork w;
  prepare(w);
  if (w.empty) return intermediateResult;
  if (w.sortL) w.lir->sortByFirstColumn();
  if (w.sortR) w.rir->sortByFirstColumn();
  vg::Rel joined;
  vg::join(*ex->ctx, w.lir->rel(), w.rir->rel(), false, joined);
  TYPEID fl[2] = {0, 0};
  std::vector<TYPEID> c0;
  if (joined.nrows > 0) {
    VG_CUDA(cudaMemcpyAsync(&fl[0], joined.cols[0], 4, cudaMemcpyDeviceToHost, ex->ctx->stream));
    VG_CUDA(cudaMemcpyAsync(&fl[1], joined.cols[0] + joined.nrows - 1, 4, cudaMemcpyDeviceToHost,
                            ex->ctx->stream));
    if (joined.nrows > 2 && joined.nrows < 100) {
      c0.resize(joined.nrows);
      VG_CUDA(cudaMemcpyAsync(c0.data(), joined.cols[0], joined.nrows * 4, cudaMemcpyDeviceToHost,
                              ex->ctx->stream));
    }
    ex->ctx->sync();
  }
  finish(w, joined, fl[0], fl[1], &c0);
  return intermediateResult;
}

void JoinQueryJob::setHeaders(JoinWork& w, FullRelationIR* out) {
  const size_t ls = w.lir->getColumnNum(), rs = w.rir->getColumnNum();
  size_t h = 0;
  out->setHeader(h++, w.lir->getHeader(0), w.lir->getIsPredicate(0));
  for (size_t i = 1; i < ls; ++i) out->setHeader(h++, w.lir->getHeader(i), w.lir->getIsPredicate(i));
  for (size_t i = 1; i < rs; ++i) out->setHeader(h++, w.rir->getHeader(i), w.rir->getIsPredicate(i));
}

void JoinQueryJob::finish(JoinWork& w, vg::Rel& joined, TYPEID first, TYPEID last,
                          const std::vector<TYPEID>* col0) {
  auto* out = new FullRelationIR(ex->ctx, w.new_col_num, 0);
  out->adopt(joined);
  setHeaders(w, out);
  intermediateResult = out;
  const size_t result_size = out->size();
  ex->exe_log.push_back(ExecuteLogRecord(gpuId, JOIN_OP,
                                         ex->log_text ? w.lir->getHeaders("") + " x " + w.rir->getHeaders("")
                                                      : std::string(),
                                         w.lir->size(), w.rir->size(), result_size));
  if (QueryExecutor::ENABLE_UPDATE_BOUND_AFTER_JOIN) {
    if (result_size > 0) {
      QueryExecutor::updateBoundDict(&ex->variables_bound, joinVariable, first, last);
      if (!lastJoinForVar && result_size > 2 && result_size < 100) {
        if (!col0 || col0->size() != result_size) throw vg::Error(VG_ERR_INVALID, "join: column 0 not staged");
        size_t b[4];
        QueryExecutor::eifBounds(col0->data(), result_size, b);
        ex->empty_interval_dict.updateBound(joinVariable, b[0], b[1], b[2], b[3]);
      }
    } else {
      QueryExecutor::updateBoundDict(&ex->variables_bound, joinVariable, 0, 0);
    }
  }
}

void JoinQueryJob::prepare(JoinWork& w) {
  auto* lir = dynamic_cast<FullRelationIR*>(leftJob->getIR());
  auto* rir = dynamic_cast<FullRelationIR*>(rightJob->getIR());
  if (!lir || !rir) throw vg::Error(VG_ERR_INVALID, "join operands are not relations");
  if (lir->size() > rir->size()) std::swap(lir, rir);
  std::vector<std::string> jvs;
  {
    std::string cur;
    for (char c : joinVariable) {
      if (c == ',') {
        if (!cur.empty()) jvs.push_back(cur);
        cur.clear();
      } else {
        cur += c;
      }
    }
    if (!cur.empty()) jvs.push_back(cur);
  }
  if (jvs.size() != 1) throw vg::Error(VG_ERR_UNSUPPORTED, "multi-variable joins are not planned");
  const std::string& jv = jvs[0];
  auto& counter = *query_variable_counter;
  size_t new_col_num = lir->getColumnNum() + rir->getColumnNum() - 1;
  // Pruning (src/JoinQueryJob.cu:136-155).  Removing column 0 re-sorts the
  // relation by the join variable; that sort is deferred to the caller.
  bool sortL = false, sortR = false;
  for (int i = static_cast<int>(lir->getColumnNum()) - 1; i >= 0; --i)
    if (counter[lir->getHeader(i)] == 0 && lir->getHeader(i) != jv) {
      sortL = lir->removeColumnDeferSort(static_cast<size_t>(i), jv) || sortL;
      new_col_num -= 1;
    }
  for (int i = static_cast<int>(rir->getColumnNum()) - 1; i >= 0; --i)
    if (counter[rir->getHeader(i)] == 0 && rir->getHeader(i) != jv) {
      sortR = rir->removeColumnDeferSort(static_cast<size_t>(i), jv) || sortR;
      new_col_num -= 1;
    }
  counter[jv] -= 1;
  // Implicit index swaps (src/JoinQueryJob.cu:162-180).
  const size_t lj = lir->getColumnId(jv), rj = rir->getColumnId(jv);
  if (lj != 0) {
    lir->swapColumn(0, lj);
    sortL = true;
    ex->exe_log.push_back(ExecuteLogRecord(gpuId, SWAP_OP, "", lir->size(), lir->getColumnNum()));
  }
  if (rj != 0) {
    rir->swapColumn(0, rj);
    sortR = true;
    ex->exe_log.push_back(ExecuteLogRecord(gpuId, SWAP_OP, "", rir->size(), rir->getColumnNum()));
  }
  w.lir = lir;
  w.rir = rir;
  w.sortL = sortL;
  w.sortR = sortR;
  w.new_col_num = new_col_num;
  w.empty = false;
  if (lir->size() == 0 || rir->size() == 0) {
    // Output decided on the host; the operands' re-sorts cannot be observed.
    w.empty = true;
    w.sortL = w.sortR = false;
    auto* out = new FullRelationIR(ex->ctx, new_col_num, 0);
    setHeaders(w, out);
    intermediateResult = out;
    ex->exe_log.push_back(ExecuteLogRecord(gpuId, JOIN_OP,
                                           ex->log_text ? lir->getHeaders("") + " x " + rir->getHeaders("")
                                                        : std::string(),
                                           lir->size(), rir->size(), 0));
  }
}

// ---------------------------------------------------------------------------
// IndexSwapJob (src/IndexSwapJob.cu:28-95) and TransferJob
// ---------------------------------------------------------------------------
IndexSwapJob::IndexSwapJob(QueryExecutor* e, QueryJob* before, std::string v)
    : ex(e), beforeJob(before), swapVar(std::move(v)) {}

int IndexSwapJob::startJob(int gpu) {
  gpuId = gpu;
  FullRelationIR* ir = prepare();
  ir->sortByFirstColumn();
  std::vector<TYPEID> c0;
  if (ir->size() > 2 && ir->size() < 100) {
    c0.resize(ir->size());
    vg::download(*ex->ctx, ir->getRelationRawPointer(0), ir->size(), c0.data());
  }
  finish(&c0);
  return 0;
}

FullRelationIR* IndexSwapJob::prepare() {
  auto* ir = dynamic_cast<FullRelationIR*>(beforeJob->getIR());
  if (!ir) throw vg::Error(VG_ERR_INVALID, "swap operand is not a relation");
  swapped_col = ir->getColumnId(swapVar);
  ir->swapColumn(0, swapped_col);
  intermediateResult = ir;
  return ir;
}

void IndexSwapJob::finish(const std::vector<TYPEID>* col0) {
  auto* ir = dynamic_cast<FullRelationIR*>(intermediateResult);
  ex->exe_log.push_back(ExecuteLogRecord(gpuId, SWAP_OP,
                                         ex->log_text ? ir->getHeader(0) + " <-> " + ir->getHeader(swapped_col)
                                                      : std::string(),
                                         ir->size(),
                                         ir->getColumnNum()));
  if (ir->size() > 2 && ir->size() < 100) {
    if (!col0 || col0->size() != ir->size()) throw vg::Error(VG_ERR_INVALID, "swap: column 0 not staged");
    size_t b[4];
    QueryExecutor::eifBounds(col0->data(), ir->size(), b);
    ex->empty_interval_dict.updateBound(ir->getHeader(0), b[0], b[1], b[2], b[3]);
  }
}

TransferJob::TransferJob(size_t, size_t, int src, int dest, QueryJob* j)
    : job(j), src_gpu_id(src), dest_gpu_id(dest) {}

int TransferJob::startJob(int gpu) {
  gpuId = gpu;
  if (src_gpu_id != dest_gpu_id)
    throw vg::Error(VG_ERR_UNSUPPORTED, "one GPU per process: cross-device transfer is not built");
  intermediateResult = job->getIR();
  return 0;
}

// ---------------------------------------------------------------------------
// QueryPlan (src/QueryPlan.cu:34-43, :114-257 single-GPU branch)
// ---------------------------------------------------------------------------
QueryPlan::QueryPlan(std::set<std::string>& sel) {
  for (const std::string& v : sel) select_variables.push_back(v);
}

QueryPlan::~QueryPlan() {
  for (QueryJob* j : jobs) delete j;
}

void QueryPlan::pushJob(QueryJob* job) {
  jobs.push_back(job);
  if (auto* jj = dynamic_cast<JoinQueryJob*>(job)) query_variable_counter[jj->getJoinVariable()] += 1;
}

void QueryPlan::beginExecution() {
  for (const std::string& v : select_variables) query_variable_counter[v] = ULONG_MAX;
  for (QueryJob* job : jobs)
    if (auto* jj = dynamic_cast<JoinQueryJob*>(job)) jj->setQueryVarCounter(&query_variable_counter);
}

FullRelationIR* QueryPlan::project() {
  auto* res = dynamic_cast<FullRelationIR*>(jobs.back()->getIR());
  for (int i = static_cast<int>(res->getColumnNum()) - 1; i >= 1; --i)
    if (query_variable_counter[res->getHeader(static_cast<size_t>(i))] == 0)
      res->removeColumn(static_cast<size_t>(i));
  return res;
}

void QueryPlan::execute(SparqlResult& sr) {
  beginExecution();
  for (QueryJob* job : jobs) job->startJob(0);
  FullRelationIR* res = project();
  res->removeDuplicate();
  sr.setResult(res);
}

// ---------------------------------------------------------------------------
// QueryGraph (src/QueryGraph.cu).  Tie-breaks follow std::unordered_map
// iteration order, so the same container types see the same operations in
// the same order as the reference.
// ---------------------------------------------------------------------------
QueryGraph::QueryGraph(SparqlQuery* q) {
  for (size_t i = 0; i < q->getPatternNum(); ++i) {
    TriplePattern* tp = q->getPatternPtr(i);
    const std::string s = tp->subjectIsVariable() ? tp->getSubject() : std::to_string(tp->getSubjectId());
    const std::string o = tp->objectIsVariable() ? tp->getObject() : std::to_string(tp->getObjectId());
    auto e = std::make_unique<GraphEdge>();
    e->id = std::to_string(tp->getPredicateId());
    if (s[0] == '?') {
      e->vars.insert(s);
      e->indexVar1 = s;
    }
    if (o[0] == '?') {
      e->vars.insert(o);
      if (e->indexVar1.empty()) e->indexVar1 = o;
      else e->indexVar2 = o;
    }
    e->tp = tp;
    e->estimateCardinality = tp->estimate_rows * tp->getVariableNum();
    addEdge(s, o, e.get());
    edges.push_back(std::move(e));
  }
}

PlanTreeNode* QueryGraph::newNode(PlanOperation op) {
  nodes.push_back(std::make_unique<PlanTreeNode>());
  nodes.back()->op = op;
  return nodes.back().get();
}

void QueryGraph::addEdge(const std::string& a, const std::string& b, GraphEdge* e) {
  adjacencyList[a].push_back(std::make_pair(b, e));
  adjacencyList[b].push_back(std::make_pair(a, e));
}

bool QueryGraph::edgeExist(const std::string& a, const std::string& b) {
  for (auto& l : adjacencyList[a])
    if (l.first == b) return true;
  return false;
}

void QueryGraph::mergeEdge(const std::string end1, const std::string end2) {
  for (auto edge : adjacencyList[end2]) {
    // a pattern whose subject and object are one variable: the reference
    // would erase from the list it is walking (src/QueryGraph.cu:101-113)
    if (edge.first == end2) throw ReferenceUB("planner: merging a variable joined to itself");
    if (!edgeExist(end1, edge.first)) addEdge(end1, edge.first, edge.second);
    auto& other = adjacencyList[edge.first];
    for (auto it = other.rbegin(); it != other.rend(); ++it) {
      if (it->first == end2) {
        other.erase(--(it.base()));
        break;
      }
    }
  }
  adjacencyList.erase(end2);
}

std::tuple<size_t, size_t, std::string> QueryGraph::sameMaxDegAndTotalCard(
    std::vector<std::pair<std::string, GraphEdge*>>& links) {
  // One map holds both the reference's varCount and varEstCard: the same keys
  // go in in the same order, so it iterates in varCount's order, on which the
  // tie-break depends.
  std::unordered_map<std::string, std::pair<size_t, size_t>> var;   // count, estimated cardinality
  for (const auto& node : links) {
    for (const auto& v : node.second->vars) {
      auto ins = var.try_emplace(v, 0, 0);
      ins.first->second.first += 1;
      ins.first->second.second += node.second->estimateCardinality;
    }
  }
  size_t maxDeg = 0, maxDegMinCard = 0;
  std::string bestVar;
  for (const auto& v : var) {
    const size_t deg = v.second.first, est = v.second.second;
    if (deg > maxDeg || (deg == maxDeg && est < maxDegMinCard)) {
      maxDeg = deg;
      maxDegMinCard = est;
      bestVar = v.first;
    }
  }
  return std::make_tuple(maxDeg, maxDegMinCard, bestVar);
}

std::pair<std::string, std::string> QueryGraph::findBestStarNode() {
  std::string bestNode, bestVar;
  size_t maxDegree = 0, maxDegCardSum = 0;
  for (auto& node : adjacencyList) {
    auto t = sameMaxDegAndTotalCard(node.second);
    const size_t degree = std::get<0>(t), est = std::get<1>(t);
    if (degree > maxDegree || (degree == maxDegree && est < maxDegCardSum)) {
      maxDegree = degree;
      bestNode = node.first;
      maxDegCardSum = est;
      bestVar = std::get<2>(t);
    }
  }
  return std::make_pair(bestNode, bestVar);
}

PlanTreeNode* QueryGraph::generateJoinPlanForNode(const std::string& vertex, const std::string& joinVar) {
  auto& adj = adjacencyList[vertex];
  std::sort(adj.begin(), adj.end(),
            [](const std::pair<std::string, GraphEdge*>& a, const std::pair<std::string, GraphEdge*>& b) {
              return a.second->estimateCardinality < b.second->estimateCardinality;
            });
  size_t first = 0;
  while (first < adj.size() && !adj[first].second->hasVariable(joinVar)) ++first;
  if (first == adj.size()) throw ReferenceUB("planner: no edge holds the join variable");
  size_t last = 0;
  for (size_t i = first; i < adj.size(); ++i)
    if (adj[i].second->hasVariable(joinVar)) last = i;
  for (size_t i = first; i < adj.size(); ++i) {
    if (!adj[i].second->hasVariable(joinVar)) continue;
    if (!adj[i].second->treeNode) {
      PlanTreeNode* u = newNode(UPLOAD);
      u->tp = adj[i].second->tp;
      u->var = joinVar;
      adj[i].second->treeNode = u;
    }
    if (i > first) {
      GraphEdge* e1 = adj[first].second;
      GraphEdge* e2 = adj[i].second;
      if (e1->indexVar1 != joinVar && e1->indexVar2 != joinVar) {
        PlanTreeNode* s = newNode(INDEXSWAP);
        s->child1 = e1->treeNode;
        s->var = joinVar;
        e1->treeNode = s;
        e1->indexVar1 = joinVar;
        e1->indexVar2 = "";
      }
      if (e2->indexVar1 != joinVar && e2->indexVar2 != joinVar) {
        PlanTreeNode* s = newNode(INDEXSWAP);
        s->child1 = e2->treeNode;
        s->var = joinVar;
        e2->treeNode = s;
      }
      PlanTreeNode* j = newNode(JOIN);
      j->child1 = e1->treeNode;
      j->child2 = e2->treeNode;
      j->var = joinVar;
      j->reuseVar = (i != last);
      e1->treeNode = j;
      double sigma = 0.000001;
      if (e1->estimateCardinality < 1000 && e2->estimateCardinality < 1000) sigma = 0.001;
      else if (e1->estimateCardinality < 1000 || e2->estimateCardinality < 1000) sigma = 0.0001;
      e1->estimateCardinality *= std::ceil(e2->estimateCardinality * sigma);
      for (const auto& v : e2->vars) e1->vars.insert(v);
    }
  }
  // A merge can remove entries of this very list (two patterns between the
  // same two variables): the reference then reads past the list's end
  // (src/QueryGraph.cu:268-274), or erases the list itself (a pattern whose
  // subject and object are one variable).
  for (int i = static_cast<int>(adj.size()) - 1; i > static_cast<int>(first); --i) {
    if (static_cast<size_t>(i) >= adj.size()) throw ReferenceUB("planner: a merge removed edges of its own star");
    if (!adj[i].second->hasVariable(joinVar)) continue;
    if (adj[i].first == vertex) throw ReferenceUB("planner: a star merges its own vertex");
    mergeEdge(adj[first].first, adj[i].first);
  }
  if (first >= adj.size()) throw ReferenceUB("planner: a merge removed edges of its own star");
  adj[first].second->indexVar1 = joinVar;
  adj[first].second->indexVar2 = "";
  return adj[first].second->treeNode;
}

PlanTreeNode* QueryGraph::generateQueryPlan() {
  PlanTreeNode* root = nullptr;
  int guard = 0;
  while (adjacencyList.size() > 2) {
    if (++guard > 64) throw ReferenceUB("planner does not terminate on this query graph");
    auto st = findBestStarNode();
    root = generateJoinPlanForNode(st.first, st.second);
  }
  return root;
}

// ---------------------------------------------------------------------------
// Self-check of the index lookups against the reference's searches
// ---------------------------------------------------------------------------
namespace {

struct Lookup {
  bool ub = false;   // the reference would read out of bounds (ReferenceUB)
  size_t a = 0, b = 0;
};

template <typename F>
Lookup run_lookup(F&& f) {
  Lookup r;
  try {
    auto p = f();
    r.a = p.first;
    r.b = p.second;
  } catch (const ReferenceUB&) {
    r.ub = true;
  }
  return r;
}

// findL2OffsetFromL1 followed by the index form of findDataOffsetFromL2, as
// the reference writes them (src/QueryExecutor.cu:596-633).
std::pair<size_t, size_t> reference_key_lookup(const TYPEID_HOST_VEC& l1v, const TYPEID_HOST_VEC& l1o,
                                               const TYPEID_HOST_VEC& l2v, const TYPEID_HOST_VEC& l2o, TYPEID id1,
                                               TYPEID id2, size_t n) {
  if (l1v.empty()) return {0, 0};
  const size_t s = std::lower_bound(l1v.begin(), l1v.end(), id1) - l1v.begin();
  if (s >= l1o.size()) throw ReferenceUB("level 1");
  const size_t lo = l1o[s], hi = (s + 1 == l1o.size()) ? n : l1o[s + 1];
  if (l2o.empty()) return {0, 0};
  const size_t b = std::lower_bound(l2o.begin(), l2o.end(), static_cast<TYPEID>(lo)) - l2o.begin();
  const size_t e = std::lower_bound(l2o.begin(), l2o.end(), static_cast<TYPEID>(hi)) - l2o.begin();
  const size_t s2 = std::lower_bound(l2v.begin() + b, l2v.begin() + e, id2) - l2v.begin();
  const size_t e2 = std::upper_bound(l2v.begin() + b, l2v.begin() + e, id2) - l2v.begin();
  if (s2 >= l2o.size() || e2 >= l2o.size()) throw ReferenceUB("level 2");
  return {l2o[s2], l2o[e2]};
}

}  // namespace

uint64_t selfcheck_l2_lookup(uint32_t seed, uint32_t graphs, uint32_t lookups) {
  uint64_t x = 0x9E3779B97F4A7C15ull ^ seed;
  auto rnd = [&x](uint64_t m) {
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return m ? x % m : 0;
  };
  uint64_t bad = 0;
  for (uint32_t gi = 0; gi < graphs; ++gi) {
    // predicates with runs of level-2 keys, each key a run of data rows; some
    // graphs repeat level-2 keys within a predicate, which real indexes never do
    const bool dups = gi % 4 == 3;
    const size_t np = rnd(40);
    TYPEID_HOST_VEC l1v, l1o, l2v, l2o, data;
    TYPEID pid = 0;
    for (size_t p = 0; p < np; ++p) {
      pid += 1 + static_cast<TYPEID>(rnd(3));
      l1v.push_back(pid);
      l1o.push_back(static_cast<TYPEID>(data.size()));
      const size_t nk = 1 + rnd(gi % 2 ? 3000 : 60);   // long predicates exercise the fenced searches
      TYPEID key = static_cast<TYPEID>(rnd(5));
      for (size_t k = 0; k < nk; ++k) {
        key += (dups && rnd(4) == 0) ? 0 : 1 + static_cast<TYPEID>(rnd(4));
        l2v.push_back(key);
        l2o.push_back(static_cast<TYPEID>(data.size()));
        const size_t rows = 1 + rnd(4);
        for (size_t r = 0; r < rows; ++r) data.push_back(key);
      }
    }
    const size_t n = data.size();
    const std::vector<size_t> l2r = QueryExecutor::l2RangesOfL1(l1o, l2o, n);
    const std::vector<uint32_t> fences = make_fences(data.data(), data.size());
    for (uint32_t li = 0; li < lookups; ++li) {
      const TYPEID id1 = static_cast<TYPEID>(rnd(pid + 3));
      const TYPEID id2 = static_cast<TYPEID>(rnd(l2v.empty() ? 8 : l2v.back() + 3));
      const Lookup want = run_lookup([&] { return reference_key_lookup(l1v, l1o, l2v, l2o, id1, id2, n); });
      const Lookup got = run_lookup(
          [&] { return QueryExecutor::findDataOffsetForKey(&l1v, &l1o, &l2v, &l2o, l2r, id1, id2, n); });
      if (want.ub != got.ub || (!want.ub && (want.a != got.a || want.b != got.b))) ++bad;
      // the data form over a random range of one predicate's rows
      if (n > 0) {
        size_t lo = rnd(n + 1), hi = rnd(n + 1);
        if (lo > hi) std::swap(lo, hi);
        const size_t ps = l1o.empty() ? 0 : std::upper_bound(l1o.begin(), l1o.end(), lo) - l1o.begin();
        const size_t pend = ps < l1o.size() ? l1o[ps] : n;   // stay inside one predicate's sorted rows
        hi = std::min(hi, std::max(lo, pend));
        const auto d = QueryExecutor::findDataOffsetFromL2(&data, lo, hi, id2);
        const size_t ws = std::lower_bound(data.begin() + lo, data.begin() + hi, id2) - data.begin();
        const size_t we = std::upper_bound(data.begin() + lo, data.begin() + hi, id2) - data.begin();
        if (d.first != ws || d.second != we) ++bad;
        // the fenced searches of the select bounds and empty-interval pieces
        if (fenced_bound(data.data(), fences, lo, hi, id2, false) != ws) ++bad;
        if (fenced_bound(data.data(), fences, lo, hi, id2, true) != we) ++bad;
      }
    }
  }
  return bad;
}

}  // namespace vedas
