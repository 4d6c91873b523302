// CPU oracle for N-Triples ingest -- TEST INFRASTRUCTURE ONLY.
//
// Restates the reference loader's statement handler (src/loader.cu:19-53)
// and its dictionaries (src/VedasBuild.cu:63-70): statements are read in
// file order; the subject, then the object, then the predicate of each
// statement get the next id of their dictionary on first appearance.
// Subjects and non-literal objects share one dictionary (ids from 1),
// predicates have their own (ids from 1), literal objects a third (ids from
// LITERAL_START_ID = 5e7, src/vedas.h:31) when the literal dictionary is
// enabled (-ldict) and share the first otherwise.  A term is keyed by its
// N-Triples text: the reference keys by raptor_term_to_string(), which for
// ASCII terms without escape sequences is the text as written.
//
// Raptor itself (an un-vendored dependency, absent here) cannot be run, so
// this restatement is not pinned against the reference: parity unpinned.
// The tokenizer is a plain sequential scanner of the N-Triples line grammar.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <string_view>
#include <unordered_map>
#include <vector>

namespace {

bool ws(char c) { return c == ' ' || c == '\t' || c == '\r'; }

// One term starting at line[i]: returns its length, 0 if malformed.
// what: 0 subject (IRI or blank node), 1 predicate (IRI), 2 object (any).
size_t scan_term(std::string_view line, size_t i, int what, bool* literal) {
  *literal = false;
  if (i >= line.size()) return 0;
  if (line[i] == '<') {
    size_t j = i + 1;
    while (j < line.size() && line[j] != '>') {
      if (line[j] == ' ' || line[j] == '\t') return 0;
      ++j;
    }
    return j < line.size() ? j + 1 - i : 0;
  }
  if (what == 1) return 0;
  if (line[i] == '_') {
    if (i + 1 >= line.size() || line[i + 1] != ':') return 0;
    size_t j = i + 2;
    while (j < line.size() && !ws(line[j])) ++j;
    if (j == i + 2) return 0;
    if (line[j - 1] == '.' && j - 1 > i + 2) --j;   // the statement's dot
    return j - i;
  }
  if (what == 0 || line[i] != '"') return 0;
  size_t j = i + 1;
  for (;;) {
    if (j >= line.size()) return 0;
    if (line[j] == '\\') {
      j += 2;
      continue;
    }
    if (line[j] == '"') break;
    ++j;
  }
  ++j;
  *literal = true;
  if (j < line.size() && line[j] == '@') {
    size_t k = j + 1;
    while (k < line.size() && (isalnum(static_cast<unsigned char>(line[k])) || line[k] == '-')) ++k;
    return k == j + 1 ? 0 : k - i;
  }
  if (j + 1 < line.size() && line[j] == '^' && line[j + 1] == '^') {
    bool l2;
    const size_t d = scan_term(line, j + 2, 1, &l2);
    return d ? j + 2 + d - i : 0;
  }
  return j - i;
}

struct DictState {
  std::unordered_map<std::string, uint32_t> ids;
  std::vector<std::string> terms;
  uint32_t next;
  explicit DictState(uint32_t base) : next(base) {}
  uint32_t id(std::string_view t) {
    auto it = ids.find(std::string(t));
    if (it != ids.end()) return it->second;
    ids.emplace(std::string(t), next);
    terms.emplace_back(t);
    return next++;
  }
};

char* join_terms(const std::vector<std::string>& v) {
  size_t n = 0;
  for (const auto& t : v) n += t.size() + 1;
  char* out = static_cast<char*>(malloc(n + 1));
  size_t o = 0;
  for (const auto& t : v) {
    memcpy(out + o, t.data(), t.size());
    o += t.size();
    out[o++] = '\n';
  }
  out[o] = 0;
  return out;
}

}  // namespace

extern "C" {

// Returns 0 and malloc'd columns and '\n'-joined dictionaries (terms in id
// order), or the 1-based number of the first malformed line.
uint64_t vo_ingest_ntriples(const char* text, uint64_t len, int literal_dict, uint64_t* n_out, uint32_t** s,
                            uint32_t** p, uint32_t** o, char** so_terms, char** p_terms, char** l_terms) {
  DictState so(1), pd(1), ld(50000000u);
  std::vector<uint32_t> S, P, O;
  uint64_t line_no = 0;
  size_t start = 0;
  while (start < len) {
    size_t end = start;
    while (end < len && text[end] != '\n') ++end;
    ++line_no;
    const std::string_view line(text + start, end - start);
    start = end + 1;
    size_t i = 0;
    while (i < line.size() && ws(line[i])) ++i;
    if (i >= line.size() || line[i] == '#') continue;
    bool l0, l1, lit;
    const size_t ls = scan_term(line, i, 0, &l0);
    if (!ls) return line_no;
    const std::string_view st = line.substr(i, ls);
    i += ls;
    size_t w = i;
    while (i < line.size() && ws(line[i])) ++i;
    if (i == w) return line_no;
    const size_t lp = scan_term(line, i, 1, &l1);
    if (!lp) return line_no;
    const std::string_view pt = line.substr(i, lp);
    i += lp;
    w = i;
    while (i < line.size() && ws(line[i])) ++i;
    if (i == w) return line_no;
    const size_t lo = scan_term(line, i, 2, &lit);
    if (!lo) return line_no;
    const std::string_view ot = line.substr(i, lo);
    i += lo;
    while (i < line.size() && ws(line[i])) ++i;
    if (i >= line.size() || line[i] != '.') return line_no;
    ++i;
    while (i < line.size() && ws(line[i])) ++i;
    if (i < line.size() && line[i] != '#') return line_no;
    // src/loader.cu:27-52: subject, object, predicate
    const uint32_t sid = so.id(st);
    const uint32_t oid = (lit && literal_dict) ? ld.id(ot) : so.id(ot);
    const uint32_t pid = pd.id(pt);
    S.push_back(sid);
    P.push_back(pid);
    O.push_back(oid);
  }
  const uint64_t n = S.size();
  *n_out = n;
  *s = static_cast<uint32_t*>(malloc((n ? n : 1) * 4));
  *p = static_cast<uint32_t*>(malloc((n ? n : 1) * 4));
  *o = static_cast<uint32_t*>(malloc((n ? n : 1) * 4));
  if (n) {
    memcpy(*s, S.data(), n * 4);
    memcpy(*p, P.data(), n * 4);
    memcpy(*o, O.data(), n * 4);
  }
  *so_terms = join_terms(so.terms);
  *p_terms = join_terms(pd.terms);
  *l_terms = join_terms(ld.terms);
  return 0;
}

void vo_free(void* ptr) { free(ptr); }

}  // extern "C"
