// Minimal host stand-in for the part of the Rasqal query API that the VEDAS
// reference's SparqlQuery.cu calls (rasqal/raptor2 are not installed here).
// Test infrastructure only: it lets the reference's own SparqlQuery.cu compile
// unmodified for the reference-as-oracle build.  It understands the basic
// graph pattern subset used by the workloads:
//   SELECT * | ?v1 ?v2 ... WHERE { term term term . term term term . ... }
// where a term is ?name, <iri> or "literal".  IRIs are returned verbatim
// (no base-URI resolution).
#ifndef VEDAS_ORACLE_RASQAL_STUB_H
#define VEDAS_ORACLE_RASQAL_STUB_H

#include <cctype>
#include <cstring>
#include <string>
#include <vector>

#include "../raptor2/raptor2.h"

typedef struct rasqal_world_s {
  int unused;
} rasqal_world;

typedef struct rasqal_variable_s {
  unsigned char* name;
} rasqal_variable;

typedef enum {
  RASQAL_LITERAL_UNKNOWN = 0,
  RASQAL_LITERAL_URI,
  RASQAL_LITERAL_STRING,
  RASQAL_LITERAL_UDT,
  RASQAL_LITERAL_VARIABLE
} rasqal_literal_type;

typedef struct rasqal_literal_s {
  rasqal_literal_type type;
  unsigned char* string;
  union {
    rasqal_variable* variable;
    raptor_uri* uri;
  } value;
} rasqal_literal;

typedef struct rasqal_triple_s {
  rasqal_literal* subject;
  rasqal_literal* predicate;
  rasqal_literal* object;
} rasqal_triple;

typedef struct rasqal_graph_pattern_s {
  std::vector<rasqal_triple*> triples;
} rasqal_graph_pattern;

typedef struct rasqal_query_s {
  std::vector<rasqal_variable*> vars;      // all variables, first-mention order
  std::vector<rasqal_variable*> selected;  // projected variables
  rasqal_graph_pattern gp;
  raptor_sequence all_seq, sel_seq;
  std::vector<rasqal_literal*> lits;
} rasqal_query;

static inline rasqal_world* rasqal_new_world() { return new rasqal_world(); }
static inline void rasqal_free_world(rasqal_world* w) { delete w; }
static inline rasqal_query* rasqal_new_query(rasqal_world*, const char*, const unsigned char*) {
  return new rasqal_query();
}

namespace vedas_rasqal_stub {
static inline unsigned char* dup_str(const std::string& s) {
  unsigned char* p = new unsigned char[s.size() + 1];
  std::memcpy(p, s.c_str(), s.size() + 1);
  return p;
}
static inline rasqal_variable* find_or_add(rasqal_query* q, const std::string& name) {
  for (rasqal_variable* v : q->vars)
    if (name == reinterpret_cast<const char*>(v->name)) return v;
  rasqal_variable* v = new rasqal_variable();
  v->name = dup_str(name);
  q->vars.push_back(v);
  return v;
}
static inline bool next_token(const std::string& s, size_t& i, std::string& tok) {
  while (i < s.size() && std::isspace(static_cast<unsigned char>(s[i]))) ++i;
  if (i >= s.size()) return false;
  size_t b = i;
  char c = s[i];
  if (c == '<') {
    size_t e = s.find('>', i);
    i = (e == std::string::npos) ? s.size() : e + 1;
  } else if (c == '"') {
    size_t e = s.find('"', i + 1);
    i = (e == std::string::npos) ? s.size() : e + 1;
  } else if (c == '{' || c == '}' || c == '.' || c == '*') {
    ++i;
  } else {
    while (i < s.size() && !std::isspace(static_cast<unsigned char>(s[i])) && s[i] != '{' &&
           s[i] != '}' && s[i] != '.')
      ++i;
  }
  tok = s.substr(b, i - b);
  return true;
}
static inline rasqal_literal* make_term(rasqal_query* q, const std::string& t) {
  rasqal_literal* l = new rasqal_literal();
  l->string = nullptr;
  if (!t.empty() && (t[0] == '?' || t[0] == '$')) {
    l->type = RASQAL_LITERAL_VARIABLE;
    l->value.variable = find_or_add(q, t.substr(1));
  } else if (!t.empty() && t[0] == '<') {
    l->type = RASQAL_LITERAL_URI;
    l->value.uri = new raptor_uri();
    l->value.uri->s = dup_str(t.substr(1, t.size() - 2));
  } else {
    l->type = RASQAL_LITERAL_STRING;
    std::string body = (t.size() >= 2 && t[0] == '"') ? t.substr(1, t.size() - 2) : t;
    l->string = dup_str(body);
  }
  q->lits.push_back(l);
  return l;
}
}  // namespace vedas_rasqal_stub

static inline int rasqal_query_prepare(rasqal_query* q, const unsigned char* text, raptor_uri*) {
  using namespace vedas_rasqal_stub;
  std::string s(reinterpret_cast<const char*>(text));
  size_t i = 0;
  std::string tok;
  bool star = false;
  std::vector<std::string> proj;
  while (next_token(s, i, tok)) {
    std::string up = tok;
    for (auto& ch : up) ch = static_cast<char>(std::toupper(static_cast<unsigned char>(ch)));
    if (up == "SELECT" || up == "DISTINCT") continue;
    if (up == "WHERE") continue;
    if (tok == "*") {
      star = true;
      continue;
    }
    if (tok == "{") break;
    if (!tok.empty() && tok[0] == '?') proj.push_back(tok.substr(1));
  }
  for (const std::string& v : proj) q->selected.push_back(find_or_add(q, v));
  std::vector<std::string> terms;
  while (next_token(s, i, tok)) {
    if (tok == "}") break;
    if (tok == ".") continue;
    terms.push_back(tok);
    if (terms.size() == 3) {
      rasqal_triple* t = new rasqal_triple();
      t->subject = make_term(q, terms[0]);
      t->predicate = make_term(q, terms[1]);
      t->object = make_term(q, terms[2]);
      q->gp.triples.push_back(t);
      terms.clear();
    }
  }
  if (star) q->selected = q->vars;
  q->all_seq.items.assign(q->vars.begin(), q->vars.end());
  q->sel_seq.items.assign(q->selected.begin(), q->selected.end());
  return 0;
}

static inline raptor_sequence* rasqal_query_get_all_variable_sequence(rasqal_query* q) {
  return &q->all_seq;
}
static inline raptor_sequence* rasqal_query_get_bound_variable_sequence(rasqal_query* q) {
  return &q->sel_seq;
}
static inline rasqal_variable* rasqal_query_get_variable(rasqal_query* q, int i) {
  return q->vars[static_cast<size_t>(i)];
}
static inline rasqal_graph_pattern* rasqal_query_get_query_graph_pattern(rasqal_query* q) {
  return &q->gp;
}
static inline rasqal_triple* rasqal_graph_pattern_get_triple(rasqal_graph_pattern* gp, int idx) {
  if (idx < 0 || static_cast<size_t>(idx) >= gp->triples.size()) return nullptr;
  return gp->triples[static_cast<size_t>(idx)];
}
static inline void rasqal_free_query(rasqal_query* q) { delete q; }

#endif
