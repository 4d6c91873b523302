// N-Triples ingest on the device: parse and dictionary encoding (the step
// before index build; the reference does it on the host with Raptor,
// src/loader.cu:19-93).
#pragma once

#include <string>
#include <unordered_map>
#include <vector>

#include "compat/vedas_compat.h"
#include "vg_ctx.h"

namespace vg {

// Literal ids start here when literals have their own dictionary
// (LITERAL_START_ID, src/vedas.h:31).
constexpr uint32_t kLiteralStartId = 50000000u;

// The three dictionaries of the reference's loader: subjects and non-literal
// objects share one (ids from 1), predicates have their own (ids from 1), and
// literal objects have a third (ids from kLiteralStartId) when it is enabled,
// otherwise they share the first.  Terms are their N-Triples text.
struct Dict {
  std::vector<std::string> so, p, l;   // term of id base + i
  bool literal_dict = false;
  const std::string* term(int kind, uint32_t id) const;   // kind 0 so, 1 p, 2 l
  uint32_t lookup(int kind, const std::string& term);     // 0 when absent
  std::unordered_map<std::string, uint32_t> rev_[3];     // built on first lookup
};

// Query constants through the dictionaries, with the reference's rules
// (src/TriplePattern.cu:24-43 and toVedasString, src/SparqlQuery.cu:12-27):
// a subject is looked up among subjects/objects, a predicate among
// predicates, an object among literals when it is quoted (only its quoted
// part: Rasqal drops the language tag and datatype) and among
// subjects/objects otherwise.  Absent terms give 0.
class DictResolver : public vedas::TermResolver {
 public:
  explicit DictResolver(const Dict* d);   // builds the reverse maps once
  vedas::TYPEID resolve(int pos, const std::string& term) const override;

 private:
  std::unordered_map<std::string, uint32_t> rev_[3];
};

struct Ingested {
  uint64_t n = 0;                                      // triples
  uint32_t *s = nullptr, *p = nullptr, *o = nullptr;   // device columns (context arena)
  Dict dict;
  uint32_t collisions = 0;   // hash groups that held different terms (resolved exactly)
};

// Parses `len` bytes of N-Triples text and assigns ids in order of first
// appearance, exactly as the reference's statement handler does.  Malformed
// lines raise VG_ERR_PARSE with the line number.
void ingest_ntriples(Ctx& ctx, const char* text, uint64_t len, bool literal_dict, Ingested& out);

// Result rows as text, one line per row, terms separated by tabs: an id
// decodes through the literal dictionary when that dictionary is in use and
// the id is a literal id, through the subject/object dictionary otherwise
// (SparqlResult::printResult, src/SparqlResult.cu:95-104; result columns
// never hold predicates here).  Unknown ids print as "?<id>".
std::string decode_rows(const Dict& d, const std::vector<const uint32_t*>& cols, uint64_t nrows);

// Reads and writes the reference's .vdd dictionary text: three sections
// (subject/object, predicate, literal), each its size and then "id term"
// lines (src/VedasBuild.cu:145-160; written here in id order).
void write_vdd(const Dict& d, const char* path);
void read_vdd(const char* path, Dict& d);

// Test hook: the number of hash bits used to group terms (63 by default);
// fewer bits force collisions so that the exact resolution path runs.
void set_ingest_hash_bits(int bits);

}  // namespace vg
