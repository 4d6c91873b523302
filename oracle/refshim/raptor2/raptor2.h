// Minimal host stand-in for the raptor2 names used by the VEDAS reference's
// SparqlQuery.cu (raptor2 is not installed here).  Test infrastructure only.
#ifndef VEDAS_ORACLE_RAPTOR2_STUB_H
#define VEDAS_ORACLE_RAPTOR2_STUB_H

#include <vector>

typedef struct raptor_world_s {
  int unused;
} raptor_world;

typedef struct raptor_uri_s {
  unsigned char* s;
} raptor_uri;

typedef struct raptor_sequence_s {
  std::vector<void*> items;
} raptor_sequence;

static inline raptor_world* raptor_new_world() { return new raptor_world(); }
static inline raptor_uri* raptor_new_uri(raptor_world*, const unsigned char* s) {
  raptor_uri* u = new raptor_uri();
  u->s = const_cast<unsigned char*>(s);
  return u;
}
static inline void raptor_free_uri(raptor_uri* u) { delete u; }
static inline unsigned char* raptor_uri_as_string(raptor_uri* u) { return u->s; }
static inline int raptor_sequence_size(raptor_sequence* s) { return static_cast<int>(s->items.size()); }
static inline void* raptor_sequence_get_at(raptor_sequence* s, int i) {
  return s->items[static_cast<size_t>(i)];
}

#endif
