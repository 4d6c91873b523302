#pragma once

#include <map>
#include <string>
#include <vector>

#include "vg_ctx.h"

namespace vg {

// A uint32 array resident in the context arena.
struct DevArray {
  uint32_t* ptr = nullptr;
  uint64_t len = 0;
  DevArray() = default;
  DevArray(uint32_t* p, uint64_t n) : ptr(p), len(n) {}
  void clear() {
    ptr = nullptr;
    len = 0;
  }
};

// What one permutation build produces (any subset).
struct PermOutputs {
  bool want_col1 = false, want_col2 = false, want_l1 = false, want_l2 = false;
  DevArray col1, col2, l1_vals, l1_offs, l2_vals, l2_offs;
};

void column_max3(Ctx& ctx, const uint32_t* a, const uint32_t* b, const uint32_t* c, uint64_t n,
                 uint32_t out[3]);

// Sorts the triples (k0, k1, k2) lexicographically and emits the requested
// outputs: col1/col2 = k1/k2 in sorted order, level-1 = (k0 run value, first
// row), level-2 = (k1 of each (k0,k1) run, first row).
void build_permutation(Ctx& ctx, const uint32_t* k0, const uint32_t* k1, const uint32_t* k2,
                       uint64_t n, const uint32_t maxes[3], PermOutputs& out);
// Two permutations sharing their leading column: (k0, k1, k2) into `first`
// and (k0, k2, k1) into `second`, the second re-sorted from the first's
// sorted keys by (k0, k2) bits only (fewer radix passes than a full sort).
void build_permutation_pair(Ctx& ctx, const uint32_t* k0, const uint32_t* k1, const uint32_t* k2, uint64_t n,
                            const uint32_t maxes[3], PermOutputs& first, PermOutputs& second);

// The resident permutation indexes in the reference's VedasStorage layout.
struct Index {
  Ctx* ctx = nullptr;
  bool full = false;
  uint64_t n = 0;
  uint32_t max_id = 0;   // largest subject, predicate or object id (bounds relation values)
  std::map<std::string, DevArray> dev;
  std::map<std::string, std::vector<uint32_t>> host;  // mirrors, made on request

  const DevArray& get(const std::string& name) const;
  const std::vector<uint32_t>& host_array(const std::string& name);
  void release();
};

// Builds the index from device-resident columns (hot path a).
void build_index(Ctx& ctx, const uint32_t* s, const uint32_t* p, const uint32_t* o, uint64_t n,
                 bool full, Index& ix);

// .vds files in the reference's layout (VedasStorage::write / open).
void write_vds(Index& ix, const char* path);
void open_vds(Ctx& ctx, const char* path, bool full, Index& ix);

}  // namespace vg
