// Batched (multi-query) versions of the relation kernels: every call takes
// the work of many queries and issues a fixed, small number of launches.
#pragma once

#include <vector>

#include "vg_relops.h"

namespace vg {

// All pieces in one launch (any number of pieces).
void batched_copy(Ctx& ctx, const std::vector<CopyPiece>& pieces);

// One relation segment: ncols columns of n rows, read from `in`, written to `out`.
struct SegRows {
  uint32_t ncols = 0;
  uint64_t n = 0;
  const uint32_t* in[VG_MAX_COLS] = {nullptr};
  uint32_t* out[VG_MAX_COLS] = {nullptr};
};

// Adjacent-unique compaction of every segment; returns each segment's kept
// row count (synchronizes once).
std::vector<uint64_t> batched_unique(Ctx& ctx, const std::vector<SegRows>& segs);

// Stable sort of every relation by its column 0: one onesweep sort over
// (segment, key) composite keys, then one gather.  Columns are replaced.
void batched_sort_by_first(Ctx& ctx, const std::vector<Rel*>& rels);

// Inner joins on column 0 (l[j] with r[j], both sorted by column 0 and
// non-empty).  Outputs are allocated from the arena; first_last[2j..2j+1]
// receives column 0's first and last value of out[j] (when non-empty).
void batched_join(Ctx& ctx, const std::vector<const Rel*>& l, const std::vector<const Rel*>& r,
                  std::vector<Rel>& out, std::vector<uint32_t>& first_last);

// Column 0 of each relation copied to the host (one launch, one copy).
void batched_col0(Ctx& ctx, const std::vector<const Rel*>& rels, std::vector<std::vector<uint32_t>>& out);

}  // namespace vg
