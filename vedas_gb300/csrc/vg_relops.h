#pragma once

#include <vector>

#include "vg_ctx.h"

namespace vg {

// A device relation: ncols uint32 columns of nrows rows (column-major).
// Bit c of `borrowed` marks column c as a view into memory the relation does
// not own (a slice of an index array): it is never freed or written through
// the relation, and it may start at any 4-byte boundary.
struct Rel {
  uint32_t ncols = 0;
  uint64_t nrows = 0;
  uint32_t* cols[VG_MAX_COLS] = {nullptr};
  uint32_t borrowed = 0;
};

Rel rel_alloc(Ctx& ctx, uint32_t ncols, uint64_t nrows);
// Frees the owned columns.
void rel_free(Ctx& ctx, Rel& r);
// Frees column c if the relation owns it, and marks the slot owned (the
// caller stores an owned column there or drops it).
void rel_drop_col(Ctx& ctx, Rel& r, uint32_t c);
// Replaces every borrowed column by an owned copy (stream-ordered).
void rel_own(Ctx& ctx, Rel& r);

// One contiguous copy src[0, len) -> dst[0, len).
struct CopyPiece {
  const uint32_t* src;
  uint32_t* dst;
  uint64_t len;
};
// All pieces in one launch (up to 16).
void multi_copy(Ctx& ctx, const CopyPiece* pieces, int np);

// Adjacent-unique compaction of the rows of `in` (ncols columns, n rows) into
// `out`; returns the number of rows kept (synchronizes).
uint64_t unique_rows(Ctx& ctx, const uint32_t* const* in, uint32_t* const* out, uint32_t ncols,
                     uint64_t n);

// Sorted inner join of l and r on column 0 (two_keys: on columns 0 and 1).
// Output layout: key column(s), l's other columns, r's other columns; rows
// ordered by (left row, right row).  Allocates `out` from the arena.
void join(Ctx& ctx, const Rel& l, const Rel& r, bool two_keys, Rel& out);

// The same join on a caller's stream with caller-provided scratch and output
// columns (nothing is allocated): lo/cnt/offs hold l.nrows entries, status
// div_up(l.nrows, 2048) words; status, ticket and err must be zero.  Returns
// the result row count; the outputs are written only when it fits `capacity`.
uint64_t join_into(cudaStream_t stream, int num_sms, const Rel& l, const Rel& r, uint32_t* const* out_cols,
                   uint64_t capacity, uint32_t* lo, uint32_t* cnt, uint64_t* offs, uint64_t* status,
                   uint32_t* ticket, uint64_t* total, DeviceErrors* err);

// out[c][i] = in[c][perm[i]] for every column.
void gather_cols(Ctx& ctx, const uint32_t* const* in, uint32_t* const* out, uint32_t ncols,
                 const uint32_t* perm, uint64_t n);

// Stable sort of the rows by column 0 (in place; columns are replaced).
void sort_by_first(Ctx& ctx, Rel& r);
// Lexicographic sort of the rows over all columns (in place).
void sort_rows(Ctx& ctx, Rel& r);
// Adjacent duplicate-row removal in place.
void unique_in_place(Ctx& ctx, Rel& r);

// Copies `n` values of a device column to the host (synchronizes).
void download(Ctx& ctx, const uint32_t* dev, uint64_t n, uint32_t* host);

}  // namespace vg
