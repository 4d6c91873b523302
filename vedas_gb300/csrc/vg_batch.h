// Batched (multi-query) versions of the relation kernels: every call takes
// the work of many queries and issues a fixed, small number of launches.
//
// The *_enqueue / *_count / *_write forms only enqueue work on the context
// stream; the values they hand back land in page-locked host memory that is
// valid once the stream has passed that point (the caller records an event).
// The plain forms wait for their results.
#pragma once

#include <vector>

#include "vg_relops.h"

namespace vg {

// Page-locked host words for device->host reads of one pipeline stage,
// taken from and returned to the context's pool of page-locked chunks.
class PinnedWords {
 public:
  explicit PinnedWords(Ctx& ctx) : ctx_(ctx) {}
  PinnedWords(const PinnedWords&) = delete;
  PinnedWords& operator=(const PinnedWords&) = delete;
  ~PinnedWords();
  // At least `words` 64-bit words; may switch buffers, so only call it while
  // no copy into the buffer is pending.
  uint64_t* reserve(size_t words);
  uint64_t* data() const { return p_; }

 private:
  Ctx& ctx_;
  uint64_t* p_ = nullptr;
  size_t cap_ = 0;   // bytes
};

// All pieces in one launch (any number of pieces).
void batched_copy(Ctx& ctx, const std::vector<CopyPiece>& pieces);

// One relation segment: ncols columns of n rows, read from `in`, written to `out`.
struct SegRows {
  uint32_t ncols = 0;
  uint64_t n = 0;
  const uint32_t* in[VG_MAX_COLS] = {nullptr};
  uint32_t* out[VG_MAX_COLS] = {nullptr};
};

// Adjacent-unique compaction of every segment; each segment's kept row count
// goes to counts_host[s].
void batched_unique_enqueue(Ctx& ctx, const std::vector<SegRows>& segs, uint64_t* counts_host);
// Adds the compaction's written bytes to the kernel statistics once the
// counts are known.
void note_unique_writes(Ctx& ctx, const std::vector<SegRows>& segs, const uint64_t* counts);
std::vector<uint64_t> batched_unique(Ctx& ctx, const std::vector<SegRows>& segs);

// Stable sort of every relation by its column 0: one onesweep sort over
// (segment, key) composite keys, then one gather.  Columns are replaced.
// key_bits (1..32) bounds every key (keys < 2^key_bits): the passes are then
// fixed and nothing waits on the device; 0 reads the digit histogram on the
// host to skip passes.
void batched_sort_by_first(Ctx& ctx, const std::vector<Rel*>& rels, int key_bits);

// Inner joins on column 0 (l[j] with r[j], both sorted by column 0 and
// non-empty), in two halves.  batched_join_count enqueues the per-key match
// counts and their scan and copies each join's output size to
// totals_host[j]; batched_join_write, given those sizes, allocates the
// outputs from the arena, enqueues the output write, and copies column 0's
// first and last value of out[j] to first_last_host[2j], [2j+1] (zero for an
// empty output).  The relations must stay alive and unchanged in between.
struct JoinBatch {
  uint32_t J = 0;
  std::vector<const Rel*> l, r;
  std::vector<uint64_t> row0;   // offset of each join's left rows in lo/offs
  uint32_t* lo = nullptr;       // lower bound in r of every left key
  uint64_t* offs = nullptr;     // exclusive scan of the match counts
  uint64_t* d_totals = nullptr; // every join's output rows, on the device
  // Frees lo, offs and d_totals (in stream order).
  void release(Ctx& ctx);
};
void batched_join_count(Ctx& ctx, const std::vector<const Rel*>& l, const std::vector<const Rel*>& r, JoinBatch& jb,
                        uint64_t* totals_host);
// skip (optional, J flags): joins whose outputs are in out[] already; the
// others are allocated and written.  Releases jb's device arrays.
void batched_join_write(Ctx& ctx, JoinBatch& jb, const uint64_t* totals, std::vector<Rel>& out,
                        uint32_t* first_last_host, const uint8_t* skip = nullptr);

constexpr uint32_t kSmallC0Words = 100;   // staged column-0 words per small join output

// The join write without a host round trip after the count: the outputs are
// placed on the device in `region` (its bump pointer at d_bump, whose value
// after the wave is copied to *bump_host), written, and their first/last
// values copied to first_last_host and, for the joins with c0_slot[j] >= 0
// and 2 < rows < kSmallC0Words, column 0 to c0_host + slot * kSmallC0Words.
// Outputs that do not fit stay unplaced.  jb's device arrays stay alive:
// place_outputs_on_host then tells which joins were placed (the same
// arithmetic on the copied totals), and the caller writes the others with
// batched_join_write(..., skip = placed), or releases jb.
void batched_join_place_write(Ctx& ctx, JoinBatch& jb, const Arena::Region* region, uint64_t* d_bump,
                              const std::vector<int32_t>& c0_slot, uint32_t nslots, uint32_t* first_last_host,
                              uint32_t* c0_host, uint64_t* bump_host);
// Returns the region's bump after the wave; out[j] is the placed output of
// join j (placed[j] = 1) and `blocks` the number of its columns in the region.
uint64_t place_outputs_on_host(const JoinBatch& jb, const uint64_t* totals, const Arena::Region* region,
                               uint64_t bump, std::vector<Rel>& out, std::vector<uint8_t>& placed,
                               int64_t& blocks);
void batched_join(Ctx& ctx, const std::vector<const Rel*>& l, const std::vector<const Rel*>& r,
                  std::vector<Rel>& out, std::vector<uint32_t>& first_last);

// Column 0 of each relation copied to the host, back to back (one launch,
// one copy): col0_words(rels) uint32 words.
uint64_t col0_words(const std::vector<const Rel*>& rels);
void batched_col0_enqueue(Ctx& ctx, const std::vector<const Rel*>& rels, uint32_t* host);
void batched_col0(Ctx& ctx, const std::vector<const Rel*>& rels, std::vector<std::vector<uint32_t>>& out);

}  // namespace vg
