#pragma once

#include "vg_ctx.h"

namespace vg {

// Stable LSD radix sort of n keys over bits [0, end_bit).  When `vals` is
// non-null the uint32 values move with their keys; with vals_iota the values
// are generated as 0..n-1 (the input value buffer is not read).  Double
// buffered: returns true when the result is in (keys_alt, vals_alt).  With
// host_skip the digit histogram is read on the host (one synchronisation)
// and passes with a single digit value are skipped; without it nothing
// waits on the device.
bool radix_sort_u32(Ctx& ctx, uint32_t* keys, uint32_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                    uint64_t n, int end_bit, bool vals_iota, bool host_skip = true);
bool radix_sort_u64(Ctx& ctx, uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                    uint64_t n, int end_bit, bool vals_iota, bool host_skip = true);
// Keys only, ordered by bits [begin_bit, end_bit): a stable sort, so keys
// equal in those bits keep their input order (their lower bits included).
bool radix_sort_u64_bits(Ctx& ctx, uint64_t* keys, uint64_t* keys_alt, uint64_t n, int begin_bit, int end_bit);
void fill_iota(Ctx& ctx, uint32_t* out, uint64_t n);

}  // namespace vg
