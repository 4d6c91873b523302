// Host worker pool shared by the batched engine (defined in vg_batch_host.cpp).
#pragma once

#include <stddef.h>

#include <functional>

namespace vg {

// Runs f(0) .. f(n - 1) on the host worker pool and the calling thread; small
// loops run on the caller alone.  One parallel loop at a time, so callers from
// other threads take turns.  The first exception an item throws is rethrown
// here once every item has run.
void parallel_for(size_t n, const std::function<void(size_t)>& f);

}  // namespace vg
