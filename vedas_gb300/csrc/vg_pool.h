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

// Queues fn(arg) for the pool's idle workers: work that no caller waits for
// (releasing the host state and intermediate relations of finished queries).
// Workers take it between parallel loops.
void post_background(void (*fn)(void*), void* arg);
// Runs the queued work on the caller and waits for what workers are running;
// rethrows the first error a queued task raised.  Called before a context or
// an index is destroyed, before memory statistics are read, and by the arena
// before it reports that it is out of memory.
void drain_background();

}  // namespace vg
