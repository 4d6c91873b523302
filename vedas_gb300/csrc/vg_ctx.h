// Execution context: one device, one stream, one HBM arena.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <unordered_map>
#include <vector>

#include "vg_common.cuh"

namespace vg {

// Allocator over one cudaMalloc'd slab.  Allocation is host-side bookkeeping
// only (no device call), so intermediate relations never pay a cudaMalloc.
// All work on the slab is ordered on the context stream, so a block may be
// handed out again as soon as the work that last used it has been enqueued.
//
// Blocks up to kSmallMax come from power-of-two size classes carved from
// kChunk-aligned chunks of the slab.  A directory with one entry per kChunk
// of the slab gives the class of any small block without a lock, and free lists
// are sharded by host thread, so the parallel host phases of a batch (which
// allocate and free relations of thousands of queries at once) almost never
// wait on each other.  Shards hand surplus blocks back to a global list and
// refill from it in batches.  Larger blocks are best-fit with coalescing
// under one lock.
// Called by Arena::alloc when a request does not fit, before it fails: frees
// whose release was deferred (drain_background) get their chance first.
void set_arena_reclaim(void (*fn)());

class Arena {
 public:
  Arena() = default;
  Arena(const Arena&) = delete;
  Arena& operator=(const Arena&) = delete;
  ~Arena() { release(); }
  void init(size_t bytes);                 // cudaMalloc's the slab
  // Manages [base, base + bytes), owned by the caller; the arena never
  // dereferences it (host-side tests use this).
  void init_at(void* base, size_t bytes);
  void release();
  void* alloc(size_t bytes);      // throws VG_ERR_OOM
  void* try_alloc(size_t bytes);  // nullptr when it does not fit
  void free(void* p);
  // Returns the tail of a live large block beyond new_bytes to the free list
  // (small blocks keep their class).
  void shrink(void* p, size_t new_bytes);
  size_t capacity() const { return cap_; }
  // Bytes in live blocks (small blocks count their class size).  Exact once
  // no other thread allocates or frees.
  size_t used() const;
  // The highest used() seen at a large allocation, a small-block refill from
  // the shared lists, or a call of used()/peak(): small blocks are counted in
  // their thread's shard, so no shared counter is touched per block.
  size_t peak() const;
  size_t largest_free() const;

  // Regions: one large block whose interior another allocator hands out (a
  // bump pointer on the device, which places every join output of a wave
  // without a host round trip).  The region holds one reference for its
  // opener; region_adopt adds one per interior block the host learns was
  // handed out, free() of an interior pointer drops one, and region_close
  // drops the opener's.  The block returns to the arena with the last
  // reference, so interior blocks may outlive the opener.
  struct Region {
    char* begin = nullptr;
    size_t bytes = 0;
    std::atomic<int64_t> refs{0};
  };
  Region* region_open(size_t bytes);      // nullptr when no block of that size is free or no slot is left
  void region_adopt(Region* r, int64_t blocks);
  void region_close(Region* r);

  static constexpr size_t kAlign = 256;
  static constexpr int kClasses = 16;                  // 256 B .. 8 MiB
  static constexpr size_t kSmallMax = kAlign << (kClasses - 1);
  static constexpr size_t kChunk = 4u << 20;           // directory granularity; chunks are kChunk-aligned
  // A class's chunk: 4 MiB, or two blocks for classes above 2 MiB.
  static constexpr size_t chunk_bytes(int c) {
    return (kAlign << c) * 2 > kChunk ? (kAlign << c) * 2 : kChunk;
  }

 private:
  static constexpr int kShards = 32;
  struct alignas(64) Shard {
    std::mutex mu;
    std::vector<size_t> free[kClasses];
    // bytes allocated minus bytes freed by the threads of this shard (a block
    // may be freed by another shard's thread, so one shard may go negative)
    std::atomic<int64_t> used{0};
  };
  char* base_ = nullptr;
  bool owned_ = false;
  size_t cap_ = 0;
  size_t big_used_ = 0;                                // live large blocks, under mu_
  mutable std::atomic<size_t> peak_{0};
  // under mu_
  std::map<size_t, size_t> free_;                      // offset -> size (large free blocks)
  std::set<std::pair<size_t, size_t>> by_size_;        // (size, offset) of the same blocks
  std::unordered_map<size_t, size_t> live_;            // offset -> size (large live blocks)
  std::vector<size_t> small_free_[kClasses];           // global lists of free small blocks
  mutable std::mutex mu_;
  // chunk position -> size class, -1 where no small chunk lies (read without a lock)
  std::unique_ptr<std::atomic<int8_t>[]> chunk_class_;
  size_t nchunks_ = 0;
  std::unique_ptr<Shard[]> shards_;

  static constexpr int kRegions = 64;
  Region regions_[kRegions];
  // [lo, hi) of each open region (lo null: slot free), read by free() without a lock
  std::atomic<char*> region_lo_[kRegions] = {};
  std::atomic<char*> region_hi_[kRegions] = {};
  std::atomic<int> nregions_{0};
  std::mutex region_mu_;
  void region_unref(int slot);

  void setup(char* base, size_t bytes, bool owned);
  size_t big_alloc(size_t bytes);                      // SIZE_MAX when it does not fit
  size_t chunk_alloc(size_t bytes);                    // a kChunk-aligned chunk, or SIZE_MAX
  void big_free(size_t off, size_t sz);
  void erase_by_size(size_t sz, size_t off);
  void take_free(size_t off, size_t sz);               // removes a free block from both indexes
  void add_free(size_t off, size_t sz);
  size_t sample_peak() const;                          // used(), folded into peak_
  int small_class(size_t off) const;
  static int my_shard();
};

// Per-kernel accounting: launches, algorithmic bytes (the bytes the
// operation must move, not what the kernel happens to move) and, when timing
// is on, CUDA-event durations on the context stream.
struct KernelStat {
  uint64_t launches = 0;
  double bytes = 0;
  double ms = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
};

// Frees held back until the work that may still read the blocks is known to
// be done: a wave engine with a stream of its own collects its frees here
// while its stage runs and hands them to the arena after its next wait on
// that stream (flush), so that no other engine's stream reuses a block that
// a kernel still in flight reads.
struct DeferredFrees {
  std::mutex mu;
  std::vector<void*> blocks;
  void push(void* p) {
    std::lock_guard<std::mutex> lk(mu);
    blocks.push_back(p);
  }
};

// Per host thread: the stream its work goes to (null: the context's own) and
// where its frees go (null: to the arena at once).  A wave engine sets both
// on its thread; the worker pools carry them into the items of a parallel
// loop.
struct ThreadExec {
  cudaStream_t stream = nullptr;
  DeferredFrees* defer = nullptr;
};
inline thread_local ThreadExec tl_exec;

// Sets the calling thread's ThreadExec for a scope.
struct ThreadExecScope {
  ThreadExec saved;
  explicit ThreadExecScope(const ThreadExec& e) : saved(tl_exec) { tl_exec = e; }
  ~ThreadExecScope() { tl_exec = saved; }
  ThreadExecScope(const ThreadExecScope&) = delete;
  ThreadExecScope& operator=(const ThreadExecScope&) = delete;
};

// The context's stream as seen by the calling thread: the thread's own
// stream when it has one (a wave engine's), else the context's.  Converts to
// cudaStream_t wherever a stream is passed.
struct StreamRef {
  cudaStream_t main = nullptr;
  operator cudaStream_t() const { return tl_exec.stream ? tl_exec.stream : main; }
};

// Launch parameters chosen per context (vg_tune_set; the autotuner picks
// them from timed trials).  Each choice changes only speed, never results.
struct TuneParams {
  uint32_t sort_items = 16;          // onesweep keys per thread: 8, 12 or 16
  uint32_t sort_lookback = 4;        // onesweep look-back words loaded at once: 1 or 4
  uint32_t join_small_rows = 256;    // joins with at most this many left rows: one warp each (0..256)
  uint32_t write_small_rows = 1024;  // outputs with at most this many rows: one warp each (0..4096)
  uint32_t unique_small_rows = 256;  // final compactions with at most this many rows: one warp each (0..256)
  uint32_t write_blocks_per_sm = 5;  // blocks per SM of a join write whose size is on the device (1..8; 5 fit)
};

struct Ctx {
  int device = 0;
  TuneParams tune;
  StreamRef stream;   // the context's stream (stream.main), or the calling thread's own
  Arena arena;
  DeviceErrors* d_err = nullptr;   // device error record
  int num_sms = 0;
  // pinned staging for small device->host reads (sizes, first/last keys)
  uint64_t* h_small = nullptr;
  static constexpr int kSmallWords = 1024;

  bool timing = false;
  uint64_t launches = 0;
  // page-locked upload ring: [ring_, ring_ + ring_cap_), regions in flight in FIFO order
  char* ring_ = nullptr;
  size_t ring_cap_ = 0, ring_head_ = 0;
  struct RingUse {
    size_t begin, end;
    cudaEvent_t done;
  };
  std::deque<RingUse> ring_used_;
  std::map<std::string, KernelStat> kstats;
  std::vector<cudaEvent_t> event_pool;

  // Guards the host-side state below (statistics, event pool, upload ring,
  // page-locked pool, download stream) when several threads issue work on
  // the context's stream at once (the wave engines of a batch).  Recursive: a
  // launch may upload.
  std::recursive_mutex host_mu;

  // Wraps one kernel launch on `stream`.
  template <typename F>
  void launch(const char* name, double algo_bytes, F&& f) {
    std::lock_guard<std::recursive_mutex> lk(host_mu);
    ++launches;
    KernelStat& k = kstats[name];
    k.launches++;
    k.bytes += algo_bytes;
    if (!timing) {
      f();
      return;
    }
    cudaEvent_t a = take_event(), b = take_event();
    VG_CUDA(cudaEventRecord(a, stream));
    f();
    VG_CUDA(cudaEventRecord(b, stream));
    k.pending.emplace_back(a, b);
  }
  cudaEvent_t take_event();
  // Converts recorded event pairs into milliseconds (synchronizes).
  void collect_timing();
  void reset_stats();

  // Page-locked host chunks kept for reuse (pinning memory is slow):
  // take_pinned returns one of at least `bytes`, give_pinned returns it.
  void* take_pinned(size_t bytes, size_t* got);
  void give_pinned(void* p, size_t bytes);
  // Adds algorithmic bytes to a kernel's statistics.
  void add_bytes(const char* name, double bytes) {
    std::lock_guard<std::recursive_mutex> lk(host_mu);
    kstats[name].bytes += bytes;
  }
  void release_pinned();
  std::vector<std::pair<void*, size_t>> pinned_free_;
  // A second stream for result downloads (created on first use).
  cudaStream_t dl_stream();
  void release_dl_stream();
  cudaStream_t dl_stream_ = nullptr;

  // Copies `bytes` from host memory to device memory `dst` on the stream,
  // through a page-locked ring, so the copy never waits for earlier work
  // (a copy from pageable memory may).  The caller's buffer is free to reuse
  // on return.
  void upload_bytes(void* dst, const void* src, size_t bytes);
  void release_upload_ring();

  template <typename T>
  T* alloc(uint64_t n) {
    return static_cast<T*>(arena.alloc((n ? n : 1) * sizeof(T)));
  }
  void free(void* p) {
    if (!p) return;
    if (tl_exec.defer) tl_exec.defer->push(p);
    else arena.free(p);
  }
  // Hands a collection of held-back frees to the arena (their work is done).
  void flush(DeferredFrees& d) {
    std::vector<void*> v;
    {
      std::lock_guard<std::mutex> lk(d.mu);
      v.swap(d.blocks);
    }
    for (void* p : v) arena.free(p);
  }
  void sync() { VG_CUDA(cudaStreamSynchronize(stream)); }
  // Raises VG_ERR_TIMEOUT / VG_ERR_OVERFLOW if a kernel recorded one (syncs).
  void check_device_errors();
  // The same for a copy of the record the caller already read back: clears
  // the device record and raises when `h` holds an error.
  void raise_device_errors(const DeviceErrors& h);
};

// RAII scratch buffer from the arena.
template <typename T>
struct Scratch {
  Ctx* ctx = nullptr;
  T* p = nullptr;
  Scratch() = default;
  Scratch(Ctx& c, uint64_t n) : ctx(&c), p(c.alloc<T>(n)) {}
  Scratch(const Scratch&) = delete;
  Scratch& operator=(const Scratch&) = delete;
  Scratch(Scratch&& o) noexcept : ctx(o.ctx), p(o.p) { o.p = nullptr; }
  ~Scratch() {
    if (p) ctx->free(p);
  }
  T* get() const { return p; }
};

}  // namespace vg
