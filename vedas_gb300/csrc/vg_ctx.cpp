#include "vg_ctx.h"

#include <algorithm>
#include <cstring>

namespace vg {

void Arena::init(size_t bytes) {
  bytes = (bytes + kAlign - 1) / kAlign * kAlign;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) fail(VG_ERR_OOM, std::string("arena cudaMalloc: ") + cudaGetErrorString(e));
  setup(static_cast<char*>(p), bytes, true);
}

void Arena::init_at(void* base, size_t bytes) {
  setup(static_cast<char*>(base), bytes / kAlign * kAlign, false);
}

void Arena::setup(char* base, size_t bytes, bool owned) {
  release();
  base_ = base;
  owned_ = owned;
  cap_ = bytes;
  nchunks_ = bytes / kChunk + 1;
  chunk_class_.reset(new std::atomic<int8_t>[nchunks_]);
  for (size_t k = 0; k < nchunks_; ++k) chunk_class_[k].store(-1, std::memory_order_relaxed);
  shards_.reset(new Shard[kShards]);
  if (bytes) add_free(0, bytes);
  big_used_ = 0;
  peak_.store(0);
}

void Arena::release() {
  if (base_ && owned_) cudaFree(base_);
  base_ = nullptr;
  owned_ = false;
  cap_ = 0;
  free_.clear();
  by_size_.clear();
  live_.clear();
  for (auto& v : small_free_) v.clear();
  chunk_class_.reset();
  nchunks_ = 0;
  shards_.reset();
}

int Arena::my_shard() {
  static std::atomic<int> next{0};
  thread_local int idx = next.fetch_add(1, std::memory_order_relaxed) % kShards;
  return idx;
}

int Arena::small_class(size_t off) const {
  return chunk_class_[off / kChunk].load(std::memory_order_relaxed);
}

size_t Arena::used() const {
  if (!shards_) return 0;
  int64_t u = 0;
  for (int k = 0; k < kShards; ++k) u += shards_[k].used.load(std::memory_order_relaxed);
  std::lock_guard<std::mutex> lk(mu_);
  return static_cast<size_t>(u) + big_used_;
}

size_t Arena::sample_peak() const {
  const size_t u = used();
  size_t pk = peak_.load(std::memory_order_relaxed);
  while (u > pk && !peak_.compare_exchange_weak(pk, u, std::memory_order_relaxed)) {
  }
  return u;
}

size_t Arena::peak() const {
  sample_peak();
  return peak_.load(std::memory_order_relaxed);
}

void Arena::erase_by_size(size_t sz, size_t off) { by_size_.erase({sz, off}); }

void Arena::take_free(size_t off, size_t sz) {
  by_size_.erase({sz, off});
  free_.erase(off);
}

void Arena::add_free(size_t off, size_t sz) {
  free_[off] = sz;
  by_size_.emplace(sz, off);
}

// Best fit among the large free blocks; the remainder stays free.
size_t Arena::big_alloc(size_t bytes) {
  auto it = by_size_.lower_bound({bytes, size_t{0}});
  if (it == by_size_.end()) return SIZE_MAX;
  const size_t sz = it->first, off = it->second;
  take_free(off, sz);
  if (sz > bytes) add_free(off + bytes, sz - bytes);
  return off;
}

// Small-class chunks are carved from the top of the slab (the highest free
// block that holds a kChunk-aligned chunk of `bytes`, at its highest aligned
// position), while large blocks are split from the low end of their best fit,
// so chunks cluster at one end and do not fragment the space large relations
// need.
size_t Arena::chunk_alloc(size_t bytes) {
  auto carve = [&](size_t off, size_t sz) {
    if (sz < bytes) return SIZE_MAX;
    const size_t a = (off + sz - bytes) / kChunk * kChunk;
    if (a < off) return SIZE_MAX;
    take_free(off, sz);
    if (a > off) add_free(off, a - off);
    if (a + bytes < off + sz) add_free(a + bytes, off + sz - (a + bytes));
    return a;
  };
  int tries = 0;
  for (auto it = free_.rbegin(); it != free_.rend() && tries < 256; ++it, ++tries) {
    const size_t a = carve(it->first, it->second);
    if (a != SIZE_MAX) return a;
  }
  // none near the top: any block of bytes + kChunk - kAlign or more holds one
  auto it = by_size_.lower_bound({bytes + kChunk - kAlign, size_t{0}});
  if (it == by_size_.end()) return SIZE_MAX;
  return carve(it->second, it->first);
}

void Arena::big_free(size_t off, size_t sz) {
  auto nx = free_.lower_bound(off);
  if (nx != free_.end() && off + sz == nx->first) {
    erase_by_size(nx->second, nx->first);
    sz += nx->second;
    nx = free_.erase(nx);
  }
  if (nx != free_.begin()) {
    auto pv = std::prev(nx);
    if (pv->first + pv->second == off) {
      erase_by_size(pv->second, pv->first);
      pv->second += sz;
      by_size_.emplace(pv->second, pv->first);
      return;
    }
  }
  add_free(off, sz);
}

void* Arena::try_alloc(size_t bytes) {
  if (!base_) return nullptr;
  bytes = (bytes + kAlign - 1) / kAlign * kAlign;
  if (bytes == 0) bytes = kAlign;
  if (bytes <= kSmallMax) {
    int c = 0;
    while ((kAlign << c) < bytes) ++c;
    const size_t csz = kAlign << c;
    Shard& sh = shards_[my_shard()];
    {
      std::lock_guard<std::mutex> lk(sh.mu);
      if (!sh.free[c].empty()) {
        const size_t off = sh.free[c].back();
        sh.free[c].pop_back();
        sh.used.fetch_add(static_cast<int64_t>(csz), std::memory_order_relaxed);
        return base_ + off;
      }
    }
    // refill from the global list (a quarter of a chunk's worth of blocks,
    // at least two), or carve a new chunk
    std::vector<size_t> got;
    size_t big_off = SIZE_MAX;
    {
      std::lock_guard<std::mutex> lk(mu_);
      std::vector<size_t>& g = small_free_[c];
      if (!g.empty()) {
        const size_t batch = std::max<size_t>(2, kChunk / csz / 4);
        const size_t n = std::min(batch, g.size());
        got.assign(g.end() - static_cast<long>(n), g.end());
        g.resize(g.size() - n);
      } else {
        const size_t cb = chunk_bytes(c);
        const size_t a = chunk_alloc(cb);
        if (a != SIZE_MAX) {
          for (size_t k = 0; k < cb / kChunk; ++k)
            chunk_class_[a / kChunk + k].store(static_cast<int8_t>(c), std::memory_order_relaxed);
          for (size_t k = cb / csz; k-- > 0;) got.push_back(a + k * csz);
        } else {
          // no aligned chunk left: serve it as a large block
          big_off = big_alloc(bytes);
          if (big_off == SIZE_MAX) return nullptr;
          live_[big_off] = bytes;
          big_used_ += bytes;
        }
      }
    }
    if (big_off != SIZE_MAX) {
      sample_peak();
      return base_ + big_off;
    }
    const size_t off = got.back();
    got.pop_back();
    {
      std::lock_guard<std::mutex> lk(sh.mu);
      sh.free[c].insert(sh.free[c].end(), got.begin(), got.end());
      sh.used.fetch_add(static_cast<int64_t>(csz), std::memory_order_relaxed);
    }
    sample_peak();
    return base_ + off;
  }
  size_t off;
  {
    std::lock_guard<std::mutex> lk(mu_);
    off = big_alloc(bytes);
    if (off == SIZE_MAX) return nullptr;
    live_[off] = bytes;
    big_used_ += bytes;
  }
  sample_peak();
  return base_ + off;
}

namespace {
std::atomic<void (*)()> g_reclaim{nullptr};
}

void set_arena_reclaim(void (*fn)()) { g_reclaim.store(fn); }

void* Arena::alloc(size_t bytes) {
  void* p = try_alloc(bytes);
  if (!p) {
    if (void (*fn)() = g_reclaim.load()) {
      fn();
      p = try_alloc(bytes);
    }
  }
  if (!p)
    fail(VG_ERR_OOM, "arena exhausted: requested " + std::to_string(bytes) + " bytes, used " +
                         std::to_string(used()) + " of " + std::to_string(cap_));
  return p;
}

void Arena::free(void* p) {
  if (!p) return;
  if (nregions_.load(std::memory_order_acquire) > 0) {
    char* c = static_cast<char*>(p);
    for (int i = 0; i < kRegions; ++i) {
      char* lo = region_lo_[i].load(std::memory_order_acquire);
      if (lo && c >= lo && c < region_hi_[i].load(std::memory_order_acquire)) {
        region_unref(i);
        return;
      }
    }
  }
  const size_t off = static_cast<size_t>(static_cast<char*>(p) - base_);
  if (!base_ || off >= cap_) fail(VG_ERR_INVALID, "arena free of a pointer outside the slab");
  const int c = small_class(off);
  if (c >= 0) {
    const size_t csz = kAlign << c;
    Shard& sh = shards_[my_shard()];
    std::vector<size_t> spill;
    {
      std::lock_guard<std::mutex> lk(sh.mu);
      sh.used.fetch_sub(static_cast<int64_t>(csz), std::memory_order_relaxed);
      std::vector<size_t>& v = sh.free[c];
      v.push_back(off);
      // a shard keeps up to a chunk's worth of a class (at least 8 blocks);
      // the older half of a longer list goes back to the global list
      if (v.size() > std::max<size_t>(8, kChunk / csz)) {
        const size_t half = v.size() / 2;
        spill.assign(v.begin(), v.begin() + static_cast<long>(half));
        v.erase(v.begin(), v.begin() + static_cast<long>(half));
      }
    }
    if (!spill.empty()) {
      std::lock_guard<std::mutex> lk(mu_);
      small_free_[c].insert(small_free_[c].end(), spill.begin(), spill.end());
    }
    return;
  }
  std::lock_guard<std::mutex> lk(mu_);
  auto it = live_.find(off);
  if (it == live_.end()) fail(VG_ERR_INVALID, "arena free of an unknown block");
  const size_t sz = it->second;
  live_.erase(it);
  big_used_ -= sz;
  big_free(off, sz);
}

Arena::Region* Arena::region_open(size_t bytes) {
  bytes = std::max(bytes, kSmallMax + kAlign);      // always a large block
  void* p = try_alloc(bytes);
  if (!p) return nullptr;
  std::lock_guard<std::mutex> lk(region_mu_);
  for (int i = 0; i < kRegions; ++i) {
    if (region_lo_[i].load(std::memory_order_acquire) || regions_[i].refs.load() != 0) continue;
    Region& r = regions_[i];
    r.begin = static_cast<char*>(p);
    r.bytes = bytes;
    r.refs.store(1);
    region_hi_[i].store(r.begin + bytes, std::memory_order_release);
    region_lo_[i].store(r.begin, std::memory_order_release);
    nregions_.fetch_add(1, std::memory_order_acq_rel);
    return &r;
  }
  free(p);
  return nullptr;
}

void Arena::region_adopt(Region* r, int64_t blocks) {
  if (r && blocks > 0) r->refs.fetch_add(blocks, std::memory_order_acq_rel);
}

void Arena::region_close(Region* r) {
  if (!r) return;
  region_unref(static_cast<int>(r - regions_));
}

void Arena::region_unref(int slot) {
  Region& r = regions_[slot];
  if (r.refs.fetch_sub(1, std::memory_order_acq_rel) != 1) return;
  // the last reference: the slot is cleared before the block goes back, so no
  // later free of a block carved from the same bytes is taken for the region's
  char* b = r.begin;
  {
    std::lock_guard<std::mutex> lk(region_mu_);
    region_lo_[slot].store(nullptr, std::memory_order_release);
    region_hi_[slot].store(nullptr, std::memory_order_release);
    nregions_.fetch_sub(1, std::memory_order_acq_rel);
    r.begin = nullptr;
    r.bytes = 0;
  }
  free(b);
}

void Arena::shrink(void* p, size_t new_bytes) {
  if (!p) return;
  new_bytes = (new_bytes + kAlign - 1) / kAlign * kAlign;
  if (new_bytes == 0) new_bytes = kAlign;
  const size_t off = static_cast<size_t>(static_cast<char*>(p) - base_);
  if (!base_ || off >= cap_) fail(VG_ERR_INVALID, "arena shrink of a pointer outside the slab");
  if (small_class(off) >= 0) return;
  std::lock_guard<std::mutex> lk(mu_);
  auto it = live_.find(off);
  if (it == live_.end()) fail(VG_ERR_INVALID, "arena shrink of an unknown block");
  if (new_bytes >= it->second) return;
  const size_t tail = it->second - new_bytes;
  it->second = new_bytes;
  big_used_ -= tail;
  big_free(off + new_bytes, tail);
}

size_t Arena::largest_free() const {
  std::lock_guard<std::mutex> lk(mu_);
  size_t m = 0;
  for (auto& kv : free_) m = kv.second > m ? kv.second : m;
  return m;
}

void Ctx::upload_bytes(void* dst, const void* src, size_t bytes) {
  std::lock_guard<std::recursive_mutex> lk(host_mu);
  if (bytes == 0) return;
  constexpr size_t kRingMin = size_t{16} << 20;
  const size_t need = (bytes + 255) / 256 * 256;
  if (need > ring_cap_) {
    // grow: wait for every copy out of the old ring, then replace it
    for (RingUse& u : ring_used_) {
      VG_CUDA(cudaEventSynchronize(u.done));
      event_pool.push_back(u.done);
    }
    ring_used_.clear();
    if (ring_) VG_CUDA(cudaFreeHost(ring_));
    ring_ = nullptr;
    ring_cap_ = 0;
    size_t cap = kRingMin;
    while (cap < 4 * need) cap *= 2;
    VG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&ring_), cap, cudaHostAllocDefault));
    ring_cap_ = cap;
    ring_head_ = 0;
  }
  if (ring_head_ + need > ring_cap_) ring_head_ = 0;
  const size_t b = ring_head_, e = ring_head_ + need;
  // regions are reused in FIFO order: retire the oldest copies until [b, e) is free
  while (!ring_used_.empty()) {
    const RingUse& u = ring_used_.front();
    const bool overlaps = u.begin < e && b < u.end;
    if (!overlaps && cudaEventQuery(u.done) != cudaSuccess) break;
    VG_CUDA(cudaEventSynchronize(u.done));
    event_pool.push_back(u.done);
    ring_used_.pop_front();
  }
  for (const RingUse& u : ring_used_)
    if (u.begin < e && b < u.end) fail(VG_ERR_CUDA, "upload ring bookkeeping");
  std::memcpy(ring_ + b, src, bytes);
  VG_CUDA(cudaMemcpyAsync(dst, ring_ + b, bytes, cudaMemcpyHostToDevice, stream));
  cudaEvent_t ev = take_event();
  VG_CUDA(cudaEventRecord(ev, stream));
  ring_used_.push_back({b, e, ev});
  ring_head_ = e;
}

void Ctx::release_upload_ring() {
  for (RingUse& u : ring_used_) {
    cudaEventSynchronize(u.done);
    cudaEventDestroy(u.done);
  }
  ring_used_.clear();
  if (ring_) cudaFreeHost(ring_);
  ring_ = nullptr;
  ring_cap_ = ring_head_ = 0;
  for (cudaEvent_t e : event_pool) cudaEventDestroy(e);
  event_pool.clear();
}

void* Ctx::take_pinned(size_t bytes, size_t* got) {
  std::lock_guard<std::recursive_mutex> lk(host_mu);
  // best fit among chunks no more than four times the request, so small
  // buffers do not tie up the large result chunks
  size_t best = SIZE_MAX;
  for (size_t i = 0; i < pinned_free_.size(); ++i) {
    const size_t sz = pinned_free_[i].second;
    if (sz >= bytes && sz / 4 <= bytes && (best == SIZE_MAX || sz < pinned_free_[best].second)) best = i;
  }
  if (best != SIZE_MAX) {
    auto pr = pinned_free_[best];
    pinned_free_.erase(pinned_free_.begin() + static_cast<long>(best));
    *got = pr.second;
    return pr.first;
  }
  void* p = nullptr;
  VG_CUDA(cudaHostAlloc(&p, bytes, cudaHostAllocDefault));
  *got = bytes;
  return p;
}

void Ctx::give_pinned(void* p, size_t bytes) {
  std::lock_guard<std::recursive_mutex> lk(host_mu);
  if (p) pinned_free_.emplace_back(p, bytes);
}

void Ctx::release_pinned() {
  for (auto& pr : pinned_free_) cudaFreeHost(pr.first);
  pinned_free_.clear();
}

cudaStream_t Ctx::dl_stream() {
  std::lock_guard<std::recursive_mutex> lk(host_mu);
  if (!dl_stream_) VG_CUDA(cudaStreamCreateWithFlags(&dl_stream_, cudaStreamNonBlocking));
  return dl_stream_;
}

void Ctx::release_dl_stream() {
  if (dl_stream_) {
    cudaStreamSynchronize(dl_stream_);
    cudaStreamDestroy(dl_stream_);
  }
  dl_stream_ = nullptr;
}

cudaEvent_t Ctx::take_event() {
  std::lock_guard<std::recursive_mutex> lk(host_mu);
  if (!event_pool.empty()) {
    cudaEvent_t e = event_pool.back();
    event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  VG_CUDA(cudaEventCreate(&e));
  return e;
}

void Ctx::collect_timing() {
  std::lock_guard<std::recursive_mutex> lk(host_mu);
  sync();
  for (auto& kv : kstats) {
    for (auto& pr : kv.second.pending) {
      float ms = 0;
      VG_CUDA(cudaEventElapsedTime(&ms, pr.first, pr.second));
      kv.second.ms += ms;
      event_pool.push_back(pr.first);
      event_pool.push_back(pr.second);
    }
    kv.second.pending.clear();
  }
}

void Ctx::reset_stats() {
  std::lock_guard<std::recursive_mutex> lk(host_mu);
  collect_timing();
  launches = 0;
  kstats.clear();
}

void Ctx::check_device_errors() {
  DeviceErrors h{};
  VG_CUDA(cudaMemcpyAsync(&h, d_err, sizeof(h), cudaMemcpyDeviceToHost, stream));
  sync();
  raise_device_errors(h);
}

void Ctx::raise_device_errors(const DeviceErrors& h) {
  if (h.timeout || h.overflow) {
    VG_CUDA(cudaMemsetAsync(d_err, 0, sizeof(DeviceErrors), stream));
    if (h.timeout) fail(VG_ERR_TIMEOUT, "a bounded device wait expired");
    fail(VG_ERR_OVERFLOW, "device output overflowed its reservation");
  }
}

}  // namespace vg
