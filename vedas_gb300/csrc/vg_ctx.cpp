#include "vg_ctx.h"

namespace vg {

void Arena::init(size_t bytes) {
  bytes = (bytes + kAlign - 1) / kAlign * kAlign;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) fail(VG_ERR_OOM, std::string("arena cudaMalloc: ") + cudaGetErrorString(e));
  base_ = static_cast<char*>(p);
  cap_ = bytes;
  free_.clear();
  by_size_.clear();
  live_.clear();
  small_live_.clear();
  for (auto& v : small_free_) v.clear();
  free_[0] = bytes;
  by_size_.emplace(bytes, size_t{0});
  used_ = peak_ = 0;
}

void Arena::release() {
  if (base_) cudaFree(base_);
  base_ = nullptr;
  cap_ = used_ = 0;
  free_.clear();
  by_size_.clear();
  live_.clear();
  small_live_.clear();
  for (auto& v : small_free_) v.clear();
}

void Arena::erase_by_size(size_t sz, size_t off) { by_size_.erase({sz, off}); }

// Best fit among the large free blocks; the remainder stays free.
size_t Arena::big_alloc(size_t bytes) {
  auto it = by_size_.lower_bound({bytes, size_t{0}});
  if (it == by_size_.end()) return SIZE_MAX;
  const size_t sz = it->first, off = it->second;
  by_size_.erase(it);
  free_.erase(off);
  if (sz > bytes) {
    free_[off + bytes] = sz - bytes;
    by_size_.emplace(sz - bytes, off + bytes);
  }
  return off;
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
  free_[off] = sz;
  by_size_.emplace(sz, off);
}

void* Arena::try_alloc(size_t bytes) {
  std::lock_guard<std::mutex> lk(mu_);
  bytes = (bytes + kAlign - 1) / kAlign * kAlign;
  if (bytes == 0) bytes = kAlign;
  if (bytes <= kSmallMax) {
    int c = 0;
    while ((kAlign << c) < bytes) ++c;
    const size_t csz = kAlign << c;
    if (small_free_[c].empty()) {
      const size_t chunk = csz * 16 > kChunk ? csz * 16 : kChunk;
      const size_t off = big_alloc(chunk);
      if (off == SIZE_MAX) return nullptr;
      for (size_t k = chunk / csz; k-- > 0;) small_free_[c].push_back(off + k * csz);
    }
    const size_t off = small_free_[c].back();
    small_free_[c].pop_back();
    small_live_[off] = c;
    used_ += csz;
    if (used_ > peak_) peak_ = used_;
    return base_ + off;
  }
  const size_t off = big_alloc(bytes);
  if (off == SIZE_MAX) return nullptr;
  live_[off] = bytes;
  used_ += bytes;
  if (used_ > peak_) peak_ = used_;
  return base_ + off;
}

void* Arena::alloc(size_t bytes) {
  void* p = try_alloc(bytes);
  if (!p)
    fail(VG_ERR_OOM, "arena exhausted: requested " + std::to_string(bytes) + " bytes, used " +
                         std::to_string(used_) + " of " + std::to_string(cap_));
  return p;
}

void Arena::free(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(mu_);
  const size_t off = static_cast<size_t>(static_cast<char*>(p) - base_);
  auto sm = small_live_.find(off);
  if (sm != small_live_.end()) {
    const int c = sm->second;
    small_live_.erase(sm);
    small_free_[c].push_back(off);
    used_ -= kAlign << c;
    return;
  }
  auto it = live_.find(off);
  if (it == live_.end()) fail(VG_ERR_INVALID, "arena free of an unknown block");
  const size_t sz = it->second;
  live_.erase(it);
  used_ -= sz;
  big_free(off, sz);
}

void Arena::shrink(void* p, size_t new_bytes) {
  if (!p) return;
  new_bytes = (new_bytes + kAlign - 1) / kAlign * kAlign;
  if (new_bytes == 0) new_bytes = kAlign;
  std::lock_guard<std::mutex> lk(mu_);
  const size_t off = static_cast<size_t>(static_cast<char*>(p) - base_);
  if (small_live_.count(off)) return;
  auto it = live_.find(off);
  if (it == live_.end()) fail(VG_ERR_INVALID, "arena shrink of an unknown block");
  if (new_bytes >= it->second) return;
  const size_t tail = it->second - new_bytes;
  it->second = new_bytes;
  used_ -= tail;
  big_free(off + new_bytes, tail);
}

size_t Arena::largest_free() const {
  std::lock_guard<std::mutex> lk(mu_);
  size_t m = 0;
  for (auto& kv : free_) m = kv.second > m ? kv.second : m;
  return m;
}

cudaEvent_t Ctx::take_event() {
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
  collect_timing();
  launches = 0;
  kstats.clear();
}

void Ctx::check_device_errors() {
  DeviceErrors h{};
  VG_CUDA(cudaMemcpyAsync(&h, d_err, sizeof(h), cudaMemcpyDeviceToHost, stream));
  sync();
  if (h.timeout || h.overflow) {
    VG_CUDA(cudaMemsetAsync(d_err, 0, sizeof(DeviceErrors), stream));
    if (h.timeout) fail(VG_ERR_TIMEOUT, "a bounded device wait expired");
    fail(VG_ERR_OVERFLOW, "device output overflowed its reservation");
  }
}

}  // namespace vg
