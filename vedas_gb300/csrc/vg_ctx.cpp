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
  live_.clear();
  free_[0] = bytes;
  used_ = peak_ = 0;
}

void Arena::release() {
  if (base_) cudaFree(base_);
  base_ = nullptr;
  cap_ = used_ = 0;
  free_.clear();
  live_.clear();
}

void* Arena::try_alloc(size_t bytes) {
  std::lock_guard<std::mutex> lk(mu_);
  bytes = (bytes + kAlign - 1) / kAlign * kAlign;
  if (bytes == 0) bytes = kAlign;
  for (auto it = free_.begin(); it != free_.end(); ++it) {
    if (it->second >= bytes) {
      size_t off = it->first, sz = it->second;
      free_.erase(it);
      if (sz > bytes) free_[off + bytes] = sz - bytes;
      live_[off] = bytes;
      used_ += bytes;
      if (used_ > peak_) peak_ = used_;
      return base_ + off;
    }
  }
  return nullptr;
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
  size_t off = static_cast<size_t>(static_cast<char*>(p) - base_);
  auto it = live_.find(off);
  if (it == live_.end()) fail(VG_ERR_INVALID, "arena free of an unknown block");
  size_t sz = it->second;
  live_.erase(it);
  used_ -= sz;
  auto nx = free_.lower_bound(off);
  if (nx != free_.end() && off + sz == nx->first) {
    sz += nx->second;
    nx = free_.erase(nx);
  }
  if (nx != free_.begin()) {
    auto pv = std::prev(nx);
    if (pv->first + pv->second == off) {
      pv->second += sz;
      return;
    }
  }
  free_[off] = sz;
}

void Arena::shrink(void* p, size_t new_bytes) {
  if (!p) return;
  new_bytes = (new_bytes + kAlign - 1) / kAlign * kAlign;
  if (new_bytes == 0) new_bytes = kAlign;
  size_t off;
  size_t tail_off, tail_sz;
  {
    std::lock_guard<std::mutex> lk(mu_);
    off = static_cast<size_t>(static_cast<char*>(p) - base_);
    auto it = live_.find(off);
    if (it == live_.end()) fail(VG_ERR_INVALID, "arena shrink of an unknown block");
    if (new_bytes >= it->second) return;
    tail_off = off + new_bytes;
    tail_sz = it->second - new_bytes;
    it->second = new_bytes;
    live_[tail_off] = tail_sz;
  }
  free(base_ + tail_off);
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
