// Fenced binary search: std::lower_bound / std::upper_bound over a sorted
// range of a large host array, with a sampled copy of every kFenceStride-th
// element (the fences, small enough to stay in the CPU caches) searched
// first, so that a search of a range of millions of elements touches the
// large array in one or two cache lines instead of a cache miss per halving.
// The answers are exactly the standard algorithms' answers.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

namespace vedas {

constexpr size_t kFenceStride = 64;

// fences[j] = a[j * kFenceStride]
inline std::vector<uint32_t> make_fences(const uint32_t* a, size_t n) {
  std::vector<uint32_t> f((n + kFenceStride - 1) / kFenceStride);
  for (size_t j = 0; j < f.size(); ++j) f[j] = a[j * kFenceStride];
  return f;
}

// First i in [lo, hi) with a[i] >= key (upper: a[i] > key), hi if none;
// a must be sorted on [lo, hi) and fences made from a.
inline size_t fenced_bound(const uint32_t* a, const std::vector<uint32_t>& fences, size_t lo, size_t hi,
                           uint64_t key, bool upper) {
  auto below = [&](uint32_t x) { return upper ? x <= key : x < key; };
  if (hi <= lo) return lo;
  if (hi - lo < 4 * kFenceStride || fences.empty()) {
    size_t l = lo, len = hi - lo;
    while (len > 0) {
      const size_t half = len >> 1;
      if (below(a[l + half])) {
        l += half + 1;
        len -= half + 1;
      } else {
        len = half;
      }
    }
    return l;
  }
  // fences whose positions lie in [lo, hi): j in [jl, jh)
  const size_t jl = (lo + kFenceStride - 1) / kFenceStride;
  const size_t jh = std::min(fences.size(), (hi - 1) / kFenceStride + 1);
  size_t p = jl, len = jh > jl ? jh - jl : 0;   // first fence in [jl, jh) that is not below key
  while (len > 0) {
    const size_t half = len >> 1;
    if (below(fences[p + half])) {
      p += half + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  // every fence before p is below key, fence p (if any) is not
  size_t l = (p > jl) ? (p - 1) * kFenceStride + 1 : lo;
  const size_t r = (p < jh) ? p * kFenceStride : hi;
  l = std::max(l, lo);
  size_t n = r > l ? r - l : 0;
  while (n > 0) {
    const size_t half = n >> 1;
    if (below(a[l + half])) {
      l += half + 1;
      n -= half + 1;
    } else {
      n = half;
    }
  }
  return l;
}

}  // namespace vedas
