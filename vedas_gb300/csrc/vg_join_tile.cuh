// Join count over one tile of left keys, with the matching window of right
// keys staged in shared memory by a bulk (TMA) copy.
#pragma once

#include "vg_prims.cuh"

namespace vg {

constexpr int kJcBlock = 256;
constexpr int kJcKeys = 8;                      // left keys per thread, consecutive
constexpr int kJcTile = kJcBlock * kJcKeys;     // 2048 left keys per block
constexpr int kJcWindow = 11264;                // right keys staged per block (44 KiB)

struct JoinCountSmem {
  alignas(16) uint32_t keys[kJcWindow + 8];
  alignas(8) uint64_t bar;
  uint64_t w0, w1;
  uint32_t staged;   // 0: search global memory, 1: window loaded by threads, 2: bulk copy
  uint32_t failed;
};

__device__ __forceinline__ uint64_t smem_lower(const uint32_t* keys, uint64_t base, uint64_t lo, uint64_t hi,
                                               uint32_t key) {
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (keys[mid - base] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint64_t smem_upper(const uint32_t* keys, uint64_t base, uint64_t lo, uint64_t hi,
                                               uint32_t key) {
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (key < keys[mid - base]) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// Lower bound (in R) and match count of L[i0, min(i0 + kJcTile, nl)).  R is
// sorted; the window of R that can match the tile, [lower(L[i0]),
// upper(L[last])), is staged in shared memory when it fits: its 16-byte
// aligned middle by one cp.async.bulk completed on an mbarrier, its ragged
// ends by plain loads.  A window that does not fit (a heavy key, or a right
// side much larger than the left) is searched in global memory instead.
__device__ __forceinline__ void join_count_tile(const uint32_t* __restrict__ L, uint64_t nl,
                                                const uint32_t* __restrict__ R, uint64_t nr, uint64_t i0,
                                                uint32_t* __restrict__ lo_out, uint32_t* __restrict__ cnt_out,
                                                JoinCountSmem& sm, DeviceErrors* err) {
  const uint32_t tid = threadIdx.x;
  const uint64_t i_end = (i0 + kJcTile < nl) ? i0 + kJcTile : nl;
  if (tid == 0) {
    const uint64_t w0 = lower_bound_dev(R, 0, nr, L[i0]);
    const uint64_t w1 = upper_bound_dev(R, w0, nr, L[i_end - 1]);
    sm.w0 = w0;
    sm.w1 = w1;
    sm.staged = 0;
    sm.failed = 0;
    if (w1 > w0 && w1 - w0 <= kJcWindow) {
      const uint64_t base = w0 & ~3ull;
      const uint64_t a0 = (w0 + 3) & ~3ull, a1 = w1 & ~3ull;
      if ((reinterpret_cast<uintptr_t>(R) & 15) == 0 && a1 > a0) {
        mbar_init(&sm.bar, 1);
        const uint32_t bytes = static_cast<uint32_t>((a1 - a0) * 4);
        mbar_arrive_expect_tx(&sm.bar, bytes);
        bulk_copy_g2s(&sm.keys[a0 - base], R + a0, bytes, &sm.bar);
        sm.staged = 2;
      } else {
        sm.staged = 1;
      }
    }
  }
  __syncthreads();
  const uint64_t w0 = sm.w0, w1 = sm.w1;
  const uint32_t staged = sm.staged;
  const uint64_t base = w0 & ~3ull;
  if (staged) {
    const uint64_t a0 = (staged == 2) ? ((w0 + 3) & ~3ull) : w1;
    const uint64_t a1 = (staged == 2) ? (w1 & ~3ull) : w1;
    for (uint64_t e = w0 + tid; e < a0; e += kJcBlock) sm.keys[e - base] = R[e];
    for (uint64_t e = a1 + tid; e < w1; e += kJcBlock) sm.keys[e - base] = R[e];
  }
  if (staged == 2) {
    // every consumer observes the barrier phase itself (bounded)
    if (!mbar_wait_bounded(&sm.bar, 0, err)) {
      sm.failed = 1;
      mbar_wait_bounded(&sm.bar, 0, err);  // a late copy gets a second bounded chance to land
    }
  }
  __syncthreads();
  const bool use_smem = staged != 0 && sm.failed == 0;

  uint64_t prev = w0;
#pragma unroll
  for (int j = 0; j < kJcKeys; ++j) {
    const uint64_t i = i0 + static_cast<uint64_t>(tid) * kJcKeys + j;
    if (i >= i_end) break;
    const uint32_t key = L[i];
    uint64_t lo, hi;
    if (use_smem) {
      lo = smem_lower(sm.keys, base, prev, w1, key);
      hi = smem_upper(sm.keys, base, lo, w1, key);
    } else {
      lo = lower_bound_dev(R, prev, w1, key);
      hi = upper_bound_dev(R, lo, w1, key);
    }
    prev = lo;
    lo_out[i] = static_cast<uint32_t>(lo);
    cnt_out[i] = static_cast<uint32_t>(hi - lo);
  }
}

}  // namespace vg
