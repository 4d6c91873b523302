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

// Searches over the staged window, in 32-bit offsets from its first key
// (s points at it in shared memory, n keys).  kUpper: first offset whose key
// is above `key`; otherwise first offset whose key is not below it.
template <bool kUpper>
__device__ __forceinline__ bool smem_below(const uint32_t* s, uint32_t i, uint32_t key) {
  const uint32_t a = s[i];
  return kUpper ? (a <= key) : (a < key);
}

// Binary search over [lo, n).
template <bool kUpper>
__device__ __forceinline__ uint32_t smem_search(const uint32_t* s, uint32_t lo, uint32_t n, uint32_t key) {
  uint32_t len = n - lo;
  while (len > 0) {
    const uint32_t half = len >> 1;
    if (smem_below<kUpper>(s, lo + half, key)) {
      lo += half + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  return lo;
}

// The same answer at or after `from`, galloping from there (steps 1, 2, 4,
// ... then a binary search inside the last step): a thread's left keys are
// consecutive, so the next bound is usually a few keys further on.
template <bool kUpper>
__device__ __forceinline__ uint32_t smem_gallop(const uint32_t* s, uint32_t from, uint32_t n, uint32_t key) {
  if (from >= n || !smem_below<kUpper>(s, from, key)) return from;
  uint32_t lo = from, step = 1, hi = n;
  while (true) {
    const uint32_t nx = lo + step;
    if (nx >= n) break;
    if (!smem_below<kUpper>(s, nx, key)) {
      hi = nx;
      break;
    }
    lo = nx;
    step <<= 1;
  }
  // below(lo) holds and the answer lies in (lo, hi]
  return smem_search<kUpper>(s, lo + 1, hi, key);
}

// First index in R[lo, hi) whose key is not below `key` (kUpper: above it),
// found by one warp: each round 31 lanes probe evenly spaced keys and the
// ballot of their comparisons narrows the range 32-fold, so a search over
// 10^8 keys takes six rounds of parallel loads instead of 27 dependent ones.
// Every lane of the warp must call it with the same arguments.
template <bool kUpper, typename T>
__device__ __forceinline__ uint64_t warp_bound(const T* __restrict__ R, uint64_t lo, uint64_t hi, T key) {
  const uint32_t lane = threadIdx.x & 31;
  while (hi - lo > 32) {
    const uint64_t step = (hi - lo + 31) >> 5;
    const uint64_t p = lo + static_cast<uint64_t>(lane + 1) * step;
    bool below = false;
    if (lane < 31 && p < hi) {
      const T a = __ldg(R + p);
      below = kUpper ? (a <= key) : (a < key);
    }
    const uint32_t c = __popc(__ballot_sync(0xffffffffu, below));
    const uint64_t nlo = c ? lo + static_cast<uint64_t>(c) * step + 1 : lo;
    const uint64_t cap = lo + static_cast<uint64_t>(c + 1) * step;
    hi = cap < hi ? cap : hi;
    lo = nlo;
  }
  bool below = false;
  if (lo + lane < hi) {
    const T a = __ldg(R + lo + lane);
    below = kUpper ? (a <= key) : (a < key);
  }
  return lo + __popc(__ballot_sync(0xffffffffu, below));
}

// Two bounds in R[0, n) by one warp at once: lanes 0-15 find the first
// index whose key is above ka (kUpperA) or not below it, lanes 16-31 the
// same for kb (kUpperB).  Each round every half-warp probes 15 evenly spaced
// keys of its range and the ballot of its comparisons narrows the range
// 16-fold.  Every lane of the warp must call it with the same arguments;
// every lane gets both bounds.
template <bool kUpperA, bool kUpperB, typename T>
__device__ __forceinline__ void warp_bound_pair(const T* __restrict__ R, uint64_t n, T ka, T kb, uint64_t& ra,
                                                uint64_t& rb) {
  const uint32_t lane = threadIdx.x & 31, sl = lane & 15;
  const bool second = lane >= 16;
  const bool upper = second ? kUpperB : kUpperA;
  const uint32_t half = second ? 0xffff0000u : 0x0000ffffu;
  const T key = second ? kb : ka;
  uint64_t lo = 0, hi = n;
  while (true) {
    const bool wide = hi - lo > 16;
    if (__ballot_sync(0xffffffffu, wide) == 0) break;
    uint64_t step = 0;
    bool below = false;
    if (wide) {
      step = (hi - lo + 15) >> 4;
      const uint64_t p = lo + static_cast<uint64_t>(sl + 1) * step;
      if (sl < 15 && p < hi) {
        const T a = __ldg(R + p);
        below = upper ? (a <= key) : (a < key);
      }
    }
    const uint32_t c = __popc(__ballot_sync(0xffffffffu, below) & half);
    if (wide) {
      const uint64_t nlo = c ? lo + static_cast<uint64_t>(c) * step + 1 : lo;
      const uint64_t cap = lo + static_cast<uint64_t>(c + 1) * step;
      hi = cap < hi ? cap : hi;
      lo = nlo;
    }
  }
  bool below = false;
  if (lo + sl < hi) {
    const T a = __ldg(R + lo + sl);
    below = upper ? (a <= key) : (a < key);
  }
  const uint64_t res = lo + __popc(__ballot_sync(0xffffffffu, below) & half);
  ra = __shfl_sync(0xffffffffu, res, 0);
  rb = __shfl_sync(0xffffffffu, res, 16);
}

// A tile's right-key window: the lower bound of klo and the upper bound of
// khi in R[0, nr), by one warp.
__device__ __forceinline__ void warp_window(const uint32_t* __restrict__ R, uint64_t nr, uint32_t klo,
                                            uint32_t khi, uint64_t& w0, uint64_t& w1) {
  warp_bound_pair<false, true, uint32_t>(R, nr, klo, khi, w0, w1);
}

// Lower and upper bounds of K keys in R[w0, w1) at once: branchless binary
// searches advanced in lockstep, so each round has 2K independent loads in
// flight instead of one dependent chain per key.
template <int K>
__device__ __forceinline__ void lockstep_bounds(const uint32_t* __restrict__ R, uint64_t w0, uint64_t w1,
                                                const uint32_t (&key)[K], uint64_t (&lo)[K], uint64_t (&hi)[K]) {
  if (w1 <= w0) {
#pragma unroll
    for (int j = 0; j < K; ++j) lo[j] = hi[j] = w0;
    return;
  }
#pragma unroll
  for (int j = 0; j < K; ++j) lo[j] = hi[j] = w0;
  uint64_t n = w1 - w0;
  while (n > 1) {
    const uint64_t half = n >> 1;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const uint32_t a = __ldg(R + lo[j] + half);
      const uint32_t b = __ldg(R + hi[j] + half);
      lo[j] = (a < key[j]) ? lo[j] + half : lo[j];
      hi[j] = (b <= key[j]) ? hi[j] + half : hi[j];
    }
    n -= half;
  }
#pragma unroll
  for (int j = 0; j < K; ++j) {
    lo[j] += (__ldg(R + lo[j]) < key[j]) ? 1 : 0;
    hi[j] += (__ldg(R + hi[j]) <= key[j]) ? 1 : 0;
  }
}

// lockstep_bounds with 32-bit positions (every join side has fewer than 2^32
// rows), which halves the registers the bounds hold.
template <int K>
__device__ __forceinline__ void lockstep_bounds32(const uint32_t* __restrict__ R, uint32_t w0, uint32_t w1,
                                                  const uint32_t (&key)[K], uint32_t (&lo)[K], uint32_t (&hi)[K]) {
#pragma unroll
  for (int j = 0; j < K; ++j) lo[j] = hi[j] = w0;
  if (w1 <= w0) return;
  uint32_t n = w1 - w0;
  while (n > 1) {
    const uint32_t half = n >> 1;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      const uint32_t a = __ldg(R + lo[j] + half);
      const uint32_t b = __ldg(R + hi[j] + half);
      lo[j] = (a < key[j]) ? lo[j] + half : lo[j];
      hi[j] = (b <= key[j]) ? hi[j] + half : hi[j];
    }
    n -= half;
  }
#pragma unroll
  for (int j = 0; j < K; ++j) {
    lo[j] += (__ldg(R + lo[j]) < key[j]) ? 1 : 0;
    hi[j] += (__ldg(R + hi[j]) <= key[j]) ? 1 : 0;
  }
}

// Thread 0 of the block: records the tile's right-key window [w0, w1) and
// decides how it is staged in shared memory (sm.staged: 0 not staged, 1 by
// the block's threads, 2 its 16-byte aligned middle by one cp.async.bulk
// completed on sm.bar, its ragged ends by the threads).  The block must pass
// a barrier before jc_count_staged.
__device__ __forceinline__ void jc_issue_window(const uint32_t* __restrict__ R, uint64_t w0, uint64_t w1,
                                                JoinCountSmem& sm) {
  sm.w0 = w0;
  sm.w1 = w1;
  sm.staged = 0;
  sm.failed = 0;
  // R may start at any 4-byte boundary (a view of an index slice): element e
  // sits on a 16-byte boundary when (e + mis) % 4 == 0, and the window is laid
  // out in shared memory from `base`, the aligned element at or below w0
  // (index arithmetic is modulo 2^64, so base may lie below element 0).
  const uint64_t mis = (reinterpret_cast<uintptr_t>(R) >> 2) & 3u;
  if (w1 > w0 && w1 - w0 <= kJcWindow) {
    const uint64_t base = ((w0 + mis) & ~3ull) - mis;
    const uint64_t a0 = ((w0 + mis + 3) & ~3ull) - mis, a1 = ((w1 + mis) & ~3ull) - mis;
    if (a1 > a0 && a1 <= w1) {
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

// Lower bound (in R) and match count of L[i0, min(i0 + kJcTile, nl)), given
// the window that jc_issue_window recorded: every left key of the tile lies
// in it.  A staged window is searched in shared memory; one that does not
// fit (a heavy key, or a right side much longer than the left) is searched in
// global memory with lockstep bounds instead.
// The tile's counts stay in registers: thread t holds the counts of left
// keys i0 + 8t .. i0 + 8t + 7 in cnt[] and their lower bounds in lov[] (zero
// past the end).  Every thread of the block must call it.
__device__ __forceinline__ void jc_count_staged(const uint32_t* __restrict__ L, uint64_t nl,
                                                const uint32_t* __restrict__ R, uint64_t i0,
                                                uint32_t (&lov)[kJcKeys], uint32_t (&cnt)[kJcKeys],
                                                JoinCountSmem& sm, DeviceErrors* err) {
#pragma unroll
  for (int j = 0; j < kJcKeys; ++j) cnt[j] = lov[j] = 0;
  const uint32_t tid = threadIdx.x;
  const uint64_t i_end = (i0 + kJcTile < nl) ? i0 + kJcTile : nl;
  const uint64_t mis = (reinterpret_cast<uintptr_t>(R) >> 2) & 3u;
  const uint64_t w0 = sm.w0, w1 = sm.w1 > sm.w0 ? sm.w1 : sm.w0;
  const uint32_t staged = sm.staged;
  const uint64_t base = ((w0 + mis) & ~3ull) - mis;
  // the thread's left keys are loaded while the window's bulk copy is in flight
  const uint64_t first = i0 + static_cast<uint64_t>(tid) * kJcKeys;
  uint32_t key[kJcKeys];
  if (first + kJcKeys <= i_end && (reinterpret_cast<uintptr_t>(L + first) & 15u) == 0) {
    // two 16-byte loads (the thread's keys are consecutive)
    const uint4 a = *reinterpret_cast<const uint4*>(L + first);
    const uint4 b = *reinterpret_cast<const uint4*>(L + first + 4);
    key[0] = a.x, key[1] = a.y, key[2] = a.z, key[3] = a.w;
    key[4] = b.x, key[5] = b.y, key[6] = b.z, key[7] = b.w;
  } else if (first < i_end) {
#pragma unroll
    for (int j = 0; j < kJcKeys; ++j) {
      const uint64_t i = first + j;
      key[j] = L[i < i_end ? i : i_end - 1];
    }
  }
  static_assert(kJcKeys == 8, "the vector loads above take 8 keys");
  if (staged) {
    const uint64_t a0 = (staged == 2) ? ((w0 + mis + 3) & ~3ull) - mis : w1;
    const uint64_t a1 = (staged == 2) ? ((w1 + mis) & ~3ull) - mis : w1;
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
  if (first >= i_end) return;   // counts stay zero

  if (!use_smem) {
    uint32_t lo[kJcKeys], hi[kJcKeys];
    lockstep_bounds32<kJcKeys>(R, static_cast<uint32_t>(w0), static_cast<uint32_t>(w1), key, lo, hi);
#pragma unroll
    for (int j = 0; j < kJcKeys; ++j) {
      const uint64_t i = first + j;
      if (i < i_end) {
        lov[j] = static_cast<uint32_t>(lo[j]);
        cnt[j] = static_cast<uint32_t>(hi[j] - lo[j]);
      }
    }
    return;
  }
  // staged window: the thread's first key is searched in full, the others
  // gallop from the previous key's upper bound; equal keys reuse its bounds
  const uint32_t* win = sm.keys + (w0 - base);
  const uint32_t n = static_cast<uint32_t>(w1 - w0);
  uint32_t plo = 0, phi = 0, pkey = 0;
#pragma unroll
  for (int j = 0; j < kJcKeys; ++j) {
    const uint64_t i = first + j;
    if (i < i_end) {
      const uint32_t k = key[j];
      uint32_t lo, hi;
      if (j > 0 && k == pkey) {
        lo = plo;
        hi = phi;
      } else {
        lo = (j == 0) ? smem_search<false>(win, 0, n, k) : smem_gallop<false>(win, phi, n, k);
        hi = smem_gallop<true>(win, lo, n, k);
      }
      lov[j] = static_cast<uint32_t>(w0 + lo);
      cnt[j] = hi - lo;
      plo = lo;
      phi = hi;
      pkey = k;
    }
  }
}

// A tile's lower bounds and output offsets, staged in the window's shared
// memory after the search so that they leave in coalesced stores: element e
// of the tile (thread e / 8's key e % 8) sits at e + e / 32 (lower bounds,
// 32-bit) and at e + e / 16 of the 64-bit area (offsets), which keeps both
// the per-thread writes and the row-order reads free of bank conflicts.
constexpr uint32_t kJcStageLoWords = kJcTile + kJcTile / 32;
__device__ __forceinline__ uint32_t* jc_stage_lo(JoinCountSmem& sm) { return sm.keys; }
__device__ __forceinline__ uint64_t* jc_stage_off(JoinCountSmem& sm) {
  return reinterpret_cast<uint64_t*>(sm.keys + kJcStageLoWords);
}
static_assert(kJcStageLoWords % 2 == 0, "the 64-bit staging area starts 8-byte aligned");
static_assert(kJcStageLoWords + 2 * (kJcTile + kJcTile / 16) <= kJcWindow, "staging fits in the window");

// Called by one thread after the block's last use of the window: a bulk copy
// whose wait gave up may still be in flight into this block's shared memory,
// and must land before the block exits (bounded again; a copy that still has
// not landed is recorded as one more timeout).
__device__ __forceinline__ void jc_drain_window(JoinCountSmem& sm, DeviceErrors* err) {
  if (sm.staged == 2 && sm.failed) (void)mbar_wait_bounded(&sm.bar, 0, err);
}

// The tile's window: lower bound of its first key and upper bound of its
// last key in R, found by one warp each (every lane of the warp calls it).
__device__ __forceinline__ uint64_t jc_window_bound(const uint32_t* __restrict__ L, uint64_t nl,
                                                    const uint32_t* __restrict__ R, uint64_t nr, uint64_t i0,
                                                    bool upper) {
  const uint64_t i_end = (i0 + kJcTile < nl) ? i0 + kJcTile : nl;
  return upper ? warp_bound<true, uint32_t>(R, 0, nr, L[i_end - 1]) : warp_bound<false, uint32_t>(R, 0, nr, L[i0]);
}

// jc_count_staged with the window found by the block itself: two warps
// search R at once, then thread 0 stages the window.
__device__ __forceinline__ void join_count_tile_regs(const uint32_t* __restrict__ L, uint64_t nl,
                                                     const uint32_t* __restrict__ R, uint64_t nr, uint64_t i0,
                                                     uint32_t* __restrict__ lo_out, uint32_t (&cnt)[kJcKeys],
                                                     JoinCountSmem& sm, DeviceErrors* err) {
  const uint32_t tid = threadIdx.x;
  if (tid < 64) {
    const uint64_t w = jc_window_bound(L, nl, R, nr, i0, tid >= 32);
    if (tid == 0) sm.w0 = w;
    if (tid == 32) sm.w1 = w;
  }
  __syncthreads();
  if (tid == 0) jc_issue_window(R, sm.w0, sm.w1, sm);
  __syncthreads();
  uint32_t lov[kJcKeys];
  jc_count_staged(L, nl, R, i0, lov, cnt, sm, err);
  const uint64_t first = i0 + static_cast<uint64_t>(tid) * kJcKeys;
#pragma unroll
  for (int j = 0; j < kJcKeys; ++j)
    if (first + j < nl) lo_out[first + j] = lov[j];
}

// Lower bound and match count of every left key of the tile, to lo_out and
// cnt_out.
__device__ __forceinline__ void join_count_tile(const uint32_t* __restrict__ L, uint64_t nl,
                                                const uint32_t* __restrict__ R, uint64_t nr, uint64_t i0,
                                                uint32_t* __restrict__ lo_out, uint32_t* __restrict__ cnt_out,
                                                JoinCountSmem& sm, DeviceErrors* err) {
  uint32_t cnt[kJcKeys];
  join_count_tile_regs(L, nl, R, nr, i0, lo_out, cnt, sm, err);
  const uint64_t first = i0 + static_cast<uint64_t>(threadIdx.x) * kJcKeys;
  const uint64_t i_end = (i0 + kJcTile < nl) ? i0 + kJcTile : nl;
#pragma unroll
  for (int j = 0; j < kJcKeys; ++j)
    if (first + j < i_end) cnt_out[first + j] = cnt[j];
}

}  // namespace vg
