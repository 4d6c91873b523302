// Block-level building blocks: warp/block scans and single-pass decoupled
// look-back across tiles (bounded spin-waits).
#pragma once

#include "vg_common.cuh"

namespace vg {

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, d);
    if (lane_id() >= static_cast<uint32_t>(d)) v += t;
  }
  return v;
}

__device__ __forceinline__ uint64_t warp_incl_scan64(uint64_t v) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint64_t t = __shfl_up_sync(0xffffffffu, v, d);
    if (lane_id() >= static_cast<uint32_t>(d)) v += t;
  }
  return v;
}

__device__ __forceinline__ uint64_t warp_sum64(uint64_t v) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
  return v;
}

// Exclusive scan of one value per thread over a BLOCK-thread block.
// s_warp: BLOCK/32 words of shared memory.  Contains __syncthreads().
template <int BLOCK>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t& total, uint32_t* s_warp) {
  constexpr int W = BLOCK / 32;
  uint32_t incl = warp_incl_scan(v);
  uint32_t w = threadIdx.x >> 5;
  if (lane_id() == 31) s_warp[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t x = lane_id() < W ? s_warp[lane_id()] : 0u;
    uint32_t xi = warp_incl_scan(x);
    if (lane_id() < W) s_warp[lane_id()] = xi - x;
    if (lane_id() == W - 1) s_warp[W] = xi;
  }
  __syncthreads();
  uint32_t res = s_warp[w] + incl - v;
  total = s_warp[W];
  __syncthreads();
  return res;
}

// 64-bit variant; s_warp: BLOCK/32 + 1 words.
template <int BLOCK>
__device__ __forceinline__ uint64_t block_excl_scan64(uint64_t v, uint64_t& total, uint64_t* s_warp) {
  constexpr int W = BLOCK / 32;
  uint64_t incl = warp_incl_scan64(v);
  uint32_t w = threadIdx.x >> 5;
  if (lane_id() == 31) s_warp[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint64_t x = lane_id() < W ? s_warp[lane_id()] : 0ull;
    uint64_t xi = warp_incl_scan64(x);
    if (lane_id() < W) s_warp[lane_id()] = xi - x;
    if (lane_id() == W - 1) s_warp[W] = xi;
  }
  __syncthreads();
  uint64_t res = s_warp[w] + incl - v;
  total = s_warp[W];
  __syncthreads();
  return res;
}

// Polls a look-back status word until a predecessor has published it.
// Gives up after kSpinLimit polls: records the timeout and returns an
// inclusive zero so that every waiter still terminates.
__device__ __forceinline__ uint64_t wait_status(const uint64_t* p, DeviceErrors* err) {
  uint64_t s = ld_status_u64(p);
  uint32_t spins = 0;
  while ((s & ~kValueMask) == 0) {
    if (++spins > kSpinLimit) {
      atomicExch(&err->timeout, 1u);
      return kFlagInc;
    }
    __nanosleep(32);
    s = ld_status_u64(p);
  }
  return s;
}

// Decoupled look-back (single counter per tile): publishes this tile's total
// and returns the exclusive prefix of all earlier tiles.  Executed by one full
// warp; `status` must be zero before the launch.
__device__ __forceinline__ uint64_t warp_lookback(uint64_t* status, uint32_t tile, uint64_t tile_total,
                                                  DeviceErrors* err) {
  const uint32_t lane = lane_id();
  if (lane == 0) st_status_u64(&status[tile], (tile == 0 ? kFlagInc : kFlagAgg) | tile_total);
  uint64_t prefix = 0;
  if (tile > 0) {
    int64_t j = static_cast<int64_t>(tile) - 1 - lane;
    while (true) {
      uint64_t s = (j >= 0) ? wait_status(&status[j], err) : kFlagInc;
      bool inc = (s & kFlagInc) != 0;
      uint32_t inc_mask = __ballot_sync(0xffffffffu, inc);
      uint64_t v = s & kValueMask;
      if (inc_mask) {
        uint32_t lim = __ffs(inc_mask) - 1;
        prefix += warp_sum64(lane <= lim ? v : 0);
        break;
      }
      prefix += warp_sum64(v);
      j -= 32;
    }
    if (lane == 0) st_status_u64(&status[tile], kFlagInc | (prefix + tile_total));
  }
  return prefix;
}

// Segmented variant: tiles [first_tile, tile) of one segment only; the
// segment's first tile starts a new chain.
__device__ __forceinline__ uint64_t warp_lookback_seg(uint64_t* status, uint64_t tile, uint64_t first_tile,
                                                      uint64_t tile_total, DeviceErrors* err) {
  const uint32_t lane = lane_id();
  const bool head = tile == first_tile;
  if (lane == 0) st_status_u64(&status[tile], (head ? kFlagInc : kFlagAgg) | tile_total);
  uint64_t prefix = 0;
  if (!head) {
    int64_t j = static_cast<int64_t>(tile) - 1 - lane;
    while (true) {
      uint64_t s = (j >= static_cast<int64_t>(first_tile)) ? wait_status(&status[j], err) : kFlagInc;
      bool inc = (s & kFlagInc) != 0;
      uint32_t inc_mask = __ballot_sync(0xffffffffu, inc);
      uint64_t v = s & kValueMask;
      if (inc_mask) {
        uint32_t lim = __ffs(inc_mask) - 1;
        prefix += warp_sum64(lane <= lim ? v : 0);
        break;
      }
      prefix += warp_sum64(v);
      j -= 32;
    }
    if (lane == 0) st_status_u64(&status[tile], kFlagInc | (prefix + tile_total));
  }
  return prefix;
}

// Whole-block wrapper: warp 0 looks back, the prefix is broadcast.
__device__ __forceinline__ uint64_t block_lookback(uint64_t* status, uint32_t tile, uint64_t tile_total,
                                                   DeviceErrors* err, uint64_t* s_bcast) {
  if (threadIdx.x < 32) {
    uint64_t p = warp_lookback(status, tile, tile_total, err);
    if (threadIdx.x == 0) *s_bcast = p;
  }
  __syncthreads();
  uint64_t r = *s_bcast;
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// Bulk (TMA) global->shared copies completed on an mbarrier.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// One bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of an mbarrier; false (and a recorded
// timeout) when it did not complete.
// Non-blocking test of phase `parity`.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Polls with non-blocking tests and short sleeps, so the bound is in time
// (about kSpinLimit x 64 ns) and not in hardware suspend periods.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, DeviceErrors* err) {
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    if (mbar_test_wait(bar, parity)) return true;
    __nanosleep(64);
  }
  atomicExch(&err->timeout, 1u);
  return false;
}

// Adjacent-unique building blocks (a thread owns 8 consecutive rows r0..r0+7,
// r0 a multiple of 8).  unique_diff_bits: bit i set when row r0 + i (< n)
// differs from the row before it in column `col` (row 0 is left to the
// caller); a 16-byte aligned column is read with two 16-byte loads.
__device__ __forceinline__ uint32_t unique_diff_bits(const uint32_t* __restrict__ col, uint64_t n, uint64_t r0) {
  uint32_t v[8];
  if ((reinterpret_cast<uintptr_t>(col) & 15u) == 0 && r0 + 8 <= n) {
    const uint4 a = *reinterpret_cast<const uint4*>(col + r0);
    const uint4 b = *reinterpret_cast<const uint4*>(col + r0 + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = (r0 + i < n) ? col[r0 + i] : 0u;
  }
  uint32_t prev = (r0 > 0 && r0 - 1 < n) ? col[r0 - 1] : 0u;
  uint32_t d = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint64_t r = r0 + i;
    if (r < n && r > 0 && v[i] != prev) d |= 1u << i;
    prev = v[i];
  }
  return d;
}

// Row copies between column sets.  Every value of the row is loaded before
// any is stored, through the read-only path (the source columns are never
// written while a kernel copies from them): the loads of a row are in flight
// together, where a load after each store would wait for that store (the
// compiler cannot tell the column pointers apart).
// out[c][dst] = in[c][src] for c < ncols.
__device__ __forceinline__ void copy_row(uint32_t* const* out, const uint32_t* const* in, uint32_t ncols,
                                         uint64_t src, uint64_t dst) {
  uint32_t v[VG_MAX_COLS];
#pragma unroll
  for (int c = 0; c < VG_MAX_COLS; ++c)
    if (c < static_cast<int>(ncols)) v[c] = __ldg(in[c] + src);
#pragma unroll
  for (int c = 0; c < VG_MAX_COLS; ++c)
    if (c < static_cast<int>(ncols)) out[c][dst] = v[c];
}

// A join output row: out[c][k] = lc[c][a] for c < nlc, then
// out[nlc + x][k] = rc[x][b] for x < nrc.
__device__ __forceinline__ void copy_join_row(uint32_t* const* out, const uint32_t* const* lc, uint32_t nlc,
                                              const uint32_t* const* rc, uint32_t nrc, uint64_t a, uint64_t b,
                                              uint64_t k) {
  uint32_t v[VG_MAX_COLS];
  const int ncols = static_cast<int>(nlc + nrc);
#pragma unroll
  for (int c = 0; c < VG_MAX_COLS; ++c)
    if (c < ncols) v[c] = c < static_cast<int>(nlc) ? __ldg(lc[c] + a) : __ldg(rc[c - nlc] + b);
#pragma unroll
  for (int c = 0; c < VG_MAX_COLS; ++c)
    if (c < ncols) out[c][k] = v[c];
}

// compact_store: the kept rows of a tile (bit i of `keep` for row r0 + i,
// the thread's first kept row at tile position e, the tile's first at output
// row g) written by each warp on its own: a warp's kept rows are one
// contiguous run of the output, so the warp stages two columns at a time in
// its own slice of shared memory (s_buf: 2 * BLOCK * 8 words, 512 words per
// warp) and stores the run with coalesced stores, between warp barriers only.
// Every thread of the block calls it (no block barrier inside).
template <int BLOCK>
__device__ __forceinline__ void compact_store(const uint32_t* const* in, uint32_t* const* out, uint32_t ncols,
                                              uint64_t n, uint64_t r0, uint32_t keep, uint32_t e, uint32_t tot,
                                              uint64_t g, uint32_t* s_buf) {
  (void)tot;
  constexpr uint32_t kSlice = 32 * 8;   // one column of a warp's rows
  const uint32_t lane = lane_id();
  uint32_t mine = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i)
    if ((keep >> i & 1u) && r0 + i < n) ++mine;
  const uint32_t w0 = __shfl_sync(0xffffffffu, e, 0);                 // the warp's first kept row in the tile
  const uint32_t wtot = __shfl_sync(0xffffffffu, e + mine, 31) - w0;  // the warp's kept rows
  uint32_t* sw = s_buf + (threadIdx.x >> 5) * 2 * kSlice;
  const uint64_t dst0 = g + w0;
  for (uint32_t c = 0; c < ncols; c += 2) {
    const bool two = c + 1 < ncols;
    const uint32_t* col_a = in[c];
    const uint32_t* col_b = two ? in[c + 1] : nullptr;
    uint32_t o = e - w0;
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if ((keep >> i & 1u) && r0 + i < n) {
        sw[o] = __ldg(col_a + r0 + i);
        if (two) sw[kSlice + o] = __ldg(col_b + r0 + i);
        ++o;
      }
    __syncwarp();
    uint32_t* dst_a = out[c] + dst0;
    for (uint32_t k = lane; k < wtot; k += 32) dst_a[k] = sw[k];
    if (two) {
      uint32_t* dst_b = out[c + 1] + dst0;
      for (uint32_t k = lane; k < wtot; k += 32) dst_b[k] = sw[kSlice + k];
    }
    __syncwarp();
  }
}

// Branch-free lower/upper bound over a sorted device array.
template <typename T, typename V>
__device__ __forceinline__ uint64_t lower_bound_dev(const T* a, uint64_t lo, uint64_t hi, V key) {
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
template <typename T, typename V>
__device__ __forceinline__ uint64_t upper_bound_dev(const T* a, uint64_t lo, uint64_t hi, V key) {
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (key < a[mid]) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// Four source elements starting at s, read as aligned 16-byte vectors: the
// vector holding s and, when s is not 16-byte aligned, the next one.  Only
// called where both vectors lie inside the piece.
__device__ __forceinline__ uint4 load4_realigned(const uint32_t* s) {
  const uint32_t sh = static_cast<uint32_t>(reinterpret_cast<uintptr_t>(s) >> 2) & 3u;
  const uint4* a = reinterpret_cast<const uint4*>(s - sh);
  const uint4 x = __ldg(a);
  if (sh == 0) return x;
  const uint4 y = __ldg(a + 1);
  uint4 v;
  if (sh == 1) v = make_uint4(x.y, x.z, x.w, y.x);
  else if (sh == 2) v = make_uint4(x.z, x.w, y.x, y.y);
  else v = make_uint4(x.w, y.x, y.y, y.z);
  return v;
}

}  // namespace vg
