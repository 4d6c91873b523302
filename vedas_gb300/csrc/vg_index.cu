// Permutation-index construction (hot path a).
//
// For each permutation (k0, k1, k2) of (s, p, o) the three uint32 columns are
// packed into one 64-bit key (k0 | k1 | k2 at their measured bit widths),
// radix-sorted, and a single fused pass unpacks the sorted keys into the data
// columns and run-length encodes the level-1 (k0) and level-2 (k0, k1)
// boundaries into (value, first row) arrays -- the reduce_by_key + exclusive
// scan pair of the reference -- with a decoupled look-back for the output
// positions.
#include "vg_index.h"

#include <algorithm>

#include "vg_prims.cuh"
#include "vg_sort.h"

namespace vg {
namespace {

constexpr int kBlock = 256;
constexpr int kRows = 8;                 // rows per thread (blocked)
constexpr int kTileRows = kBlock * kRows;
static_assert(kRows % 4 == 0, "unpack_rle_kernel moves a thread's rows in 16-byte pieces");

__global__ void max3_kernel(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                            const uint32_t* __restrict__ c, uint64_t n, uint32_t* out3) {
  uint32_t ma = 0, mb = 0, mc = 0;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    ma = max(ma, a[i]);
    mb = max(mb, b[i]);
    mc = max(mc, c[i]);
  }
  for (int d = 16; d > 0; d >>= 1) {
    ma = max(ma, __shfl_xor_sync(0xffffffffu, ma, d));
    mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, d));
    mc = max(mc, __shfl_xor_sync(0xffffffffu, mc, d));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out3[0], ma);
    atomicMax(&out3[1], mb);
    atomicMax(&out3[2], mc);
  }
}

__global__ void pack_kernel(const uint32_t* __restrict__ k0, const uint32_t* __restrict__ k1,
                            const uint32_t* __restrict__ k2, uint64_t n, uint32_t sh0, uint32_t sh1,
                            uint64_t* __restrict__ keys) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    keys[i] = (static_cast<uint64_t>(k0[i]) << sh0) | (static_cast<uint64_t>(k1[i]) << sh1) |
              static_cast<uint64_t>(k2[i]);
}

struct UnpackArgs {
  const uint64_t* keys;
  uint64_t n;
  uint32_t sh0, sh1;       // k0 = key >> sh0, k1 = (key >> sh1) & m1, k2 = key & m2
  uint64_t m1, m2;
  uint32_t* col1;          // k1 per row (nullable)
  uint32_t* col2;          // k2 per row (nullable)
  uint32_t* l1_vals;       // level-1 run values (k0) (nullable)
  uint32_t* l1_offs;
  uint32_t* l2_vals;       // level-2 run values (k1) (nullable)
  uint32_t* l2_offs;
  uint64_t* status1;
  uint64_t* status2;
  uint32_t* ticket;
  uint64_t* counts;        // [0] level-1 runs, [1] level-2 runs
  uint64_t tiles;
  DeviceErrors* err;
};

__global__ void __launch_bounds__(kBlock) unpack_rle_kernel(UnpackArgs a) {
  __shared__ uint32_t s_scan[kBlock / 32 + 1];
  __shared__ uint64_t s_b;
  __shared__ uint32_t s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(a.ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint64_t r0 = static_cast<uint64_t>(tile) * kTileRows + threadIdx.x * kRows;

  uint64_t key[kRows];
  if (r0 + kRows <= a.n) {
    // the thread's rows are consecutive and 64-byte aligned (r0 is a multiple
    // of kRows, the keys an arena block): 16-byte loads
#pragma unroll
    for (int i = 0; i < kRows; i += 2) {
      const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(a.keys + r0 + i);
      key[i] = v.x;
      key[i + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < kRows; ++i) key[i] = (r0 + i < a.n) ? a.keys[r0 + i] : 0ull;
  }
  uint64_t prev = (r0 > 0 && r0 - 1 < a.n) ? a.keys[r0 - 1] : 0ull;
  uint32_t f1 = 0, f2 = 0;
#pragma unroll
  for (int i = 0; i < kRows; ++i) {
    const uint64_t r = r0 + i;
    if (r < a.n) {
      const uint64_t pv = (i == 0) ? prev : key[i - 1];
      if (r == 0 || (key[i] >> a.sh0) != (pv >> a.sh0)) f1 |= 1u << i;
      if (r == 0 || (key[i] >> a.sh1) != (pv >> a.sh1)) f2 |= 1u << i;
    }
  }
  // both levels' run counts in one scan (a tile has at most kTileRows < 2^16
  // of each) and, when the row count allows, one look-back over both
  // (level 1 above bit 31, level 2 below)
  uint32_t tt;
  const uint32_t ee = block_excl_scan<kBlock>((__popc(f1) << 16) | __popc(f2), tt, s_scan);
  const uint32_t e1 = ee >> 16, e2 = ee & 0xFFFFu, t1 = tt >> 16, t2 = tt & 0xFFFFu;
  uint64_t g1 = 0, g2 = 0;
  if (a.l1_vals && a.l2_vals && a.n < (1ull << 31)) {
    const uint64_t g = block_lookback(a.status1, tile, (static_cast<uint64_t>(t1) << 31) | t2, a.err, &s_b);
    g1 = g >> 31;
    g2 = g & ((1ull << 31) - 1);
  } else {
    g1 = a.l1_vals ? block_lookback(a.status1, tile, t1, a.err, &s_b) : 0;
    g2 = a.l2_vals ? block_lookback(a.status2, tile, t2, a.err, &s_b) : 0;
  }
  static_assert(kTileRows < (1 << 16), "a tile's run counts fit 16 bits each");
  if (tile == a.tiles - 1 && threadIdx.x == 0) {
    a.counts[0] = g1 + t1;
    a.counts[1] = g2 + t2;
  }
  if (r0 + kRows <= a.n) {
    // the columns' words of the thread's rows: 16-byte stores (32-byte aligned)
    uint32_t w1[kRows], w2[kRows];
#pragma unroll
    for (int i = 0; i < kRows; ++i) {
      w1[i] = static_cast<uint32_t>((key[i] >> a.sh1) & a.m1);
      w2[i] = static_cast<uint32_t>(key[i] & a.m2);
    }
#pragma unroll
    for (int i = 0; i < kRows; i += 4) {
      if (a.col1) *reinterpret_cast<uint4*>(a.col1 + r0 + i) = make_uint4(w1[i], w1[i + 1], w1[i + 2], w1[i + 3]);
      if (a.col2) *reinterpret_cast<uint4*>(a.col2 + r0 + i) = make_uint4(w2[i], w2[i + 1], w2[i + 2], w2[i + 3]);
    }
  } else {
#pragma unroll
    for (int i = 0; i < kRows; ++i) {
      const uint64_t r = r0 + i;
      if (r >= a.n) break;
      if (a.col1) a.col1[r] = static_cast<uint32_t>((key[i] >> a.sh1) & a.m1);
      if (a.col2) a.col2[r] = static_cast<uint32_t>(key[i] & a.m2);
    }
  }
  uint32_t c1 = 0, c2 = 0;
#pragma unroll
  for (int i = 0; i < kRows; ++i) {
    const uint64_t r = r0 + i;
    if (r >= a.n) break;
    const uint32_t v0 = static_cast<uint32_t>(key[i] >> a.sh0);
    const uint32_t v1 = static_cast<uint32_t>((key[i] >> a.sh1) & a.m1);
    if (a.l1_vals && (f1 >> i & 1u)) {
      const uint64_t o = g1 + e1 + c1++;
      a.l1_vals[o] = v0;
      a.l1_offs[o] = static_cast<uint32_t>(r);
    }
    if (a.l2_vals && (f2 >> i & 1u)) {
      const uint64_t o = g2 + e2 + c2++;
      a.l2_vals[o] = v1;
      a.l2_offs[o] = static_cast<uint32_t>(r);
    }
  }
}

// (k0, k1, k2) keys packed at widths (b0, b1, b2) repacked as (k0, k2, k1).
__global__ void repack_swap12_kernel(const uint64_t* __restrict__ in, uint64_t* __restrict__ out, uint64_t n,
                                     uint32_t b1, uint32_t b2) {
  const uint64_t m1 = (1ull << b1) - 1, m2 = (1ull << b2) - 1;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t k = in[i];
    const uint64_t k2 = k & m2, k1 = (k >> b2) & m1, k0 = k >> (b1 + b2);
    out[i] = (k0 << (b1 + b2)) | (k2 << b1) | k1;
  }
}

int bits_for(uint32_t maxv) { return maxv == 0 ? 1 : 32 - __builtin_clz(maxv); }

unsigned grid_for(const Ctx& ctx, uint64_t n, int per_thread) {
  uint64_t g = div_up(n, static_cast<uint64_t>(kBlock) * per_thread);
  const uint64_t gmax = static_cast<uint64_t>(ctx.num_sms) * 16;
  if (g > gmax) g = gmax;
  return static_cast<unsigned>(g < 1 ? 1 : g);
}

}  // namespace

void column_max3(Ctx& ctx, const uint32_t* a, const uint32_t* b, const uint32_t* c, uint64_t n,
                 uint32_t out[3]) {
  Scratch<uint32_t> d(ctx, 3);
  VG_CUDA(cudaMemsetAsync(d.get(), 0, 3 * sizeof(uint32_t), ctx.stream));
  if (n) {
    ctx.launch("column_max", 12.0 * n,
               [&] { max3_kernel<<<grid_for(ctx, n, 8), kBlock, 0, ctx.stream>>>(a, b, c, n, d.get()); });
    VG_CUDA(cudaGetLastError());
  }
  VG_CUDA(cudaMemcpyAsync(out, d.get(), 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
}

namespace {

// Run-length encodes and unpacks sorted packed keys (widths b0, b1, b2) into
// the requested outputs.
void unpack_outputs(Ctx& ctx, const uint64_t* sorted, uint64_t n, int b0, int b1, int b2, PermOutputs& out) {
  (void)b0;
  const uint32_t sh1 = static_cast<uint32_t>(b2), sh0 = static_cast<uint32_t>(b1 + b2);
  UnpackArgs a{};
  a.keys = sorted;
  a.n = n;
  a.sh0 = sh0;
  a.sh1 = sh1;
  a.m1 = (b1 >= 64) ? ~0ull : ((1ull << b1) - 1);
  a.m2 = (b2 >= 64) ? ~0ull : ((1ull << b2) - 1);
  a.col1 = out.want_col1 ? ctx.alloc<uint32_t>(n) : nullptr;
  a.col2 = out.want_col2 ? ctx.alloc<uint32_t>(n) : nullptr;
  a.l1_vals = out.want_l1 ? ctx.alloc<uint32_t>(n) : nullptr;
  a.l1_offs = out.want_l1 ? ctx.alloc<uint32_t>(n) : nullptr;
  a.l2_vals = out.want_l2 ? ctx.alloc<uint32_t>(n) : nullptr;
  a.l2_offs = out.want_l2 ? ctx.alloc<uint32_t>(n) : nullptr;
  a.tiles = div_up(n, kTileRows);
  Scratch<uint64_t> st1(ctx, a.tiles), st2(ctx, a.tiles), counts(ctx, 2);
  Scratch<uint32_t> ticket(ctx, 1);
  VG_CUDA(cudaMemsetAsync(st1.get(), 0, a.tiles * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(st2.get(), 0, a.tiles * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(counts.get(), 0, 2 * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(uint32_t), ctx.stream));
  a.status1 = st1.get();
  a.status2 = st2.get();
  a.ticket = ticket.get();
  a.counts = counts.get();
  a.err = ctx.d_err;
  const double ub = 8.0 * n + 4.0 * n * ((a.col1 ? 1 : 0) + (a.col2 ? 1 : 0));
  ctx.launch("index_unpack_rle", ub,
             [&] { unpack_rle_kernel<<<static_cast<unsigned>(a.tiles), kBlock, 0, ctx.stream>>>(a); });
  VG_CUDA(cudaGetLastError());
  uint64_t hc[2];
  VG_CUDA(cudaMemcpyAsync(hc, counts.get(), sizeof(hc), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  ctx.check_device_errors();
  out.col1 = DevArray(a.col1, a.col1 ? n : 0);
  out.col2 = DevArray(a.col2, a.col2 ? n : 0);
  if (a.l1_vals) {
    ctx.arena.shrink(a.l1_vals, hc[0] * 4);
    ctx.arena.shrink(a.l1_offs, hc[0] * 4);
    out.l1_vals = DevArray(a.l1_vals, hc[0]);
    out.l1_offs = DevArray(a.l1_offs, hc[0]);
  }
  if (a.l2_vals) {
    ctx.arena.shrink(a.l2_vals, hc[1] * 4);
    ctx.arena.shrink(a.l2_offs, hc[1] * 4);
    out.l2_vals = DevArray(a.l2_vals, hc[1]);
    out.l2_offs = DevArray(a.l2_offs, hc[1]);
  }
}

// Packs (k0, k1, k2) at widths (b0, b1, b2) and sorts the keys; returns the
// sorted array (the caller frees it).
uint64_t* sort_packed(Ctx& ctx, const uint32_t* k0, const uint32_t* k1, const uint32_t* k2, uint64_t n, int b0,
                      int b1, int b2) {
  const uint32_t sh1 = static_cast<uint32_t>(b2), sh0 = static_cast<uint32_t>(b1 + b2);
  uint64_t* keys = ctx.alloc<uint64_t>(n);
  uint64_t* keys_alt = ctx.alloc<uint64_t>(n);
  ctx.launch("index_pack", 20.0 * n,
             [&] { pack_kernel<<<grid_for(ctx, n, 8), kBlock, 0, ctx.stream>>>(k0, k1, k2, n, sh0, sh1, keys); });
  VG_CUDA(cudaGetLastError());
  const bool alt = radix_sort_u64(ctx, keys, keys_alt, nullptr, nullptr, n, b0 + b1 + b2, false);
  ctx.free(alt ? keys : keys_alt);
  return alt ? keys_alt : keys;
}

}  // namespace

void build_permutation(Ctx& ctx, const uint32_t* k0, const uint32_t* k1, const uint32_t* k2,
                       uint64_t n, const uint32_t maxes[3], PermOutputs& out) {
  const int b0 = bits_for(maxes[0]), b1 = bits_for(maxes[1]), b2 = bits_for(maxes[2]);
  if (b0 + b1 + b2 > 64)
    fail(VG_ERR_UNSUPPORTED, "triple ids need more than 64 key bits for the packed index sort");
  out.col1.clear();
  out.col2.clear();
  if (n == 0) return;
  uint64_t* sorted = sort_packed(ctx, k0, k1, k2, n, b0, b1, b2);
  unpack_outputs(ctx, sorted, n, b0, b1, b2, out);
  ctx.free(sorted);
}

void build_permutation_pair(Ctx& ctx, const uint32_t* k0, const uint32_t* k1, const uint32_t* k2, uint64_t n,
                            const uint32_t maxes[3], PermOutputs& first, PermOutputs& second) {
  const int b0 = bits_for(maxes[0]), b1 = bits_for(maxes[1]), b2 = bits_for(maxes[2]);
  if (b0 + b1 + b2 > 64)
    fail(VG_ERR_UNSUPPORTED, "triple ids need more than 64 key bits for the packed index sort");
  first.col1.clear();
  first.col2.clear();
  second.col1.clear();
  second.col2.clear();
  if (n == 0) return;
  uint64_t* sorted = sort_packed(ctx, k0, k1, k2, n, b0, b1, b2);
  unpack_outputs(ctx, sorted, n, b0, b1, b2, first);
  // (k0, k2, k1) order from (k0, k1, k2) order: a stable sort by (k0, k2)
  // alone keeps equal (k0, k2) keys in (k0, k1, k2) order, i.e. by k1
  uint64_t* re = ctx.alloc<uint64_t>(n);
  uint64_t* re_alt = ctx.alloc<uint64_t>(n);
  ctx.launch("index_repack", 16.0 * n, [&] {
    repack_swap12_kernel<<<grid_for(ctx, n, 8), kBlock, 0, ctx.stream>>>(sorted, re, n, static_cast<uint32_t>(b1),
                                                                         static_cast<uint32_t>(b2));
  });
  VG_CUDA(cudaGetLastError());
  ctx.free(sorted);
  const bool alt = radix_sort_u64_bits(ctx, re, re_alt, n, b1, b0 + b1 + b2);
  uint64_t* s2 = alt ? re_alt : re;
  ctx.free(alt ? re : re_alt);
  unpack_outputs(ctx, s2, n, b0, b2, b1, second);
  ctx.free(s2);
}

}  // namespace vg
