// Stable LSD radix sort, onesweep style (one upfront histogram pass, then one
// pass per 8-bit digit whose tile offsets come from a decoupled look-back).
//
// A tile is 256 threads x 16 keys (or 8, a per-context tuning choice).  Keys are ranked inside each warp with
// __match_any_sync in input order, so equal digits keep their order and the
// sort is stable; tiles take their index from an atomic ticket in launch
// order, which guarantees that every look-back predecessor is running.
// Passes whose digit is the same for every key are skipped (the permutation
// would be the identity), unless the caller asks for the variant without a
// host round trip, which scans the bucket bases on the device and runs every
// pass over [0, end_bit).
#include "vg_sort.h"

#include <vector>

#include "vg_prims.cuh"

namespace vg {
namespace {

constexpr int kBlock = 256;
// Keys per thread of a onesweep tile: 16 (tiles of 4096 keys) or 8 (2048),
// chosen per context (Ctx::tune.sort_items).
constexpr int kItemsMax = 16;
constexpr int kRadix = 256;
constexpr int kMaxPasses = 8;

template <typename K>
__global__ void __launch_bounds__(kBlock) radix_hist_kernel(const K* __restrict__ keys, uint64_t n,
                                                            uint32_t passes, uint32_t begin_bit,
                                                            unsigned long long* __restrict__ hist) {
  __shared__ uint32_t sh[kMaxPasses * kRadix];
  for (uint32_t i = threadIdx.x; i < kMaxPasses * kRadix; i += kBlock) sh[i] = 0;
  __syncthreads();
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * kBlock;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * kBlock + threadIdx.x; i < n; i += stride) {
    K k = keys[i];
    for (uint32_t p = 0; p < passes; ++p)
      atomicAdd(&sh[p * kRadix + (static_cast<uint32_t>(k >> (begin_bit + 8 * p)) & 0xFFu)], 1u);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < passes * kRadix; i += kBlock)
    if (sh[i]) atomicAdd(&hist[i], static_cast<unsigned long long>(sh[i]));
}

// Exclusive scan of each pass's 256 digit counts (one block per pass).
__global__ void __launch_bounds__(kRadix) radix_bases_kernel(const unsigned long long* __restrict__ hist,
                                                              uint64_t* __restrict__ bases) {
  __shared__ uint64_t s[kRadix];
  const uint32_t p = blockIdx.x, d = threadIdx.x;
  s[d] = hist[p * kRadix + d];
  __syncthreads();
  for (uint32_t off = 1; off < kRadix; off <<= 1) {
    const uint64_t v = d >= off ? s[d - off] : 0;
    __syncthreads();
    s[d] += v;
    __syncthreads();
  }
  bases[p * kRadix + d] = s[d] - hist[p * kRadix + d];
}

__global__ void iota_kernel(uint32_t* out, uint64_t n) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = static_cast<uint32_t>(i);
}

template <typename K, bool HAS_V, bool IOTA, int kItems, int kLook>
__global__ void __launch_bounds__(kBlock, kItems <= 12 ? 4 : 3) onesweep_kernel(
    const K* __restrict__ kin, K* __restrict__ kout, const uint32_t* __restrict__ vin,
    uint32_t* __restrict__ vout, uint64_t n, uint32_t shift, const uint64_t* __restrict__ bucket_base,
    uint64_t* status, uint32_t* ticket, DeviceErrors* err) {
  constexpr int kTile = kBlock * kItems;
  extern __shared__ __align__(16) unsigned char smem[];
  K* s_keys = reinterpret_cast<K*>(smem);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(smem + kTile * sizeof(K));
  __shared__ uint32_t s_whist[8 * kRadix];
  __shared__ uint32_t s_dstart[kRadix];
  __shared__ uint64_t s_dglob[kRadix];
  __shared__ uint32_t s_scan[9];
  __shared__ uint32_t s_tile;

  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(ticket, 1u);
  for (uint32_t i = tid; i < 8 * kRadix; i += kBlock) s_whist[i] = 0;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint64_t base = static_cast<uint64_t>(tile) * kTile;
  const uint64_t wbase = base + warp * (32u * kItems);

  K key[kItems];
  uint32_t val[kItems];
  uint32_t rank[kItems];
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    const uint64_t idx = wbase + i * 32u + lane;
    const bool ok = idx < n;
    key[i] = ok ? kin[idx] : K(0);
    if (HAS_V) val[i] = IOTA ? static_cast<uint32_t>(idx) : (ok ? vin[idx] : 0u);
  }
  // Rank every key among the equal digits before it in this warp's chunk.
  uint32_t* wh = s_whist + warp * kRadix;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    const bool ok = wbase + i * 32u + lane < n;
    const uint32_t d = static_cast<uint32_t>(key[i] >> shift) & 0xFFu;
    const uint32_t peers = __match_any_sync(0xffffffffu, ok ? d : 0x100u);
    uint32_t prior = 0;
    if (ok) prior = wh[d];
    __syncwarp();
    rank[i] = prior + __popc(peers & lanemask_lt());
    if (ok && lane == static_cast<uint32_t>(__ffs(peers) - 1)) wh[d] = prior + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Thread d owns digit d: per-warp exclusive offsets and the tile count.
  const uint32_t d = tid;
  uint32_t run = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    uint32_t c = s_whist[w * kRadix + d];
    s_whist[w * kRadix + d] = run;
    run += c;
  }
  // Decoupled look-back for digit d over earlier tiles ([tile][digit] layout):
  // kLook earlier tiles' words are loaded at once, then summed in order until
  // one holds an inclusive prefix (a word not yet published is waited for).
  uint64_t prefix = 0;
  uint64_t* my = status + static_cast<uint64_t>(tile) * kRadix + d;
  if (tile == 0) {
    st_status_u64(my, kFlagInc | run);
  } else {
    st_status_u64(my, kFlagAgg | run);
    int64_t j = static_cast<int64_t>(tile) - 1;
    bool found = false;
    while (!found) {
      uint64_t w[kLook];
#pragma unroll
      for (int q = 0; q < kLook; ++q)
        w[q] = (j - q >= 0) ? ld_status_u64(status + static_cast<uint64_t>(j - q) * kRadix + d) : kFlagInc;
#pragma unroll
      for (int q = 0; q < kLook; ++q) {
        if (found) break;
        uint64_t v = w[q];
        if ((v & ~kValueMask) == 0) v = wait_status(status + static_cast<uint64_t>(j - q) * kRadix + d, err);
        prefix += v & kValueMask;
        found = (v & kFlagInc) != 0;
      }
      j -= kLook;
    }
    st_status_u64(my, kFlagInc | (prefix + run));
  }
  uint32_t tot;
  const uint32_t excl = block_excl_scan<kBlock>(run, tot, s_scan);
  s_dstart[d] = excl;
  s_dglob[d] = bucket_base[d] + prefix - excl;
  __syncthreads();

  // Local scatter into digit order, then a mostly-coalesced global write.
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    if (wbase + i * 32u + lane < n) {
      const uint32_t dd = static_cast<uint32_t>(key[i] >> shift) & 0xFFu;
      const uint32_t pos = s_dstart[dd] + wh[dd] + rank[i];
      s_keys[pos] = key[i];
      if (HAS_V) s_vals[pos] = val[i];
    }
  }
  __syncthreads();
  const uint32_t tile_n = static_cast<uint32_t>(n - base < kTile ? n - base : kTile);
  for (uint32_t p = tid; p < tile_n; p += kBlock) {
    const K k = s_keys[p];
    const uint32_t dd = static_cast<uint32_t>(k >> shift) & 0xFFu;
    const uint64_t o = s_dglob[dd] + p;
    kout[o] = k;
    if (HAS_V) vout[o] = s_vals[p];
  }
}

template <typename K, bool HAS_V, bool IOTA, int kItems, int kLook>
void launch_pass_items(Ctx& ctx, const K* kin, K* kout, const uint32_t* vin, uint32_t* vout, uint64_t n,
                       uint32_t shift, const uint64_t* bases, uint64_t* status, uint32_t* ticket) {
  constexpr int kTile = kBlock * kItems;
  const size_t smem = kTile * sizeof(K) + (HAS_V ? kTile * sizeof(uint32_t) : 0);
  // once per instantiation (thread-safe static initialisation)
  static const bool attr_set = [smem] {
    VG_CUDA(cudaFuncSetAttribute(onesweep_kernel<K, HAS_V, IOTA, kItems, kLook>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    // all of the unified L1/shared storage as shared memory: three or more
    // blocks of a tile's keys (and values) per SM
    VG_CUDA(cudaFuncSetAttribute(onesweep_kernel<K, HAS_V, IOTA, kItems, kLook>,
                                 cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
    return true;
  }();
  (void)attr_set;
  const uint64_t tiles = div_up(n, kTile);
  const double bytes = static_cast<double>(n) * (2 * sizeof(K) + (HAS_V ? (IOTA ? 4 : 8) : 0));
  ctx.launch("radix_onesweep", bytes, [&] {
    onesweep_kernel<K, HAS_V, IOTA, kItems, kLook><<<static_cast<unsigned>(tiles), kBlock, smem, ctx.stream>>>(
        kin, kout, vin, vout, n, shift, bases, status, ticket, ctx.d_err);
  });
  VG_CUDA(cudaGetLastError());
}

template <typename K, bool HAS_V, bool IOTA>
void launch_pass(Ctx& ctx, int items, const K* kin, K* kout, const uint32_t* vin, uint32_t* vout, uint64_t n,
                 uint32_t shift, const uint64_t* bases, uint64_t* status, uint32_t* ticket) {
  const bool look4 = ctx.tune.sort_lookback == 4;
  if (items == 12) {
    if (look4) launch_pass_items<K, HAS_V, IOTA, 12, 4>(ctx, kin, kout, vin, vout, n, shift, bases, status, ticket);
    else launch_pass_items<K, HAS_V, IOTA, 12, 1>(ctx, kin, kout, vin, vout, n, shift, bases, status, ticket);
  } else if (items == 8) {
    if (look4) launch_pass_items<K, HAS_V, IOTA, 8, 4>(ctx, kin, kout, vin, vout, n, shift, bases, status, ticket);
    else launch_pass_items<K, HAS_V, IOTA, 8, 1>(ctx, kin, kout, vin, vout, n, shift, bases, status, ticket);
  } else {
    if (look4)
      launch_pass_items<K, HAS_V, IOTA, kItemsMax, 4>(ctx, kin, kout, vin, vout, n, shift, bases, status, ticket);
    else
      launch_pass_items<K, HAS_V, IOTA, kItemsMax, 1>(ctx, kin, kout, vin, vout, n, shift, bases, status, ticket);
  }
}

template <typename K>
bool radix_sort_impl(Ctx& ctx, K* keys, K* keys_alt, uint32_t* vals, uint32_t* vals_alt, uint64_t n,
                     int begin_bit, int end_bit, bool vals_iota, bool host_skip) {
  const bool has_v = vals != nullptr;
  if (n == 0) return false;
  if (n > 0xFFFFFFFFull && has_v) fail(VG_ERR_OVERFLOW, "radix sort values are 32-bit row ids");
  if (begin_bit < 0 || begin_bit >= end_bit) begin_bit = 0;
  int passes = (end_bit - begin_bit + 7) / 8;
  if (passes < 1) passes = 1;
  // the last pass may read bits above end_bit; it must not shift past the key
  while (passes > 1 && begin_bit + 8 * (passes - 1) >= static_cast<int>(8 * sizeof(K))) --passes;

  Scratch<unsigned long long> hist(ctx, passes * kRadix);
  VG_CUDA(cudaMemsetAsync(hist.get(), 0, passes * kRadix * sizeof(unsigned long long), ctx.stream));
  uint64_t grid = div_up(n, kBlock * 16);
  const uint64_t gmax = static_cast<uint64_t>(ctx.num_sms) * 8;
  if (grid > gmax) grid = gmax;
  if (grid < 1) grid = 1;
  ctx.launch("radix_histogram", static_cast<double>(n) * sizeof(K), [&] {
    radix_hist_kernel<K><<<static_cast<unsigned>(grid), kBlock, 0, ctx.stream>>>(keys, n, passes, begin_bit,
                                                                                hist.get());
  });
  VG_CUDA(cudaGetLastError());
  Scratch<uint64_t> d_bases(ctx, passes * kRadix);
  std::vector<int> todo;
  if (host_skip) {
    std::vector<unsigned long long> h(passes * kRadix);
    VG_CUDA(cudaMemcpyAsync(h.data(), hist.get(), h.size() * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    std::vector<uint64_t> bases(passes * kRadix);
    for (int p = 0; p < passes; ++p) {
      uint64_t run = 0;
      bool trivial = false;
      for (int d = 0; d < kRadix; ++d) {
        const uint64_t c = h[p * kRadix + d];
        if (c == n) trivial = true;
        bases[p * kRadix + d] = run;
        run += c;
      }
      if (!trivial) todo.push_back(p);
    }
    if (todo.empty()) {
      if (has_v && vals_iota) {
        ctx.launch("iota", 4.0 * n, [&] { iota_kernel<<<static_cast<unsigned>(grid), kBlock, 0, ctx.stream>>>(vals, n); });
        VG_CUDA(cudaGetLastError());
      }
      return false;
    }
    VG_CUDA(cudaMemcpyAsync(d_bases.get(), bases.data(), bases.size() * sizeof(uint64_t),
                            cudaMemcpyHostToDevice, ctx.stream));
  } else {
    // no host round trip: bases scanned on the device and every pass runs
    ctx.launch("radix_bases", 0.0, [&] {
      radix_bases_kernel<<<static_cast<unsigned>(passes), kRadix, 0, ctx.stream>>>(hist.get(), d_bases.get());
    });
    VG_CUDA(cudaGetLastError());
    for (int p = 0; p < passes; ++p) todo.push_back(p);
  }
  const int items = (ctx.tune.sort_items == 8 || ctx.tune.sort_items == 12) ? static_cast<int>(ctx.tune.sort_items)
                                                                            : kItemsMax;
  const uint64_t tiles = div_up(n, static_cast<uint64_t>(kBlock) * items);
  Scratch<uint64_t> status(ctx, tiles * kRadix);
  Scratch<uint32_t> ticket(ctx, todo.size());
  VG_CUDA(cudaMemsetAsync(ticket.get(), 0, todo.size() * sizeof(uint32_t), ctx.stream));

  K* kin = keys;
  K* kout = keys_alt;
  uint32_t* vin = vals;
  uint32_t* vout = vals_alt;
  for (size_t t = 0; t < todo.size(); ++t) {
    const int p = todo[t];
    VG_CUDA(cudaMemsetAsync(status.get(), 0, tiles * kRadix * sizeof(uint64_t), ctx.stream));
    const uint64_t* pb = d_bases.get() + p * kRadix;
    const uint32_t shift = static_cast<uint32_t>(begin_bit + 8 * p);
    if (!has_v)
      launch_pass<K, false, false>(ctx, items, kin, kout, nullptr, nullptr, n, shift, pb, status.get(),
                                   ticket.get() + t);
    else if (t == 0 && vals_iota)
      launch_pass<K, true, true>(ctx, items, kin, kout, nullptr, vout, n, shift, pb, status.get(),
                                 ticket.get() + t);
    else
      launch_pass<K, true, false>(ctx, items, kin, kout, vin, vout, n, shift, pb, status.get(),
                                  ticket.get() + t);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  return kin == keys_alt;
}

}  // namespace

bool radix_sort_u32(Ctx& ctx, uint32_t* keys, uint32_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                    uint64_t n, int end_bit, bool vals_iota, bool host_skip) {
  return radix_sort_impl<uint32_t>(ctx, keys, keys_alt, vals, vals_alt, n, 0, end_bit, vals_iota, host_skip);
}

bool radix_sort_u64(Ctx& ctx, uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                    uint64_t n, int end_bit, bool vals_iota, bool host_skip) {
  return radix_sort_impl<uint64_t>(ctx, keys, keys_alt, vals, vals_alt, n, 0, end_bit, vals_iota, host_skip);
}

bool radix_sort_u64_bits(Ctx& ctx, uint64_t* keys, uint64_t* keys_alt, uint64_t n, int begin_bit, int end_bit) {
  return radix_sort_impl<uint64_t>(ctx, keys, keys_alt, nullptr, nullptr, n, begin_bit, end_bit, false, true);
}

void fill_iota(Ctx& ctx, uint32_t* out, uint64_t n) {
  if (n == 0) return;
  uint64_t grid = div_up(n, kBlock * 8);
  const uint64_t gmax = static_cast<uint64_t>(ctx.num_sms) * 8;
  if (grid > gmax) grid = gmax;
  ctx.launch("iota", 4.0 * n, [&] { iota_kernel<<<static_cast<unsigned>(grid), kBlock, 0, ctx.stream>>>(out, n); });
  VG_CUDA(cudaGetLastError());
}

}  // namespace vg
