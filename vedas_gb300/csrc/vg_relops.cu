// Relation kernels: select copies, adjacent-unique compaction, sort-merge
// join (count -> scan -> load-balanced write), gathers and relation sorts.
#include "vg_relops.h"

#include <cstring>

#include <algorithm>

#include "vg_join_tile.cuh"
#include "vg_prims.cuh"
#include "vg_sort.h"

namespace vg {
namespace {

constexpr int kBlock = 256;
constexpr int kRows = 8;
constexpr int kTileRows = kBlock * kRows;

unsigned grid_for(const Ctx& ctx, uint64_t n, int per_thread, int per_sm = 16) {
  uint64_t g = div_up(n, static_cast<uint64_t>(kBlock) * per_thread);
  const uint64_t gmax = static_cast<uint64_t>(ctx.num_sms) * per_sm;
  if (g > gmax) g = gmax;
  return static_cast<unsigned>(g < 1 ? 1 : g);
}

// ---------------------------------------------------------------------------
// Multi-piece copy: destination-aligned 128-bit stores, source loads
// vectorised when the source shares the destination's 16-byte phase.
// ---------------------------------------------------------------------------
struct CopyArgs {
  CopyPiece p[16];
  uint64_t start[17];  // prefix of vector-chunk counts per piece
  int np;
};

__global__ void __launch_bounds__(kBlock) multi_copy_kernel(CopyArgs a) {
  const uint64_t total = a.start[a.np];
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * kBlock;
  for (uint64_t q = static_cast<uint64_t>(blockIdx.x) * kBlock + threadIdx.x; q < total; q += stride) {
    int k = 0;
    while (q >= a.start[k + 1]) ++k;
    const CopyPiece& pc = a.p[k];
    const uint64_t c = q - a.start[k];
    // head: elements before the first 16-byte aligned destination address
    const uint64_t head = (4 - ((reinterpret_cast<uintptr_t>(pc.dst) >> 2) & 3)) & 3;
    const uint64_t h = head < pc.len ? head : pc.len;
    if (c == 0) {
      for (uint64_t e = 0; e < h; ++e) pc.dst[e] = pc.src[e];
      // tail after the last full vector
      const uint64_t body = (pc.len - h) / 4 * 4;
      for (uint64_t e = h + body; e < pc.len; ++e) pc.dst[e] = pc.src[e];
    }
    const uint64_t e0 = h + c * 4;
    if (e0 + 4 > pc.len) continue;
    uint4 v;
    const uint32_t* s = pc.src + e0;
    if (c > 0 && e0 + 8 <= pc.len) {
      v = load4_realigned(s);   // both aligned vectors inside the piece
    } else {
      v.x = s[0];
      v.y = s[1];
      v.z = s[2];
      v.w = s[3];
    }
    *reinterpret_cast<uint4*>(pc.dst + e0) = v;
  }
}

// ---------------------------------------------------------------------------
// Adjacent-unique compaction (thrust::unique over zipped columns).
// ---------------------------------------------------------------------------
struct UniqueArgs {
  const uint32_t* in[VG_MAX_COLS];
  uint32_t* out[VG_MAX_COLS];
  uint32_t ncols;
  uint64_t n;
  uint64_t* status;
  uint32_t* ticket;
  uint64_t* count;
  uint64_t tiles;
  DeviceErrors* err;
};

// Adjacent-unique compaction: each thread flags its kRows rows (16-byte
// loads of aligned columns), a block scan and a look-back place the tile's
// kept rows, which are stored column by column through shared memory so
// that every store is coalesced.
__global__ void __launch_bounds__(kBlock) unique_kernel(UniqueArgs a) {
  static_assert(kRows == 8, "unique_diff_bits and compact_store take 8 rows per thread");
  __shared__ uint32_t s_scan[kBlock / 32 + 1];
  __shared__ uint64_t s_b;
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_keep[2 * kTileRows];   // compact_store: two columns at a time
  if (threadIdx.x == 0) s_tile = atomicAdd(a.ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint64_t r0 = static_cast<uint64_t>(tile) * kTileRows + threadIdx.x * kRows;
  uint32_t diff = (r0 == 0) ? 1u : 0u;
  for (uint32_t c = 0; c < a.ncols; ++c) diff |= unique_diff_bits(a.in[c], a.n, r0);
  if (r0 >= a.n) diff = 0;
  else if (a.n - r0 < kRows) diff &= (1u << (a.n - r0)) - 1u;
  uint32_t tot;
  const uint32_t e = block_excl_scan<kBlock>(__popc(diff), tot, s_scan);
  const uint64_t g = block_lookback(a.status, tile, tot, a.err, &s_b);
  if (tile == a.tiles - 1 && threadIdx.x == 0) *a.count = g + tot;
  compact_store<kBlock>(a.in, a.out, a.ncols, a.n, r0, diff, e, tot, g, s_keep);
}

// ---------------------------------------------------------------------------
// Join.  Count: lower bound and match count of every left key in the right
// keys, searching inside the right-key window of the block's left keys.
// Scan: exclusive scan of counts to output offsets.  Write: every output row
// finds its left row by an upper-bound search of the offsets (load-balanced
// across heavy keys) and gathers its columns.
// ---------------------------------------------------------------------------
template <bool TWO>
struct KeyOf {
  const uint32_t* c0;
  const uint32_t* c1;
  __device__ __forceinline__ uint64_t operator()(uint64_t i) const {
    return TWO ? ((static_cast<uint64_t>(c0[i]) << 32) | c1[i]) : static_cast<uint64_t>(c0[i]);
  }
};

template <bool TWO>
__device__ uint64_t key_lower_bound(const KeyOf<TWO>& k, uint64_t lo, uint64_t hi, uint64_t key) {
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (k(mid) < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
template <bool TWO>
__device__ uint64_t key_upper_bound(const KeyOf<TWO>& k, uint64_t lo, uint64_t hi, uint64_t key) {
  while (lo < hi) {
    uint64_t mid = (lo + hi) >> 1;
    if (key < k(mid)) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

template <bool TWO>
__global__ void __launch_bounds__(kBlock) join_count_kernel(KeyOf<TWO> L, uint64_t nl, KeyOf<TWO> R,
                                                            uint64_t nr, uint32_t* __restrict__ lo_out,
                                                            uint32_t* __restrict__ cnt_out) {
  __shared__ uint64_t s_win[2];
  const uint64_t i0 = static_cast<uint64_t>(blockIdx.x) * kBlock;
  if (threadIdx.x == 0) {
    const uint64_t i1 = (i0 + kBlock < nl ? i0 + kBlock : nl) - 1;
    const uint64_t w0 = key_lower_bound(R, 0, nr, L(i0));
    s_win[0] = w0;
    s_win[1] = key_upper_bound(R, w0, nr, L(i1));
  }
  __syncthreads();
  const uint64_t i = i0 + threadIdx.x;
  if (i >= nl) return;
  const uint64_t k = L(i);
  const uint64_t lo = key_lower_bound(R, s_win[0], s_win[1], k);
  const uint64_t hi = key_upper_bound(R, lo, s_win[1], k);
  lo_out[i] = static_cast<uint32_t>(lo);
  cnt_out[i] = static_cast<uint32_t>(hi - lo);
}

// One block per 2048 left keys; the right-key window is staged in shared
// memory by a bulk copy (vg_join_tile.cuh).
__global__ void __launch_bounds__(kJcBlock, 4) join_count_tiled_kernel(const uint32_t* __restrict__ L, uint64_t nl,
                                                                    const uint32_t* __restrict__ R, uint64_t nr,
                                                                    uint32_t* __restrict__ lo,
                                                                    uint32_t* __restrict__ cnt, DeviceErrors* err) {
  __shared__ JoinCountSmem sm;
  join_count_tile(L, nl, R, nr, static_cast<uint64_t>(blockIdx.x) * kJcTile, lo, cnt, sm, err);
  if (threadIdx.x == 0) jc_drain_window(sm, err);
}

// Exclusive scan of uint32 counts into uint64 offsets (+ total).
__global__ void __launch_bounds__(kBlock) scan_counts_kernel(const uint32_t* __restrict__ in,
                                                             uint64_t* __restrict__ out, uint64_t n,
                                                             uint64_t* status, uint32_t* ticket,
                                                             uint64_t* total, uint64_t tiles,
                                                             DeviceErrors* err) {
  __shared__ uint64_t s_scan[kBlock / 32 + 1];
  __shared__ uint64_t s_b;
  __shared__ uint32_t s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint64_t r0 = static_cast<uint64_t>(tile) * kTileRows + threadIdx.x * kRows;
  uint32_t v[kRows];
  uint64_t sum = 0;
#pragma unroll
  for (int i = 0; i < kRows; ++i) {
    v[i] = (r0 + i < n) ? in[r0 + i] : 0u;
    sum += v[i];
  }
  uint64_t tot;
  const uint64_t e = block_excl_scan64<kBlock>(sum, tot, s_scan);
  const uint64_t g = block_lookback(status, tile, tot, err, &s_b);
  if (tile == tiles - 1 && threadIdx.x == 0) *total = g + tot;
  uint64_t run = g + e;
#pragma unroll
  for (int i = 0; i < kRows; ++i) {
    if (r0 + i < n) out[r0 + i] = run;
    run += v[i];
  }
}

struct JoinWriteArgs {
  const uint64_t* offs;
  const uint32_t* lo;
  uint64_t nl, total;
  const uint32_t* lc[VG_MAX_COLS];
  const uint32_t* rc[VG_MAX_COLS];
  uint32_t* oc[VG_MAX_COLS];
  uint32_t nlc, nrc;
};

__global__ void __launch_bounds__(kBlock) join_write_kernel(JoinWriteArgs a) {
  __shared__ uint64_t s_i[2];
  const uint64_t kb = static_cast<uint64_t>(blockIdx.x) * kTileRows;
  if (threadIdx.x == 0) {
    const uint64_t klast = (kb + kTileRows < a.total ? kb + kTileRows : a.total) - 1;
    const uint64_t f = upper_bound_dev(a.offs, 0, a.nl, kb) - 1;
    s_i[0] = f;
    s_i[1] = upper_bound_dev(a.offs, f, a.nl, klast);
  }
  __syncthreads();
  const uint64_t ib = s_i[0], ie = s_i[1];
#pragma unroll 2
  for (int it = 0; it < kRows; ++it) {
    const uint64_t k = kb + static_cast<uint64_t>(it) * kBlock + threadIdx.x;
    if (k >= a.total) break;
    const uint64_t i = upper_bound_dev(a.offs, ib, ie, k) - 1;
    const uint64_t j = a.lo[i] + (k - a.offs[i]);
    // every value of the row loaded (read-only path) before any is stored
    uint32_t v[VG_MAX_COLS];
    const int ncols = static_cast<int>(a.nlc + a.nrc);
#pragma unroll
    for (int c = 0; c < VG_MAX_COLS; ++c)
      if (c < ncols) v[c] = c < static_cast<int>(a.nlc) ? __ldg(a.lc[c] + i) : __ldg(a.rc[c - a.nlc] + j);
#pragma unroll
    for (int c = 0; c < VG_MAX_COLS; ++c)
      if (c < ncols) a.oc[c][k] = v[c];
  }
}

struct GatherCols {
  const uint32_t* in[VG_MAX_COLS];
  uint32_t* out[VG_MAX_COLS];
  uint32_t ncols;
};

__global__ void __launch_bounds__(kBlock) gather_kernel(const uint32_t* __restrict__ perm, uint64_t n,
                                                        GatherCols g) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * kBlock;
  for (uint64_t r = static_cast<uint64_t>(blockIdx.x) * kBlock + threadIdx.x; r < n; r += stride) {
    const uint32_t p = perm[r];
    uint32_t v[VG_MAX_COLS];
#pragma unroll
    for (int c = 0; c < VG_MAX_COLS; ++c)
      if (c < static_cast<int>(g.ncols)) v[c] = __ldg(g.in[c] + p);
#pragma unroll
    for (int c = 0; c < VG_MAX_COLS; ++c)
      if (c < static_cast<int>(g.ncols)) g.out[c][r] = v[c];
  }
}
}  // namespace

Rel rel_alloc(Ctx& ctx, uint32_t ncols, uint64_t nrows) {
  if (ncols > VG_MAX_COLS) fail(VG_ERR_UNSUPPORTED, "more than 9 columns");
  Rel r;
  r.ncols = ncols;
  r.nrows = nrows;
  for (uint32_t c = 0; c < ncols; ++c) r.cols[c] = ctx.alloc<uint32_t>(nrows);
  return r;
}

void rel_free(Ctx& ctx, Rel& r) {
  for (uint32_t c = 0; c < r.ncols; ++c) {
    if (!(r.borrowed >> c & 1u)) ctx.free(r.cols[c]);
    r.cols[c] = nullptr;
  }
  r.ncols = 0;
  r.nrows = 0;
  r.borrowed = 0;
}

void rel_drop_col(Ctx& ctx, Rel& r, uint32_t c) {
  if (!(r.borrowed >> c & 1u)) ctx.free(r.cols[c]);
  r.borrowed &= ~(1u << c);
}

void rel_own(Ctx& ctx, Rel& r) {
  for (uint32_t c = 0; c < r.ncols; ++c) {
    if (!(r.borrowed >> c & 1u)) continue;
    uint32_t* o = ctx.alloc<uint32_t>(r.nrows);
    if (r.nrows)
      VG_CUDA(cudaMemcpyAsync(o, r.cols[c], r.nrows * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx.stream));
    r.cols[c] = o;
  }
  r.borrowed = 0;
}

void multi_copy(Ctx& ctx, const CopyPiece* pieces, int np) {
  if (np > 16) fail(VG_ERR_INVALID, "multi_copy: too many pieces");
  CopyArgs a{};
  a.np = 0;
  a.start[0] = 0;
  for (int k = 0; k < np; ++k) {
    if (pieces[k].len == 0) continue;
    const uint64_t head = (4 - ((reinterpret_cast<uintptr_t>(pieces[k].dst) >> 2) & 3)) & 3;
    const uint64_t h = head < pieces[k].len ? head : pieces[k].len;
    const uint64_t chunks = (pieces[k].len - h) / 4;
    a.p[a.np] = pieces[k];
    a.start[a.np + 1] = a.start[a.np] + (chunks ? chunks : 1);
    ++a.np;
  }
  if (a.np == 0) return;
  double bytes = 0;
  for (int k = 0; k < a.np; ++k) bytes += 8.0 * a.p[k].len;
  ctx.launch("select_copy", bytes,
             [&] { multi_copy_kernel<<<grid_for(ctx, a.start[a.np], 2), kBlock, 0, ctx.stream>>>(a); });
  VG_CUDA(cudaGetLastError());
}

uint64_t unique_rows(Ctx& ctx, const uint32_t* const* in, uint32_t* const* out, uint32_t ncols,
                     uint64_t n) {
  if (n == 0) return 0;
  UniqueArgs a{};
  for (uint32_t c = 0; c < ncols; ++c) {
    a.in[c] = in[c];
    a.out[c] = out[c];
  }
  a.ncols = ncols;
  a.n = n;
  a.tiles = div_up(n, kTileRows);
  Scratch<uint64_t> status(ctx, a.tiles), count(ctx, 1);
  Scratch<uint32_t> ticket(ctx, 1);
  VG_CUDA(cudaMemsetAsync(status.get(), 0, a.tiles * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(uint32_t), ctx.stream));
  a.status = status.get();
  a.ticket = ticket.get();
  a.count = count.get();
  a.err = ctx.d_err;
  ctx.launch("unique_compact", 4.0 * n * ncols,
             [&] { unique_kernel<<<static_cast<unsigned>(a.tiles), kBlock, 0, ctx.stream>>>(a); });
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaMemcpyAsync(ctx.h_small, count.get(), sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  const uint64_t kept = ctx.h_small[0];
  ctx.add_bytes("unique_compact", 4.0 * kept * ncols);
  return kept;
}

void join(Ctx& ctx, const Rel& l, const Rel& r, bool two_keys, Rel& out) {
  const uint32_t nk = two_keys ? 2 : 1;
  if (l.ncols < nk || r.ncols < nk) fail(VG_ERR_INVALID, "join: missing key columns");
  const uint32_t ncols = l.ncols + r.ncols - nk;
  if (ncols > VG_MAX_COLS) fail(VG_ERR_UNSUPPORTED, "join output has more than 9 columns");
  if (l.nrows > 0xFFFFFFFFull || r.nrows > 0xFFFFFFFFull)
    fail(VG_ERR_OVERFLOW, "join inputs are limited to 2^32 rows");
  if (l.nrows == 0 || r.nrows == 0) {
    out = rel_alloc(ctx, ncols, 0);
    return;
  }
  Scratch<uint32_t> lo(ctx, l.nrows), cnt(ctx, l.nrows);
  const unsigned cgrid = static_cast<unsigned>(div_up(l.nrows, kBlock));
  const double cbytes = 4.0 * nk * (l.nrows + r.nrows);
  if (two_keys) {
    KeyOf<true> kl{l.cols[0], l.cols[1]}, kr{r.cols[0], r.cols[1]};
    ctx.launch("join_count", cbytes, [&] {
      join_count_kernel<true><<<cgrid, kBlock, 0, ctx.stream>>>(kl, l.nrows, kr, r.nrows, lo.get(), cnt.get());
    });
  } else {
    ctx.launch("join_count", cbytes, [&] {
      join_count_tiled_kernel<<<static_cast<unsigned>(div_up(l.nrows, kJcTile)), kJcBlock, 0, ctx.stream>>>(
          l.cols[0], l.nrows, r.cols[0], r.nrows, lo.get(), cnt.get(), ctx.d_err);
    });
  }
  VG_CUDA(cudaGetLastError());
  const uint64_t tiles = div_up(l.nrows, kTileRows);
  Scratch<uint64_t> offs(ctx, l.nrows), status(ctx, tiles), total(ctx, 1);
  Scratch<uint32_t> ticket(ctx, 1);
  VG_CUDA(cudaMemsetAsync(status.get(), 0, tiles * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(uint32_t), ctx.stream));
  ctx.launch("join_scan", 12.0 * l.nrows, [&] {
    scan_counts_kernel<<<static_cast<unsigned>(tiles), kBlock, 0, ctx.stream>>>(
        cnt.get(), offs.get(), l.nrows, status.get(), ticket.get(), total.get(), tiles, ctx.d_err);
  });
  VG_CUDA(cudaGetLastError());
  // the total and the error record come back together: a look-back that gave
  // up leaves the offsets wrong, and the write must then not run
  VG_CUDA(cudaMemcpyAsync(ctx.h_small, total.get(), sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx.stream));
  VG_CUDA(cudaMemcpyAsync(ctx.h_small + 1, ctx.d_err, sizeof(DeviceErrors), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  const uint64_t t = ctx.h_small[0];
  {
    DeviceErrors he;
    std::memcpy(&he, ctx.h_small + 1, sizeof(he));
    ctx.raise_device_errors(he);
  }
  if (t > 0xFFFFFFFFull) fail(VG_ERR_OVERFLOW, "join output exceeds 2^32 rows");
  out = rel_alloc(ctx, ncols, t);
  if (t == 0) return;
  JoinWriteArgs a{};
  a.offs = offs.get();
  a.lo = lo.get();
  a.nl = l.nrows;
  a.total = t;
  for (uint32_t c = 0; c < l.ncols; ++c) a.lc[c] = l.cols[c];
  for (uint32_t c = nk; c < r.ncols; ++c) a.rc[c - nk] = r.cols[c];
  for (uint32_t c = 0; c < ncols; ++c) a.oc[c] = out.cols[c];
  a.nlc = l.ncols;
  a.nrc = r.ncols - nk;
  ctx.launch("join_write", 4.0 * t * (2.0 * ncols - 1), [&] {
    join_write_kernel<<<static_cast<unsigned>(div_up(t, kTileRows)), kBlock, 0, ctx.stream>>>(a);
  });
  VG_CUDA(cudaGetLastError());
}

uint64_t join_into(cudaStream_t stream, int num_sms, const Rel& l, const Rel& r, uint32_t* const* out_cols,
                   uint64_t capacity, uint32_t* lo, uint32_t* cnt, uint64_t* offs, uint64_t* status,
                   uint32_t* ticket, uint64_t* total, DeviceErrors* err) {
  (void)num_sms;
  if (l.nrows == 0 || r.nrows == 0) return 0;
  const uint32_t ncols = l.ncols + r.ncols - 1;
  join_count_tiled_kernel<<<static_cast<unsigned>(div_up(l.nrows, kJcTile)), kJcBlock, 0, stream>>>(
      l.cols[0], l.nrows, r.cols[0], r.nrows, lo, cnt, err);
  VG_CUDA(cudaGetLastError());
  const uint64_t tiles = div_up(l.nrows, kTileRows);
  scan_counts_kernel<<<static_cast<unsigned>(tiles), kBlock, 0, stream>>>(cnt, offs, l.nrows, status, ticket,
                                                                         total, tiles, err);
  VG_CUDA(cudaGetLastError());
  uint64_t t = 0;
  DeviceErrors he{};
  VG_CUDA(cudaMemcpyAsync(&t, total, sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
  VG_CUDA(cudaMemcpyAsync(&he, err, sizeof(he), cudaMemcpyDeviceToHost, stream));
  VG_CUDA(cudaStreamSynchronize(stream));
  // a look-back that gave up leaves the offsets wrong: no write then
  if (he.timeout) fail(VG_ERR_TIMEOUT, "join_into: a bounded device wait expired");
  if (t == 0 || t > capacity) return t;
  JoinWriteArgs a{};
  a.offs = offs;
  a.lo = lo;
  a.nl = l.nrows;
  a.total = t;
  for (uint32_t c = 0; c < l.ncols; ++c) a.lc[c] = l.cols[c];
  for (uint32_t c = 1; c < r.ncols; ++c) a.rc[c - 1] = r.cols[c];
  for (uint32_t c = 0; c < ncols; ++c) a.oc[c] = out_cols[c];
  a.nlc = l.ncols;
  a.nrc = r.ncols - 1;
  join_write_kernel<<<static_cast<unsigned>(div_up(t, kTileRows)), kBlock, 0, stream>>>(a);
  VG_CUDA(cudaGetLastError());
  return t;
}

void gather_cols(Ctx& ctx, const uint32_t* const* in, uint32_t* const* out, uint32_t ncols,
                 const uint32_t* perm, uint64_t n) {
  if (n == 0 || ncols == 0) return;
  GatherCols g{};
  for (uint32_t c = 0; c < ncols; ++c) {
    g.in[c] = in[c];
    g.out[c] = out[c];
  }
  g.ncols = ncols;
  ctx.launch("gather", static_cast<double>(n) * (4.0 + 8.0 * ncols),
             [&] { gather_kernel<<<grid_for(ctx, n, 4), kBlock, 0, ctx.stream>>>(perm, n, g); });
  VG_CUDA(cudaGetLastError());
}

void sort_by_first(Ctx& ctx, Rel& r) {
  const uint64_t n = r.nrows;
  if (n <= 1 || r.ncols == 0) return;
  if (n > 0xFFFFFFFFull) fail(VG_ERR_OVERFLOW, "relation sorts are limited to 2^32 rows");
  if (r.borrowed & 1u) {
    // the sort uses column 0 as its key buffer: take a copy of a view
    Rel k0;
    k0.ncols = 1;
    k0.nrows = n;
    k0.cols[0] = r.cols[0];
    k0.borrowed = 1;
    rel_own(ctx, k0);
    r.cols[0] = k0.cols[0];
    r.borrowed &= ~1u;
  }
  uint32_t* keys_alt = ctx.alloc<uint32_t>(n);
  if (r.ncols == 1) {
    const bool alt = radix_sort_u32(ctx, r.cols[0], keys_alt, nullptr, nullptr, n, 32, false);
    if (alt) {
      ctx.free(r.cols[0]);
      r.cols[0] = keys_alt;
    } else {
      ctx.free(keys_alt);
    }
    return;
  }
  uint32_t* vals = ctx.alloc<uint32_t>(n);
  uint32_t* vals_alt = ctx.alloc<uint32_t>(n);
  const bool alt = radix_sort_u32(ctx, r.cols[0], keys_alt, vals, vals_alt, n, 32, true);
  uint32_t* perm = alt ? vals_alt : vals;
  if (alt) {
    ctx.free(r.cols[0]);
    r.cols[0] = keys_alt;
  } else {
    ctx.free(keys_alt);
  }
  ctx.free(alt ? vals : vals_alt);
  for (uint32_t c = 1; c < r.ncols; ++c) {
    uint32_t* nc = ctx.alloc<uint32_t>(n);
    const uint32_t* in[1] = {r.cols[c]};
    uint32_t* out[1] = {nc};
    gather_cols(ctx, in, out, 1, perm, n);
    rel_drop_col(ctx, r, c);
    r.cols[c] = nc;
  }
  ctx.free(perm);
}

void sort_rows(Ctx& ctx, Rel& r) {
  const uint64_t n = r.nrows;
  if (n <= 1 || r.ncols <= 1) return;  // one column: a no-op in the reference
  if (n > 0xFFFFFFFFull) fail(VG_ERR_OVERFLOW, "relation sorts are limited to 2^32 rows");
  uint32_t* perm = ctx.alloc<uint32_t>(n);
  uint32_t* perm_alt = ctx.alloc<uint32_t>(n);
  uint32_t* keys = ctx.alloc<uint32_t>(n);
  uint32_t* keys_alt = ctx.alloc<uint32_t>(n);
  fill_iota(ctx, perm, n);
  // LSD over columns: stable sorts from the last column to the first.
  for (int c = static_cast<int>(r.ncols) - 1; c >= 0; --c) {
    const uint32_t* in[1] = {r.cols[c]};
    uint32_t* out[1] = {keys};
    gather_cols(ctx, in, out, 1, perm, n);
    const bool alt = radix_sort_u32(ctx, keys, keys_alt, perm, perm_alt, n, 32, false);
    if (alt) std::swap(perm, perm_alt);
  }
  for (uint32_t c = 0; c < r.ncols; ++c) {
    uint32_t* nc = ctx.alloc<uint32_t>(n);
    const uint32_t* in[1] = {r.cols[c]};
    uint32_t* out[1] = {nc};
    gather_cols(ctx, in, out, 1, perm, n);
    rel_drop_col(ctx, r, c);
    r.cols[c] = nc;
  }
  ctx.free(perm);
  ctx.free(perm_alt);
  ctx.free(keys);
  ctx.free(keys_alt);
}

void unique_in_place(Ctx& ctx, Rel& r) {
  if (r.nrows <= 1 || r.ncols == 0) return;
  Rel out = rel_alloc(ctx, r.ncols, r.nrows);
  const uint64_t kept = unique_rows(ctx, r.cols, out.cols, r.ncols, r.nrows);
  rel_free(ctx, r);
  for (uint32_t c = 0; c < out.ncols; ++c) ctx.arena.shrink(out.cols[c], kept * sizeof(uint32_t));
  out.nrows = kept;
  r = out;
}

void download(Ctx& ctx, const uint32_t* dev, uint64_t n, uint32_t* host) {
  if (n) VG_CUDA(cudaMemcpyAsync(host, dev, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
}

}  // namespace vg
