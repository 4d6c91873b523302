// Batched relation kernels.  Work from many queries is laid out as segments;
// a kernel maps its tile or chunk to its segments through a table made on the
// host (the tile's first segment), and a row to its segment by a search
// between the tile's first and last segments only.
#include "vg_batch.h"

#include <algorithm>
#include <cstring>

#include "vg_join_tile.cuh"
#include "vg_pool.h"
#include "vg_prims.cuh"
#include "vg_sort.h"

namespace vg {
namespace {

constexpr int kBlock = 256;
constexpr int kRows = 8;
constexpr int kTileRows = kBlock * kRows;

template <typename T>
T* upload(Ctx& ctx, const std::vector<T>& v) {
  T* d = static_cast<T*>(ctx.arena.alloc((v.empty() ? 1 : v.size()) * sizeof(T)));
  if (!v.empty()) ctx.upload_bytes(d, v.data(), v.size() * sizeof(T));
  return d;
}

unsigned grid_cap(const Ctx& ctx, uint64_t units, int per_thread) {
  uint64_t g = div_up(units, static_cast<uint64_t>(kBlock) * per_thread);
  const uint64_t gmax = static_cast<uint64_t>(ctx.num_sms) * 16;
  if (g > gmax) g = gmax;
  return static_cast<unsigned>(g < 1 ? 1 : g);
}

// ---------------------------------------------------------------------------
constexpr int kCopyPer = 4;                                   // 16-byte chunks per thread per tile
constexpr uint64_t kCopyTile = static_cast<uint64_t>(kBlock) * kCopyPer;

// Copies every piece; destination chunks are 16-byte aligned (head and tail
// elements are copied by the piece's first chunk).  Blocks take tiles of
// kCopyTile consecutive chunks; a tile's first piece comes from a table made
// on the host and the next tile's bounds its last, so a thread's piece lookup
// is a search over those few pieces only (no global search, no barrier).
__global__ void __launch_bounds__(kBlock) bcopy_kernel(const CopyPiece* __restrict__ p,
                                                       const uint64_t* __restrict__ cstart, uint32_t P,
                                                       const uint32_t* __restrict__ tile_piece, uint64_t ntiles) {
  const uint64_t total = cstart[P];
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint64_t q0 = t * kCopyTile;
    const uint64_t q1 = (q0 + kCopyTile < total) ? q0 + kCopyTile : total;
    const uint32_t k0 = tile_piece[t], k1 = t + 1 < ntiles ? tile_piece[t + 1] : P - 1;
#pragma unroll
    for (int i = 0; i < kCopyPer; ++i) {
      const uint64_t q = q0 + static_cast<uint64_t>(i) * kBlock + threadIdx.x;
      if (q >= q1) break;
      uint32_t k = k0;
      if (k1 > k0) {
        uint32_t lo = k0, hi = k1;   // last k in [k0, k1] with cstart[k] <= q
        while (lo < hi) {
          const uint32_t mid = (lo + hi + 1) >> 1;
          if (cstart[mid] <= q) lo = mid;
          else hi = mid - 1;
        }
        k = lo;
      }
      const CopyPiece pc = p[k];
      const uint64_t c = q - cstart[k];
      const uint64_t head = (4 - ((reinterpret_cast<uintptr_t>(pc.dst) >> 2) & 3)) & 3;
      const uint64_t h = head < pc.len ? head : pc.len;
      if (c == 0) {
        for (uint64_t e = 0; e < h; ++e) pc.dst[e] = pc.src[e];
        const uint64_t body = (pc.len - h) / 4 * 4;
        for (uint64_t e = h + body; e < pc.len; ++e) pc.dst[e] = pc.src[e];
      }
      const uint64_t e0 = h + c * 4;
      if (e0 + 4 > pc.len) continue;
      const uint32_t* s = pc.src + e0;
      uint4 v;
      // vectors [s - sh, s - sh + 8) stay inside the piece for every chunk
      // but the first and the last
      if (c > 0 && e0 + 8 <= pc.len) {
        v = load4_realigned(s);
      } else {
        v.x = s[0];
        v.y = s[1];
        v.z = s[2];
        v.w = s[3];
      }
      *reinterpret_cast<uint4*>(pc.dst + e0) = v;
    }
  }
}

// ---------------------------------------------------------------------------
// Adjacent-unique compaction of every segment.  Segments of at most
// kSmallSeg rows (most final results) take one warp each in the first
// small_blocks blocks: each lane flags its kRows consecutive rows, a warp
// scan places the kept ones.  Larger segments take tiles of kTileRows rows
// in ticket order (the tile's segment from a per-tile table), with a block
// scan and a segmented look-back over the segment's earlier tiles.
constexpr uint32_t kSmallSeg = 32 * kRows;

__device__ __forceinline__ void unique_small_segment(const SegRows& g, uint64_t* count) {
  const uint32_t lane = lane_id();
  const uint64_t n = g.n, r0 = static_cast<uint64_t>(lane) * kRows;
  uint32_t diff = (r0 == 0 && n > 0) ? 1u : 0u;
  for (uint32_t c = 0; c < g.ncols; ++c) diff |= unique_diff_bits(g.in[c], n, r0);
  if (r0 >= n) diff = 0;
  else if (n - r0 < kRows) diff &= (1u << (n - r0)) - 1u;
  const uint32_t cnt = __popc(diff);
  const uint32_t incl = warp_incl_scan(cnt);
  uint64_t o = incl - cnt;
  for (int i = 0; i < kRows; ++i) {
    if (!(diff >> i & 1u)) continue;
    copy_row(g.out, g.in, g.ncols, r0 + i, o);
    ++o;
  }
  if (lane == 31) *count = incl;
}

__global__ void __launch_bounds__(kBlock) bunique_kernel(const SegRows* __restrict__ segs,
                                                         const uint64_t* __restrict__ tstart,
                                                         const uint32_t* __restrict__ tile_seg,
                                                         const uint32_t* __restrict__ small, uint32_t nsmall,
                                                         uint32_t small_blocks, uint64_t* status, uint32_t* ticket,
                                                         uint64_t* counts, DeviceErrors* err) {
  if (blockIdx.x < small_blocks) {   // block-uniform: this block only compacts small segments
    const uint64_t w = static_cast<uint64_t>(blockIdx.x) * (kBlock / 32) + (threadIdx.x >> 5);
    if (w < nsmall) unique_small_segment(segs[small[w]], &counts[small[w]]);
    return;
  }
  __shared__ uint32_t s_scan[kBlock / 32 + 1];
  __shared__ uint64_t s_b;
  __shared__ uint32_t s_tile;
  __shared__ SegRows s_seg;
  __shared__ uint32_t s_s;
  __shared__ uint32_t s_keep[2 * kTileRows];   // compact_store: two columns at a time
  if (threadIdx.x == 0) {
    s_tile = atomicAdd(ticket, 1u);
    s_s = tile_seg[s_tile];
    s_seg = segs[s_s];
  }
  __syncthreads();
  const uint64_t tile = s_tile;
  const uint32_t s = s_s;
  const uint64_t n = s_seg.n;
  const uint32_t ncols = s_seg.ncols;
  const uint64_t r0 = (tile - tstart[s]) * kTileRows + threadIdx.x * kRows;
  uint32_t diff = (r0 == 0) ? 1u : 0u;
  for (uint32_t c = 0; c < ncols; ++c) diff |= unique_diff_bits(s_seg.in[c], n, r0);
  if (r0 >= n) diff = 0;
  else if (n - r0 < kRows) diff &= (1u << (n - r0)) - 1u;
  uint32_t tot;
  const uint32_t e = block_excl_scan<kBlock>(__popc(diff), tot, s_scan);
  if (threadIdx.x < 32) {
    const uint64_t p = warp_lookback_seg(status, tile, tstart[s], tot, err);
    if (threadIdx.x == 0) s_b = p;
  }
  __syncthreads();
  const uint64_t g = s_b;
  if (tile == tstart[s + 1] - 1 && threadIdx.x == 0) counts[s] = g + tot;
  compact_store<kBlock>(s_seg.in, s_seg.out, ncols, n, r0, diff, e, tot, g, s_keep);
}

// ---------------------------------------------------------------------------
// Rows [r0, r0 + kBlock) of a grid-stride loop over segmented rows: the
// block finds the segments of its first and last row once (two searches of
// the segment starts), then each row searches only between those, which is
// usually one or two segments.
__device__ __forceinline__ uint32_t seg_of_row(const uint64_t* __restrict__ rstart, uint32_t k0, uint32_t k1,
                                               uint64_t r) {
  uint32_t lo = k0, hi = k1;   // last k in [k0, k1] with rstart[k] <= r
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (rstart[mid] <= r) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Segmented row loops: blocks take chunks of kChunkRows consecutive rows
// (each thread kRows of them, kBlock apart, so loads and stores coalesce);
// a chunk's first segment comes from a table made on the host and the next
// chunk's bounds its last, so each row searches only between those two
// (usually one segment).
constexpr uint32_t kChunkRows = kBlock * kRows;

__device__ __forceinline__ void chunk_segments(const uint32_t* __restrict__ chunk_seg, uint64_t nchunks,
                                               uint32_t S, uint64_t c, uint32_t& k0, uint32_t& k1) {
  k0 = chunk_seg[c];
  k1 = c + 1 < nchunks ? chunk_seg[c + 1] : S - 1;
}

// (segment, key) composite sort keys: the segment sits above the key's
// key_bits bits, so one sort orders rows by segment and, within it, by key.
__global__ void __launch_bounds__(kBlock) composite_keys_kernel(const uint32_t* const* __restrict__ col0,
                                                                const uint64_t* __restrict__ rstart, uint32_t S,
                                                                const uint32_t* __restrict__ chunk_seg,
                                                                uint64_t nchunks, uint32_t key_bits,
                                                                uint64_t* __restrict__ keys) {
  const uint64_t total = rstart[S];
  for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    uint32_t k0, k1;
    chunk_segments(chunk_seg, nchunks, S, c, k0, k1);
#pragma unroll
    for (int it = 0; it < kRows; ++it) {
      const uint64_t r = c * kChunkRows + static_cast<uint64_t>(it) * kBlock + threadIdx.x;
      if (r < total) {
        const uint32_t s = seg_of_row(rstart, k0, k1, r);
        keys[r] = (static_cast<uint64_t>(s) << key_bits) | __ldg(col0[s] + (r - rstart[s]));
      }
    }
  }
}

__global__ void __launch_bounds__(kBlock) seg_gather_kernel(const SegRows* __restrict__ segs,
                                                            const uint64_t* __restrict__ rstart, uint32_t S,
                                                            const uint32_t* __restrict__ chunk_seg,
                                                            uint64_t nchunks, const uint32_t* __restrict__ perm) {
  const uint64_t total = rstart[S];
  for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    uint32_t k0, k1;
    chunk_segments(chunk_seg, nchunks, S, c, k0, k1);
#pragma unroll 2
    for (int it = 0; it < kRows; ++it) {
      const uint64_t r = c * kChunkRows + static_cast<uint64_t>(it) * kBlock + threadIdx.x;
      if (r < total) {
        const uint32_t s = seg_of_row(rstart, k0, k1, r);
        const uint64_t base = rstart[s];
        const SegRows& g = segs[s];
        copy_row(g.out, g.in, g.ncols, perm[r] - base, r - base);
      }
    }
  }
}

// ---------------------------------------------------------------------------
struct JoinSeg {
  const uint32_t* lk;
  const uint32_t* rk;
  uint64_t nl, nr;
  uint64_t row0;   // offset of this join's left rows in the lo/cnt/offs arrays
};

// One block per tile of kJcTile left keys of one join, tiles taken in ticket
// order (the tile's join from a per-tile table, one load instead of a search
// of the join starts).  The tile's match counts stay in registers (the
// right-key window, found beforehand by jc_window_kernel, is staged by a bulk
// copy when it fits); their block scan
// and a segmented decoupled look-back over the join's earlier tiles give
// every left key its output offset directly, and the join's last tile writes
// its total.
//
// Joins with at most kSmallJoin left rows (most joins of a wave have a few)
// take one warp each instead: the first small_blocks blocks hold
// kJcBlock / 32 such joins, one per warp.  The warp finds the join's window
// of right keys with two 32-ary searches, each lane counts the matches of
// its kJcKeys keys with lockstep searches in that window, and a warp scan
// gives the offsets and the total (no shared memory, no look-back).
constexpr uint32_t kSmallJoin = 32 * kJcKeys;

__device__ __forceinline__ void count_small_join(const JoinSeg& g, uint32_t* __restrict__ lo,
                                                 uint64_t* __restrict__ offs, uint64_t* total) {
  const uint32_t lane = lane_id();
  const uint64_t nl = g.nl;
  const uint64_t w0 = warp_bound<false, uint32_t>(g.rk, 0, g.nr, g.lk[0]);
  const uint64_t w1 = warp_bound<true, uint32_t>(g.rk, w0, g.nr, g.lk[nl - 1]);
  const uint64_t first = static_cast<uint64_t>(lane) * kJcKeys;
  uint32_t key[kJcKeys];
  uint32_t lb[kJcKeys], ub[kJcKeys];
#pragma unroll
  for (int q = 0; q < kJcKeys; ++q) key[q] = g.lk[first + q < nl ? first + q : nl - 1];
  lockstep_bounds32<kJcKeys>(g.rk, static_cast<uint32_t>(w0), static_cast<uint32_t>(w1), key, lb, ub);
  uint64_t sum = 0;
#pragma unroll
  for (int q = 0; q < kJcKeys; ++q)
    if (first + q < nl) sum += ub[q] - lb[q];
  const uint64_t incl = warp_incl_scan64(sum);
  uint64_t run = incl - sum;
#pragma unroll
  for (int q = 0; q < kJcKeys; ++q)
    if (first + q < nl) {
      lo[g.row0 + first + q] = static_cast<uint32_t>(lb[q]);
      offs[g.row0 + first + q] = run;
      run += ub[q] - lb[q];
    }
  if (lane == 31) *total = incl;
}

// Every tile's right-key window [win.x, win.y) (one warp per tile, both ends
// at once), so that the counting blocks start their bulk copies at once
// instead of each searching the right keys first.
__global__ void __launch_bounds__(kJcBlock) jc_window_kernel(const JoinSeg* __restrict__ js,
                                                             const uint64_t* __restrict__ bstart,
                                                             const uint32_t* __restrict__ tile_join, uint64_t T,
                                                             uint2* __restrict__ win) {
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * (kJcBlock / 32);
  for (uint64_t t = static_cast<uint64_t>(blockIdx.x) * (kJcBlock / 32) + (threadIdx.x >> 5); t < T; t += nw) {
    const uint32_t j = tile_join[t];
    const uint64_t nl = js[j].nl;
    const uint32_t* lk = js[j].lk;
    const uint64_t i0 = (t - bstart[j]) * static_cast<uint64_t>(kJcTile);
    const uint64_t i1 = (i0 + kJcTile < nl ? i0 + kJcTile : nl) - 1;
    uint64_t w0, w1;
    warp_window(js[j].rk, js[j].nr, lk[i0], lk[i1], w0, w1);
    if ((threadIdx.x & 31) == 0) win[t] = make_uint2(static_cast<uint32_t>(w0), static_cast<uint32_t>(w1));
  }
}

__global__ void __launch_bounds__(kJcBlock, 4) bjoin_count_scan_kernel(
    const JoinSeg* __restrict__ js, const uint64_t* __restrict__ bstart, const uint32_t* __restrict__ tile_join,
    const uint2* __restrict__ win, const uint32_t* __restrict__ small, uint32_t nsmall, uint32_t small_blocks,
    uint32_t* __restrict__ lo, uint64_t* __restrict__ offs, uint64_t* status, uint32_t* ticket,
    uint64_t* __restrict__ totals, DeviceErrors* err) {
  if (blockIdx.x < small_blocks) {   // block-uniform: this block only counts small joins
    const uint64_t sj = static_cast<uint64_t>(blockIdx.x) * (kJcBlock / 32) + (threadIdx.x >> 5);
    if (sj < nsmall) {
      const uint32_t j = small[sj];
      count_small_join(js[j], lo, offs, &totals[j]);
    }
    return;
  }
  __shared__ JoinCountSmem sm;
  __shared__ uint64_t s_scan[kJcBlock / 32 + 1];
  __shared__ uint64_t s_b;
  __shared__ uint32_t s_tile, s_j;
  if (threadIdx.x == 0) {
    // the window is known: its bulk copy starts before the block's first barrier
    const uint32_t t = atomicAdd(ticket, 1u);
    const uint32_t jj = tile_join[t];
    const uint2 w = win[t];
    s_tile = t;
    s_j = jj;
    jc_issue_window(js[jj].rk, w.x, w.y, sm);
  }
  __syncthreads();
  const uint64_t tile = s_tile;
  const uint32_t j = s_j;
  const JoinSeg g = js[j];
  const uint64_t i0 = (tile - bstart[j]) * static_cast<uint64_t>(kJcTile);
  uint32_t cnt[kJcKeys], lov[kJcKeys];
  jc_count_staged(g.lk, g.nl, g.rk, i0, lov, cnt, sm, err);
  uint64_t sum = 0;
#pragma unroll
  for (int k = 0; k < kJcKeys; ++k) sum += cnt[k];
  uint64_t tot;
  const uint64_t e = block_excl_scan64<kJcBlock>(sum, tot, s_scan);   // every thread is past its search
  const uint32_t tid = threadIdx.x;
  const uint64_t first = i0 + static_cast<uint64_t>(tid) * kJcKeys;
  const uint32_t tile_n = static_cast<uint32_t>(g.nl - i0 < kJcTile ? g.nl - i0 : kJcTile);
  // a bulk copy that gave up may still land in the window: no staging there
  const bool stage = !(sm.staged == 2 && sm.failed);
  if (stage) {
    // lower bounds and tile-relative offsets staged in the window while warp 0
    // looks back; the tile's prefix is added when they are stored
    uint32_t* s_lo = jc_stage_lo(sm);
    uint64_t* s_off = jc_stage_off(sm);
    uint64_t run = e;
#pragma unroll
    for (int k = 0; k < kJcKeys; ++k) {
      const uint32_t q = tid * kJcKeys + k;
      s_lo[q + q / 32] = lov[k];
      s_off[q + q / 16] = run;
      run += cnt[k];
    }
  }
  if (threadIdx.x < 32) {
    const uint64_t p = warp_lookback_seg(status, tile, bstart[j], tot, err);
    if (threadIdx.x == 0) s_b = p;
  }
  __syncthreads();
  const uint64_t base = s_b;
  if (tile == bstart[j + 1] - 1 && tid == 0) totals[j] = base + tot;
  if (!stage) {
    uint64_t run = base + e;
#pragma unroll
    for (int k = 0; k < kJcKeys; ++k) {
      if (first + k < g.nl) {
        offs[g.row0 + first + k] = run;
        lo[g.row0 + first + k] = lov[k];
      }
      run += cnt[k];
    }
    if (tid == 0) jc_drain_window(sm, err);
    return;
  }
  const uint32_t* s_lo = jc_stage_lo(sm);
  const uint64_t* s_off = jc_stage_off(sm);
  uint32_t* lo_t = lo + g.row0 + i0;
  uint64_t* off_t = offs + g.row0 + i0;
  for (uint32_t q = tid; q < tile_n; q += kJcBlock) {
    lo_t[q] = s_lo[q + q / 32];
    off_t[q] = base + s_off[q + q / 16];
  }
}

struct JoinOut {
  const uint64_t* offs;
  const uint32_t* lo;
  uint64_t nl, total;
  const uint32_t* lc[VG_MAX_COLS];
  const uint32_t* rc[VG_MAX_COLS];
  uint32_t* oc[VG_MAX_COLS];
  uint32_t nlc, nrc;
};

// Output rows [kb, kb + kTileRows) of one join per tile (the tile's join
// from a per-tile table).  Blocks loop over tiles [blockIdx.x, T) with
// stride gridDim.x; T is read from the device when ostart_end is given (a
// device-side placement wrote it there).  Output row k comes from the left
// row i with offs[i] <= k < offs[i + 1] and the right row lo[i] + (k -
// offs[i]).  Two warps find the tile's left-row range at once; when it holds
// at most kTileRows + 1 rows, its offsets and lower bounds are staged in
// shared memory, and each thread walks its rows (k increasing, consecutive
// threads on consecutive rows, so loads and stores coalesce) from the
// previous one's left row.  Hub keys thus spread over many blocks.
//
// Small outputs (at most Ctx::tune.write_small_rows rows of a join with at most kSmallJoin
// left rows; most outputs of a wave) are written one join per warp first,
// before the tiles: the warp stages the join's offsets and lower bounds in
// its own slice of the shared arrays and each lane writes every 32nd row.
// Their list (small, nsmall of them; nsmall_dev when on the device) holds no
// tiles.

__device__ __forceinline__ void write_small_join(const JoinOut* __restrict__ src, JoinOut* jp, uint64_t* s_off,
                                                 uint32_t* s_lo) {
  const uint32_t lane = lane_id();
  // the join's description in the warp's shared slot: the row loop reads its
  // column pointers from shared memory
  {
    const uint32_t* a = reinterpret_cast<const uint32_t*>(src);
    uint32_t* b = reinterpret_cast<uint32_t*>(jp);
    for (uint32_t w = lane; w < sizeof(JoinOut) / 4; w += 32) b[w] = a[w];
    __syncwarp();
  }
  const uint64_t total = jp->total, nl = jp->nl;
  const uint64_t* offs = jp->offs;
  const uint32_t* lov = jp->lo;
  for (uint32_t e = lane; e < nl; e += 32) {
    s_off[e] = offs[e];
    s_lo[e] = lov[e];
  }
  __syncwarp();
  const uint32_t nlc = jp->nlc, nrc = jp->nrc;
  for (uint64_t k = lane; k < total; k += 32) {
    uint32_t a = 0, b = static_cast<uint32_t>(nl);   // last p with s_off[p] <= k
    while (b - a > 1) {
      const uint32_t mid = (a + b) >> 1;
      if (s_off[mid] <= k) a = mid;
      else b = mid;
    }
    const uint64_t jj = s_lo[a] + (k - s_off[a]);
    copy_join_row(jp->oc, jp->lc, nlc, jp->rc, nrc, a, jj, k);
  }
  __syncwarp();   // the slice is free for the warp's next join
}

// Every output tile's left rows [x, y): x the last row whose output starts
// at or before the tile's first row, y the first row whose output starts
// after its last (one warp per tile, both searches at once), so that the
// writing blocks start staging at once.  T as for bjoin_write_kernel.
__global__ void __launch_bounds__(kBlock) jw_range_kernel(const JoinOut* __restrict__ jo,
                                                          const uint64_t* __restrict__ ostart,
                                                          const uint32_t* __restrict__ tile_join, uint64_t T_host,
                                                          const uint64_t* ostart_end, uint2* __restrict__ ranges) {
  const uint64_t T = ostart_end ? *ostart_end : T_host;
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * (kBlock / 32);
  for (uint64_t t = static_cast<uint64_t>(blockIdx.x) * (kBlock / 32) + (threadIdx.x >> 5); t < T; t += nw) {
    const uint32_t jn = tile_join[t];
    const uint64_t total = jo[jn].total, nl = jo[jn].nl;
    const uint64_t kb = (t - ostart[jn]) * static_cast<uint64_t>(kTileRows);
    const uint64_t kend = (kb + kTileRows < total) ? kb + kTileRows : total;
    uint64_t a, b;
    warp_bound_pair<true, true, uint64_t>(jo[jn].offs, nl, kb, kend - 1, a, b);
    if ((threadIdx.x & 31) == 0) ranges[t] = make_uint2(static_cast<uint32_t>(a - 1), static_cast<uint32_t>(b));
  }
}

__global__ void __launch_bounds__(kBlock, 5) bjoin_write_kernel(const JoinOut* __restrict__ jo,
                                                             const uint64_t* __restrict__ ostart,
                                                             const uint32_t* __restrict__ tile_join,
                                                             const uint2* __restrict__ ranges,
                                                             uint64_t T_host, const uint64_t* ostart_end,
                                                             const uint32_t* __restrict__ small, uint32_t nsmall_host,
                                                             const uint32_t* nsmall_dev) {
  constexpr int kStage = kTileRows + 1;
  static_assert(kStage >= (kBlock / 32) * kSmallJoin, "a warp's slice holds a small join's left rows");
  __shared__ JoinOut s_o;
  __shared__ JoinOut s_w[kBlock / 32];
  __shared__ uint64_t s_off[kStage];
  __shared__ uint32_t s_lo[kStage];
  {
    const uint32_t nsm = nsmall_dev ? *nsmall_dev : nsmall_host;
    const uint32_t warp = threadIdx.x >> 5, nwarps = kBlock / 32;
    for (uint64_t w = static_cast<uint64_t>(blockIdx.x) * nwarps + warp; w < nsm;
         w += static_cast<uint64_t>(gridDim.x) * nwarps)
      write_small_join(&jo[small[w]], &s_w[warp], s_off + warp * kSmallJoin, s_lo + warp * kSmallJoin);
  }
  const uint64_t T = ostart_end ? *ostart_end : T_host;
#pragma unroll 1
  for (uint64_t tile = blockIdx.x; tile < T; tile += gridDim.x) {
    __syncthreads();   // the previous tile's readers of the shared arrays are done
    const uint32_t jn = tile_join[tile];
    const uint2 rg = ranges[tile];
    const uint64_t tile0 = ostart[jn];
    {
      const uint32_t* src = reinterpret_cast<const uint32_t*>(&jo[jn]);
      uint32_t* dst = reinterpret_cast<uint32_t*>(&s_o);
      for (uint32_t w = threadIdx.x; w < sizeof(JoinOut) / 4; w += kBlock) dst[w] = src[w];
    }
    __syncthreads();
    const uint64_t kb = (tile - tile0) * static_cast<uint64_t>(kTileRows);
    const uint64_t kend = (kb + kTileRows < s_o.total) ? kb + kTileRows : s_o.total;
    const uint64_t ib = rg.x, ie = rg.y;
    const uint64_t m = ie - ib;
    const bool staged = m <= static_cast<uint64_t>(kStage);
    if (staged)
      for (uint32_t e = threadIdx.x; e < m; e += kBlock) {
        s_off[e] = s_o.offs[ib + e];
        s_lo[e] = s_o.lo[ib + e];
      }
    __syncthreads();
    // 1. the left and right row of each of the thread's output rows
    uint32_t li[kRows], ri[kRows];
    if (staged) {
      uint32_t p = 0;   // the current left row, relative to ib
#pragma unroll
      for (int it = 0; it < kRows; ++it) {
        const uint64_t k = kb + static_cast<uint64_t>(it) * kBlock + threadIdx.x;
        li[it] = ri[it] = 0;
        if (k < kend) {
          // last p with s_off[p] <= k, moving forward from the previous row's p
          uint32_t step = 1;
          while (p + step < m && s_off[p + step] <= k) {
            p += step;
            step <<= 1;
          }
          while (step > 1) {
            step >>= 1;
            if (p + step < m && s_off[p + step] <= k) p += step;
          }
          li[it] = static_cast<uint32_t>(ib + p);
          ri[it] = static_cast<uint32_t>(s_lo[p] + (k - s_off[p]));
        }
      }
    } else {
      // a sparse tile (more than kStage left rows, most without matches): the
      // left rows of kGroup of the thread's output rows at a time come from
      // kGroup binary searches of the offsets advanced in lockstep, so each
      // round has kGroup independent loads in flight
      constexpr int kGroup = 4;
#pragma unroll
      for (int g0 = 0; g0 < kRows; g0 += kGroup) {
        uint64_t lq[kGroup], kk[kGroup];
#pragma unroll
        for (int q = 0; q < kGroup; ++q) {
          const uint64_t k = kb + static_cast<uint64_t>(g0 + q) * kBlock + threadIdx.x;
          kk[q] = k < kend ? k : kend - 1;
          lq[q] = ib;
        }
        uint64_t n = ie - ib;                     // last i in [ib, ie) with offs[i] <= k
        while (n > 1) {
          const uint64_t half = n >> 1;
#pragma unroll
          for (int q = 0; q < kGroup; ++q) lq[q] = (s_o.offs[lq[q] + half] <= kk[q]) ? lq[q] + half : lq[q];
          n -= half;
        }
#pragma unroll
        for (int q = 0; q < kGroup; ++q) {
          li[g0 + q] = static_cast<uint32_t>(lq[q]);
          ri[g0 + q] = static_cast<uint32_t>(s_o.lo[lq[q]] + (kk[q] - s_o.offs[lq[q]]));
        }
      }
    }
    // 2. column by column: each thread's kRows loads of a column are in
    // flight together (read-only path), each store instruction writes
    // consecutive rows, and one column's pointers are live at a time
    const uint32_t nlc = s_o.nlc, ncols = s_o.nlc + s_o.nrc;
    for (uint32_t c = 0; c < ncols; ++c) {
      const bool left = c < nlc;
      const uint32_t* src = left ? s_o.lc[c] : s_o.rc[c - nlc];
      uint32_t* dst = s_o.oc[c];
      uint32_t v[kRows];
#pragma unroll
      for (int it = 0; it < kRows; ++it) {
        const uint64_t k = kb + static_cast<uint64_t>(it) * kBlock + threadIdx.x;
        if (k < kend) v[it] = __ldg(src + (left ? li[it] : ri[it]));
      }
#pragma unroll
      for (int it = 0; it < kRows; ++it) {
        const uint64_t k = kb + static_cast<uint64_t>(it) * kBlock + threadIdx.x;
        if (k < kend) dst[k] = v[it];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Device-side placement of a wave's join outputs in a region (no host round
// trip between the count and the write).  One block: every join's output
// size comes from its count, each column is rounded up to 256 bytes, and the
// outputs are laid out back to back after the bytes the region handed out in
// earlier waves (*bump).  A join whose output does not fit is left unplaced
// (total 0, no columns; the host writes it itself); the offsets only grow,
// so every later join with rows is unplaced too.  The same arithmetic on the
// host (place_outputs_on_host) reproduces every placement from the totals.
constexpr int kPlaceBlock = 1024;

__host__ __device__ inline uint64_t place_stride(uint64_t rows) { return (rows * 4 + 255) / 256 * 256; }

struct JoinPlace {
  char* base;            // the region
  uint64_t cap;          // its bytes
  uint64_t* bump;        // bytes handed out before this wave (updated)
  uint64_t* ostart;      // J + 1 output-tile starts (written; small outputs have no tiles)
  uint32_t* small;       // joins whose outputs are written one per warp (written)
  uint32_t* nsmall;      // their number (written)
  uint32_t small_rows;   // outputs of at most this many rows are small
};

__global__ void __launch_bounds__(kPlaceBlock) join_place_kernel(JoinOut* __restrict__ jo,
                                                                 const uint64_t* __restrict__ totals, uint32_t J,
                                                                 JoinPlace pl) {
  __shared__ uint64_t s_scan[kPlaceBlock / 32 + 1];
  const uint64_t bump0 = *pl.bump;
  uint64_t carry_b = 0, carry_t = 0, carry_s = 0, fit_b = 0;
  for (uint32_t c0 = 0; c0 < J; c0 += kPlaceBlock) {
    const uint32_t j = c0 + threadIdx.x;
    const uint64_t t = j < J ? totals[j] : 0;
    const uint32_t ncols = j < J ? jo[j].nlc + jo[j].nrc : 0;
    const uint64_t stride = place_stride(t);
    const uint64_t bytes = t ? ncols * stride : 0;
    uint64_t tot_b, tot_t, fb_sum;
    const uint64_t eb = block_excl_scan64<kPlaceBlock>(bytes, tot_b, s_scan);
    const uint64_t off = bump0 + carry_b + eb;
    const bool fits = off + bytes <= pl.cap;
    const bool is_small = fits && t > 0 && t <= pl.small_rows && j < J && jo[j].nl <= kSmallJoin;
    const uint64_t tiles = (fits && t && !is_small) ? div_up(t, kTileRows) : 0;
    const uint64_t et = block_excl_scan64<kPlaceBlock>(tiles, tot_t, s_scan);
    (void)block_excl_scan64<kPlaceBlock>(fits ? bytes : 0, fb_sum, s_scan);
    uint64_t tot_s;
    const uint64_t es = block_excl_scan64<kPlaceBlock>(is_small ? 1 : 0, tot_s, s_scan);
    if (j < J) {
      JoinOut& o = jo[j];
      o.total = fits ? t : 0;
      for (uint32_t c = 0; c < VG_MAX_COLS; ++c)
        o.oc[c] = (fits && t && c < ncols) ? reinterpret_cast<uint32_t*>(pl.base + off + c * stride) : nullptr;
      pl.ostart[j] = carry_t + et;
      if (is_small) pl.small[carry_s + es] = j;
    }
    carry_b += tot_b;
    carry_t += tot_t;
    carry_s += tot_s;
    fit_b += fb_sum;
  }
  if (threadIdx.x == 0) {
    pl.ostart[J] = carry_t;
    *pl.nsmall = static_cast<uint32_t>(carry_s);
    *pl.bump = bump0 + fit_b;
  }
}

// tile_join[ostart[j] .. ostart[j + 1]) = j.
__global__ void tile_join_fill_kernel(const uint64_t* __restrict__ ostart, uint32_t J,
                                      uint32_t* __restrict__ tile_join) {
  for (uint32_t j = blockIdx.x; j < J; j += gridDim.x)
    for (uint64_t t = ostart[j] + threadIdx.x; t < ostart[j + 1]; t += blockDim.x) tile_join[t] = j;
}

// After a placed write, one warp per join: lane 0 writes the output's first
// and last key; when the join has a stage slot (its host-side completion
// scans column 0 for empty intervals) and a small output (2 < rows <
// kSmallC0Words), the warp copies that column 0 into the slot's
// kSmallC0Words-word stage.
__global__ void __launch_bounds__(kBlock) join_edges_kernel(const JoinOut* __restrict__ jo, uint32_t J,
                                                            uint32_t* __restrict__ fl,
                                                            const int32_t* __restrict__ slot,
                                                            uint32_t* __restrict__ stage) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nw = static_cast<uint64_t>(gridDim.x) * (kBlock / 32);
  for (uint64_t j = static_cast<uint64_t>(blockIdx.x) * (kBlock / 32) + (threadIdx.x >> 5); j < J; j += nw) {
    const uint64_t t = jo[j].total;
    if (t == 0) continue;
    const uint32_t* c0 = jo[j].oc[0];
    if (lane == 0) {
      fl[2 * j] = c0[0];
      fl[2 * j + 1] = c0[t - 1];
    }
    const int32_t sl = slot ? slot[j] : -1;
    if (sl < 0 || t <= 2 || t >= kSmallC0Words) continue;
    for (uint32_t i = lane; i < t; i += 32) stage[static_cast<uint64_t>(sl) * kSmallC0Words + i] = c0[i];
  }
}

__global__ void first_last_kernel(const JoinOut* __restrict__ jo, uint32_t J, uint32_t* __restrict__ fl) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= J) return;
  const JoinOut& o = jo[j];
  if (o.total == 0) return;
  fl[2 * j] = o.oc[0][0];
  fl[2 * j + 1] = o.oc[0][o.total - 1];
}

struct Col0Req {
  const uint32_t* src;
  uint64_t n;
  uint64_t dst;
};

__global__ void col0_kernel(const Col0Req* __restrict__ rq, uint32_t R, uint32_t* __restrict__ out) {
  for (uint32_t q = blockIdx.x; q < R; q += gridDim.x)
    for (uint64_t i = threadIdx.x; i < rq[q].n; i += blockDim.x) out[rq[q].dst + i] = rq[q].src[i];
}

int bits_for_segments(uint32_t S) {
  int b = 0;
  while ((1ull << b) < S) ++b;
  return b;
}

}  // namespace

void batched_copy(Ctx& ctx, const std::vector<CopyPiece>& pieces) {
  std::vector<CopyPiece> p;
  std::vector<uint64_t> cstart(1, 0);
  double bytes = 0;
  for (const CopyPiece& pc : pieces) {
    if (pc.len == 0) continue;
    const uint64_t head = (4 - ((reinterpret_cast<uintptr_t>(pc.dst) >> 2) & 3)) & 3;
    const uint64_t h = head < pc.len ? head : pc.len;
    const uint64_t chunks = (pc.len - h) / 4;
    p.push_back(pc);
    cstart.push_back(cstart.back() + (chunks ? chunks : 1));
    bytes += 8.0 * pc.len;
  }
  if (p.empty()) return;
  const uint32_t P = static_cast<uint32_t>(p.size());
  // each tile's first piece
  const uint64_t ntiles = div_up(cstart.back(), kCopyTile);
  std::vector<uint32_t> tile_piece(ntiles);
  {
    uint32_t k = 0;
    for (uint64_t t = 0; t < ntiles; ++t) {
      const uint64_t q = t * kCopyTile;
      while (cstart[k + 1] <= q) ++k;
      tile_piece[t] = k;
    }
  }
  CopyPiece* dp = upload(ctx, p);
  uint64_t* dc = upload(ctx, cstart);
  uint32_t* dtp = upload(ctx, tile_piece);
  ctx.launch("select_copy", bytes, [&] {
    bcopy_kernel<<<grid_cap(ctx, cstart.back(), kCopyPer), kBlock, 0, ctx.stream>>>(dp, dc, P, dtp, ntiles);
  });
  VG_CUDA(cudaGetLastError());
  ctx.free(dp);
  ctx.free(dc);
  ctx.free(dtp);
}

void batched_unique_enqueue(Ctx& ctx, const std::vector<SegRows>& segs, uint64_t* counts_host) {
  const uint32_t S = static_cast<uint32_t>(segs.size());
  if (S == 0) return;
  std::vector<uint64_t> tstart(S + 1, 0);
  std::vector<uint32_t> small;
  double bytes = 0;
  for (uint32_t s = 0; s < S; ++s) {
    const bool is_small = segs[s].n > 0 && segs[s].n <= std::min<uint32_t>(kSmallSeg, ctx.tune.unique_small_rows);
    if (is_small) small.push_back(s);
    tstart[s + 1] = tstart[s] + (is_small ? 0 : div_up(segs[s].n, kTileRows));
    bytes += 4.0 * segs[s].n * segs[s].ncols;
  }
  const uint64_t tiles = tstart[S];
  const uint32_t nsmall = static_cast<uint32_t>(small.size());
  const uint32_t small_blocks = static_cast<uint32_t>(div_up(nsmall, kBlock / 32));
  if (tiles == 0 && nsmall == 0) {
    for (uint32_t s = 0; s < S; ++s) counts_host[s] = 0;
    return;
  }
  std::vector<uint32_t> tile_seg(tiles);
  for (uint32_t s = 0; s < S; ++s)
    for (uint64_t t = tstart[s]; t < tstart[s + 1]; ++t) tile_seg[t] = s;
  SegRows* ds = upload(ctx, segs);
  uint64_t* dt = upload(ctx, tstart);
  uint32_t* dts = upload(ctx, tile_seg);
  uint32_t* dsm = upload(ctx, small);
  Scratch<uint64_t> status(ctx, tiles), dcount(ctx, S);
  Scratch<uint32_t> ticket(ctx, 1);
  VG_CUDA(cudaMemsetAsync(status.get(), 0, tiles * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(dcount.get(), 0, S * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(uint32_t), ctx.stream));
  ctx.launch("unique_compact", bytes, [&] {
    bunique_kernel<<<static_cast<unsigned>(small_blocks + tiles), kBlock, 0, ctx.stream>>>(
        ds, dt, dts, dsm, nsmall, small_blocks, status.get(), ticket.get(), dcount.get(), ctx.d_err);
  });
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaMemcpyAsync(counts_host, dcount.get(), S * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.free(ds);
  ctx.free(dt);
  ctx.free(dts);
  ctx.free(dsm);
}

void note_unique_writes(Ctx& ctx, const std::vector<SegRows>& segs, const uint64_t* counts) {
  double wb = 0;
  for (size_t s = 0; s < segs.size(); ++s) wb += 4.0 * counts[s] * segs[s].ncols;
  ctx.add_bytes("unique_compact", wb);
}

std::vector<uint64_t> batched_unique(Ctx& ctx, const std::vector<SegRows>& segs) {
  std::vector<uint64_t> counts(segs.size(), 0);
  if (segs.empty()) return counts;
  PinnedWords h(ctx);
  batched_unique_enqueue(ctx, segs, h.reserve(segs.size()));
  ctx.sync();
  std::copy(h.data(), h.data() + segs.size(), counts.begin());
  note_unique_writes(ctx, segs, counts.data());
  return counts;
}

void batched_sort_by_first(Ctx& ctx, const std::vector<Rel*>& rels_in, int key_bits) {
  std::vector<Rel*> rels;
  for (Rel* r : rels_in)
    if (r->nrows > 1 && r->ncols > 0) rels.push_back(r);
  const uint32_t S = static_cast<uint32_t>(rels.size());
  if (S == 0) return;
  std::vector<uint64_t> rstart(S + 1, 0);
  std::vector<const uint32_t*> col0(S);
  for (uint32_t s = 0; s < S; ++s) {
    rstart[s + 1] = rstart[s] + rels[s]->nrows;
    col0[s] = rels[s]->cols[0];
  }
  const uint64_t N = rstart[S];
  if (N > 0xFFFFFFFFull) fail(VG_ERR_OVERFLOW, "batched sort is limited to 2^32 rows");
  const bool known = key_bits > 0 && key_bits <= 32;
  const int kb = known ? key_bits : 32;
  uint64_t* drs = upload(ctx, rstart);
  const uint32_t** dc0 = upload(ctx, col0);
  // each chunk's first segment
  const uint64_t nchunks = div_up(N, static_cast<uint64_t>(kChunkRows));
  std::vector<uint32_t> chunk_seg(nchunks);
  {
    uint32_t sg = 0;
    for (uint64_t c = 0; c < nchunks; ++c) {
      const uint64_t r = c * kChunkRows;
      while (rstart[sg + 1] <= r) ++sg;
      chunk_seg[c] = sg;
    }
  }
  uint32_t* dcs = upload(ctx, chunk_seg);
  const unsigned cgrid = static_cast<unsigned>(std::min<uint64_t>(nchunks, static_cast<uint64_t>(ctx.num_sms) * 8));
  uint64_t* keys = ctx.alloc<uint64_t>(N);
  uint64_t* keys_alt = ctx.alloc<uint64_t>(N);
  uint32_t* vals = ctx.alloc<uint32_t>(N);
  uint32_t* vals_alt = ctx.alloc<uint32_t>(N);
  ctx.launch("sort_keys", 12.0 * N, [&] {
    composite_keys_kernel<<<cgrid, kBlock, 0, ctx.stream>>>(dc0, drs, S, dcs, nchunks, static_cast<uint32_t>(kb),
                                                            keys);
  });
  VG_CUDA(cudaGetLastError());
  // with the key width known the passes are fixed and nothing waits on the device
  const bool alt = radix_sort_u64(ctx, keys, keys_alt, vals, vals_alt, N, kb + bits_for_segments(S), true, !known);
  uint32_t* perm = alt ? vals_alt : vals;
  ctx.free(keys);
  ctx.free(keys_alt);
  std::vector<SegRows> segs(S);
  double bytes = 4.0 * N;
  for (uint32_t s = 0; s < S; ++s) bytes += 8.0 * rels[s]->nrows * rels[s]->ncols;
  parallel_for(S, [&](size_t s) {
    segs[s].ncols = rels[s]->ncols;
    segs[s].n = rels[s]->nrows;
    for (uint32_t c = 0; c < rels[s]->ncols; ++c) {
      segs[s].in[c] = rels[s]->cols[c];
      segs[s].out[c] = ctx.alloc<uint32_t>(rels[s]->nrows);
    }
  });
  SegRows* dsg = upload(ctx, segs);
  ctx.launch("gather", bytes, [&] {
    seg_gather_kernel<<<cgrid, kBlock, 0, ctx.stream>>>(dsg, drs, S, dcs, nchunks, perm);
  });
  VG_CUDA(cudaGetLastError());
  parallel_for(S, [&](size_t s) {
    for (uint32_t c = 0; c < rels[s]->ncols; ++c) {
      rel_drop_col(ctx, *rels[s], c);
      rels[s]->cols[c] = segs[s].out[c];
    }
  });
  ctx.free(vals);
  ctx.free(vals_alt);
  ctx.free(dsg);
  ctx.free(drs);
  ctx.free(dcs);
  ctx.free(const_cast<uint32_t**>(dc0));
}

void batched_join_count(Ctx& ctx, const std::vector<const Rel*>& l, const std::vector<const Rel*>& r, JoinBatch& jb,
                        uint64_t* totals_host) {
  const uint32_t J = static_cast<uint32_t>(l.size());
  jb = JoinBatch();
  jb.J = J;
  jb.l = l;
  jb.r = r;
  if (J == 0) return;
  std::vector<JoinSeg> js(J);
  std::vector<uint64_t> bstart(J + 1, 0);
  uint64_t rows = 0;
  double cbytes = 0;
  jb.row0.resize(J);
  std::vector<uint32_t> small;   // joins counted by one warp each
  for (uint32_t j = 0; j < J; ++j) {
    if (l[j]->nrows == 0 || r[j]->nrows == 0) fail(VG_ERR_INVALID, "batched join of an empty relation");
    if (l[j]->nrows > 0xFFFFFFFFull || r[j]->nrows > 0xFFFFFFFFull)
      fail(VG_ERR_OVERFLOW, "join inputs are limited to 2^32 rows");
    if (l[j]->ncols + r[j]->ncols - 1 > VG_MAX_COLS) fail(VG_ERR_UNSUPPORTED, "join output has more than 9 columns");
    js[j] = {l[j]->cols[0], r[j]->cols[0], l[j]->nrows, r[j]->nrows, rows};
    jb.row0[j] = rows;
    rows += l[j]->nrows;
    const bool is_small = l[j]->nrows <= std::min<uint32_t>(kSmallJoin, ctx.tune.join_small_rows);
    if (is_small) small.push_back(j);
    bstart[j + 1] = bstart[j] + (is_small ? 0 : div_up(l[j]->nrows, kJcTile));
    cbytes += 4.0 * (l[j]->nrows + r[j]->nrows);
  }
  const uint32_t nsmall = static_cast<uint32_t>(small.size());
  const uint32_t small_blocks = static_cast<uint32_t>(div_up(nsmall, kJcBlock / 32));
  const uint64_t T = bstart[J];
  if (T > 0x7FFFFFFFull) fail(VG_ERR_OVERFLOW, "batched join count: too many tiles");
  std::vector<uint32_t> tile_join(T);
  for (uint32_t j = 0; j < J; ++j)
    for (uint64_t t = bstart[j]; t < bstart[j + 1]; ++t) tile_join[t] = j;
  JoinSeg* djs = upload(ctx, js);
  uint64_t* dbs = upload(ctx, bstart);
  uint32_t* dtj = upload(ctx, tile_join);
  uint32_t* dsm = upload(ctx, small);
  jb.lo = ctx.alloc<uint32_t>(rows);
  jb.offs = ctx.alloc<uint64_t>(rows);
  uint64_t* status = ctx.alloc<uint64_t>(T);
  uint64_t* totals = ctx.alloc<uint64_t>(J);
  uint32_t* ticket = ctx.alloc<uint32_t>(1);
  uint2* dwin = ctx.alloc<uint2>(T ? T : 1);
  VG_CUDA(cudaMemsetAsync(status, 0, T * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(ticket, 0, sizeof(uint32_t), ctx.stream));
  if (T) {
    const uint64_t wblocks = std::min<uint64_t>(div_up(T, kJcBlock / 32), static_cast<uint64_t>(ctx.num_sms) * 8);
    ctx.launch("join_windows", 8.0 * T, [&] {
      jc_window_kernel<<<static_cast<unsigned>(wblocks), kJcBlock, 0, ctx.stream>>>(djs, dbs, dtj, T, dwin);
    });
    VG_CUDA(cudaGetLastError());
  }
  ctx.launch("join_count_scan", cbytes + 12.0 * rows, [&] {
    bjoin_count_scan_kernel<<<static_cast<unsigned>(small_blocks + T), kJcBlock, 0, ctx.stream>>>(
        djs, dbs, dtj, dwin, dsm, nsmall, small_blocks, jb.lo, jb.offs, status, ticket, totals, ctx.d_err);
  });
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaMemcpyAsync(totals_host, totals, J * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx.stream));
  jb.d_totals = totals;   // for a device-side placement; released with lo and offs
  // the stream orders every later use of these blocks after the kernel above
  ctx.free(status);
  ctx.free(ticket);
  ctx.free(dwin);
  ctx.free(djs);
  ctx.free(dbs);
  ctx.free(dtj);
  ctx.free(dsm);
}

void batched_join_write(Ctx& ctx, JoinBatch& jb, const uint64_t* totals, std::vector<Rel>& out,
                        uint32_t* first_last_host, const uint8_t* skip) {
  const uint32_t J = jb.J;
  if (!skip) out.assign(J, Rel());
  if (J == 0) return;
  std::vector<JoinOut> jo(J);
  std::vector<uint64_t> ostart(J + 1, 0);
  double wbytes = 0;
  auto rows = [&](uint32_t j) -> uint64_t { return (skip && skip[j]) ? 0 : totals[j]; };
  std::vector<uint32_t> small;   // outputs written one join per warp
  for (uint32_t j = 0; j < J; ++j) {
    if (rows(j) > 0xFFFFFFFFull) fail(VG_ERR_OVERFLOW, "join output exceeds 2^32 rows");
    const bool is_small = rows(j) > 0 && rows(j) <= ctx.tune.write_small_rows && jb.l[j]->nrows <= kSmallJoin;
    if (is_small) small.push_back(j);
    ostart[j + 1] = ostart[j] + (is_small ? 0 : div_up(rows(j), kTileRows));
    wbytes += 4.0 * rows(j) * (2.0 * (jb.l[j]->ncols + jb.r[j]->ncols - 1) - 1);
  }
  const uint32_t nsmall = static_cast<uint32_t>(small.size());
  const uint64_t small_blocks = div_up(nsmall, kBlock / 32);
  // the outputs of a wave's joins are allocated and described on the host pool
  parallel_for(J, [&](size_t j) {
    JoinOut& o = jo[j];
    std::memset(&o, 0, sizeof(o));
    if (skip && skip[j]) return;                // written already: out[j] stays as it is
    const Rel* l = jb.l[j];
    const Rel* r = jb.r[j];
    const uint32_t ncols = l->ncols + r->ncols - 1;
    out[j] = rel_alloc(ctx, ncols, totals[j]);
    o.offs = jb.offs + jb.row0[j];
    o.lo = jb.lo + jb.row0[j];
    o.nl = l->nrows;
    o.total = totals[j];
    for (uint32_t c = 0; c < l->ncols; ++c) o.lc[c] = l->cols[c];
    for (uint32_t c = 1; c < r->ncols; ++c) o.rc[c - 1] = r->cols[c];
    for (uint32_t c = 0; c < ncols; ++c) o.oc[c] = out[j].cols[c];
    o.nlc = l->ncols;
    o.nrc = r->ncols - 1;
  });
  JoinOut* djo = upload(ctx, jo);
  uint32_t* dfl = ctx.alloc<uint32_t>(2 * J);
  VG_CUDA(cudaMemsetAsync(dfl, 0, 2 * J * sizeof(uint32_t), ctx.stream));
  if (ostart[J] > 0 || nsmall > 0) {
    if (ostart[J] > 0x7FFFFFFFull) fail(VG_ERR_OVERFLOW, "batched join write: too many tiles");
    std::vector<uint32_t> tile_join(ostart[J]);
    for (uint32_t j = 0; j < J; ++j)
      for (uint64_t t = ostart[j]; t < ostart[j + 1]; ++t) tile_join[t] = j;
    uint64_t* dos = upload(ctx, ostart);
    uint32_t* dtj = upload(ctx, tile_join);
    uint32_t* dsm = upload(ctx, small);
    uint2* drg = ctx.alloc<uint2>(ostart[J] ? ostart[J] : 1);
    if (ostart[J]) {
      const uint64_t rblocks =
          std::min<uint64_t>(div_up(ostart[J], kBlock / 32), static_cast<uint64_t>(ctx.num_sms) * 8);
      ctx.launch("join_write_ranges", 8.0 * ostart[J], [&] {
        jw_range_kernel<<<static_cast<unsigned>(rblocks), kBlock, 0, ctx.stream>>>(djo, dos, dtj, ostart[J], nullptr,
                                                                                   drg);
      });
      VG_CUDA(cudaGetLastError());
    }
    const unsigned grid = static_cast<unsigned>(std::max<uint64_t>(ostart[J], small_blocks));
    ctx.launch("join_write", wbytes, [&] {
      bjoin_write_kernel<<<grid, kBlock, 0, ctx.stream>>>(djo, dos, dtj, drg, ostart[J], nullptr, dsm, nsmall,
                                                          nullptr);
    });
    VG_CUDA(cudaGetLastError());
    ctx.free(drg);
    ctx.free(dos);
    ctx.free(dtj);
    ctx.free(dsm);
  }
  ctx.launch("join_first_last", 8.0 * J, [&] {
    first_last_kernel<<<static_cast<unsigned>(div_up(J, 128)), 128, 0, ctx.stream>>>(djo, J, dfl);
  });
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaMemcpyAsync(first_last_host, dfl, 2 * J * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.free(dfl);
  ctx.free(djo);
  jb.release(ctx);
}

uint64_t place_outputs_on_host(const JoinBatch& jb, const uint64_t* totals, const Arena::Region* region,
                               uint64_t bump, std::vector<Rel>& out, std::vector<uint8_t>& placed,
                               int64_t& blocks) {
  const uint32_t J = jb.J;
  out.assign(J, Rel());
  placed.assign(J, 0);
  blocks = 0;
  uint64_t off = bump, fit = 0;
  for (uint32_t j = 0; j < J; ++j) {
    const uint64_t t = totals[j];
    const uint32_t ncols = jb.l[j]->ncols + jb.r[j]->ncols - 1;
    const uint64_t stride = place_stride(t);
    const uint64_t bytes = t ? ncols * stride : 0;
    const bool fits = off + bytes <= region->bytes;
    if (fits && t) {
      Rel& r = out[j];
      r.ncols = ncols;
      r.nrows = t;
      for (uint32_t c = 0; c < ncols; ++c) r.cols[c] = reinterpret_cast<uint32_t*>(region->begin + off + c * stride);
      placed[j] = 1;
      blocks += ncols;
    }
    if (fits) fit += bytes;
    off += bytes;
  }
  return bump + fit;
}

void batched_join_place_write(Ctx& ctx, JoinBatch& jb, const Arena::Region* region, uint64_t* d_bump,
                              const std::vector<int32_t>& c0_slot, uint32_t nslots, uint32_t* first_last_host,
                              uint32_t* c0_host, uint64_t* bump_host) {
  const uint32_t J = jb.J;
  if (J == 0) return;
  std::vector<JoinOut> jo(J);
  parallel_for(J, [&](size_t j) {
    const Rel* l = jb.l[j];
    const Rel* r = jb.r[j];
    JoinOut& o = jo[j];
    std::memset(&o, 0, sizeof(o));
    o.offs = jb.offs + jb.row0[j];
    o.lo = jb.lo + jb.row0[j];
    o.nl = l->nrows;
    for (uint32_t c = 0; c < l->ncols; ++c) o.lc[c] = l->cols[c];
    for (uint32_t c = 1; c < r->ncols; ++c) o.rc[c - 1] = r->cols[c];
    o.nlc = l->ncols;
    o.nrc = r->ncols - 1;
  });
  JoinOut* djo = upload(ctx, jo);
  int32_t* dslot = upload(ctx, c0_slot);
  uint64_t* dos = ctx.alloc<uint64_t>(J + 1);
  uint32_t* dsm = ctx.alloc<uint32_t>(J + 1);   // small list, then its length
  // every placed output tile covers kTileRows rows of at least one 4-byte column
  const uint64_t tile_cap = region->bytes / (4ull * kTileRows) + J + 1;
  uint32_t* dtj = ctx.alloc<uint32_t>(tile_cap);
  uint32_t* dfl = ctx.alloc<uint32_t>(2 * J);
  uint32_t* dstage = ctx.alloc<uint32_t>(static_cast<uint64_t>(nslots ? nslots : 1) * kSmallC0Words);
  VG_CUDA(cudaMemsetAsync(dfl, 0, 2 * J * sizeof(uint32_t), ctx.stream));
  JoinPlace pl{region->begin, region->bytes, d_bump, dos, dsm, dsm + J, ctx.tune.write_small_rows};
  ctx.launch("join_place", 16.0 * J, [&] {
    join_place_kernel<<<1, kPlaceBlock, 0, ctx.stream>>>(djo, jb.d_totals, J, pl);
  });
  VG_CUDA(cudaGetLastError());
  const unsigned jgrid = static_cast<unsigned>(std::min<uint64_t>(J, static_cast<uint64_t>(ctx.num_sms) * 8));
  ctx.launch("join_tile_map", 0.0, [&] { tile_join_fill_kernel<<<jgrid, 128, 0, ctx.stream>>>(dos, J, dtj); });
  VG_CUDA(cudaGetLastError());
  // the tile count is on the device: fixed grids loop over the tiles (the
  // algorithmic bytes are added when the host reads the totals)
  uint2* drg = ctx.alloc<uint2>(tile_cap);
  ctx.launch("join_write_ranges", 0.0, [&] {
    jw_range_kernel<<<static_cast<unsigned>(ctx.num_sms) * 8, kBlock, 0, ctx.stream>>>(djo, dos, dtj, 0, dos + J,
                                                                                       drg);
  });
  VG_CUDA(cudaGetLastError());
  ctx.launch("join_write", 0.0, [&] {
    bjoin_write_kernel<<<static_cast<unsigned>(ctx.num_sms) * ctx.tune.write_blocks_per_sm, kBlock, 0,
                         ctx.stream>>>(djo, dos, dtj, drg, 0, dos + J, dsm, 0, dsm + J);
  });
  VG_CUDA(cudaGetLastError());
  {
    const uint64_t eblocks = std::min<uint64_t>(div_up(J, kBlock / 32), static_cast<uint64_t>(ctx.num_sms) * 8);
    ctx.launch("join_first_last", 8.0 * J + 8.0 * nslots * kSmallC0Words, [&] {
      join_edges_kernel<<<static_cast<unsigned>(eblocks), kBlock, 0, ctx.stream>>>(djo, J, dfl,
                                                                                   nslots ? dslot : nullptr, dstage);
    });
    VG_CUDA(cudaGetLastError());
  }
  if (nslots)
    VG_CUDA(cudaMemcpyAsync(c0_host, dstage, static_cast<size_t>(nslots) * kSmallC0Words * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, ctx.stream));
  VG_CUDA(cudaMemcpyAsync(first_last_host, dfl, 2 * J * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx.stream));
  VG_CUDA(cudaMemcpyAsync(bump_host, d_bump, sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.free(djo);
  ctx.free(dslot);
  ctx.free(dos);
  ctx.free(dsm);
  ctx.free(dtj);
  ctx.free(drg);
  ctx.free(dfl);
  ctx.free(dstage);
}

void JoinBatch::release(Ctx& ctx) {
  ctx.free(lo);
  ctx.free(offs);
  ctx.free(d_totals);
  lo = nullptr;
  offs = nullptr;
  d_totals = nullptr;
}

void batched_join(Ctx& ctx, const std::vector<const Rel*>& l, const std::vector<const Rel*>& r,
                  std::vector<Rel>& out, std::vector<uint32_t>& first_last) {
  const uint32_t J = static_cast<uint32_t>(l.size());
  out.assign(J, Rel());
  first_last.assign(2 * J, 0);
  if (J == 0) return;
  PinnedWords tot(ctx), fl(ctx);
  JoinBatch jb;
  uint64_t* ht = tot.reserve(J + 1);
  batched_join_count(ctx, l, r, jb, ht);
  // the error record comes back with the totals: a look-back that gave up
  // leaves the offsets wrong, and the write must then not run
  VG_CUDA(cudaMemcpyAsync(ht + J, ctx.d_err, sizeof(DeviceErrors), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  {
    DeviceErrors he;
    std::memcpy(&he, ht + J, sizeof(he));
    if (he.timeout) {
      jb.release(ctx);
      ctx.raise_device_errors(he);
    }
  }
  batched_join_write(ctx, jb, tot.data(), out, reinterpret_cast<uint32_t*>(fl.reserve(J)));
  ctx.sync();
  const uint32_t* f = reinterpret_cast<const uint32_t*>(fl.data());
  std::copy(f, f + 2 * J, first_last.begin());
}

uint64_t col0_words(const std::vector<const Rel*>& rels) {
  uint64_t t = 0;
  for (const Rel* r : rels) t += r->nrows;
  return t;
}

void batched_col0_enqueue(Ctx& ctx, const std::vector<const Rel*>& rels, uint32_t* host) {
  const uint32_t R = static_cast<uint32_t>(rels.size());
  if (R == 0) return;
  std::vector<Col0Req> rq(R);
  uint64_t total = 0;
  for (uint32_t q = 0; q < R; ++q) {
    rq[q] = {rels[q]->cols[0], rels[q]->nrows, total};
    total += rels[q]->nrows;
  }
  if (total == 0) return;
  Col0Req* drq = upload(ctx, rq);
  uint32_t* buf = ctx.alloc<uint32_t>(total);
  ctx.launch("col0_stage", 8.0 * total, [&] {
    col0_kernel<<<R < 1024 ? R : 1024, 128, 0, ctx.stream>>>(drq, R, buf);
  });
  VG_CUDA(cudaGetLastError());
  VG_CUDA(cudaMemcpyAsync(host, buf, total * 4, cudaMemcpyDeviceToHost, ctx.stream));
  ctx.free(buf);
  ctx.free(drq);
}

void batched_col0(Ctx& ctx, const std::vector<const Rel*>& rels, std::vector<std::vector<uint32_t>>& out) {
  const uint32_t R = static_cast<uint32_t>(rels.size());
  out.assign(R, {});
  const uint64_t total = col0_words(rels);
  if (R == 0 || total == 0) return;
  PinnedWords h(ctx);
  uint32_t* p = reinterpret_cast<uint32_t*>(h.reserve((total + 1) / 2));
  batched_col0_enqueue(ctx, rels, p);
  ctx.sync();
  uint64_t off = 0;
  for (uint32_t q = 0; q < R; ++q) {
    out[q].assign(p + off, p + off + rels[q]->nrows);
    off += rels[q]->nrows;
  }
}

PinnedWords::~PinnedWords() { ctx_.give_pinned(p_, cap_); }

uint64_t* PinnedWords::reserve(size_t words) {
  const size_t bytes = std::max<size_t>(words, 1) * sizeof(uint64_t);
  if (p_ && bytes <= cap_) return p_;
  ctx_.give_pinned(p_, cap_);
  p_ = static_cast<uint64_t*>(ctx_.take_pinned(std::max<size_t>(bytes, size_t{1} << 16), &cap_));
  return p_;
}

}  // namespace vg
