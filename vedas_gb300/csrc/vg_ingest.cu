// N-Triples ingest on the device.
//
// 1. newline positions: tiles of 4096 bytes, counts scanned with a decoupled
//    look-back, positions written in order;
// 2. one thread parses each line into term spans (subject, predicate,
//    object, literal flag); valid lines are compacted in order by a second
//    look-back scan, so triple t is the t-th statement of the file;
// 3. per dictionary, every occurrence gets a 63-bit hash of its text; a
//    stable radix sort by hash keeps equal hashes in order of appearance, so
//    the first element of each run is the term's first occurrence;
// 4. run heads are counted (look-back scan), every member is checked against
//    its head byte by byte (a run holding different terms is a hash collision:
//    that dictionary is then resolved exactly on the host), and the heads are
//    sorted by first occurrence: rank r gets id base + r;
// 5. ids are scattered back to the s, p, o columns, and the term of every id
//    is read from the host copy of the text.
#include "vg_ingest.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string_view>

#include "vg_pool.h"
#include "vg_prims.cuh"
#include "vg_sort.h"

namespace vg {
namespace {

constexpr int kBlock = 256;
constexpr int kNlBytes = 16;                      // bytes per thread
constexpr uint64_t kNlTile = kBlock * kNlBytes;   // 4096
constexpr int kRows = 8;
constexpr uint64_t kTileRows = kBlock * kRows;

std::atomic<int> g_hash_bits{63};

struct Spans {
  uint64_t* s_off;
  uint64_t* p_off;
  uint64_t* o_off;
  uint32_t* s_len;
  uint32_t* p_len;
  uint32_t* o_len;
  uint8_t* lit;
};

// ---------------------------------------------------------------------------
// 1. newline positions (a counting pass sizes the position array)
__global__ void newline_count_kernel(const uint8_t* __restrict__ text, uint64_t len,
                                     unsigned long long* __restrict__ count) {
  const uint64_t words = len / 16;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  uint32_t c = 0;
  for (uint64_t w = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; w < words; w += stride) {
    const uint4 v = reinterpret_cast<const uint4*>(text)[w];
    const uint32_t x[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int k = 0; k < 4; ++k) c += ((x[q] >> (8 * k)) & 0xFFu) == '\n' ? 1u : 0u;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (uint64_t b = words * 16; b < len; ++b) c += text[b] == '\n' ? 1u : 0u;
  c = static_cast<uint32_t>(warp_sum64(c));
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, static_cast<unsigned long long>(c));
}

__global__ void __launch_bounds__(kBlock) newline_kernel(const uint8_t* __restrict__ text, uint64_t len,
                                                         uint64_t* __restrict__ nl, uint64_t* status,
                                                         uint32_t* ticket, uint64_t* total, DeviceErrors* err) {
  __shared__ uint32_t s_scan[kBlock / 32 + 1];
  __shared__ uint64_t s_b;
  __shared__ uint32_t s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint64_t tile = s_tile;
  const uint64_t b0 = tile * kNlTile + static_cast<uint64_t>(threadIdx.x) * kNlBytes;
  uint32_t mask = 0;   // bit k: byte b0 + k is a newline
  if (b0 + kNlBytes <= len) {
    const uint4 v = *reinterpret_cast<const uint4*>(text + b0);
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (((w[q] >> (8 * k)) & 0xFFu) == '\n') mask |= 1u << (4 * q + k);
  } else {
    for (int k = 0; k < kNlBytes && b0 + k < len; ++k)
      if (text[b0 + k] == '\n') mask |= 1u << k;
  }
  uint32_t tot;
  const uint32_t e = block_excl_scan<kBlock>(__popc(mask), tot, s_scan);
  if (threadIdx.x < 32) {
    const uint64_t p = warp_lookback(status, static_cast<uint32_t>(tile), tot, err);
    if (threadIdx.x == 0) s_b = p;
  }
  __syncthreads();
  uint64_t o = s_b + e;
  while (mask) {
    const int k = __ffs(mask) - 1;
    nl[o++] = b0 + k;
    mask &= mask - 1;
  }
  if (tile == gridDim.x - 1 && threadIdx.x == 0) *total = s_b + tot;
}

// ---------------------------------------------------------------------------
// 2. line parser (N-Triples statements)
__device__ __forceinline__ bool is_ws(uint8_t c) { return c == ' ' || c == '\t' || c == '\r'; }

// Term at text[i]; returns its end (one past) or 0 on a malformed term.
// kind: 0 any, 1 IRI only (predicate), 2 IRI or blank node (subject).
__device__ uint64_t term_end(const uint8_t* t, uint64_t i, uint64_t end, int kind, bool& literal) {
  literal = false;
  if (i >= end) return 0;
  const uint8_t c = t[i];
  if (c == '<') {
    for (uint64_t j = i + 1; j < end; ++j) {
      if (t[j] == '>') return j + 1;
      if (t[j] == ' ' || t[j] == '\t') return 0;
    }
    return 0;
  }
  if (kind == 1) return 0;
  if (c == '_') {
    if (i + 1 >= end || t[i + 1] != ':') return 0;
    uint64_t j = i + 2;
    while (j < end && !is_ws(t[j])) ++j;
    if (j == i + 2) return 0;
    // a label does not end with '.': "_:b1." before the statement's dot
    if (t[j - 1] == '.' && j - 1 > i + 2) --j;
    return j;
  }
  if (kind == 2 || c != '"') return 0;
  uint64_t j = i + 1;
  while (j < end) {
    if (t[j] == '\\') {
      j += 2;
      continue;
    }
    if (t[j] == '"') break;
    ++j;
  }
  if (j >= end) return 0;
  ++j;   // past the closing quote
  literal = true;
  if (j < end && t[j] == '@') {
    uint64_t k = j + 1;
    while (k < end && ((t[k] >= 'a' && t[k] <= 'z') || (t[k] >= 'A' && t[k] <= 'Z') ||
                       (t[k] >= '0' && t[k] <= '9') || t[k] == '-'))
      ++k;
    if (k == j + 1) return 0;
    return k;
  }
  if (j + 1 < end && t[j] == '^' && t[j + 1] == '^') {
    bool dummy;
    const uint64_t k = term_end(t, j + 2, end, 1, dummy);
    return k;
  }
  return j;
}

__global__ void __launch_bounds__(kBlock) parse_kernel(const uint8_t* __restrict__ text, uint64_t len,
                                                       const uint64_t* __restrict__ nl, uint64_t nnl, uint64_t lines,
                                                       Spans out, uint64_t* status, uint32_t* ticket,
                                                       uint64_t* count, unsigned long long* bad_line,
                                                       DeviceErrors* err) {
  __shared__ uint32_t s_scan[kBlock / 32 + 1];
  __shared__ uint64_t s_b;
  __shared__ uint32_t s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint64_t tile = s_tile;
  const uint64_t line = tile * kBlock + threadIdx.x;
  bool valid = false, lit = false;
  uint64_t so = 0, se = 0, po = 0, pe = 0, oo = 0, oe = 0;
  if (line < lines) {
    const uint64_t b = line == 0 ? 0 : nl[line - 1] + 1;
    const uint64_t e = line < nnl ? nl[line] : len;
    uint64_t i = b;
    while (i < e && is_ws(text[i])) ++i;
    if (i < e && text[i] != '#') {
      bool ok = true, l0 = false, l1 = false;
      so = i;
      se = term_end(text, i, e, 2, l0);
      ok = se != 0;
      if (ok) {
        i = se;
        const uint64_t ws0 = i;
        while (i < e && is_ws(text[i])) ++i;
        ok = i > ws0;
      }
      if (ok) {
        po = i;
        pe = term_end(text, i, e, 1, l1);
        ok = pe != 0;
      }
      if (ok) {
        i = pe;
        const uint64_t ws0 = i;
        while (i < e && is_ws(text[i])) ++i;
        ok = i > ws0;
      }
      if (ok) {
        oo = i;
        oe = term_end(text, i, e, 0, lit);
        ok = oe != 0;
      }
      if (ok) {
        i = oe;
        while (i < e && is_ws(text[i])) ++i;
        ok = i < e && text[i] == '.';
        ++i;
        while (ok && i < e && is_ws(text[i])) ++i;
        ok = ok && (i >= e || text[i] == '#');
      }
      if (ok) valid = true;
      else atomicMin(bad_line, static_cast<unsigned long long>(line + 1));
    }
  }
  uint32_t tot;
  const uint32_t ex = block_excl_scan<kBlock>(valid ? 1u : 0u, tot, s_scan);
  if (threadIdx.x < 32) {
    const uint64_t p = warp_lookback(status, static_cast<uint32_t>(tile), tot, err);
    if (threadIdx.x == 0) s_b = p;
  }
  __syncthreads();
  if (valid) {
    const uint64_t t = s_b + ex;
    out.s_off[t] = so;
    out.s_len[t] = static_cast<uint32_t>(se - so);
    out.p_off[t] = po;
    out.p_len[t] = static_cast<uint32_t>(pe - po);
    out.o_off[t] = oo;
    out.o_len[t] = static_cast<uint32_t>(oe - oo);
    out.lit[t] = lit ? 1 : 0;
  }
  if (tile == gridDim.x - 1 && threadIdx.x == 0) *count = s_b + tot;
}

// ---------------------------------------------------------------------------
// 3. hashing of the occurrences of one dictionary
// A 64-bit multiply-xorshift mix over 8-byte words (this project's own; any
// good mix works, equality is checked byte by byte afterwards).
__device__ __forceinline__ uint64_t mix64(uint64_t h) {
  h ^= h >> 31;
  h *= 0x7fb5d329728ea185ull;
  h ^= h >> 27;
  h *= 0x81dadef4bc2dd44dull;
  h ^= h >> 33;
  return h;
}

__device__ uint64_t term_hash(const uint8_t* t, uint64_t off, uint32_t len, int bits) {
  uint64_t h = 0x243f6a8885a308d3ull ^ len;
  uint32_t i = 0;
  for (; i + 8 <= len; i += 8) {
    uint64_t w = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) w |= static_cast<uint64_t>(t[off + i + k]) << (8 * k);
    h = mix64(h ^ w);
  }
  uint64_t w = 0;
  for (int k = 0; i + k < len; ++k) w |= static_cast<uint64_t>(t[off + i + k]) << (8 * k);
  h = mix64(h ^ w ^ (static_cast<uint64_t>(len) << 56));
  return bits >= 63 ? (h >> 1) : (h >> (64 - bits));
}

// kind 0: subject/object dictionary over 2n occurrences (2t subject, 2t+1
// object); kind 1: predicates; kind 2: literal objects.  Non-members get the
// key ~0 (sorted after every member).
__global__ void hash_kernel(const uint8_t* __restrict__ text, Spans sp, uint64_t n, int kind, bool literal_dict,
                            int bits, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                            unsigned long long* members) {
  const uint64_t m = kind == 0 ? 2 * n : n;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  uint32_t mine = 0;
  for (uint64_t k = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < m; k += stride) {
    uint64_t off = 0;
    uint32_t len = 0;
    bool member = true;
    if (kind == 0) {
      const uint64_t t = k >> 1;
      if (k & 1) {
        member = !(literal_dict && sp.lit[t]);
        off = sp.o_off[t];
        len = sp.o_len[t];
      } else {
        off = sp.s_off[t];
        len = sp.s_len[t];
      }
    } else if (kind == 1) {
      off = sp.p_off[k];
      len = sp.p_len[k];
    } else {
      member = sp.lit[k] != 0;
      off = sp.o_off[k];
      len = sp.o_len[k];
    }
    keys[k] = member ? term_hash(text, off, len, bits) : ~0ull;
    vals[k] = static_cast<uint32_t>(k);
    mine += member ? 1u : 0u;
  }
  if (mine) atomicAdd(members, static_cast<unsigned long long>(mine));
}

__device__ __forceinline__ void occ_span(const Spans& sp, int kind, uint32_t k, uint64_t& off, uint32_t& len) {
  if (kind == 0) {
    const uint32_t t = k >> 1;
    if (k & 1) {
      off = sp.o_off[t];
      len = sp.o_len[t];
    } else {
      off = sp.s_off[t];
      len = sp.s_len[t];
    }
  } else if (kind == 1) {
    off = sp.p_off[k];
    len = sp.p_len[k];
  } else {
    off = sp.o_off[k];
    len = sp.o_len[k];
  }
}

// ---------------------------------------------------------------------------
// 4. run heads: seg[i] = index of the run holding element i; head_pos[r] =
// first element of run r.
__global__ void __launch_bounds__(kBlock) heads_kernel(const uint64_t* __restrict__ keys, uint64_t m,
                                                       uint32_t* __restrict__ seg, uint32_t* __restrict__ head_pos,
                                                       uint64_t* status, uint32_t* ticket, uint64_t* total,
                                                       DeviceErrors* err) {
  __shared__ uint32_t s_scan[kBlock / 32 + 1];
  __shared__ uint64_t s_b;
  __shared__ uint32_t s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint64_t tile = s_tile;
  const uint64_t r0 = tile * kTileRows + static_cast<uint64_t>(threadIdx.x) * kRows;
  uint32_t flags = 0;
  uint64_t prev = (r0 > 0 && r0 - 1 < m) ? keys[r0 - 1] : 0;
#pragma unroll
  for (int i = 0; i < kRows; ++i) {
    const uint64_t r = r0 + i;
    if (r < m) {
      const uint64_t k = keys[r];
      if (r == 0 || k != prev) flags |= 1u << i;
      prev = k;
    }
  }
  uint32_t tot;
  const uint32_t e = block_excl_scan<kBlock>(__popc(flags), tot, s_scan);
  if (threadIdx.x < 32) {
    const uint64_t p = warp_lookback(status, static_cast<uint32_t>(tile), tot, err);
    if (threadIdx.x == 0) s_b = p;
  }
  __syncthreads();
  uint64_t run = s_b + e;   // heads before this thread's rows
#pragma unroll
  for (int i = 0; i < kRows; ++i) {
    const uint64_t r = r0 + i;
    if (r >= m) break;
    if (flags >> i & 1u) {
      head_pos[run] = static_cast<uint32_t>(r);
      ++run;
    }
    seg[r] = static_cast<uint32_t>(run - 1);
  }
  if (tile == gridDim.x - 1 && threadIdx.x == 0) *total = s_b + tot;
}

// Every member's text equals its run head's text (else a hash collision).
__global__ void verify_kernel(const uint8_t* __restrict__ text, Spans sp, int kind, const uint32_t* __restrict__ vals,
                              const uint32_t* __restrict__ seg, const uint32_t* __restrict__ head_pos, uint64_t m,
                              unsigned int* collision) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < m; i += stride) {
    const uint32_t h = head_pos[seg[i]];
    if (h == i) continue;
    uint64_t a, b;
    uint32_t la, lb;
    occ_span(sp, kind, vals[i], a, la);
    occ_span(sp, kind, vals[h], b, lb);
    bool same = la == lb;
    for (uint32_t k = 0; same && k < la; ++k) same = text[a + k] == text[b + k];
    if (!same) atomicExch(collision, 1u);
  }
}

// First occurrence of every run, to be sorted into id order.
__global__ void first_pos_kernel(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ head_pos,
                                 uint64_t runs, uint32_t* __restrict__ fpos, uint32_t* __restrict__ rid) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < runs; r += stride) {
    fpos[r] = vals[head_pos[r]];
    rid[r] = static_cast<uint32_t>(r);
  }
}

__global__ void rank_kernel(const uint32_t* __restrict__ sorted_rid, uint64_t runs, uint32_t base,
                            uint32_t* __restrict__ id_of_run) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < runs; r += stride)
    id_of_run[sorted_rid[r]] = base + static_cast<uint32_t>(r);
}

// 5. ids back to the columns
__global__ void scatter_kernel(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ seg,
                               const uint32_t* __restrict__ id_of_run, uint64_t m, int kind, uint32_t* __restrict__ s,
                               uint32_t* __restrict__ p, uint32_t* __restrict__ o) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < m; i += stride) {
    const uint32_t k = vals[i];
    const uint32_t id = id_of_run[seg[i]];
    if (kind == 0) {
      if (k & 1) o[k >> 1] = id;
      else s[k >> 1] = id;
    } else if (kind == 1) {
      p[k] = id;
    } else {
      o[k] = id;
    }
  }
}

// Spans of the terms in id order.
__global__ void dict_spans_kernel(Spans sp, int kind, const uint32_t* __restrict__ fpos_sorted, uint64_t runs,
                                  uint64_t* __restrict__ off, uint32_t* __restrict__ len) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t r = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < runs; r += stride)
    occ_span(sp, kind, fpos_sorted[r], off[r], len[r]);
}

unsigned grid(const Ctx& ctx, uint64_t units) {
  uint64_t g = div_up(units, static_cast<uint64_t>(kBlock));
  const uint64_t gmax = static_cast<uint64_t>(ctx.num_sms) * 16;
  if (g > gmax) g = gmax;
  return static_cast<unsigned>(g < 1 ? 1 : g);
}

template <typename T>
void download(Ctx& ctx, std::vector<T>& h, const T* d, uint64_t n) {
  h.resize(n);
  if (n) VG_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, ctx.stream));
}

// Exact first-appearance ids on the host for one dictionary (after a hash
// collision): the statement handler's own rule, src/loader.cu:19-53.
void resolve_exact(Ctx& ctx, const char* text, const Spans& sp, uint64_t n, int kind, bool literal_dict,
                   uint32_t base, uint32_t* s, uint32_t* p, uint32_t* o, std::vector<std::string>& terms) {
  std::vector<uint64_t> so, po, oo;
  std::vector<uint32_t> sl, pl, ol;
  std::vector<uint8_t> lit;
  download(ctx, so, sp.s_off, n);
  download(ctx, sl, sp.s_len, n);
  download(ctx, po, sp.p_off, n);
  download(ctx, pl, sp.p_len, n);
  download(ctx, oo, sp.o_off, n);
  download(ctx, ol, sp.o_len, n);
  download(ctx, lit, sp.lit, n);
  std::vector<uint32_t> hs, hp, ho;
  download(ctx, hs, s, n);
  download(ctx, hp, p, n);
  download(ctx, ho, o, n);
  ctx.sync();
  std::unordered_map<std::string_view, uint32_t> ids;
  terms.clear();
  auto id_of = [&](uint64_t off, uint32_t len) {
    const std::string_view v(text + off, len);
    auto it = ids.find(v);
    if (it != ids.end()) return it->second;
    const uint32_t id = base + static_cast<uint32_t>(terms.size());
    ids.emplace(v, id);
    terms.emplace_back(v);
    return id;
  };
  for (uint64_t t = 0; t < n; ++t) {
    if (kind == 0) {
      hs[t] = id_of(so[t], sl[t]);
      if (!(literal_dict && lit[t])) ho[t] = id_of(oo[t], ol[t]);
    } else if (kind == 1) {
      hp[t] = id_of(po[t], pl[t]);
    } else if (lit[t]) {
      ho[t] = id_of(oo[t], ol[t]);
    }
  }
  if (n) {
    VG_CUDA(cudaMemcpyAsync(s, hs.data(), n * 4, cudaMemcpyHostToDevice, ctx.stream));
    VG_CUDA(cudaMemcpyAsync(p, hp.data(), n * 4, cudaMemcpyHostToDevice, ctx.stream));
    VG_CUDA(cudaMemcpyAsync(o, ho.data(), n * 4, cudaMemcpyHostToDevice, ctx.stream));
  }
  ctx.sync();
}

// One dictionary: hash, sort, runs, check, ids, scatter, terms.  Returns
// false when a hash collision was found (nothing was written).
bool encode_dict(Ctx& ctx, const char* host_text, const uint8_t* text, const Spans& sp, uint64_t n, int kind,
                 bool literal_dict, uint32_t base, uint32_t* s, uint32_t* p, uint32_t* o,
                 std::vector<std::string>& terms) {
  const uint64_t m_all = kind == 0 ? 2 * n : n;
  terms.clear();
  if (m_all == 0) return true;
  if (m_all > 0xFFFFFFFFull) fail(VG_ERR_OVERFLOW, "ingest is limited to 2^31 triples");
  Scratch<uint64_t> keys(ctx, m_all), keys_alt(ctx, m_all);
  Scratch<uint32_t> vals(ctx, m_all), vals_alt(ctx, m_all);
  Scratch<unsigned long long> dm(ctx, 1);
  VG_CUDA(cudaMemsetAsync(dm.get(), 0, sizeof(unsigned long long), ctx.stream));
  ctx.launch("ingest_hash", 12.0 * m_all, [&] {
    hash_kernel<<<grid(ctx, m_all), kBlock, 0, ctx.stream>>>(text, sp, n, kind, literal_dict, g_hash_bits.load(),
                                                              keys.get(), vals.get(), dm.get());
  });
  VG_CUDA(cudaGetLastError());
  const bool alt = radix_sort_u64(ctx, keys.get(), keys_alt.get(), vals.get(), vals_alt.get(), m_all, 64, false, true);
  uint64_t* k = alt ? keys_alt.get() : keys.get();
  uint32_t* v = alt ? vals_alt.get() : vals.get();
  uint64_t m = 0;
  VG_CUDA(cudaMemcpyAsync(&m, dm.get(), sizeof(m), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  if (m == 0) return true;
  const uint64_t tiles = div_up(m, kTileRows);
  Scratch<uint32_t> seg(ctx, m), head_pos(ctx, m), ticket(ctx, 1);
  Scratch<uint64_t> status(ctx, tiles), runs_d(ctx, 1);
  Scratch<unsigned int> coll(ctx, 1);
  VG_CUDA(cudaMemsetAsync(status.get(), 0, tiles * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(uint32_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(coll.get(), 0, sizeof(unsigned int), ctx.stream));
  ctx.launch("ingest_runs", 12.0 * m, [&] {
    heads_kernel<<<static_cast<unsigned>(tiles), kBlock, 0, ctx.stream>>>(k, m, seg.get(), head_pos.get(),
                                                                           status.get(), ticket.get(), runs_d.get(),
                                                                           ctx.d_err);
  });
  VG_CUDA(cudaGetLastError());
  ctx.launch("ingest_verify", 8.0 * m, [&] {
    verify_kernel<<<grid(ctx, m), kBlock, 0, ctx.stream>>>(text, sp, kind, v, seg.get(), head_pos.get(), m,
                                                            coll.get());
  });
  VG_CUDA(cudaGetLastError());
  uint64_t runs = 0;
  unsigned int collided = 0;
  VG_CUDA(cudaMemcpyAsync(&runs, runs_d.get(), sizeof(runs), cudaMemcpyDeviceToHost, ctx.stream));
  VG_CUDA(cudaMemcpyAsync(&collided, coll.get(), sizeof(collided), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  if (collided) return false;
  if (static_cast<uint64_t>(base) + runs > 0xFFFFFFFFull) fail(VG_ERR_OVERFLOW, "dictionary ids exceed 32 bits");
  Scratch<uint32_t> fpos(ctx, runs), fpos_alt(ctx, runs), rid(ctx, runs), rid_alt(ctx, runs), id_of_run(ctx, runs);
  ctx.launch("ingest_ids", 8.0 * runs, [&] {
    first_pos_kernel<<<grid(ctx, runs), kBlock, 0, ctx.stream>>>(v, head_pos.get(), runs, fpos.get(), rid.get());
  });
  VG_CUDA(cudaGetLastError());
  const bool alt2 = radix_sort_u32(ctx, fpos.get(), fpos_alt.get(), rid.get(), rid_alt.get(), runs, 32, false, true);
  const uint32_t* fs = alt2 ? fpos_alt.get() : fpos.get();
  const uint32_t* rs = alt2 ? rid_alt.get() : rid.get();
  ctx.launch("ingest_ids", 8.0 * runs, [&] {
    rank_kernel<<<grid(ctx, runs), kBlock, 0, ctx.stream>>>(rs, runs, base, id_of_run.get());
  });
  VG_CUDA(cudaGetLastError());
  ctx.launch("ingest_scatter", 12.0 * m, [&] {
    scatter_kernel<<<grid(ctx, m), kBlock, 0, ctx.stream>>>(v, seg.get(), id_of_run.get(), m, kind, s, p, o);
  });
  VG_CUDA(cudaGetLastError());
  Scratch<uint64_t> toff(ctx, runs);
  Scratch<uint32_t> tlen(ctx, runs);
  ctx.launch("ingest_terms", 12.0 * runs, [&] {
    dict_spans_kernel<<<grid(ctx, runs), kBlock, 0, ctx.stream>>>(sp, kind, fs, runs, toff.get(), tlen.get());
  });
  VG_CUDA(cudaGetLastError());
  std::vector<uint64_t> ho;
  std::vector<uint32_t> hl;
  download(ctx, ho, toff.get(), runs);
  download(ctx, hl, tlen.get(), runs);
  ctx.sync();
  terms.resize(runs);
  parallel_for(runs, [&](size_t r) { terms[r].assign(host_text + ho[r], hl[r]); });
  return true;
}

}  // namespace

void set_ingest_hash_bits(int bits) { g_hash_bits.store(bits < 1 ? 1 : (bits > 63 ? 63 : bits)); }

const std::string* Dict::term(int kind, uint32_t id) const {
  const std::vector<std::string>& v = kind == 0 ? so : (kind == 1 ? p : l);
  const uint32_t base = kind == 2 ? kLiteralStartId : 1u;
  if (id < base || id - base >= v.size()) return nullptr;
  return &v[id - base];
}

uint32_t Dict::lookup(int kind, const std::string& t) {
  if (kind < 0 || kind > 2) return 0;
  auto& rev = rev_[kind];
  const std::vector<std::string>& v = kind == 0 ? so : (kind == 1 ? p : l);
  const uint32_t base = kind == 2 ? kLiteralStartId : 1u;
  if (rev.size() != v.size()) {
    rev.clear();
    rev.reserve(v.size());
    for (size_t i = 0; i < v.size(); ++i) rev.emplace(v[i], base + static_cast<uint32_t>(i));
  }
  auto it = rev.find(t);
  return it == rev.end() ? 0 : it->second;
}

void ingest_ntriples(Ctx& ctx, const char* text, uint64_t len, bool literal_dict, Ingested& out) {
  out = Ingested();
  out.dict.literal_dict = literal_dict;
  if (len == 0) return;
  // the text, padded to whole 16-byte words
  Scratch<uint8_t> dtext(ctx, div_up(len, 16) * 16);
  VG_CUDA(cudaMemcpyAsync(dtext.get(), text, len, cudaMemcpyHostToDevice, ctx.stream));
  // 1. newlines
  const uint64_t ntiles = div_up(len, kNlTile);
  if (ntiles > 0xFFFFFFFFull) fail(VG_ERR_OVERFLOW, "ingest text too long");
  Scratch<unsigned long long> ncount(ctx, 1);
  VG_CUDA(cudaMemsetAsync(ncount.get(), 0, sizeof(unsigned long long), ctx.stream));
  ctx.launch("ingest_newlines", static_cast<double>(len), [&] {
    newline_count_kernel<<<grid(ctx, div_up(len, 16)), kBlock, 0, ctx.stream>>>(dtext.get(), len, ncount.get());
  });
  VG_CUDA(cudaGetLastError());
  unsigned long long nl_count = 0;
  VG_CUDA(cudaMemcpyAsync(&nl_count, ncount.get(), sizeof(nl_count), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  Scratch<uint64_t> nl(ctx, nl_count + 1), st1(ctx, ntiles), tot1(ctx, 1);
  Scratch<uint32_t> tk1(ctx, 1);
  VG_CUDA(cudaMemsetAsync(st1.get(), 0, ntiles * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(tk1.get(), 0, sizeof(uint32_t), ctx.stream));
  ctx.launch("ingest_newlines", static_cast<double>(len), [&] {
    newline_kernel<<<static_cast<unsigned>(ntiles), kBlock, 0, ctx.stream>>>(dtext.get(), len, nl.get(), st1.get(),
                                                                            tk1.get(), tot1.get(), ctx.d_err);
  });
  VG_CUDA(cudaGetLastError());
  uint64_t nnl = 0;
  VG_CUDA(cudaMemcpyAsync(&nnl, tot1.get(), sizeof(nnl), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  const uint64_t lines = nnl + (text[len - 1] != '\n' ? 1 : 0);
  // 2. statements
  Scratch<uint64_t> s_off(ctx, lines), p_off(ctx, lines), o_off(ctx, lines);
  Scratch<uint32_t> s_len(ctx, lines), p_len(ctx, lines), o_len(ctx, lines);
  Scratch<uint8_t> lit(ctx, lines);
  const Spans sp{s_off.get(), p_off.get(), o_off.get(), s_len.get(), p_len.get(), o_len.get(), lit.get()};
  const uint64_t ptiles = div_up(lines, static_cast<uint64_t>(kBlock));
  Scratch<uint64_t> st2(ctx, ptiles), cnt(ctx, 1);
  Scratch<uint32_t> tk2(ctx, 1);
  Scratch<unsigned long long> bad(ctx, 1);
  VG_CUDA(cudaMemsetAsync(st2.get(), 0, ptiles * sizeof(uint64_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(tk2.get(), 0, sizeof(uint32_t), ctx.stream));
  VG_CUDA(cudaMemsetAsync(bad.get(), 0xFF, sizeof(unsigned long long), ctx.stream));
  ctx.launch("ingest_parse", static_cast<double>(len) + 37.0 * lines, [&] {
    parse_kernel<<<static_cast<unsigned>(ptiles), kBlock, 0, ctx.stream>>>(
        dtext.get(), len, nl.get(), nnl, lines, sp, st2.get(), tk2.get(), cnt.get(), bad.get(), ctx.d_err);
  });
  VG_CUDA(cudaGetLastError());
  uint64_t n = 0;
  unsigned long long bad_line = 0;
  VG_CUDA(cudaMemcpyAsync(&n, cnt.get(), sizeof(n), cudaMemcpyDeviceToHost, ctx.stream));
  VG_CUDA(cudaMemcpyAsync(&bad_line, bad.get(), sizeof(bad_line), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  ctx.check_device_errors();
  if (bad_line != ~0ull) fail(VG_ERR_PARSE, "malformed N-Triples statement on line " + std::to_string(bad_line));
  if (n > 0x7FFFFFFFull) fail(VG_ERR_OVERFLOW, "ingest is limited to 2^31 triples");
  out.n = n;
  out.s = ctx.alloc<uint32_t>(n);
  out.p = ctx.alloc<uint32_t>(n);
  out.o = ctx.alloc<uint32_t>(n);
  if (n == 0) return;
  // 3-5. the dictionaries
  struct Job {
    int kind;
    uint32_t base;
    std::vector<std::string>* terms;
  };
  std::vector<Job> jobs = {{0, 1u, &out.dict.so}, {1, 1u, &out.dict.p}};
  if (literal_dict) jobs.push_back({2, kLiteralStartId, &out.dict.l});
  for (const Job& j : jobs) {
    if (!encode_dict(ctx, text, dtext.get(), sp, n, j.kind, literal_dict, j.base, out.s, out.p, out.o, *j.terms)) {
      ++out.collisions;
      resolve_exact(ctx, text, sp, n, j.kind, literal_dict, j.base, out.s, out.p, out.o, *j.terms);
    }
  }
  ctx.sync();
  ctx.check_device_errors();
}

DictResolver::DictResolver(const Dict* d) {
  const std::vector<std::string>* v[3] = {&d->so, &d->p, &d->l};
  for (int k = 0; k < 3; ++k) {
    const uint32_t base = k == 2 ? kLiteralStartId : 1u;
    rev_[k].reserve(v[k]->size());
    for (size_t i = 0; i < v[k]->size(); ++i) rev_[k].emplace((*v[k])[i], base + static_cast<uint32_t>(i));
  }
}

vedas::TYPEID DictResolver::resolve(int pos, const std::string& term) const {
  int kind = pos == 1 ? 1 : 0;
  std::string key = term;
  if (pos == 2 && !term.empty() && term[0] == '"') {
    kind = 2;
    key = term.substr(0, term.find('"', 1) + 1);   // "text" without @lang / ^^<type>
  }
  auto it = rev_[kind].find(key);
  return it == rev_[kind].end() ? 0 : it->second;
}

std::string decode_rows(const Dict& d, const std::vector<const uint32_t*>& cols, uint64_t nrows) {
  // rows are decoded in parallel blocks, then joined
  constexpr uint64_t kRowsPerPart = 4096;
  const uint64_t parts = (nrows + kRowsPerPart - 1) / kRowsPerPart;
  std::vector<std::string> out(parts);
  parallel_for(parts, [&](size_t b) {
    std::string& o = out[b];
    const uint64_t r1 = std::min<uint64_t>(nrows, (b + 1) * kRowsPerPart);
    for (uint64_t r = b * kRowsPerPart; r < r1; ++r) {
      for (size_t c = 0; c < cols.size(); ++c) {
        if (c) o += '\t';
        const uint32_t id = cols[c][r];
        const std::string* t = (d.literal_dict && id >= kLiteralStartId) ? d.term(2, id) : d.term(0, id);
        if (t) o += *t;
        else o += "?" + std::to_string(id);
      }
      o += '\n';
    }
  });
  size_t total = 0;
  for (const auto& x : out) total += x.size();
  std::string all;
  all.reserve(total);
  for (const auto& x : out) all += x;
  return all;
}

void write_vdd(const Dict& d, const char* path) {
  std::ofstream out(path);
  if (!out) fail(VG_ERR_INVALID, std::string("cannot write ") + path);
  auto section = [&](const std::vector<std::string>& v, uint32_t base) {
    out << v.size() << "\n";
    for (size_t i = 0; i < v.size(); ++i) out << (base + i) << " " << v[i] << "\n";
  };
  section(d.so, 1u);
  section(d.p, 1u);
  section(d.l, kLiteralStartId);
  if (!out) fail(VG_ERR_INVALID, std::string("write failed: ") + path);
}

void read_vdd(const char* path, Dict& d) {
  std::ifstream in(path);
  if (!in) fail(VG_ERR_INVALID, std::string("cannot open ") + path);
  d = Dict();
  auto section = [&](std::vector<std::string>& v, uint32_t base) {
    std::string line;
    if (!std::getline(in, line)) fail(VG_ERR_INVALID, "truncated .vdd");
    const uint64_t count = std::stoull(line);
    // entries may come in any order (the reference writes hash-map order)
    std::vector<std::pair<uint32_t, std::string>> e;
    e.reserve(count);
    for (uint64_t i = 0; i < count; ++i) {
      if (!std::getline(in, line)) fail(VG_ERR_INVALID, "truncated .vdd");
      const size_t sp = line.find(' ');
      if (sp == std::string::npos) fail(VG_ERR_INVALID, "malformed .vdd line");
      e.emplace_back(static_cast<uint32_t>(std::stoul(line.substr(0, sp))), line.substr(sp + 1));
    }
    std::sort(e.begin(), e.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    for (size_t i = 0; i < e.size(); ++i)
      if (e[i].first != base + i) fail(VG_ERR_INVALID, ".vdd ids are not dense");
    v.resize(e.size());
    for (size_t i = 0; i < e.size(); ++i) v[i] = std::move(e[i].second);
  };
  section(d.so, 1u);
  section(d.p, 1u);
  section(d.l, kLiteralStartId);
  d.literal_dict = !d.l.empty();
}

}  // namespace vg
