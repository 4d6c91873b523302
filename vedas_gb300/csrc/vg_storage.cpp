// Resident index: build orchestration, host mirrors and the .vds format.
#include <algorithm>
#include <cstring>
#include <cstdio>
#include <fstream>

#include "vg_index.h"

namespace vg {

const DevArray& Index::get(const std::string& name) const {
  static const DevArray empty;
  auto it = dev.find(name);
  return it == dev.end() ? empty : it->second;
}

const std::vector<uint32_t>& Index::host_array(const std::string& name) {
  auto it = host.find(name);
  if (it != host.end()) return it->second;
  const DevArray& d = get(name);
  std::vector<uint32_t>& v = host[name];
  v.resize(d.len);
  if (d.len) {
    VG_CUDA(cudaMemcpyAsync(v.data(), d.ptr, d.len * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
  }
  return v;
}

void Index::release() {
  if (ctx)
    for (auto& kv : dev)
      if (kv.second.ptr) ctx->free(kv.second.ptr);
  dev.clear();
  host.clear();
}

// Permutations and their outputs follow VedasStorage::VedasStorage
// (src/VedasStorage.cu:25-73): PSO and POS always; SPO, SOP, OS and OPS with
// the full index.  The subject level-1 index is never filled there (its code
// is commented out at src/VedasStorage.cu:319-339), so s_idx_* stay empty.
void build_index(Ctx& ctx, const uint32_t* s, const uint32_t* p, const uint32_t* o, uint64_t n,
                 bool full, Index& ix) {
  ix.ctx = &ctx;
  ix.full = full;
  ix.n = n;
  uint32_t mx[3];
  column_max3(ctx, s, p, o, n, mx);
  const uint32_t ms = mx[0], mp = mx[1], mo = mx[2];
  ix.max_id = std::max(ms, std::max(mp, mo));
  auto put = [&](const char* name, const DevArray& a) { ix.dev[name] = a; };
  {
    // PSO by a full sort; POS from PSO's sorted keys by a sort of (p, o) only
    PermOutputs pso, pos;
    pso.want_col1 = pso.want_col2 = pso.want_l1 = pso.want_l2 = true;
    pos.want_col1 = pos.want_col2 = pos.want_l2 = true;
    const uint32_t m[3] = {mp, ms, mo};
    build_permutation_pair(ctx, p, s, o, n, m, pso, pos);
    put("p_idx_values", pso.l1_vals);
    put("p_idx_offsets", pso.l1_offs);
    put("ps_data", pso.col1);
    put("pso_data", pso.col2);
    put("ps_s_idx_values", pso.l2_vals);
    put("ps_idx_offsets", pso.l2_offs);
    put("po_data", pos.col1);
    put("pos_data", pos.col2);
    put("po_o_idx_values", pos.l2_vals);
    put("po_idx_offsets", pos.l2_offs);
  }
  if (full) {
    put("s_idx_values", DevArray());
    put("s_idx_offsets", DevArray());
    PermOutputs spo;
    spo.want_col2 = spo.want_l2 = true;
    const uint32_t m1[3] = {ms, mp, mo};
    build_permutation(ctx, s, p, o, n, m1, spo);
    put("spo_data", spo.col2);
    put("sp_p_idx_values", spo.l2_vals);
    put("sp_idx_offsets", spo.l2_offs);
    PermOutputs sop;
    sop.want_col2 = sop.want_l2 = true;
    const uint32_t m2[3] = {ms, mo, mp};
    build_permutation(ctx, s, o, p, n, m2, sop);
    put("sop_data", sop.col2);
    put("so_o_idx_values", sop.l2_vals);
    put("so_idx_offsets", sop.l2_offs);
    PermOutputs os;
    os.want_col1 = os.want_col2 = os.want_l1 = true;
    const uint32_t m3[3] = {mo, ms, mp};
    build_permutation(ctx, o, s, p, n, m3, os);
    put("o_idx_values", os.l1_vals);
    put("o_idx_offsets", os.l1_offs);
    put("os_data", os.col1);
    put("osp_data", os.col2);
    PermOutputs ops;
    ops.want_col2 = ops.want_l2 = true;
    const uint32_t m4[3] = {mo, mp, ms};
    build_permutation(ctx, o, p, s, n, m4, ops);
    put("ops_data", ops.col2);
    put("op_p_idx_values", ops.l2_vals);
    put("op_idx_offsets", ops.l2_offs);
  }
}

// .vds: a sequence of [size_t n][n x uint32] arrays in the order of
// VedasStorage::write (src/VedasStorage.cu:486-516).
static const char* kVdsOrder[] = {"p_idx_values", "p_idx_offsets", "ps_s_idx_values", "ps_idx_offsets",
                                  "po_o_idx_values", "po_idx_offsets", "ps_data", "po_data",
                                  "pso_data", "pos_data"};
static const char* kVdsFullOrder[] = {"s_idx_values", "s_idx_offsets", "sp_p_idx_values",
                                      "sp_idx_offsets", "so_o_idx_values", "so_idx_offsets",
                                      "o_idx_values", "o_idx_offsets", "os_data", "op_p_idx_values",
                                      "op_idx_offsets", "spo_data", "sop_data", "ops_data", "osp_data"};

void write_vds(Index& ix, const char* path) {
  std::ofstream out(path, std::ios::binary);
  if (!out) fail(VG_ERR_INVALID, std::string("cannot open ") + path);
  auto w = [&](const char* name) {
    const std::vector<uint32_t>& v = ix.host_array(name);
    uint64_t n = v.size();
    out.write(reinterpret_cast<const char*>(&n), sizeof(n));
    out.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(n * 4));
  };
  for (const char* n : kVdsOrder) w(n);
  if (ix.full)
    for (const char* n : kVdsFullOrder) w(n);
  if (!out) fail(VG_ERR_INVALID, std::string("write failed: ") + path);
}

// Reads the file in chunks into two page-locked buffers taken in turn: while
// one chunk's host-to-device copy runs, the next chunk is read into the
// other buffer (a buffer is refilled only after its copy's event).  The
// level-1/level-2 index arrays and the level-2 key columns, which the
// host-side lookups search, are kept as host mirrors from the same chunks;
// the other data columns go to the device only (a mirror is copied back on
// request).
void open_vds(Ctx& ctx, const char* path, bool full, Index& ix) {
  std::ifstream in(path, std::ios::binary);
  if (!in) fail(VG_ERR_INVALID, std::string("cannot open ") + path);
  ix.ctx = &ctx;
  ix.full = full;
  constexpr size_t kStageBytes = size_t{64} << 20;
  struct Stage {
    char* p = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
    bool busy = false;
  } st[2];
  auto release = [&] {
    for (Stage& x : st) {
      if (x.done) {
        cudaEventSynchronize(x.done);
        cudaEventDestroy(x.done);
      }
      if (x.p) ctx.give_pinned(x.p, x.cap);
      x = Stage();
    }
  };
  try {
    for (Stage& x : st) {
      x.p = static_cast<char*>(ctx.take_pinned(kStageBytes, &x.cap));
      VG_CUDA(cudaEventCreateWithFlags(&x.done, cudaEventDisableTiming));
    }
    int turn = 0;
    auto r = [&](const char* name, bool mirror) {
      uint64_t n = 0;
      in.read(reinterpret_cast<char*>(&n), sizeof(n));
      if (!in || n > (1ull << 36)) fail(VG_ERR_INVALID, std::string("corrupt .vds array ") + name);
      std::vector<uint32_t>* v = nullptr;
      if (mirror) {
        v = &ix.host[name];
        v->resize(n);
      }
      DevArray d(n ? ctx.alloc<uint32_t>(n) : nullptr, n);
      ix.dev[name] = d;
      const size_t bytes = n * 4;
      for (size_t off = 0; off < bytes;) {
        Stage& x = st[turn];
        turn ^= 1;
        if (x.busy) VG_CUDA(cudaEventSynchronize(x.done));
        const size_t len = std::min(bytes - off, x.cap);
        in.read(x.p, static_cast<std::streamsize>(len));
        if (!in) fail(VG_ERR_INVALID, std::string("truncated .vds array ") + name);
        VG_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(d.ptr) + off, x.p, len, cudaMemcpyHostToDevice,
                                ctx.stream));
        VG_CUDA(cudaEventRecord(x.done, ctx.stream));
        x.busy = true;
        if (v) std::memcpy(reinterpret_cast<char*>(v->data()) + off, x.p, len);
        off += len;
      }
    };
    // the host-side lookups search the level-1/level-2 arrays and the
    // level-2 key columns (ps_data, po_data); the last data column of each
    // permutation stays on the device
    for (const char* n : kVdsOrder)
      r(n, std::strcmp(n, "pso_data") != 0 && std::strcmp(n, "pos_data") != 0);
    if (full)
      for (const char* n : kVdsFullOrder) r(n, std::strstr(n, "_idx_") != nullptr);
    ctx.sync();
  } catch (...) {
    release();
    throw;
  }
  release();
  ix.n = ix.get("pso_data").len;
  // subjects and objects are the level-2 keys and data of PSO (their maxima
  // taken on the device); predicates the level-1 keys
  ix.max_id = 0;
  if (ix.n) {
    uint32_t m3[3] = {0, 0, 0};
    column_max3(ctx, ix.get("ps_data").ptr, ix.get("pso_data").ptr, ix.get("ps_data").ptr, ix.n, m3);
    ix.max_id = std::max(m3[0], m3[1]);
  }
  for (uint32_t v : ix.host_array("p_idx_values")) ix.max_id = std::max(ix.max_id, v);
}

}  // namespace vg
