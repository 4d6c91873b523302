// vg_join_noalloc: the sorted inner join for callers that must not allocate
// device memory.
//
// Who needs it: hosts that have already handed all of the GPU's memory to
// their own pools and forbid libraries from calling cudaMalloc/cudaFree (a
// cudaMalloc can also synchronize the device and stall other streams), and
// latency-critical serving threads that may only launch work.  Such a caller
// cannot create a vg_ctx, whose arena is one cudaMalloc.
//
// The join's scratch (per-left-row lower bound, match count and output
// offset, plus the look-back status words) lives in one file-scope
// __device__ array instead.  Its size is fixed: at most kMaxLeftRows left
// rows (about 32 MiB of device memory, held by every GPU that loads this
// library until the process exits).  Host code may not use the array's name
// as a device address, so on the first call on each device, with that device
// current, the entry point looks the address up with cudaGetSymbolAddress and
// keeps it for later calls.  Make that first call before any stream capture.
// All calls share the one array and it keeps the last call's contents: the
// parts that must start at zero are cleared on every call, and calls whose
// work overlaps on the GPU (other streams, other threads) race on it.
#include <map>
#include <mutex>

#include "vg_relops.h"

namespace {

constexpr uint64_t kMaxLeftRows = 1ull << 21;     // 2,097,152 left rows
constexpr uint64_t kTileRows = 2048;              // rows per scan tile (vg_relops.cu)
constexpr uint64_t kMaxTiles = kMaxLeftRows / kTileRows;

struct NoAllocScratch {
  uint32_t lo[kMaxLeftRows];
  uint32_t cnt[kMaxLeftRows];
  uint64_t offs[kMaxLeftRows];
  uint64_t status[kMaxTiles];
  uint64_t total;
  uint32_t ticket;
  uint32_t pad;
  vg::DeviceErrors err;
};

static __device__ __align__(256) NoAllocScratch g_join_scratch;

std::mutex g_mu;
std::map<int, NoAllocScratch*> g_addr;  // device id -> device address of g_join_scratch

NoAllocScratch* scratch_for_current_device() {
  int dev = 0;
  VG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_addr.find(dev);
  if (it != g_addr.end()) return it->second;
  void* p = nullptr;
  VG_CUDA(cudaGetSymbolAddress(&p, g_join_scratch));
  g_addr[dev] = static_cast<NoAllocScratch*>(p);
  return g_addr[dev];
}

thread_local std::string g_err;

}  // namespace

extern "C" const char* vg_noalloc_last_error(void) { return g_err.c_str(); }

extern "C" vg_status vg_join_noalloc(const uint32_t* const* l_cols, uint32_t l_ncols, uint64_t l_rows,
                                     const uint32_t* const* r_cols, uint32_t r_ncols, uint64_t r_rows,
                                     uint32_t* const* out_cols, uint64_t out_capacity, uint64_t* out_rows,
                                     void* stream) {
  if (!l_cols || !r_cols || !out_rows || l_ncols == 0 || r_ncols == 0 || l_ncols > VG_MAX_COLS ||
      r_ncols > VG_MAX_COLS || l_ncols + r_ncols - 1 > VG_MAX_COLS || (out_capacity && !out_cols))
    return VG_ERR_INVALID;
  *out_rows = 0;
  if (l_rows > kMaxLeftRows) {
    g_err = "vg_join_noalloc: the left relation has more than 2097152 rows (its fixed scratch limit)";
    return VG_ERR_OVERFLOW;
  }
  if (r_rows > 0xFFFFFFFFull) {
    g_err = "vg_join_noalloc: the right relation is limited to 2^32 rows";
    return VG_ERR_OVERFLOW;
  }
  try {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    NoAllocScratch* sc = scratch_for_current_device();
    vg::Rel l, r;
    l.ncols = l_ncols;
    l.nrows = l_rows;
    r.ncols = r_ncols;
    r.nrows = r_rows;
    for (uint32_t c = 0; c < l_ncols; ++c) l.cols[c] = const_cast<uint32_t*>(l_cols[c]);
    for (uint32_t c = 0; c < r_ncols; ++c) r.cols[c] = const_cast<uint32_t*>(r_cols[c]);
    // The previous call's contents are still there: zero what the look-back
    // and the error record read before they are written.
    const uint64_t tiles = (l_rows + kTileRows - 1) / kTileRows;
    VG_CUDA(cudaMemsetAsync(sc->status, 0, (tiles ? tiles : 1) * sizeof(uint64_t), s));
    VG_CUDA(cudaMemsetAsync(&sc->total, 0, sizeof(uint64_t), s));
    VG_CUDA(cudaMemsetAsync(&sc->ticket, 0, sizeof(uint32_t), s));
    VG_CUDA(cudaMemsetAsync(&sc->err, 0, sizeof(vg::DeviceErrors), s));
    const uint64_t t = vg::join_into(s, 0, l, r, out_cols, out_capacity, sc->lo, sc->cnt, sc->offs, sc->status,
                                     &sc->ticket, &sc->total, &sc->err);
    vg::DeviceErrors he{};
    VG_CUDA(cudaMemcpyAsync(&he, &sc->err, sizeof(he), cudaMemcpyDeviceToHost, s));
    VG_CUDA(cudaStreamSynchronize(s));
    *out_rows = t;
    if (he.timeout) {
      g_err = "vg_join_noalloc: a bounded device wait expired";
      return VG_ERR_TIMEOUT;
    }
    if (t > out_capacity) {
      g_err = "vg_join_noalloc: the result has more rows than out_capacity (required count in *out_rows)";
      return VG_ERR_OVERFLOW;
    }
    return VG_OK;
  } catch (const vg::Error& e) {
    g_err = e.what();
    return e.status;
  }
}
