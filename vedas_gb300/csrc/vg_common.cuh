// Shared definitions for the VEDAS GB300 query-execution core (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/vedas_gb300.h"

namespace vg {

// An error carrying a vg_status; caught at the C-ABI boundary.
struct Error : std::runtime_error {
  vg_status status;
  Error(vg_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

[[noreturn]] inline void fail(vg_status s, const std::string& m) { throw Error(s, m); }

inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    fail(VG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define VG_CUDA(x) ::vg::check_cuda((x), #x)

// Spin-waits on flags written by other CTAs give up after this many polls,
// record an error and let the kernel finish.
constexpr uint32_t kSpinLimit = 1u << 24;

// Device-side error record, one per context (zeroed on creation).
struct DeviceErrors {
  uint32_t timeout;   // a bounded wait expired
  uint32_t overflow;  // an output did not fit the space reserved for it
};

__host__ __device__ inline uint64_t div_up(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Look-back status words.  A word carries its flag and its value together
// and a reader uses nothing but that value, so the accesses need to be
// single-copy atomic and coherent at GPU scope, not ordered against the
// thread's other memory operations: relaxed loads and stores, without the
// fences that acquire and release semantics add to every publish and probe.
__device__ __forceinline__ uint64_t ld_status_u64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_status_u64(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
#endif  // __CUDACC__

// Look-back status word: 2 flag bits over a 62-bit value.
constexpr uint64_t kFlagAgg = 1ull << 62;
constexpr uint64_t kFlagInc = 2ull << 62;
constexpr uint64_t kValueMask = (1ull << 62) - 1;

}  // namespace vg
