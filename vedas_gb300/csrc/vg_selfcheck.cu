// Self-check of the bounded device waits: each kernel waits on something
// that never happens (a look-back status word nobody publishes, an mbarrier
// expecting bytes no copy delivers) and must give up with a timeout status
// that the host reads, leaving the context usable.  Nothing faults or hangs.
#include "vg_selfcheck.h"

#include "vg_prims.cuh"

namespace vg {
namespace {

__global__ void status_never_kernel(const uint64_t* word, DeviceErrors* err) {
  if (threadIdx.x == 0) (void)wait_status(word, err);
}

__global__ void mbar_never_kernel(DeviceErrors* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_arrive_expect_tx(&bar, 16);   // 16 bytes announced; no copy is issued
  }
  __syncthreads();
  if (threadIdx.x == 0) (void)mbar_wait_bounded(&bar, 0, err);
}

}  // namespace

void selfcheck_bounded_wait(Ctx& ctx, int which) {
  if (which == 0) {
    Scratch<uint64_t> word(ctx, 1);
    VG_CUDA(cudaMemsetAsync(word.get(), 0, sizeof(uint64_t), ctx.stream));
    status_never_kernel<<<1, 32, 0, ctx.stream>>>(word.get(), ctx.d_err);
  } else {
    mbar_never_kernel<<<1, 32, 0, ctx.stream>>>(ctx.d_err);
  }
  VG_CUDA(cudaGetLastError());
  ctx.check_device_errors();   // raises VG_ERR_TIMEOUT and clears the record
}

}  // namespace vg
