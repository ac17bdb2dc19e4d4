// selftest.cu -- a GPU self-test of the device-side bounded waits.
//
// Every spin in the tensor-core kernels (mbarrier waits for tiles, MMA
// commits and bulk copies) gives up after a poll limit, records the failure
// in the scratch error word and leaves through the kernel's one uniform exit,
// which frees the CTA's tensor memory; the host then returns NES_ETIMEDOUT
// and the context stays usable.  neserver's analogue is the 1 s LockTimeout
// of its frame queue (src/base/video/frame_queue.cc:14-22), which turns a
// stuck hand-off into an exception instead of a hang.
//
// The probe kernel runs that same path on demand without faulting anything:
// one CTA allocates tensor memory like the march, thread 0 waits with the
// march's bounded wait (with a short, caller-given poll limit) on an mbarrier
// that nothing arrives at -- or, as the positive control, at which it has
// arrived itself -- the outcome reaches every thread through the same
// barrier reduction the march uses, and all threads leave through the
// fence + __syncthreads + tcgen05.dealloc exit.
#include "kernels.h"
#include "tc_ptx.cuh"

namespace nes {

namespace {

constexpr int kProbeThreads = 128;
constexpr uint32_t kProbeTmemCols = 32;  // the smallest allocation

__global__ void __launch_bounds__(kProbeThreads)
bounded_wait_probe_kernel(uint32_t poll_limit, int arrive, uint32_t* __restrict__ counters) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t slot;
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&slot, kProbeTmemCols);
    tc::tmem_relinquish();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = slot;
  bool ok = true;
  if (threadIdx.x == 0) {
    if (arrive) tc::mbar_arrive(&bar);  // completes phase 0: the wait succeeds
    ok = tc::mbar_wait(&bar, 0, poll_limit);
  }
  // Every thread learns the outcome (no thread is left at a barrier).
  const bool fail = tc::named_sync_or(1, kProbeThreads, !ok);
  if (fail && threadIdx.x == 0) atomicExch(counters + kCtrError, 1u);
  tc::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after();
    tc::tmem_dealloc(tmem, kProbeTmemCols);
  }
}

}  // namespace

cudaError_t launch_bounded_wait_probe(uint32_t poll_limit, int arrive, uint32_t* counters, cudaStream_t stream) {
  if (poll_limit == 0 || poll_limit > tc::kSpinLimit) return cudaErrorInvalidValue;
  bounded_wait_probe_kernel<<<1, kProbeThreads, 0, stream>>>(poll_limit, arrive, counters);
  return cudaGetLastError();
}

}  // namespace nes
