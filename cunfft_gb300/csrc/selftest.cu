// selftest.cu -- failure-reporting check: a kernel whose completion wait gives up.
//
// The tensor-core kernels wait on mbarriers with a bounded number of polls; a wait that
// gives up sets the plan's device status flag, and cunfft_x_synchronize reports it.
// k_wait_gives_up runs that same bounded wait on an mbarrier that nothing arrives on,
// with a short bound (polls x <= 1 us each), so the report path can be exercised on a
// GPU without a fault or a hang.
#include "runtime.h"
#include "tc_sm100.cuh"

namespace cg {

__global__ void k_wait_gives_up(int32_t* status, uint32_t polls) {
  __shared__ uint64_t bar;
  if (threadIdx.x != 0) return;
  tc::mbar_init(&bar, 1);
  tc::mbar_fence_init();
  if (!tc::mbar_wait_bounded(&bar, 0u, polls)) atomicExch(status, 3);
}

cudaError_t launch_wait_gives_up(int32_t* status, cudaStream_t st) {
  k_wait_gives_up<<<1, 32, 0, st>>>(status, 1000u);
  return cudaGetLastError();
}

}  // namespace cg
