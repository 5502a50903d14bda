// Check of the stage kernel's bounded-wait path without a fault: one thread waits, with a
// given poll budget, on an mbarrier phase that nothing completes (no arrival, no copy), gives
// up, records DEVERR_TMA_TIMEOUT in the solver's device error word exactly as the stage
// kernel does on an expired wait, and invalidates the barrier.  The host then reads the word
// through the same path as after a stage launch.
#include "stage_impl.cuh"

namespace fw {
namespace {

__global__ void wait_timeout_probe(int spins, int* err) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x != 0) return;
  const uint32_t b = smem_u32(&bar);
  mbar_init(b, 1);
  if (!mbar_wait(b, 0, spins)) atomicExch(err, DEVERR_TMA_TIMEOUT);
  mbar_inval(b);
}

}  // namespace

void launch_wait_timeout_probe(int spins, int* err, void* stream) {
  wait_timeout_probe<<<1, 32, 0, (cudaStream_t)stream>>>(spins, err);
}

}  // namespace fw
