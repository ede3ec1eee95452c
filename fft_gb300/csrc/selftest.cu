// Self-test of the bounded-wait path used by the tensor-core form: a kernel
// waits on an mbarrier that nothing arrives at, gives up after `iters`
// polls, sets the error word and returns.  The host reads the word back; the
// context stays usable.  No fault, trap or hang is involved.
#include <cuda_runtime.h>

#include "../../include/afft_gb300.h"
#include "plan.h"
#include "tc_dft.cuh"

namespace agb {

__global__ void bounded_wait_selftest(int* err, int iters) {
  __shared__ __align__(8) uint64_t mbar;
  if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
  __syncthreads();
  // nobody arrives: phase 0 never completes
  bool done = false;
  for (int it = 0; it < iters && !done; it++) {
    uint32_t d;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(d)
        : "r"(smem_u32(&mbar)));
    done = d != 0;
  }
  if (!done && threadIdx.x == 0) atomicExch(err, AFFT_GB300_ETIMEOUT);
}

}  // namespace agb

using namespace agb;

extern "C" int afft_gb300_selftest_bounded_wait(int iters) {
  clear_error();
  int* d = nullptr;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    set_error(AFFT_GB300_ENOMEM, "self-test allocation failed");
    return -1;
  }
  cudaMemset(d, 0, sizeof(int));
  bounded_wait_selftest<<<1, 32>>>(d, iters < 1 ? 1 : iters);
  int v = -1;
  cudaError_t e = cudaMemcpy(&v, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_error(AFFT_GB300_ECUDA, cudaGetErrorString(e));
    return -1;
  }
  return v;   // AFFT_GB300_ETIMEOUT when the wait gave up as designed
}
