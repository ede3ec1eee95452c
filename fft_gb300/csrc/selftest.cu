// Self-tests of the bounded waits the kernels use.
//  - afft_gb300_selftest_bounded_wait: a kernel waits on an mbarrier that
//    nothing arrives at, gives up after `iters` polls, sets the error word
//    and returns.
//  - afft_gb300_selftest_tma_wait: the TMA tile wait of the cols passes.  A
//    kernel announces twice the bytes of the one tensor-map copy it issues,
//    so the barrier's phase never completes; the wait (the kernels' own
//    time-bounded helper, with a short limit) gives up, sets the error word
//    and returns.  The one copy it issued lands within microseconds, long
//    before the limit, so nothing is in flight when the CTA exits.
// The host reads the word back; the context stays usable.  No fault, trap or
// hang is involved.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include "../../include/afft_gb300.h"
#include "kernels.h"
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

// one 8-float x 64-row box (2 KB) into shared memory, expecting 4 KB
__global__ void tma_wait_selftest(const __grid_constant__ TmaTile tm, int* err, unsigned long long limit_ns) {
  __shared__ __align__(8) uint64_t mbar;
  __shared__ __align__(128) float buf[2 * 8 * 64];
  const uint32_t mb = smem_u32(&mbar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(2u * 8u * 64u * 4u)
                 : "memory");
    tma_load_3d(smem_u32(buf), &tm.re, 0, 0, 0, mb);
  }
  const bool ok = __syncthreads_and(mbar_wait_ns(mb, 0, limit_ns));
  if (!ok && threadIdx.x == 0) atomicExch(err, AFFT_GB300_ETIMEOUT);
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

extern "C" int afft_gb300_selftest_tma_wait(int limit_us) {
  clear_error();
  void* f = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !f) {
    cudaGetLastError();
    set_error(AFFT_GB300_ECUDA, "tensor-map encoder unavailable");
    return -1;
  }
  auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  float* data = nullptr;
  int* d = nullptr;
  if (cudaMalloc(&data, 64 * 64 * sizeof(float)) != cudaSuccess || cudaMalloc(&d, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    if (data) cudaFree(data);
    set_error(AFFT_GB300_ENOMEM, "self-test allocation failed");
    return -1;
  }
  cudaMemset(data, 0, 64 * 64 * sizeof(float));
  cudaMemset(d, 0, sizeof(int));
  // a 64 x 64 float matrix viewed as {64 columns, 64 rows, 1}; box 8 x 64 at the origin
  TmaTile tm{};
  const cuuint64_t dims[3] = {64, 64, 1};
  const cuuint64_t strides[2] = {64 * sizeof(float), 64 * 64 * sizeof(float)};
  const cuuint32_t box[3] = {8, 64, 1}, estr[3] = {1, 1, 1};
  int v = -1;
  if (encode(&tm.re, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, data, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
      CUDA_SUCCESS) {
    tma_wait_selftest<<<1, 32>>>(tm, d, (unsigned long long)(limit_us < 1 ? 1 : limit_us) * 1000ull);
    if (cudaMemcpy(&v, d, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
      cudaGetLastError();
      set_error(AFFT_GB300_ECUDA, "self-test kernel failed");
      v = -1;
    }
  } else {
    set_error(AFFT_GB300_ECUDA, "tensor-map encoding failed");
  }
  cudaFree(data);
  cudaFree(d);
  return v;   // AFFT_GB300_ETIMEOUT when the wait gave up as designed
}
