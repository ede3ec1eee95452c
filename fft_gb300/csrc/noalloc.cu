// afft_gb300_c2c_noalloc: a batched 1D complex transform that allocates
// nothing.  Some callers cannot allocate device memory when they call an FFT:
// programs that reserve their whole device memory budget at start-up and
// forbid later allocations, code running under a custom device allocator
// that owns all free memory, and latency-critical loops where cudaMalloc's
// implicit device synchronisation is not acceptable.  For them this entry
// point runs the two-pass (four-step) transform -- the path that needs
// scratch -- with its scratch and twiddle tables in fixed, file-scope device
// arrays instead of plan-owned allocations.
//
// Limits and sharing:
//  - n a power of two in [2^15, 2^21], n * batch <= 2^21 complex elements
//    (the scratch array is 16 MiB; every GPU that loads the library holds it
//    until the process exits); larger requests fail with AFFT_GB300_EINVAL;
//  - all calls on a device share the one scratch array and it keeps the last
//    call's contents; the first pass overwrites every scratch element the
//    second pass reads, so nothing needs clearing, but calls whose kernels
//    overlap on the GPU (different streams, no ordering) race on it;
//  - the first call on each device does the set-up (fills the twiddle
//    arrays with cudaMemcpyToSymbol and looks up the arrays' device addresses
//    with cudaGetSymbolAddress, with that device current); make that first
//    call before any stream capture.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/afft_gb300.h"
#include "plan.h"

namespace agb {

constexpr long long kNoallocMaxElems = 1LL << 21;   // complex elements per call
constexpr int kNoallocMinLog = 15, kNoallocMaxLog = 21;
constexpr int kNoallocLineMaxLog = 11;               // four-step passes use lines <= 2^11

template <int... Ls>
constexpr int stage_total(std::integer_sequence<int, Ls...>) {
  return (Sched<Ls>::twsize() + ... + 0);
}
constexpr int kStageTotal = stage_total(std::make_integer_sequence<int, kNoallocLineMaxLog + 1>{});

static __device__ __align__(256) float g_noalloc_scratch[2 * kNoallocMaxElems];
static __device__ __align__(256) float2 g_noalloc_stage[kStageTotal + 1];
static __device__ __align__(256) float2 g_noalloc_hi[kNoallocMaxLog - kNoallocMinLog + 1][2048];
static __device__ __align__(256) float2 g_noalloc_lo[kNoallocMaxLog - kNoallocMinLog + 1][2048];

struct NoallocDevice {
  bool ready = false;
  float* scratch = nullptr;
  float2* stage = nullptr;
  float2* hi = nullptr;
  float2* lo = nullptr;
  int stage_off[kNoallocLineMaxLog + 1] = {0};
  int lo_bits[kNoallocMaxLog + 1] = {0};
};

static std::mutex g_noalloc_mu;
static NoallocDevice g_noalloc_dev[64];

static int noalloc_setup(int dev, NoallocDevice** out) {
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (dev < 0 || dev >= 64) {
    set_error(AFFT_GB300_ENODEV, "device index out of range");
    return AFFT_GB300_ENODEV;
  }
  NoallocDevice& D = g_noalloc_dev[dev];
  if (!D.ready) {
    std::vector<float2> stage;
    for (int l = 0; l <= kNoallocLineMaxLog; l++) {
      D.stage_off[l] = (int)stage.size();
      std::vector<float2> t = stage_table_host(l);
      stage.insert(stage.end(), t.begin(), t.end());
    }
    cudaError_t e = cudaMemcpyToSymbol(g_noalloc_stage, stage.data(), stage.size() * sizeof(float2));
    for (int l = kNoallocMinLog; l <= kNoallocMaxLog && e == cudaSuccess; l++) {
      std::vector<float2> hi, lo;
      fourstep_table_host(1LL << l, &hi, &lo, &D.lo_bits[l]);
      size_t row = (size_t)(l - kNoallocMinLog) * 2048 * sizeof(float2);
      e = cudaMemcpyToSymbol(g_noalloc_hi, hi.data(), hi.size() * sizeof(float2), row);
      if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_noalloc_lo, lo.data(), lo.size() * sizeof(float2), row);
    }
    // the arrays' device addresses, looked up with this device current
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&D.scratch, g_noalloc_scratch);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&D.stage, g_noalloc_stage);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&D.hi, g_noalloc_hi);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&D.lo, g_noalloc_lo);
    // the copies above come from pageable host memory and may return before
    // their DMA lands; the kernels run on the caller's stream, which need not
    // order after the default stream, so wait here once
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error(AFFT_GB300_ECUDA, std::string("no-alloc set-up failed: ") + cudaGetErrorString(e));
      return AFFT_GB300_ECUDA;
    }
    D.ready = true;
  }
  *out = &D;
  return 0;
}

static LineIO noalloc_bind(const IOSpec& s, float* const* base) {
  LineIO o;
  o.re = base[s.re.buf] + s.re.off;
  o.im = base[s.im.buf] + s.im.off;
  o.es = s.es;
  o.lo = s.lo;
  o.hi = s.hi;
  o.qshift = s.qshift;
  o.qmask = s.qmask;
  return o;
}

}  // namespace agb

using namespace agb;

extern "C" int afft_gb300_c2c_noalloc(const float* src_re, const float* src_im, float* dst_re, float* dst_im,
                                      size_t n, size_t batch, int inverse, void* stream) {
  clear_error();
  // batch is compared by division: n * batch can wrap in 64 bits
  if (n < (1u << kNoallocMinLog) || n > (1u << kNoallocMaxLog) || (n & (n - 1)) || batch == 0 ||
      batch > (size_t)kNoallocMaxElems / n) {
    set_error(AFFT_GB300_EINVAL,
              "no-alloc transform: n must be a power of two in [2^15, 2^21] and n*batch <= 2^21 "
              "(its scratch is a fixed 16 MiB device array)");
    return AFFT_GB300_EINVAL;
  }
  if (!src_re || !src_im || !dst_re || !dst_im) {
    set_error(AFFT_GB300_EINVAL, "null data pointer");
    return AFFT_GB300_EINVAL;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    set_error(AFFT_GB300_ENODEV, "no CUDA device");
    return AFFT_GB300_ENODEV;
  }
  NoallocDevice* D = nullptr;
  if (int rc = noalloc_setup(dev, &D)) return rc;
  long long dims[1] = {(long long)n};
  // the launch list of the ordinary plan in its two-pass form (the one the
  // fixed scratch array is sized for), built without touching the device
  Tuning two;
  two.passes = 2;
  auto P = build_plan(inverse ? K_CI : K_C, 1, dims, (long long)batch, afft_split, true, 0, &two);
  if (!P || P->scratch_elems > 2 * kNoallocMaxElems) {
    set_error(AFFT_GB300_EINVAL, "no-alloc transform: unsupported shape");
    return AFFT_GB300_EINVAL;
  }
  float* base[B_NBUF] = {(float*)src_re, (float*)src_im, dst_re, dst_im, D->scratch};
  int lN = 0;
  while ((1ULL << lN) < n) lN++;
  for (const Op& op : P->ops) {
    if (op.type != OP_LINE || op.k.logl > kNoallocLineMaxLog) {
      set_error(AFFT_GB300_EINVAL, "no-alloc transform: unsupported pass");
      return AFFT_GB300_EINVAL;
    }
    LineParams p = op.p;
    p.in = noalloc_bind(op.in, base);
    p.out = noalloc_bind(op.out, base);
    p.tw = D->stage + D->stage_off[op.k.logl];
    if (p.tw_n) {
      p.tw_full = nullptr;   // the static tables are the hi/lo pair
      p.tw_hi = D->hi + (size_t)(lN - kNoallocMinLog) * 2048;
      p.tw_lo = D->lo + (size_t)(lN - kNoallocMinLog) * 2048;
      p.tw_lo_bits = D->lo_bits[lN];
    }
    if (op.k.smem > 48 * 1024 &&
        cudaFuncSetAttribute((const void*)op.k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)op.k.smem) !=
            cudaSuccess) {
      cudaGetLastError();
      set_error(AFFT_GB300_ECUDA, "kernel shared memory configuration failed");
      return AFFT_GB300_ECUDA;
    }
    op.k.fn<<<(unsigned)op.grid, op.threads, op.smem, (cudaStream_t)stream>>>(p);
    // stop at the first failed pass: a later pass would read stale scratch
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error(AFFT_GB300_ECUDA, std::string("kernel launch failed (pass ") + std::to_string(&op - P->ops.data()) +
                                      "): " + cudaGetErrorString(e));
      return AFFT_GB300_ECUDA;
    }
  }
  return 0;
}
