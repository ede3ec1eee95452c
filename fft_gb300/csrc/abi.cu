// The C ABI: afft's fft.h entry points (fft.h:22-84, fft.cpp:139-308) and
// the extensions declared in include/afft_gb300.h.
//
// afft builds a plan by placement into caller memory and has no destroy call
// (fft_internal.hpp:114-119, fft.hpp:18-44).  Here the caller's `mem` holds a
// small header (magic, id); the plan object with its device resources lives
// in a registry keyed by that address, replaced if a new plan is created at
// the same address, and freed by afft_gb300_release or at unload.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>

#include "../../include/afft_gb300.h"
#include "plan.h"

namespace agb {

static thread_local int g_err = 0;
static thread_local std::string g_msg;

void set_error(int code, const std::string& msg) {
  g_err = code;
  g_msg = msg;
}
void clear_error() {
  g_err = 0;
  g_msg.clear();
}

// Makes the plan's device current for the duration of a call and restores
// the caller's device afterwards.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
    }
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

static const uint64_t kMagic = 0x3030334247544641ULL;  // "AFTGB300"

struct Header {
  uint64_t magic;
  uint64_t id;
};

struct Registry {
  std::mutex mu;
  std::unordered_map<const void*, std::pair<uint64_t, std::shared_ptr<Plan>>> plans;
  std::atomic<uint64_t> next{1};
};
static Registry& reg() {
  static Registry* r = new Registry();  // leaked on purpose: no teardown-order hazards
  return *r;
}

static std::shared_ptr<Plan> lookup(const void* mem) {
  if (!mem) {
    set_error(AFFT_GB300_ESTATE, "null plan");
    return nullptr;
  }
  Header h;
  std::memcpy(&h, mem, sizeof(h));
  if (h.magic != kMagic) {
    set_error(AFFT_GB300_ESTATE, "not a plan of this library");
    return nullptr;
  }
  auto& R = reg();
  std::lock_guard<std::mutex> g(R.mu);
  auto it = R.plans.find(mem);
  if (it == R.plans.end() || it->second.first != h.id) {
    set_error(AFFT_GB300_ESTATE, "plan released or unknown");
    return nullptr;
  }
  return it->second.second;
}

static int device_ok() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return 0;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return 0;
  return prop.major == 10 && prop.minor == 3;
}

static const size_t kPlanMem = 128;

// memsize checks shared by all kinds: returns 0 when OK, else the value to
// return from memsize (0 for an error, (size_t)-1 for an unknown format)
static size_t check_args(size_t ndim, const size_t* dim, int format, int impl, int* nd, long long* dims) {
  clear_error();
  if (impl != afft_auto && impl != afft_gb300) {
    set_error(AFFT_GB300_EINVAL, "impl selects a CPU backend this library does not have");
    return 0;
  }
  if (format != afft_split && format != afft_interleaved) {
    set_error(AFFT_GB300_EINVAL, "unknown format");
    return (size_t)-1;
  }
  if (ndim > 64 || (ndim > 0 && !dim)) {
    set_error(AFFT_GB300_EINVAL, "bad ndim");
    return 0;
  }
  if (validate_shape((int)ndim, dim, nd, dims)) {
    set_error(AFFT_GB300_EINVAL, "dimensions must be powers of two, at most 2^31 elements");
    return 0;
  }
  if (!device_ok()) {
    set_error(AFFT_GB300_ENODEV, "no GB300 (sm_103) CUDA device");
    return 0;
  }
  return 1;
}

static size_t memsize_impl(int kind, size_t ndim, const size_t* dim, size_t batch, int format, int impl,
                           int form = 0) {
  int nd;
  long long dims[64];
  size_t r = check_args(ndim, dim, format, impl, &nd, dims);
  if (r != 1) return r;
  if (batch == 0) {
    set_error(AFFT_GB300_EINVAL, "batch must be positive");
    return 0;
  }
  // build a throwaway plan so unsupported shapes fail here, as afft's
  // memsize is the call that reports them
  auto P = build_plan(kind, nd, dims, (long long)batch, format, false, form);
  if (!P) return 0;
  return kPlanMem;
}

static void* create_impl(int kind, size_t ndim, const size_t* dim, size_t batch, int format, void* mem,
                         int impl, int form = 0) {
  int nd;
  long long dims[64];
  size_t r = check_args(ndim, dim, format, impl, &nd, dims);
  if (r != 1) return nullptr;
  if (!mem || batch == 0) {
    set_error(AFFT_GB300_EINVAL, "null mem or zero batch");
    return nullptr;
  }
  auto P = build_plan(kind, nd, dims, (long long)batch, format, false, form);
  if (!P) return nullptr;
  // device scratch now, so later launches allocate nothing (and can be
  // captured into CUDA graphs)
  if (P->scratch_elems > 0 && cudaMalloc(&P->scratch, (size_t)P->scratch_elems * P->esize()) != cudaSuccess) {
    cudaGetLastError();
    set_error(AFFT_GB300_ENOMEM, "scratch allocation failed");
    return nullptr;
  }
  // A blocking stream: the synchronous transform calls are ordered after
  // work the caller queued on the default stream (the input is complete),
  // as afft's synchronous calls read finished data.
  if (cudaStreamCreateWithFlags(&P->stream, cudaStreamDefault) != cudaSuccess) {
    cudaGetLastError();
    set_error(AFFT_GB300_ECUDA, "stream creation failed");
    return nullptr;
  }
  auto& R = reg();
  Header h{kMagic, R.next++};
  std::shared_ptr<Plan> sp(P.release());
  {
    std::lock_guard<std::mutex> g(R.mu);
    R.plans[mem] = std::make_pair(h.id, sp);  // replaces a plan built earlier at mem
  }
  std::memcpy(mem, &h, sizeof(h));
  return mem;
}

static bool is_device_ptr(const void* p) {
  if (!p) return true;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Whether the current device reads pageable host memory coherently through
// the host's page tables (address translation services, as on Grace-based
// systems), cached per device.  Devices whose pageable access migrates pages
// instead do not qualify.
static bool device_uses_host_page_tables() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  static std::mutex mu;
  static std::map<int, bool> known;
  std::lock_guard<std::mutex> g(mu);
  auto it = known.find(dev);
  if (it != known.end()) return it->second;
  int pageable = 0, host_tables = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
    cudaGetLastError();
    pageable = host_tables = 0;
  }
  return known[dev] = pageable == 1 && host_tables == 1;
}

// Host memory that kernels can reach at the same address: pinned and mapped
// (cudaHostAlloc / cudaHostRegister), or pageable memory on a device that
// reads it through the host's page tables.
static bool is_direct_host_ptr(const void* p) {
  if (!p) return true;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeHost) return a.devicePointer == p;
  return a.type == cudaMemoryTypeUnregistered && device_uses_host_page_tables();
}

// Whether a launch's accesses to a caller array suit the host link: whole
// lines (rows mode) or tiles of at least 16 adjacent lines (64-byte or wider
// row segments).  Narrower segments crawl across the link (a 64 x 2^20 real
// transform, whose passes touch host memory in 32-byte pieces, ran 3.5x
// slower end to end than with staged copies).
static bool host_access_ok(const Op& op) {
  if (op.type != OP_LINE) return false;
  if (!op.k.cols) return true;
  return op.k.kind == LK_C2C && op.k.lines_per_cta >= 16;
}

// A plan can run on mapped host buffers directly when the caller's arrays are
// touched once each: only the first launch reads src, only the last writes
// dst, and nothing reads dst (no in-place passes over it).  Each element then
// crosses the host link once in each direction, as with staged copies, but
// without the staging buffers and with transfer and compute overlapped.
static bool host_direct_ok(const Plan& P) {
  const size_t n = P.ops.size();
  if (n == 0 || !host_access_ok(P.ops[0]) || !host_access_ok(P.ops[n - 1])) return false;
  for (size_t i = 0; i < n; i++) {
    const Op& op = P.ops[i];
    auto is_src = [](int b) { return b == B_SRC_RE || b == B_SRC_IM; };
    auto is_dst = [](int b) { return b == B_DST_RE || b == B_DST_IM; };
    if ((is_src(op.in.re.buf) || is_src(op.in.im.buf)) && i != 0) return false;
    if (is_dst(op.in.re.buf) || is_dst(op.in.im.buf)) return false;
    if ((is_dst(op.out.re.buf) || is_dst(op.out.im.buf)) && i != n - 1) return false;
    if (is_src(op.out.re.buf) || is_src(op.out.im.buf)) return false;
  }
  return n > 0;
}

// Elements per array of one call: input and output, for each data argument
static void io_elems(const Plan& P, long long* in_n, long long* out_n) {
  *in_n = P.in_elems * P.batch;
  *out_n = P.out_elems * P.batch;
}

// A kernel whose bounded wait gave up (a TC-form kernel waiting for its
// tensor-core results: 1; a cols pass waiting for its TMA-loaded tile: 2)
// sets the device error word instead of hanging; report and clear it.
static int check_tc_error(const Plan& P) {
  if (P.form != FORM_TC && !P.has_tma) return 0;
  int* w = tc_error_word();
  int v = 0;
  if (w && cudaMemcpy(&v, w, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && v) {
    cudaMemset(w, 0, sizeof(int));
    set_error(AFFT_GB300_ETIMEOUT, v == 2 ? "TMA tile wait timed out" : "tensor-core stage wait timed out");
    return AFFT_GB300_ETIMEOUT;
  }
  return 0;
}

// The data arguments a plan reads and writes: src_re and dst_re always, the
// im arrays of complex split data.  A missing one is reported, never
// launched on (a kernel would fault on it).
static bool data_args(const Plan& P, const float* sr, const float* si, const float* dr, const float* di,
                      bool* use_si, bool* use_di) {
  const bool real_in = P.kind == K_R, real_out = P.kind == K_RI;
  const bool inter = P.format == afft_interleaved;
  *use_si = !real_in && !inter;
  *use_di = !real_out && !inter;
  if (!sr || !dr || (*use_si && !si) || (*use_di && !di)) {
    set_error(AFFT_GB300_EINVAL, "a data pointer this transform reads or writes is NULL");
    return false;
  }
  // the FP64 kernels load and store whole doubles: a misaligned double array
  // (possible only through casts) is reported, never launched on
  if (P.f64()) {
    auto mis = [](const float* p) { return (reinterpret_cast<uintptr_t>(p) & 7) != 0; };
    if (mis(sr) || mis(dr) || (*use_si && mis(si)) || (*use_di && mis(di))) {
      set_error(AFFT_GB300_EINVAL, "an FP64 data pointer is not 8-byte aligned");
      return false;
    }
  }
  return true;
}

// f64: the call is one of the afft_64_* transforms (data are doubles, passed
// here as float pointers); a plan of the other precision is refused.
static int transform_sync(void* plan, const float* sr, const float* si, float* dr, float* di, bool f64 = false) {
  clear_error();
  auto P = lookup(plan);
  if (!P) return AFFT_GB300_ESTATE;
  if (P->f64() != f64) {
    set_error(AFFT_GB300_EINVAL, f64 ? "an FP32 plan passed to an afft_64 transform"
                                     : "an FP64 plan passed to an afft_32 transform");
    return AFFT_GB300_EINVAL;
  }
  std::lock_guard<std::mutex> g(P->mu);
  DeviceGuard dg(P->device);
  const bool real_in = P->kind == K_R, real_out = P->kind == K_RI;
  const bool inter = P->format == afft_interleaved;
  // arguments that carry data for this kind/format
  bool use_si, use_di;
  if (!data_args(*P, sr, si, dr, di, &use_si, &use_di)) return AFFT_GB300_EINVAL;
  bool dev = is_device_ptr(sr) && is_device_ptr(dr) && (!use_si || is_device_ptr(si)) &&
             (!use_di || is_device_ptr(di));
  if (dev) {
    int rc = P->launch(sr, use_si ? si : nullptr, dr, use_di ? di : nullptr, P->stream);
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(P->stream);
    if (e != cudaSuccess) {
      set_error(AFFT_GB300_ECUDA, cudaGetErrorString(e));
      return AFFT_GB300_ECUDA;
    }
    return check_tc_error(*P);
  }
  // host data the kernels can reach: run on it directly when the plan
  // touches each caller array once (measured on GB300 for a 512 MB array
  // pair: 3.3 ms pinned and 5.1 ms pageable, against 6.3 ms for pageable
  // data staged through copies)
  bool mapped = is_direct_host_ptr(sr) && is_direct_host_ptr(dr) && (!use_si || is_direct_host_ptr(si)) &&
                (!use_di || is_direct_host_ptr(di));
  if (mapped && P->form != FORM_TC && host_direct_ok(*P)) {
    int rc = P->launch(sr, use_si ? si : nullptr, dr, use_di ? di : nullptr, P->stream);
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(P->stream);
    if (e != cudaSuccess) {
      set_error(AFFT_GB300_ECUDA, cudaGetErrorString(e));
      return AFFT_GB300_ECUDA;
    }
    return 0;
  }
  // host data: stage through plan-owned device buffers.  A batch is cut
  // into chunks so the copy of chunk i+1 in, the transform of chunk i and the
  // copy of chunk i-1 out overlap (three streams, ordered by events).
  long long in_n, out_n;
  io_elems(*P, &in_n, &out_n);
  const size_t esz = P->esize();
  const size_t fin = (size_t)in_n * (inter && !real_in ? 2 : 1) * esz;   // bytes of src_re
  const size_t fout = (size_t)out_n * (inter && !real_out ? 2 : 1) * esz;
  const size_t need = fin + (use_si ? fin : 0) + fout + (use_di ? fout : 0);
  if (P->stage_bytes < need) {
    if (P->stage) cudaFree(P->stage);
    P->stage = nullptr;
    P->stage_bytes = 0;
    if (cudaMalloc(&P->stage, need) != cudaSuccess) {
      cudaGetLastError();
      set_error(AFFT_GB300_ENOMEM, "staging allocation failed");
      return AFFT_GB300_ENOMEM;
    }
    P->stage_bytes = need;
  }
  char* d_sr = reinterpret_cast<char*>(P->stage);
  char* d_si = use_si ? d_sr + fin : nullptr;
  char* d_dr = d_sr + fin + (use_si ? fin : 0);
  char* d_di = use_di ? d_dr + fout : nullptr;
  const char* h_sr = reinterpret_cast<const char*>(sr);
  const char* h_si = reinterpret_cast<const char*>(si);
  char* h_dr = reinterpret_cast<char*>(dr);
  char* h_di = reinterpret_cast<char*>(di);
  if (!P->copy_in) {
    // chunking: the largest divisor of the batch up to 8, for batches whose
    // data is worth overlapping (>= 8 MiB)
    long long k = 1;
    if (need >= (8u << 20))
      for (long long d = 8; d >= 2; d--)
        if (P->batch % d == 0) { k = d; break; }
    if (k > 1) {
      P->chunk = build_plan(P->kind, P->ndim, P->dims, P->batch / k, P->format, false, P->form);
      if (!P->chunk) k = 1;
    }
    // streams and events are set up all or nothing: copy_in, set last,
    // marks them ready
    cudaStream_t s_in = nullptr, s_out = nullptr;
    std::vector<cudaEvent_t> ev(2 * k, nullptr);
    bool ok = cudaStreamCreateWithFlags(&s_in, cudaStreamDefault) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s_out, cudaStreamDefault) == cudaSuccess;
    for (auto& e : ev) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      for (auto e : ev)
        if (e) cudaEventDestroy(e);
      if (s_in) cudaStreamDestroy(s_in);
      if (s_out) cudaStreamDestroy(s_out);
      set_error(AFFT_GB300_ECUDA, "stream or event creation failed");
      return AFFT_GB300_ECUDA;
    }
    P->nchunks = k;
    P->ev = std::move(ev);
    P->copy_out = s_out;
    P->copy_in = s_in;
  }
  const long long k = P->nchunks;
  const size_t cin = fin / k, cout = fout / k;    // bytes per chunk, per array
  auto f = [](char* p) { return reinterpret_cast<float*>(p); };
  // the first error of any enqueue call (a rejected copy is reported by the
  // call itself, not by a later synchronize)
  cudaError_t ce = cudaSuccess;
  auto chk = [&ce](cudaError_t r) {
    if (ce == cudaSuccess) ce = r;
  };
  for (long long i = 0; i < k; i++) {
    chk(cudaMemcpyAsync(d_sr + i * cin, h_sr + i * cin, cin, cudaMemcpyDefault, P->copy_in));
    if (use_si) chk(cudaMemcpyAsync(d_si + i * cin, h_si + i * cin, cin, cudaMemcpyDefault, P->copy_in));
    chk(cudaEventRecord(P->ev[2 * i], P->copy_in));
  }
  Plan& C = k > 1 ? *P->chunk : *P;
  int rc = 0;
  for (long long i = 0; i < k; i++) {
    chk(cudaStreamWaitEvent(P->stream, P->ev[2 * i], 0));
    rc = C.launch(f(d_sr + i * cin), use_si ? f(d_si + i * cin) : nullptr, f(d_dr + i * cout),
                  use_di ? f(d_di + i * cout) : nullptr, P->stream);
    if (rc) break;
    chk(cudaEventRecord(P->ev[2 * i + 1], P->stream));
    chk(cudaStreamWaitEvent(P->copy_out, P->ev[2 * i + 1], 0));
    chk(cudaMemcpyAsync(h_dr + i * cout, d_dr + i * cout, cout, cudaMemcpyDefault, P->copy_out));
    if (use_di) chk(cudaMemcpyAsync(h_di + i * cout, d_di + i * cout, cout, cudaMemcpyDefault, P->copy_out));
  }
  // every copy from or to the caller's memory has ended when the call returns
  cudaError_t e = cudaStreamSynchronize(P->copy_in);
  if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(P->copy_out);
  if (rc) {
    cudaGetLastError();
    return rc;   // the launch reported its own error
  }
  if (e == cudaSuccess) e = ce;
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(AFFT_GB300_ECUDA, cudaGetErrorString(e));
    return AFFT_GB300_ECUDA;
  }
  return check_tc_error(*P);
}

// double arrays of the afft_64_* calls, as the float pointers the plans bind
static const float* cfp(const double* p) { return reinterpret_cast<const float*>(p); }
static float* mfp(double* p) { return reinterpret_cast<float*>(p); }

}  // namespace agb

using namespace agb;

extern "C" {

// ---- fft.h:22-26 ----------------------------------------------------------
size_t afft_32_c_memsize(size_t ndim, const size_t* dim, int format, int impl) {
  return memsize_impl(K_C, ndim, dim, 1, format, impl);
}
afft_32_c_type* afft_32_c_create(size_t ndim, const size_t* dim, int format, void* mem, int impl) {
  return (afft_32_c_type*)create_impl(K_C, ndim, dim, 1, format, mem, impl);
}
void afft_32_c_transform(afft_32_c_type* st, const float* sr, const float* si, float* dr, float* di) {
  transform_sync(st, sr, si, dr, di);
}

// ---- fft.h:28-32 ----------------------------------------------------------
size_t afft_32_ci_memsize(size_t ndim, const size_t* dim, int format, int impl) {
  return memsize_impl(K_CI, ndim, dim, 1, format, impl);
}
afft_32_ci_type* afft_32_ci_create(size_t ndim, const size_t* dim, int format, void* mem, int impl) {
  return (afft_32_ci_type*)create_impl(K_CI, ndim, dim, 1, format, mem, impl);
}
void afft_32_ci_transform(afft_32_ci_type* st, const float* sr, const float* si, float* dr, float* di) {
  transform_sync(st, sr, si, dr, di);
}

// ---- fft.h:34-38 ----------------------------------------------------------
size_t afft_32_r_memsize(size_t ndim, const size_t* dim, int format, int impl) {
  return memsize_impl(K_R, ndim, dim, 1, format, impl);
}
afft_32_r_type* afft_32_r_create(size_t ndim, const size_t* dim, int format, void* mem, int impl) {
  return (afft_32_r_type*)create_impl(K_R, ndim, dim, 1, format, mem, impl);
}
void afft_32_r_transform(afft_32_r_type* st, const float* src, float* dr, float* di) {
  transform_sync(st, src, nullptr, dr, di);
}

// ---- fft.h:40-44 ----------------------------------------------------------
size_t afft_32_ri_memsize(size_t ndim, const size_t* dim, int format, int impl) {
  return memsize_impl(K_RI, ndim, dim, 1, format, impl);
}
afft_32_ri_type* afft_32_ri_create(size_t ndim, const size_t* dim, int format, void* mem, int impl) {
  return (afft_32_ri_type*)create_impl(K_RI, ndim, dim, 1, format, mem, impl);
}
void afft_32_ri_transform(afft_32_ri_type* st, const float* sr, const float* si, float* dst) {
  transform_sync(st, sr, si, dst, nullptr);
}

// ---- fft.h:46 / common.hpp:173-176 ------------------------------------------
size_t afft_32_align_size(size_t sz) { return (sz + 15) & ~(size_t)15; }

// ---- fft.h:48-80: the same transforms on doubles (FP64 kernels) --------------
size_t afft_64_c_memsize(size_t ndim, const size_t* dim, int format, int impl) {
  return memsize_impl(K_C, ndim, dim, 1, format, impl, FORM_F64);
}
afft_64_c_type* afft_64_c_create(size_t ndim, const size_t* dim, int format, void* mem, int impl) {
  return (afft_64_c_type*)create_impl(K_C, ndim, dim, 1, format, mem, impl, FORM_F64);
}
void afft_64_c_transform(afft_64_c_type* st, const double* sr, const double* si, double* dr, double* di) {
  transform_sync(st, cfp(sr), cfp(si), mfp(dr), mfp(di), true);
}
size_t afft_64_ci_memsize(size_t ndim, const size_t* dim, int format, int impl) {
  return memsize_impl(K_CI, ndim, dim, 1, format, impl, FORM_F64);
}
afft_64_ci_type* afft_64_ci_create(size_t ndim, const size_t* dim, int format, void* mem, int impl) {
  return (afft_64_ci_type*)create_impl(K_CI, ndim, dim, 1, format, mem, impl, FORM_F64);
}
void afft_64_ci_transform(afft_64_ci_type* st, const double* sr, const double* si, double* dr, double* di) {
  transform_sync(st, cfp(sr), cfp(si), mfp(dr), mfp(di), true);
}
size_t afft_64_r_memsize(size_t ndim, const size_t* dim, int format, int impl) {
  return memsize_impl(K_R, ndim, dim, 1, format, impl, FORM_F64);
}
afft_64_r_type* afft_64_r_create(size_t ndim, const size_t* dim, int format, void* mem, int impl) {
  return (afft_64_r_type*)create_impl(K_R, ndim, dim, 1, format, mem, impl, FORM_F64);
}
void afft_64_r_transform(afft_64_r_type* st, const double* src, double* dr, double* di) {
  transform_sync(st, cfp(src), nullptr, mfp(dr), mfp(di), true);
}
size_t afft_64_ri_memsize(size_t ndim, const size_t* dim, int format, int impl) {
  return memsize_impl(K_RI, ndim, dim, 1, format, impl, FORM_F64);
}
afft_64_ri_type* afft_64_ri_create(size_t ndim, const size_t* dim, int format, void* mem, int impl) {
  return (afft_64_ri_type*)create_impl(K_RI, ndim, dim, 1, format, mem, impl, FORM_F64);
}
void afft_64_ri_transform(afft_64_ri_type* st, const double* sr, const double* si, double* dst) {
  transform_sync(st, cfp(sr), cfp(si), mfp(dst), nullptr, true);
}

// ---- fft.h:80 / common.hpp:173-176: 64 bytes of doubles = 8 elements --------
size_t afft_64_align_size(size_t sz) { return (sz + 7) & ~(size_t)7; }

// ---- fft.h:82-84 ------------------------------------------------------------
int afft_supported(int impl) {
  if (impl != afft_auto && impl != afft_gb300) return 0;
  return device_ok();
}

const size_t afft_alignment = 64;

// ---- extensions ---------------------------------------------------------------
int afft_gb300_last_error(void) { return g_err; }
const char* afft_gb300_last_error_string(void) { return g_msg.c_str(); }

// the form flags of a batched or describe call; false when both are set
static bool split_form(int* format, int* form) {
  *form = *format & (FORM_TC | FORM_F64);
  *format &= ~(FORM_TC | FORM_F64);
  return *form != (FORM_TC | FORM_F64);
}

size_t afft_gb300_batch_memsize(int kind, size_t ndim, const size_t* dim, size_t batch, int format) {
  int form;
  if (kind < 0 || kind > 3 || !split_form(&format, &form)) {
    set_error(AFFT_GB300_EINVAL, "bad kind or form");
    return 0;
  }
  return memsize_impl(kind, ndim, dim, batch, format, afft_auto, form);
}

void* afft_gb300_batch_create(int kind, size_t ndim, const size_t* dim, size_t batch, int format, void* mem) {
  int form;
  if (kind < 0 || kind > 3 || !split_form(&format, &form)) {
    set_error(AFFT_GB300_EINVAL, "bad kind or form");
    return nullptr;
  }
  return create_impl(kind, ndim, dim, batch, format, mem, afft_auto, form);
}

int afft_gb300_transform_async(void* plan, const float* sr, const float* si, float* dr, float* di,
                               void* stream) {
  clear_error();
  auto P = lookup(plan);
  if (!P) return AFFT_GB300_ESTATE;
  std::lock_guard<std::mutex> g(P->mu);
  DeviceGuard dg(P->device);
  bool use_si, use_di;
  if (!data_args(*P, sr, si, dr, di, &use_si, &use_di)) return AFFT_GB300_EINVAL;
  // NULL is the CUDA default stream, as for a kernel launch
  return P->launch(sr, use_si ? si : nullptr, dr, use_di ? di : nullptr, (cudaStream_t)stream);
}

int afft_gb300_release(void* plan) {
  clear_error();
  if (!lookup(plan)) return AFFT_GB300_ESTATE;
  auto& R = reg();
  std::shared_ptr<Plan> victim;
  {
    std::lock_guard<std::mutex> g(R.mu);
    auto it = R.plans.find(plan);
    if (it != R.plans.end()) {
      victim = it->second.second;
      R.plans.erase(it);
    }
  }
  Header h{0, 0};
  std::memcpy(plan, &h, sizeof(h));
  return 0;
}

size_t afft_gb300_plan_describe(int kind, size_t ndim, const size_t* dim, size_t batch, int format,
                                char* buf, size_t buflen) {
  clear_error();
  int nd;
  long long dims[64];
  int form;
  if (kind < 0 || kind > 3 || !split_form(&format, &form) || ndim > 64 || (ndim && !dim) || batch == 0 ||
      (format != afft_split && format != afft_interleaved) || validate_shape((int)ndim, dim, &nd, dims)) {
    set_error(AFFT_GB300_EINVAL, "bad arguments");
    return 0;
  }
  auto P = build_plan(kind, nd, dims, (long long)batch, format, true, form);
  if (!P) return 0;
  std::string s = describe_plan(*P);
  if (buf && buflen) {
    size_t n = std::min(buflen - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return s.size() + 1;
}

int afft_gb300_plan_launches(const void* plan) {
  auto P = lookup(plan);
  return P ? (int)P->ops.size() : -1;
}

}  // extern "C"
