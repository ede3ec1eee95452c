// Autotuner: per (device, kind, dims, batch, format), time the plan variants
// the shape allows and keep the fastest for later plans.
//
// The variants (Tuning in plan.h) are choices the fixed rules make
// otherwise:
//  - the four-step split of axes too long for one CTA (which half the first
//    pass takes);
//  - for long 1D real inverses, the real pre-pass riding in the first
//    four-step pass (over mirrored column pairs) or standalone;
//  - cols passes loading their input tiles by TMA or through the LSU, and the
//    1024- and 2048-point ones in the persistent pipelined form or one tile per
//    CTA;
//  - the tile width (lines per CTA) of 256- and 512-point complex cols passes;
//  - the plain FP32 form or the split-precision tensor-core form of the
//    passes that have one;
//  - 1D complex axes of 2^20 to 2^22 points in two passes or three;
//  - the last two axes of complex N-D transforms in one plane-fused pass or
//    one pass each (fusion depth; no_plane 0 the rule, 1 per axis, 2 fused
//    at any plane count).
// Each distinct variant (distinct kernels or launch shapes) is built as a
// device plan and timed with CUDA events on zeroed buffers of the current
// device (2 warm-up and 5 timed launches, median).  Choices live in a
// process-wide table and, when AFFT_GB300_TUNE_CACHE names a file, in that
// file (one entry per line, loaded on first use, rewritten after each
// tuning).  AFFT_GB300_AUTOTUNE=1 tunes every new shape when its first plan
// is built.  Queues created with AFFT_GB300_QUEUE_TUNED tune each distinct
// shape of their transforms at a batch of about 2^24 elements and keep the
// choice under batch 0 (the queue's entry for that shape).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/afft_gb300.h"
#include "plan.h"

namespace agb {

namespace {

struct Entry {
  Tuning t;
  double ms = -1;   // median time of the chosen variant (-1: nothing to choose)
};

struct TuneCache {
  std::mutex mu;
  std::map<std::string, Entry> table;
  bool loaded = false;
  std::string path;
};

TuneCache& cache() {
  static TuneCache* c = new TuneCache();   // never destroyed: used by static plans
  return *c;
}

thread_local bool in_tuning = false;

std::string device_name() {
  int dev = 0;
  cudaDeviceProp prop;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    cudaGetLastError();
    return "unknown";
  }
  std::string s = prop.name;
  for (auto& ch : s)
    if (ch == ' ' || ch == '"' || ch == '|') ch = '_';
  return s;
}

std::string key_of(int kind, int ndim, const long long* dims, long long batch, int format) {
  std::string k = device_name() + "|" + std::to_string(kind) + "|";
  for (int i = 0; i < ndim; i++) k += (i ? "x" : "") + std::to_string(dims[i]);
  k += "|" + std::to_string(batch) + "|" + std::to_string(format);
  return k;
}

// file format: a JSON object, one entry per line:
//   "<key>": {"split": S, "real_inv": R, "cols_lsu": U, "tc": T, "cols_c": C, "passes": P,
//             "no_plane": N, "no_pipe": Q, "ms": M},
// (entries of the older forms, without no_pipe, no_plane, passes or cols_lsu /
// tc / cols_c, still load)
void load_locked(TuneCache& C) {
  if (C.loaded) return;
  C.loaded = true;
  const char* p = std::getenv("AFFT_GB300_TUNE_CACHE");
  if (!p || !*p) return;
  C.path = p;
  FILE* f = std::fopen(p, "r");
  if (!f) return;
  char line[1024];
  while (std::fgets(line, sizeof line, f)) {
    char* a = std::strchr(line, '"');
    if (!a) continue;
    char* b = std::strchr(a + 1, '"');
    if (!b) continue;
    Entry e;
    if (std::sscanf(b + 1,
                    " : {\"split\": %d, \"real_inv\": %d, \"cols_lsu\": %d, \"tc\": %d, \"cols_c\": %d, "
                    "\"passes\": %d, \"no_plane\": %d, \"no_pipe\": %d, \"ms\": %lf",
                    &e.t.split, &e.t.real_inv, &e.t.cols_lsu, &e.t.tc, &e.t.cols_c, &e.t.passes, &e.t.no_plane,
                    &e.t.no_pipe, &e.ms) == 9 ||
        std::sscanf(b + 1,
                    " : {\"split\": %d, \"real_inv\": %d, \"cols_lsu\": %d, \"tc\": %d, \"cols_c\": %d, "
                    "\"passes\": %d, \"no_plane\": %d, \"ms\": %lf",
                    &e.t.split, &e.t.real_inv, &e.t.cols_lsu, &e.t.tc, &e.t.cols_c, &e.t.passes, &e.t.no_plane,
                    &e.ms) == 8 ||
        std::sscanf(b + 1,
                    " : {\"split\": %d, \"real_inv\": %d, \"cols_lsu\": %d, \"tc\": %d, \"cols_c\": %d, "
                    "\"passes\": %d, \"ms\": %lf",
                    &e.t.split, &e.t.real_inv, &e.t.cols_lsu, &e.t.tc, &e.t.cols_c, &e.t.passes, &e.ms) == 7 ||
        std::sscanf(b + 1,
                    " : {\"split\": %d, \"real_inv\": %d, \"cols_lsu\": %d, \"tc\": %d, \"cols_c\": %d, \"ms\": %lf",
                    &e.t.split, &e.t.real_inv, &e.t.cols_lsu, &e.t.tc, &e.t.cols_c, &e.ms) == 6 ||
        std::sscanf(b + 1, " : {\"split\": %d, \"real_inv\": %d, \"ms\": %lf", &e.t.split, &e.t.real_inv, &e.ms) ==
            3)
      C.table[std::string(a + 1, b)] = e;
  }
  std::fclose(f);
}

void save_locked(const TuneCache& C) {
  if (C.path.empty()) return;
  const std::string tmp = C.path + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "w");
  if (!f) return;
  std::fprintf(f, "{\n");
  size_t i = 0;
  for (const auto& kv : C.table) {
    const Tuning& t = kv.second.t;
    std::fprintf(f,
                 "\"%s\": {\"split\": %d, \"real_inv\": %d, \"cols_lsu\": %d, \"tc\": %d, \"cols_c\": %d, "
                 "\"passes\": %d, \"no_plane\": %d, \"no_pipe\": %d, \"ms\": %.6f}%s\n",
                 kv.first.c_str(), t.split, t.real_inv, t.cols_lsu, t.tc, t.cols_c, t.passes, t.no_plane, t.no_pipe,
                 kv.second.ms,
                 ++i < C.table.size() ? "," : "");
  }
  std::fprintf(f, "}\n");
  std::fclose(f);
  std::rename(tmp.c_str(), C.path.c_str());
}

// what distinguishes two built variants: the kernels they launch and how
std::string signature(const Plan& P) {
  std::string s;
  char buf[160];
  for (const Op& op : P.ops) {
    snprintf(buf, sizeof buf, "%d:%p:%p:%p:%d:%d:%d:%lld;", op.type,
             op.type == OP_LINE ? (const void*)op.k.fn : nullptr, op.type == OP_LINE ? (const void*)op.k.tma : nullptr,
             op.type == OP_LINE ? (const void*)op.k.pipe : nullptr, op.k.logl, op.k.lines_per_cta, op.k.tc,
             op.type == OP_LINE ? op.p.nlines : op.rp.nlines);
    s += buf;
  }
  return s;
}

// median time of one launch of P on zeroed buffers; <0 on failure
double time_plan(Plan& P, float* src, float* dst, size_t src_half, size_t dst_half, cudaStream_t st) {
  const bool inter = P.format == afft_interleaved;
  const bool cin = P.kind == K_C || P.kind == K_CI || P.kind == K_RI;    // complex input arrays
  const bool cout = P.kind == K_C || P.kind == K_CI || P.kind == K_R;    // complex output arrays
  float* si = (cin && !inter) ? src + src_half : nullptr;
  float* di = (cout && !inter) ? dst + dst_half : nullptr;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return -1;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return -1;
  }
  std::vector<float> ms;
  bool ok = true;
  for (int i = 0; i < 7 && ok; i++) {
    cudaEventRecord(e0, st);
    if (P.launch(src, si, dst, di, st)) ok = false;
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) ok = false;
    float t = 0;
    if (ok && i >= 2 && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess) ms.push_back(t);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!ok || ms.empty()) {
    cudaGetLastError();
    return -1;
  }
  std::sort(ms.begin(), ms.end());
  return ms[ms.size() / 2];
}

// Tune one shape; fills `out` and, if report is non-null, a JSON summary.
int tune_shape(int kind, int ndim, const long long* dims, long long batch, int format, Entry* out,
               std::string* report) {
  in_tuning = true;
  struct Reset {
    ~Reset() { in_tuning = false; }
  } reset;
  std::vector<std::pair<Tuning, std::unique_ptr<Plan>>> cands;
  std::vector<std::string> sigs;
  static const int widths[] = {0, 8, 16, 32};
  // two or three passes for long 1D axes, only where a dimension has one
  long long maxdim = 1;
  for (int i = 0; i < ndim; i++) maxdim = std::max(maxdim, dims[i]);
  static const int pass_forms[] = {0, 2, 3};
  const int npass = maxdim >= (1LL << 20) ? 3 : 1;
  // plane-fused or per-axis last two axes, only for N-D shapes
  // (innermost, so that the plain form's per-axis plan is recorded as
  // no_plane = 1 before the tensor-core form, which has no plane pass,
  // builds the same launches)
  const int nplane = ndim >= 2 ? 3 : 1;
  for (int pf = 0; pf < npass; pf++)
  for (int split = 0; split < 2; split++)
    for (int real_inv = 0; real_inv < 2; real_inv++)
      for (int lsu = 0; lsu < 2; lsu++)
        for (int tc = 0; tc < 2; tc++)
          for (int w : widths)
          for (int np = 0; np < nplane; np++)
          for (int npipe = 0; npipe < 2; npipe++) {
            Tuning t;
            t.split = split;
            t.real_inv = real_inv;
            t.cols_lsu = lsu;
            t.tc = tc;
            t.cols_c = w;
            t.passes = pass_forms[pf];
            t.no_plane = np;
            t.no_pipe = npipe;
            auto P = build_plan(kind, ndim, dims, batch, format, false, 0, &t);
            if (!P) {
              clear_error();
              continue;
            }
            // variants that build the same launches are one candidate (the
            // first, i.e. the most default, represents them)
            std::string sg = signature(*P);
            if (std::find(sigs.begin(), sigs.end(), sg) != sigs.end()) continue;
            sigs.push_back(sg);
            cands.emplace_back(t, std::move(P));
          }
  if (cands.empty()) {
    set_error(AFFT_GB300_EINVAL, "no plan for this shape");
    return AFFT_GB300_EINVAL;
  }
  std::vector<double> times(cands.size(), -1);
  if (cands.size() > 1) {
    const Plan& P0 = *cands[0].second;
    const size_t in_n = (size_t)P0.in_elems * (size_t)batch, out_n = (size_t)P0.out_elems * (size_t)batch;
    float *src = nullptr, *dst = nullptr;
    cudaStream_t st = nullptr;
    if (cudaMalloc(&src, 2 * in_n * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&dst, 2 * out_n * sizeof(float)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      if (src) cudaFree(src);
      if (dst) cudaFree(dst);
      set_error(AFFT_GB300_ENOMEM, "autotuner buffers");
      return AFFT_GB300_ENOMEM;
    }
    cudaMemsetAsync(src, 0, 2 * in_n * sizeof(float), st);
    cudaMemsetAsync(dst, 0, 2 * out_n * sizeof(float), st);
    for (size_t i = 0; i < cands.size(); i++) times[i] = time_plan(*cands[i].second, src, dst, in_n, out_n, st);
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    cudaFree(src);
    cudaFree(dst);
  }
  size_t best = 0;
  for (size_t i = 1; i < cands.size(); i++)
    if (times[i] >= 0 && (times[best] < 0 || times[i] < times[best])) best = i;
  out->t = cands[best].first;
  out->ms = times[best];
  if (report) {
    char buf[256];
    *report = "{\"key\":\"" + key_of(kind, ndim, dims, batch, format) + "\",\"candidates\":[";
    for (size_t i = 0; i < cands.size(); i++) {
      const Tuning& t = cands[i].first;
      snprintf(buf, sizeof buf,
               "%s{\"split\":%d,\"real_inv\":%d,\"cols_lsu\":%d,\"tc\":%d,\"cols_c\":%d,\"passes\":%d,"
               "\"no_plane\":%d,\"no_pipe\":%d,\"launches\":%zu,\"ms\":%.6f}",
               i ? "," : "", t.split, t.real_inv, t.cols_lsu, t.tc, t.cols_c, t.passes, t.no_plane, t.no_pipe,
               cands[i].second->ops.size(), times[i]);
      *report += buf;
    }
    const Tuning& t = out->t;
    snprintf(buf, sizeof buf,
             "],\"chosen\":{\"split\":%d,\"real_inv\":%d,\"cols_lsu\":%d,\"tc\":%d,\"cols_c\":%d,\"passes\":%d,"
             "\"no_plane\":%d,\"no_pipe\":%d,\"ms\":%.6f}}",
             t.split, t.real_inv, t.cols_lsu, t.tc, t.cols_c, t.passes, t.no_plane, t.no_pipe, out->ms);
    *report += buf;
  }
  return 0;
}

}  // namespace

Tuning tuned_choice(int kind, int ndim, const long long* dims, long long batch, int format) {
  if (in_tuning) return Tuning();
  auto& C = cache();
  std::lock_guard<std::mutex> g(C.mu);
  load_locked(C);
  const std::string key = key_of(kind, ndim, dims, batch, format);
  auto it = C.table.find(key);
  if (it != C.table.end()) return it->second.t;
  const char* a = std::getenv("AFFT_GB300_AUTOTUNE");
  if (a && a[0] == '1') {
    Entry e;
    if (tune_shape(kind, ndim, dims, batch, format, &e, nullptr) == 0) {
      C.table[key] = e;
      save_locked(C);
      return e.t;
    }
    clear_error();
  }
  return Tuning();
}

Tuning tuned_for_queue(int kind, int ndim, const long long* dims) {
  auto& C = cache();
  std::lock_guard<std::mutex> g(C.mu);
  load_locked(C);
  const std::string key = key_of(kind, ndim, dims, 0, afft_split);
  auto it = C.table.find(key);
  if (it != C.table.end()) return it->second.t;
  long long n = 1;
  for (int i = 0; i < ndim; i++) n *= dims[i];
  const long long batch = std::max(1LL, (1LL << 24) / n);
  Entry e;
  if (tune_shape(kind, ndim, dims, batch, afft_split, &e, nullptr) != 0) {
    clear_error();
    return Tuning();
  }
  C.table[key] = e;
  save_locked(C);
  return e.t;
}

}  // namespace agb

using namespace agb;

extern "C" {

int afft_gb300_tune(int kind, size_t ndim, const size_t* dim, size_t batch, int format, char* report,
                    size_t report_len) {
  clear_error();
  int nd = 0;
  long long dims[64];
  if (kind < 0 || kind > 3 || batch == 0 || (format != afft_split && format != afft_interleaved) ||
      validate_shape((int)ndim, dim, &nd, dims)) {
    set_error(AFFT_GB300_EINVAL, "bad shape for the autotuner");
    return AFFT_GB300_EINVAL;
  }
  auto& C = cache();
  std::lock_guard<std::mutex> g(C.mu);
  load_locked(C);
  Entry e;
  std::string rep;
  int rc = tune_shape(kind, nd, dims, (long long)batch, format, &e, &rep);
  if (rc) return rc;
  C.table[key_of(kind, nd, dims, (long long)batch, format)] = e;
  save_locked(C);
  if (report && report_len) {
    std::strncpy(report, rep.c_str(), report_len - 1);
    report[report_len - 1] = 0;
  }
  return 0;
}

int afft_gb300_tuned(int kind, size_t ndim, const size_t* dim, size_t batch, int format, int* split, int* real_inv) {
  clear_error();
  int nd = 0;
  long long dims[64];
  if (validate_shape((int)ndim, dim, &nd, dims)) {
    set_error(AFFT_GB300_EINVAL, "bad shape");
    return -1;
  }
  auto& C = cache();
  std::lock_guard<std::mutex> g(C.mu);
  load_locked(C);
  auto it = C.table.find(key_of(kind, nd, dims, (long long)batch, format));
  if (it == C.table.end()) return 0;
  if (split) *split = it->second.t.split;
  if (real_inv) *real_inv = it->second.t.real_inv;
  return 1;
}

}  // extern "C"
