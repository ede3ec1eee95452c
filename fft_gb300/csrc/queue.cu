// Multi-transform queue (afft_gb300_queue_*): many transforms of mixed
// sizes and kinds run as one unit.  Plans are built once per distinct
// (kind, shape); the launches of every transform are recorded into one CUDA
// graph on the first run and replayed afterwards.
#include <cuda_runtime.h>

#include <map>
#include <tuple>
#include <vector>

#include "../../include/afft_gb300.h"
#include "plan.h"

namespace agb {

struct QueueImpl {
  std::vector<afft_gb300_desc> descs;
  std::vector<std::shared_ptr<Plan>> plan_of;   // per descriptor
  std::map<std::vector<long long>, std::shared_ptr<Plan>> plans;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t stream = nullptr;
  int launches = 0;
  int device = 0;
  ~QueueImpl() {
    if (exec) cudaGraphExecDestroy(exec);
    if (stream) cudaStreamDestroy(stream);
  }
};

}  // namespace agb

using namespace agb;

struct afft_gb300_queue {
  QueueImpl impl;
};

extern "C" {

afft_gb300_queue* afft_gb300_queue_create(const afft_gb300_desc* descs, size_t count) {
  clear_error();
  if (!descs && count) {
    set_error(AFFT_GB300_EINVAL, "null descriptor array");
    return nullptr;
  }
  auto* q = new afft_gb300_queue();
  QueueImpl& Q = q->impl;
  cudaGetDevice(&Q.device);
  Q.descs.assign(descs, descs + count);
  for (const auto& d : Q.descs) {
    if (d.kind < 0 || d.kind > 3 || d.ndim < 1 || d.ndim > 3) {
      set_error(AFFT_GB300_EINVAL, "bad descriptor");
      delete q;
      return nullptr;
    }
    int nd;
    long long dims[64];
    if (validate_shape(d.ndim, d.dim, &nd, dims)) {
      set_error(AFFT_GB300_EINVAL, "descriptor dimensions must be powers of two");
      delete q;
      return nullptr;
    }
    std::vector<long long> key{d.kind};
    key.insert(key.end(), dims, dims + nd);
    auto it = Q.plans.find(key);
    if (it == Q.plans.end()) {
      auto P = build_plan(d.kind, nd, dims, 1, 0);
      if (!P) {
        delete q;
        return nullptr;
      }
      it = Q.plans.emplace(key, std::shared_ptr<Plan>(P.release())).first;
    }
    Q.plan_of.push_back(it->second);
    Q.launches += (int)it->second->ops.size();
  }
  if (cudaStreamCreateWithFlags(&Q.stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    set_error(AFFT_GB300_ECUDA, "stream creation failed");
    delete q;
    return nullptr;
  }
  return q;
}

int afft_gb300_queue_run(afft_gb300_queue* q, void* stream) {
  clear_error();
  if (!q) {
    set_error(AFFT_GB300_EINVAL, "null queue");
    return AFFT_GB300_EINVAL;
  }
  QueueImpl& Q = q->impl;
  cudaSetDevice(Q.device);
  cudaStream_t st = (cudaStream_t)stream;
  if (!Q.exec) {
    // scratch must exist before capture
    for (auto& kv : Q.plans) {
      Plan& P = *kv.second;
      if (P.scratch_floats > 0 && !P.scratch &&
          cudaMalloc(&P.scratch, (size_t)P.scratch_floats * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        set_error(AFFT_GB300_ENOMEM, "scratch allocation failed");
        return AFFT_GB300_ENOMEM;
      }
    }
    cudaStream_t cap = Q.stream;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      set_error(AFFT_GB300_ECUDA, "graph capture failed");
      return AFFT_GB300_ECUDA;
    }
    int rc = 0;
    for (size_t i = 0; i < Q.descs.size() && !rc; i++) {
      const auto& d = Q.descs[i];
      rc = Q.plan_of[i]->launch(d.src_re, d.src_im, d.dst_re, d.dst_im, cap);
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    if (rc || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      set_error(AFFT_GB300_ECUDA, "graph capture failed");
      return AFFT_GB300_ECUDA;
    }
    e = cudaGraphInstantiate(&Q.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      set_error(AFFT_GB300_ECUDA, cudaGetErrorString(e));
      return AFFT_GB300_ECUDA;
    }
  }
  cudaError_t e = cudaGraphLaunch(Q.exec, st);
  if (e != cudaSuccess) {
    set_error(AFFT_GB300_ECUDA, cudaGetErrorString(e));
    return AFFT_GB300_ECUDA;
  }
  return 0;
}

int afft_gb300_queue_launches(const afft_gb300_queue* q) { return q ? q->impl.launches : -1; }

void afft_gb300_queue_destroy(afft_gb300_queue* q) { delete q; }

}  // extern "C"
