// Multi-transform queue (afft_gb300_queue_*): many transforms of mixed sizes
// and kinds in one unit of work.
//
// At creation every transform's plan (one per distinct kind and shape) is
// resolved against the transform's own pointers into concrete launch
// segments: pass i of a transform becomes a segment of "level" i.  Segments
// are grouped by (level, kernel shape) into device-side descriptor tables;
// each group is ONE launch (line_fft_grouped or elementwise_grouped) of one
// CTA per virtual CTA, which finds its segment in a per-virtual-CTA map.
// The first run builds a CUDA graph with one kernel node per group, which
// depends on exactly the groups that ran the previous pass of its own
// transforms (the transforms are independent of each other), so a pass of
// one transform starts as soon as its own previous pass has finished; later
// runs replay the graph.
//
// Scratch for transforms whose plans need it (four-step passes, real
// inverse of N-D arrays) comes from one queue-owned arena, a disjoint region
// per transform.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <tuple>
#include <vector>

#include "../../include/afft_gb300.h"
#include "plan.h"

namespace agb {

struct Group {
  int level = 0;
  int id = 0;              // index at creation (before the groups are sorted)
  std::vector<int> trans;  // transforms with an op in this group
  std::vector<int> preds;  // groups this one waits for (sorted indices)
  bool line = true;
  LineKernel k{};
  bool pipe = false;     // the persistent pipelined kernel (grid at most pipe_ctas per SM)
  std::vector<Segment> segs;
  std::vector<EwSegment> esegs;
  long long total = 0;   // virtual CTAs / blocks
  void* d_tab = nullptr;
  int* d_map = nullptr;  // segment of each virtual CTA / block
  int grid = 0, threads = 0;
  size_t smem = 0;
};

struct QueueImpl {
  int form = 0;
  bool tuned = false;   // plans take the autotuner's per-shape queue choices
  std::vector<afft_gb300_desc> descs;
  std::map<std::vector<long long>, std::shared_ptr<Plan>> plans;
  std::vector<Group> groups;
  float* arena = nullptr;
  std::vector<TmaTile> tma_host;   // tensor maps of the TMA-fed segments
  TmaTile* d_tma = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t stream = nullptr;
  int device = 0;
  ~QueueImpl() {
    if (exec) cudaGraphExecDestroy(exec);
    for (auto& g : groups) {
      if (g.d_tab) cudaFree(g.d_tab);
      if (g.d_map) cudaFree(g.d_map);
    }
    if (arena) cudaFree(arena);
    if (d_tma) cudaFree(d_tma);
    if (stream) cudaStreamDestroy(stream);
  }
};

static LineIO bind_io(const IOSpec& s, float* const* base) {
  LineIO o;
  o.re = base[s.re.buf] ? base[s.re.buf] + s.re.off : nullptr;
  o.im = base[s.im.buf] ? base[s.im.buf] + s.im.off : nullptr;
  o.es = s.es;
  o.lo = s.lo;
  o.hi = s.hi;
  o.qshift = s.qshift;
  o.qmask = s.qmask;
  return o;
}

static LineParams bind_line_params(const Op& op, float* const* base) {
  LineParams p = op.p;
  p.in = bind_io(op.in, base);
  p.out = bind_io(op.out, base);
  return p;
}

static int build_queue(QueueImpl& Q) {
  // plans and scratch layout
  std::vector<std::shared_ptr<Plan>> plan_of;
  std::vector<long long> scr_off;
  long long arena_floats = 0;
  int dev = 0, sm_count = 0;   // SMs of the device: the pipelined groups' grid bound (0: none of those)
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    sm_count = 0;
  }
  for (const auto& d : Q.descs) {
    int nd;
    long long dims[64];
    if (d.kind < 0 || d.kind > 3 || d.ndim < 1 || d.ndim > 3 || validate_shape(d.ndim, d.dim, &nd, dims)) {
      set_error(AFFT_GB300_EINVAL, "bad descriptor (kind, ndim 1..3, power-of-two dims)");
      return AFFT_GB300_EINVAL;
    }
    // split data: src_im for complex input (c, ci, ri), dst_im for complex
    // output (c, ci, r); a missing array is reported, never launched on
    const bool cin = d.kind != K_R, cout = d.kind != K_RI;
    if (!d.src_re || !d.dst_re || (cin && !d.src_im) || (cout && !d.dst_im)) {
      set_error(AFFT_GB300_EINVAL, "bad descriptor: a data pointer the transform reads or writes is NULL");
      return AFFT_GB300_EINVAL;
    }
    std::vector<long long> key{d.kind};
    key.insert(key.end(), dims, dims + nd);
    auto it = Q.plans.find(key);
    if (it == Q.plans.end()) {
      // the tuned choice (for queues created with it), else what a plan of
      // this shape gets
      Tuning tq = Q.tuned ? tuned_for_queue(d.kind, nd, dims)
                          : (Q.form == 0 ? tuned_choice(d.kind, nd, dims, 1, 0) : Tuning{});
      if (tq.no_plane == 0) tq.no_plane = 2;   // one grouped launch gathers the planes of every transform
      auto P = build_plan(d.kind, nd, dims, 1, 0, false, Q.form, &tq);
      if (!P) return AFFT_GB300_EINVAL;
      it = Q.plans.emplace(key, std::shared_ptr<Plan>(P.release())).first;
    }
    plan_of.push_back(it->second);
    scr_off.push_back(arena_floats);
    arena_floats += (it->second->scratch_elems + 63) / 64 * 64;
  }
  if (arena_floats && cudaMalloc(&Q.arena, (size_t)arena_floats * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    set_error(AFFT_GB300_ENOMEM, "queue scratch allocation failed");
    return AFFT_GB300_ENOMEM;
  }
  // segments, grouped by (level, kernel); tgroup[j][i] = group of op i of transform j
  std::map<std::pair<int, const void*>, size_t> gidx;
  std::vector<std::vector<int>> tgroup(Q.descs.size());
  for (size_t j = 0; j < Q.descs.size(); j++) {
    const auto& d = Q.descs[j];
    float* base[B_NBUF] = {(float*)d.src_re, (float*)d.src_im, d.dst_re, d.dst_im,
                           Q.arena ? Q.arena + scr_off[j] : nullptr};
    const Plan& P = *plan_of[j];
    for (size_t i = 0; i < P.ops.size(); i++) {
      const Op& op = P.ops[i];
      if (!op_tables_ok(op)) {
        set_error(AFFT_GB300_ECUDA, "plan is missing a twiddle table");
        return AFFT_GB300_ECUDA;
      }
      // a TMA-capable pass whose tensor maps encode for this transform's
      // arrays goes to the TMA form of the grouped kernel
      // (the pipelined 2048-point passes: their persistent queue form)
      TmaTile tm;
      const bool tma = op.type == OP_LINE && op.k.grouped_tma && tma_tile(bind_line_params(op, base), op.k, &tm);
      // (2048-point passes only: the 1024-point ones measured 0.7% slower on
      // the mixed queue than their one-tile grouped form, whose CTAs share
      // the SMs with the groups running beside them)
      const bool pipe = tma && op.k.grouped_pipe && sm_count > 0 && op.k.logl == 11;
      const void* kid = op.type != OP_LINE ? (const void*)&elementwise_grouped
                        : pipe            ? (const void*)op.k.grouped_pipe
                        : tma             ? (const void*)op.k.grouped_tma
                                          : (const void*)op.k.grouped;
      auto key = std::make_pair((int)i, kid);
      auto it = gidx.find(key);
      if (it == gidx.end()) {
        Group g;
        g.level = (int)i;
        g.id = (int)Q.groups.size();
        g.line = op.type == OP_LINE;
        g.k = op.k;
        if (tma) g.k.grouped = pipe ? op.k.grouped_pipe : op.k.grouped_tma;
        g.pipe = pipe;
        it = gidx.emplace(key, Q.groups.size()).first;
        Q.groups.push_back(g);
      }
      Group& g = Q.groups[it->second];
      g.trans.push_back((int)j);
      tgroup[j].push_back((int)it->second);
      if (op.type == OP_LINE) {
        Segment s;
        s.p = op.p;
        s.p.in = bind_io(op.in, base);
        s.p.out = bind_io(op.out, base);
        s.cta0 = op.grid;  // for now the segment's CTA count
        // the tensor maps of a TMA-fed segment (the pointers are fixed now);
        // s.tma holds 1 + the map's index until the map array exists
        s.tma = nullptr;
        if (tma) {
          Q.tma_host.push_back(tm);
          s.tma = reinterpret_cast<const TmaTile*>((uintptr_t)Q.tma_host.size());
        }
        g.segs.push_back(s);
      } else {
        EwSegment s{};
        s.type = op.type == OP_REAL ? EW_REAL : (op.type == OP_COPY ? EW_COPY : EW_REAL1);
        s.rp = op.rp;
        s.cp = op.cp;
        if (op.type == OP_COPY) {
          s.cp.in = bind_io(op.in, base);
          s.cp.out = bind_io(op.out, base);
        } else {
          s.rp.in = bind_io(op.in, base);
          s.rp.out = bind_io(op.out, base);
        }
        s.blk0 = op.grid;
        g.esegs.push_back(s);
      }
    }
  }
  if (!Q.tma_host.empty() &&
      (cudaMalloc(&Q.d_tma, Q.tma_host.size() * sizeof(TmaTile)) != cudaSuccess ||
       cudaMemcpy(Q.d_tma, Q.tma_host.data(), Q.tma_host.size() * sizeof(TmaTile), cudaMemcpyHostToDevice) !=
           cudaSuccess)) {
    cudaGetLastError();
    set_error(AFFT_GB300_ENOMEM, "queue tensor-map upload failed");
    return AFFT_GB300_ENOMEM;
  }
  for (auto& g : Q.groups)
    for (auto& s : g.segs)
      if (s.tma) s.tma = Q.d_tma + ((uintptr_t)s.tma - 1);
  // largest segments first, prefix sums, device tables, launch shapes
  for (auto& g : Q.groups) {
    void* host = nullptr;
    size_t bytes = 0;
    if (g.line) {
      std::stable_sort(g.segs.begin(), g.segs.end(),
                       [](const Segment& a, const Segment& b) { return a.cta0 > b.cta0; });
      long long acc = 0;
      for (auto& s : g.segs) {
        long long n = s.cta0;
        s.cta0 = acc;
        acc += n;
      }
      g.total = acc;
      host = g.segs.data();
      bytes = g.segs.size() * sizeof(Segment);
      g.threads = g.k.threads;
      g.smem = g.pipe ? g.k.pipe_smem : g.k.smem;
      if (g.smem > 48 * 1024 &&
          cudaFuncSetAttribute((const void*)g.k.grouped, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)g.smem) != cudaSuccess) {
        cudaGetLastError();
        set_error(AFFT_GB300_ECUDA, "kernel shared memory configuration failed");
        return AFFT_GB300_ECUDA;
      }
      g.grid = (int)(g.pipe ? std::min<long long>(g.total, (long long)sm_count * g.k.pipe_ctas) : g.total);
    } else {
      std::stable_sort(g.esegs.begin(), g.esegs.end(),
                       [](const EwSegment& a, const EwSegment& b) { return a.blk0 > b.blk0; });
      long long acc = 0;
      for (auto& s : g.esegs) {
        long long n = s.blk0;
        s.blk0 = acc;
        acc += n;
      }
      g.total = acc;
      host = g.esegs.data();
      bytes = g.esegs.size() * sizeof(EwSegment);
      g.threads = 256;
      g.grid = (int)g.total;
    }
    if (g.total > 0x7fffffffLL) {
      set_error(AFFT_GB300_EINVAL, "queue group too large for one launch");
      return AFFT_GB300_EINVAL;
    }
    // the segment of every virtual CTA / block (segments are in cta0 order)
    std::vector<int> map((size_t)g.total);
    const size_t nseg = g.line ? g.segs.size() : g.esegs.size();
    for (size_t i = 0; i < nseg; i++) {
      const long long b0 = g.line ? g.segs[i].cta0 : g.esegs[i].blk0;
      const long long b1 = i + 1 < nseg ? (g.line ? g.segs[i + 1].cta0 : g.esegs[i + 1].blk0) : g.total;
      std::fill(map.begin() + b0, map.begin() + b1, (int)i);
    }
    if (cudaMalloc(&g.d_tab, bytes) != cudaSuccess ||
        cudaMemcpy(g.d_tab, host, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        (g.total && (cudaMalloc(&g.d_map, map.size() * sizeof(int)) != cudaSuccess ||
                     cudaMemcpy(g.d_map, map.data(), map.size() * sizeof(int), cudaMemcpyHostToDevice) !=
                         cudaSuccess))) {
      cudaGetLastError();
      set_error(AFFT_GB300_ENOMEM, "queue descriptor upload failed");
      return AFFT_GB300_ENOMEM;
    }
  }
  // the uploads above come from pageable memory and may return before their
  // DMA lands; the queue runs on the caller's stream, so wait once here
  if (cudaStreamSynchronize(0) != cudaSuccess) {
    cudaGetLastError();
    set_error(AFFT_GB300_ECUDA, "queue descriptor upload failed");
    return AFFT_GB300_ECUDA;
  }
  std::stable_sort(Q.groups.begin(), Q.groups.end(), [](const Group& a, const Group& b) {
    return a.level != b.level ? a.level < b.level : a.total > b.total;
  });
  // each group waits for the groups holding the previous pass of its transforms
  std::vector<int> pos(Q.groups.size());
  for (size_t n = 0; n < Q.groups.size(); n++) pos[Q.groups[n].id] = (int)n;
  for (auto& g : Q.groups) {
    if (g.level > 0)
      for (int j : g.trans) g.preds.push_back(pos[tgroup[j][g.level - 1]]);
    std::sort(g.preds.begin(), g.preds.end());
    g.preds.erase(std::unique(g.preds.begin(), g.preds.end()), g.preds.end());
  }
  return 0;
}

static int capture(QueueImpl& Q) {
  // one node per group (an empty node for a group without work, so the
  // dependency chain stays whole), with edges from its predecessor groups
  cudaGraph_t graph = nullptr;
  if (cudaGraphCreate(&graph, 0) != cudaSuccess) return AFFT_GB300_ECUDA;
  std::vector<cudaGraphNode_t> node(Q.groups.size());
  bool ok = true;
  for (size_t n = 0; n < Q.groups.size() && ok; n++) {
    Group& g = Q.groups[n];
    std::vector<cudaGraphNode_t> deps;
    for (int p : g.preds) deps.push_back(node[p]);
    if (g.total == 0) {
      ok = cudaGraphAddEmptyNode(&node[n], graph, deps.data(), deps.size()) == cudaSuccess;
      continue;
    }
    cudaKernelNodeParams kp{};
    void* args[3] = {&g.d_tab, &g.d_map, &g.total};
    kp.func = g.line ? (void*)g.k.grouped : (void*)&elementwise_grouped;
    kp.gridDim = dim3((unsigned)g.grid);
    kp.blockDim = dim3((unsigned)g.threads);
    kp.sharedMemBytes = (unsigned)g.smem;
    kp.kernelParams = args;
    ok = cudaGraphAddKernelNode(&node[n], graph, deps.data(), deps.size(), &kp) == cudaSuccess;
  }
  cudaError_t e = ok ? cudaGraphInstantiate(&Q.exec, graph, 0) : cudaErrorUnknown;
  cudaGraphDestroy(graph);
  if (!ok) cudaGetLastError();
  return e == cudaSuccess ? 0 : AFFT_GB300_ECUDA;
}

}  // namespace agb

using namespace agb;

struct afft_gb300_queue {
  QueueImpl impl;
};

extern "C" {

afft_gb300_queue* afft_gb300_queue_create(const afft_gb300_desc* descs, size_t count) {
  return afft_gb300_queue_create_ex(descs, count, 0);
}

afft_gb300_queue* afft_gb300_queue_create_ex(const afft_gb300_desc* descs, size_t count, int flags) {
  clear_error();
  if (!descs && count) {
    set_error(AFFT_GB300_EINVAL, "null descriptor array");
    return nullptr;
  }
  if (flags & ~(FORM_TC | AFFT_GB300_QUEUE_TUNED)) {   // FP32 data only (FP64 transforms have no grouped kernels)
    set_error(AFFT_GB300_EINVAL, "queue flags: AFFT_GB300_FORM_TC and/or AFFT_GB300_QUEUE_TUNED");
    return nullptr;
  }
  auto* q = new afft_gb300_queue();
  QueueImpl& Q = q->impl;
  Q.form = flags & FORM_TC;
  Q.tuned = (flags & AFFT_GB300_QUEUE_TUNED) != 0;
  cudaGetDevice(&Q.device);
  Q.descs.assign(descs, descs + count);
  if (cudaStreamCreateWithFlags(&Q.stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    set_error(AFFT_GB300_ECUDA, "stream creation failed");
    delete q;
    return nullptr;
  }
  if (build_queue(Q)) {
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
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != Q.device) cudaSetDevice(Q.device);
  struct Restore {
    int d, p;
    ~Restore() {
      if (p >= 0 && p != d) cudaSetDevice(p);
    }
  } restore{Q.device, prev};
  if (Q.groups.empty()) return 0;   // nothing queued: no graph, no launch
  if (!Q.exec && capture(Q)) {
    cudaGetLastError();
    set_error(AFFT_GB300_ECUDA, "graph capture failed");
    return AFFT_GB300_ECUDA;
  }
  cudaError_t e = cudaGraphLaunch(Q.exec, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    set_error(AFFT_GB300_ECUDA, cudaGetErrorString(e));
    return AFFT_GB300_ECUDA;
  }
  return 0;
}

int afft_gb300_queue_launches(const afft_gb300_queue* q) {
  if (!q) return -1;
  int n = 0;
  for (const auto& g : q->impl.groups) n += g.total > 0;
  return n;
}

void afft_gb300_queue_destroy(afft_gb300_queue* q) { delete q; }

}  // extern "C"
