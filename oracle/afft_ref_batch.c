/* TEST INFRASTRUCTURE ONLY: a batch driver over the reference afft library's
 * own C API (fft.h:22-50).  It is compiled into the reference library that
 * oracle/Makefile builds from the reference's sources (targets `ref` and
 * `ref_scalar`), and serves bench.py's CPU legs: afft itself timed on the
 * host cores over the same streamed arrays the GPU transforms.  Nothing in
 * the product package loads it.
 *
 * afft plans are not reentrant (their working buffers live in the plan,
 * fft_internal.hpp:18-19), so every thread builds and keeps its own plans,
 * as the reference's own multi-threaded harness does (run_all.cpp:138-146).
 * Plans are cached per thread slot in a context, so repeated timed calls do
 * not re-plan.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fft.h"

#define RB_MAX_DIMS 8
#define RB_MAX_PLANS 1024

enum { RB_C = 0, RB_CI = 1, RB_R = 2, RB_RI = 3 };

typedef struct {
  int kind, impl;
  size_t ndim, dims[RB_MAX_DIMS];
  void* mem;
  void* plan;
} rb_plan;

typedef struct {
  int nplans;
  rb_plan plans[RB_MAX_PLANS];
} rb_slot;

typedef struct {
  int threads;
  rb_slot* slots;
} refbatch_ctx;

static size_t rb_memsize(int kind, size_t ndim, const size_t* dims, int impl) {
  switch (kind) {
    case RB_C: return afft_32_c_memsize(ndim, dims, afft_split, impl);
    case RB_CI: return afft_32_ci_memsize(ndim, dims, afft_split, impl);
    case RB_R: return afft_32_r_memsize(ndim, dims, afft_split, impl);
    case RB_RI: return afft_32_ri_memsize(ndim, dims, afft_split, impl);
  }
  return 0;
}

static void* rb_create(int kind, size_t ndim, const size_t* dims, void* mem, int impl) {
  switch (kind) {
    case RB_C: return afft_32_c_create(ndim, dims, afft_split, mem, impl);
    case RB_CI: return afft_32_ci_create(ndim, dims, afft_split, mem, impl);
    case RB_R: return afft_32_r_create(ndim, dims, afft_split, mem, impl);
    case RB_RI: return afft_32_ri_create(ndim, dims, afft_split, mem, impl);
  }
  return NULL;
}

/* the plan of (kind, dims, impl) in one thread's slot, built on first use */
static rb_plan* rb_get(rb_slot* s, int kind, size_t ndim, const size_t* dims, int impl) {
  if (ndim < 1 || ndim > RB_MAX_DIMS) return NULL;
  for (int i = 0; i < s->nplans; i++) {
    rb_plan* p = &s->plans[i];
    if (p->kind == kind && p->impl == impl && p->ndim == ndim && !memcmp(p->dims, dims, ndim * sizeof(size_t)))
      return p;
  }
  if (s->nplans >= RB_MAX_PLANS) return NULL;
  size_t ms = rb_memsize(kind, ndim, dims, impl);
  if (ms == 0 || ms == (size_t)-1) return NULL;
  void* mem = aligned_alloc(64, (ms + 63) / 64 * 64);
  if (!mem) return NULL;
  void* plan = rb_create(kind, ndim, dims, mem, impl);
  if (!plan) {
    free(mem);
    return NULL;
  }
  rb_plan* p = &s->plans[s->nplans++];
  p->kind = kind;
  p->impl = impl;
  p->ndim = ndim;
  memset(p->dims, 0, sizeof(p->dims));
  memcpy(p->dims, dims, ndim * sizeof(size_t));
  p->mem = mem;
  p->plan = plan;
  return p;
}

static void rb_run(const rb_plan* p, const float* in_re, const float* in_im, float* out_re, float* out_im) {
  switch (p->kind) {
    case RB_C: afft_32_c_transform((afft_32_c_type*)p->plan, in_re, in_im, out_re, out_im); break;
    case RB_CI: afft_32_ci_transform((afft_32_ci_type*)p->plan, in_re, in_im, out_re, out_im); break;
    case RB_R: afft_32_r_transform((afft_32_r_type*)p->plan, in_re, out_re, out_im); break;
    case RB_RI: afft_32_ri_transform((afft_32_ri_type*)p->plan, in_re, in_im, out_re); break;
  }
}

/* elements per array on the input and output side of one transform */
static void rb_elems(int kind, size_t ndim, const size_t* dims, int64_t* in_n, int64_t* out_n) {
  int64_t n = 1;
  for (size_t i = 0; i < ndim; i++) n *= (int64_t)dims[i];
  /* real transforms halve the first dimension that is not 1 */
  size_t d0 = 1;
  for (size_t i = 0; i < ndim; i++)
    if (dims[i] != 1) {
      d0 = dims[i];
      break;
    }
  int64_t h = (int64_t)(d0 / 2 + 1) * (n / (int64_t)d0);
  *in_n = kind == RB_RI ? h : n;
  *out_n = kind == RB_R ? h : n;
}

refbatch_ctx* refbatch_ctx_create(int threads) {
  if (threads < 1) threads = 1;
  refbatch_ctx* c = (refbatch_ctx*)calloc(1, sizeof(refbatch_ctx));
  if (!c) return NULL;
  c->threads = threads;
  c->slots = (rb_slot*)calloc((size_t)threads, sizeof(rb_slot));
  if (!c->slots) {
    free(c);
    return NULL;
  }
  return c;
}

void refbatch_ctx_destroy(refbatch_ctx* c) {
  if (!c) return;
  for (int t = 0; t < c->threads; t++)
    for (int i = 0; i < c->slots[t].nplans; i++) free(c->slots[t].plans[i].mem);
  free(c->slots);
  free(c);
}

typedef struct {
  rb_slot* slot;
  int kind, impl;
  size_t ndim;
  const size_t* dims;
  int64_t b0, b1;
  const float *in_re, *in_im;
  float *out_re, *out_im;
  /* mixed batches */
  int64_t count;
  int64_t* next;
  const int* kinds;
  const int* ndims;
  const size_t* mdims;
  const float* const* min_re;
  const float* const* min_im;
  float* const* mout_re;
  float* const* mout_im;
  int rc;
} rb_job;

static void* rb_uniform_worker(void* arg) {
  rb_job* j = (rb_job*)arg;
  rb_plan* p = rb_get(j->slot, j->kind, j->ndim, j->dims, j->impl);
  if (!p) {
    j->rc = -1;
    return NULL;
  }
  int64_t in_n, out_n;
  rb_elems(j->kind, j->ndim, j->dims, &in_n, &out_n);
  for (int64_t b = j->b0; b < j->b1; b++)
    rb_run(p, j->in_re + b * in_n, j->in_im ? j->in_im + b * in_n : NULL, j->out_re + b * out_n,
           j->out_im ? j->out_im + b * out_n : NULL);
  j->rc = 0;
  return NULL;
}

static void* rb_mixed_worker(void* arg) {
  rb_job* j = (rb_job*)arg;
  j->rc = 0;
  for (;;) {
    int64_t i = __atomic_fetch_add(j->next, 1, __ATOMIC_RELAXED);
    if (i >= j->count) break;
    rb_plan* p = rb_get(j->slot, j->kinds[i], (size_t)j->ndims[i], j->mdims + 3 * i, j->impl);
    if (!p) {
      j->rc = -1;
      continue;
    }
    rb_run(p, j->min_re[i], j->min_im[i], j->mout_re[i], j->mout_im[i]);
  }
  return NULL;
}

static int rb_launch(refbatch_ctx* c, int threads, rb_job* proto, void* (*fn)(void*), int split) {
  if (threads > c->threads) threads = c->threads;
  if (threads < 1) threads = 1;
  pthread_t tid[256];
  rb_job jobs[256];
  if (threads > 256) threads = 256;
  for (int t = 0; t < threads; t++) {
    jobs[t] = *proto;
    jobs[t].slot = &c->slots[t];
    if (split) {
      int64_t nb = proto->b1 - proto->b0;
      jobs[t].b0 = proto->b0 + nb * t / threads;
      jobs[t].b1 = proto->b0 + nb * (t + 1) / threads;
    }
    jobs[t].rc = -1;
  }
  int started = 0;
  for (int t = 1; t < threads; t++) {
    if (pthread_create(&tid[t], NULL, fn, &jobs[t])) break;
    started = t;
  }
  fn(&jobs[0]);
  int rc = jobs[0].rc;
  for (int t = 1; t <= started; t++) {
    pthread_join(tid[t], NULL);
    if (jobs[t].rc) rc = -1;
  }
  /* threads that could not start leave their share undone */
  if (started + 1 < threads) rc = -1;
  return rc;
}

/* `batch` contiguous transforms of one shape, split into `threads`
 * contiguous ranges.  Arrays are split re/im; in_im and out_im are NULL
 * where the kind has none (r input, ri output). */
int refbatch_uniform(refbatch_ctx* c, int kind, size_t ndim, const size_t* dims, int64_t batch, int threads,
                     int impl, const float* in_re, const float* in_im, float* out_re, float* out_im) {
  if (!c || batch < 0 || ndim < 1 || ndim > RB_MAX_DIMS) return -1;
  rb_job proto;
  memset(&proto, 0, sizeof(proto));
  proto.kind = kind;
  proto.impl = impl;
  proto.ndim = ndim;
  proto.dims = dims;
  proto.b0 = 0;
  proto.b1 = batch;
  proto.in_re = in_re;
  proto.in_im = in_im;
  proto.out_re = out_re;
  proto.out_im = out_im;
  if (threads > batch) threads = (int)(batch > 0 ? batch : 1);
  return rb_launch(c, threads, &proto, rb_uniform_worker, 1);
}

/* `count` transforms of mixed shapes (dims: 3 entries per transform, ndims
 * of them used), each with its own arrays, taken by `threads` threads from a
 * shared counter. */
int refbatch_mixed(refbatch_ctx* c, int64_t count, const int* kinds, const int* ndims, const size_t* dims,
                   const float* const* in_re, const float* const* in_im, float* const* out_re,
                   float* const* out_im, int threads, int impl) {
  if (!c || count < 0) return -1;
  int64_t next = 0;
  rb_job proto;
  memset(&proto, 0, sizeof(proto));
  proto.impl = impl;
  proto.count = count;
  proto.next = &next;
  proto.kinds = kinds;
  proto.ndims = ndims;
  proto.mdims = dims;
  proto.min_re = in_re;
  proto.min_im = in_im;
  proto.mout_re = out_re;
  proto.mout_im = out_im;
  return rb_launch(c, threads, &proto, rb_mixed_worker, 0);
}
