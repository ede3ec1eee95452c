/*
 * afft_gb300 -- GB300 (sm_103a) implementation of afft's power-of-two FFT
 * path behind afft's own C API.
 *
 * Part 1 re-declares afft's fft.h with the same names, types, arguments and
 * error behaviour, so an existing afft caller links against libafft_gb300.so
 * instead of libfft.a.  Part 2 adds extensions afft has no counterpart for:
 * batches, asynchronous launch on a caller stream, explicit release of the
 * device resources a plan holds, error reporting, and a multi-transform queue.
 *
 * Semantics shared with afft (fft.h:22-50, fft_internal.hpp, onedim.hpp):
 *  - split format: separate re and im arrays, row-major, dims of size 1 are
 *    dropped (common.hpp:68-84); interleaved format: re,im pairs in one array,
 *    the *_im arguments ignored;
 *  - forward = exp(-2 pi i jk/n); inverse transforms are unnormalised
 *    (inverse(forward(x)) = n x);
 *  - real forward keeps d0/2+1 planes of the FIRST dimension (dst_re and
 *    dst_im each hold (d0/2+1)*prod(dims[1:]) values); real inverse reads
 *    that layout, using only the real part of planes 0 and d0/2;
 *  - the caller owns `mem` (size from *_memsize) and every data array; a plan
 *    is placement-built into `mem`; transform calls are synchronous: they run
 *    after work already queued on the CUDA default stream (so device inputs
 *    produced there are complete) and dst is complete when the call returns.
 *
 * Where the data lives: transform accepts device pointers (cudaMalloc,
 * managed) and host pointers (pageable or pinned).  Host data is staged
 * through device buffers owned by the plan, copies included in the call.
 * Pinned host buffers that are mapped at the same address (cudaHostAlloc,
 * cudaHostRegister), and pageable buffers on devices that read pageable
 * memory through the host's page tables (Grace-based systems), are read and
 * written by the kernels directly, without staging, when the plan touches
 * each caller array once in wide segments (one-pass plans, long 1D complex
 * axes); other plans stage them.
 *
 * Device resources (twiddle tables, scratch, staging buffers, a stream) live
 * in a library-owned registry keyed by the plan; afft has no destroy call, so
 * they persist until afft_gb300_release(plan) or library unload.
 */
#ifndef AFFT_GB300_H
#define AFFT_GB300_H

#include <stddef.h>

/* Symbols of this header are exported from the shared library even when it
 * is compiled with hidden default visibility. */
#if defined(__GNUC__)
#define AFFT_GB300_API __attribute__((visibility("default")))
#else
#define AFFT_GB300_API
#endif

/* ------------------------------------------------------------------------ */
/* Part 1: afft's fft.h                                                     */
/* ------------------------------------------------------------------------ */

/* fft.h:5-13.  Any value other than afft_auto or afft_gb300 selects a CPU
 * backend this library does not have: memsize returns 0, create NULL. */
enum
{
  afft_auto = 0,
  afft_scalar = 1,
  afft_sse2 = 2,
  afft_avx2 = 3,
  afft_avx512f = 4,
  afft_neon = 5,
  afft_gb300 = 6
};

/* fft.h:15 */
enum { afft_split = 0, afft_interleaved = 1 };

#ifdef __cplusplus
extern "C"
{
#endif

/* Replaces fft.h:22-26 (afft_32_c_*, complex forward).  memsize returns 0
 * and create NULL for a bad impl, ndim == 0 or > 64, a dimension that is not
 * a power of two, or a total size above 2^31 elements; an unknown format
 * returns (size_t)-1 / NULL as fft.cpp does for a disabled format. */
typedef struct afft_32_c_struct afft_32_c_type;
AFFT_GB300_API size_t afft_32_c_memsize(size_t ndim, const size_t* dim, int format, int impl);
AFFT_GB300_API afft_32_c_type* afft_32_c_create(
  size_t ndim, const size_t* dim, int format, void* mem, int impl);
AFFT_GB300_API void afft_32_c_transform(afft_32_c_type* state,
  const float* src_re, const float* src_im, float* dst_re, float* dst_im);

/* Replaces fft.h:28-32 (complex inverse, unnormalised). */
typedef struct afft_32_ci_struct afft_32_ci_type;
AFFT_GB300_API size_t afft_32_ci_memsize(size_t ndim, const size_t* dim, int format, int impl);
AFFT_GB300_API afft_32_ci_type* afft_32_ci_create(
  size_t ndim, const size_t* dim, int format, void* mem, int impl);
AFFT_GB300_API void afft_32_ci_transform(afft_32_ci_type* state,
  const float* src_re, const float* src_im, float* dst_re, float* dst_im);

/* Replaces fft.h:34-38 (real forward, first dimension halved).  Real
 * transforms (forward and inverse) need src and dst not to overlap;
 * complex transforms may run in place (src == dst). */
typedef struct afft_32_r_struct afft_32_r_type;
AFFT_GB300_API size_t afft_32_r_memsize(size_t ndim, const size_t* dim, int format, int impl);
AFFT_GB300_API afft_32_r_type* afft_32_r_create(
  size_t ndim, const size_t* dim, int format, void* mem, int impl);
AFFT_GB300_API void afft_32_r_transform(afft_32_r_type* state,
  const float* src, float* dst_re, float* dst_im);

/* Replaces fft.h:40-44 (real inverse, unnormalised). */
typedef struct afft_32_ri_struct afft_32_ri_type;
AFFT_GB300_API size_t afft_32_ri_memsize(size_t ndim, const size_t* dim, int format, int impl);
AFFT_GB300_API afft_32_ri_type* afft_32_ri_create(
  size_t ndim, const size_t* dim, int format, void* mem, int impl);
AFFT_GB300_API void afft_32_ri_transform(afft_32_ri_type* state,
  const float* src_re, const float* src_im, float* dst);

/* Replaces fft.h:46 / fft.cpp:221: rounds up to a multiple of 64 bytes of
 * floats (afft_alignment / sizeof(float) = 16 elements). */
AFFT_GB300_API size_t afft_32_align_size(size_t sz);

/* Replaces fft.h:48-80 (FP64): the same transforms, layouts, errors and
 * pointer rules on double arrays, computed in FP64 by the library's FP64
 * kernels (twiddles computed in FP64, never rounded).  A plan made by an
 * afft_64_*_create (or a batched plan with AFFT_GB300_FORM_F64) runs only
 * through the afft_64_* transforms, an FP32 plan only through the afft_32_*
 * ones; a mismatch sets AFFT_GB300_EINVAL and launches nothing. */
typedef struct afft_64_c_struct afft_64_c_type;
AFFT_GB300_API size_t afft_64_c_memsize(size_t ndim, const size_t* dim, int format, int impl);
AFFT_GB300_API afft_64_c_type* afft_64_c_create(
  size_t ndim, const size_t* dim, int format, void* mem, int impl);
AFFT_GB300_API void afft_64_c_transform(afft_64_c_type* state,
  const double* src_re, const double* src_im, double* dst_re, double* dst_im);

typedef struct afft_64_ci_struct afft_64_ci_type;
AFFT_GB300_API size_t afft_64_ci_memsize(size_t ndim, const size_t* dim, int format, int impl);
AFFT_GB300_API afft_64_ci_type* afft_64_ci_create(
  size_t ndim, const size_t* dim, int format, void* mem, int impl);
AFFT_GB300_API void afft_64_ci_transform(afft_64_ci_type* state,
  const double* src_re, const double* src_im, double* dst_re, double* dst_im);

typedef struct afft_64_r_struct afft_64_r_type;
AFFT_GB300_API size_t afft_64_r_memsize(size_t ndim, const size_t* dim, int format, int impl);
AFFT_GB300_API afft_64_r_type* afft_64_r_create(
  size_t ndim, const size_t* dim, int format, void* mem, int impl);
AFFT_GB300_API void afft_64_r_transform(afft_64_r_type* state,
  const double* src, double* dst_re, double* dst_im);

typedef struct afft_64_ri_struct afft_64_ri_type;
AFFT_GB300_API size_t afft_64_ri_memsize(size_t ndim, const size_t* dim, int format, int impl);
AFFT_GB300_API afft_64_ri_type* afft_64_ri_create(
  size_t ndim, const size_t* dim, int format, void* mem, int impl);
AFFT_GB300_API void afft_64_ri_transform(afft_64_ri_type* state,
  const double* src_re, const double* src_im, double* dst);

AFFT_GB300_API size_t afft_64_align_size(size_t sz);

/* Replaces fft.h:82 / fft.cpp:303-306: 1 for afft_auto and afft_gb300 when a
 * CUDA device of compute capability 10.3 is present, else 0. */
AFFT_GB300_API int afft_supported(int impl);

/* Replaces fft.h:84 / fft.cpp:308: 64. */
extern AFFT_GB300_API const size_t afft_alignment;

/* ------------------------------------------------------------------------ */
/* Part 2: extensions (no counterpart in afft)                               */
/* ------------------------------------------------------------------------ */

/* Error codes of the last failing call on the calling thread. */
enum
{
  AFFT_GB300_OK = 0,
  AFFT_GB300_EINVAL = 1,      /* bad shape, kind, format or pointer          */
  AFFT_GB300_ENODEV = 2,      /* no usable CUDA device                       */
  AFFT_GB300_ENOMEM = 3,      /* device allocation failed                    */
  AFFT_GB300_ECUDA = 4,       /* a CUDA call failed (message has the detail) */
  AFFT_GB300_ESTATE = 5,      /* plan unknown, released or corrupt           */
  AFFT_GB300_ETIMEOUT = 6     /* a bounded device wait gave up               */
};
AFFT_GB300_API int afft_gb300_last_error(void);
AFFT_GB300_API const char* afft_gb300_last_error_string(void);

/* Kinds for the batched and queue entry points. */
enum { afft_gb300_c = 0, afft_gb300_ci = 1, afft_gb300_r = 2, afft_gb300_ri = 3 };

/* Form flag, OR-ed into `format` of afft_gb300_batch_memsize/_create and
 * afft_gb300_plan_describe, or passed to afft_gb300_queue_create_ex:
 * radix-16 butterflies of complex passes of length 256 and 4096 run as
 * split-precision tensor-core DFT-matrix products (FP16 hi + scaled lo
 * operands, three products accumulated in FP32 in TMEM); other passes keep
 * the FP32 butterflies.  Accuracy bound: rel-L2 <= 5e-6 vs FP64. */
enum { AFFT_GB300_FORM_TC = 0x100 };

/* Form flag, OR-ed into `format` of afft_gb300_batch_memsize/_create and
 * afft_gb300_plan_describe: double arrays and FP64 arithmetic (the batched
 * form of the afft_64_* transforms; run it with afft_64_<kind>_transform, or
 * with afft_gb300_transform_async passing the double pointers as float*).
 * Not combinable with AFFT_GB300_FORM_TC, and not accepted by the queue. */
enum { AFFT_GB300_FORM_F64 = 0x200 };

/* Batched plans: `batch` transforms of the same shape, dense and back to
 * back (transform b at offset b*in_elems / b*out_elems of each array, where
 * in/out_elems are prod(dims) for complex and (d0/2+1)*prod(dims[1:]) for
 * the half spectrum of real transforms).  The returned plan is used with the
 * matching afft_32_<kind>_transform call.  memsize/create follow the fft.h
 * conventions (0 / NULL on bad arguments). */
AFFT_GB300_API size_t afft_gb300_batch_memsize(int kind, size_t ndim, const size_t* dim,
  size_t batch, int format);
AFFT_GB300_API void* afft_gb300_batch_create(int kind, size_t ndim, const size_t* dim,
  size_t batch, int format, void* mem);

/* Enqueue one transform of `plan` (any kind; real forward ignores src_im,
 * real inverse ignores dst_im) on `stream` (a cudaStream_t; NULL = the CUDA
 * default stream, as for a kernel launch) without waiting for it.  All four
 * data pointers must be device-accessible.  Returns 0 or an AFFT_GB300_*
 * code. */
AFFT_GB300_API int afft_gb300_transform_async(void* plan, const float* src_re,
  const float* src_im, float* dst_re, float* dst_im, void* stream);

/* Frees the device resources held for `plan` (the caller still frees mem).
 * Returns 0, or AFFT_GB300_ESTATE if the plan is unknown. */
AFFT_GB300_API int afft_gb300_release(void* plan);

/* Describes, without touching a GPU, the kernel launches a plan of this
 * kind, shape, batch and format would issue: a JSON object with the buffer
 * sizes and, per launch, the kernel shape, grid and address arithmetic.
 * Writes at most buflen bytes (NUL-terminated) and returns the length the
 * full description needs, or 0 on bad arguments. */
AFFT_GB300_API size_t afft_gb300_plan_describe(int kind, size_t ndim,
  const size_t* dim, size_t batch, int format, char* buf, size_t buflen);

/* Autotuner (no counterpart in afft): times the plan variants a shape allows
 * on the current device and keeps the fastest for later plans of the same
 * (device, kind, dims, batch, format).  The variants: the four-step split
 * of axes longer than one CTA holds (which half the first pass takes); for
 * long 1D real inverses, the real pre-pass fused into the first pass or run
 * on its own; cols passes loading their tiles by TMA or through the LSU, and
 * the 1024- and 2048-point ones pipelined or one tile per CTA;
 * 8, 16 or 32 lines per CTA for 256- and 512-point complex cols passes; the
 * plain FP32 or the split-precision tensor-core form of the passes that have
 * one; 1D complex axes of 2^20 to 2^22 points in two passes or three; and the
 * last two axes of complex N-D transforms in one plane-fused pass or one pass
 * each.  It allocates scratch device buffers for the timing.
 * Choices are kept for the process and, when the environment variable
 * AFFT_GB300_TUNE_CACHE names a file, stored there and reloaded on first use;
 * with AFFT_GB300_AUTOTUNE=1 every new shape is tuned when its first plan is
 * built.  Plans built before a choice exists use the built-in defaults, and
 * afft_gb300_plan_describe always describes the defaults.  `report` (may be
 * NULL) receives a JSON summary: the candidates with their median times and
 * the choice.  Returns 0 or an AFFT_GB300_* code. */
AFFT_GB300_API int afft_gb300_tune(int kind, size_t ndim, const size_t* dim, size_t batch, int format,
  char* report, size_t report_len);
/* The autotuner's choice for a shape on the current device: 1 and the
 * variant (split, real_inv) if one is known, 0 if not, -1 for a bad shape. */
AFFT_GB300_API int afft_gb300_tuned(int kind, size_t ndim, const size_t* dim, size_t batch, int format,
  int* split, int* real_inv);

/* Self-test of the library's bounded device waits (no counterpart in afft):
 * launches a kernel that waits on a barrier nothing releases, for `iters`
 * polls, and returns AFFT_GB300_ETIMEOUT when the kernel gave up and
 * reported it as designed (-1 on a CUDA error).  Nothing faults or hangs. */
AFFT_GB300_API int afft_gb300_selftest_bounded_wait(int iters);
/* Self-test of the cols passes' TMA tile wait (no counterpart in afft): a
 * kernel issues one tensor-map copy into shared memory while announcing
 * twice its bytes, so the wait never completes; the kernels' time-bounded
 * wait gives up after `limit_us` microseconds and the call returns
 * AFFT_GB300_ETIMEOUT (-1 on a CUDA error).  Nothing faults or hangs. */
AFFT_GB300_API int afft_gb300_selftest_tma_wait(int limit_us);

/* Number of this library's kernel launches one transform of `plan` issues. */
AFFT_GB300_API int afft_gb300_plan_launches(const void* plan);

/* Batched 1D complex transform that allocates nothing -- no counterpart in
 * the reference.  For callers that cannot allocate device memory at call
 * time (a device memory budget fixed at start-up, a custom allocator that
 * owns the free memory, or loops that cannot take cudaMalloc's implicit
 * synchronisation).  Runs the two-pass transform of `batch` dense lengths
 * `n` (forward, or unnormalised inverse when `inverse` is nonzero) from
 * src to dst (device pointers) on `stream` without waiting, with its scratch
 * in a fixed 16 MiB device array inside the library.  Limits: n a power of
 * two in [2^15, 2^21] and n * batch <= 2^21, else AFFT_GB300_EINVAL.  The
 * first call on each device sets up the library's device arrays (make it
 * before any stream capture); calls share the scratch array, so calls whose
 * kernels overlap on the GPU race.  Returns 0 or an AFFT_GB300_* code. */
AFFT_GB300_API int afft_gb300_c2c_noalloc(const float* src_re,
  const float* src_im, float* dst_re, float* dst_im, size_t n, size_t batch,
  int inverse, void* stream);

/* Descriptor of one transform in a multi-transform queue.  dims beyond ndim
 * are ignored.  Pointers are device pointers.  For 'ci' and 'ri' the output
 * is unnormalised as above. */
typedef struct afft_gb300_desc
{
  int kind;              /* afft_gb300_c / ci / r / ri */
  int ndim;              /* 1..3 */
  size_t dim[3];
  const float* src_re;
  const float* src_im;   /* unused for r */
  float* dst_re;
  float* dst_im;         /* unused for ri */
} afft_gb300_desc;

/* A queue runs many transforms of mixed sizes and kinds as one unit: plans
 * are made once per distinct (kind, shape), the launches of all transforms
 * are grouped by kernel and recorded into one CUDA graph on first run, and
 * each later run replays that graph.  The descriptor array is copied.  The
 * transforms are independent: they run in no particular order relative to
 * each other, so no transform's output may overlap another's input or
 * output. */
typedef struct afft_gb300_queue afft_gb300_queue;
AFFT_GB300_API afft_gb300_queue* afft_gb300_queue_create(const afft_gb300_desc* descs,
  size_t count);
/* Queue flag (no counterpart in afft): every distinct (kind, shape) among
 * the queue's transforms takes the autotuner's choice for queues -- tuned
 * on first use at a batch of about 2^24 elements, timed on this device, and
 * kept like afft_gb300_tune's choices (under batch 0) -- instead of the
 * built-in defaults.  Tuning allocates device buffers while the queue is
 * created. */
enum { AFFT_GB300_QUEUE_TUNED = 0x400 };
/* As afft_gb300_queue_create; flags: 0, AFFT_GB300_FORM_TC and/or
 * AFFT_GB300_QUEUE_TUNED. */
AFFT_GB300_API afft_gb300_queue* afft_gb300_queue_create_ex(
  const afft_gb300_desc* descs, size_t count, int flags);
/* `stream` as for afft_gb300_transform_async (NULL = default stream). */
AFFT_GB300_API int afft_gb300_queue_run(afft_gb300_queue* q, void* stream);
/* Kernel launches one run issues (after grouping). */
AFFT_GB300_API int afft_gb300_queue_launches(const afft_gb300_queue* q);
AFFT_GB300_API void afft_gb300_queue_destroy(afft_gb300_queue* q);

#ifdef __cplusplus
}
#endif

#endif
