/*
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the GB300 library
 * and the timed CPU baseline; it is never linked into, called by, or used as a
 * fallback of the product library (fft_gb300/).  Only tests/, the smoke check
 * and bench.py's CPU-baseline leg may load it.
 *
 * Two independent CPU restatements of the afft (jkrempus/fft) power-of-two
 * FFT path, both on split re/im arrays, row-major, size-1 dims removed
 * (common.hpp:68-84), forward = exp(-2*pi*i*jk/n), inverse unnormalised:
 *
 *   oracle64_*  FP64 restatement of the reference test harness's oracle
 *               ReferenceFft<double> (testing.cpp:870-1002): radix-2 Stockham
 *               per dimension, twiddles from cos/sin directly.  Real forward
 *               keeps planes 0..d0/2 of the first dimension (testing.cpp:
 *               529-559); real inverse is the linear map the reference's
 *               irfft computes (fft_internal.hpp:467-493): inverse transform
 *               of the trailing dims per plane, then a half-complex inverse
 *               along dim 0 that reads only the real part of planes 0 and d0/2.
 *
 *   port32_*    FP32 scalar port of afft's own algorithm (port64_*: the same
 *               on doubles), used as the CPU
 *               baseline ("port"): radix-4 decimation passes with bit-reversed
 *               twiddle order and a final radix-8 step (onedim.hpp:55-133,
 *               135-191, 312-395, 485-507), twiddles built by afft's table
 *               recurrence (common.hpp:447-546, 605-770), the real pre/post
 *               pass (onedim.hpp:1031-1108, multi.hpp:343-414) and the N-D
 *               composition (fft_internal.hpp:121-152, 320-346, 467-493).
 *
 * Parity is pinned against outputs of the reference library itself (built
 * from its sources by oracle/Makefile) through the fixtures in tests/golden/.
 */
#ifndef AFFT_ORACLE_H
#define AFFT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_C = 0, ORACLE_CI = 1, ORACLE_R = 2, ORACLE_RI = 3 };

/* std::mt19937(seed) feeding uniform_real_distribution<float>(lo, hi), the
 * input generator of the reference harness (testing.cpp:1064-1067). */
void oracle_mt19937_uniform(uint32_t seed, int64_t count, float lo, float hi,
                            float* out);
/* Raw 32-bit outputs of std::mt19937(seed). */
void oracle_mt19937_raw(uint32_t seed, int64_t count, uint32_t* out);

/* Drops size-1 dims; returns the new ndim (>= 1) and writes dims to out. */
int oracle_squeeze_dims(int ndim, const int64_t* dims, int64_t* out);

/* All return 0 on success, -1 on invalid shape (non power of two, ndim<1). */
int oracle64_c2c(int ndim, const int64_t* dims, int inverse,
                 const double* in_re, const double* in_im,
                 double* out_re, double* out_im);
int oracle64_r2c(int ndim, const int64_t* dims, const double* in,
                 double* out_re, double* out_im);
int oracle64_c2r(int ndim, const int64_t* dims, const double* in_re,
                 const double* in_im, double* out);

/* FP32 port of afft.  `kind` is ORACLE_C / CI / R / RI.  A plan precomputes
 * twiddles once; execute is reentrant (scratch is per call). */
typedef struct port32_plan port32_plan;
port32_plan* port32_plan_create(int kind, int ndim, const int64_t* dims);
void port32_plan_destroy(port32_plan* p);
/* Element counts of one transform's input and output arrays (per array). */
int64_t port32_plan_in_elems(const port32_plan* p);
int64_t port32_plan_out_elems(const port32_plan* p);
/* One transform.  Real forward: in_im ignored, out split.  Real inverse:
 * in split, out_im ignored. */
int port32_execute(const port32_plan* p, const float* in_re, const float* in_im,
                   float* out_re, float* out_im);
/* `batch` dense transforms spread over `threads` POSIX threads. */
int port32_execute_batch(const port32_plan* p, int64_t batch, int threads,
                         const float* in_re, const float* in_im,
                         float* out_re, float* out_im);

/* FP64 port of afft: the same algorithm and API on doubles (afft_64_*). */
typedef struct port64_plan port64_plan;
port64_plan* port64_plan_create(int kind, int ndim, const int64_t* dims);
void port64_plan_destroy(port64_plan* p);
int64_t port64_plan_in_elems(const port64_plan* p);
int64_t port64_plan_out_elems(const port64_plan* p);
int port64_execute(const port64_plan* p, const double* in_re, const double* in_im,
                   double* out_re, double* out_im);
int port64_execute_batch(const port64_plan* p, int64_t batch, int threads,
                         const double* in_re, const double* in_im,
                         double* out_re, double* out_im);

#ifdef __cplusplus
}
#endif

#endif
