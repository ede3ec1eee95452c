/*
 * TEST INFRASTRUCTURE ONLY -- the oracle and CPU baseline for the GB300 FFT
 * library.  Never linked into or called by the product path.  See
 * afft_oracle.h for what is restated from where.
 */
#define _GNU_SOURCE
#include "afft_oracle.h"
#include "afft_shape.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* shape helpers                                                            */
/* ------------------------------------------------------------------------ */

/* common.hpp:68-84 remove_redundant_dimensions */
int oracle_squeeze_dims(int ndim, const int64_t* dims, int64_t* out)
{
  int k = 0;
  for (int i = 0; i < ndim; i++)
    if (dims[i] != 1) out[k++] = dims[i];
  if (k == 0) out[k++] = 1;
  return k;
}

/* ------------------------------------------------------------------------ */
/* std::mt19937 + uniform_real_distribution<float> (testing.cpp:1064-1067)   */
/* The generator is the published MT19937 (Matsumoto & Nishimura 1998); the  */
/* float mapping is libstdc++'s generate_canonical<float, 24>: one 32-bit    */
/* draw, float(u) / 2^32, clamped below 1, then u * (hi - lo) + lo.          */
/* ------------------------------------------------------------------------ */

typedef struct { uint32_t s[624]; int i; } mt_state;

static void mt_seed(mt_state* m, uint32_t seed)
{
  m->s[0] = seed;
  for (int k = 1; k < 624; k++)
    m->s[k] = 1812433253u * (m->s[k - 1] ^ (m->s[k - 1] >> 30)) + (uint32_t)k;
  m->i = 624;
}

static uint32_t mt_next(mt_state* m)
{
  if (m->i >= 624) {
    for (int k = 0; k < 624; k++) {
      uint32_t y = (m->s[k] & 0x80000000u) | (m->s[(k + 1) % 624] & 0x7fffffffu);
      m->s[k] = m->s[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    m->i = 0;
  }
  uint32_t y = m->s[m->i++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

void oracle_mt19937_raw(uint32_t seed, int64_t count, uint32_t* out)
{
  mt_state m;
  mt_seed(&m, seed);
  for (int64_t k = 0; k < count; k++) out[k] = mt_next(&m);
}

void oracle_mt19937_uniform(uint32_t seed, int64_t count, float lo, float hi,
                            float* out)
{
  mt_state m;
  mt_seed(&m, seed);
  for (int64_t k = 0; k < count; k++) {
    float c = (float)mt_next(&m) / 4294967296.0f;
    if (c >= 1.0f) c = nextafterf(1.0f, 0.0f);
    out[k] = c * (hi - lo) + lo;
  }
}

/* ------------------------------------------------------------------------ */
/* FP64 oracle: testing.cpp:870-1002 ReferenceFft<double>                    */
/* ------------------------------------------------------------------------ */

/* testing.cpp:906-937 Onedim::transform -- radix-2 Stockham, interleaved.   */
static void ref64_line(int64_t n, const double* tw, double* data, double* work)
{
  for (int64_t dft = 1; dft < n; dft *= 2) {
    memcpy(work, data, sizeof(double) * 2 * (size_t)n);
    int64_t tw_stride = n / 2 / dft;
    for (int64_t i = 0; i < n / 2; i += dft) {
      for (int64_t s = i, d = 2 * i, t = 0; s < i + dft; s++, d++, t += tw_stride) {
        double ar = work[2 * s], ai = work[2 * s + 1];
        double br = work[2 * (s + n / 2)], bi = work[2 * (s + n / 2) + 1];
        double wr = tw[2 * t], wi = tw[2 * t + 1];
        double mr = wr * br - wi * bi, mi = wr * bi + wi * br;
        data[2 * d] = ar + mr;
        data[2 * d + 1] = ai + mi;
        data[2 * (d + dft)] = ar - mr;
        data[2 * (d + dft) + 1] = ai - mi;
      }
    }
  }
}

/* testing.cpp:910-920: twiddle[i] = exp(-+ i*pi*i/(n/2)), computed directly */
static double* ref64_twiddles(int64_t n, int inverse)
{
  double* tw = (double*)malloc(sizeof(double) * (size_t)(n > 1 ? n : 2));
  double pi = acos(-1.0);
  for (int64_t i = 0; i < n / 2; i++) {
    double phi = (inverse ? 1.0 : -1.0) * (double)i * pi / (double)(n / 2);
    tw[2 * i] = cos(phi);
    tw[2 * i + 1] = sin(phi);
  }
  return tw;
}

/* testing.cpp:965-1001: one 1D transform per line of every dimension,
 * buf interleaved complex of prod(dims) elements, in place. */
static void ref64_nd_inplace(int ndim, const int64_t* dims, int inverse, double* buf)
{
  for (int d = 0; d < ndim; d++) {
    int64_t n = dims[d];
    if (n == 1) continue;
    int64_t stride = prod(dims + d + 1, ndim - d - 1);
    int64_t outer = prod(dims, d);
    double* tw = ref64_twiddles(n, inverse);
    double* line = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    double* work = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    for (int64_t o = 0; o < outer; o++)
      for (int64_t c = 0; c < stride; c++) {
        double* base = buf + 2 * (o * n * stride + c);
        for (int64_t k = 0; k < n; k++) {
          line[2 * k] = base[2 * k * stride];
          line[2 * k + 1] = base[2 * k * stride + 1];
        }
        ref64_line(n, tw, line, work);
        for (int64_t k = 0; k < n; k++) {
          base[2 * k * stride] = line[2 * k];
          base[2 * k * stride + 1] = line[2 * k + 1];
        }
      }
    free(tw);
    free(line);
    free(work);
  }
}

int oracle64_c2c(int ndim_in, const int64_t* dims_in, int inverse,
                 const double* in_re, const double* in_im,
                 double* out_re, double* out_im)
{
  int64_t dims[64];
  if (ndim_in < 1 || ndim_in > 64) return -1;
  int ndim = oracle_squeeze_dims(ndim_in, dims_in, dims);
  if (!valid_shape(ndim, dims)) return -1;
  int64_t N = prod(dims, ndim);
  double* buf = (double*)malloc(sizeof(double) * 2 * (size_t)N);
  for (int64_t i = 0; i < N; i++) { buf[2 * i] = in_re[i]; buf[2 * i + 1] = in_im[i]; }
  ref64_nd_inplace(ndim, dims, inverse, buf);
  for (int64_t i = 0; i < N; i++) { out_re[i] = buf[2 * i]; out_im[i] = buf[2 * i + 1]; }
  free(buf);
  return 0;
}

/* Real forward: complex transform of (x, 0), keep planes 0..d0/2 of the
 * first (non-1) dimension, the layout of testing.cpp:529-559. */
int oracle64_r2c(int ndim_in, const int64_t* dims_in, const double* in,
                 double* out_re, double* out_im)
{
  int64_t dims[64];
  if (ndim_in < 1 || ndim_in > 64) return -1;
  int ndim = oracle_squeeze_dims(ndim_in, dims_in, dims);
  if (!valid_shape(ndim, dims)) return -1;
  int64_t N = prod(dims, ndim);
  int64_t inner = N / dims[0];
  int64_t H = (dims[0] / 2 + 1) * inner;
  double* buf = (double*)malloc(sizeof(double) * 2 * (size_t)N);
  for (int64_t i = 0; i < N; i++) { buf[2 * i] = in[i]; buf[2 * i + 1] = 0.0; }
  ref64_nd_inplace(ndim, dims, 0, buf);
  for (int64_t i = 0; i < H; i++) { out_re[i] = buf[2 * i]; out_im[i] = buf[2 * i + 1]; }
  free(buf);
  return 0;
}

/* Real inverse: the map of fft_internal.hpp:467-493 / onedim.hpp:1242-1254.
 * Inverse transform of the trailing dims per plane, then along dim 0 the
 * Hermitian extension F[k]=Y[k], F[d0-k]=conj(Y[k]) with only the real part
 * of planes 0 and d0/2 used (multi.hpp:390-402, onedim.hpp:1097-1101), then
 * the inverse along dim 0; unnormalised. */
int oracle64_c2r(int ndim_in, const int64_t* dims_in, const double* in_re,
                 const double* in_im, double* out)
{
  int64_t dims[64];
  if (ndim_in < 1 || ndim_in > 64) return -1;
  int ndim = oracle_squeeze_dims(ndim_in, dims_in, dims);
  if (!valid_shape(ndim, dims)) return -1;
  int64_t d0 = dims[0], L = d0 / 2;
  int64_t N = prod(dims, ndim);
  int64_t inner = N / d0;
  int64_t planes = L + 1;
  double* buf = (double*)malloc(sizeof(double) * 2 * (size_t)(planes * inner));
  for (int64_t i = 0; i < planes * inner; i++) {
    buf[2 * i] = in_re[i];
    buf[2 * i + 1] = in_im[i];
  }
  if (ndim > 1)
    for (int64_t p = 0; p < planes; p++)
      ref64_nd_inplace(ndim - 1, dims + 1, 1, buf + 2 * p * inner);

  if (d0 == 1) {
    for (int64_t c = 0; c < inner; c++) out[c] = buf[2 * c];
    free(buf);
    return 0;
  }
  double* tw = ref64_twiddles(d0, 1);
  double* line = (double*)malloc(sizeof(double) * 2 * (size_t)d0);
  double* work = (double*)malloc(sizeof(double) * 2 * (size_t)d0);
  for (int64_t c = 0; c < inner; c++) {
    line[0] = buf[2 * c];
    line[1] = 0.0;
    line[2 * L] = buf[2 * (L * inner + c)];
    line[2 * L + 1] = 0.0;
    for (int64_t k = 1; k < L; k++) {
      double yr = buf[2 * (k * inner + c)], yi = buf[2 * (k * inner + c) + 1];
      line[2 * k] = yr;
      line[2 * k + 1] = yi;
      line[2 * (d0 - k)] = yr;
      line[2 * (d0 - k) + 1] = -yi;
    }
    ref64_line(d0, tw, line, work);
    for (int64_t k = 0; k < d0; k++) out[k * inner + c] = line[2 * k];
  }
  free(tw);
  free(line);
  free(work);
  free(buf);
  return 0;
}
