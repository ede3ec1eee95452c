/*
 * TEST INFRASTRUCTURE ONLY -- the oracle and CPU baseline for the GB300 FFT
 * library.  Never linked into or called by the product path.  See
 * afft_oracle.h for what is restated from where.
 */
#define _GNU_SOURCE
#include "afft_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* shape helpers                                                            */
/* ------------------------------------------------------------------------ */

static int is_pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

static int ilog2(int64_t v)
{
  int r = 0;
  while (v > 1) { v >>= 1; r++; }
  return r;
}

static int64_t rev_bits(int64_t v, int nbits)
{
  int64_t r = 0;
  for (int i = 0; i < nbits; i++) { r = (r << 1) | (v & 1); v >>= 1; }
  return r;
}

/* common.hpp:68-84 remove_redundant_dimensions */
int oracle_squeeze_dims(int ndim, const int64_t* dims, int64_t* out)
{
  int k = 0;
  for (int i = 0; i < ndim; i++)
    if (dims[i] != 1) out[k++] = dims[i];
  if (k == 0) out[k++] = 1;
  return k;
}

static int valid_shape(int ndim, const int64_t* dims)
{
  if (ndim < 1 || ndim > 64) return 0;
  for (int i = 0; i < ndim; i++)
    if (!is_pow2(dims[i])) return 0;
  return 1;
}

static int64_t prod(const int64_t* d, int n)
{
  int64_t r = 1;
  for (int i = 0; i < n; i++) r *= d[i];
  return r;
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

/* ------------------------------------------------------------------------ */
/* FP32 port of afft's algorithm                                             */
/* ------------------------------------------------------------------------ */

/* common.hpp:447-546 SinCosTable<float>: sin/cos(pi * 2^-i), generated the way
 * table.cpp:5-25 does (float pi scaled by a power of two, float sin/cos). */
static float g_sin[64], g_cos[64];
static pthread_once_t g_table_once = PTHREAD_ONCE_INIT;
static void init_table(void)
{
  for (int i = 0; i < 64; i++) {
    float a = (float)M_PI * ldexpf(1.0f, -i);
    g_sin[i] = sinf(a);
    g_cos[i] = cosf(a);
  }
}

typedef struct { float re, im; } cf32;

/* common.hpp:242-254: product with separate roundings (no fused multiply). */
static inline cf32 cmul(cf32 a, cf32 b)
{
  cf32 r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}
static inline cf32 cadd(cf32 a, cf32 b) { cf32 r = {a.re + b.re, a.im + b.im}; return r; }
static inline cf32 csub(cf32 a, cf32 b) { cf32 r = {a.re - b.re, a.im - b.im}; return r; }
static inline cf32 cneg_i(cf32 a) { cf32 r = {a.im, -a.re}; return r; }   /* -i*a */
static inline cf32 cadj(cf32 a) { cf32 r = {a.re, -a.im}; return r; }
static inline cf32 cscale(cf32 a, float s) { cf32 r = {a.re * s, a.im * s}; return r; }

/* common.hpp:624-653 compute_twiddle_step */
static void twiddle_step(const float* src_re, const float* src_im, int64_t full,
                         int64_t dst_size, float* dst_re, float* dst_im)
{
  int t = ilog2(full);
  float c = g_cos[t], s = g_sin[t];
  for (int64_t j = 0; j < dst_size / 2; j++) {
    float ar = src_re[j], ai = src_im[j];
    float br = ar * c + ai * s;
    float bi = ai * c - ar * s;
    dst_re[2 * j] = ar;
    dst_re[2 * j + 1] = br;
    dst_im[2 * j] = ai;
    dst_im[2 * j + 1] = bi;
  }
}

/* common.hpp:676-695 compute_twiddle_range: row of length s at n-2s holds
 * W_{2s}^j, built by the recurrence above. */
static void twiddle_range(int64_t n, float* re, float* im)
{
  re[n - 1] = 0.0f; im[n - 1] = 0.0f;
  if (n >= 2) { re[n - 2] = 1.0f; im[n - 2] = 0.0f; }
  for (int64_t size = 2; size < n; size *= 2)
    twiddle_step(re + n - size, im + n - size, size, size,
                 re + n - 2 * size, im + n - 2 * size);
}

/* common.hpp:655-674 compute_twiddle: re/im[j] = W_{2n}^j, j < n. */
static void twiddle_full(int64_t n, float* re, float* im)
{
  re[n - 1] = 1.0f; im[n - 1] = 0.0f;
  for (int64_t size = 2; size <= n; size *= 2)
    twiddle_step(re + n - size / 2, im + n - size / 2, size, size,
                 re + n - size, im + n - size);
}

/* One length-n complex transform: the step schedule of onedim.hpp:755-797
 * for the scalar backend (first step radix-4, then radix-4 steps, the last
 * step radix-8 when dft_size*8 == n) with per-step packed twiddles of
 * common.hpp:697-770 (slot rev(i) holds W_{4d}^i, its square and cube, plus
 * W_{8d}^i and W_{8d}^{i+d} for a radix-8 step). */
typedef struct {
  int64_t n;
  int nsteps;
  int64_t dft[64];
  int npasses[64];
  cf32* tw[64];
} port1d;

static void port1d_free(port1d* p)
{
  for (int i = 0; i < p->nsteps; i++) free(p->tw[i]);
  p->nsteps = 0;
}

static void port1d_init(port1d* p, int64_t n)
{
  pthread_once(&g_table_once, init_table);
  memset(p, 0, sizeof(*p));
  p->n = n;
  if (n <= 8) return;  /* tiny sizes: direct formulas */
  float* rre = (float*)malloc(sizeof(float) * (size_t)n);
  float* rim = (float*)malloc(sizeof(float) * (size_t)n);
  twiddle_range(n, rre, rim);
  int64_t d = 4;
  while (d != n) {
    int np = ((d << 3) == n) ? 3 : 2;
    int per = np == 3 ? 5 : 3;
    cf32* t = (cf32*)malloc(sizeof(cf32) * (size_t)(per * d));
    const float* r0re = rre + (n - 4 * d);
    const float* r0im = rim + (n - 4 * d);
    int nb = ilog2(d);
    for (int64_t i = 0; i < d; i++) {
      int64_t slot = rev_bits(i, nb);
      cf32 t0 = {r0re[i], r0im[i]};
      cf32 t1 = cmul(t0, t0);         /* common.hpp:605-613 */
      cf32 t2 = cmul(t1, t0);
      t[per * slot + 0] = t0;
      t[per * slot + 1] = t1;
      t[per * slot + 2] = t2;
      if (np == 3) {
        const float* r1re = rre + (n - 8 * d);
        const float* r1im = rim + (n - 8 * d);
        cf32 t3 = {r1re[i], r1im[i]};
        cf32 t4 = {r1re[i + d], r1im[i + d]};
        t[per * slot + 3] = t3;
        t[per * slot + 4] = t4;
      }
    }
    p->dft[p->nsteps] = d;
    p->npasses[p->nsteps] = np;
    p->tw[p->nsteps] = t;
    p->nsteps++;
    d <<= np;
  }
  free(rre);
  free(rim);
}

/* A "row buffer": n rows of m contiguous complex values, split re/im, row r
 * starting at r*rs.  m == 1 is a plain 1D array (rs = 2 reads an interleaved
 * pair view, as cf::Scal does). */
typedef struct { float* re; float* im; int64_t rs; } rows_t;

static inline cf32 rget(rows_t b, int64_t r, int64_t c)
{
  cf32 v = {b.re[r * b.rs + c], b.im[r * b.rs + c]};
  return v;
}
static inline void rput(rows_t b, int64_t r, int64_t c, cf32 v)
{
  b.re[r * b.rs + c] = v.re;
  b.im[r * b.rs + c] = v.im;
}

/* onedim.hpp:55-70 two_passes_inner_unity_twiddle: DFT-4, outputs in order. */
static inline void dft4(cf32 s0, cf32 s1, cf32 s2, cf32 s3,
                        cf32* d0, cf32* d1, cf32* d2, cf32* d3)
{
  cf32 sum02 = cadd(s0, s2), dif02 = csub(s0, s2);
  cf32 sum13 = cadd(s1, s3), dif13 = csub(s1, s3);
  *d0 = cadd(sum02, sum13);
  *d2 = csub(sum02, sum13);
  *d1 = cadd(dif02, cneg_i(dif13));
  *d3 = csub(dif02, cneg_i(dif13));
}

/* Tiny sizes (the register-resident transforms of onedim.hpp:596-753),
 * written with the radix-4 / radix-8 formulas of onedim.hpp:55-81, 193-242. */
static void port_tiny(int64_t n, int64_t m, rows_t src, rows_t dst)
{
  for (int64_t c = 0; c < m; c++) {
    if (n == 1) {
      rput(dst, 0, c, rget(src, 0, c));
    } else if (n == 2) {
      cf32 a = rget(src, 0, c), b = rget(src, 1, c);
      rput(dst, 0, c, cadd(a, b));
      rput(dst, 1, c, csub(a, b));
    } else if (n == 4) {
      cf32 d0, d1, d2, d3;
      dft4(rget(src, 0, c), rget(src, 1, c), rget(src, 2, c), rget(src, 3, c),
           &d0, &d1, &d2, &d3);
      rput(dst, 0, c, d0); rput(dst, 1, c, d1);
      rput(dst, 2, c, d2); rput(dst, 3, c, d3);
    } else { /* n == 8 */
      float h = g_cos[2];
      cf32 a0, a1, a2, a3, b0, b1, b2, b3;
      dft4(rget(src, 0, c), rget(src, 2, c), rget(src, 4, c), rget(src, 6, c),
           &a0, &a1, &a2, &a3);
      dft4(rget(src, 1, c), rget(src, 3, c), rget(src, 5, c), rget(src, 7, c),
           &b0, &b1, &b2, &b3);
      cf32 m0 = b0;
      cf32 m1 = {h * (b1.re + b1.im), h * (b1.im - b1.re)};
      cf32 m2 = cneg_i(b2);
      cf32 m3 = {h * (b3.im - b3.re), h * (-b3.im - b3.re)};
      rput(dst, 0, c, cadd(a0, m0)); rput(dst, 4, c, csub(a0, m0));
      rput(dst, 1, c, cadd(a1, m1)); rput(dst, 5, c, csub(a1, m1));
      rput(dst, 2, c, cadd(a2, m2)); rput(dst, 6, c, csub(a2, m2));
      rput(dst, 3, c, cadd(a3, m3)); rput(dst, 7, c, csub(a3, m3));
    }
  }
}

/* Forward transform of n rows (each m wide): src -> work (first step,
 * onedim.hpp:135-191) -> in place middle radix-4 steps (onedim.hpp:312-353)
 * -> dst, scattered to natural order by the last step (onedim.hpp:355-395
 * radix-4, onedim.hpp:83-133 + 485-507 radix-8).  src may alias dst; work
 * must hold n*m complex values and alias neither. */
static void port_rows_fwd(const port1d* P, int64_t m, rows_t src, rows_t work,
                          rows_t dst)
{
  int64_t n = P->n;
  if (n <= 8) {
    /* stage through work so src may alias dst */
    port_tiny(n, m, src, work);
    for (int64_t r = 0; r < n; r++)
      for (int64_t c = 0; c < m; c++) rput(dst, r, c, rget(work, r, c));
    return;
  }
  int64_t q = n / 4;
  for (int64_t j = 0; j < q; j++)
    for (int64_t c = 0; c < m; c++) {
      cf32 d0, d1, d2, d3;
      dft4(rget(src, j, c), rget(src, j + q, c), rget(src, j + 2 * q, c),
           rget(src, j + 3 * q, c), &d0, &d1, &d2, &d3);
      rput(work, j, c, d0);
      rput(work, j + q, c, d2);
      rput(work, j + 2 * q, c, d1);
      rput(work, j + 3 * q, c, d3);
    }

  for (int s = 0; s < P->nsteps; s++) {
    int64_t d = P->dft[s];
    int np = P->npasses[s];
    const cf32* tw = P->tw[s];
    int last = (d << np) == n;
    if (!last) {
      int64_t off1 = n / d / 4;
      for (int64_t b = 0; b < d; b++) {
        cf32 t0 = tw[3 * b], t1 = tw[3 * b + 1], t2 = tw[3 * b + 2];
        int64_t base = b * (n / d);
        for (int64_t j = 0; j < off1; j++)
          for (int64_t c = 0; c < m; c++) {
            int64_t r = base + j;
            cf32 d0, d1, d2, d3;
            dft4(rget(work, r, c), cmul(t0, rget(work, r + off1, c)),
                 cmul(t1, rget(work, r + 2 * off1, c)),
                 cmul(t2, rget(work, r + 3 * off1, c)), &d0, &d1, &d2, &d3);
            rput(work, r, c, d0);
            rput(work, r + off1, c, d2);
            rput(work, r + 2 * off1, c, d1);
            rput(work, r + 3 * off1, c, d3);
          }
      }
    } else if (np == 2) {
      int nb = ilog2(n / 4);
      for (int64_t b = 0; b < n / 4; b++) {
        cf32 t0 = tw[3 * b], t1 = tw[3 * b + 1], t2 = tw[3 * b + 2];
        int64_t o = rev_bits(b, nb);
        for (int64_t c = 0; c < m; c++) {
          cf32 d0, d1, d2, d3;
          dft4(rget(work, 4 * b, c), cmul(t0, rget(work, 4 * b + 1, c)),
               cmul(t1, rget(work, 4 * b + 2, c)),
               cmul(t2, rget(work, 4 * b + 3, c)), &d0, &d1, &d2, &d3);
          rput(dst, o, c, d0);
          rput(dst, o + q, c, d1);
          rput(dst, o + 2 * q, c, d2);
          rput(dst, o + 3 * q, c, d3);
        }
      }
    } else {
      int64_t m8 = n / 8;
      int nb = ilog2(m8);
      for (int64_t b = 0; b < m8; b++) {
        const cf32* t = tw + 5 * b;
        int64_t o = rev_bits(b, nb);
        for (int64_t c = 0; c < m; c++) {
          int64_t r = 8 * b;
          cf32 a0, a1, a2, a3, a4, a5, a6, a7;
          dft4(rget(work, r, c), cmul(t[0], rget(work, r + 2, c)),
               cmul(t[1], rget(work, r + 4, c)), cmul(t[2], rget(work, r + 6, c)),
               &a0, &a1, &a2, &a3);
          dft4(rget(work, r + 1, c), cmul(t[0], rget(work, r + 3, c)),
               cmul(t[1], rget(work, r + 5, c)), cmul(t[2], rget(work, r + 7, c)),
               &a4, &a5, &a6, &a7);
          cf32 mul = cmul(t[3], a4);
          rput(dst, o, c, cadd(a0, mul));
          rput(dst, o + 4 * m8, c, csub(a0, mul));
          mul = cmul(cneg_i(t[3]), a6);
          rput(dst, o + 2 * m8, c, cadd(a2, mul));
          rput(dst, o + 6 * m8, c, csub(a2, mul));
          mul = cmul(t[4], a5);
          rput(dst, o + 1 * m8, c, cadd(a1, mul));
          rput(dst, o + 5 * m8, c, csub(a1, mul));
          mul = cmul(cneg_i(t[4]), a7);
          rput(dst, o + 3 * m8, c, cadd(a3, mul));
          rput(dst, o + 7 * m8, c, csub(a3, mul));
        }
      }
    }
  }
}

/* Inverse = forward with re and im exchanged on load and store, the
 * cf::Swapped trick of common.hpp:355-378 / fft_internal.hpp:185-198. */
static rows_t swapped(rows_t b)
{
  rows_t r = {b.im, b.re, b.rs};
  return r;
}

static void port_rows(const port1d* P, int64_t m, int inverse, rows_t src,
                      rows_t work, rows_t dst)
{
  if (inverse)
    port_rows_fwd(P, m, swapped(src), swapped(work), swapped(dst));
  else
    port_rows_fwd(P, m, src, work, dst);
}

/* onedim.hpp:1031-1108 real_pass (scalar), n = real length, L = n/2 complex
 * bins in z (split), tw[j] = W_n^j.  Forward writes n/2+1 bins to dst;
 * inverse reads n/2+1 bins and writes the L packed bins to dst.  src may
 * alias dst. */
static void real_pass_1d(int64_t n, int inverse, const float* s_re, const float* s_im,
                         const float* tw_re, const float* tw_im,
                         float* d_re, float* d_im)
{
  int64_t L = n / 2;
  cf32 start = {s_re[0], s_im[0]};
  cf32 end = {0.0f, 0.0f};
  if (inverse) { end.re = s_re[L]; end.im = s_im[L]; }
  cf32 middle = {s_re[n / 4], s_im[n / 4]};
  for (int64_t i0 = 1, i1 = L - 1; i0 <= i1; i0++, i1--) {
    cf32 w = {tw_re[i0], tw_im[i0]};
    cf32 s0 = {s_re[i0], s_im[i0]};
    cf32 s1 = {s_re[i1], s_im[i1]};
    cf32 a, b;
    if (inverse) {
      a = cadd(s0, cadj(s1));
      b = cmul(csub(cadj(s1), s0), cadj(w));
    } else {
      a = cscale(cadd(s0, cadj(s1)), 0.5f);
      b = cscale(cmul(csub(s0, cadj(s1)), w), 0.5f);
    }
    cf32 o0 = cadd(a, cneg_i(b));
    cf32 o1 = cadd(cadj(a), cneg_i(cadj(b)));
    d_re[i0] = o0.re; d_im[i0] = o0.im;
    d_re[i1] = o1.re; d_im[i1] = o1.im;
  }
  cf32 mid = cscale(cadj(middle), inverse ? 2.0f : 1.0f);
  d_re[n / 4] = mid.re; d_im[n / 4] = mid.im;
  if (inverse) {
    d_re[0] = start.re + end.re;
    d_im[0] = start.re - end.re;
  } else {
    d_re[0] = start.re + start.im; d_im[0] = 0.0f;
    d_re[L] = start.re - start.im; d_im[L] = 0.0f;
  }
}

/* multi.hpp:343-414 real_pass over rows (n = dim-0 length, rows of m values,
 * n/2+1 rows in b), in place, tw[j] = W_n^j. */
static void real_pass_rows(int64_t n, int64_t m, int inverse, const float* tw_re,
                           const float* tw_im, rows_t b)
{
  int64_t L = n / 2;
  for (int64_t i = 1; i <= n / 4; i++) {
    cf32 w = {tw_re[i], tw_im[i]};
    for (int64_t c = 0; c < m; c++) {
      cf32 s0 = rget(b, i, c), s1 = rget(b, L - i, c);
      cf32 a, bb;
      if (inverse) {
        a = cadd(s0, cadj(s1));
        bb = cmul(csub(cadj(s1), s0), cadj(w));
      } else {
        a = cscale(cadd(s0, cadj(s1)), 0.5f);
        bb = cscale(cmul(csub(s0, cadj(s1)), w), 0.5f);
      }
      rput(b, i, c, cadd(a, cneg_i(bb)));
      rput(b, L - i, c, cadd(cadj(a), cneg_i(cadj(bb))));
    }
  }
  for (int64_t c = 0; c < m; c++) {
    if (inverse) {
      float r0 = b.re[c], r1 = b.re[L * b.rs + c];
      cf32 v = {r0 + r1, r0 - r1};
      rput(b, 0, c, v);
    } else {
      cf32 r0 = rget(b, 0, c);
      cf32 v0 = {r0.re + r0.im, 0.0f}, v1 = {r0.re - r0.im, 0.0f};
      rput(b, 0, c, v0);
      rput(b, L, c, v1);
    }
  }
}

struct port32_plan {
  int kind;
  int ndim;
  int64_t dims[64];
  int64_t N;          /* real/complex elements of the full-size array      */
  int64_t in_elems, out_elems;
  port1d dimplan[64]; /* complex plan per dim (dim 0 halved for real N-D)   */
  port1d halfplan;    /* real 1D: length n/2                               */
  float* rtw_re;      /* real pass twiddles W_{d0}^j, j < d0/2             */
  float* rtw_im;
  int64_t scratch;    /* complex elements of scratch per transform          */
};

port32_plan* port32_plan_create(int kind, int ndim_in, const int64_t* dims_in)
{
  if (kind < 0 || kind > 3 || ndim_in < 1 || ndim_in > 64) return NULL;
  port32_plan* p = (port32_plan*)calloc(1, sizeof(port32_plan));
  p->kind = kind;
  p->ndim = oracle_squeeze_dims(ndim_in, dims_in, p->dims);
  if (!valid_shape(p->ndim, p->dims)) { free(p); return NULL; }
  p->N = prod(p->dims, p->ndim);
  int real = kind >= 2;
  int64_t d0 = p->dims[0];
  int64_t inner = p->N / d0;
  int64_t H = (d0 / 2 + 1) * inner;
  if (!real) { p->in_elems = p->N; p->out_elems = p->N; }
  else if (kind == ORACLE_R) { p->in_elems = p->N; p->out_elems = H; }
  else { p->in_elems = H; p->out_elems = p->N; }
  for (int d = 0; d < p->ndim; d++) {
    int64_t len = p->dims[d];
    if (real && d == 0) len = d0 / 2 > 0 ? d0 / 2 : 1;
    port1d_init(&p->dimplan[d], len);
  }
  if (real && d0 >= 2) {
    int64_t L = d0 / 2;
    p->rtw_re = (float*)malloc(sizeof(float) * (size_t)L);
    p->rtw_im = (float*)malloc(sizeof(float) * (size_t)L);
    twiddle_full(L, p->rtw_re, p->rtw_im);
  }
  p->scratch = 2 * (H > p->N ? H : p->N) + 16;
  return p;
}

void port32_plan_destroy(port32_plan* p)
{
  if (!p) return;
  for (int d = 0; d < p->ndim; d++) port1d_free(&p->dimplan[d]);
  free(p->rtw_re);
  free(p->rtw_im);
  free(p);
}

int64_t port32_plan_in_elems(const port32_plan* p) { return p->in_elems; }
int64_t port32_plan_out_elems(const port32_plan* p) { return p->out_elems; }

/* fft_internal.hpp:121-164: every dimension from first_dim to the last, each
 * as a row transform over blocks of (dims[d] rows x prod(later dims)), on
 * `lead` consecutive arrays of shape dims[first_dim:] (split, dense), in
 * place.  The reference walks rows in
 * bit-reversed order between dims; the port transforms to natural order at
 * each dim, which is the same DFT. */
static void port_nd_inplace(const port32_plan* p, int first_dim, int64_t lead,
                            int inverse, float* re, float* im, float* wre,
                            float* wim)
{
  int nd = p->ndim;
  for (int d = first_dim; d < nd; d++) {
    int64_t n = p->dims[d];
    if (n == 1) continue;
    int64_t m = prod(p->dims + d + 1, nd - d - 1);
    int64_t outer = lead * prod(p->dims + first_dim, d - first_dim);
    for (int64_t o = 0; o < outer; o++) {
      rows_t b = {re + o * n * m, im + o * n * m, m};
      rows_t w = {wre, wim, m};
      port_rows(&p->dimplan[d], m, inverse, b, w, b);
    }
  }
}

static int port_exec_scratch(const port32_plan* p, const float* in_re,
                             const float* in_im, float* out_re, float* out_im,
                             float* scratch)
{
  int64_t N = p->N;
  int nd = p->ndim;
  int64_t d0 = p->dims[0];
  int64_t inner = N / d0;
  if (p->kind == ORACLE_C || p->kind == ORACLE_CI) {
    int inv = p->kind == ORACLE_CI;
    float* wre = scratch;
    float* wim = scratch + N;
    if (nd == 1) {
      rows_t s = {(float*)in_re, (float*)in_im, 1};
      rows_t w = {wre, wim, 1};
      rows_t d = {out_re, out_im, 1};
      port_rows(&p->dimplan[0], 1, inv, s, w, d);
      return 0;
    }
    /* first dim reads src, the rest run in place on dst */
    rows_t s = {(float*)in_re, (float*)in_im, inner};
    rows_t w = {wre, wim, inner};
    rows_t d = {out_re, out_im, inner};
    port_rows(&p->dimplan[0], inner, inv, s, w, d);
    port_nd_inplace(p, 1, d0, inv, out_re, out_im, wre, wim);
    return 0;
  }

  if (nd == 1) {
    int64_t n = d0;
    if (n == 1) {   /* length-1 real transform: DC only */
      if (p->kind == ORACLE_R) { out_re[0] = in_re[0]; out_im[0] = 0.0f; }
      else out_re[0] = in_re[0];
      return 0;
    }
    int64_t L = n / 2;
    float* zre = scratch;
    float* zim = scratch + L + 1;
    float* wre = scratch + 2 * (L + 1);
    float* wim = wre + L;
    if (p->kind == ORACLE_R) {
      /* onedim.hpp:1175-1189: n/2-point transform of the interleaved view */
      rows_t s = {(float*)in_re, (float*)in_re + 1, 2};
      rows_t w = {wre, wim, 1};
      rows_t z = {zre, zim, 1};
      port_rows(&p->dimplan[0], 1, 0, s, w, z);
      real_pass_1d(n, 0, zre, zim, p->rtw_re, p->rtw_im, out_re, out_im);
    } else {
      /* onedim.hpp:1242-1254: real pass, then n/2-point inverse into the
       * interleaved view of dst */
      real_pass_1d(n, 1, in_re, in_im, p->rtw_re, p->rtw_im, zre, zim);
      rows_t z = {zre, zim, 1};
      rows_t w = {wre, wim, 1};
      rows_t d = {out_re, out_re + 1, 2};
      port_rows(&p->dimplan[0], 1, 1, z, w, d);
    }
    return 0;
  }

  /* N-D real, first dim halved: fft_internal.hpp:320-346 / 467-493 */
  int64_t L = d0 / 2;
  float* w0re = scratch;                 /* (L+1) rows of inner */
  float* w0im = scratch + (L + 1) * inner;
  float* wre = scratch + 2 * (L + 1) * inner;
  float* wim = wre + N / 2 + inner;
  rows_t w0 = {w0re, w0im, inner};
  if (p->kind == ORACLE_R) {
    rows_t s = {(float*)in_re, (float*)in_re + inner, 2 * inner};
    rows_t w = {wre, wim, inner};
    port_rows(&p->dimplan[0], inner, 0, s, w, w0);
    real_pass_rows(d0, inner, 0, p->rtw_re, p->rtw_im, w0);
    memcpy(out_re, w0re, sizeof(float) * (size_t)((L + 1) * inner));
    memcpy(out_im, w0im, sizeof(float) * (size_t)((L + 1) * inner));
    for (int64_t pl = 0; pl <= L; pl++)
      port_nd_inplace(p, 1, 1, 0, out_re + pl * inner, out_im + pl * inner, wre, wim);
  } else {
    memcpy(w0re, in_re, sizeof(float) * (size_t)((L + 1) * inner));
    memcpy(w0im, in_im, sizeof(float) * (size_t)((L + 1) * inner));
    for (int64_t pl = 0; pl <= L; pl++)
      port_nd_inplace(p, 1, 1, 1, w0re + pl * inner, w0im + pl * inner, wre, wim);
    real_pass_rows(d0, inner, 1, p->rtw_re, p->rtw_im, w0);
    rows_t d = {out_re, out_re + inner, 2 * inner};
    rows_t w = {wre, wim, inner};
    port_rows(&p->dimplan[0], inner, 1, w0, w, d);
  }
  return 0;
}

static int64_t scratch_floats(const port32_plan* p)
{
  return 4 * (p->N + 2 * p->out_elems + 2 * p->in_elems) + 64;
}

int port32_execute(const port32_plan* p, const float* in_re, const float* in_im,
                   float* out_re, float* out_im)
{
  if (!p) return -1;
  float* scratch = (float*)malloc(sizeof(float) * (size_t)scratch_floats(p));
  if (!scratch) return -1;
  int r = port_exec_scratch(p, in_re, in_im, out_re, out_im, scratch);
  free(scratch);
  return r;
}

typedef struct {
  const port32_plan* p;
  int64_t b0, b1;
  const float* in_re;
  const float* in_im;
  float* out_re;
  float* out_im;
  int rc;
} batch_job;

static void* batch_worker(void* arg)
{
  batch_job* j = (batch_job*)arg;
  const port32_plan* p = j->p;
  float* scratch = (float*)malloc(sizeof(float) * (size_t)scratch_floats(p));
  if (!scratch) { j->rc = -1; return NULL; }
  int64_t ie = p->in_elems, oe = p->out_elems;
  for (int64_t b = j->b0; b < j->b1; b++) {
    const float* ir = j->in_re + b * ie;
    const float* ii = j->in_im ? j->in_im + b * ie : NULL;
    float* orr = j->out_re + b * oe;
    float* oi = j->out_im ? j->out_im + b * oe : NULL;
    port_exec_scratch(p, ir, ii, orr, oi, scratch);
  }
  free(scratch);
  j->rc = 0;
  return NULL;
}

int port32_execute_batch(const port32_plan* p, int64_t batch, int threads,
                         const float* in_re, const float* in_im,
                         float* out_re, float* out_im)
{
  if (!p || batch < 0) return -1;
  if (threads < 1) threads = 1;
  if (threads > batch) threads = (int)(batch > 0 ? batch : 1);
  pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
  batch_job* jobs = (batch_job*)calloc((size_t)threads, sizeof(batch_job));
  for (int t = 0; t < threads; t++) {
    jobs[t].p = p;
    jobs[t].b0 = batch * t / threads;
    jobs[t].b1 = batch * (t + 1) / threads;
    jobs[t].in_re = in_re; jobs[t].in_im = in_im;
    jobs[t].out_re = out_re; jobs[t].out_im = out_im;
    jobs[t].rc = -1;
    pthread_create(&tid[t], NULL, batch_worker, &jobs[t]);
  }
  int rc = 0;
  for (int t = 0; t < threads; t++) {
    pthread_join(tid[t], NULL);
    if (jobs[t].rc) rc = -1;
  }
  free(tid);
  free(jobs);
  return rc;
}
