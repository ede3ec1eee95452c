/*
 * TEST INFRASTRUCTURE ONLY -- shape helpers shared by the oracle and the
 * FP32 / FP64 ports of afft (afft_oracle.c, afft_port.inc).
 */
#ifndef AFFT_SHAPE_H
#define AFFT_SHAPE_H
#include <stdint.h>

static inline int is_pow2(int64_t v) { return v > 0 && (v & (v - 1)) == 0; }

static inline int ilog2(int64_t v)
{
  int r = 0;
  while (v > 1) { v >>= 1; r++; }
  return r;
}

static inline int64_t rev_bits(int64_t v, int nbits)
{
  int64_t r = 0;
  for (int i = 0; i < nbits; i++) { r = (r << 1) | (v & 1); v >>= 1; }
  return r;
}

static inline int valid_shape(int ndim, const int64_t* dims)
{
  if (ndim < 1 || ndim > 64) return 0;
  for (int i = 0; i < ndim; i++)
    if (!is_pow2(dims[i])) return 0;
  return 1;
}

static inline int64_t prod(const int64_t* d, int n)
{
  int64_t r = 1;
  for (int i = 0; i < n; i++) r *= d[i];
  return r;
}

#endif
