// Line-FFT kernels for sm_103a: batched power-of-two FFTs along one axis.
//
// A "line" is one 1D transform of length L = 2^LOGL along an axis of an array
// in HBM.  Line q's element i sits at  off(q) + i*es  with
//     off(q) = (q >> qshift) * hi + (q & qmask) * lo
// which covers contiguous batches (rows), strided axes of N-D arrays
// (columns), the interleaved view of real data and the transposed layouts of
// the four-step decomposition with one formula.
//
// One CTA transforms C lines.  Each thread owns E (= 16, or L when L < 16)
// complex values of one line in registers, in the canonical Stockham layout
// v[e] = x[t + T*e] (T = L/E threads per line), so the first stage loads
// straight from HBM and the last stage stores straight to HBM, coalesced:
//   rows mode (COLS = false): lines are contiguous; consecutive threads walk
//                             along a line;
//   cols mode (COLS = true):  consecutive lines are adjacent in memory;
//                             consecutive threads walk across lines.
// Stages are radix-16 (one radix-2/4/8 stage first when log2 L is not a
// multiple of 4); between stages values go through shared memory with an XOR
// swizzle chosen so the Stockham scatter and the canonical gather are (almost)
// bank-conflict free.  Stage twiddles come from a per-length table computed
// in FP64 on the host and rounded once.
//
// The template parameter UNIT picks compile-time access forms: in rows mode
// unit-stride split lines (1) or re,im pairs with unit pair stride (2); in
// cols mode re,im pairs on the input (bit 0) and/or the output (bit 1).  Pair
// forms move one 8-byte value per element; they check 8-byte alignment at run
// time and fall back to 4-byte accesses (callers may pass any 4-byte-aligned
// array).
//
// Cols passes of 256 to 1024 points (and the 2048-point C2R pass) also come
// in a TMA-fed form (line_fft_tma): one thread loads the CTA's input tile
// into the exchange buffer with tensor-map copies on an mbarrier, and the
// threads read their canonical elements from shared memory.
//
// This restates the work of afft's onedim.hpp (radix-4/8/16 passes,
// onedim.hpp:55-507) and multi.hpp (passes along strided dims,
// multi.hpp:18-259) as one self-sorting (Stockham) formulation, so no
// bit-reversal pass (onedim.hpp:397-447) is needed; the real pre/post passes
// (onedim.hpp:1031-1108, multi.hpp:343-414) are fused into the first/last
// stage; inverse transforms swap re and im on load and store, the identity
// afft uses for its inverse plans (common.hpp:355-378).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "tc_dft.cuh"

namespace agb {

// LK_R2C_HALF: the cols R2C pass split over two CTAs per tile (below).
// LK_R2C_PAIRED: pass B of a long 1D real forward with the real post-pass,
// over tiles of mirrored column pairs (below).
// LK_C2R_PAIRED: pass A of a long 1D real inverse with the real pre-pass,
// over the same tiles (below).
enum LineKind { LK_C2C = 0, LK_R2C = 1, LK_C2R = 2, LK_R2C_HALF = 3, LK_R2C_PAIRED = 4, LK_C2R_PAIRED = 5 };

struct LineIO {
  float* re;
  float* im;
  long long es;       // element stride (floats)
  long long lo, hi;   // off(q) = (q >> qshift) * hi + (q & qmask) * lo
  int qshift;
  long long qmask;
};

struct LineParams {
  LineIO in, out;
  long long nlines;         // lines to transform
  const float2* tw;         // stage twiddles for this L
  // four-step twiddle W_N^{t2 k}, t2 = (q >> tw_qshift) & tw_qmask, N = tw_n
  // (0 = none): tw_full[t2 * L + k] (L: the line length) when tw_full is
  // set, else
  // W_N^m = tw_hi[m >> tw_lo_bits] * tw_lo[m & ((1 << tw_lo_bits) - 1)]
  const float2* tw_full;
  const float2* tw_hi;
  const float2* tw_lo;
  long long tw_n;
  long long tw_qmask;
  int tw_qshift;
  int tw_lo_bits;
  const float2* rtw;        // real pass twiddles W_{2L}^k, k < L
  long long pcols;          // paired passes: lines per transform (L1 for pass B, L2 for pass A)
  int inverse;              // swap re/im on load and store
  const __half* tc_b;       // TC form: Mh then Ml, 32x32 FP16 each, [n][k]
  int* err;                 // TC form: error word set when a bounded wait gives up
  const float2* tw2;        // plane passes: stage twiddles of the column axis
};

// ---------------------------------------------------------------------------
// compile-time radix schedule
// ---------------------------------------------------------------------------
template <int LOGL>
struct Sched {
  static constexpr int L = 1 << LOGL;
  static constexpr int E = LOGL < 4 ? L : 16;
  static constexpr int T = L / E;
  static constexpr int FIRST = (LOGL >= 4 && (LOGL % 4)) ? (1 << (LOGL % 4)) : 0;
  static constexpr int NSTAGES = LOGL < 4 ? 1 : (LOGL / 4 + (FIRST ? 1 : 0));
  static constexpr int radix(int s) { return LOGL < 4 ? L : (FIRST && s == 0 ? FIRST : 16); }
  static constexpr int ns(int s) {
    int r = 1;
    for (int i = 0; i < s; i++) r *= radix(i);
    return r;
  }
  static constexpr int twoff(int s) {
    int o = 0;
    for (int i = 0; i < s; i++)
      if (ns(i) > 1) o += (radix(i) - 1) * ns(i);
    return o;
  }
  static constexpr int twsize() { return twoff(NSTAGES); }
};

// ---------------------------------------------------------------------------
// complex helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// The butterflies' add / subtract: with PK one packed FP32x2 instruction each
// (sm_100+; per component the same IEEE round-to-nearest result as the scalar
// form).  Elsewhere adds stay scalar, so multiplies feeding them still
// contract into FMAs.
template <bool PK>
__device__ __forceinline__ float2 badd(float2 a, float2 b) {
  if constexpr (PK) return __fadd2_rn(a, b);
  else return cadd(a, b);
}
template <bool PK>
__device__ __forceinline__ float2 bsub(float2 a, float2 b) {
  if constexpr (PK) return __fadd2_rn(a, make_float2(-b.x, -b.y));
  else return csub(a, b);
}
// Which line kernels take the packed butterflies, measured per length on
// GB300: rows of 256 to 8192 points 1.3-2.5% faster, 256-, 1024- and
// 2048-point cols passes 1-5% faster; the warp-staged rows of up to 128
// points (6-9%), the 512-point cols passes (2-3%) and the transposing-store
// passes of 1024 points and more (the long 1D real forward's pass A, 2.4%)
// slower.
template <int LOGL, bool COLS, bool TSTORE = false>
constexpr bool packed_bfly() {
  return COLS ? (LOGL != 9 && !(TSTORE && LOGL >= 10)) : LOGL >= 8;
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cmul_negi(float2 a) { return make_float2(a.y, -a.x); }   // -i*a
__device__ __forceinline__ float2 cswap(float2 a) { return make_float2(a.y, a.x); }

// constants: cos/sin(pi/8), sqrt(1/2)
#define AFFT_C8 0.92387953251128674f
#define AFFT_S8 0.38268343236508979f
#define AFFT_R2 0.70710678118654752f

// W16^k * a for k = 1..9 (forward, exp(-2 pi i k/16))
template <int K>
__device__ __forceinline__ float2 w16(float2 a) {
  if constexpr (K == 0) return a;
  else if constexpr (K == 1) return cmul(a, make_float2(AFFT_C8, -AFFT_S8));
  else if constexpr (K == 2) return make_float2(AFFT_R2 * (a.x + a.y), AFFT_R2 * (a.y - a.x));
  else if constexpr (K == 3) return cmul(a, make_float2(AFFT_S8, -AFFT_C8));
  else if constexpr (K == 4) return cmul_negi(a);
  else if constexpr (K == 6) return make_float2(AFFT_R2 * (a.y - a.x), -AFFT_R2 * (a.x + a.y));
  else if constexpr (K == 9) return cmul(a, make_float2(-AFFT_C8, AFFT_S8));
  else return a;  // unused
}

template <bool PK>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  float2 t = a;
  a = badd<PK>(t, b);
  b = bsub<PK>(t, b);
}

// in-place DFT-4 on (a0, a1, a2, a3), natural order out
template <bool PK>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  float2 s02 = badd<PK>(a0, a2), d02 = bsub<PK>(a0, a2);
  float2 s13 = badd<PK>(a1, a3), d13 = bsub<PK>(a1, a3);
  a0 = badd<PK>(s02, s13);
  a2 = bsub<PK>(s02, s13);
  a1 = badd<PK>(d02, cmul_negi(d13));
  a3 = bsub<PK>(d02, cmul_negi(d13));
}

template <int R, bool PK = false>
__device__ __forceinline__ void dft(float2 (&x)[R]) {
  if constexpr (R == 1) {
  } else if constexpr (R == 2) {
    dft2<PK>(x[0], x[1]);
  } else if constexpr (R == 4) {
    dft4<PK>(x[0], x[1], x[2], x[3]);
  } else if constexpr (R == 8) {
    // 2 x 4: E = DFT4(even), O = DFT4(odd) * W8^k
    dft4<PK>(x[0], x[2], x[4], x[6]);
    dft4<PK>(x[1], x[3], x[5], x[7]);
    x[3] = w16<2>(x[3]);
    x[5] = w16<4>(x[5]);
    x[7] = w16<6>(x[7]);
    float2 y[8];
    y[0] = badd<PK>(x[0], x[1]); y[4] = bsub<PK>(x[0], x[1]);
    y[1] = badd<PK>(x[2], x[3]); y[5] = bsub<PK>(x[2], x[3]);
    y[2] = badd<PK>(x[4], x[5]); y[6] = bsub<PK>(x[4], x[5]);
    y[3] = badd<PK>(x[6], x[7]); y[7] = bsub<PK>(x[6], x[7]);
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = y[i];
  } else if constexpr (R == 16) {
    // n = n1 + 4 n2, k = k2 + 4 k1
#pragma unroll
    for (int n1 = 0; n1 < 4; n1++) dft4<PK>(x[n1], x[n1 + 4], x[n1 + 8], x[n1 + 12]);
    // now x[n1 + 4 k2] = Y[n1][k2]; twiddle W16^{n1 k2}
    x[5] = w16<1>(x[5]);  x[9] = w16<2>(x[9]);   x[13] = w16<3>(x[13]);
    x[6] = w16<2>(x[6]);  x[10] = w16<4>(x[10]); x[14] = w16<6>(x[14]);
    x[7] = w16<3>(x[7]);  x[11] = w16<6>(x[11]); x[15] = w16<9>(x[15]);
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) dft4<PK>(x[4 * k2], x[4 * k2 + 1], x[4 * k2 + 2], x[4 * k2 + 3]);
    // now x[4 k2 + k1] = X[k2 + 4 k1]: transpose the 4x4 index
    float2 y[16];
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++)
#pragma unroll
      for (int k1 = 0; k1 < 4; k1++) y[k2 + 4 * k1] = x[4 * k2 + k1];
#pragma unroll
    for (int i = 0; i < 16; i++) x[i] = y[i];
  }
}

// ---------------------------------------------------------------------------
// shared-memory layout: complex values as float2, arranged so the Stockham
// scatter and the canonical gather hit distinct bank pairs per half-warp and
// every per-element offset is a compile-time constant:
//   rows mode: line c at c * LP, element j at j + j/16   (LP = L + L/16);
//              short lines, where a warp spans 8 to 16 lines, instead:
//              L = 128: j + j/8 (LP 152), L = 64: j + j/4 (LP 84),
//              L = 32: j ^ (3 (c >> 2) mod 32) (LP 36), each found by an
//              exhaustive bank count (the j/16 form costs 1.5 to 2.5 times
//              the minimum wavefronts at these lengths)
//   cols mode: element j of line c at j * CP + c          (CP = C + 1)
//   cols mode, SWAP = k >= 0 (8 lines): element j of line c at
//              (j ^ bit_k(j >> 1)) * 8 + c, unpadded (XOR: c ^ ((j >> 1) & 7)).
//              A half-warp of the cols mapping touches two rows; the padded
//              layout puts both in the same bank half for the strided
//              scatter of the stages (2-way conflicts).  Swapping the rows
//              of a pair keyed on bit k = log2(first radix / 2) of the pair
//              index separates them for the scatter and the gather.  With
//              XOR, 16 consecutive elements of one line (the transposing
//              store's reads) also spread over all banks.  Both checked by an
//              exhaustive bank count over all stages and warps.
// ---------------------------------------------------------------------------
template <int L, int C, bool COLS, int SWAP = -1, bool XOR = false>
struct Smem {
  static_assert(SWAP < 0 || (COLS && C == 8), "row-pair swap layout: cols mode, 8 lines");
  static constexpr int LP = L == 32 ? 36 : (L == 64 ? 84 : (L == 128 ? 152 : L + L / 16));
  static constexpr int CP = SWAP >= 0 ? C : C + 1;
  static constexpr int FLOAT2S = COLS ? L * CP : C * LP;
  float2* s;
  __device__ __forceinline__ int idx(int c, int j) const {
    if constexpr (COLS && SWAP >= 0 && XOR) return (j ^ ((j >> (SWAP + 1)) & 1)) * C + (c ^ ((j >> 1) & 7));
    else if constexpr (COLS && SWAP >= 0) return (j ^ ((j >> (SWAP + 1)) & 1)) * C + c;
    else if constexpr (COLS) return j * CP + c;
    else if constexpr (L == 32) return c * LP + (j ^ (((c >> 2) * 3) & 31));
    else if constexpr (L == 64) return c * LP + j + (j >> 2);
    else if constexpr (L == 128) return c * LP + j + (j >> 3);
    else return c * LP + j + (j >> 4);
  }
  __device__ __forceinline__ void put(int c, int j, float2 v) const { s[idx(c, j)] = v; }
  __device__ __forceinline__ float2 get(int c, int j) const { return s[idx(c, j)]; }
};

// The layout a line kernel uses: the row-pair swap for 8-line cols tiles
// (not the TC operand tiles, which have their own layout), with the XOR when
// the transposing store reads the buffer along lines.
template <int LOGL>
constexpr int swap_bit() {
  return LOGL % 4 == 0 ? 3 : LOGL % 4 - 1;
}
template <int LOGL, int C, bool COLS, bool TSTORE, bool TC>
using LineSmem = Smem<(1 << LOGL), C, COLS, (COLS && C == 8 && !TC && LOGL >= 8) ? swap_bit<LOGL>() : -1, TSTORE>;

template <bool WARP_ONLY>
__device__ __forceinline__ void line_sync() {
  if constexpr (WARP_ONLY) __syncwarp();
  else __syncthreads();
}

__device__ __forceinline__ long long line_off(const LineIO& io, long long q) {
  return (q >> io.qshift) * io.hi + (q & io.qmask) * io.lo;
}

__device__ __forceinline__ float2 ldg2(const float2* p) { return __ldg(p); }

// One Stockham stage: B = E/R butterflies per thread, butterfly b = t + T*u
// reads slots u + B*r, applies W_{NS*R}^{r*(b mod NS)}, DFT-R, and either
// scatters to shared memory (non-last) or keeps the canonical layout (last).
template <int R, int NS, int E, int T, bool LAST, bool TC, int NT, bool PK, class SM>
__device__ __forceinline__ void stage(float2 (&v)[E], int t, int c, const float2* tw, const SM& sm,
                                      bool do_write, TcState* ts) {
  constexpr int B = E / R;
#pragma unroll
  for (int u = 0; u < B; u++) {
    const int b = t + T * u;
    float2 x[R];
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = v[u + B * r];
    if constexpr (NS > 1) {
      const int k = b & (NS - 1);
#pragma unroll
      for (int r = 1; r < R; r++) x[r] = cmul(x[r], ldg2(tw + (r - 1) * NS + k));
    }
    if constexpr (TC && R == 16) {
      static_assert(E == 16, "TC form: one butterfly per thread");
      tc_dft16<NT>(x, threadIdx.x, *ts);
    } else {
      dft<R, PK>(x);
    }
    if constexpr (LAST) {
#pragma unroll
      for (int r = 0; r < R; r++) v[u + B * r] = x[r];
    } else {
      if (do_write) {
        const int base = (b / NS) * NS * R + (b & (NS - 1));
#pragma unroll
        for (int r = 0; r < R; r++) sm.put(c, base + r * NS, x[r]);
      }
    }
  }
}

// All stages; v holds the input in canonical layout on entry and the output
// in canonical layout on exit.
template <int LOGL, int C, bool COLS, bool WARP_ONLY, int S, bool TC = false, bool PK = packed_bfly<LOGL, COLS>(),
          class SM>
__device__ __forceinline__ void run_stages(float2 (&v)[Sched<LOGL>::E], int t, int c, const float2* tw,
                                           const SM& sm, TcState* ts = nullptr) {
  using Sc = Sched<LOGL>;
  constexpr int E = Sc::E, T = Sc::T;
  constexpr int NT = (Sc::T * C) / 128;
  if constexpr (S < Sc::NSTAGES) {
    constexpr int R = Sc::radix(S);
    constexpr int NS = Sc::ns(S);
    constexpr bool LAST = S == Sc::NSTAGES - 1;
    if constexpr (S > 0) {
      // values of the previous stage are in shared memory
#pragma unroll
      for (int e = 0; e < E; e++) v[e] = sm.get(c, t + T * e);
    }
    // everyone finished reading before the buffer is written again (the TC
    // form writes its operand tiles there even in the last stage)
    if constexpr (S > 0 && (!LAST || TC)) line_sync<WARP_ONLY && !TC>();
    if constexpr (!LAST) {
      stage<R, NS, E, T, false, TC, NT, PK>(v, t, c, tw + Sc::twoff(S), sm, true, ts);
      line_sync<WARP_ONLY && !TC>();                   // writes visible
      run_stages<LOGL, C, COLS, WARP_ONLY, S + 1, TC, PK>(v, t, c, tw, sm, ts);
    } else {
      stage<R, NS, E, T, true, TC, NT, PK>(v, t, c, tw + Sc::twoff(S), sm, false, ts);
    }
  }
}

// t2 < 2^11 and k < 2^11, so t2 * k fits 32 bits; L is the line length.
// FULL: read the matrix table tw_full, else the hi/lo pair.
template <int L, bool FULL>
__device__ __forceinline__ float2 fourstep_twiddle(const LineParams& p, long long q, int k) {
  const int t2 = (int)((q >> p.tw_qshift) & p.tw_qmask);
  if constexpr (FULL) {
    return ldg2(p.tw_full + t2 * L + k);
  } else {
    const int m = (t2 * k) & ((int)p.tw_n - 1);
    float2 a = ldg2(p.tw_hi + (m >> p.tw_lo_bits));
    float2 b = ldg2(p.tw_lo + (m & ((1 << p.tw_lo_bits) - 1)));
    return cmul(a, b);
  }
}

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
// Register budget per thread: with 64 the allocator keeps 4 CTAs of 256
// threads resident per SM, which measured faster at every length than the
// unconstrained (~80 register) build.
#ifndef AFFT_REG_CAP
#define AFFT_REG_CAP 64
#endif
template <int NT>
constexpr int min_ctas() {
  return AFFT_REG_CAP ? (65536 / (AFFT_REG_CAP * NT) > 0 ? 65536 / (AFFT_REG_CAP * NT) : 1) : 1;
}

// The real forward (R2C) pass along a strided axis of Z = 2 Lh complex
// points (Lh = 2^LOGL), split over two CTAs per tile of C lines.  With the
// first radix-2 step of a decimation in frequency,
//   a[j] = z[j] + z[j + Lh],  b[j] = (z[j] - z[j + Lh]) W_{2Lh}^j,
// FFT_Lh(a) gives the even bins Z[2m] and FFT_Lh(b) the odd bins Z[2m+1].
// CTA half h = cta & 1 computes one of them, so it needs the exchange buffer
// of Lh points per line, not 2 Lh: twice the CTAs fit on an SM.  The real
// post-pass pairs bin k with 2 Lh - k, which has the same parity, so both
// halves finish on their own: h = 0 pairs m with Lh - m (mod Lh), h = 1 pairs
// m with Lh - 1 - m.  Both CTAs of a tile read the whole tile (the second
// read is served by L2).  rtw = W_{4Lh}^k, k < 2 Lh, as for the unsplit pass;
// W_{2Lh}^j = rtw[2j].  The stage twiddles are those of Lh.
template <int LOGL, int C>
__device__ __forceinline__ void r2c_half_body(const LineParams& p, long long cta) {
  using Sc = Sched<LOGL>;
  constexpr int Lh = Sc::L, E = Sc::E, T = Sc::T, L = 2 * Lh;
  constexpr bool WARP_ONLY = T * C <= 32;
  extern __shared__ __align__(1024) float2 smem_raw[];
  LineSmem<LOGL, C, true, false, false> sm{smem_raw};
  const int tid = threadIdx.x;
  const int c = tid % C, t = tid / C;
  const int h = (int)(cta & 1);
  const long long q = (cta >> 1) * C + c;
  const bool active = q < p.nlines;

  float2 v[E];
  if (active) {
    const long long base = line_off(p.in, q);
    const long long half = (long long)Lh * p.in.es;
    const long long S = (long long)T * p.in.es;
    const float* pr = p.in.re + base + (long long)t * p.in.es;
    const float* pi = p.in.im + base + (long long)t * p.in.es;
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int j = t + T * e;
      const float2 x0 = make_float2(__ldg(pr + e * S), __ldg(pi + e * S));
      const float2 x1 = make_float2(__ldg(pr + e * S + half), __ldg(pi + e * S + half));
      v[e] = h ? cmul(csub(x0, x1), ldg2(p.rtw + 2 * j)) : cadd(x0, x1);
    }
  } else {
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = make_float2(0.f, 0.f);
  }

  run_stages<LOGL, C, true, WARP_ONLY, 0>(v, t, c, p.tw, sm);

  // real forward post-pass on this half's bins (the formula of the unsplit
  // pass below: X[k] = a - i b, X[0] and X[L] from Z[0])
  if constexpr (Sc::NSTAGES > 1) line_sync<WARP_ONLY>();
#pragma unroll
  for (int e = 0; e < E; e++) sm.put(c, t + T * e, v[e]);
  line_sync<WARP_ONLY>();
  if (active) {
    const long long base = line_off(p.out, q);
    const long long S2 = 2LL * T * p.out.es;
    float* pr = p.out.re + base + (long long)(2 * t + h) * p.out.es;
    float* pi = p.out.im + base + (long long)(2 * t + h) * p.out.es;
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int m = t + T * e;
      const int k = 2 * m + h;
      const float2 s0 = v[e];
      const float2 s1 = sm.get(c, h ? (Lh - 1 - m) : ((Lh - m) & (Lh - 1)));
      float2 x;
      if (k == 0) {
        x = make_float2(s0.x + s0.y, 0.f);
        const long long aL = base + (long long)L * p.out.es;
        p.out.re[aL] = s0.x - s0.y;
        p.out.im[aL] = 0.f;
      } else {
        const float2 w = ldg2(p.rtw + k);
        const float2 a = make_float2(0.5f * (s0.x + s1.x), 0.5f * (s0.y - s1.y));
        const float2 d = make_float2(0.5f * (s0.x - s1.x), 0.5f * (s0.y + s1.y));
        x = cadd(a, cmul_negi(cmul(d, w)));
      }
      pr[e * S2] = x.x;
      pi[e * S2] = x.y;
    }
  }
}

// Column of slot c in a mirrored-pair tile (r2c_paired_body, c2r_paired_body): slots
// 0 .. C/2-1 hold columns a + c, slots C/2 + m hold L1 - a - m, and in tile
// 0 (a = 0) the slot C/2 holds L1/2.
template <int C>
__device__ __forceinline__ long long paired_column(int c, long long a, long long ncols) {
  constexpr int H = C / 2;
  if (c < H) return a + c;
  const int m = c - H;
  return (a == 0 && m == 0) ? ncols / 2 : ncols - a - m;
}

// Pass B of the four-step transform of a long 1D real forward (n/2 = L =
// L1 L2 complex points of the interleaved view) with the real post-pass
// (onedim.hpp:1058-1108) fused in.  Pass B line (o, k1) holds Z[k1 + L1 k2]
// for k2 < L2; the post-pass pairs Z[k] with Z[L - k], and for k1 > 0 that
// is element L2 - 1 - k2 of column L1 - k1 (column 0 pairs with itself,
// element (L2 - k2) mod L2).  So a CTA takes C/2 columns a .. a + C/2 - 1
// (slots 0 .. C/2-1, a = tile C/2) and their mirrors L1 - a - m (slots
// C/2 + m); in tile 0 the slot of the mirror "L1" holds column L1/2, which
// pairs with itself.  After the FFTs every element yields its own bin X[k]
// (k = k1 + L1 k2, written where the unfused pass B would write Z[k]), and
// the column-0 thread of k2 = 0 also writes X[L] (element L2 of line
// (o, 0)).  Lines come in whole tiles: L1 is a multiple of C.
// TMA: the tile is already in shared memory as line_fft_paired_tma lays it
// out: the aligned half [L2 rows][2H floats] (columns a .. a+H-1), the
// mirrored half from the 16-byte boundary below it [L2 rows][2H + 4 floats]
// (columns L1-a-H .. L1-a+1), and in tile 0 column L1/2 [L2 rows][4 floats].
template <int LOGL, int C, bool PIN = false, bool TMA = false>
__device__ __forceinline__ void r2c_paired_body(const LineParams& p, long long cta) {
  using Sc = Sched<LOGL>;
  constexpr int L2 = Sc::L, E = Sc::E, T = Sc::T, H = C / 2;
  static_assert(C % 2 == 0 && T * C > 32, "paired tiles: even C, CTA-wide exchange");
  extern __shared__ __align__(1024) float2 smem_raw[];
  LineSmem<LOGL, C, true, false, false> sm{smem_raw};
  const int tid = threadIdx.x;
  const int c = tid % C, t = tid / C;
  const long long L1 = p.pcols, tiles = L1 / C;
  const long long o = cta / tiles, a = (cta % tiles) * H;
  // this slot's column and its partner slot
  const long long k1 = paired_column<C>(c, a, L1);
  const int cp = c < H ? ((a == 0 && c == 0) ? 0 : c + H) : ((a == 0 && c == H) ? c : c - H);
  const long long q = o * L1 + k1;

  float2 v[E];
  if constexpr (TMA) {
    static_assert(PIN, "TMA tiles: the paired pass over input pairs");
    const float* raw = reinterpret_cast<const float*>(smem_raw);
    const float* mi = raw + L2 * 2 * H;
    const float* src = c < H ? raw + 2 * c
                       : (a == 0 && c == H) ? mi + L2 * (2 * H + 4)
                                            : mi + 2 * (H - (c - H));   // column L1 - a - m at H - m
    const int pitch = c < H ? 2 * H : (a == 0 && c == H) ? 4 : 2 * H + 4;
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = *reinterpret_cast<const float2*>(src + (t + T * e) * pitch);
    __syncthreads();   // the tile is read before the stages reuse the buffer
  } else {
    const long long base = line_off(p.in, q);
    const long long S = (long long)T * p.in.es;
    const float* pr = p.in.re + base + (long long)t * p.in.es;
    const float* pi = p.in.im + base + (long long)t * p.in.es;
    bool loaded = false;
    if constexpr (PIN) {
      // input pairs (im = re + 1, even element stride): 8-byte loads
      if (!(reinterpret_cast<uintptr_t>(pr) & 7)) {
        const float2* pz = reinterpret_cast<const float2*>(pr);
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = __ldg(pz + e * (S >> 1));
        loaded = true;
      }
    }
    if (!loaded) {
#pragma unroll
      for (int e = 0; e < E; e++) v[e] = make_float2(__ldg(pr + e * S), __ldg(pi + e * S));
    }
  }
  run_stages<LOGL, C, true, false, 0>(v, t, c, p.tw, sm);

  if constexpr (Sc::NSTAGES > 1) __syncthreads();
#pragma unroll
  for (int e = 0; e < E; e++) sm.put(c, t + T * e, v[e]);
  __syncthreads();
  const long long base = line_off(p.out, q);
  const long long SO = (long long)T * p.out.es;
  float* por = p.out.re + base + (long long)t * p.out.es;
  float* poi = p.out.im + base + (long long)t * p.out.es;
#pragma unroll
  for (int e = 0; e < E; e++) {
    const int k2 = t + T * e;
    const long long k = k1 + L1 * k2;
    const float2 s0 = v[e];
    const float2 s1 = sm.get(cp, k1 == 0 ? ((L2 - k2) & (L2 - 1)) : (L2 - 1 - k2));
    float2 x;
    if (k == 0) {
      x = make_float2(s0.x + s0.y, 0.f);
      const long long aL = base + (long long)L2 * p.out.es;
      p.out.re[aL] = s0.x - s0.y;
      p.out.im[aL] = 0.f;
    } else {
      const float2 w = ldg2(p.rtw + k);
      const float2 ha = make_float2(0.5f * (s0.x + s1.x), 0.5f * (s0.y - s1.y));
      const float2 d = make_float2(0.5f * (s0.x - s1.x), 0.5f * (s0.y + s1.y));
      x = cadd(ha, cmul_negi(cmul(d, w)));
    }
    por[e * SO] = x.x;
    poi[e * SO] = x.y;
  }
}

// Pass A of the inverse four-step of a long 1D real inverse (n/2 = L = L1 L2)
// with the real pre-pass (onedim.hpp:1064-1068) fused into its loads.  Line
// (o, t2) of pass A reads Z'[t2 + L2 t1], t1 < L1, and Z'[k] needs X[k] and
// X[L - k]; for t2 > 0 the latter is element L1 - 1 - t1 of line
// (o, L2 - t2), for t2 = 0 element (L1 - t1) of line (o, 0) (X[L] for
// t1 = 0).  Tiles of mirrored column pairs (as in r2c_paired_body) keep both
// reads inside one CTA, so the second hits the cache.  Then the ordinary pass
// A work: inverse (re/im swapped) stages, the four-step twiddle and the
// transposing store, all with the paired line mapping.
template <int LOGL, int C, bool POUT = false>
__device__ __forceinline__ void c2r_paired_body(const LineParams& p, long long cta) {
  using Sc = Sched<LOGL>;
  constexpr int L1 = Sc::L, E = Sc::E, T = Sc::T;
  static_assert(C % 2 == 0 && T * C > 32, "paired tiles: even C, CTA-wide exchange");
  extern __shared__ __align__(1024) float2 smem_raw[];
  LineSmem<LOGL, C, true, true, false> sm{smem_raw};
  const int tid = threadIdx.x;
  const int c = tid % C, t = tid / C;
  const long long L2 = p.pcols, tiles = L2 / C;
  const long long o = cta / tiles, a = (cta % tiles) * (C / 2);
  const long long t2 = paired_column<C>(c, a, L2);
  const long long q = o * L2 + t2;

  float2 v[E];
  {
    const long long base = line_off(p.in, q);
    const long long pbase = line_off(p.in, o * L2 + ((L2 - t2) & (L2 - 1)));
    // element t1 = t + T e at b0 + e S, its mirror at b1 - e S
    const long long S = (long long)T * p.in.es;
    const long long b0 = base + (long long)t * p.in.es;
    const long long b1 = t2 ? pbase + (long long)(L1 - 1 - t) * p.in.es : base + (long long)(L1 - t) * p.in.es;
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int t1 = t + T * e;
      const long long k = t2 + L2 * t1;
      const float2 s0 = make_float2(__ldg(p.in.re + b0 + e * S), __ldg(p.in.im + b0 + e * S));
      const float2 s1 = make_float2(__ldg(p.in.re + b1 - e * S), __ldg(p.in.im + b1 - e * S));
      float2 z;
      if (k == 0) {
        z = make_float2(s0.x + s1.x, s0.x - s1.x);
      } else {
        const float2 w = ldg2(p.rtw + k);
        const float2 ha = cadd(s0, cconj(s1));
        const float2 hb = cmul(csub(cconj(s1), s0), cconj(w));
        z = cadd(ha, cmul_negi(hb));
      }
      v[e] = cswap(z);
    }
  }
  run_stages<LOGL, C, true, false, 0>(v, t, c, p.tw, sm);

  if constexpr (Sc::NSTAGES > 1) __syncthreads();
#pragma unroll
  for (int e = 0; e < E; e++) sm.put(c, t + T * e, v[e]);
  __syncthreads();
  const int c2 = tid / T, tt = tid % T;
  const long long q2 = o * L2 + paired_column<C>(c2, a, L2);
  const long long base = line_off(p.out, q2);
  const long long SO = (long long)T * p.out.es;
  float* por = p.out.re + base + (long long)tt * p.out.es;
  float* poi = p.out.im + base + (long long)tt * p.out.es;
  if constexpr (POUT) {
    // output pairs (im = re + 1, element stride 2): 8-byte stores
    float* pz = p.out.re + base + 2LL * tt;
    if (p.out.es == 2 && !(reinterpret_cast<uintptr_t>(pz) & 7)) {
      float2* pp = reinterpret_cast<float2*>(pz);
      auto emit2 = [&](auto full) {
#pragma unroll
        for (int e = 0; e < E; e++) {
          const int k1 = tt + T * e;
          pp[T * e] = cswap(cmul(sm.get(c2, k1), fourstep_twiddle<L1, decltype(full)::value>(p, q2, k1)));
        }
      };
      if (p.tw_full) emit2(std::true_type{});
      else emit2(std::false_type{});
      return;
    }
  }
  auto emit = [&](auto full) {
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int k1 = tt + T * e;
      float2 x = cmul(sm.get(c2, k1), fourstep_twiddle<L1, decltype(full)::value>(p, q2, k1));
      x = cswap(x);
      por[e * SO] = x.x;
      poi[e * SO] = x.y;
    }
  };
  if (p.tw_full) emit(std::true_type{});
  else emit(std::false_type{});
}

#ifndef AFFT_STAGE_T
#define AFFT_STAGE_T 8
#endif
#ifndef AFFT_C2R_OUT_T
#define AFFT_C2R_OUT_T 8
#endif
// Rows of at most 128 points (T <= 8 threads per line): a warp holds 32/T
// whole lines, 32 E consecutive elements when the lines are contiguous.
// Plain 4-byte accesses of the canonical layout touch 4 to 32 lines per warp
// instruction; staging moves the warp's chunk with coalesced 16-byte accesses
// through the exchange buffer instead.  Usable when the lines are contiguous
// (hi == L) and both arrays are 16-byte aligned.
__device__ __forceinline__ bool rows_contiguous(const LineIO& io, int L) {
  return io.hi == L && io.qshift == 0 && io.qmask == 0 &&
         ((reinterpret_cast<uintptr_t>(io.re) | reinterpret_cast<uintptr_t>(io.im)) & 15) == 0;
}

// The staging pass's own view of the exchange buffer and its lane order,
// chosen by an exhaustive bank count so both the 4-element groups a lane
// moves and the canonical reads hit distinct bank pairs per half-warp:
// 32-point lines use pitch 34 with one pad per 16 elements (the stages'
// layout costs 4x there); 128-point lines keep the stages' layout with lane
// bits 3 and 4 swapped (2x otherwise).  Warps synchronise only among their
// own lanes, so each warp's staging view stays inside the region its lines
// occupy in the stages' layout (WL lines of pitch LP from WL * LP * warp).
template <int L, class SM>
__device__ __forceinline__ int stage_idx(const SM& sm, int c, int j) {
  if constexpr (L == 32) {
    constexpr int WL = 16;   // lines per warp (2 threads per line)
    return (c / WL) * (WL * SM::LP) + (c % WL) * 34 + j + (j >> 4);
  } else {
    return sm.idx(c, j);
  }
}
template <int L>
__device__ __forceinline__ int stage_lane(int lane) {
  if constexpr (L == 128) return (lane & 7) | (((lane >> 3) & 1) << 4) | (((lane >> 4) & 1) << 3);
  else return lane;
}

template <int LOGL, int C, class SM>
__device__ __forceinline__ void rows_stage_in(const LineParams& p, long long cta, const SM& sm,
                                              float2 (&v)[Sched<LOGL>::E], int t, int c) {
  using Sc = Sched<LOGL>;
  constexpr int L = Sc::L, E = Sc::E, T = Sc::T, WL = 32 / T;
  const int lane = stage_lane<L>(threadIdx.x & 31), w = threadIdx.x >> 5;
  const long long q0 = cta * C + (long long)w * WL;
  const float4* gr = reinterpret_cast<const float4*>(p.in.re + q0 * L);
  const float4* gi = reinterpret_cast<const float4*>(p.in.im + q0 * L);
#pragma unroll
  for (int i = 0; i < E / 4; i++) {
    const int f = 32 * i + lane;   // float4 of the warp's chunk
    const int cl = (4 * f) / L, j = (4 * f) % L;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (q0 + cl < p.nlines) {
      a = __ldg(gr + f);
      b = __ldg(gi + f);
    }
    const int cc = w * WL + cl;
    sm.s[stage_idx<L>(sm, cc, j)] = make_float2(a.x, b.x);
    sm.s[stage_idx<L>(sm, cc, j + 1)] = make_float2(a.y, b.y);
    sm.s[stage_idx<L>(sm, cc, j + 2)] = make_float2(a.z, b.z);
    sm.s[stage_idx<L>(sm, cc, j + 3)] = make_float2(a.w, b.w);
  }
  __syncwarp();
#pragma unroll
  for (int e = 0; e < E; e++) v[e] = sm.s[stage_idx<L>(sm, c, t + T * e)];
  __syncwarp();   // every lane has its values before the stages reuse the buffer
}

template <int LOGL, int C, class SM>
__device__ __forceinline__ void rows_stage_out(const LineParams& p, long long cta, const SM& sm,
                                               const float2 (&v)[Sched<LOGL>::E], int t, int c) {
  using Sc = Sched<LOGL>;
  constexpr int L = Sc::L, E = Sc::E, T = Sc::T, WL = 32 / T;
  const int lane = stage_lane<L>(threadIdx.x & 31), w = threadIdx.x >> 5;
  const long long q0 = cta * C + (long long)w * WL;
  __syncwarp();   // the last stage's reads of the buffer are done
#pragma unroll
  for (int e = 0; e < E; e++) sm.s[stage_idx<L>(sm, c, t + T * e)] = v[e];
  __syncwarp();
  float4* gr = reinterpret_cast<float4*>(p.out.re + q0 * L);
  float4* gi = reinterpret_cast<float4*>(p.out.im + q0 * L);
#pragma unroll
  for (int i = 0; i < E / 4; i++) {
    const int f = 32 * i + lane;
    const int cl = (4 * f) / L, j = (4 * f) % L;
    if (q0 + cl < p.nlines) {
      const int cc = w * WL + cl;
      const float2 x0 = sm.s[stage_idx<L>(sm, cc, j)], x1 = sm.s[stage_idx<L>(sm, cc, j + 1)],
                   x2 = sm.s[stage_idx<L>(sm, cc, j + 2)], x3 = sm.s[stage_idx<L>(sm, cc, j + 3)];
      gr[f] = make_float4(x0.x, x1.x, x2.x, x3.x);
      gi[f] = make_float4(x0.y, x1.y, x2.y, x3.y);
    }
  }
}

// Short real rows (r2c: L <= 128 complex points of the interleaved view;
// c2r: input for L <= 32, measured slower beyond, output for L <= 128),
// staged
// per warp like rows_stage_in/out: the 2L reals of a line are contiguous
// (float4 accesses, 16-byte aligned), and the L + 1 bins of consecutive
// lines are contiguous in each split array (coalesced 4-byte accesses, any
// alignment), kept during staging in a pitch-(L + 1) view inside the warp's
// region of the exchange buffer.
__device__ __forceinline__ bool reals_contiguous(const LineIO& io, int L) {
  return io.es == 2 && io.im == io.re + 1 && io.hi == 2 * L && io.qshift == 0 && io.qmask == 0 &&
         (reinterpret_cast<uintptr_t>(io.re) & 15) == 0;
}
__device__ __forceinline__ bool bins_contiguous(const LineIO& io, int L) {
  return io.es == 1 && io.hi == L + 1 && io.qshift == 0 && io.qmask == 0;
}
template <int L, int WL, class SM>
__device__ __forceinline__ int bins_idx(int c, int k) {
  static_assert(L + 1 <= SM::LP, "a line's bins fit its slot of the exchange buffer");
  return (c / WL) * (WL * SM::LP) + (c % WL) * (L + 1) + k;
}

// r2c: the interleaved reals of the warp's lines into the canonical layout
template <int LOGL, int C, class SM>
__device__ __forceinline__ void rows_stage_in_reals(const LineParams& p, long long cta, const SM& sm,
                                                    float2 (&v)[Sched<LOGL>::E], int t, int c) {
  using Sc = Sched<LOGL>;
  constexpr int L = Sc::L, E = Sc::E, T = Sc::T, WL = 32 / T;
  const int lane = stage_lane<L>(threadIdx.x & 31), w = threadIdx.x >> 5;
  const long long q0 = cta * C + (long long)w * WL;
  const float4* g = reinterpret_cast<const float4*>(p.in.re + q0 * 2 * L);
#pragma unroll
  for (int i = 0; i < E / 2; i++) {
    const int f = 32 * i + lane;   // float4 = 2 complex of the warp's chunk
    const int cl = (2 * f) / L, j = (2 * f) % L;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
    if (q0 + cl < p.nlines) a = __ldg(g + f);
    const int cc = w * WL + cl;
    sm.s[stage_idx<L>(sm, cc, j)] = make_float2(a.x, a.y);
    sm.s[stage_idx<L>(sm, cc, j + 1)] = make_float2(a.z, a.w);
  }
  __syncwarp();
#pragma unroll
  for (int e = 0; e < E; e++) v[e] = sm.s[stage_idx<L>(sm, c, t + T * e)];
  __syncwarp();
}

// r2c: the warp's bins X[0..L] (x[e] at k = t + T e, xl = X[L]) out
template <int LOGL, int C, class SM>
__device__ __forceinline__ void rows_stage_out_bins(const LineParams& p, long long cta, const SM& sm,
                                                    const float2 (&x)[Sched<LOGL>::E], float2 xl, int t, int c) {
  using Sc = Sched<LOGL>;
  constexpr int L = Sc::L, E = Sc::E, T = Sc::T, WL = 32 / T, B = WL * (L + 1);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long q0 = cta * C + (long long)w * WL;
  __syncwarp();   // the post-pass reads of the buffer are done
#pragma unroll
  for (int e = 0; e < E; e++) sm.s[bins_idx<L, WL, SM>(c, t + T * e)] = x[e];
  if (t == 0) sm.s[bins_idx<L, WL, SM>(c, L)] = xl;
  __syncwarp();
  const int wb = bins_idx<L, WL, SM>(w * WL, 0);
  float* gr = p.out.re + q0 * (L + 1);
  float* gi = p.out.im + q0 * (L + 1);
  for (int i = lane; i < B; i += 32) {
    if (q0 + i / (L + 1) < p.nlines) {
      const float2 b = sm.s[wb + i];
      gr[i] = b.x;
      gi[i] = b.y;
    }
  }
}

// c2r: the warp's bins in, the pre-pass (as in line_fft_body) into the
// canonical layout
template <int LOGL, int C, class SM>
__device__ __forceinline__ void rows_stage_in_bins(const LineParams& p, long long cta, const SM& sm,
                                                   float2 (&v)[Sched<LOGL>::E], int t, int c) {
  using Sc = Sched<LOGL>;
  constexpr int L = Sc::L, E = Sc::E, T = Sc::T, WL = 32 / T, B = WL * (L + 1);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long q0 = cta * C + (long long)w * WL;
  const int wb = bins_idx<L, WL, SM>(w * WL, 0);
  const float* gr = p.in.re + q0 * (L + 1);
  const float* gi = p.in.im + q0 * (L + 1);
  for (int i = lane; i < B; i += 32) {
    float2 b = make_float2(0.f, 0.f);
    if (q0 + i / (L + 1) < p.nlines) b = make_float2(__ldg(gr + i), __ldg(gi + i));
    sm.s[wb + i] = b;
  }
  __syncwarp();
#pragma unroll
  for (int e = 0; e < E; e++) {
    const int i = t + T * e;
    const float2 s0 = sm.s[bins_idx<L, WL, SM>(c, i)];
    const float2 s1 = sm.s[bins_idx<L, WL, SM>(c, L - i)];
    float2 z;
    if (i == 0) {
      z = make_float2(s0.x + s1.x, s0.x - s1.x);
    } else {
      const float2 wt = ldg2(p.rtw + i);
      const float2 a = cadd(s0, cconj(s1));
      const float2 b = cmul(csub(cconj(s1), s0), cconj(wt));
      z = cadd(a, cmul_negi(b));
    }
    v[e] = cswap(z);
  }
  __syncwarp();
}

// c2r: the canonical outputs z (reals x[2k], x[2k+1]) out as float4
template <int LOGL, int C, class SM>
__device__ __forceinline__ void rows_stage_out_reals(const LineParams& p, long long cta, const SM& sm,
                                                     const float2 (&z)[Sched<LOGL>::E], int t, int c) {
  using Sc = Sched<LOGL>;
  constexpr int L = Sc::L, E = Sc::E, T = Sc::T, WL = 32 / T;
  const int lane = stage_lane<L>(threadIdx.x & 31), w = threadIdx.x >> 5;
  const long long q0 = cta * C + (long long)w * WL;
  __syncwarp();   // the last stage's reads of the buffer are done
#pragma unroll
  for (int e = 0; e < E; e++) sm.s[stage_idx<L>(sm, c, t + T * e)] = z[e];
  __syncwarp();
  float4* g = reinterpret_cast<float4*>(p.out.re + q0 * 2 * L);
#pragma unroll
  for (int i = 0; i < E / 2; i++) {
    const int f = 32 * i + lane;
    const int cl = (2 * f) / L, j = (2 * f) % L;
    if (q0 + cl < p.nlines) {
      const int cc = w * WL + cl;
      const float2 z0 = sm.s[stage_idx<L>(sm, cc, j)], z1 = sm.s[stage_idx<L>(sm, cc, j + 1)];
      g[f] = make_float4(z0.x, z0.y, z1.x, z1.y);
    }
  }
}

// The body of one CTA's work: lines [cta*C, cta*C + C) of the launch `p`.
// UNIT, rows mode: 1 both element strides are 1 (split complex rows), 2 both
// are 2 with im = re + 1 (interleaved complex rows, loaded and stored as
// float2; for the real kinds the real side: R2C's input, C2R's output), so
// element offsets are compile-time constants instead of runtime 64-bit
// products.  Cols mode: bit 0 the input, bit 1 the output are
// interleaved pairs (im = re + 1, even strides), accessed as float2 (the
// paired R2C pass: bit 0 only; the paired C2R pass: bit 1 only).
// TMA: the CTA's input tile is already in the exchange buffer, put there by
// tma_load_tile (cols mode, split planes): [re: L rows x C][im: L rows x C]
// floats; C2R tiles hold bins 0 .. L-1 there and read bin L directly.
// The output planes of a cols tile (element t + T e of line c in v[e]) into
// the tile's buffer st, [L][C] floats each, re then im, for TMA stores: a
// half-warp writes 16 adjacent columns of one row (no bank conflicts).  The
// first barrier waits for the stages' last reads of the buffer; the proxy
// fence makes the writes visible to the TMA unit.
template <int L, int C, int T, int E>
__device__ __forceinline__ void bulk_stage_out(const float2 (&v)[E], int t, int c, float* st) {
  __syncthreads();
#pragma unroll
  for (int e = 0; e < E; e++) {
    st[(t + T * e) * C + c] = v[e].x;
    st[L * C + (t + T * e) * C + c] = v[e].y;
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
}

// BULK: a C2C or C2R cols pass over a TMA-loaded tile leaves its output
// planes in the tile's buffer (bulk_stage_out) for the caller to store by TMA
// (line_fft_tma_bulk) instead of storing them itself.
template <int LOGL, int C, bool COLS, int KIND, bool TSTORE, bool TC = false, int UNIT = 0, bool TMA = false,
          bool BULK = false>
__device__ __forceinline__ void line_fft_body(const LineParams& p, long long cta, TcState* ts = nullptr) {
  static_assert(!TMA || (COLS && !TC && (UNIT == 0 || KIND == LK_C2C) && (!TSTORE || KIND == LK_C2C)),
                "TMA tiles: cols passes");
  static_assert(!BULK || (TMA && (KIND == LK_C2C || KIND == LK_C2R) && !TSTORE && UNIT == 0),
                "TMA stores: split C2C and C2R cols tiles");
  if constexpr (KIND == LK_R2C_HALF) {
    static_assert(COLS && !TSTORE && !TC, "the split R2C pass is a plain cols pass");
    r2c_half_body<LOGL, C>(p, cta);
    return;
  }
  if constexpr (KIND == LK_R2C_PAIRED) {
    static_assert(COLS && !TSTORE && !TC, "the paired R2C pass is a plain cols pass");
    r2c_paired_body<LOGL, C, (UNIT & 1) != 0>(p, cta);
    return;
  }
  if constexpr (KIND == LK_C2R_PAIRED) {
    static_assert(COLS && TSTORE && !TC, "the paired C2R pass is pass A of a four-step");
    c2r_paired_body<LOGL, C, (UNIT & 2) != 0>(p, cta);
    return;
  }
  using Sc = Sched<LOGL>;
  constexpr int L = Sc::L, E = Sc::E, T = Sc::T;
  constexpr int RU = COLS ? 0 : UNIT;       // rows: unit-stride variants
  constexpr int CPAIRS = COLS ? UNIT : 0;   // cols: interleaved-pair input / output
  // a line lives inside one warp: rows mode with T <= 32, or a single line
  constexpr bool WARP_ONLY = (!COLS && T <= 32) || (T * C <= 32);
  extern __shared__ __align__(1024) float2 smem_raw[];
  LineSmem<LOGL, C, COLS, TSTORE, TC> sm{smem_raw};

  const int tid = threadIdx.x;
  const int c = COLS ? (tid % C) : (tid / T);
  const int t = COLS ? (tid / C) : (tid % T);
  const long long q = cta * C + c;
  const bool active = q < p.nlines;

  float2 v[E];
  if constexpr (KIND == LK_C2R) {
    // real inverse pre-pass (onedim.hpp:1064-1068 / multi.hpp:366-370 with
    // inverse): Z'[i] = a - i*b, a = X[i] + conj(X[L-i]),
    // b = (conj(X[L-i]) - X[i]) * conj(w_i); Z'[0] from the real parts of
    // X[0] and X[L]; then the inverse transform of Z' (swap trick).
    bool staged = false;
    // (lines of at most 32 points: at 128 points staging measured 1.4x slower)
    if constexpr (!COLS && T <= 2 && E == 16 && !TC) {
      if (bins_contiguous(p.in, L)) {
        rows_stage_in_bins<LOGL, C>(p, cta, sm, v, t, c);
        staged = true;
      }
    }
    if constexpr (TMA) {
      // bins from the tile: bin i of column c at raw[i C + c] (re plane) and
      // raw[L C + i C + c] (im plane); bin L (the mirror of bin 0) from HBM
      const float* raw = reinterpret_cast<const float*>(smem_raw);
      float2 bl = make_float2(0.f, 0.f);
      if (t == 0 && active) {
        const long long oL = line_off(p.in, q) + (long long)L * p.in.es;
        bl = make_float2(__ldg(p.in.re + oL), __ldg(p.in.im + oL));
      }
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int i = t + T * e;
        const float2 s0 = make_float2(raw[i * C + c], raw[L * C + i * C + c]);
        const int im = (L - i) & (L - 1);
        const float2 s1 = i == 0 ? bl : make_float2(raw[im * C + c], raw[L * C + im * C + c]);
        float2 z;
        if (i == 0) {
          z = make_float2(s0.x + s1.x, s0.x - s1.x);
        } else {
          float2 w = ldg2(p.rtw + i);
          float2 a = cadd(s0, cconj(s1));
          float2 b = cmul(csub(cconj(s1), s0), cconj(w));
          z = cadd(a, cmul_negi(b));
        }
        v[e] = cswap(z);
      }
      __syncthreads();   // the tile is read before the stages reuse the buffer
    } else if (staged) {
    } else if (active) {
      // bin i = t + T e at p0 + e S, its mirror L - i at p1 - e S
      const long long base = line_off(p.in, q);
      const long long S = (long long)T * p.in.es;
      const long long o0 = base + (long long)t * p.in.es, o1 = base + (long long)(L - t) * p.in.es;
      const float *p0r = p.in.re + o0, *p0i = p.in.im + o0, *p1r = p.in.re + o1, *p1i = p.in.im + o1;
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int i = t + T * e;
        float2 s0 = make_float2(__ldg(p0r + e * S), __ldg(p0i + e * S));
        float2 s1 = make_float2(__ldg(p1r - e * S), __ldg(p1i - e * S));
        float2 z;
        if (i == 0) {
          z = make_float2(s0.x + s1.x, s0.x - s1.x);
        } else {
          float2 w = ldg2(p.rtw + i);
          float2 a = cadd(s0, cconj(s1));
          float2 b = cmul(csub(cconj(s1), s0), cconj(w));
          z = cadd(a, cmul_negi(b));
        }
        v[e] = cswap(z);
      }
    } else {
#pragma unroll
      for (int e = 0; e < E; e++) v[e] = make_float2(0.f, 0.f);
    }
  } else {
    // short contiguous rows: warp-staged coalesced loads (rows_stage_in)
    bool staged = false;
    if constexpr (KIND == LK_R2C && !COLS && T <= AFFT_STAGE_T && E == 16 && !TC) {
      if (reals_contiguous(p.in, L)) {
        rows_stage_in_reals<LOGL, C>(p, cta, sm, v, t, c);
        staged = true;
      }
    }
    if constexpr (RU == 1 && T <= AFFT_STAGE_T && E == 16 && !TC) {
      if (rows_contiguous(p.in, L)) {
        rows_stage_in<LOGL, C>(p, cta, sm, v, t, c);
        staged = true;
      }
    }
    if constexpr (RU == 2 && T <= AFFT_STAGE_T && E == 16 && !TC) {
      if (reals_contiguous(p.in, L)) {   // interleaved pairs: the same view as real rows
        rows_stage_in_reals<LOGL, C>(p, cta, sm, v, t, c);
        staged = true;
      }
    }
    if constexpr (RU != 0) {
      if (staged && p.inverse) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
      }
    }
    if constexpr (TMA) {
      if constexpr (CPAIRS & 1) {
        // input pairs: element i of column c is the pair raw2[i C + c]; a
        // warp's lanes read 32 consecutive pairs
        const float2* raw2 = reinterpret_cast<const float2*>(smem_raw);
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = raw2[(t + T * e) * C + c];
      } else {
        // element i of column c at raw[i C + c] (re plane), raw[L C + i C + c]
        // (im plane): a warp's 32 lanes read 32 consecutive words
        const float* raw = reinterpret_cast<const float*>(smem_raw);
#pragma unroll
        for (int e = 0; e < E; e++) {
          const int i = t + T * e;
          v[e] = make_float2(raw[i * C + c], raw[L * C + i * C + c]);
        }
      }
      if (p.inverse) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
      }
      __syncthreads();   // the tile is read before the stages reuse the buffer
    } else if (staged) {
    } else if (active) {
      const long long base = line_off(p.in, q);
      if constexpr (RU == 1) {
        const float* pr = p.in.re + base + t;
        const float* pi = p.in.im + base + t;
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = make_float2(__ldg(pr + T * e), __ldg(pi + T * e));
      } else if constexpr (RU == 2) {
        const float* pz = p.in.re + base;
        if ((reinterpret_cast<uintptr_t>(pz) & 7) == 0) {
          const float2* pp = reinterpret_cast<const float2*>(pz) + t;
#pragma unroll
          for (int e = 0; e < E; e++) v[e] = __ldg(pp + T * e);
        } else {
#pragma unroll
          for (int e = 0; e < E; e++) v[e] = make_float2(__ldg(pz + 2 * (t + T * e)), __ldg(pz + 2 * (t + T * e) + 1));
        }
      } else {
        // per-thread line pointers and one warp-uniform stride between a
        // thread's elements (T * es), so each element costs one uniform
        // multiple instead of a 64-bit multiply-add per array
        const long long S = (long long)T * p.in.es;
        const float* pr = p.in.re + base + (long long)t * p.in.es;
        const float* pi = p.in.im + base + (long long)t * p.in.es;
        // cols kernels built for interleaved input pairs (UNIT bit 0: im right
        // after re, even stride): one 8-byte load per element where the line
        // starts 8-byte aligned
        if ((CPAIRS & 1) && !(reinterpret_cast<uintptr_t>(pr) & 7)) {
          const float2* pz = reinterpret_cast<const float2*>(pr);
#pragma unroll
          for (int e = 0; e < E; e++) v[e] = __ldg(pz + e * (S >> 1));
        } else {
#pragma unroll
          for (int e = 0; e < E; e++) v[e] = make_float2(__ldg(pr + e * S), __ldg(pi + e * S));
        }
      }
      if (p.inverse) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
      }
    } else {
#pragma unroll
      for (int e = 0; e < E; e++) v[e] = make_float2(0.f, 0.f);
    }
  }

  run_stages<LOGL, C, COLS, WARP_ONLY, 0, TC, packed_bfly<LOGL, COLS, TSTORE>()>(v, t, c, p.tw, sm, ts);

  if constexpr (KIND == LK_C2C) {
    if constexpr (TSTORE) {
      // computed with the cols mapping, stored with the rows mapping; the
      // four-step twiddle is applied here, where consecutive threads walk
      // along one line (coalesced table reads, no values held across it)
      if constexpr (Sc::NSTAGES > 1) line_sync<false>();
#pragma unroll
      for (int e = 0; e < E; e++) sm.put(c, t + T * e, v[e]);
      __syncthreads();
      const int c2 = tid / T, t2 = tid % T;
      const long long q2 = cta * C + c2;
      if (q2 < p.nlines) {
        const long long base = line_off(p.out, q2);
        const bool inv = p.inverse;
        // one branch-free loop per case, so the twiddle loads issue together
        // tw: 0 none, 1 matrix table, 2 hi/lo pair
        // the four-step passes store with unit element stride: compile-time
        // offsets from one pointer per array; other strides as the loads
        const long long S = (long long)T * p.out.es;
        float* pr = p.out.re + base + (long long)t2 * p.out.es;
        float* pi = p.out.im + base + (long long)t2 * p.out.es;
        auto emit = [&](auto tw, auto unit) {
          constexpr int TW = decltype(tw)::value;
#pragma unroll
          for (int e = 0; e < E; e++) {
            float2 x = sm.get(c2, t2 + T * e);
            if constexpr (TW) x = cmul(x, fourstep_twiddle<L, TW == 1>(p, q2, t2 + T * e));
            x = inv ? cswap(x) : x;
            const long long o = decltype(unit)::value ? (long long)(T * e) : e * S;
            pr[o] = x.x;
            pi[o] = x.y;
          }
        };
        auto emit_tw = [&](auto unit) {
          if (!p.tw_n) emit(std::integral_constant<int, 0>{}, unit);
          else if (p.tw_full) emit(std::integral_constant<int, 1>{}, unit);
          else emit(std::integral_constant<int, 2>{}, unit);
        };
        bool stored = false;
        if constexpr ((CPAIRS & 2) != 0) {
          // output pairs (im = re + 1, element stride 2): one 8-byte store
          // per element
          float* pz = p.out.re + base + 2LL * t2;
          if (p.out.es == 2 && !(reinterpret_cast<uintptr_t>(pz) & 7)) {
            float2* pp = reinterpret_cast<float2*>(pz);
            auto emit2 = [&](auto tw) {
              constexpr int TW = decltype(tw)::value;
#pragma unroll
              for (int e = 0; e < E; e++) {
                float2 x = sm.get(c2, t2 + T * e);
                if constexpr (TW) x = cmul(x, fourstep_twiddle<L, TW == 1>(p, q2, t2 + T * e));
                pp[T * e] = inv ? cswap(x) : x;
              }
            };
            if (!p.tw_n) emit2(std::integral_constant<int, 0>{});
            else if (p.tw_full) emit2(std::integral_constant<int, 1>{});
            else emit2(std::integral_constant<int, 2>{});
            stored = true;
          }
        }
        if (stored) {
        } else if (p.out.es == 1) {
          emit_tw(std::true_type{});
        } else {
          emit_tw(std::false_type{});
        }
      }
    } else {
      // four-step twiddles only occur in cols passes
      if constexpr (COLS) {
        if (p.tw_n && p.tw_full) {
#pragma unroll
          for (int e = 0; e < E; e++) v[e] = cmul(v[e], fourstep_twiddle<L, true>(p, q, t + T * e));
        } else if (p.tw_n) {
#pragma unroll
          for (int e = 0; e < E; e++) v[e] = cmul(v[e], fourstep_twiddle<L, false>(p, q, t + T * e));
        }
      }
      if (p.inverse) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
      }
      if constexpr (BULK) {
        bulk_stage_out<L, C, T>(v, t, c, reinterpret_cast<float*>(smem_raw));
        return;
      }
      bool staged_out = false;
      if constexpr (RU == 1 && T <= AFFT_STAGE_T && E == 16 && !TC) {
        if (rows_contiguous(p.out, L)) {
          rows_stage_out<LOGL, C>(p, cta, sm, v, t, c);
          staged_out = true;
        }
      }
      if constexpr (RU == 2 && T <= AFFT_STAGE_T && E == 16 && !TC) {
        if (reals_contiguous(p.out, L)) {
          rows_stage_out_reals<LOGL, C>(p, cta, sm, v, t, c);
          staged_out = true;
        }
      }
      if (!staged_out && active) {
        const long long base = line_off(p.out, q);
        if constexpr (RU == 1) {
          float* pr = p.out.re + base + t;
          float* pi = p.out.im + base + t;
#pragma unroll
          for (int e = 0; e < E; e++) {
            pr[T * e] = v[e].x;
            pi[T * e] = v[e].y;
          }
        } else if constexpr (RU == 2) {
          float* pz = p.out.re + base;
          if ((reinterpret_cast<uintptr_t>(pz) & 7) == 0) {
            float2* pp = reinterpret_cast<float2*>(pz) + t;
#pragma unroll
            for (int e = 0; e < E; e++) pp[T * e] = v[e];
          } else {
#pragma unroll
            for (int e = 0; e < E; e++) {
              pz[2 * (t + T * e)] = v[e].x;
              pz[2 * (t + T * e) + 1] = v[e].y;
            }
          }
        } else {
          const long long S = (long long)T * p.out.es;
          float* pr = p.out.re + base + (long long)t * p.out.es;
          float* pi = p.out.im + base + (long long)t * p.out.es;
          if ((CPAIRS & 2) && !(reinterpret_cast<uintptr_t>(pr) & 7)) {
            float2* pz = reinterpret_cast<float2*>(pr);   // output pairs (UNIT bit 1): 8-byte stores
#pragma unroll
            for (int e = 0; e < E; e++) pz[e * (S >> 1)] = v[e];
          } else {
#pragma unroll
            for (int e = 0; e < E; e++) {
              pr[e * S] = v[e].x;
              pi[e * S] = v[e].y;
            }
          }
        }
      }
    }
  } else if constexpr (KIND == LK_C2R) {
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
    if constexpr (BULK) {
      bulk_stage_out<L, C, T>(v, t, c, reinterpret_cast<float*>(smem_raw));
      return;
    }
    bool staged_out = false;
    if constexpr (!COLS && T <= AFFT_C2R_OUT_T && E == 16 && !TC) {
      if (reals_contiguous(p.out, L)) {
        rows_stage_out_reals<LOGL, C>(p, cta, sm, v, t, c);
        staged_out = true;
      }
    }
    if (!staged_out && active) {
      const long long base = line_off(p.out, q);
      if constexpr (RU == 2) {
        // the real output as pairs (x[2i], x[2i+1]) with unit pair stride
        float* pz = p.out.re + base;
        if (!(reinterpret_cast<uintptr_t>(pz) & 7)) {
          float2* pp = reinterpret_cast<float2*>(pz) + t;
#pragma unroll
          for (int e = 0; e < E; e++) pp[T * e] = v[e];
        } else {
#pragma unroll
          for (int e = 0; e < E; e++) {
            pz[2 * (t + T * e)] = v[e].x;
            pz[2 * (t + T * e) + 1] = v[e].y;
          }
        }
      } else {
        const long long S = (long long)T * p.out.es;
        float* pr = p.out.re + base + (long long)t * p.out.es;
        float* pi = p.out.im + base + (long long)t * p.out.es;
#pragma unroll
        for (int e = 0; e < E; e++) {
          pr[e * S] = v[e].x;
          pi[e * S] = v[e].y;
        }
      }
    }
  } else {
    // real forward post-pass (onedim.hpp:1058-1108 / multi.hpp:354-414):
    // X[k] = a - i*b, a = (Z[k] + conj(Z[L-k]))/2,
    // b = (Z[k] - conj(Z[L-k])) * w_k / 2; X[0], X[L] from Z[0].
    if constexpr (Sc::NSTAGES > 1) line_sync<WARP_ONLY>();
#pragma unroll
    for (int e = 0; e < E; e++) sm.put(c, t + T * e, v[e]);
    line_sync<WARP_ONLY>();
    if constexpr (!COLS && T <= AFFT_STAGE_T && E == 16 && !TC) {
      // bins X[k] (k = t + T e) replace v; xl = X[L] (from the k = 0 thread)
      float2 xl = make_float2(0.f, 0.f);
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int k = t + T * e;
        const float2 s0 = v[e];
        const float2 s1 = sm.get(c, (L - k) & (L - 1));
        if (k == 0) {
          v[e] = make_float2(s0.x + s0.y, 0.f);
          xl = make_float2(s0.x - s0.y, 0.f);
        } else {
          const float2 w = ldg2(p.rtw + k);
          const float2 a = make_float2(0.5f * (s0.x + s1.x), 0.5f * (s0.y - s1.y));
          const float2 d = make_float2(0.5f * (s0.x - s1.x), 0.5f * (s0.y + s1.y));
          const float2 b = cmul(d, w);
          v[e] = cadd(a, cmul_negi(b));
        }
      }
      bool staged_out = false;
      if constexpr (!COLS && T <= AFFT_STAGE_T && E == 16 && !TC) {
        if (bins_contiguous(p.out, L)) {
          rows_stage_out_bins<LOGL, C>(p, cta, sm, v, xl, t, c);
          staged_out = true;
        }
      }
      if (!staged_out && active) {
        const long long base = line_off(p.out, q);
#pragma unroll
        for (int e = 0; e < E; e++) {
          const long long a = base + (long long)(t + T * e) * p.out.es;
          p.out.re[a] = v[e].x;
          p.out.im[a] = v[e].y;
        }
        if (t == 0) {
          const long long aL = base + (long long)L * p.out.es;
          p.out.re[aL] = xl.x;
          p.out.im[aL] = xl.y;
        }
      }
    } else {
      if (active) {
        const long long base = line_off(p.out, q);
        const long long S = (long long)T * p.out.es;
        float* pr = p.out.re + base + (long long)t * p.out.es;
        float* pi = p.out.im + base + (long long)t * p.out.es;
#pragma unroll
        for (int e = 0; e < E; e++) {
          const int k = t + T * e;
          const float2 s0 = v[e];
          const float2 s1 = sm.get(c, (L - k) & (L - 1));
          float2 x;
          if (k == 0) {
            x = make_float2(s0.x + s0.y, 0.f);
            const long long aL = base + (long long)L * p.out.es;
            p.out.re[aL] = s0.x - s0.y;
            p.out.im[aL] = 0.f;
          } else {
            const float2 w = ldg2(p.rtw + k);
            const float2 a = make_float2(0.5f * (s0.x + s1.x), 0.5f * (s0.y - s1.y));
            const float2 d = make_float2(0.5f * (s0.x - s1.x), 0.5f * (s0.y + s1.y));
            const float2 b = cmul(d, w);
            x = cadd(a, cmul_negi(b));
          }
          pr[e * S] = x.x;
          pi[e * S] = x.y;
        }
      }
    }
  }
}

// Per-CTA set-up of the TC form: TMEM columns (64 per 128-row tile), the
// mbarrier and the DFT matrix tiles Mh, Ml in the K-major core layout.
template <int NTHREADS>
__device__ __forceinline__ void tc_setup(TcState& S, const LineParams& p, unsigned char* bt,
                                         uint64_t* mbar, uint32_t* tmem_slot, float2* exch) {
  constexpr int NT = NTHREADS / 128;
  constexpr int COLS = NT * 64;   // 128 or 256: a power of two as tcgen05.alloc needs
  static_assert(NT == 2 || NT == 4, "TC form: 256 or 512 threads");
  const int tid = threadIdx.x;
  if (tid < 256) {
    const int mat = tid >> 7, n = (tid & 127) >> 2, g = tid & 3;
    *(uint4*)(bt + mat * 2048 + tc_core_off(n, 8 * g)) = *(const uint4*)(p.tc_b + mat * 1024 + n * 32 + 8 * g);
  }
  if (tid < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "n"(COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  S.a = (unsigned char*)exch;
  S.b = bt;
  S.mbar = smem_u32(mbar);
  S.tmem = *tmem_slot;
  S.phase = 0;
  S.err = p.err;
}

template <int NTHREADS>
__device__ __forceinline__ void tc_teardown(const TcState& S) {
  constexpr int COLS = (NTHREADS / 128) * 64;
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(S.tmem), "n"(COLS));
}

template <int LOGL, int C, bool COLS, int KIND, bool TSTORE, bool TC = false, int UNIT = 0>
__global__ void __launch_bounds__(Sched<LOGL>::T * C, min_ctas<Sched<LOGL>::T * C>())
line_fft(const LineParams p) {
  if constexpr (TC) {
    __shared__ __align__(1024) unsigned char bt[4096];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    extern __shared__ __align__(1024) float2 smem_raw[];
    TcState S;
    tc_setup<Sched<LOGL>::T * C>(S, p, bt, &mbar, &tmem_slot, smem_raw);
    line_fft_body<LOGL, C, COLS, KIND, TSTORE, true, UNIT>(p, blockIdx.x, &S);
    tc_teardown<Sched<LOGL>::T * C>(S);
  } else {
    line_fft_body<LOGL, C, COLS, KIND, TSTORE, false, UNIT>(p, blockIdx.x);
  }
}

// ---------------------------------------------------------------------------
// TMA-fed cols passes
// ---------------------------------------------------------------------------
// A cols tile of C lines reads C * 4 bytes (32 for C = 8) of each row it
// touches.  Through the LSU every load wavefront then carries one 32-byte
// segment, and the 1024- and 2048-point passes saturate L1 (74-84% of its
// throughput for 25% of HBM's).  Here one thread loads the CTA's whole input
// tile with tensor-map copies (cp.async.bulk.tensor, 3D boxes of C columns x
// BR rows) into the exchange buffer, completing on an mbarrier; the threads
// then read their canonical elements from shared memory.
//
// The maps (encoded on the host per launch) view a plane of the input as
// {columns of one outer block, L rows (stride es), outer blocks (stride
// hi)}: line q = o * ncols + col is column col of block o, and a CTA's C
// lines are C adjacent columns of one block.  Both planes' bases, es * 4 and
// hi * 4 are multiples of 16 bytes and the column of a tile is a multiple of
// C (>= 4 floats), so every box starts on a 16-byte boundary.
struct TmaTile {
  CUtensorMap re, im;   // the input's re and im planes (pairs: re maps the interleaved array, im unused)
  int box_rows;         // rows per box (<= 256, divides L)
  int rows;             // rows loaded per plane (L)
  int pairs;            // 1: one interleaved array of re,im pairs, boxes of 2 C floats
};

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z,
                                            uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(mbar)
      : "memory");
}

// Thread 0's part of a tile load: (re)initialise the barrier at mb and issue
// the tile of CTA `cta` into dst ([re rows][C] then [im rows][C] floats, or
// [rows][2 C] for pairs).  The coordinates need only the input's column mask
// and shift.  Other threads may wait on the barrier only after a CTA barrier
// that follows this call.
template <int C>
__device__ __forceinline__ void tma_issue_tile(long long qmask, int qshift, const TmaTile& tm, long long cta,
                                               uint32_t mb, void* dst) {
  const long long q0 = cta * C;
  const int col = (int)(q0 & qmask);
  const int outer = (int)(q0 >> qshift);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  const int rows = tm.rows, br = tm.box_rows;
  const uint32_t bytes = 2u * (uint32_t)rows * C * 4u;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
  const uint32_t d = smem_u32(dst);
  if (tm.pairs) {
    // one array of pairs: the tile is [rows][2 C floats], column col at float 2 col
    for (int r = 0; r < rows; r += br) tma_load_3d(d + (uint32_t)r * C * 8u, &tm.re, 2 * col, r, outer, mb);
  } else {
    const uint32_t plane = (uint32_t)rows * C * 4u;
    for (int r = 0; r < rows; r += br) {
      tma_load_3d(d + (uint32_t)r * C * 4u, &tm.re, col, r, outer, mb);
      tma_load_3d(d + plane + (uint32_t)r * C * 4u, &tm.im, col, r, outer, mb);
    }
  }
}

// Every thread waits for the tile, bounded; on success thread 0 invalidates
// the barrier (a later tile of the same CTA sets it up again); on a timeout
// the error word is set, the copies get a second bounded wait, and the whole
// CTA returns false.
__device__ __forceinline__ bool tma_wait_tile(uint32_t mb, int* err) {
  const bool ok = __syncthreads_and(tc_wait(mb, 0));
  if (ok && threadIdx.x == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(mb) : "memory");
  if (!ok) {
    if (threadIdx.x == 0) {
      if (err) atomicExch(err, 2);
      tc_wait(mb, 0);   // let copies still in flight land before the CTA's shared memory goes away
    }
    __syncthreads();
  }
  return ok;
}

// Loads the tile of CTA `cta` into dst (as tma_issue_tile) and waits for it.
template <int C>
__device__ __forceinline__ bool tma_load_tile(const LineParams& p, const TmaTile& tm, long long cta, uint64_t* mbar,
                                              void* dst) {
  const uint32_t mb = smem_u32(mbar);
  if (threadIdx.x == 0) tma_issue_tile<C>(p.in.qmask, p.in.qshift, tm, cta, mb, dst);
  __syncthreads();   // the barrier's set-up is visible before anyone waits on it
  return tma_wait_tile(mb, p.err);
}

template <int LOGL, int C, int KIND, bool TSTORE = false, int UNIT = 0>
__global__ void __launch_bounds__(Sched<LOGL>::T * C, min_ctas<Sched<LOGL>::T * C>())
line_fft_tma(const LineParams p, const __grid_constant__ TmaTile tm) {
  __shared__ __align__(8) uint64_t mbar;
  extern __shared__ __align__(1024) float2 smem_raw[];
  if (!tma_load_tile<C>(p, tm, blockIdx.x, &mbar, smem_raw)) return;
  line_fft_body<LOGL, C, true, KIND, TSTORE, false, UNIT, true>(p, blockIdx.x);
}

// The paired R2C pass (four-step pass B of a long 1D real forward, input
// pairs) with its tile loaded by TMA.  Its mirrored half starts 8 bytes off a
// 16-byte boundary, so it comes as a box of H + 2 pair-columns from the
// boundary below (tile 0's box runs past the last column and reads the fill
// value there), the aligned half as a box of H, and tile 0's column L1/2 as a
// box of 2 (16 bytes).  Maps over the pairs array as {2 L1 floats, L2 rows,
// transforms}.
struct PairedTma {
  CUtensorMap al, mi, sp;   // boxes of 2H, 2H + 4 and 4 floats x box_rows rows
  int box_rows;
};

template <int LOGL, int C>
__global__ void __launch_bounds__(Sched<LOGL>::T * C, min_ctas<Sched<LOGL>::T * C>())
line_fft_paired_tma(const LineParams p, const __grid_constant__ PairedTma pt) {
  constexpr int L2 = Sched<LOGL>::L, H = C / 2;
  __shared__ __align__(8) uint64_t mbar;
  extern __shared__ __align__(1024) float2 smem_raw[];
  const long long L1 = p.pcols, tiles = L1 / C, cta = blockIdx.x;
  const long long o = cta / tiles, a = (cta % tiles) * H;
  const uint32_t mb = smem_u32(&mbar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t bytes = (uint32_t)L2 * (2 * H + 2 * H + 4 + (a == 0 ? 4 : 0)) * 4u;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
    const uint32_t d = smem_u32(smem_raw);
    const uint32_t mi = (uint32_t)L2 * 2 * H * 4u, sp = mi + (uint32_t)L2 * (2 * H + 4) * 4u;
    const int z = (int)o;
    for (int r = 0; r < L2; r += pt.box_rows) {
      tma_load_3d(d + (uint32_t)r * 2 * H * 4u, &pt.al, (int)(2 * a), r, z, mb);
      tma_load_3d(d + mi + (uint32_t)r * (2 * H + 4) * 4u, &pt.mi, (int)(2 * (L1 - a - H)), r, z, mb);
      if (a == 0) tma_load_3d(d + sp + (uint32_t)r * 16u, &pt.sp, (int)L1, r, z, mb);
    }
  }
  __syncthreads();   // the barrier's set-up is visible before anyone waits on it
  if (!tma_wait_tile(mb, p.err)) return;
  r2c_paired_body<LOGL, C, true, true>(p, cta);
}

// One launch of a multi-transform queue: a device-side table of segments
// (one per transform pass of this kernel shape), each covering `nctas`
// virtual CTAs starting at cta0, and seg_of[v], the segment of virtual CTA v.
// One CTA per virtual CTA (a persistent grid walking them in turn measured
// 1.2-1.6x slower: a CTA that loops cannot overlap its loads with another
// virtual CTA's compute the way separate CTAs do).  Warp 0 stages the
// segment's parameters in shared memory.
struct Segment {
  LineParams p;
  long long cta0;
  const TmaTile* tma;   // TMA-capable kernels: this segment's tensor maps (global memory), or null
};

__device__ __forceinline__ void stage_params(LineParams& dst, const LineParams& src) {
  static_assert(sizeof(LineParams) % 4 == 0, "parameters copy as words");
  if (threadIdx.x < 32) {
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&src);
    uint32_t* d = reinterpret_cast<uint32_t*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(LineParams) / 4); i += 32) d[i] = __ldg(s + i);
  }
}

// TMA: every segment has tensor maps and loads its tiles by TMA (as
// line_fft_tma); segments without them go to the LSU form of the kernel.
template <int LOGL, int C, bool COLS, int KIND, bool TSTORE, bool TC = false, int UNIT = 0, bool TMA = false>
__global__ void __launch_bounds__(Sched<LOGL>::T * C, min_ctas<Sched<LOGL>::T * C>())
line_fft_grouped(const Segment* __restrict__ segs, const int* __restrict__ seg_of, long long total) {
  __shared__ LineParams sp;
  if constexpr (TMA) {
    static_assert(COLS && !TC, "TMA tiles: cols passes");
    __shared__ __align__(8) uint64_t mbar;
    extern __shared__ __align__(1024) float2 smem_raw[];
    const uint32_t mb = smem_u32(&mbar);
    for (long long v = blockIdx.x; v < total; v += gridDim.x) {
      const int sg = __ldg(seg_of + v);
      const long long cta = v - __ldg(&segs[sg].cta0);
      __syncthreads();   // the previous virtual CTA is done with sp, the barrier and the buffer
      // the tile's loads go out before the parameters are staged, straight
      // from the segment's column mask, shift and tensor maps (the mixed
      // queue 12.52 -> 12.45 ms against loading after the staging)
      if (threadIdx.x == 0)
        tma_issue_tile<C>(__ldg(&segs[sg].p.in.qmask), __ldg(&segs[sg].p.in.qshift), *segs[sg].tma, cta, mb,
                          smem_raw);
      stage_params(sp, segs[sg].p);
      __syncthreads();   // parameters staged, the barrier's set-up visible
      if (!tma_wait_tile(mb, sp.err)) return;
      line_fft_body<LOGL, C, true, KIND, TSTORE, false, UNIT, true>(sp, cta);
    }
    return;
  }
  if constexpr (TC) {
    __shared__ __align__(1024) unsigned char bt[4096];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    extern __shared__ __align__(1024) float2 smem_raw[];
    TcState S;
    tc_setup<Sched<LOGL>::T * C>(S, segs[0].p, bt, &mbar, &tmem_slot, smem_raw);
    for (long long v = blockIdx.x; v < total; v += gridDim.x) {
      const int sg = __ldg(seg_of + v);
      __syncthreads();
      stage_params(sp, segs[sg].p);
      __syncthreads();
      line_fft_body<LOGL, C, COLS, KIND, TSTORE, true, UNIT>(sp, v - segs[sg].cta0, &S);
    }
    tc_teardown<Sched<LOGL>::T * C>(S);
  } else {
    for (long long v = blockIdx.x; v < total; v += gridDim.x) {
      const int sg = __ldg(seg_of + v);
      __syncthreads();   // a previous iteration is done with sp and the staging buffers
      stage_params(sp, segs[sg].p);
      __syncthreads();
      line_fft_body<LOGL, C, COLS, KIND, TSTORE, false, UNIT>(sp, v - segs[sg].cta0);
    }
  }
}

// ---------------------------------------------------------------------------
// standalone real pre/post pass for transforms too long for one CTA
// ---------------------------------------------------------------------------
struct RealPassParams {
  LineIO in, out;
  long long nlines;
  long long L;            // complex length (real length 2L)
  const float2* rtw;      // W_{2L}^k, k < L
  int inverse;            // 0: Z -> X (forward post), 1: X -> Z' (inverse pre)
  int lines_fastest;      // thread index walks lines first (cols layout)
};

// Thread (q, k) with k in [0, L/2] handles the pair (k, L-k) of line q, so
// the pass can run in place.
__global__ void real_pass_kernel(const RealPassParams p);

// Copies `nlines` lines of `len` complex elements between two layouts (used
// to pack/unpack the row-pair view of N-D real data around a four-step pass).
struct CopyParams {
  LineIO in, out;
  long long nlines, len;
};
__global__ void copy_lines_kernel(const CopyParams p);

// Elementwise ops of a multi-transform queue (real pass, copy, size-1 real)
// in one launch over a segment table, as for line_fft_grouped; every segment
// covers `nblocks` virtual blocks of 256 threads.
enum { EW_REAL = 0, EW_COPY = 1, EW_REAL1 = 2 };
struct EwSegment {
  int type;
  RealPassParams rp;
  CopyParams cp;
  long long blk0;
};
__global__ void elementwise_grouped(const EwSegment* __restrict__ segs, const int* __restrict__ seg_of,
                                    long long total);

// Real transforms of total size 1: X[0] = x[0] + 0i (forward), x[0] = re X[0]
// (inverse), one element per line.
__global__ void real1_kernel(const RealPassParams p);

}  // namespace agb
