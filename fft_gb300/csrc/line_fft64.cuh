// FP64 line-FFT kernels for sm_103a: the double-precision transforms of
// afft's fft.h (afft_64_*, fft.h:52-80; fft.cpp:221-300 instantiates the same
// plans for double).
//
// Same line addressing as the FP32 kernels (LineIO: offsets and strides count
// elements, here doubles) and the same self-sorting Stockham formulation,
// sized for FP64: each thread owns E = 8 complex doubles of one line in the
// canonical layout v[e] = x[t + T*e] (T = L/8), and the stages are radix-8,
// with one radix-2 or radix-4 stage first when log2 L is not a multiple of 3.
// On GB300 FP64 arithmetic, not HBM, bounds these transforms (two FP64 FMA
// lanes per SM per clock, 1/64 of the FP32 rate), and radix-8 stages cost
// about as many FP64 instructions per point and log2 L as radix-16 ones
// (3.5 vs 3.4) with half the registers.
//
// Twiddles are FP64 tables computed on the host (no rounding step).  They
// travel in the LineParams / RealPassParams table fields (tw, tw_full, rtw),
// which point to double2 arrays for these kernels; the four-step twiddle
// always comes from the full matrix table tw_full[t2 * L + k].
#pragma once

#include "line_fft.cuh"

namespace agb {

template <int LOGL>
struct Sched64 {
  static constexpr int L = 1 << LOGL;
  static constexpr int E = LOGL < 3 ? L : 8;
  static constexpr int T = L / E;
  static constexpr int FIRST = (LOGL >= 3 && (LOGL % 3)) ? (1 << (LOGL % 3)) : 0;
  static constexpr int NSTAGES = LOGL < 3 ? 1 : (LOGL / 3 + (FIRST ? 1 : 0));
  static constexpr int radix(int s) { return LOGL < 3 ? L : (FIRST && s == 0 ? FIRST : 8); }
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

// Lines per CTA: rows as the FP32 kernels (256 threads, or one line of up to
// 1024 threads); cols 2048 points per tile up to 256-point lines (256
// threads), 8 lines at 512 and 1024 points (64-byte row segments), 4 at 2048
// (32-byte segments, 128 KB of shared memory).
template <int LOGL, bool COLS>
constexpr int lines_per_cta64() {
  constexpr int L = 1 << LOGL, T = Sched64<LOGL>::T;
  if constexpr (COLS) return L <= 8 ? 256 : (L <= 256 ? 2048 / L : (L <= 1024 ? 8 : 4));
  else return T >= 256 ? 1 : 256 / T;
}

constexpr int ROWS_MAX_LOG64 = 13;   // rows mode: one CTA up to 8192 points (147 KB)
constexpr int COLS_MAX_LOG64 = 11;   // cols mode: up to 2048 points (4 lines, 128 KB)

// ---------------------------------------------------------------------------
// complex double helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 zmul_negi(double2 a) { return make_double2(a.y, -a.x); }   // -i*a
__device__ __forceinline__ double2 zswap(double2 a) { return make_double2(a.y, a.x); }
__device__ __forceinline__ double2 ldz(const double2* p) { return __ldg(p); }

#define AFFT_R2D 0.70710678118654752440   // sqrt(1/2)

__device__ __forceinline__ void zdft2(double2& a, double2& b) {
  const double2 t = a;
  a = zadd(t, b);
  b = zsub(t, b);
}

__device__ __forceinline__ void zdft4(double2& a0, double2& a1, double2& a2, double2& a3) {
  const double2 s02 = zadd(a0, a2), d02 = zsub(a0, a2);
  const double2 s13 = zadd(a1, a3), d13 = zmul_negi(zsub(a1, a3));
  a0 = zadd(s02, s13);
  a2 = zsub(s02, s13);
  a1 = zadd(d02, d13);
  a3 = zsub(d02, d13);
}

// in-place DFT-R, natural order in and out (forward sign)
template <int R>
__device__ __forceinline__ void zdft(double2 (&x)[R]) {
  if constexpr (R == 2) {
    zdft2(x[0], x[1]);
  } else if constexpr (R == 4) {
    zdft4(x[0], x[1], x[2], x[3]);
  } else if constexpr (R == 8) {
    // E = DFT4(even), O = DFT4(odd); X[k] = E[k] + W8^k O[k], X[k+4] = E[k] - W8^k O[k]
    zdft4(x[0], x[2], x[4], x[6]);
    zdft4(x[1], x[3], x[5], x[7]);
    x[3] = make_double2(AFFT_R2D * (x[3].x + x[3].y), AFFT_R2D * (x[3].y - x[3].x));    // W8^1
    x[5] = zmul_negi(x[5]);                                                             // W8^2
    x[7] = make_double2(AFFT_R2D * (x[7].y - x[7].x), -AFFT_R2D * (x[7].x + x[7].y));   // W8^3
    double2 y[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      y[k] = zadd(x[2 * k], x[2 * k + 1]);
      y[k + 4] = zsub(x[2 * k], x[2 * k + 1]);
    }
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = y[i];
  }
}

// ---------------------------------------------------------------------------
// shared-memory layouts for 16-byte elements (a wavefront serves 8 lanes):
//   rows:          line c at c * LP, element j at j + j/8 (LP = L + L/8):
//                  the first stage's stride-R scatter lands in 8 distinct
//                  16-byte bank groups
//   cols, C >= 8:  element j of line c at j * C + (c ^ (j & 7)): 8 lanes
//                  across lines (the stages) and 8 lanes along one line (the
//                  transposing store) both hit distinct bank groups
//   cols, C = 4:   (j ^ bit2(j)) * 4 + c: the two rows a quarter-warp
//                  touches have opposite parity in the scatter and the gather
// ---------------------------------------------------------------------------
template <int L, int C, bool COLS>
struct Smem64 {
  static constexpr int LP = L + L / 8;
  static constexpr int ELEMS = COLS ? L * C : C * LP;
  double2* s;
  __device__ __forceinline__ int idx(int c, int j) const {
    if constexpr (COLS && C >= 8) return j * C + (c ^ (j & 7));
    else if constexpr (COLS) return (j ^ ((j >> 2) & 1)) * C + c;
    else return c * LP + j + (j >> 3);
  }
  __device__ __forceinline__ void put(int c, int j, double2 v) const { s[idx(c, j)] = v; }
  __device__ __forceinline__ double2 get(int c, int j) const { return s[idx(c, j)]; }
};

// One Stockham stage (as the FP32 kernels): butterfly b = t + T*u reads
// slots u + B*r, applies W_{NS R}^{r (b mod NS)}, DFT-R, and scatters to
// shared memory (non-last) or keeps the canonical layout (last).
template <int R, int NS, int E, int T, bool LAST, class SM>
__device__ __forceinline__ void stage64(double2 (&v)[E], int t, int c, const double2* tw, const SM& sm) {
  constexpr int B = E / R;
#pragma unroll
  for (int u = 0; u < B; u++) {
    const int b = t + T * u;
    double2 x[R];
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = v[u + B * r];
    if constexpr (NS > 1) {
      const int k = b & (NS - 1);
#pragma unroll
      for (int r = 1; r < R; r++) x[r] = zmul(x[r], ldz(tw + (r - 1) * NS + k));
    }
    zdft<R>(x);
    if constexpr (LAST) {
#pragma unroll
      for (int r = 0; r < R; r++) v[u + B * r] = x[r];
    } else {
      const int base = (b / NS) * NS * R + (b & (NS - 1));
#pragma unroll
      for (int r = 0; r < R; r++) sm.put(c, base + r * NS, x[r]);
    }
  }
}

template <int LOGL, bool WARP_ONLY, int S, class SM>
__device__ __forceinline__ void run_stages64(double2 (&v)[Sched64<LOGL>::E], int t, int c, const double2* tw,
                                             const SM& sm) {
  using Sc = Sched64<LOGL>;
  if constexpr (S < Sc::NSTAGES) {
    constexpr int R = Sc::radix(S), NS = Sc::ns(S), E = Sc::E, T = Sc::T;
    constexpr bool LAST = S == Sc::NSTAGES - 1;
    if constexpr (S > 0) {
      line_sync<WARP_ONLY>();   // the previous stage's scatter is complete
#pragma unroll
      for (int e = 0; e < E; e++) v[e] = sm.get(c, t + T * e);
      if constexpr (!LAST) line_sync<WARP_ONLY>();   // every gather is done before this stage scatters
    }
    if constexpr (R > 1) stage64<R, NS, E, T, LAST>(v, t, c, tw + Sc::twoff(S), sm);
    run_stages64<LOGL, WARP_ONLY, S + 1>(v, t, c, tw, sm);
  }
}

__device__ __forceinline__ double ldd(const float* base, long long off) {
  return __ldg(reinterpret_cast<const double*>(base) + off);
}
__device__ __forceinline__ void std_(float* base, long long off, double v) {
  reinterpret_cast<double*>(base)[off] = v;
}

// The kernel body for one CTA (C lines).  KIND: LK_C2C, LK_R2C (real forward
// with the post-pass fused after the last stage), LK_C2R (real inverse with
// the pre-pass fused into the loads), with the algebra of afft's real_pass
// (onedim.hpp:1031-1108, multi.hpp:343-414).  TSTORE (cols c2c): computed
// with the cols mapping, stored with the rows mapping, the four-step twiddle
// applied on the way out.
template <int LOGL, int C, bool COLS, int KIND, bool TSTORE>
__device__ __forceinline__ void line_fft64_body(const LineParams& p, long long cta) {
  using Sc = Sched64<LOGL>;
  constexpr int L = Sc::L, E = Sc::E, T = Sc::T;
  constexpr bool WARP_ONLY = (!COLS && T <= 32) || (T * C <= 32);
  extern __shared__ __align__(1024) double2 smem64[];
  Smem64<L, C, COLS> sm{smem64};
  const double2* tw = reinterpret_cast<const double2*>(p.tw);
  const double2* rtw = reinterpret_cast<const double2*>(p.rtw);

  const int tid = threadIdx.x;
  const int c = COLS ? (tid % C) : (tid / T);
  const int t = COLS ? (tid / C) : (tid % T);
  const long long q = cta * C + c;
  const bool active = q < p.nlines;

  double2 v[E];
  if (!active) {
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = make_double2(0.0, 0.0);
  } else if constexpr (KIND == LK_C2R) {
    // Z'[i] = a - i*b, a = X[i] + conj(X[L-i]), b = (conj(X[L-i]) - X[i]) * conj(w_i);
    // Z'[0] from the real parts of X[0] and X[L]; then the inverse transform
    // of Z' as a forward transform with re/im swapped
    const long long base = line_off(p.in, q);
#pragma unroll
    for (int e = 0; e < E; e++) {
      const int i = t + T * e;
      const long long a0 = base + (long long)i * p.in.es;
      const long long a1 = base + (long long)(L - i) * p.in.es;
      const double2 s0 = make_double2(ldd(p.in.re, a0), ldd(p.in.im, a0));
      const double2 s1 = make_double2(ldd(p.in.re, a1), ldd(p.in.im, a1));
      double2 z;
      if (i == 0) {
        z = make_double2(s0.x + s1.x, s0.x - s1.x);
      } else {
        const double2 w = ldz(rtw + i);
        const double2 a = zadd(s0, zconj(s1));
        const double2 b = zmul(zsub(zconj(s1), s0), zconj(w));
        z = zadd(a, zmul_negi(b));
      }
      v[e] = zswap(z);
    }
  } else {
    const long long base = line_off(p.in, q);
#pragma unroll
    for (int e = 0; e < E; e++) {
      const long long a = base + (long long)(t + T * e) * p.in.es;
      v[e] = make_double2(ldd(p.in.re, a), ldd(p.in.im, a));
    }
    if (p.inverse) {
#pragma unroll
      for (int e = 0; e < E; e++) v[e] = zswap(v[e]);
    }
  }

  run_stages64<LOGL, WARP_ONLY, 0>(v, t, c, tw, sm);

  if constexpr (KIND == LK_C2C && TSTORE) {
    if constexpr (Sc::NSTAGES > 1) __syncthreads();
#pragma unroll
    for (int e = 0; e < E; e++) sm.put(c, t + T * e, v[e]);
    __syncthreads();
    const int c2 = tid / T, t2 = tid % T;
    const long long q2 = cta * C + c2;
    if (q2 < p.nlines) {
      const long long base = line_off(p.out, q2);
      const double2* twf = reinterpret_cast<const double2*>(p.tw_full);
      const int r2 = (int)((q2 >> p.tw_qshift) & p.tw_qmask);
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int k = t2 + T * e;
        double2 x = sm.get(c2, k);
        if (p.tw_n) x = zmul(x, ldz(twf + (long long)r2 * L + k));
        if (p.inverse) x = zswap(x);
        const long long a = base + (long long)k * p.out.es;
        std_(p.out.re, a, x.x);
        std_(p.out.im, a, x.y);
      }
    }
  } else if constexpr (KIND == LK_C2C) {
    if constexpr (COLS) {
      if (p.tw_n) {
        const double2* twf = reinterpret_cast<const double2*>(p.tw_full);
        const int r2 = (int)((q >> p.tw_qshift) & p.tw_qmask);
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = zmul(v[e], ldz(twf + (long long)r2 * L + t + T * e));
      }
    }
    if (active) {
      const long long base = line_off(p.out, q);
#pragma unroll
      for (int e = 0; e < E; e++) {
        const double2 x = p.inverse ? zswap(v[e]) : v[e];
        const long long a = base + (long long)(t + T * e) * p.out.es;
        std_(p.out.re, a, x.x);
        std_(p.out.im, a, x.y);
      }
    }
  } else if constexpr (KIND == LK_C2R) {
    if (active) {
      const long long base = line_off(p.out, q);
#pragma unroll
      for (int e = 0; e < E; e++) {
        const double2 x = zswap(v[e]);
        const long long a = base + (long long)(t + T * e) * p.out.es;
        std_(p.out.re, a, x.x);
        std_(p.out.im, a, x.y);
      }
    }
  } else {
    // real forward post-pass: X[k] = a - i*b, a = (Z[k] + conj(Z[L-k]))/2,
    // b = (Z[k] - conj(Z[L-k])) * w_k / 2; X[0], X[L] from Z[0]
    if constexpr (Sc::NSTAGES > 1) line_sync<WARP_ONLY>();
#pragma unroll
    for (int e = 0; e < E; e++) sm.put(c, t + T * e, v[e]);
    line_sync<WARP_ONLY>();
    if (active) {
      const long long base = line_off(p.out, q);
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int k = t + T * e;
        const double2 s0 = v[e];
        const double2 s1 = sm.get(c, (L - k) & (L - 1));
        double2 x;
        if (k == 0) {
          x = make_double2(s0.x + s0.y, 0.0);
          const long long aL = base + (long long)L * p.out.es;
          std_(p.out.re, aL, s0.x - s0.y);
          std_(p.out.im, aL, 0.0);
        } else {
          const double2 w = ldz(rtw + k);
          const double2 a = make_double2(0.5 * (s0.x + s1.x), 0.5 * (s0.y - s1.y));
          const double2 d = make_double2(0.5 * (s0.x - s1.x), 0.5 * (s0.y + s1.y));
          x = zadd(a, zmul_negi(zmul(d, w)));
        }
        const long long a = base + (long long)k * p.out.es;
        std_(p.out.re, a, x.x);
        std_(p.out.im, a, x.y);
      }
    }
  }
}

template <int LOGL, int C, bool COLS, int KIND, bool TSTORE>
__global__ void __launch_bounds__(Sched64<LOGL>::T * C) line_fft64(const LineParams p) {
  line_fft64_body<LOGL, C, COLS, KIND, TSTORE>(p, blockIdx.x);
}

// FP64 forms of the standalone real pass, the line copy and the size-1 real
// transform (the FP32 ones are in real_pass.cu); their table is double2.
__global__ void real_pass_kernel64(const RealPassParams p);
__global__ void copy_lines_kernel64(const CopyParams p);
__global__ void real1_kernel64(const RealPassParams p);

}  // namespace agb
