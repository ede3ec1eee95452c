// Persistent, TMA-pipelined cols passes of 2048 and 1024 points
// (line_fft_pipe, and line_fft_pipe_grouped for the multi-transform queue).
//
// A 2048-point cols tile of 8 lines is 128 KB, so the one-tile-per-CTA
// kernels (line_fft, line_fft_tma) fit one CTA per SM.  Each SM then loads
// a tile, runs its stages and stores it in sequence, and HBM idles while the
// SMs compute.  Here one CTA per SM (two for 1024-point tiles) walks the
// tiles blockIdx.x, blockIdx.x + gridDim.x, ...  As soon as its threads have taken tile i out
// of the raw buffer (into registers), one thread issues the TMA loads of the
// CTA's next tile into that buffer.  Those land while tile i's stages run and
// its results are stored (the C2C passes and the 1024-point C2R pass: by TMA
// from the exchange buffer, one plane at a time).
//
// Shared memory: the raw tile ([re: L rows x C][im: L rows x C] floats,
// 128 KB at 2048 points, as tma_load_tile lays it out) and a separate exchange buffer through
// which the stages pass the re parts first, then the im parts.  Element j of
// line c sits at float (j + j/8) * C + c there (one pad row per 8: 72 KB;
// 1024-point tiles pad one row per 4, below).  A
// warp covers 4 consecutive threads t (lanes 8 apart share a line), so each
// access touches 4 rows, and the padding puts them on 4 different 8-bank
// groups for the radix-8 scatter (rows 8 apart), the radix-16 scatter
// (consecutive rows) and the canonical gather: one wavefront per access.  Each
// pattern's row is a per-thread base plus a compile-time offset per element.
//
// Every wait on the tile barrier is bounded (one second); a timeout sets the
// error word to 2, waits once more (bounded) for the copies in flight, and the
// CTA returns.
#pragma once
#include "line_fft.cuh"

// LATE_ISSUE: the next tile's loads go out after the first exchange barrier
// (which then also marks the raw tile consumed) instead of after a barrier of
// their own: 1% faster for C2R, and for C2C with BULK_STORE.  BULK_STORE: the
// C2C pass stages each output plane in the exchange buffer and stores it with
// TMA (cp.async.bulk.tensor) instead of per-thread stores: 1-3% faster for
// C2C, 1-2.5% slower for the 2048-point C2R pass (which keeps per-thread
// stores; the 1024-point one below gains from them).
#ifndef AFFT_PIPE_LATE_ISSUE
#define AFFT_PIPE_LATE_ISSUE 1
#endif
#ifndef AFFT_PIPE_BULK_STORE
#define AFFT_PIPE_BULK_STORE 1
#endif
// the 2048-point R2C pass in this form too (unsplit, the post-pass mirrors
// through the exchange buffer) instead of the split one-tile-per-two-CTAs
// form: built and taken only when set (measured 20% slower)
#ifndef AFFT_PIPE_R2C
#define AFFT_PIPE_R2C 0
#endif
// lines per tile: 8 (one 1024-thread CTA per SM, 200 KB) or 4 (two
// 512-thread CTAs per SM, 100 KB each)
#ifndef AFFT_PIPE_C
#define AFFT_PIPE_C 8
#endif
// the 1024-point complex and C2R cols passes in this form too (8-line tiles,
// two 512-thread CTAs per SM, 104 KB each)
#ifndef AFFT_PIPE10
#define AFFT_PIPE10 1
#endif
// and the 1024-point four-step pass A (transposing store): built and taken
// only when set (measured 2-4% slower than the one-tile TMA kernel at large
// batches: 2^20 x 64 c2c 0.4717 vs 0.4553 ms)
#ifndef AFFT_PIPE10_TSTORE
#define AFFT_PIPE10_TSTORE 0
#endif
// the one-tile TMA kernels of 512-point (AFFT_TMA_BULK9) and 256-point
// (AFFT_TMA_BULK8) complex cols passes store their tile by TMA too
// (line_fft_tma_bulk).  Measured against per-thread stores: 512² x 64 c2c
// 0.1010 vs 0.1092 ms; at 256 points 256³ c2c 0.1358 vs 0.1338 ms (slower,
// off) and 2^16 x 256 c2c 0.0990 vs 0.1000-0.1010 ms
#ifndef AFFT_TMA_BULK9
#define AFFT_TMA_BULK9 1
#endif
#ifndef AFFT_TMA_BULK8
#define AFFT_TMA_BULK8 0
#endif
// the same for the 512- and 256-point C2R cols passes: 512 x 64 x 64 x 16
// c2r 0.1113 vs 0.1133 ms at 256 points (on); 1024² x 16 c2r 0.0703 vs
// 0.0683 ms at 512 points (slower, off)
#ifndef AFFT_TMA_BULK_C2R9
#define AFFT_TMA_BULK_C2R9 0
#endif
#ifndef AFFT_TMA_BULK_C2R8
#define AFFT_TMA_BULK_C2R8 1
#endif
// the one-tile 1024-point complex and C2R kernels (taken where the tiles are
// too few for the pipelined ones): 1024² x 2 c2c 0.0272 vs 0.0293-0.0304
// ms, 1024 x 512 x 4 ci 0.0272 vs 0.0293 ms (on); C2R level (off)
#ifndef AFFT_TMA_BULK10
#define AFFT_TMA_BULK10 1
#endif
#ifndef AFFT_TMA_BULK_C2R10
#define AFFT_TMA_BULK_C2R10 0
#endif

namespace agb {

#ifndef AFFT_PIPE_BULK10
#define AFFT_PIPE_BULK10 1
#endif
#ifndef AFFT_PIPE_BULK_C2R10
#define AFFT_PIPE_BULK_C2R10 1
#endif
// the passes that store by TMA (the complex ones; at 1024 points when
// AFFT_PIPE_BULK10; the 1024-point C2R pass when AFFT_PIPE_BULK_C2R10:
// 3.5-5.5% faster there, where at 2048 points the C2R pass measured 1-2.5%
// slower with them)
template <int LOGL, int KIND>
constexpr bool pipe_bulk() {
  return AFFT_PIPE_BULK_STORE && ((KIND == LK_C2C && (LOGL == 11 || AFFT_PIPE_BULK10)) ||
                                  (KIND == LK_C2R && LOGL == 10 && AFFT_PIPE_BULK_C2R10));
}

// Rows of the exchange buffer.  2048-point schedule (radix 8, 16, 16; T =
// 128): row = j + j/8.  Stage 0 scatters output e = u + 2 r of butterfly
// b = t + 128 u to element 8 b + r, stage 1 output e of butterfly t to
// element 128 (t / 8) + t % 8 + 8 e, and the gather takes element t + 128 e.
// 1024-point schedule (radix 4, 16, 16; T = 64): row = j + j/4.  Stage 0
// scatters output e = u + 4 r of butterfly b = t + 64 u to element 4 b + r,
// stage 1 output e of butterfly t to element 64 (t / 4) + t % 4 + 4 e, the
// gather takes element t + 64 e.  Each is base(t) + offset(e).
template <int LOGL>
__host__ __device__ constexpr int pipe_rows() {
  return LOGL == 11 ? 2048 + 2048 / 8 : 1024 + 1024 / 4;
}
template <int LOGL>
__device__ __forceinline__ int pipe_row(int j) {
  return LOGL == 11 ? j + (j >> 3) : j + (j >> 2);
}
template <int LOGL, int S>
__device__ __forceinline__ int pipe_wbase(int t) {
  if constexpr (LOGL == 11) return S == 0 ? 9 * t : 144 * (t >> 3) + (t & 7);
  else return S == 0 ? 5 * t : 80 * (t >> 2) + (t & 3);
}
template <int LOGL, int S>
__host__ __device__ constexpr int pipe_woff(int e) {
  if constexpr (LOGL == 11) return S == 0 ? 1152 * (e % 2) + e / 2 : 9 * e;
  else return S == 0 ? 320 * (e % 4) + e / 4 : 5 * e;
}
template <int LOGL>
__device__ __forceinline__ int pipe_gbase(int t) {
  return LOGL == 11 ? t + (t >> 3) : t + (t >> 2);
}
template <int LOGL>
__host__ __device__ constexpr int pipe_goff(int e) {
  return LOGL == 11 ? 144 * e : 80 * e;
}

// The transposing store's staging of 8-line 1024-point tiles: element k of
// line c at k * 8 + ((c + k / 4) & 7).  Written in the cols mapping (4
// consecutive k x 8 lines per warp) and read along lines (32 consecutive k of
// one line per warp), both on 32 distinct banks.
__device__ __forceinline__ int pipe_tsidx(int k, int c) { return k * 8 + ((c + (k >> 2)) & 7); }

// The exchange after stage S: every value to its stage-S position, then
// element t + T e of this thread's line back, re parts first, then im parts.
// TRAIL: the buffer is written again before the next CTA-wide barrier.
// hook: run by every thread after the first barrier (the late tile issue).
template <int LOGL, int C, int S, bool TRAIL, class Hook>
__device__ __forceinline__ void pipe_exchange(float2 (&v)[Sched<LOGL>::E], int t, int c, float* xs, const Hook& hook) {
  constexpr int E = Sched<LOGL>::E;
  float* w = xs + pipe_wbase<LOGL, S>(t) * C + c;
  const float* g = xs + pipe_gbase<LOGL>(t) * C + c;
  float nx[E];
#pragma unroll
  for (int e = 0; e < E; e++) w[pipe_woff<LOGL, S>(e) * C] = v[e].x;
  __syncthreads();
  hook();
#pragma unroll
  for (int e = 0; e < E; e++) nx[e] = g[pipe_goff<LOGL>(e) * C];
  __syncthreads();
#pragma unroll
  for (int e = 0; e < E; e++) w[pipe_woff<LOGL, S>(e) * C] = v[e].y;
  __syncthreads();
#pragma unroll
  for (int e = 0; e < E; e++) v[e] = make_float2(nx[e], g[pipe_goff<LOGL>(e) * C]);
  if constexpr (TRAIL) __syncthreads();
}

// All stages of one tile, values in registers in the canonical layout on
// entry and exit (as run_stages).
// XOUT: the exchange buffer is written again after the stages (TMA stores,
// the transposing store), so the last exchange ends with a barrier.
template <int LOGL, int C, int KIND, bool XOUT, int S, class Hook>
__device__ __forceinline__ void pipe_stages(float2 (&v)[Sched<LOGL>::E], int t, int c, const float2* tw,
                                            float* xs, const Hook& hook) {
  using Sc = Sched<LOGL>;
  if constexpr (S < Sc::NSTAGES) {
    constexpr int R = Sc::radix(S), NS = Sc::ns(S);
    // the butterflies with their outputs kept in registers (stage()'s last-stage form)
    stage<R, NS, Sc::E, Sc::T, true, false, 0, packed_bfly<LOGL, true>()>(v, t, c, tw + Sc::twoff(S), xs, false,
                                                                         nullptr);
    if constexpr (S + 1 < Sc::NSTAGES) {
      constexpr bool TRAIL = S + 2 < Sc::NSTAGES || KIND == LK_R2C || XOUT;
      if constexpr (S == 0) {
        pipe_exchange<LOGL, C, S, TRAIL>(v, t, c, xs, hook);
      } else {
        pipe_exchange<LOGL, C, S, TRAIL>(v, t, c, xs, [] {});
      }
      pipe_stages<LOGL, C, KIND, XOUT, S + 1>(v, t, c, tw, xs, hook);
    }
  }
}

// Issue the TMA loads of tile `tile` (C adjacent columns of one outer block,
// both planes, boxes of C columns x box_rows rows) on the barrier at mb.
template <int L, int C>
__device__ __forceinline__ void pipe_issue(long long qmask, int qshift, const TmaTile& tm, long long tile,
                                           uint32_t raw, uint32_t mb) {
  const long long q0 = tile * C;
  const int col = (int)(q0 & qmask);
  const int outer = (int)(q0 >> qshift);
  constexpr uint32_t plane = (uint32_t)L * C * 4u;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(2u * plane) : "memory");
  for (int r = 0; r < L; r += tm.box_rows) {
    tma_load_3d(raw + (uint32_t)r * C * 4u, &tm.re, col, r, outer, mb);
    tma_load_3d(raw + plane + (uint32_t)r * C * 4u, &tm.im, col, r, outer, mb);
  }
}

__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, int x, int y, int z, uint32_t src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(z), "r"(src)
               : "memory");
}

// Store one output plane of tile `tile` from the dense [L][C] staging in the
// exchange buffer (boxes of C columns x box_rows rows), as one bulk group.
template <int L, int C>
__device__ __forceinline__ void pipe_store_plane(const LineParams& p, const CUtensorMap* map, int box_rows,
                                                 long long tile, uint32_t xs) {
  const long long q0 = tile * C;
  const int col = (int)(q0 & p.out.qmask);
  const int outer = (int)(q0 >> p.out.qshift);
  for (int r = 0; r < L; r += box_rows) tma_store_3d(map, col, r, outer, xs + (uint32_t)r * C * 4u);
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// The tile loop of the pipelined kernels.  This CTA takes tiles first,
// first + gridDim.x, ... < ntiles; prep(v, &cta) returns the parameters of
// tile v (and its CTA index within them), and issue(v) (thread 0) issues
// tile v's loads on the barrier at mb.  The grouped form's prep stages the
// parameters in shared memory, behind a CTA barrier of its own.
//
// KIND: LK_C2C (with the four-step twiddle when p.tw_n), LK_R2C (unsplit:
// the post-pass through the exchange buffer), LK_C2R (the pre-pass from the
// raw tile, bin L read directly).  Split planes in, split planes out; every
// tile whole (the host's tma_tile rules).  BULK: the output planes go out by
// TMA (the output maps tmo; C2C and C2R).
template <int LOGL, int C, int KIND, bool BULK, bool TSTORE, class Prep, class Issue>
__device__ __forceinline__ void pipe_loop(long long first, long long ntiles, uint32_t mb, float* raw, float* xs,
                                          const TmaTile* tmo, const Prep& prep, const Issue& issue) {
  using Sc = Sched<LOGL>;
  constexpr int L = Sc::L, E = Sc::E, T = Sc::T;
  static_assert(KIND == LK_C2C || KIND == LK_R2C || KIND == LK_C2R, "plain cols kinds");
  static_assert(((LOGL == 11 && (C == 8 || C == 4) && Sc::radix(0) == 8) || (LOGL == 10 && C == 8 && Sc::radix(0) == 4)) &&
                    E == 16,
                "the exchange rows are those of 8- or 4-line 2048-point and 8-line 1024-point tiles");
  static_assert(!BULK || KIND == LK_C2C || KIND == LK_C2R, "TMA stores: the complex and C2R passes");
  static_assert(!TSTORE || (KIND == LK_C2C && LOGL == 10 && C == 8 && !BULK),
                "the transposing store: 8-line 1024-point complex tiles");
  const int tid = threadIdx.x;
  const int c = tid % C, t = tid / C;

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0 && first < ntiles) issue(first);

  uint32_t phase = 0;
  for (long long tile = first; tile < ntiles; tile += gridDim.x, phase ^= 1u) {
    // the previous tile's bulk stores have read the exchange buffer before
    // anyone writes it again
    if (BULK && tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    long long cta;
    const LineParams& p = prep(tile, &cta);
    if (!__syncthreads_and(tc_wait(mb, phase))) {
      if (tid == 0) {
        if (p.err) atomicExch(p.err, 2);
        tc_wait(mb, phase);   // let copies still in flight land before shared memory goes away
      }
      __syncthreads();
      return;
    }
    const long long q = cta * C + c;
    float2 v[E];
    if constexpr (KIND == LK_C2R) {
      // real inverse pre-pass (onedim.hpp:1064-1068 / multi.hpp:366-370 with
      // inverse): Z'[i] = a - i b, a = X[i] + conj(X[L-i]),
      // b = (conj(X[L-i]) - X[i]) conj(w_i); Z'[0] from the real parts of
      // X[0] and X[L]; then the inverse transform of Z' (swap trick)
      float2 bl = make_float2(0.f, 0.f);
      if (t == 0) {
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
          const float2 w = ldg2(p.rtw + i);
          const float2 a = cadd(s0, cconj(s1));
          const float2 b = cmul(csub(cconj(s1), s0), cconj(w));
          z = cadd(a, cmul_negi(b));
        }
        v[e] = cswap(z);
      }
    } else {
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int i = t + T * e;
        v[e] = make_float2(raw[i * C + c], raw[L * C + i * C + c]);
      }
      if (KIND == LK_C2C && p.inverse) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
      }
    }
    // every thread has its tile: the raw buffer takes the next one
    auto issue_next = [&] {
      if (tid == 0 && tile + gridDim.x < ntiles) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(tile + gridDim.x);
      }
    };
    if constexpr (AFFT_PIPE_LATE_ISSUE) {
      pipe_stages<LOGL, C, KIND, BULK || TSTORE, 0>(v, t, c, p.tw, xs, issue_next);
    } else {
      __syncthreads();
      issue_next();
      pipe_stages<LOGL, C, KIND, BULK || TSTORE, 0>(v, t, c, p.tw, xs, [] {});
    }

    const long long base = line_off(p.out, q);
    const long long S = (long long)T * p.out.es;
    float* pr = p.out.re + base + (long long)t * p.out.es;
    float* pi = p.out.im + base + (long long)t * p.out.es;
    if constexpr (TSTORE) {
      // four-step pass A: computed across lines, stored along them with the
      // four-step twiddle (as line_fft_body's transposing store), re parts
      // then im parts through the staging layout
      const int c2 = tid / T, t2 = tid % T;
      const long long q2 = cta * C + c2;
      float rx[E];
#pragma unroll
      for (int e = 0; e < E; e++) xs[pipe_tsidx(t + T * e, c)] = v[e].x;
      __syncthreads();
#pragma unroll
      for (int e = 0; e < E; e++) rx[e] = xs[pipe_tsidx(t2 + T * e, c2)];
      __syncthreads();
#pragma unroll
      for (int e = 0; e < E; e++) xs[pipe_tsidx(t + T * e, c)] = v[e].y;
      __syncthreads();
#pragma unroll
      for (int e = 0; e < E; e++) v[e] = make_float2(rx[e], xs[pipe_tsidx(t2 + T * e, c2)]);
      if (p.tw_n && p.tw_full) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cmul(v[e], fourstep_twiddle<L, true>(p, q2, t2 + T * e));
      } else if (p.tw_n) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cmul(v[e], fourstep_twiddle<L, false>(p, q2, t2 + T * e));
      }
      if (p.inverse) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
      }
      const long long b2 = line_off(p.out, q2);
      const long long S2 = (long long)T * p.out.es;
      float* r2 = p.out.re + b2 + (long long)t2 * p.out.es;
      float* i2 = p.out.im + b2 + (long long)t2 * p.out.es;
#pragma unroll
      for (int e = 0; e < E; e++) {
        r2[e * S2] = v[e].x;
        i2[e * S2] = v[e].y;
      }
      continue;   // the next tile's first write to the buffer follows its own barriers
    }
    if constexpr (KIND == LK_C2C) {
      if (p.tw_n && p.tw_full) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cmul(v[e], fourstep_twiddle<L, true>(p, q, t + T * e));
      } else if (p.tw_n) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cmul(v[e], fourstep_twiddle<L, false>(p, q, t + T * e));
      }
      if (p.inverse) {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
      }
    } else if constexpr (KIND == LK_C2R) {
#pragma unroll
      for (int e = 0; e < E; e++) v[e] = cswap(v[e]);   // re of the output is im of the swapped transform
    }
    if constexpr (BULK) {
      // each plane through the exchange buffer, dense [L][C] as the boxes
      // lay it out (a warp writes 32 consecutive words)
      float* st = xs + t * C + c;
      const uint32_t xs_s = smem_u32(xs);
#pragma unroll
      for (int e = 0; e < E; e++) st[e * T * C] = v[e].x;
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        pipe_store_plane<L, C>(p, &tmo->re, tmo->box_rows, cta, xs_s);
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
      }
      __syncthreads();
#pragma unroll
      for (int e = 0; e < E; e++) st[e * T * C] = v[e].y;
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) pipe_store_plane<L, C>(p, &tmo->im, tmo->box_rows, cta, xs_s);
    } else if constexpr (KIND == LK_C2C || KIND == LK_C2R) {
#pragma unroll
      for (int e = 0; e < E; e++) {
        pr[e * S] = v[e].x;
        pi[e * S] = v[e].y;
      }
    } else {
      // real forward post-pass (onedim.hpp:1058-1108 / multi.hpp:354-414):
      // X[k] = a - i b, a = (Z[k] + conj(Z[L-k]))/2,
      // b = (Z[k] - conj(Z[L-k])) w_k / 2; X[0], X[L] from Z[0].  The mirror
      // Z[L-k] comes through the exchange buffer, re parts then im parts.
      float mx[E];
#pragma unroll
      for (int e = 0; e < E; e++) xs[(pipe_gbase<LOGL>(t) + pipe_goff<LOGL>(e)) * C + c] = v[e].x;
      __syncthreads();
#pragma unroll
      for (int e = 0; e < E; e++) mx[e] = xs[pipe_row<LOGL>((L - (t + T * e)) & (L - 1)) * C + c];
      __syncthreads();
#pragma unroll
      for (int e = 0; e < E; e++) xs[(pipe_gbase<LOGL>(t) + pipe_goff<LOGL>(e)) * C + c] = v[e].y;
      __syncthreads();
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int k = t + T * e;
        const float2 s0 = v[e];
        const float2 s1 = make_float2(mx[e], xs[pipe_row<LOGL>((L - k) & (L - 1)) * C + c]);
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
        pr[e * S] = x.x;
        pi[e * S] = x.y;
      }
    }
  }
  // the last tile's bulk stores have read shared memory before the CTA ends
  if (BULK && tid == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// One plan launch: tiles 0 .. ntiles - 1 of the parameters p, their input
// maps tm (and output maps tmo for the TMA stores).
template <int LOGL, int C, int KIND, bool TSTORE = false>
__global__ void __launch_bounds__(Sched<LOGL>::T * C, 1024 / (Sched<LOGL>::T * C))
line_fft_pipe(const __grid_constant__ LineParams p, const __grid_constant__ TmaTile tm,
              const __grid_constant__ TmaTile tmo, long long ntiles) {
  __shared__ __align__(8) uint64_t mbar;
  extern __shared__ __align__(1024) float2 smem_raw[];
  float* raw = reinterpret_cast<float*>(smem_raw);
  const uint32_t mb = smem_u32(&mbar), raw_s = smem_u32(raw);
  pipe_loop<LOGL, C, KIND, pipe_bulk<LOGL, KIND>() && !TSTORE, TSTORE>(
      blockIdx.x, ntiles, mb, raw, raw + 2 * Sched<LOGL>::L * C, &tmo,
      [&](long long tile, long long* cta) -> const LineParams& {
        *cta = tile;
        return p;
      },
      [&](long long tile) { pipe_issue<Sched<LOGL>::L, C>(p.in.qmask, p.in.qshift, tm, tile, raw_s, mb); });
}

// The queue form: the group's virtual tiles (segments of several transforms,
// every one with tensor maps), one persistent CTA per SM walking them; each
// tile's loads go out from its segment's column mask, shift and maps, and
// its parameters are staged in shared memory when its turn comes.
template <int LOGL, int C, int KIND>
__global__ void __launch_bounds__(Sched<LOGL>::T * C, 1024 / (Sched<LOGL>::T * C))
line_fft_pipe_grouped(const Segment* __restrict__ segs, const int* __restrict__ seg_of, long long total) {
  __shared__ LineParams sp;
  __shared__ __align__(8) uint64_t mbar;
  extern __shared__ __align__(1024) float2 smem_raw[];
  float* raw = reinterpret_cast<float*>(smem_raw);
  const uint32_t mb = smem_u32(&mbar), raw_s = smem_u32(raw);
  pipe_loop<LOGL, C, KIND, false, false>(
      blockIdx.x, total, mb, raw, raw + 2 * Sched<LOGL>::L * C, nullptr,
      [&](long long v, long long* cta) -> const LineParams& {
        const int sg = __ldg(seg_of + v);
        *cta = v - __ldg(&segs[sg].cta0);
        __syncthreads();   // the previous tile is done with sp
        stage_params(sp, segs[sg].p);   // visible after the tile wait's barrier
        return sp;
      },
      [&](long long v) {
        const int sg = __ldg(seg_of + v);
        pipe_issue<Sched<LOGL>::L, C>(__ldg(&segs[sg].p.in.qmask), __ldg(&segs[sg].p.in.qshift), *segs[sg].tma,
                                      v - __ldg(&segs[sg].cta0), raw_s, mb);
      });
}

// A one-tile C2C or C2R cols pass (as line_fft_tma) whose output planes go
// back out by TMA from the tile's buffer (output maps tmo; whole tiles, the
// host's tma_tile rules for the output).  Thread 0 waits until the stores
// have read the buffer before the CTA ends.
template <int LOGL, int C, int KIND>
__global__ void __launch_bounds__(Sched<LOGL>::T * C, min_ctas<Sched<LOGL>::T * C>())
line_fft_tma_bulk(const __grid_constant__ LineParams p, const __grid_constant__ TmaTile tm,
                  const __grid_constant__ TmaTile tmo) {
  constexpr int L = Sched<LOGL>::L;
  __shared__ __align__(8) uint64_t mbar;
  extern __shared__ __align__(1024) float2 smem_raw[];
  if (!tma_load_tile<C>(p, tm, blockIdx.x, &mbar, smem_raw)) return;
  line_fft_body<LOGL, C, true, KIND, false, false, 0, true, true>(p, blockIdx.x);
  if (threadIdx.x == 0) {
    const uint32_t s = smem_u32(smem_raw);
    pipe_store_plane<L, C>(p, &tmo.re, tmo.box_rows, blockIdx.x, s);
    pipe_store_plane<L, C>(p, &tmo.im, tmo.box_rows, blockIdx.x, s + (uint32_t)L * C * 4u);
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
  }
}

}  // namespace agb
