// Plane-fused complex passes (plane_fft): the last two axes of an N-D
// complex transform in one pass when a whole plane fits one CTA.
//
// A plane is D1 rows of D2 contiguous points (2^8 to 2^14 points, both sides
// 16 to 512), planes dense one after another: split planes at unit element
// stride (UNIT 1) or interleaved re,im pairs (UNIT 2, 8-byte accesses).  A CTA transforms PPC = max(1, 2^12 / (D1 D2)) consecutive planes
// with D1 D2 / 16 threads each (256 threads or more):
//   - rows phase: the PPC D1 rows as rows-mode lines of D2 points (thread t
//     of row r holds points t + T2 e), loaded as the rows kernels load them
//     (warp-staged 16-byte loads for rows of at most 128 points);
//   - handoff: every value goes through shared memory into its plane's cols
//     layout, element j = r of line k at j * CP + k with CP = D2 + D2 / 16
//     (D2 + 1 for 16-point rows).  A half-warp of the rows mapping covers
//     16 / T2 rows x T2 threads (T2 = D2 / 16), so r * CP + t runs over 16
//     distinct bank pairs;
//   - cols phase: the D2 columns of each plane as cols-mode lines of D1
//     points (a half-warp covers 16 adjacent columns at one row: consecutive
//     words), stored straight to HBM.
// The three-pass 3D transforms of such planes become two passes, and 2D
// transforms of such sizes one.  The rows phase reads the stage twiddles of
// D2 (p.tw), the cols phase those of D1 (p.tw2).
#pragma once
#include "line_fft.cuh"

namespace agb {

// The cols phase's view of one plane's part of the exchange buffer (element
// j of line c).
template <int D1, int D2>
struct PlaneCols {
  static constexpr int CP = D2 == 16 ? D2 + 1 : D2 + D2 / 16;
  static constexpr int FLOAT2S = D1 * CP;
  float2* s;
  __device__ __forceinline__ int idx(int c, int j) const { return j * CP + c; }
  __device__ __forceinline__ void put(int c, int j, float2 v) const { s[idx(c, j)] = v; }
  __device__ __forceinline__ float2 get(int c, int j) const { return s[idx(c, j)]; }
};

template <int LOG1, int LOG2>
struct PlaneShape {
  static constexpr int D1 = 1 << LOG1, D2 = 1 << LOG2, P = D1 * D2;
  static constexpr int PPC = P >= 4096 ? 1 : 4096 / P;   // planes per CTA
  static constexpr int NTP = P / 16, NT = PPC * NTP;      // threads per plane, per CTA
  using Rows = Smem<D2, PPC * D1, false>;
  using Cols = PlaneCols<D1, D2>;
  static constexpr int FLOAT2S =
      Rows::FLOAT2S > PPC * Cols::FLOAT2S ? Rows::FLOAT2S : PPC * Cols::FLOAT2S;
  static_assert(LOG1 >= 4 && LOG2 >= 4 && LOG1 <= 9 && LOG2 <= 9 && LOG1 + LOG2 >= 8 && LOG1 + LOG2 <= 14,
                "planes of 2^8 .. 2^14 points, sides 16 .. 512");
  static_assert(Sched<LOG1>::E == 16 && Sched<LOG2>::E == 16 && Sched<LOG2>::T * D1 == NTP &&
                    Sched<LOG1>::T * D2 == NTP,
                "16 points per thread in both phases");
};

// CTA `cta` of the launch: planes cta PPC .. cta PPC + PPC - 1 of the
// p.nlines / D1 planes; p.in / p.out give plane q's base (line_off of q),
// elements at unit stride, planes PPC apart contiguous (a multi-plane CTA
// reads its planes as PPC D1 contiguous rows).
template <int LOG1, int LOG2, int UNIT>
__device__ __forceinline__ void plane_body(const LineParams& p, long long cta) {
  static_assert(UNIT == 1 || UNIT == 2, "split planes or interleaved pairs");
  using PS = PlaneShape<LOG1, LOG2>;
  using S1 = Sched<LOG1>;
  using S2 = Sched<LOG2>;
  constexpr int D1 = PS::D1, D2 = PS::D2, T1 = S1::T, T2 = S2::T, PPC = PS::PPC, E = 16;
  extern __shared__ __align__(1024) float2 smem_raw[];
  typename PS::Rows smr{smem_raw};
  const int tid = threadIdx.x;
  const long long nplanes = p.nlines / D1, q0 = cta * PPC;
  const int here = (int)(nplanes - q0 < PPC ? nplanes - q0 : PPC);   // planes of this CTA

  // rows phase: row r (of the CTA's PPC D1 rows), thread t of the row
  const int r = tid / T2, t = tid % T2;
  const long long bin = line_off(p.in, q0);
  float2 v[E];
  bool staged = false;
  if constexpr (T2 <= AFFT_STAGE_T) {
    if (((reinterpret_cast<uintptr_t>(p.in.re + bin) | reinterpret_cast<uintptr_t>(p.in.im + bin)) & 15) == 0) {
      // the CTA's planes as PPC D1 contiguous lines of D2 points from the first one's base
      LineParams pr = p;
      pr.in.re = p.in.re + bin;
      pr.in.im = p.in.im + bin;
      pr.nlines = (long long)here * D1;
      if constexpr (UNIT == 1) rows_stage_in<LOG2, PPC * D1>(pr, 0, smr, v, t, r);
      else rows_stage_in_reals<LOG2, PPC * D1>(pr, 0, smr, v, t, r);   // pair lines: 2 D2 floats each
      staged = true;
    }
  }
  if (!staged) {
    if (r < here * D1) {
      if constexpr (UNIT == 1) {
        const float* pr = p.in.re + bin + r * D2 + t;
        const float* pi = p.in.im + bin + r * D2 + t;
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = make_float2(__ldg(pr + T2 * e), __ldg(pi + T2 * e));
      } else {
        const float* pz = p.in.re + bin + 2 * (r * D2 + t);
        if (!(reinterpret_cast<uintptr_t>(pz) & 7)) {
#pragma unroll
          for (int e = 0; e < E; e++) v[e] = __ldg(reinterpret_cast<const float2*>(pz) + T2 * e);
        } else {
#pragma unroll
          for (int e = 0; e < E; e++) v[e] = make_float2(__ldg(pz + 2 * T2 * e), __ldg(pz + 2 * T2 * e + 1));
        }
      }
    } else {
#pragma unroll
      for (int e = 0; e < E; e++) v[e] = make_float2(0.f, 0.f);
    }
  }
  if (p.inverse) {
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
  }
  run_stages<LOG2, PPC * D1, false, (T2 <= 32), 0, false, packed_bfly<LOG2, false>()>(v, t, r, p.tw, smr);

  // handoff to the cols layout of the row's plane (the rows phase's last
  // reads of the buffer are done everywhere first)
  __syncthreads();
  {
    const typename PS::Cols smc{smem_raw + (r / D1) * PS::Cols::FLOAT2S};
#pragma unroll
    for (int e = 0; e < E; e++) smc.put(t + T2 * e, r % D1, v[e]);
  }
  __syncthreads();
  // cols phase: plane g of the CTA, column c2, thread t2 of the column
  const int g = tid / PS::NTP, tl = tid % PS::NTP;
  const int c2 = tl % D2, t2 = tl / D2;
  const typename PS::Cols smc{smem_raw + g * PS::Cols::FLOAT2S};
#pragma unroll
  for (int e = 0; e < E; e++) v[e] = smc.get(c2, t2 + T1 * e);
  __syncthreads();   // every value is read before the cols stages write the buffer
  run_stages<LOG1, D2, true, false, 0, false, packed_bfly<LOG1, true>()>(v, t2, c2, p.tw2, smc);

  if (g < here) {
    if (p.inverse) {
#pragma unroll
      for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
    }
    const long long bout = line_off(p.out, q0 + g);
    if constexpr (UNIT == 1) {
      float* pr = p.out.re + bout + t2 * D2 + c2;
      float* pi = p.out.im + bout + t2 * D2 + c2;
#pragma unroll
      for (int e = 0; e < E; e++) {
        pr[T1 * D2 * e] = v[e].x;
        pi[T1 * D2 * e] = v[e].y;
      }
    } else {
      float* pz = p.out.re + bout + 2 * (t2 * D2 + c2);
      if (!(reinterpret_cast<uintptr_t>(pz) & 7)) {
#pragma unroll
        for (int e = 0; e < E; e++) reinterpret_cast<float2*>(pz)[T1 * D2 * e] = v[e];
      } else {
#pragma unroll
        for (int e = 0; e < E; e++) {
          pz[2 * T1 * D2 * e] = v[e].x;
          pz[2 * T1 * D2 * e + 1] = v[e].y;
        }
      }
    }
  }
}

template <int LOG1, int LOG2, int UNIT>
__global__ void __launch_bounds__(PlaneShape<LOG1, LOG2>::NT, min_ctas<PlaneShape<LOG1, LOG2>::NT>())
plane_fft(const LineParams p) {
  plane_body<LOG1, LOG2, UNIT>(p, blockIdx.x);
}

// Its queue form (as line_fft_grouped): one CTA per virtual CTA.
template <int LOG1, int LOG2, int UNIT>
__global__ void __launch_bounds__(PlaneShape<LOG1, LOG2>::NT, min_ctas<PlaneShape<LOG1, LOG2>::NT>())
plane_fft_grouped(const Segment* __restrict__ segs, const int* __restrict__ seg_of, long long total) {
  __shared__ LineParams sp;
  for (long long v = blockIdx.x; v < total; v += gridDim.x) {
    const int sg = __ldg(seg_of + v);
    __syncthreads();   // a previous iteration is done with sp and the buffer
    stage_params(sp, segs[sg].p);
    __syncthreads();
    plane_body<LOG1, LOG2, UNIT>(sp, v - segs[sg].cta0);
  }
}

}  // namespace agb
