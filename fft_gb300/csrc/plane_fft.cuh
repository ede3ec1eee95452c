// Plane-fused complex passes (plane_fft): the last two axes of an N-D
// complex transform in one pass when a whole plane fits one CTA.
//
// A plane is D1 rows of D2 contiguous points (2^12 to 2^14 points, both
// sides 32 to 512), stored densely at a per-plane base (split planes, unit
// element stride).  One CTA of D1 D2 / 16 threads transforms one plane:
//   - rows phase: the D1 rows as rows-mode lines of D2 points (thread t of
//     row r holds points t + T2 e), loaded as the rows kernels load them
//     (warp-staged 16-byte loads for rows of at most 128 points);
//   - handoff: every value goes through shared memory into the cols layout,
//     element j = r of line k at j * CP + k with CP = D2 + D2 / 16.  A
//     half-warp of the rows mapping covers 16 / T2 rows x T2 threads (T2 =
//     D2 / 16), so r * CP + t runs over 16 distinct bank pairs;
//   - cols phase: the D2 columns as cols-mode lines of D1 points (a warp
//     covers 32 adjacent columns at one row: 32 consecutive words), stored
//     straight to HBM as 128-byte row segments.
// The three-pass 3D transforms of such planes become two passes, and 2D
// transforms of such sizes one.  The rows phase reads the stage twiddles of
// D2 (p.tw), the cols phase those of D1 (p.tw2).
#pragma once
#include "line_fft.cuh"

namespace agb {

// The cols phase's view of the exchange buffer (element j of line c).
template <int D1, int D2>
struct PlaneCols {
  static constexpr int CP = D2 + D2 / 16;
  static constexpr int FLOAT2S = D1 * CP;
  float2* s;
  __device__ __forceinline__ int idx(int c, int j) const { return j * CP + c; }
  __device__ __forceinline__ void put(int c, int j, float2 v) const { s[idx(c, j)] = v; }
  __device__ __forceinline__ float2 get(int c, int j) const { return s[idx(c, j)]; }
};

template <int LOG1, int LOG2>
struct PlaneShape {
  static constexpr int D1 = 1 << LOG1, D2 = 1 << LOG2, P = D1 * D2, NT = P / 16;
  using Rows = Smem<D2, D1, false>;
  using Cols = PlaneCols<D1, D2>;
  static constexpr int FLOAT2S = Rows::FLOAT2S > Cols::FLOAT2S ? Rows::FLOAT2S : Cols::FLOAT2S;
  static_assert(LOG1 >= 5 && LOG2 >= 5 && LOG1 <= 9 && LOG2 <= 9 && LOG1 + LOG2 >= 12 && LOG1 + LOG2 <= 14,
                "planes of 2^12 .. 2^14 points, sides 32 .. 512");
  static_assert(Sched<LOG1>::E == 16 && Sched<LOG2>::E == 16 && Sched<LOG2>::T * D1 == NT &&
                    Sched<LOG1>::T * D2 == NT,
                "16 points per thread in both phases");
};

// Plane q of the launch: p.in / p.out give its base (line_off of plane q),
// elements at unit stride; p.nlines = planes * D1 (the rows).
template <int LOG1, int LOG2>
__device__ __forceinline__ void plane_body(const LineParams& p, long long q) {
  using PS = PlaneShape<LOG1, LOG2>;
  using S1 = Sched<LOG1>;
  using S2 = Sched<LOG2>;
  constexpr int D1 = PS::D1, D2 = PS::D2, T1 = S1::T, T2 = S2::T, E = 16;
  extern __shared__ __align__(1024) float2 smem_raw[];
  typename PS::Rows smr{smem_raw};
  typename PS::Cols smc{smem_raw};
  const int tid = threadIdx.x;

  // rows phase: row r, thread t of the row
  const int r = tid / T2, t = tid % T2;
  const long long bin = line_off(p.in, q);
  float2 v[E];
  bool staged = false;
  if constexpr (T2 <= AFFT_STAGE_T) {
    if (((reinterpret_cast<uintptr_t>(p.in.re + bin) | reinterpret_cast<uintptr_t>(p.in.im + bin)) & 15) == 0) {
      // the plane's rows as D1 contiguous lines of D2 points from its base
      LineParams pr = p;
      pr.in.re = p.in.re + bin;
      pr.in.im = p.in.im + bin;
      pr.nlines = D1;
      rows_stage_in<LOG2, D1>(pr, 0, smr, v, t, r);
      staged = true;
    }
  }
  if (!staged) {
    const float* pr = p.in.re + bin + r * D2 + t;
    const float* pi = p.in.im + bin + r * D2 + t;
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = make_float2(__ldg(pr + T2 * e), __ldg(pi + T2 * e));
  }
  if (p.inverse) {
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
  }
  run_stages<LOG2, D1, false, (T2 <= 32), 0, false, packed_bfly<LOG2, false>()>(v, t, r, p.tw, smr);

  // handoff to the cols layout (the rows phase's last reads of the buffer
  // are done everywhere first)
  __syncthreads();
#pragma unroll
  for (int e = 0; e < E; e++) smc.put(t + T2 * e, r, v[e]);
  __syncthreads();
  const int c2 = tid % D2, t2 = tid / D2;
#pragma unroll
  for (int e = 0; e < E; e++) v[e] = smc.get(c2, t2 + T1 * e);
  __syncthreads();   // every value is read before the cols stages write the buffer
  run_stages<LOG1, D2, true, false, 0, false, packed_bfly<LOG1, true>()>(v, t2, c2, p.tw2, smc);

  if (p.inverse) {
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = cswap(v[e]);
  }
  const long long bout = line_off(p.out, q);
  float* pr = p.out.re + bout + t2 * D2 + c2;
  float* pi = p.out.im + bout + t2 * D2 + c2;
#pragma unroll
  for (int e = 0; e < E; e++) {
    pr[T1 * D2 * e] = v[e].x;
    pi[T1 * D2 * e] = v[e].y;
  }
}

template <int LOG1, int LOG2>
__global__ void __launch_bounds__(PlaneShape<LOG1, LOG2>::NT, min_ctas<PlaneShape<LOG1, LOG2>::NT>())
plane_fft(const LineParams p) {
  plane_body<LOG1, LOG2>(p, blockIdx.x);
}

// Its queue form (as line_fft_grouped): one CTA per virtual CTA (plane).
template <int LOG1, int LOG2>
__global__ void __launch_bounds__(PlaneShape<LOG1, LOG2>::NT, min_ctas<PlaneShape<LOG1, LOG2>::NT>())
plane_fft_grouped(const Segment* __restrict__ segs, const int* __restrict__ seg_of, long long total) {
  __shared__ LineParams sp;
  for (long long v = blockIdx.x; v < total; v += gridDim.x) {
    const int sg = __ldg(seg_of + v);
    __syncthreads();   // a previous iteration is done with sp and the buffer
    stage_params(sp, segs[sg].p);
    __syncthreads();
    plane_body<LOG1, LOG2>(sp, v - segs[sg].cta0);
  }
}

}  // namespace agb
