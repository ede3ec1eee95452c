// Standalone real pre/post pass for real transforms whose half-length complex
// transform takes more than one pass (so the pass cannot be fused into a
// line kernel).  The algebra is afft's real_pass (onedim.hpp:1031-1108,
// multi.hpp:343-414):
//   forward  X[k] = a - i b,  a = (Z[k] + conj Z[L-k]) / 2,
//                             b = (Z[k] - conj Z[L-k]) w_k / 2,
//            X[0] = re Z0 + im Z0, X[L] = re Z0 - im Z0 (imaginary parts 0);
//   inverse  Z'[k] = a - i b, a = X[k] + conj X[L-k],
//                             b = (conj X[L-k] - X[k]) conj(w_k),
//            Z'[0] = (re X0 + re XL) + i (re X0 - re XL);
// with w_k = exp(-i pi k / L).  Each thread owns the pair (k, L-k) of one
// line, so the pass may run in place.
#include "line_fft.cuh"

namespace agb {

__device__ __forceinline__ float2 post_one(float2 s0, float2 s1, float2 w) {
  const float2 a = make_float2(0.5f * (s0.x + s1.x), 0.5f * (s0.y - s1.y));
  const float2 d = make_float2(0.5f * (s0.x - s1.x), 0.5f * (s0.y + s1.y));
  return cadd(a, cmul_negi(cmul(d, w)));
}

__device__ __forceinline__ float2 pre_one(float2 s0, float2 s1, float2 w) {
  const float2 a = cadd(s0, cconj(s1));
  const float2 b = cmul(csub(cconj(s1), s0), cconj(w));
  return cadd(a, cmul_negi(b));
}

__device__ __forceinline__ void real_pass_body(const RealPassParams& p, long long idx) {
  const long long half = p.L / 2 + 1;
  long long q, k;
  if (p.lines_fastest) {
    q = idx % p.nlines;
    k = idx / p.nlines;
  } else {
    k = idx % half;
    q = idx / half;
  }
  if (q >= p.nlines || k >= half) return;
  const long long L = p.L;
  const long long bi = line_off(p.in, q), bo = line_off(p.out, q);
  const long long ik = bi + k * p.in.es, iL = bi + (L - k) * p.in.es;
  const long long ok = bo + k * p.out.es, oL = bo + (L - k) * p.out.es;
  const float2 s0 = make_float2(p.in.re[ik], p.in.im[ik]);
  const float2 s1 = make_float2(p.in.re[iL], p.in.im[iL]);
  if (!p.inverse) {
    if (k == 0) {
      p.out.re[ok] = s0.x + s0.y;
      p.out.im[ok] = 0.f;
      p.out.re[oL] = s0.x - s0.y;
      p.out.im[oL] = 0.f;
      return;
    }
    const float2 xk = post_one(s0, s1, __ldg(p.rtw + k));
    const float2 xl = post_one(s1, s0, __ldg(p.rtw + (L - k)));
    p.out.re[ok] = xk.x;
    p.out.im[ok] = xk.y;
    if (L - k != k) {
      p.out.re[oL] = xl.x;
      p.out.im[oL] = xl.y;
    }
  } else {
    if (k == 0) {
      p.out.re[ok] = s0.x + s1.x;
      p.out.im[ok] = s0.x - s1.x;
      return;
    }
    const float2 zk = pre_one(s0, s1, __ldg(p.rtw + k));
    const float2 zl = pre_one(s1, s0, __ldg(p.rtw + (L - k)));
    p.out.re[ok] = zk.x;
    p.out.im[ok] = zk.y;
    if (L - k != k) {
      p.out.re[oL] = zl.x;
      p.out.im[oL] = zl.y;
    }
  }
}

__device__ __forceinline__ void copy_body(const CopyParams& p, long long idx) {
  if (idx >= p.nlines * p.len) return;
  const long long q = idx / p.len, i = idx - q * p.len;
  const long long a = line_off(p.in, q) + i * p.in.es;
  const long long b = line_off(p.out, q) + i * p.out.es;
  p.out.re[b] = p.in.re[a];
  p.out.im[b] = p.in.im[a];
}

__device__ __forceinline__ void real1_body(const RealPassParams& p, long long q) {
  if (q >= p.nlines) return;
  const long long i = line_off(p.in, q), o = line_off(p.out, q);
  if (!p.inverse) {
    p.out.re[o] = p.in.re[i];
    p.out.im[o] = 0.f;
  } else {
    p.out.re[o] = p.in.re[i];
  }
}

__global__ void real_pass_kernel(const RealPassParams p) {
  real_pass_body(p, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void copy_lines_kernel(const CopyParams p) {
  copy_body(p, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void real1_kernel(const RealPassParams p) {
  real1_body(p, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void elementwise_grouped(const EwSegment* __restrict__ segs, const int* __restrict__ seg_of,
                                    long long total) {
  for (long long v = blockIdx.x; v < total; v += gridDim.x) {
    const EwSegment& s = segs[__ldg(seg_of + v)];
    const long long idx = (v - s.blk0) * blockDim.x + threadIdx.x;
    if (s.type == EW_REAL) real_pass_body(s.rp, idx);
    else if (s.type == EW_COPY) copy_body(s.cp, idx);
    else real1_body(s.rp, idx);
  }
}

}  // namespace agb
