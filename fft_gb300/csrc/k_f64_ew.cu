// FP64 elementwise kernels (standalone real pass, line copy, size-1 real
// transform) and the FP64 kernel lookup.  Same algebra and thread mapping as
// the FP32 ones in real_pass.cu (afft's real_pass, onedim.hpp:1031-1108,
// multi.hpp:343-414): thread (q, k), k in [0, L/2], owns the pair (k, L-k)
// of line q, so the pass may run in place.
#include "kernels64.h"

namespace agb {

namespace {

__device__ __forceinline__ double2 post_one64(double2 s0, double2 s1, double2 w) {
  const double2 a = make_double2(0.5 * (s0.x + s1.x), 0.5 * (s0.y - s1.y));
  const double2 d = make_double2(0.5 * (s0.x - s1.x), 0.5 * (s0.y + s1.y));
  return zadd(a, zmul_negi(zmul(d, w)));
}

__device__ __forceinline__ double2 pre_one64(double2 s0, double2 s1, double2 w) {
  const double2 a = zadd(s0, zconj(s1));
  const double2 b = zmul(zsub(zconj(s1), s0), zconj(w));
  return zadd(a, zmul_negi(b));
}

__device__ __forceinline__ double ld64(const float* base, long long off) {
  return reinterpret_cast<const double*>(base)[off];
}

}  // namespace

__global__ void real_pass_kernel64(const RealPassParams p) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
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
  const double2* rtw = reinterpret_cast<const double2*>(p.rtw);
  const long long bi = line_off(p.in, q), bo = line_off(p.out, q);
  const long long ik = bi + k * p.in.es, iL = bi + (L - k) * p.in.es;
  const long long ok = bo + k * p.out.es, oL = bo + (L - k) * p.out.es;
  const double2 s0 = make_double2(ld64(p.in.re, ik), ld64(p.in.im, ik));
  const double2 s1 = make_double2(ld64(p.in.re, iL), ld64(p.in.im, iL));
  double* ore = reinterpret_cast<double*>(p.out.re);
  double* oim = reinterpret_cast<double*>(p.out.im);
  if (!p.inverse) {
    if (k == 0) {
      ore[ok] = s0.x + s0.y;
      oim[ok] = 0.0;
      ore[oL] = s0.x - s0.y;
      oim[oL] = 0.0;
      return;
    }
    const double2 xk = post_one64(s0, s1, rtw[k]);
    const double2 xl = post_one64(s1, s0, rtw[L - k]);
    ore[ok] = xk.x;
    oim[ok] = xk.y;
    if (L - k != k) {
      ore[oL] = xl.x;
      oim[oL] = xl.y;
    }
  } else {
    if (k == 0) {
      ore[ok] = s0.x + s1.x;
      oim[ok] = s0.x - s1.x;
      return;
    }
    const double2 zk = pre_one64(s0, s1, rtw[k]);
    const double2 zl = pre_one64(s1, s0, rtw[L - k]);
    ore[ok] = zk.x;
    oim[ok] = zk.y;
    if (L - k != k) {
      ore[oL] = zl.x;
      oim[oL] = zl.y;
    }
  }
}

__global__ void copy_lines_kernel64(const CopyParams p) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= p.nlines * p.len) return;
  const long long q = idx / p.len, i = idx - q * p.len;
  const long long a = line_off(p.in, q) + i * p.in.es;
  const long long b = line_off(p.out, q) + i * p.out.es;
  reinterpret_cast<double*>(p.out.re)[b] = ld64(p.in.re, a);
  reinterpret_cast<double*>(p.out.im)[b] = ld64(p.in.im, a);
}

__global__ void real1_kernel64(const RealPassParams p) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.nlines) return;
  const long long i = line_off(p.in, q), o = line_off(p.out, q);
  reinterpret_cast<double*>(p.out.re)[o] = ld64(p.in.re, i);
  if (!p.inverse) reinterpret_cast<double*>(p.out.im)[o] = 0.0;
}

bool get_line_kernel64(int logl, bool cols, int kind, bool tstore, LineKernel* out) {
  if (kind != LK_C2C && kind != LK_R2C && kind != LK_C2R) return false;
  if (!cols) return !tstore && get_rows64(logl, kind, out);
  return get_cols64(logl, kind, tstore, out);
}

}  // namespace agb
