// Plan construction and execution.
//
// Mapping of afft's composition (fft_internal.hpp) onto GPU passes:
//  - complex N-D (fft_internal.hpp:121-164): one pass per axis, last axis
//    first; the first pass reads src and writes dst, the others run in place
//    on dst.  An axis of length <= 2^14 (contiguous) or <= 2^11 (strided) is
//    one pass; a longer axis takes two passes (four-step: L = L1*L2, a pass
//    over L1 with the W_L^{t2 k1} twiddle fused into its epilogue, then a pass
//    over L2), through a plan-owned scratch buffer.  Contiguous complex axes
//    of 2^21 and 2^22 points take three: L1 = 256, then the L2 pass as a
//    strided four-step of its own.
//  - inverse (fft_internal.hpp:166-198): the same passes with re/im swapped
//    on load and store.
//  - real 1D (onedim.hpp:1110-1254): the n/2-point complex transform of the
//    interleaved view with the real post/pre pass fused into the kernel; for
//    n/2 > 2^14 the four-step passes plus a standalone real pass.
//  - real N-D (fft_internal.hpp:200-493): dim 0 is halved; the halved dim-0
//    pass with the fused real pass, and the complex (N-1)-D transform of each
//    of the d0/2+1 planes in place on dst (reverse order for the inverse,
//    through scratch).
#include <cuda_fp16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>

#include "plan.h"

#include <cudaTypedefs.h>
#include "line_fft64.cuh"

namespace agb {

// ---------------------------------------------------------------------------
// twiddles: exp(-2 pi i m / N) in FP64 with exact quadrant/octant symmetry,
// rounded once to FP32
// ---------------------------------------------------------------------------
static void unit_root(long long m, long long N, double* c, double* s) {
  m %= N;
  if (m < 0) m += N;
  if (N == 1 || m == 0) { *c = 1.0; *s = 0.0; return; }
  if (N == 2) { *c = -1.0; *s = 0.0; return; }
  const double pi = 3.14159265358979323846;
  double cc, ss;  // cos/sin of +2 pi m / N
  if (N % 4 == 0) {
    long long q4 = N / 4;
    long long quad = m / q4, r = m % q4;
    double c0, s0;
    if (N % 8 == 0 && r > N / 8) {
      long long r2 = q4 - r;  // complementary angle
      double a = 2.0 * pi * (double)r2 / (double)N;
      c0 = std::sin(a);
      s0 = std::cos(a);
    } else {
      double a = 2.0 * pi * (double)r / (double)N;
      c0 = std::cos(a);
      s0 = std::sin(a);
    }
    if (r == 0) { c0 = 1.0; s0 = 0.0; }
    switch (quad) {
      case 0: cc = c0; ss = s0; break;
      case 1: cc = -s0; ss = c0; break;
      case 2: cc = -c0; ss = -s0; break;
      default: cc = s0; ss = -c0; break;
    }
  } else {
    double a = 2.0 * pi * (double)m / (double)N;
    cc = std::cos(a);
    ss = std::sin(a);
  }
  *c = cc;
  *s = -ss;  // forward sign
}

static float2 root_f(long long m, long long N) {
  double c, s;
  unit_root(m, N, &c, &s);
  return make_float2((float)c, (float)s);
}

struct TableCache {
  std::mutex mu;
  std::map<std::pair<int, long long>, void*> tables;  // (device * 8 + type, key)
};
static TableCache& tcache() {
  static TableCache* c = new TableCache();  // never destroyed: outlives static plans
  return *c;
}

// Device copy of table (type, key) on the current device; `make` builds the
// host table (a std::vector of float2 or double2) on the first request only.
template <class F>
static auto cached_table(int type, long long key, F make) -> const typename decltype(make())::value_type* {
  using V = typename decltype(make())::value_type;
  int dev = 0;
  cudaGetDevice(&dev);
  auto& C = tcache();
  std::lock_guard<std::mutex> g(C.mu);
  auto id = std::make_pair(dev * 8 + type, key);
  auto it = C.tables.find(id);
  if (it != C.tables.end()) return static_cast<const V*>(it->second);
  const std::vector<V> host = make();
  V* d = nullptr;
  size_t bytes = std::max<size_t>(host.size(), 1) * sizeof(V);
  if (cudaMalloc(&d, bytes) != cudaSuccess) return nullptr;
  // a copy from pageable memory may return before its DMA lands, and plans
  // launch on streams that need not order after the default stream: wait
  // once, before the table is published
  if (!host.empty() && (cudaMemcpy(d, host.data(), host.size() * sizeof(V), cudaMemcpyHostToDevice) != cudaSuccess ||
                        cudaStreamSynchronize(0) != cudaSuccess)) {
    cudaGetLastError();
    cudaFree(d);
    return nullptr;
  }
  C.tables[id] = d;
  return d;
}

// Stage twiddles of the line kernel for L = 2^logl: for each stage s with
// NS = ns(s) > 1 and radix R, entries [(r-1)*NS + k] = W_{NS R}^{r k}.
template <int LOGL>
static std::vector<float2> stage_table() {
  using S = Sched<LOGL>;
  std::vector<float2> t(S::twsize());
  for (int s = 0; s < S::NSTAGES; s++) {
    int ns = S::ns(s), R = S::radix(s);
    if (ns == 1) continue;
    int off = S::twoff(s);
    for (int r = 1; r < R; r++)
      for (int k = 0; k < ns; k++) t[off + (r - 1) * ns + k] = root_f((long long)r * k, (long long)ns * R);
  }
  return t;
}

template <int... Ls>
static std::vector<float2> stage_table_dispatch(int logl, std::integer_sequence<int, Ls...>) {
  std::vector<float2> out;
  ((logl == Ls ? (void)(out = stage_table<Ls>()) : (void)0), ...);
  return out;
}

std::vector<float2> stage_table_host(int logl) {
  return stage_table_dispatch(logl, std::make_integer_sequence<int, 15>{});
}

void fourstep_table_host(long long N, std::vector<float2>* hi, std::vector<float2>* lo, int* lo_bits) {
  int lb = 0;
  while ((1LL << (2 * lb)) < N) lb++;
  long long nlo = 1LL << lb, nhi = (N + nlo - 1) / nlo;
  hi->resize(nhi);
  lo->resize(nlo);
  for (long long j = 0; j < nhi; j++) (*hi)[j] = root_f(j * nlo, N);
  for (long long j = 0; j < nlo; j++) (*lo)[j] = root_f(j, N);
  *lo_bits = lb;
}

const float2* stage_twiddles(int logl) {
  return cached_table(0, logl, [&] { return stage_table_dispatch(logl, std::make_integer_sequence<int, 15>{}); });
}

const float2* real_twiddles(long long L) {
  return cached_table(1, L, [&] {
    std::vector<float2> t(L);
    for (long long k = 0; k < L; k++) t[k] = root_f(k, 2 * L);
    return t;
  });
}

// The real 32x32 DFT-16 matrix M = [[Wr, Wi], [-Wi, Wr]] of the TC form,
// stored [n][k] (K-major B operand), as Mh = fp16(M) then
// Ml = fp16((M - Mh) * 2048); entries computed in FP64.
const __half* tc_matrix_table() {
  int dev = 0;
  cudaGetDevice(&dev);
  static std::mutex mu;
  static std::map<int, __half*> tabs;
  std::lock_guard<std::mutex> g(mu);
  auto it = tabs.find(dev);
  if (it != tabs.end()) return it->second;
  std::vector<__half> h(2048);
  for (int kk = 0; kk < 32; kk++)      // K index: input row (re 0..15, im 16..31)
    for (int nn = 0; nn < 32; nn++) {  // N index: output (re 0..15, im 16..31)
      int n = kk & 15, k = nn & 15;
      double c, sn;
      unit_root((long long)n * k, 16, &c, &sn);  // exp(-2 pi i nk/16) = c + i sn
      double m;
      if (kk < 16 && nn < 16) m = c;            // Xr -> Yr
      else if (kk >= 16 && nn < 16) m = -sn;    // Xi -> Yr
      else if (kk < 16) m = sn;                 // Xr -> Yi
      else m = c;                               // Xi -> Yi
      __half mh = __double2half(m);
      h[nn * 32 + kk] = mh;
      h[1024 + nn * 32 + kk] = __double2half((m - (double)__half2float(mh)) * 2048.0);
    }
  __half* d = nullptr;
  if (cudaMalloc(&d, 2048 * sizeof(__half)) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (cudaMemcpy(d, h.data(), 2048 * sizeof(__half), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaStreamSynchronize(0) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d);
    return nullptr;
  }
  tabs[dev] = d;
  return d;
}

int* tc_error_word() {
  int dev = 0;
  cudaGetDevice(&dev);
  static std::mutex mu;
  static std::map<int, int*> words;
  std::lock_guard<std::mutex> g(mu);
  auto it = words.find(dev);
  if (it != words.end()) return it->second;
  int* d = nullptr;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (cudaMemset(d, 0, sizeof(int)) != cudaSuccess || cudaStreamSynchronize(0) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d);
    return nullptr;
  }
  words[dev] = d;
  return d;
}

void fourstep_tables(long long N, const float2** hi, const float2** lo, int* lo_bits) {
  int lb = 0;
  while ((1LL << (2 * lb)) < N) lb++;  // lo covers about sqrt(N) entries
  const long long nlo = 1LL << lb, nhi = (N + nlo - 1) / nlo;
  *hi = cached_table(2, N, [&] {
    std::vector<float2> th(nhi);
    for (long long j = 0; j < nhi; j++) th[j] = root_f(j * nlo, N);
    return th;
  });
  *lo = cached_table(3, N, [&] {
    std::vector<float2> tl(nlo);
    for (long long j = 0; j < nlo; j++) tl[j] = root_f(j, N);
    return tl;
  });
  *lo_bits = lb;
}

std::vector<float2> fourstep_full_table_host(long long N, long long L2) {
  const long long L1 = N / L2;
  std::vector<float2> t(N);
  for (long long j = 0; j < L2; j++)
    for (long long k = 0; k < L1; k++) t[j * L1 + k] = root_f(j * k, N);
  return t;
}

const float2* fourstep_full_table(long long N, long long L2) {
  if (N > kFullTableMax) return nullptr;
  int l2 = 0;
  while ((1LL << l2) < L2) l2++;
  return cached_table(4, (N << 6) | l2, [&] { return fourstep_full_table_host(N, L2); });
}

// FP64 tables: the same roots without the rounding to FP32
static double2 root_d(long long m, long long N) {
  double c, s;
  unit_root(m, N, &c, &s);
  return make_double2(c, s);
}

template <int LOGL>
static std::vector<double2> stage_table64() {
  using S = Sched64<LOGL>;
  std::vector<double2> t(S::twsize());
  for (int s = 0; s < S::NSTAGES; s++) {
    int ns = S::ns(s), R = S::radix(s);
    if (ns == 1) continue;
    int off = S::twoff(s);
    for (int r = 1; r < R; r++)
      for (int k = 0; k < ns; k++) t[off + (r - 1) * ns + k] = root_d((long long)r * k, (long long)ns * R);
  }
  return t;
}

template <int... Ls>
static std::vector<double2> stage_table64_dispatch(int logl, std::integer_sequence<int, Ls...>) {
  std::vector<double2> out;
  ((logl == Ls ? (void)(out = stage_table64<Ls>()) : (void)0), ...);
  return out;
}

std::vector<double2> stage_table64_host(int logl) {
  return stage_table64_dispatch(logl, std::make_integer_sequence<int, ROWS_MAX_LOG64 + 1>{});
}

const double2* stage_twiddles64(int logl) {
  return cached_table(5, logl, [&] { return stage_table64_host(logl); });
}

const double2* real_twiddles64(long long L) {
  return cached_table(6, L, [&] {
    std::vector<double2> t(L);
    for (long long k = 0; k < L; k++) t[k] = root_d(k, 2 * L);
    return t;
  });
}

const double2* fourstep_full_table64(long long N, long long L2) {
  int l2 = 0;
  while ((1LL << l2) < L2) l2++;
  return cached_table(7, (N << 6) | l2, [&] {
    const long long L1 = N / L2;
    std::vector<double2> t(N);
    for (long long j = 0; j < L2; j++)
      for (long long k = 0; k < L1; k++) t[j * L1 + k] = root_d(j * k, N);
    return t;
  });
}

// ---------------------------------------------------------------------------
// plan building
// ---------------------------------------------------------------------------
static int ilog2ll(long long v) {
  int r = 0;
  while ((1LL << r) < v) r++;
  return r;
}

// A complex array view: element i of re at re.off + i*unit (floats), im
// likewise.  bstride = complex elements between consecutive outer blocks.
struct View {
  Ref re, im;
  long long unit = 1;
};

static View split_view(int bre, int bim, long long off = 0) {
  View v;
  v.re = {bre, off};
  v.im = {bim, off};
  v.unit = 1;
  return v;
}
static View inter_view(int b, long long off = 0) {  // re,im pairs in one array
  View v;
  v.re = {b, off};
  v.im = {b, off + 1};
  v.unit = 2;
  return v;
}

// Four-step split L = L1 * L2: L1 (the first, transposing pass) takes the
// larger half for odd log2 L (measured the better split on GB300).
#define AFFT_L1(logl) (((logl) + 1) / 2)
// cols passes take their TMA-fed kernels where one exists (0: LSU loads only)
#ifndef AFFT_COLS_TMA
#define AFFT_COLS_TMA 1
#endif
// ... and of the 2048-point passes, per kind.  There one CTA fills an SM
// (128 KB tiles), so a TMA-loaded tile cannot overlap another CTA's work:
// measured on GB300, the C2C pass is 3% slower with TMA (2048^2 x 8: 0.2628
// vs 0.2710 ms), the unsplit R2C pass 7-9% slower than the split LSU form
// (4096^2 r2c: 0.0826 vs 0.0897 ms), 4-line tiles slower still; the C2R
// pass, whose LSU form reads every bin twice, 9% faster (4096^2 c2r: 0.0959
// vs 0.0867 ms).
#ifndef AFFT_TMA_C2C11
#define AFFT_TMA_C2C11 0
#endif
// 1D complex axes from 2^AFFT_THREE_PASS_LOG points run as three passes
#ifndef AFFT_THREE_PASS_LOG
#define AFFT_THREE_PASS_LOG 21
#endif
// ... and of the transposing-store passes (four-step pass A)
#ifndef AFFT_TMA_TSTORE
#define AFFT_TMA_TSTORE 1
#endif
// ... and of complex cols passes over interleaved input pairs
#ifndef AFFT_TMA_PAIRS
#define AFFT_TMA_PAIRS 1
#endif
#ifndef AFFT_TMA_R2C11
#define AFFT_TMA_R2C11 0
#endif
#ifndef AFFT_TMA_C2R11
#define AFFT_TMA_C2R11 1
#endif
// 1024- and 2048-point cols passes over split planes: the persistent
// TMA-pipelined kernels (one or two CTAs per SM, each loading its next tile
// under the current one's stages)
#ifndef AFFT_COLS_PIPE
#define AFFT_COLS_PIPE 1
#endif
// the last two axes of complex N-D transforms in one plane-fused pass
// (plane_fft) where a plane of 2^8 .. 2^14 points fits one CTA
#ifndef AFFT_PLANE
#define AFFT_PLANE 1
#endif


static IOSpec io(const View& v, long long es, long long lo, long long hi, int qshift, long long qmask) {
  IOSpec s;
  s.re = v.re;
  s.im = v.im;
  s.es = es * v.unit;
  s.lo = lo * v.unit;
  s.hi = hi * v.unit;
  s.qshift = qshift;
  s.qmask = qmask;
  return s;
}

struct Builder {
  Plan& P;
  bool ok = true;
  std::string err;
  long long scr_base = 0;  // floats of scratch reserved below four-step use
  bool dry = false;        // describe only: no device tables
  Tuning tune;             // plan variant
  const bool f64;          // FP64 kernels and tables (afft_64_*)
  explicit Builder(Plan& p, bool d = false) : P(p), dry(d), f64(p.f64()) {}

  // longest line one rows-mode CTA transforms
  int rows_max() const { return f64 ? ROWS_MAX_LOG64 : ROWS_MAX_LOG; }

  // four-step split of an axis of 2^logl points: L1 takes the larger half
  // (measured the better default on GB300 for odd logl), or the smaller one
  // when tuned so
  int l1_of(int logl) const { return tune.split ? logl / 2 : AFFT_L1(logl); }

  void fail(const std::string& m) {
    if (ok) err = m;
    ok = false;
  }

  void need_scratch(long long elems) { P.scratch_elems = std::max(P.scratch_elems, elems); }

  void line(int kind, bool cols, bool tstore, int logl, const IOSpec& in, const IOSpec& out,
            long long nlines, bool inverse, long long tw_n = 0, long long tw_qmask = 0,
            int tw_qshift = 0, long long real_L = 0) {
    if (!ok) return;
    if (tw_n && !cols) {
      fail("four-step twiddles need a cols pass");
      return;
    }
    Op op;
    op.type = OP_LINE;
    bool tc = P.form == FORM_TC && kind == LK_C2C && get_tc_kernel(logl, cols, tstore, &op.k);
    const bool unit = !f64 && !cols && !tstore && kind == LK_C2C && in.es == 1 && out.es == 1;
    // interleaved pairs (im right after re in the same array) with unit pair strides
    auto pairs = [](const IOSpec& v) { return v.es == 2 && v.re.buf == v.im.buf && v.im.off == v.re.off + 1; };
    const bool iunit = !f64 && !cols && !tstore && kind == LK_C2C && !tc && pairs(in) && pairs(out);
    // cols c2c on interleaved pairs (im right after re, every stride even,
    // so a line's pairs are 8-byte aligned when its array is): 8-byte accesses
    auto cpair = [](const IOSpec& v) {
      return v.re.buf == v.im.buf && v.im.off == v.re.off + 1 && v.es % 2 == 0 && v.lo % 2 == 0 && v.hi % 2 == 0;
    };
    const int cpairs = (!f64 && cols && kind == LK_C2C && !tc) ? (cpair(in) ? 1 : 0) | (cpair(out) ? 2 : 0) : 0;
    // rows real kernels whose real side is pairs with unit pair stride: every
    // C2R of 256 points and more (4-8% faster); R2C only from 4096 points
    // (shorter R2C pair variants spill and measured 0-6% slower)
    const bool rpairs = !f64 && !cols && !tstore &&
                        ((kind == LK_R2C && pairs(in) && logl >= 12) || (kind == LK_C2R && pairs(out)));
    if (f64) {
      if (!get_line_kernel64(logl, cols, kind, tstore, &op.k)) {
        fail("no FP64 kernel for this line length");
        return;
      }
    } else if (unit && get_rows_c2c_unit(logl, tc, &op.k)) {
      // same kernel with compile-time element offsets
    } else if (iunit && get_rows_c2c_iunit(logl, &op.k)) {
      // the same on interleaved pairs
    } else if (cpairs && get_cols_c2c_pairs(logl, tstore, cpairs, &op.k)) {
      // cols passes over interleaved pairs
    } else if (!f64 && kind == LK_R2C_PAIRED && cpair(in) && get_r2c_paired_pairs(logl, &op.k)) {
      // the paired R2C pass over pairs
    } else if (!f64 && kind == LK_C2R_PAIRED && cpair(out) && get_c2r_paired_pairs(logl, &op.k)) {
      // the paired C2R pass into pairs
    } else if (rpairs && get_rows_real_pairs(logl, kind, &op.k)) {
      // rows real passes with float2 accesses on the real side
    } else if (!tc && !get_line_kernel(logl, cols, kind, tstore, &op.k)) {
      fail("no kernel for this line length");
      return;
    }
    // cols passes over split planes: the variant with TMA-loaded input tiles
    // (taken at launch when the bound arrays meet its alignment rules)
    if (AFFT_COLS_TMA && !f64 && !tc && cols && !tune.cols_lsu && (kind == LK_C2C || kind == LK_R2C || kind == LK_C2R) &&
        (!tstore || kind == LK_C2C) && (cpairs == 0 || (cpairs & 1))) {
      LineKernel kt;
      // (the 2048-point R2C pass: unsplit, one CTA per tile, replacing the
      // split form; its LSU kernel is the fallback)
      // (kernels compare by shape: each translation unit has its own host
      // stub of a template kernel, so their addresses differ)
      const bool want = logl < 11 || (kind == LK_C2C ? AFFT_TMA_C2C11 : kind == LK_R2C ? AFFT_TMA_R2C11 : AFFT_TMA_C2R11);
      const bool have = (cpairs & 1) ? AFFT_TMA_PAIRS && get_cols_tma_pairs(logl, tstore, cpairs, &kt)
                        : tstore   ? AFFT_TMA_TSTORE && get_cols_tma_tstore(logl, &kt)
                                   : get_cols_tma(logl, kind, &kt);
      if (want && have && kt.kind == op.k.kind && kt.logl == op.k.logl && kt.unit == op.k.unit &&
          kt.tstore == op.k.tstore && !op.k.tc)
        op.k = kt;
    }
    // 1024- and 2048-point cols passes: the persistent pipelined form (C2C
    // and C2R; the unsplit R2C and the transposing store only in their opt-in
    // builds); at launch the one-tile-per-CTA kernels of the same shape run
    // where the bound arrays miss the TMA rules or, at 1024 points, the tiles
    // are too few
    LineKernel kp;
    if (AFFT_COLS_PIPE && !f64 && !tc && cols && cpairs == 0 && !tune.cols_lsu && !tune.no_pipe && !op.k.tc &&
        (tstore ? kind == LK_C2C && get_cols_pipe_tstore(logl, &kp)
                : (kind == LK_C2C || (kind == LK_R2C && AFFT_PIPE_R2C) || kind == LK_C2R) &&
                      get_cols_pipe(logl, kind, &kp)) &&
        kp.kind == op.k.kind && kp.logl == op.k.logl && kp.tstore == op.k.tstore)
      op.k = kp;
    // another tile width for 256- and 512-point complex cols passes, when tuned so
    LineKernel ka;
    if (tune.cols_c && !f64 && !tc && cols && !tstore && !cpairs && kind == LK_C2C &&
        get_cols_c2c_alt(logl, tune.cols_c, &ka)) {
      op.k = ka;
      if (!AFFT_COLS_TMA || tune.cols_lsu) op.k.tma = nullptr, op.k.grouped_tma = nullptr, op.k.tma_bulk = nullptr;
    }
    op.in = in;
    op.out = out;
    op.p.nlines = nlines;
    op.p.inverse = inverse ? 1 : 0;
    op.real_L = real_L;
    op.p.tw_n = tw_n;
    op.p.tw_qmask = tw_qmask;
    op.p.tw_qshift = tw_qshift;
    if (!dry) {
      if (op.k.smem > 48 * 1024 &&
          (cudaFuncSetAttribute((const void*)op.k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)op.k.smem) != cudaSuccess ||
           (op.k.tma && cudaFuncSetAttribute((const void*)op.k.tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)op.k.smem) != cudaSuccess) ||
           (op.k.tma_bulk && cudaFuncSetAttribute((const void*)op.k.tma_bulk,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)op.k.smem) != cudaSuccess) ||
           (op.k.pipe && cudaFuncSetAttribute((const void*)op.k.pipe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)op.k.pipe_smem) != cudaSuccess))) {
        cudaGetLastError();
        fail("kernel shared memory configuration failed");
        return;
      }
      if (op.k.paired_tma && op.k.paired_smem > 48 * 1024 &&
          cudaFuncSetAttribute((const void*)op.k.paired_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)op.k.paired_smem) != cudaSuccess) {
        cudaGetLastError();
        fail("kernel shared memory configuration failed");
        return;
      }
      if (op.k.tma || op.k.paired_tma) {
        op.p.err = tc_error_word();
        if (!op.p.err) {
          fail("error word allocation failed");
          return;
        }
        P.has_tma = true;
      }
      if (f64) {
        // the FP64 kernels read double2 tables through the same fields
        op.p.tw = reinterpret_cast<const float2*>(stage_twiddles64(op.k.stage_logl));
        if (tw_n) op.p.tw_full = reinterpret_cast<const float2*>(fourstep_full_table64(tw_n, tw_qmask + 1));
        if (real_L) op.p.rtw = reinterpret_cast<const float2*>(real_twiddles64(real_L));
      } else {
        op.p.tw = stage_twiddles(op.k.stage_logl);
        if (tw_n) {
          fourstep_tables(tw_n, &op.p.tw_hi, &op.p.tw_lo, &op.p.tw_lo_bits);
          op.p.tw_full = fourstep_full_table(tw_n, tw_qmask + 1);
        }
        if (real_L) op.p.rtw = real_twiddles(real_L);
      }
      if (tc) {
        op.p.tc_b = tc_matrix_table();
        op.p.err = tc_error_word();
        if (!op.p.tc_b || !op.p.err) {
          fail("tensor-core table allocation failed");
          return;
        }
      }
    }
    op.grid = (nlines + op.k.lines_per_cta - 1) / op.k.lines_per_cta * op.k.halves;
    op.threads = op.k.threads;
    op.smem = op.k.smem;
    if (!dry && (!op.p.tw || (tw_n && !f64 && (!op.p.tw_hi || !op.p.tw_lo)) ||
                 (tw_n && (f64 || tw_n <= kFullTableMax) && !op.p.tw_full) || (real_L && !op.p.rtw))) {
      fail("twiddle table allocation failed");
      return;
    }
    P.ops.push_back(op);
  }

  // Whether the last two axes (d1 rows of d2 points) of a complex N-D
  // transform from A to B take one plane-fused pass: both views split or
  // both interleaved pairs, the shapes plane_fft is built for, FP32 (the
  // plane pass is plain FP32 in the tensor-core form too, as every pass
  // without a tensor-core kernel), not tuned off.
  // A 2^14-point plane fills an SM with one CTA, so below 256 planes per
  // launch the per-axis passes keep more of the GPU busy (32 planes of
  // 128 x 128: 0.0184 vs 0.0198 ms) unless the plane is asked for (the
  // queue, whose grouped launches gather the planes of many transforms).
  bool plane_fits(long long d1, long long d2, long long count, const View& A, const View& B) const {
    if (!AFFT_PLANE || f64 || tune.no_plane == 1 || A.unit != B.unit || A.unit > 2) return false;
    if (d1 < 2 || d2 < 2 || (d1 & (d1 - 1)) || (d2 & (d2 - 1))) return false;
    if (tune.no_plane == 0 && d1 * d2 >= (1LL << 14) && count < 256) return false;
    LineKernel k;
    return get_plane_kernel(ilog2ll(d1), ilog2ll(d2), (int)A.unit, &k);
  }

  // `count` dense planes of d1 rows x d2 points from A to B (one or, for
  // planes under 2^12 points, several per CTA).
  void plane(long long d1, long long d2, long long count, const View& A, const View& B, bool inverse) {
    if (!ok) return;
    Op op;
    op.type = OP_LINE;
    const int log1 = ilog2ll(d1), log2 = ilog2ll(d2);
    if (A.unit != B.unit || !get_plane_kernel(log1, log2, (int)A.unit, &op.k)) {
      fail("no plane kernel for this shape");
      return;
    }
    const long long pl = d1 * d2;
    op.in = io(A, 1, 0, pl, 0, 0);
    op.out = io(B, 1, 0, pl, 0, 0);
    op.p.nlines = count * d1;   // rows; the grid is one CTA per plane
    op.p.inverse = inverse ? 1 : 0;
    if (!dry) {
      if (op.k.smem > 48 * 1024 &&
          cudaFuncSetAttribute((const void*)op.k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)op.k.smem) !=
              cudaSuccess) {
        cudaGetLastError();
        fail("kernel shared memory configuration failed");
        return;
      }
      op.p.tw = stage_twiddles(log2);
      op.p.tw2 = stage_twiddles(log1);
      if (!op.p.tw || !op.p.tw2) {
        fail("twiddle table allocation failed");
        return;
      }
    }
    const long long ppc = op.k.lines_per_cta / d1;   // planes per CTA
    op.grid = (count + ppc - 1) / ppc;
    op.threads = op.k.threads;
    op.smem = op.k.smem;
    P.ops.push_back(op);
  }

  void real_pass(const IOSpec& in, const IOSpec& out, long long nlines, long long L, bool inverse,
                 bool lines_fastest) {
    if (!ok) return;
    Op op;
    op.type = OP_REAL;
    op.in = in;
    op.out = out;
    op.rp.nlines = nlines;
    op.rp.L = L;
    op.rp.rtw = dry ? nullptr : (f64 ? reinterpret_cast<const float2*>(real_twiddles64(L)) : real_twiddles(L));
    op.rp.inverse = inverse ? 1 : 0;
    op.rp.lines_fastest = lines_fastest ? 1 : 0;
    op.threads = 256;
    op.grid = (nlines * (L / 2 + 1) + 255) / 256;
    if (!dry && !op.rp.rtw) fail("twiddle table allocation failed");
    P.ops.push_back(op);
  }

  void copy(const IOSpec& in, const IOSpec& out, long long nlines, long long len) {
    if (!ok) return;
    Op op;
    op.type = OP_COPY;
    op.in = in;
    op.out = out;
    op.cp.nlines = nlines;
    op.cp.len = len;
    op.threads = 256;
    op.grid = (nlines * len + 255) / 256;
    P.ops.push_back(op);
  }

  void real1(bool forward, long long count) {
    if (!ok) return;
    Op op;
    op.type = OP_REAL1;
    op.rp.nlines = count;
    op.rp.inverse = forward ? 0 : 1;
    if (forward) {
      op.in = io(split_view(B_SRC_RE, B_SRC_RE), 1, 0, 1, 0, 0);
      op.out = io(P.format == 1 ? inter_view(B_DST_RE) : split_view(B_DST_RE, B_DST_IM), 1, 0, 1, 0, 0);
    } else {
      op.in = io(P.format == 1 ? inter_view(B_SRC_RE) : split_view(B_SRC_RE, B_SRC_IM), 1, 0, 1, 0, 0);
      op.out = io(split_view(B_DST_RE, B_DST_RE), 1, 0, 1, 0, 0);
    }
    op.threads = 256;
    op.grid = (count + 255) / 256;
    P.ops.push_back(op);
  }

  // Complex transform along the middle axis of a dense (outer, L, inner)
  // array, from view A to view B (may be the same).  a_bs / b_bs: complex
  // elements between outer blocks (default L*inner).
  void axis(long long outer, long long L, long long inner, const View& A, const View& B,
            bool inverse, long long a_bs = 0, long long b_bs = 0) {
    if (!ok) return;
    if (a_bs == 0) a_bs = L * inner;
    if (b_bs == 0) b_bs = L * inner;
    int logl = ilog2ll(L);
    if (inner == 1) {
      if (logl <= rows_max()) {
        line(LK_C2C, false, false, logl, io(A, 1, 0, a_bs, 0, 0), io(B, 1, 0, b_bs, 0, 0), outer, inverse);
        return;
      }
      // four-step along a contiguous axis; from 2^AFFT_THREE_PASS_LOG points
      // (FP32) pass A takes 256 points and pass B becomes a strided
      // four-step of its own: three passes of 64 to 256 points instead of two
      // of 1024 / 2048, whose one-CTA-per-SM tiles run at about half the
      // rate per pass
      const bool three =
          !f64 && (tune.passes == 3 ? logl >= 20 : tune.passes == 2 ? false : logl >= AFFT_THREE_PASS_LOG);
      int l1 = three ? 8 : l1_of(logl), l2 = logl - l1;
      if (l1 > COLS_MAX_LOG || (l2 > COLS_MAX_LOG && !three)) {
        fail("axis longer than 2^22 points");
        return;
      }
      long long L1 = 1LL << l1, L2 = 1LL << l2;
      View S = split_view(B_SCR, B_SCR, scr_base);
      S.im.off = scr_base + outer * L;  // scratch: re block then im block
      need_scratch(scr_base + 2 * outer * L);
      // pass A: lines (o, t2), points t1 -> Y[o][t2][k1] (transposed store)
      line(LK_C2C, true, true, l1, io(A, L2, 1, a_bs, l2, L2 - 1), io(S, 1, L1, L, l2, L2 - 1),
           outer * L2, inverse, L, L2 - 1, 0);
      // pass B: lines (o, k1), points t2 -> X[o][k1 + L1 k2]
      if (l2 > COLS_MAX_LOG) {
        // the same as a strided axis: (outer, L2, inner L1) from Y to X,
        // its own scratch above Y's
        const long long save = scr_base;
        scr_base += 2 * outer * L;
        axis(outer, L2, L1, S, B, inverse, L, b_bs);
        scr_base = save;
        return;
      }
      line(LK_C2C, true, false, l2, io(S, L1, 1, L, l1, L1 - 1), io(B, L1, 1, b_bs, l1, L1 - 1),
           outer * L1, inverse);
      return;
    }
    int lin = ilog2ll(inner);
    if (logl <= COLS_MAX_LOG) {
      line(LK_C2C, true, false, logl, io(A, inner, 1, a_bs, lin, inner - 1),
           io(B, inner, 1, b_bs, lin, inner - 1), outer * inner, inverse);
      return;
    }
    // four-step along a strided axis
    int l1 = l1_of(logl), l2 = logl - l1;
    if (l1 > COLS_MAX_LOG || l2 > COLS_MAX_LOG) {
      fail("axis longer than 2^22 points");
      return;
    }
    long long L1 = 1LL << l1, L2 = 1LL << l2;
    long long N = outer * L * inner;
    View S = split_view(B_SCR, B_SCR, scr_base);
    S.im.off = scr_base + N;
    need_scratch(scr_base + 2 * N);
    // pass A: lines (o, t2, m), points t1 (stride L2*inner) -> Y(k1, t2, m)
    line(LK_C2C, true, false, l1, io(A, L2 * inner, 1, a_bs, l2 + lin, L2 * inner - 1),
         io(S, L2 * inner, 1, L * inner, l2 + lin, L2 * inner - 1), outer * L2 * inner, inverse, L,
         L2 - 1, lin);
    // pass B: lines (o, k1, m), points t2 (stride inner) -> X(k1 + L1 k2, m)
    line(LK_C2C, true, false, l2, io(S, inner, 1, L2 * inner, lin, inner - 1),
         io(B, L1 * inner, 1, b_bs, l1 + lin, L1 * inner - 1), outer * L1 * inner, inverse);
  }

  // Complex N-D transform of `count` dense arrays of shape dims[0..nd) from
  // view A to view B: last axis first, then in place on B.
  void nd(int nd, const long long* dims, long long count, const View& A, const View& B, bool inverse) {
    long long total = count;
    for (int i = 0; i < nd; i++) total *= dims[i];
    bool first = true;
    int ax0 = nd - 1;
    if (nd >= 2 && plane_fits(dims[nd - 2], dims[nd - 1], total / (dims[nd - 2] * dims[nd - 1]), A, B)) {
      // the last two axes in one pass, then the others in place
      plane(dims[nd - 2], dims[nd - 1], total / (dims[nd - 2] * dims[nd - 1]), A, B, inverse);
      first = false;
      ax0 = nd - 3;
    }
    for (int ax = ax0; ax >= 0; ax--) {
      long long L = dims[ax];
      if (L == 1) continue;
      long long inner = 1;
      for (int j = ax + 1; j < nd; j++) inner *= dims[j];
      long long outer = total / (L * inner);
      axis(outer, L, inner, first ? A : B, B, inverse);
      first = false;
    }
    if (first) {
      // every dim is 1: copy (a length-1 transform)
      axis(total, 1, 1, A, B, inverse);
    }
  }
};

std::unique_ptr<Plan> build_plan(int kind, int ndim, const long long* dims, long long batch, int format,
                                 bool dry, int form, const Tuning* tune) {
  std::unique_ptr<Plan> P(new Plan());
  P->kind = kind;
  P->format = format;
  P->form = form;
  P->ndim = ndim;
  for (int i = 0; i < ndim; i++) P->dims[i] = dims[i];
  P->batch = batch;
  if (!dry) {
    cudaGetDevice(&P->device);
    if (cudaDeviceGetAttribute(&P->sm_count, cudaDevAttrMultiProcessorCount, P->device) != cudaSuccess) {
      cudaGetLastError();
      P->sm_count = 0;   // the pipelined kernels stay off
    }
  }

  long long N = 1;
  for (int i = 0; i < ndim; i++) N *= dims[i];
  long long d0 = dims[0];
  long long inner = N / d0;
  long long H = (d0 / 2 + 1) * inner;
  bool inter = format == 1;

  View src = inter ? inter_view(B_SRC_RE) : split_view(B_SRC_RE, B_SRC_IM);
  View dst = inter ? inter_view(B_DST_RE) : split_view(B_DST_RE, B_DST_IM);

  Tuning tn;
  if (tune) tn = *tune;
  else if (!dry && form == 0) tn = tuned_choice(kind, ndim, dims, batch, format);
  if (tn.tc && form == 0) P->form = form = FORM_TC;   // tuned to the tensor-core form
  Builder b(*P, dry);
  b.tune = tn;
  if (kind == K_C || kind == K_CI) {
    P->in_elems = N;
    P->out_elems = N;
    b.nd(ndim, dims, batch, src, dst, kind == K_CI);
  } else if (ndim == 1) {
    // 1D real: L = n/2 complex points of the interleaved view
    long long n = d0, L = n / 2;
    P->in_elems = kind == K_R ? n : H;
    P->out_elems = kind == K_R ? H : n;
    View realv = inter_view(kind == K_R ? B_SRC_RE : B_DST_RE);
    if (n == 1) {
      // a real transform of total size 1 (the reference crashes here):
      // the length-1 DFT, X[0] = x[0] + 0i and x[0] = re X[0]
      b.real1(kind == K_R, batch);
    } else if (ilog2ll(L) <= b.rows_max()) {
      int logl = ilog2ll(L);
      if (kind == K_R)
        b.line(LK_R2C, false, false, logl, io(realv, 1, 0, L, 0, 0), io(dst, 1, 0, L + 1, 0, 0), batch,
               false, 0, 0, 0, L);
      else
        b.line(LK_C2R, false, false, logl, io(src, 1, 0, L + 1, 0, 0), io(realv, 1, 0, L, 0, 0), batch,
               false, 0, 0, 0, L);
    } else if (kind == K_R && b.f64) {
      // FP64: the complex four-step into scratch (its own scratch above),
      // then the standalone real post-pass into dst
      View S = split_view(B_SCR, B_SCR, 0);
      S.im.off = batch * L;
      b.need_scratch(2 * batch * L);
      b.scr_base = 2 * batch * L;
      b.axis(batch, L, 1, realv, S, false, L, L);
      b.real_pass(io(S, 1, 0, L, 0, 0), io(dst, 1, 0, L + 1, 0, 0), batch, L, false, false);
    } else if (kind == K_R) {
      // four-step pass A (twiddle, transposing store) into scratch, then
      // pass B over mirrored column pairs with the real post-pass fused,
      // into dst lines of L + 1 bins; the scratch holds re,im pairs (8-byte
      // accesses on both sides)
      const int logl = ilog2ll(L), l1 = b.l1_of(logl), l2 = logl - l1;
      const long long L1 = 1LL << l1, L2 = 1LL << l2;
      View S = inter_view(B_SCR, 0);
      b.need_scratch(2 * batch * L);
      b.line(LK_C2C, true, true, l1, io(realv, L2, 1, L, l2, L2 - 1), io(S, 1, L1, L, l2, L2 - 1), batch * L2,
             false, L, L2 - 1, 0);
      b.line(LK_R2C_PAIRED, true, false, l2, io(S, L1, 1, L, l1, L1 - 1), io(dst, L1, 1, L + 1, l1, L1 - 1),
             batch * L1, false, 0, 0, 0, L);
      if (b.ok) {
        Op& ob = P->ops.back();
        ob.p.pcols = L1;
        if (L1 % ob.k.lines_per_cta) b.fail("paired pass: columns not a multiple of the tile");
      }
    } else {
      const int logl = ilog2ll(L);
      // the paired pass A runs over the shorter half by default (the longer
      // one when tuned so, where its kernel exists: pass A lengths <= 512)
      const int l1p = b.tune.split ? (logl + 1) / 2 : logl / 2;
      if (!b.f64 && logl <= 18 && b.tune.real_inv == 0 && l1p <= 9) {
        // inverse four-step pass A over mirrored column pairs with the real
        // pre-pass fused into its loads (twiddle, transposing store into
        // scratch), then pass B into dst's interleaved view.  Pass A takes
        // the shorter half, L1 <= 512: tiles of 16 lines, so each mirrored
        // half-tile is a 32-byte row segment (8-line tiles of the longer
        // lengths leave 16-byte halves, measured slower than the unfused
        // form below).  Up to n = 2^19: at 2^20 the unfused form measured
        // faster on GB300 (64 x 2^20: 0.369 vs 0.384 ms)
        const int l1 = l1p, l2 = logl - l1;
        const long long L1 = 1LL << l1, L2 = 1LL << l2;
        View S = inter_view(B_SCR, 0);   // re,im pairs: 8-byte accesses on both sides
        b.need_scratch(2 * batch * L);
        b.line(LK_C2R_PAIRED, true, true, l1, io(src, L2, 1, L + 1, l2, L2 - 1), io(S, 1, L1, L, l2, L2 - 1),
               batch * L2, true, L, L2 - 1, 0, L);
        if (b.ok) {
          Op& oa = P->ops.back();
          oa.p.pcols = L2;
          if (L2 % oa.k.lines_per_cta) b.fail("paired pass: columns not a multiple of the tile");
        }
        b.line(LK_C2C, true, false, l2, io(S, L1, 1, L, l1, L1 - 1), io(realv, L1, 1, L, l1, L1 - 1),
               batch * L1, true);
      } else {
        // real pre-pass into scratch (Z', as re,im pairs so that pass A
        // takes its 8-byte-pair loads), then the inverse four-step from
        // there into dst's interleaved view, its own scratch above Z'
        View S = inter_view(B_SCR, 0);
        b.need_scratch(2 * batch * L);
        b.real_pass(io(src, 1, 0, L + 1, 0, 0), io(S, 1, 0, L, 0, 0), batch, L, true, false);
        b.scr_base = 2 * batch * L;
        b.axis(batch, L, 1, S, realv, true, L, L);
      }
    }
  } else {
    // N-D real, dim 0 halved
    long long L = d0 / 2;
    int logl = ilog2ll(L);
    int lin = ilog2ll(inner);
    P->in_elems = kind == K_R ? N : H;
    P->out_elems = kind == K_R ? H : N;
    // the row-pair view of the real array: z(k, m) = x[2k][m] + i x[2k+1][m]
    // (fft_internal.hpp:281-283, multi.hpp:261-272)
    View rows;
    rows.re = {kind == K_R ? B_SRC_RE : B_DST_RE, 0};
    rows.im = {kind == K_R ? B_SRC_RE : B_DST_RE, inner};
    rows.unit = 1;
    if (logl <= COLS_MAX_LOG) {
      if (kind == K_R) {
        b.line(LK_R2C, true, false, logl, io(rows, 2 * inner, 1, N, lin, inner - 1),
               io(dst, inner, 1, H, lin, inner - 1), batch * inner, false, 0, 0, 0, L);
        b.nd(ndim - 1, dims + 1, batch * (L + 1), dst, dst, false);
      } else {
        View S = split_view(B_SCR, B_SCR, 0);
        S.im.off = batch * H;
        b.need_scratch(2 * batch * H);
        b.scr_base = 2 * batch * H;
        b.nd(ndim - 1, dims + 1, batch * (L + 1), src, S, true);
        b.line(LK_C2R, true, false, logl, io(S, inner, 1, H, lin, inner - 1),
               io(rows, 2 * inner, 1, N, lin, inner - 1), batch * inner, false, 0, 0, 0, L);
      }
    } else {
      // dim 0 too long for one CTA: pack the row pairs, four-step along
      // dim 0, standalone real pass along dim 0 (multi.hpp:343-414)
      long long Z = batch * L * inner;  // complex elements of the packed array
      int ll = ilog2ll(L);
      if (kind == K_R) {
        View S = split_view(B_SCR, B_SCR, 0);
        S.im.off = Z;
        b.need_scratch(2 * Z);
        b.copy(io(rows, 1, 2 * inner, 2 * L * inner, ll, L - 1), io(S, 1, inner, L * inner, ll, L - 1),
               batch * L, inner);
        b.scr_base = 2 * Z;
        b.axis(batch, L, inner, S, dst, false, L * inner, (L + 1) * inner);
        b.real_pass(io(dst, inner, 1, H, lin, inner - 1), io(dst, inner, 1, H, lin, inner - 1), batch * inner,
                    L, false, true);
        b.nd(ndim - 1, dims + 1, batch * (L + 1), dst, dst, false);
      } else {
        View S = split_view(B_SCR, B_SCR, 0);   // planes after the (N-1)-D inverse
        S.im.off = batch * H;
        View S2 = split_view(B_SCR, B_SCR, 2 * batch * H);   // Z'
        S2.im.off = 2 * batch * H + Z;
        View S3 = split_view(B_SCR, B_SCR, 2 * batch * H + 2 * Z);   // z
        S3.im.off = 2 * batch * H + 3 * Z;
        long long base = 2 * batch * H + 4 * Z;
        b.need_scratch(base);
        b.scr_base = base;
        b.nd(ndim - 1, dims + 1, batch * (L + 1), src, S, true);
        b.real_pass(io(S, inner, 1, H, lin, inner - 1), io(S2, inner, 1, L * inner, lin, inner - 1),
                    batch * inner, L, true, true);
        b.axis(batch, L, inner, S2, S3, true);
        b.copy(io(S3, 1, inner, L * inner, ll, L - 1), io(rows, 1, 2 * inner, 2 * L * inner, ll, L - 1),
               batch * L, inner);
      }
    }
  }
  if (!b.ok) {
    set_error(1, b.err);
    return nullptr;
  }
  return P;
}

static std::string io_json(const IOSpec& s) {
  char buf[512];
  snprintf(buf, sizeof buf,
           "{\"re\":[%d,%lld],\"im\":[%d,%lld],\"es\":%lld,\"lo\":%lld,\"hi\":%lld,\"qshift\":%d,"
           "\"qmask\":%lld}",
           s.re.buf, s.re.off, s.im.buf, s.im.off, s.es, s.lo, s.hi, s.qshift, s.qmask);
  return buf;
}

std::string describe_plan(const Plan& P) {
  std::string o = "{";
  char buf[1024];
  snprintf(buf, sizeof buf,
           "\"kind\":%d,\"format\":%d,\"f64\":%d,\"batch\":%lld,\"in_elems\":%lld,\"out_elems\":%lld,"
           "\"scratch_elems\":%lld,\"ops\":[",
           P.kind, P.format, P.f64() ? 1 : 0, P.batch, P.in_elems, P.out_elems, P.scratch_elems);
  o += buf;
  for (size_t i = 0; i < P.ops.size(); i++) {
    const Op& op = P.ops[i];
    if (i) o += ",";
    if (op.type == OP_LINE) {
      snprintf(buf, sizeof buf,
               "{\"type\":\"line\",\"logl\":%d,\"cols\":%d,\"lk\":%d,\"tstore\":%d,\"tc\":%d,\"C\":%d,"
               "\"halves\":%d,\"unit\":%d,\"tma\":%d,\"tma_store\":%d,\"pipe\":%d,\"plane\":%d,"
               "\"threads\":%d,\"smem\":%zu,\"grid\":%lld,\"nlines\":%lld,\"inverse\":%d,"
               "\"tw_n\":%lld,\"tw_qmask\":%lld,\"tw_qshift\":%d,\"real_L\":%lld,\"pcols\":%lld,",
               op.k.logl, op.k.cols, op.k.kind, op.k.tstore, op.k.tc, op.k.lines_per_cta, op.k.halves, op.k.unit,
               op.k.tma != nullptr, op.k.tma_bulk != nullptr, op.k.pipe != nullptr, op.k.plane_log1, op.threads,
               op.smem,
               op.grid, op.p.nlines, op.p.inverse, op.p.tw_n, op.p.tw_qmask, op.p.tw_qshift, op.real_L, op.p.pcols);
    } else if (op.type == OP_REAL) {
      snprintf(buf, sizeof buf,
               "{\"type\":\"real\",\"threads\":%d,\"grid\":%lld,\"nlines\":%lld,\"L\":%lld,"
               "\"inverse\":%d,\"lines_fastest\":%d,",
               op.threads, op.grid, op.rp.nlines, op.rp.L, op.rp.inverse, op.rp.lines_fastest);
    } else if (op.type == OP_COPY) {
      snprintf(buf, sizeof buf, "{\"type\":\"copy\",\"threads\":%d,\"grid\":%lld,\"nlines\":%lld,\"len\":%lld,",
               op.threads, op.grid, op.cp.nlines, op.cp.len);
    } else {
      snprintf(buf, sizeof buf, "{\"type\":\"real1\",\"threads\":%d,\"grid\":%lld,\"nlines\":%lld,\"inverse\":%d,",
               op.threads, op.grid, op.rp.nlines, op.rp.inverse);
    }
    o += buf;
    o += "\"in\":" + io_json(op.in) + ",\"out\":" + io_json(op.out) + "}";
  }
  o += "]}";
  return o;
}

Plan::~Plan() {
  if (scratch) cudaFree(scratch);
  if (stage) cudaFree(stage);
  if (stream) cudaStreamDestroy(stream);
  if (copy_in) cudaStreamDestroy(copy_in);
  if (copy_out) cudaStreamDestroy(copy_out);
  for (auto e : ev) cudaEventDestroy(e);
}

// element `off` of buffer `buf`, elements of `esz` bytes (4, or 8 in FP64 plans)
static inline float* resolve(const Ref& r, float* const* base, size_t esz) {
  return base[r.buf] ? reinterpret_cast<float*>(reinterpret_cast<char*>(base[r.buf]) + r.off * (long long)esz)
                     : nullptr;
}

static LineIO bind(const IOSpec& s, float* const* base, size_t esz) {
  LineIO o;
  o.re = resolve(s.re, base, esz);
  o.im = resolve(s.im, base, esz);
  o.es = s.es;
  o.lo = s.lo;
  o.hi = s.hi;
  o.qshift = s.qshift;
  o.qmask = s.qmask;
  return o;
}

// The driver's tensor-map encoder, looked up once.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      f = nullptr;
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// The tensor maps of one side (input or output planes) of a cols pass, when
// the bound arrays allow them: lines are whole tiles of C adjacent columns of
// one outer block (lo = 1, ncols = 2^qshift a multiple of C, every block
// whole), both plane bases 16-byte aligned, row and block strides multiples
// of 16 bytes.  Boxes of C columns x min(L, 256) rows.
static bool encode_tile(const LineIO& io, long long nlines, long long L, long long C, bool pairs, TmaTile* tm) {
  const long long ncols = io.qmask + 1;
  // pairs: one interleaved array, adjacent columns adjacent pairs
  if (io.lo != (pairs ? 2 : 1) || ncols != (1LL << io.qshift) || ncols % C || nlines % ncols || L > (1LL << 16))
    return false;
  if (pairs ? (io.im != io.re + 1 || (reinterpret_cast<uintptr_t>(io.re) & 15))
            : ((reinterpret_cast<uintptr_t>(io.re) | reinterpret_cast<uintptr_t>(io.im)) & 15))
    return false;
  const long long nouter = nlines / ncols;
  const long long rs = io.es * 4, bs = nouter > 1 ? io.hi * 4 : L * io.es * 4;
  if (rs % 16 || bs % 16 || rs <= 0 || bs <= 0 || rs >= (1LL << 40) || bs >= (1LL << 40)) return false;
  auto encode = tensor_map_encoder();
  if (!encode) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)(pairs ? 2 * ncols : ncols), (cuuint64_t)L, (cuuint64_t)nouter};
  const cuuint64_t strides[2] = {(cuuint64_t)rs, (cuuint64_t)bs};
  const int br = (int)std::min<long long>(L, 256);
  const cuuint32_t box[3] = {(cuuint32_t)(pairs ? 2 * C : C), (cuuint32_t)br, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  for (int i = 0; i < (pairs ? 1 : 2); i++) {
    if (encode(i ? &tm->im : &tm->re, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)(i ? io.im : io.re), dims, strides,
               box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  if (pairs) tm->im = tm->re;
  tm->box_rows = br;
  tm->rows = (int)L;
  tm->pairs = pairs ? 1 : 0;
  return true;
}

// The input planes' maps (false: launch the LSU kernel instead).  Input
// pairs for cols kernels with pairs bit 0.
bool tma_tile(const LineParams& p, const LineKernel& k, TmaTile* tm) {
  return encode_tile(p.in, p.nlines, 1LL << k.logl, k.lines_per_cta, (k.unit & 1) != 0, tm);
}

// The output planes' maps of a pipelined pass that stores by TMA.
bool tma_tile_out(const LineParams& p, const LineKernel& k, TmaTile* tm) {
  return encode_tile(p.out, p.nlines, 1LL << k.logl, k.lines_per_cta, false, tm);
}

// The paired R2C pass's maps (line_fft_paired_tma): its input is one
// interleaved array of pairs, lines (o, k1) the columns of L1 = pcols per
// transform, rows at element stride es, transforms hi apart; whole
// transforms, 16-byte aligned base and strides.
bool tma_paired(const LineParams& p, const LineKernel& k, PairedTma* pt) {
  const LineIO& in = p.in;
  const long long L2 = 1LL << k.logl, C = k.lines_per_cta, H = C / 2, L1 = p.pcols;
  if (in.im != in.re + 1 || in.lo != 2 || L1 <= 0 || (1LL << in.qshift) != L1 || in.qmask != L1 - 1 || L1 % C ||
      p.nlines % L1 || (reinterpret_cast<uintptr_t>(in.re) & 15))
    return false;
  const long long nouter = p.nlines / L1;
  const long long rs = in.es * 4, bs = nouter > 1 ? in.hi * 4 : L2 * in.es * 4;
  if (rs % 16 || bs % 16 || rs <= 0 || bs <= 0 || rs >= (1LL << 40) || bs >= (1LL << 40)) return false;
  auto encode = tensor_map_encoder();
  if (!encode) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)(2 * L1), (cuuint64_t)L2, (cuuint64_t)nouter};
  const cuuint64_t strides[2] = {(cuuint64_t)rs, (cuuint64_t)bs};
  const int br = (int)std::min<long long>(L2, 256);
  const cuuint32_t estr[3] = {1, 1, 1};
  const cuuint32_t widths[3] = {(cuuint32_t)(2 * H), (cuuint32_t)(2 * H + 4), 4};
  CUtensorMap* maps[3] = {&pt->al, &pt->mi, &pt->sp};
  for (int i = 0; i < 3; i++) {
    const cuuint32_t box[3] = {widths[i], (cuuint32_t)br, 1};
    if (encode(maps[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)in.re, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  pt->box_rows = br;
  return true;
}

bool op_tables_ok(const Op& op) {
  if (op.type != OP_LINE) return op.type != OP_REAL || op.rp.rtw;
  return op.p.tw && (op.k.kind == LK_C2C || op.p.rtw) &&
         (!op.p.tw_n || op.p.tw_full || (op.p.tw_hi && op.p.tw_lo)) && (!op.k.tc || op.p.tc_b) &&
         (!op.k.plane_log1 || op.p.tw2);
}

int Plan::launch(const float* src_re, const float* src_im, float* dst_re, float* dst_im, cudaStream_t st) {
  if (scratch_elems > 0 && !scratch) {
    if (cudaMalloc(&scratch, (size_t)scratch_elems * esize()) != cudaSuccess) {
      cudaGetLastError();
      set_error(3, "scratch allocation failed");
      return 3;
    }
  }
  float* base[B_NBUF] = {(float*)src_re, (float*)src_im, dst_re, dst_im, scratch};
  // every table a line kernel reads must exist: a plan-building mistake is
  // reported here instead of reaching the GPU as a NULL pointer
  for (const auto& op : ops) {
    if (!op_tables_ok(op)) {
      set_error(4, "plan is missing a twiddle table");
      return 4;
    }
  }
  const size_t esz = esize();
  const bool dbl = f64();
  for (auto& op : ops) {
    if (op.type == OP_LINE) {
      LineParams p = op.p;
      p.in = bind(op.in, base, esz);
      p.out = bind(op.out, base, esz);
      TmaTile tm, tmo{};
      PairedTma pt;
      // (1024-point tiles take the pipelined kernel from two per CTA slot:
      // with one each it has nothing to prefetch and its float exchange
      // costs more, 2048² c2r 0.0324 vs 0.0300 ms)
      const long long slots = (long long)sm_count * op.k.pipe_ctas;
      if (op.k.paired_tma && tma_paired(p, op.k, &pt)) {
        op.k.paired_tma<<<(unsigned)op.grid, op.threads, op.k.paired_smem, st>>>(p, pt);
      } else if (op.k.pipe && sm_count > 0 && (op.k.logl == 11 || op.grid >= 2 * slots) && tma_tile(p, op.k, &tm) &&
          (!(AFFT_PIPE_BULK_STORE && !op.k.tstore &&
             ((op.k.kind == LK_C2C && (op.k.logl == 11 || AFFT_PIPE_BULK10)) ||
              (op.k.kind == LK_C2R && op.k.logl == 10 && AFFT_PIPE_BULK_C2R10))) ||
           tma_tile_out(p, op.k, &tmo))) {
        // persistent: at most pipe_ctas CTAs per SM, each walking tiles gridDim.x apart
        const long long g = std::min<long long>(op.grid, slots);
        op.k.pipe<<<(unsigned)g, op.threads, op.k.pipe_smem, st>>>(p, tm, tmo, op.grid);
      } else if (op.k.tma_bulk && tma_tile(p, op.k, &tm) && tma_tile_out(p, op.k, &tmo)) {
        op.k.tma_bulk<<<(unsigned)op.grid, op.threads, op.smem, st>>>(p, tm, tmo);
      } else if (op.k.tma && tma_tile(p, op.k, &tm)) {
        op.k.tma<<<(unsigned)op.grid, op.threads, op.smem, st>>>(p, tm);
      } else {
        op.k.fn<<<(unsigned)op.grid, op.threads, op.smem, st>>>(p);
      }
    } else if (op.type == OP_REAL) {
      RealPassParams rp = op.rp;
      rp.in = bind(op.in, base, esz);
      rp.out = bind(op.out, base, esz);
      if (dbl) real_pass_kernel64<<<(unsigned)op.grid, op.threads, 0, st>>>(rp);
      else real_pass_kernel<<<(unsigned)op.grid, op.threads, 0, st>>>(rp);
    } else if (op.type == OP_COPY) {
      CopyParams cp = op.cp;
      cp.in = bind(op.in, base, esz);
      cp.out = bind(op.out, base, esz);
      if (dbl) copy_lines_kernel64<<<(unsigned)op.grid, op.threads, 0, st>>>(cp);
      else copy_lines_kernel<<<(unsigned)op.grid, op.threads, 0, st>>>(cp);
    } else {
      RealPassParams rp = op.rp;
      rp.in = bind(op.in, base, esz);
      rp.out = bind(op.out, base, esz);
      if (dbl) real1_kernel64<<<(unsigned)op.grid, op.threads, 0, st>>>(rp);
      else real1_kernel<<<(unsigned)op.grid, op.threads, 0, st>>>(rp);
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(4, std::string("kernel launch failed: ") + cudaGetErrorString(e));
    return 4;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// kernel registry
// ---------------------------------------------------------------------------
bool get_line_kernel(int logl, bool cols, int kind, bool tstore, LineKernel* out) {
  if (logl < 0) return false;
  if (!cols) {
    if (tstore || logl > ROWS_MAX_LOG) return false;
    if (kind == LK_C2C) return get_rows_c2c(logl, out);
    if (kind == LK_R2C) return get_rows_r2c(logl, out);
    if (kind == LK_C2R) return get_rows_c2r(logl, out);
    return false;
  }
  if (logl > COLS_MAX_LOG) return false;
  if (kind == LK_C2C) return get_cols_c2c(logl, tstore, out);
  if (tstore != (kind == LK_C2R_PAIRED)) return false;
  return get_cols_real(logl, kind, out);
}

int validate_shape(int ndim, const size_t* dim, int* ndim_out, long long* dims_out) {
  if (ndim > 64) return 1;
  int k = 0;
  long long total = 1;
  for (int i = 0; i < ndim; i++) {
    size_t d = dim[i];
    if (d == 0 || (d & (d - 1)) != 0) return 1;
    if (d > (1ULL << 31)) return 1;
    total *= (long long)d;
    if (total > (1LL << 31)) return 1;
    if (d != 1) dims_out[k++] = (long long)d;
  }
  if (k == 0) dims_out[k++] = 1;
  *ndim_out = k;
  return 0;
}

}  // namespace agb
