// A libbench2-style driver for afft's libbench2 test program
// (misc/libbench2-test/doit.cpp, compiled unchanged), linked against
// libafft_gb300.so through afft's own C++ wrapper fft.hpp.  For each problem
// (complex, interleaved float data, forward and backward, 1D to 3D) it fills
// the input, runs the program's hooks (can_do, setup, doit, done) the way the
// harness does, and checks the output against a separable naive DFT in
// double precision.  Exits non-zero on a mismatch.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <vector>

#include "bench-user.h"

using cd = std::complex<double>;

// naive DFT along each dimension of a row-major array, exponent sign `sign`
static std::vector<cd> reference(const std::vector<int>& dims, std::vector<cd> x, int sign) {
  const int nd = (int)dims.size();
  size_t total = 1;
  for (int d : dims) total *= (size_t)d;
  size_t inner = total;
  for (int a = 0; a < nd; a++) {
    const int n = dims[a];
    inner /= (size_t)n;
    const size_t outer = total / ((size_t)n * inner);
    std::vector<cd> line(n), res(n);
    for (size_t o = 0; o < outer; o++)
      for (size_t m = 0; m < inner; m++) {
        for (int i = 0; i < n; i++) line[i] = x[(o * n + i) * inner + m];
        for (int k = 0; k < n; k++) {
          cd acc = 0;
          for (int i = 0; i < n; i++) {
            const double ang = sign * 2.0 * M_PI * (double)(((long long)i * k) % n) / n;
            acc += line[i] * cd(std::cos(ang), std::sin(ang));
          }
          res[k] = acc;
        }
        for (int k = 0; k < n; k++) x[(o * n + k) * inner + m] = res[k];
      }
  }
  return x;
}

static int run_case(const std::vector<int>& dims, int sign) {
  const int nd = (int)dims.size();
  std::vector<bench_iodim> io(nd);
  int stride = 1;
  for (int a = nd - 1; a >= 0; a--) {
    io[a].n = dims[a];
    io[a].is = io[a].os = stride;
    stride *= dims[a];
  }
  const size_t n = (size_t)stride;
  bench_tensor sz{nd, io.data()};
  bench_tensor vecsz{0, nullptr};
  std::vector<float> in(2 * n), out(2 * n, 0.f);
  std::vector<cd> x(n);
  for (size_t i = 0; i < n; i++) {
    x[i] = cd(std::sin(0.37 * (double)i + 0.1), std::cos(0.11 * (double)i * (double)(i % 7)));
    in[2 * i] = (float)x[i].real();
    in[2 * i + 1] = (float)x[i].imag();
    x[i] = cd(in[2 * i], in[2 * i + 1]);
  }
  bench_problem p;
  std::memset(&p, 0, sizeof p);
  p.kind = PROBLEM_COMPLEX;
  p.sz = &sz;
  p.vecsz = &vecsz;
  p.sign = sign;
  p.in = in.data();
  p.out = out.data();
  if (!can_do(&p)) {
    std::printf("can_do refused a complex problem\n");
    return 1;
  }
  setup(&p);
  doit(1, &p);
  done(&p);
  const std::vector<cd> ref = reference(dims, x, sign);
  double num = 0, den = 0;
  for (size_t i = 0; i < n; i++) {
    const cd y(out[2 * i], out[2 * i + 1]);
    num += std::norm(y - ref[i]);
    den += std::norm(ref[i]);
  }
  const double err = std::sqrt(num / den);
  std::printf("dims");
  for (int d : dims) std::printf(" %d", d);
  std::printf(" sign %+d: rel-L2 %.3g\n", sign, err);
  return err < 2e-6 ? 0 : 1;
}

int main(int argc, char** argv) {
  main_init(&argc, &argv);
  if (!bench_doc[0].key || std::strcmp(bench_doc[0].key, "name") != 0 || std::strcmp(bench_doc[0].val, "afft") != 0) {
    std::printf("unexpected bench_doc table\n");
    return 1;
  }
  bench_problem real{};
  bench_tensor sz{0, nullptr};
  real.kind = PROBLEM_REAL;
  real.sz = &sz;
  if (can_do(&real)) {
    std::printf("can_do accepted a rank-0 real problem\n");
    return 1;
  }
  int rc = 0;
  const std::vector<std::vector<int>> shapes = {{1024}, {4096}, {64, 128}, {16, 16, 16}, {2, 512}};
  for (const auto& s : shapes)
    for (int sign : {-1, 1}) rc |= run_case(s, sign);
  cleanup();
  std::printf(rc ? "FAILED\n" : "ok\n");
  return rc;
}
