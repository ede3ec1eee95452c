// afft's C++ wrapper (fft.hpp:48-234), unchanged, driving libafft_gb300.so
// for T = float (afft_32_*) and T = double (afft_64_*).  Without a GPU every
// plan is empty (memsize returns 0); with one, complex and real forward +
// inverse round trips of n=1024 through host buffers recover n*x.
#include <cmath>
#include <cstdio>
#include <vector>

#include "fft.hpp"

template <class T>
static int round_trips(const char* name, double bound) {
  const size_t n = 1024;
  size_t dims[1] = {n};
  afft::complex_transform<T> fwd(1, dims);
  afft::inverse_complex_transform<T> inv(1, dims);
  afft::real_transform<T> rf(1, dims);
  afft::inverse_real_transform<T> ri(1, dims);
  const int have_gpu = afft_supported(afft_auto);
  if (bool(fwd) != bool(have_gpu) || bool(inv) != bool(have_gpu) || bool(rf) != bool(have_gpu) ||
      bool(ri) != bool(have_gpu)) {
    std::printf("%s: plan state does not match afft_supported\n", name);
    return 1;
  }
  if (!have_gpu) {
    std::printf("%s ok (no device: plans empty)\n", name);
    return 0;
  }
  std::vector<T> xr(n), xi(n), yr(n), yi(n), zr(n), zi(n), hr(n / 2 + 1), hi(n / 2 + 1), w(n);
  for (size_t i = 0; i < n; i++) {
    xr[i] = std::sin(T(0.1) * T(i));
    xi[i] = std::cos(T(0.37) * T(i));
  }
  fwd(xr.data(), xi.data(), yr.data(), yi.data());
  inv(yr.data(), yi.data(), zr.data(), zi.data());
  rf(xr.data(), hr.data(), hi.data());
  ri(hr.data(), hi.data(), w.data());
  double err = 0, ref = 0, err_r = 0, ref_r = 0;
  for (size_t i = 0; i < n; i++) {
    err += std::pow(double(zr[i]) / n - xr[i], 2) + std::pow(double(zi[i]) / n - xi[i], 2);
    ref += double(xr[i]) * xr[i] + double(xi[i]) * xi[i];
    err_r += std::pow(double(w[i]) / n - xr[i], 2);
    ref_r += double(xr[i]) * xr[i];
  }
  const double e = std::sqrt(err / ref), er = std::sqrt(err_r / ref_r);
  std::printf("%s round trip rel-L2: complex %.3g, real %.3g\n", name, e, er);
  return e < bound && er < bound ? 0 : 1;
}

int main() {
  int rc = round_trips<float>("float", 2e-6);
  rc |= round_trips<double>("double", 1e-13);
  return rc;
}
