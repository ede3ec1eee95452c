// afft's C++ wrapper (fft.hpp:48-234), unchanged, driving libafft_gb300.so.
// Without a GPU every plan is empty (memsize returns 0); with one, a
// forward + inverse round trip of n=1024 through host buffers recovers n*x.
#include <cmath>
#include <cstdio>
#include <vector>

#include "fft.hpp"

int main() {
  const size_t n = 1024;
  size_t dims[1] = {n};
  afft::complex_transform<float> fwd(1, dims);
  afft::inverse_complex_transform<float> inv(1, dims);
  afft::real_transform<float> rf(1, dims);
  afft::inverse_real_transform<float> ri(1, dims);
  const int have_gpu = afft_supported(afft_auto);
  if (bool(fwd) != bool(have_gpu) || bool(inv) != bool(have_gpu) || bool(rf) != bool(have_gpu) ||
      bool(ri) != bool(have_gpu)) {
    std::printf("plan state does not match afft_supported\n");
    return 1;
  }
  if (!have_gpu) {
    std::printf("ok (no device: plans empty)\n");
    return 0;
  }
  std::vector<float> xr(n), xi(n), yr(n), yi(n), zr(n), zi(n);
  for (size_t i = 0; i < n; i++) {
    xr[i] = std::sin(0.1f * i);
    xi[i] = std::cos(0.37f * i);
  }
  fwd(xr.data(), xi.data(), yr.data(), yi.data());
  inv(yr.data(), yi.data(), zr.data(), zi.data());
  double err = 0, ref = 0;
  for (size_t i = 0; i < n; i++) {
    err += std::pow(zr[i] / n - xr[i], 2) + std::pow(zi[i] / n - xi[i], 2);
    ref += xr[i] * xr[i] + xi[i] * xi[i];
  }
  std::printf("round trip rel-L2 %.3g\n", std::sqrt(err / ref));
  return std::sqrt(err / ref) < 2e-6 ? 0 : 1;
}
