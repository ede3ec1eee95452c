// cols-mode complex line FFTs with other tile widths than the measured
// default, for the autotuner to weigh per shape: 256 points in 8- and
// 32-line tiles (default 16), 512 points in 16-line tiles (default 8); each
// with its TMA-fed variant
#include "kernels.h"
namespace agb {
bool get_cols_c2c_alt(int logl, int lines, LineKernel* out) {
  if (logl == 8 && lines == 8) *out = make_tma_kernel<8, LK_C2C, 8>();
  else if (logl == 8 && lines == 32) *out = make_tma_kernel<8, LK_C2C, 32>();
  else if (logl == 9 && lines == 16) *out = make_tma_kernel<9, LK_C2C, 16>();
  else return false;
  return true;
}
}  // namespace agb
