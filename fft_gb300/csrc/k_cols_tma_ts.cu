// cols-mode complex line FFTs with the transposing store (four-step pass A)
// whose input tile is loaded by TMA, 2^8 .. 2^10 points
#include "kernels.h"
namespace agb {
bool get_cols_tma_tstore(int logl, LineKernel* out) {
  switch (logl) {
    case 8: *out = make_tma_kernel<8, LK_C2C, 0, true>(); return true;
    case 9: *out = make_tma_kernel<9, LK_C2C, 0, true>(); return true;
    case 10: *out = make_tma_kernel<10, LK_C2C, 0, true>(); return true;
  }
  return false;
}
}  // namespace agb
