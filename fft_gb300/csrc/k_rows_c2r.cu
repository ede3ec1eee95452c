// rows-mode line FFT instantiations, kind LK_C2R, L = 2^0 .. 2^14
#include "kernels.h"
namespace agb {
bool get_rows_c2r(int logl, LineKernel* out) {
  switch (logl) {
    case 0: *out = make_line_kernel<0, false, LK_C2R, false>(); return true;
    case 1: *out = make_line_kernel<1, false, LK_C2R, false>(); return true;
    case 2: *out = make_line_kernel<2, false, LK_C2R, false>(); return true;
    case 3: *out = make_line_kernel<3, false, LK_C2R, false>(); return true;
    case 4: *out = make_line_kernel<4, false, LK_C2R, false>(); return true;
    case 5: *out = make_line_kernel<5, false, LK_C2R, false>(); return true;
    case 6: *out = make_line_kernel<6, false, LK_C2R, false>(); return true;
    case 7: *out = make_line_kernel<7, false, LK_C2R, false>(); return true;
    case 8: *out = make_line_kernel<8, false, LK_C2R, false>(); return true;
    case 9: *out = make_line_kernel<9, false, LK_C2R, false>(); return true;
    case 10: *out = make_line_kernel<10, false, LK_C2R, false>(); return true;
    case 11: *out = make_line_kernel<11, false, LK_C2R, false>(); return true;
    case 12: *out = make_line_kernel<12, false, LK_C2R, false>(); return true;
    case 13: *out = make_line_kernel<13, false, LK_C2R, false>(); return true;
    case 14: *out = make_line_kernel<14, false, LK_C2R, false>(); return true;
  }
  return false;
}
}  // namespace agb
