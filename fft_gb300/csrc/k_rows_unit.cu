// rows-mode complex line FFTs with unit element strides (split complex data,
// contiguous lines): every element offset is a compile-time constant.
// L = 2^4 .. 2^14, plus the tensor-core form at L = 256 and 4096.
#include "kernels.h"
namespace agb {
bool get_rows_c2c_unit(int logl, bool tc, LineKernel* out) {
  if (tc) {
    if (logl == 8) { *out = make_line_kernel<8, false, LK_C2C, false, true, true>(); return true; }
    if (logl == 12) { *out = make_line_kernel<12, false, LK_C2C, false, true, true>(); return true; }
    return false;
  }
  switch (logl) {
    case 4: *out = make_line_kernel<4, false, LK_C2C, false, false, true>(); return true;
    case 5: *out = make_line_kernel<5, false, LK_C2C, false, false, true>(); return true;
    case 6: *out = make_line_kernel<6, false, LK_C2C, false, false, true>(); return true;
    case 7: *out = make_line_kernel<7, false, LK_C2C, false, false, true>(); return true;
    case 8: *out = make_line_kernel<8, false, LK_C2C, false, false, true>(); return true;
    case 9: *out = make_line_kernel<9, false, LK_C2C, false, false, true>(); return true;
    case 10: *out = make_line_kernel<10, false, LK_C2C, false, false, true>(); return true;
    case 11: *out = make_line_kernel<11, false, LK_C2C, false, false, true>(); return true;
    case 12: *out = make_line_kernel<12, false, LK_C2C, false, false, true>(); return true;
    case 13: *out = make_line_kernel<13, false, LK_C2C, false, false, true>(); return true;
    case 14: *out = make_line_kernel<14, false, LK_C2C, false, false, true>(); return true;
  }
  return false;
}
}  // namespace agb
