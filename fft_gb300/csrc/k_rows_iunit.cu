// rows-mode complex line FFTs on interleaved (re, im) pairs with unit pair
// strides: one float2 access per element, and warp-staged float4 accesses
// for contiguous lines of up to 128 points.  L = 2^4 .. 2^14.
#include "kernels.h"
namespace agb {
bool get_rows_c2c_iunit(int logl, LineKernel* out) {
  switch (logl) {
    case 4: *out = make_line_kernel<4, false, LK_C2C, false, false, 2>(); return true;
    case 5: *out = make_line_kernel<5, false, LK_C2C, false, false, 2>(); return true;
    case 6: *out = make_line_kernel<6, false, LK_C2C, false, false, 2>(); return true;
    case 7: *out = make_line_kernel<7, false, LK_C2C, false, false, 2>(); return true;
    case 8: *out = make_line_kernel<8, false, LK_C2C, false, false, 2>(); return true;
    case 9: *out = make_line_kernel<9, false, LK_C2C, false, false, 2>(); return true;
    case 10: *out = make_line_kernel<10, false, LK_C2C, false, false, 2>(); return true;
    case 11: *out = make_line_kernel<11, false, LK_C2C, false, false, 2>(); return true;
    case 12: *out = make_line_kernel<12, false, LK_C2C, false, false, 2>(); return true;
    case 13: *out = make_line_kernel<13, false, LK_C2C, false, false, 2>(); return true;
    case 14: *out = make_line_kernel<14, false, LK_C2C, false, false, 2>(); return true;
  }
  return false;
}
}  // namespace agb
