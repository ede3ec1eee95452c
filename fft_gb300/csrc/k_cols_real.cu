// cols-mode real line FFT instantiations (N-D real, first dim halved),
// L = 2^0 .. 2^11; the 2048-point R2C pass is the two-CTA split form
#include "kernels.h"
namespace agb {
bool get_cols_real(int logl, int kind, LineKernel* out) {
  if (kind == LK_R2C) {
    switch (logl) {
      case 0: *out = make_line_kernel<0, true, LK_R2C, false>(); return true;
      case 1: *out = make_line_kernel<1, true, LK_R2C, false>(); return true;
      case 2: *out = make_line_kernel<2, true, LK_R2C, false>(); return true;
      case 3: *out = make_line_kernel<3, true, LK_R2C, false>(); return true;
      case 4: *out = make_line_kernel<4, true, LK_R2C, false>(); return true;
      case 5: *out = make_line_kernel<5, true, LK_R2C, false>(); return true;
      case 6: *out = make_line_kernel<6, true, LK_R2C, false>(); return true;
      case 7: *out = make_line_kernel<7, true, LK_R2C, false>(); return true;
      case 8: *out = make_line_kernel<8, true, LK_R2C, false>(); return true;
      case 9: *out = make_line_kernel<9, true, LK_R2C, false>(); return true;
      case 10: *out = make_line_kernel<10, true, LK_R2C, false>(); return true;
      // 2048 points: split over two CTAs of 1024-point stages (2 CTAs/SM
      // instead of one)
      case 11: *out = make_line_kernel<10, true, LK_R2C_HALF, false>(); return true;
    }
  } else if (kind == LK_R2C_PAIRED) {
    // pass B of long 1D real forwards: L2 = 2^7 .. 2^11
    switch (logl) {
      case 7: *out = make_line_kernel<7, true, LK_R2C_PAIRED, false>(); return true;
      case 8: *out = make_line_kernel<8, true, LK_R2C_PAIRED, false>(); return true;
      case 9: *out = make_line_kernel<9, true, LK_R2C_PAIRED, false>(); return true;
      case 10: *out = make_line_kernel<10, true, LK_R2C_PAIRED, false>(); return true;
      case 11: *out = make_line_kernel<11, true, LK_R2C_PAIRED, false>(); return true;
    }
  } else if (kind == LK_C2R_PAIRED) {
    // pass A of long 1D real inverses: L1 = 2^7 .. 2^9
    switch (logl) {
      case 7: *out = make_line_kernel<7, true, LK_C2R_PAIRED, true>(); return true;
      case 8: *out = make_line_kernel<8, true, LK_C2R_PAIRED, true>(); return true;
      case 9: *out = make_line_kernel<9, true, LK_C2R_PAIRED, true>(); return true;
    }
  } else if (kind == LK_C2R) {
    switch (logl) {
      case 0: *out = make_line_kernel<0, true, LK_C2R, false>(); return true;
      case 1: *out = make_line_kernel<1, true, LK_C2R, false>(); return true;
      case 2: *out = make_line_kernel<2, true, LK_C2R, false>(); return true;
      case 3: *out = make_line_kernel<3, true, LK_C2R, false>(); return true;
      case 4: *out = make_line_kernel<4, true, LK_C2R, false>(); return true;
      case 5: *out = make_line_kernel<5, true, LK_C2R, false>(); return true;
      case 6: *out = make_line_kernel<6, true, LK_C2R, false>(); return true;
      case 7: *out = make_line_kernel<7, true, LK_C2R, false>(); return true;
      case 8: *out = make_line_kernel<8, true, LK_C2R, false>(); return true;
      case 9: *out = make_line_kernel<9, true, LK_C2R, false>(); return true;
      case 10: *out = make_line_kernel<10, true, LK_C2R, false>(); return true;
      case 11: *out = make_line_kernel<11, true, LK_C2R, false>(); return true;
    }
  }
  return false;
}
}  // namespace agb
