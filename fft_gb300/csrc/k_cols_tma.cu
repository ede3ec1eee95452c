// cols-mode line FFTs whose input tile is loaded by TMA (line_fft_tma):
// complex, real forward and real inverse passes of 2^8 .. 2^11 points
#include "kernels.h"
// lines per CTA of the 2048-point TMA kernels
#ifndef AFFT_TMA_C11
#define AFFT_TMA_C11 8
#endif
namespace agb {
bool get_cols_tma(int logl, int kind, LineKernel* out) {
  if (kind == LK_C2C) {
    switch (logl) {
      case 8: *out = make_tma_kernel<8, LK_C2C>(); return true;
      case 9: *out = make_tma_kernel<9, LK_C2C>(); return true;
      case 10: *out = make_tma_kernel<10, LK_C2C>(); return true;
      case 11: *out = make_tma_kernel<11, LK_C2C, AFFT_TMA_C11>(); return true;
    }
  } else if (kind == LK_R2C) {
    switch (logl) {
      case 8: *out = make_tma_kernel<8, LK_R2C>(); return true;
      case 9: *out = make_tma_kernel<9, LK_R2C>(); return true;
      case 10: *out = make_tma_kernel<10, LK_R2C>(); return true;
      case 11: *out = make_tma_kernel<11, LK_R2C, AFFT_TMA_C11>(); return true;
    }
  } else if (kind == LK_C2R) {
    switch (logl) {
      case 8: *out = make_tma_kernel<8, LK_C2R>(); return true;
      case 9: *out = make_tma_kernel<9, LK_C2R>(); return true;
      case 10: *out = make_tma_kernel<10, LK_C2R>(); return true;
      case 11: *out = make_tma_kernel<11, LK_C2R, AFFT_TMA_C11>(); return true;
    }
  }
  return false;
}
}  // namespace agb
