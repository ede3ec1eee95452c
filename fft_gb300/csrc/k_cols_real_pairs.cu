// four-step pass B of a long 1D real forward transform (the paired R2C pass)
// reading its input as float2 pairs, L = 2^7 .. 2^11; pass A of a long 1D
// real inverse (the paired C2R pass) writing its output so, L = 2^7 .. 2^9
#include "kernels.h"

// lines per CTA of the 512-point paired R2C pass (16: the cols default)
#ifndef AFFT_PAIRED_C9
#define AFFT_PAIRED_C9 16
#endif
// the TMA-fed form of the 512- and 1024-point paired R2C passes: built and
// taken only when set (measured 3-5% slower: 64 x 2^20 r2c 0.324 vs 0.308 ms)
#ifndef AFFT_PAIRED_TMA
#define AFFT_PAIRED_TMA 0
#endif

namespace agb {

bool get_r2c_paired_pairs(int logl, LineKernel* out) {
  switch (logl) {
    case 7: *out = make_line_kernel<7, true, LK_R2C_PAIRED, false, false, 1>(); return true;
    case 8: *out = make_line_kernel<8, true, LK_R2C_PAIRED, false, false, 1>(); return true;
#if AFFT_PAIRED_C9 == 16 && AFFT_PAIRED_TMA
    case 9: *out = make_paired_tma_kernel<9>(); return true;
    case 10: *out = make_paired_tma_kernel<10>(); return true;
#else
    case 9: *out = make_line_kernel<9, true, LK_R2C_PAIRED, false, false, 1, AFFT_PAIRED_C9>(); return true;
    case 10: *out = make_line_kernel<10, true, LK_R2C_PAIRED, false, false, 1>(); return true;
#endif
    case 11: *out = make_line_kernel<11, true, LK_R2C_PAIRED, false, false, 1>(); return true;
    default: return false;
  }
}

bool get_c2r_paired_pairs(int logl, LineKernel* out) {
  switch (logl) {
    case 7: *out = make_line_kernel<7, true, LK_C2R_PAIRED, true, false, 2>(); return true;
    case 8: *out = make_line_kernel<8, true, LK_C2R_PAIRED, true, false, 2>(); return true;
    case 9: *out = make_line_kernel<9, true, LK_C2R_PAIRED, true, false, 2>(); return true;
    default: return false;
  }
}

}  // namespace agb
