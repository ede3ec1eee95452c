// plane-fused passes (plane_fft): split planes of 2^12 .. 2^14 points, sides 16 .. 512
#include "kernels.h"
namespace agb {
bool get_plane_split_big(int log1, int log2, LineKernel* out) {
  switch (log1 * 16 + log2) {
    case 4 * 16 + 8: *out = make_plane_kernel<4, 8, 1>(); return true;
    case 5 * 16 + 7: *out = make_plane_kernel<5, 7, 1>(); return true;
    case 6 * 16 + 6: *out = make_plane_kernel<6, 6, 1>(); return true;
    case 7 * 16 + 5: *out = make_plane_kernel<7, 5, 1>(); return true;
    case 8 * 16 + 4: *out = make_plane_kernel<8, 4, 1>(); return true;
    case 4 * 16 + 9: *out = make_plane_kernel<4, 9, 1>(); return true;
    case 5 * 16 + 8: *out = make_plane_kernel<5, 8, 1>(); return true;
    case 6 * 16 + 7: *out = make_plane_kernel<6, 7, 1>(); return true;
    case 7 * 16 + 6: *out = make_plane_kernel<7, 6, 1>(); return true;
    case 8 * 16 + 5: *out = make_plane_kernel<8, 5, 1>(); return true;
    case 9 * 16 + 4: *out = make_plane_kernel<9, 4, 1>(); return true;
    case 5 * 16 + 9: *out = make_plane_kernel<5, 9, 1>(); return true;
    case 6 * 16 + 8: *out = make_plane_kernel<6, 8, 1>(); return true;
    case 7 * 16 + 7: *out = make_plane_kernel<7, 7, 1>(); return true;
    case 8 * 16 + 6: *out = make_plane_kernel<8, 6, 1>(); return true;
    case 9 * 16 + 5: *out = make_plane_kernel<9, 5, 1>(); return true;
  }
  return false;
}
}  // namespace agb
