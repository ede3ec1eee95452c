// plane-fused passes (plane_fft): interleaved planes of 2^8 .. 2^11 points
// (several planes per CTA), sides 16 .. 128
#include "kernels.h"
namespace agb {
bool get_plane_pairs_small(int log1, int log2, LineKernel* out) {
  switch (log1 * 16 + log2) {
    case 4 * 16 + 4: *out = make_plane_kernel<4, 4, 2>(); return true;
    case 4 * 16 + 5: *out = make_plane_kernel<4, 5, 2>(); return true;
    case 5 * 16 + 4: *out = make_plane_kernel<5, 4, 2>(); return true;
    case 4 * 16 + 6: *out = make_plane_kernel<4, 6, 2>(); return true;
    case 5 * 16 + 5: *out = make_plane_kernel<5, 5, 2>(); return true;
    case 6 * 16 + 4: *out = make_plane_kernel<6, 4, 2>(); return true;
    case 4 * 16 + 7: *out = make_plane_kernel<4, 7, 2>(); return true;
    case 5 * 16 + 6: *out = make_plane_kernel<5, 6, 2>(); return true;
    case 6 * 16 + 5: *out = make_plane_kernel<6, 5, 2>(); return true;
    case 7 * 16 + 4: *out = make_plane_kernel<7, 4, 2>(); return true;
  }
  return false;
}
}  // namespace agb
