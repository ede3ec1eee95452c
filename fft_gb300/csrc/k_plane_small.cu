// plane-fused passes (plane_fft): split planes of 2^8 .. 2^11 points (several
// planes per CTA), sides 16 .. 128
#include "kernels.h"
namespace agb {
bool get_plane_split_small(int log1, int log2, LineKernel* out) {
  switch (log1 * 16 + log2) {
    case 4 * 16 + 4: *out = make_plane_kernel<4, 4, 1>(); return true;
    case 4 * 16 + 5: *out = make_plane_kernel<4, 5, 1>(); return true;
    case 5 * 16 + 4: *out = make_plane_kernel<5, 4, 1>(); return true;
    case 4 * 16 + 6: *out = make_plane_kernel<4, 6, 1>(); return true;
    case 5 * 16 + 5: *out = make_plane_kernel<5, 5, 1>(); return true;
    case 6 * 16 + 4: *out = make_plane_kernel<6, 4, 1>(); return true;
    case 4 * 16 + 7: *out = make_plane_kernel<4, 7, 1>(); return true;
    case 5 * 16 + 6: *out = make_plane_kernel<5, 6, 1>(); return true;
    case 6 * 16 + 5: *out = make_plane_kernel<6, 5, 1>(); return true;
    case 7 * 16 + 4: *out = make_plane_kernel<7, 4, 1>(); return true;
  }
  return false;
}
}  // namespace agb
namespace agb {
bool get_plane_kernel(int log1, int log2, int unit, LineKernel* out) {
  if (unit == 1) return log1 + log2 <= 11 ? get_plane_split_small(log1, log2, out) : get_plane_split_big(log1, log2, out);
  if (unit == 2) return log1 + log2 <= 11 ? get_plane_pairs_small(log1, log2, out) : get_plane_pairs_big(log1, log2, out);
  return false;
}
}  // namespace agb
