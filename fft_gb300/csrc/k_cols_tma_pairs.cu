// cols-mode complex line FFTs over interleaved input pairs whose input tile
// is loaded by TMA (one tensor map over the interleaved array), plain and
// with the transposing store, 2^8 and 2^9 points.  Measured on GB300:
// interleaved 65536 x 4096 c2c 1.344 -> 1.318 ms; at 2^10 points (the long
// 1D real transforms' pass A) the TMA kernels spill and ran 0.6% slower, so
// those keep LSU loads.
#include "kernels.h"
namespace agb {
template <int LOGL>
static bool tma_pairs_one(bool tstore, int pairs, LineKernel* out) {
  if (tstore && pairs == 1) *out = make_tma_kernel<LOGL, LK_C2C, 0, true, 1>();
  else if (tstore && pairs == 3) *out = make_tma_kernel<LOGL, LK_C2C, 0, true, 3>();
  else if (!tstore && pairs == 1) *out = make_tma_kernel<LOGL, LK_C2C, 0, false, 1>();
  else if (!tstore && pairs == 3) *out = make_tma_kernel<LOGL, LK_C2C, 0, false, 3>();
  else return false;
  return true;
}
bool get_cols_tma_pairs(int logl, bool tstore, int pairs, LineKernel* out) {
  switch (logl) {
    case 8: return tma_pairs_one<8>(tstore, pairs, out);
    case 9: return tma_pairs_one<9>(tstore, pairs, out);
  }
  return false;
}
}  // namespace agb
