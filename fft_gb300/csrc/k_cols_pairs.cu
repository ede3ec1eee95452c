// cols-mode complex line FFT on interleaved pairs (one 8-byte access per
// element): the real transforms' interleaved views and the interleaved
// format, L = 2^5 .. 2^11
#include <utility>

#include "kernels.h"

namespace agb {

template <int LOGL>
static bool cols_pairs_one(bool tstore, int pairs, LineKernel* out) {
  if (tstore) return get_cols_c2c_pairs_tstore(LOGL, pairs, out);
  if (pairs == 1) *out = make_line_kernel<LOGL, true, LK_C2C, false, false, 1>();
  else if (pairs == 2) *out = make_line_kernel<LOGL, true, LK_C2C, false, false, 2>();
  else if (pairs == 3) *out = make_line_kernel<LOGL, true, LK_C2C, false, false, 3>();
  else return false;
  return true;
}

template <int... Ls>
static bool cols_pairs_dispatch(int logl, bool tstore, int pairs, LineKernel* out,
                                std::integer_sequence<int, Ls...>) {
  bool ok = false;
  ((logl == Ls + 5 ? (void)(ok = cols_pairs_one<Ls + 5>(tstore, pairs, out)) : (void)0), ...);
  return ok;
}

bool get_cols_c2c_pairs(int logl, bool tstore, int pairs, LineKernel* out) {
  if (logl < 5 || logl > COLS_MAX_LOG) return false;
  return cols_pairs_dispatch(logl, tstore, pairs, out, std::make_integer_sequence<int, COLS_MAX_LOG - 4>{});
}

}  // namespace agb
