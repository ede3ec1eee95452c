// four-step pass A (cols mode, transposing store) on interleaved pairs: the
// input (pairs = 1) or both sides (pairs = 3) as 8-byte values, L = 2^5 .. 2^11
// (its own translation unit so the pair variants compile in parallel)
#include <utility>

#include "kernels.h"

namespace agb {

template <int LOGL>
static bool ts_pairs_one(int pairs, LineKernel* out) {
  if (pairs == 1) *out = make_line_kernel<LOGL, true, LK_C2C, true, false, 1>();
  else if (pairs == 3) *out = make_line_kernel<LOGL, true, LK_C2C, true, false, 3>();
  else return false;
  return true;
}

template <int... Ls>
static bool ts_pairs_dispatch(int logl, int pairs, LineKernel* out, std::integer_sequence<int, Ls...>) {
  bool ok = false;
  ((logl == Ls + 5 ? (void)(ok = ts_pairs_one<Ls + 5>(pairs, out)) : (void)0), ...);
  return ok;
}

bool get_cols_c2c_pairs_tstore(int logl, int pairs, LineKernel* out) {
  if (logl < 5 || logl > COLS_MAX_LOG) return false;
  return ts_pairs_dispatch(logl, pairs, out, std::make_integer_sequence<int, COLS_MAX_LOG - 4>{});
}

}  // namespace agb
