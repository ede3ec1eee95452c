// FP64 cols-mode line kernels, L = 2^0 .. 2^11: complex (plain and with the
// transposing store of the four-step first pass), real forward, real inverse
#include <utility>

#include "kernels64.h"

namespace agb {

template <int LOGL>
static bool cols64_one(int kind, bool tstore, LineKernel* out) {
  if (kind == LK_C2C && tstore) *out = make_line_kernel64<LOGL, true, LK_C2C, true>();
  else if (kind == LK_C2C) *out = make_line_kernel64<LOGL, true, LK_C2C, false>();
  else if (kind == LK_R2C && !tstore) *out = make_line_kernel64<LOGL, true, LK_R2C, false>();
  else if (kind == LK_C2R && !tstore) *out = make_line_kernel64<LOGL, true, LK_C2R, false>();
  else return false;
  return true;
}

template <int... Ls>
static bool cols64_dispatch(int logl, int kind, bool tstore, LineKernel* out, std::integer_sequence<int, Ls...>) {
  bool ok = false;
  ((logl == Ls ? (void)(ok = cols64_one<Ls>(kind, tstore, out)) : (void)0), ...);
  return ok;
}

bool get_cols64(int logl, int kind, bool tstore, LineKernel* out) {
  if (logl < 0 || logl > COLS_MAX_LOG64) return false;
  return cols64_dispatch(logl, kind, tstore, out, std::make_integer_sequence<int, COLS_MAX_LOG64 + 1>{});
}

}  // namespace agb
