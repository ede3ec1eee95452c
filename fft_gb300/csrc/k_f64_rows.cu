// FP64 rows-mode line kernels, L = 2^0 .. 2^13: complex, real forward, real inverse
#include <utility>

#include "kernels64.h"

namespace agb {

template <int LOGL>
static bool rows64_one(int kind, LineKernel* out) {
  if (kind == LK_C2C) *out = make_line_kernel64<LOGL, false, LK_C2C, false>();
  else if (kind == LK_R2C) *out = make_line_kernel64<LOGL, false, LK_R2C, false>();
  else if (kind == LK_C2R) *out = make_line_kernel64<LOGL, false, LK_C2R, false>();
  else return false;
  return true;
}

template <int... Ls>
static bool rows64_dispatch(int logl, int kind, LineKernel* out, std::integer_sequence<int, Ls...>) {
  bool ok = false;
  ((logl == Ls ? (void)(ok = rows64_one<Ls>(kind, out)) : (void)0), ...);
  return ok;
}

bool get_rows64(int logl, int kind, LineKernel* out) {
  if (logl < 0 || logl > ROWS_MAX_LOG64) return false;
  return rows64_dispatch(logl, kind, out, std::make_integer_sequence<int, ROWS_MAX_LOG64 + 1>{});
}

}  // namespace agb
