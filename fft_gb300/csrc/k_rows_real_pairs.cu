// rows-mode real line FFTs whose real side is accessed as float2 pairs: the
// C2R output for L = 2^8 .. 2^14 (shorter lines take the warp-staged
// accesses), the R2C input for L = 2^12 .. 2^14
#include <utility>

#include "kernels.h"

namespace agb {

template <int LOGL>
static bool rows_real_pairs_one(int kind, LineKernel* out) {
  if constexpr (LOGL >= 12) {
    if (kind == LK_R2C) {
      *out = make_line_kernel<LOGL, false, LK_R2C, false, false, 2>();
      return true;
    }
  }
  if (kind != LK_C2R) return false;
  *out = make_line_kernel<LOGL, false, LK_C2R, false, false, 2>();
  return true;
}

template <int... Ls>
static bool rows_real_pairs_dispatch(int logl, int kind, LineKernel* out, std::integer_sequence<int, Ls...>) {
  bool ok = false;
  ((logl == Ls + 8 ? (void)(ok = rows_real_pairs_one<Ls + 8>(kind, out)) : (void)0), ...);
  return ok;
}

bool get_rows_real_pairs(int logl, int kind, LineKernel* out) {
  if (logl < 8 || logl > ROWS_MAX_LOG) return false;
  return rows_real_pairs_dispatch(logl, kind, out, std::make_integer_sequence<int, ROWS_MAX_LOG - 7>{});
}

}  // namespace agb
