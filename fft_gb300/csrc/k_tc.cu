// Split-precision tensor-core form (tcgen05 DFT-16 butterflies) of the line
// kernel, for the lengths whose stages are all radix-16 with one butterfly
// per thread and 256 or 512 threads per CTA: rows c2c L = 256 and 4096, cols
// c2c L = 256 (plain and with the four-step transposing store).
#include "kernels.h"
namespace agb {
bool get_tc_kernel(int logl, bool cols, bool tstore, LineKernel* out) {
  if (!cols && !tstore && logl == 8) { *out = make_line_kernel<8, false, LK_C2C, false, true>(); return true; }
  if (!cols && !tstore && logl == 12) { *out = make_line_kernel<12, false, LK_C2C, false, true>(); return true; }
  if (cols && !tstore && logl == 8) { *out = make_line_kernel<8, true, LK_C2C, false, true>(); return true; }
  if (cols && tstore && logl == 8) { *out = make_line_kernel<8, true, LK_C2C, true, true>(); return true; }
  return false;
}
}  // namespace agb
