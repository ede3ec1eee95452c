// 1024- and 2048-point cols passes in the persistent TMA-pipelined form (line_fft_pipe)
#include "kernels.h"
namespace agb {
bool get_cols_pipe(int logl, int kind, LineKernel* out) {
#if AFFT_PIPE10
  if (logl == 10) {
    switch (kind) {
      case LK_C2C: *out = make_pipe_kernel<10, LK_C2C>(); return true;
      case LK_C2R: *out = make_pipe_kernel<10, LK_C2R>(); return true;
    }
    return false;
  }
#endif
  if (logl != 11) return false;
  switch (kind) {
    case LK_C2C: *out = make_pipe_kernel<11, LK_C2C>(); return true;
#if AFFT_PIPE_R2C
    case LK_R2C: *out = make_pipe_kernel<11, LK_R2C>(); return true;
#endif
    case LK_C2R: *out = make_pipe_kernel<11, LK_C2R>(); return true;
  }
  return false;
}
bool get_cols_pipe_tstore(int logl, LineKernel* out) {
#if AFFT_PIPE10_TSTORE
  if (logl == 10) {
    *out = make_pipe_kernel<10, LK_C2C, true>();
    return true;
  }
#endif
  return false;
}
}  // namespace agb
