// Registry entries of the FP64 line kernels (line_fft64.cuh).
#pragma once
#include "kernels.h"
#include "line_fft64.cuh"

namespace agb {

template <int LOGL, bool COLS, int KIND, bool TSTORE>
LineKernel make_line_kernel64() {
  constexpr int C = lines_per_cta64<LOGL, COLS>();
  LineKernel k{};
  k.fn = &line_fft64<LOGL, C, COLS, KIND, TSTORE>;
  k.grouped = nullptr;
  k.logl = LOGL;
  k.cols = COLS;
  k.kind = KIND;
  k.tstore = TSTORE;
  k.tc = 0;
  k.unit = 0;
  k.lines_per_cta = C;
  k.threads = Sched64<LOGL>::T * C;
  k.smem = (size_t)Smem64<(1 << LOGL), C, COLS>::ELEMS * sizeof(double2);
  k.halves = 1;
  k.stage_logl = LOGL;
  return k;
}

}  // namespace agb
