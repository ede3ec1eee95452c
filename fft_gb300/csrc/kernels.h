// Registry of the line-FFT kernel instantiations (one translation unit per
// family so they compile in parallel).
#pragma once
#include "line_fft.cuh"
#include "line_fft_pipe.cuh"
#include "plane_fft.cuh"

namespace agb {

typedef void (*LineKernelFn)(LineParams);
typedef void (*GroupedKernelFn)(const Segment*, const int*, long long);
typedef void (*LineKernelTmaFn)(LineParams, TmaTile);
typedef void (*LineKernelPipeFn)(LineParams, TmaTile, TmaTile, long long);
typedef void (*LineKernelPairedFn)(LineParams, PairedTma);
typedef void (*LineKernelTmaBulkFn)(LineParams, TmaTile, TmaTile);

struct LineKernel {
  LineKernelFn fn;
  GroupedKernelFn grouped;
  int logl;
  int cols;            // thread mapping: 1 = across lines, 0 = along a line
  int kind;            // LK_C2C / LK_R2C / LK_C2R
  int tstore;          // store with the along-line mapping (four-step pass A)
  int tc;              // split-precision tensor-core butterflies
  int unit;            // rows: unit element strides, 1 split, 2 pairs (c2c interleaved, or the
                       // real side of R2C / C2R); cols: pairs, bit 0 input, bit 1 output
  int lines_per_cta;   // C
  int threads;         // T * C
  size_t smem;         // bytes of dynamic shared memory
  int halves;          // CTAs per tile of C lines (2: the split R2C pass)
  int stage_logl;      // log2 length of the stage twiddle table the kernel reads
  LineKernelTmaFn tma; // the same pass with its input tile loaded by TMA (cols passes over
                       // split planes), or null
  GroupedKernelFn grouped_tma;   // its grouped form (queue segments with tensor maps), or null
  LineKernelTmaBulkFn tma_bulk = nullptr;   // the TMA-fed form that also stores by TMA
                                            // (line_fft_tma_bulk), or null
  LineKernelPipeFn pipe = nullptr;   // the persistent TMA-pipelined form (line_fft_pipe), or null;
                                     // launched on at most one CTA per SM with the tile count
  size_t pipe_smem = 0;              // its dynamic shared memory (raw tile + exchange buffer)
  int pipe_ctas = 1;                 // its resident CTAs per SM (the grid is at most that many per SM)
  GroupedKernelFn grouped_pipe = nullptr;   // its queue form (segments with tensor maps), or null
  LineKernelPairedFn paired_tma = nullptr;  // the paired R2C pass over input pairs with TMA-loaded tiles
                                            // (line_fft_paired_tma), or null
  size_t paired_smem = 0;                   // its dynamic shared memory
  int plane_log1 = 0;                // plane kernels (plane_fft): log2 of the rows per plane (the column
                                     // axis); logl is then log2 of the row length; 0 for line kernels
};

constexpr int ROWS_MAX_LOG = 14;   // rows mode: one CTA up to 16384 points
constexpr int COLS_MAX_LOG = 11;   // cols mode: one CTA up to 2048 points

// rows: kind in {LK_C2C, LK_R2C, LK_C2R}; cols: tstore only with LK_C2C
bool get_line_kernel(int logl, bool cols, int kind, bool tstore, LineKernel* out);
// rows c2c with unit element strides (split data): compile-time offsets
bool get_rows_c2c_unit(int logl, bool tc, LineKernel* out);
// rows c2c on interleaved pairs with unit pair strides (float2 accesses)
bool get_rows_c2c_iunit(int logl, LineKernel* out);
// cols c2c on interleaved pairs (im right after re, even element stride):
// pairs bit 0 = input, bit 1 = output (the kernels' UNIT in cols mode), for
// lines of 2^5 .. 2^11 points; the transposing store with pairs 1 or 3
bool get_cols_c2c_pairs(int logl, bool tstore, int pairs, LineKernel* out);
// the transposing-store half of it (k_cols_pairs_ts.cu)
bool get_cols_c2c_pairs_tstore(int logl, int pairs, LineKernel* out);
// the paired R2C pass (four-step pass B of a long 1D real forward) with its
// input as float2 pairs, lines of 2^7 .. 2^11 points; at 2^9 and 2^10 points
// with the TMA-fed form (paired_tma) too
bool get_r2c_paired_pairs(int logl, LineKernel* out);
// the paired C2R pass (four-step pass A of a long 1D real inverse) with its
// output as float2 pairs, lines of 2^7 .. 2^9 points
bool get_c2r_paired_pairs(int logl, LineKernel* out);
// rows C2R (lines of 2^8 .. 2^14 points) and R2C (2^12 .. 2^14) whose real
// side (C2R output, R2C input) is written / read as pairs with unit pair
// stride (float2 accesses)
bool get_rows_real_pairs(int logl, int kind, LineKernel* out);

// FP64 kernels (line_fft64.cuh, k_f64_*.cu): rows {C2C, R2C, C2R} up to
// 2^13 points, cols {C2C (also with the transposing store), R2C, C2R} up to
// 2^11; `grouped` is null (the multi-transform queue is FP32 only)
bool get_line_kernel64(int logl, bool cols, int kind, bool tstore, LineKernel* out);
bool get_rows64(int logl, int kind, LineKernel* out);
bool get_cols64(int logl, int kind, bool tstore, LineKernel* out);

// cols passes {C2C, R2C, C2R} of 2^8 .. 2^11 points whose input tile is
// loaded by TMA (line_fft_tma); out->tma set, the rest as the LSU kernel
// of the same shape (the R2C pass of 2^11 points unsplit: one CTA per tile)
bool get_cols_tma(int logl, int kind, LineKernel* out);
// the transposing-store complex cols passes (four-step pass A) of 2^8 ..
// 2^10 points with TMA-loaded input tiles (k_cols_tma_ts.cu)
bool get_cols_tma_tstore(int logl, LineKernel* out);
// complex cols passes over interleaved input pairs (pairs bit 0 set: 1 or
// 3), plain or with the transposing store, 2^8 and 2^9 points, with TMA
// loads of the interleaved tile (k_cols_tma_pairs.cu)
bool get_cols_tma_pairs(int logl, bool tstore, int pairs, LineKernel* out);

// 2048-point cols passes {C2C, C2R, and R2C unsplit when AFFT_PIPE_R2C} and
// 1024-point {C2C, C2R} over split planes in the persistent TMA-pipelined
// form (k_cols_pipe.cu): out->pipe (and out->grouped_pipe) set, out->tma and
// out->fn the one-tile-per-CTA kernels of the same shape
bool get_cols_pipe(int logl, int kind, LineKernel* out);
// the 1024-point four-step pass A (transposing store, split planes) in that form
bool get_cols_pipe_tstore(int logl, LineKernel* out);

// plane-fused passes (plane_fft.cuh, k_plane*.cu): the last two axes of a
// complex N-D transform, planes of 2^log1 rows x 2^log2 points with
// 8 <= log1 + log2 <= 14 and both in [4, 9]
// (unit 1 split planes, 2 interleaved pairs), by the per-unit, per-size
// lookups of k_plane*.cu
bool get_plane_kernel(int log1, int log2, int unit, LineKernel* out);
bool get_plane_split_small(int log1, int log2, LineKernel* out);   // 2^8 .. 2^11 points
bool get_plane_split_big(int log1, int log2, LineKernel* out);     // 2^12 .. 2^14 points
bool get_plane_pairs_small(int log1, int log2, LineKernel* out);
bool get_plane_pairs_big(int log1, int log2, LineKernel* out);

// cols c2c passes (not transposing) with another tile width, for the
// autotuner: 256 points in 8 or 32 lines, 512 points in 16; TMA-fed
// variant included (k_cols_alt.cu)
bool get_cols_c2c_alt(int logl, int lines, LineKernel* out);

// split-precision tensor-core form: rows c2c L = 256 or 4096, cols c2c L = 256
bool get_tc_kernel(int logl, bool cols, bool tstore, LineKernel* out);

// per-family lookups (defined in k_*.cu)
bool get_rows_c2c(int logl, LineKernel* out);
bool get_rows_r2c(int logl, LineKernel* out);
bool get_rows_c2r(int logl, LineKernel* out);
bool get_cols_c2c(int logl, bool tstore, LineKernel* out);
bool get_cols_real(int logl, int kind, LineKernel* out);

// Lines per cols-mode CTA, measured per length on GB300: 32 lines up to
// 128 points, 16 for 256 and 512 (256/512 threads, several CTAs per SM),
// 8 for 1024 and 2048 (narrower tiles lose DRAM locality: 32-byte row
// segments are the floor).  Complex 512-point cols passes take 8 lines
// (32 KB tiles, 4 CTAs per SM): 4-6% faster for four-step 2^17/2^18 axes;
// the real 512-point cols passes measured 7% slower that way and keep 16.
template <int LOGL, bool COLS>
constexpr int lines_per_cta() {
  constexpr int T = Sched<LOGL>::T;
  if constexpr (COLS) return LOGL <= 7 ? 32 : (LOGL <= 9 ? 16 : 8);
  else return T >= 256 ? 1 : 256 / T;
}

// lines per CTA of the split R2C pass
#ifndef AFFT_HALF_C
#define AFFT_HALF_C 8
#endif
// lines per CTA of the complex and of the real 512-point cols passes
#ifndef AFFT_COLS_C9
#define AFFT_COLS_C9 8
#endif
#ifndef AFFT_COLS_RC9
#define AFFT_COLS_RC9 16
#endif
template <int LOGL, bool COLS, int KIND>
constexpr int lines_per_cta_k() {
  if constexpr (KIND == LK_R2C_HALF) return AFFT_HALF_C;
  else if constexpr (COLS && LOGL == 9 && KIND == LK_C2C) return AFFT_COLS_C9;
  else if constexpr (COLS && LOGL == 9 && (KIND == LK_R2C || KIND == LK_C2R)) return AFFT_COLS_RC9;
  else return lines_per_cta<LOGL, COLS>();
}

// CC: lines per CTA when not the measured default of lines_per_cta_k
template <int LOGL, bool COLS, int KIND, bool TSTORE, bool TC = false, int UNIT = 0, int CC = 0>
LineKernel make_line_kernel() {
  constexpr int C = CC ? CC : lines_per_cta_k<LOGL, COLS, KIND>();
  static_assert(!TC || (size_t)LineSmem<LOGL, C, COLS, TSTORE, TC>::FLOAT2S * 8 >= (size_t)(Sched<LOGL>::T * C / 128) * 16384,
                "TC operand tiles must fit in the exchange buffer");
  LineKernel k;
  k.fn = &line_fft<LOGL, C, COLS, KIND, TSTORE, TC, UNIT>;
  k.tma = nullptr;
  k.grouped_tma = nullptr;
  k.grouped = &line_fft_grouped<LOGL, C, COLS, KIND, TSTORE, TC, UNIT>;
  k.tc = TC;
  k.unit = UNIT;
  // the split R2C pass transforms lines of 2^(LOGL+1) points with stages of 2^LOGL
  k.logl = KIND == LK_R2C_HALF ? LOGL + 1 : LOGL;
  k.cols = COLS;
  k.kind = KIND == LK_R2C_HALF ? LK_R2C : KIND;
  k.halves = KIND == LK_R2C_HALF ? 2 : 1;
  k.stage_logl = LOGL;
  k.tstore = TSTORE;
  k.lines_per_cta = C;
  k.threads = Sched<LOGL>::T * C;
  k.smem = (size_t)LineSmem<LOGL, C, COLS, TSTORE, TC>::FLOAT2S * sizeof(float2);
  return k;
}

// a cols pass with its TMA-fed variant (CC: lines per CTA, 0 = the default)
template <int LOGL, int KIND, int CC = 0, bool TSTORE = false, int UNIT = 0>
LineKernel make_tma_kernel() {
  constexpr int C = CC ? CC : lines_per_cta_k<LOGL, true, KIND>();
  static_assert((size_t)LineSmem<LOGL, C, true, TSTORE, false>::FLOAT2S * sizeof(float2) >=
                    (size_t)2 * (1 << LOGL) * C * sizeof(float),
                "the input tile fits the exchange buffer it aliases");
  static_assert(C * sizeof(float) % 16 == 0, "tile columns span whole 16-byte units");
  LineKernel k = make_line_kernel<LOGL, true, KIND, TSTORE, false, UNIT, C>();
  k.tma = &line_fft_tma<LOGL, C, KIND, TSTORE, UNIT>;
  k.grouped_tma = &line_fft_grouped<LOGL, C, true, KIND, TSTORE, false, UNIT, true>;
  if constexpr (!TSTORE && UNIT == 0 &&
                ((KIND == LK_C2C &&
                  ((LOGL == 10 && AFFT_TMA_BULK10) || (LOGL == 9 && AFFT_TMA_BULK9) || (LOGL == 8 && AFFT_TMA_BULK8))) ||
                 (KIND == LK_C2R && ((LOGL == 10 && AFFT_TMA_BULK_C2R10) || (LOGL == 9 && AFFT_TMA_BULK_C2R9) ||
                                     (LOGL == 8 && AFFT_TMA_BULK_C2R8)))))
    k.tma_bulk = &line_fft_tma_bulk<LOGL, C, KIND>;
  return k;
}

// the paired R2C pass over input pairs, with its TMA-fed form
template <int LOGL>
LineKernel make_paired_tma_kernel() {
  LineKernel k = make_line_kernel<LOGL, true, LK_R2C_PAIRED, false, false, 1>();
  constexpr int C = lines_per_cta_k<LOGL, true, LK_R2C_PAIRED>(), H = C / 2, L2 = 1 << LOGL;
  k.paired_tma = &line_fft_paired_tma<LOGL, C>;
  const size_t raw = (size_t)L2 * (2 * H + 2 * H + 4 + 4) * sizeof(float);
  k.paired_smem = raw > k.smem ? raw : k.smem;   // the raw tile aliases the exchange buffer
  return k;
}

// a plane pass: PPC planes per CTA, D1 D2 / 16 threads each
template <int LOG1, int LOG2, int UNIT>
LineKernel make_plane_kernel() {
  using PS = PlaneShape<LOG1, LOG2>;
  LineKernel k;
  k.fn = &plane_fft<LOG1, LOG2, UNIT>;
  k.grouped = &plane_fft_grouped<LOG1, LOG2, UNIT>;
  k.tma = nullptr;
  k.grouped_tma = nullptr;
  k.logl = LOG2;
  k.plane_log1 = LOG1;
  k.cols = 0;
  k.kind = LK_C2C;
  k.tstore = 0;
  k.tc = 0;
  k.unit = UNIT;
  k.lines_per_cta = PS::PPC * PS::D1;   // rows per CTA: PPC planes of D1 rows
  k.threads = PS::NT;
  k.smem = (size_t)PS::FLOAT2S * sizeof(float2);
  k.halves = 1;
  k.stage_logl = LOG2;
  return k;
}

// a 1024- or 2048-point cols pass with its pipelined form (8 lines per tile;
// AFFT_PIPE_C at 2048 points)
template <int LOGL, int KIND, bool TSTORE = false>
LineKernel make_pipe_kernel() {
  constexpr int C = LOGL == 11 ? AFFT_PIPE_C : 8;
  LineKernel k = make_tma_kernel<LOGL, KIND, C, TSTORE>();
  k.pipe = &line_fft_pipe<LOGL, C, KIND, TSTORE>;
  k.grouped_pipe = TSTORE ? nullptr : &line_fft_pipe_grouped<LOGL, C, KIND>;
  static_assert(LOGL == 11 || LOGL == 10, "the pipelined kernels are built for 1024- and 2048-point lines");
  k.pipe_smem = ((size_t)2 * (1 << LOGL) + pipe_rows<LOGL>()) * C * sizeof(float);   // raw tile + exchange rows
  k.pipe_ctas = 1024 / (Sched<LOGL>::T * C);
  return k;
}

}  // namespace agb
