// Host-side plans: a transform is compiled into a short list of kernel
// launches ("ops") over named buffers; executing a plan binds the buffers to
// the caller's pointers and launches the ops on one stream.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.h"

namespace agb {

enum Kind { K_C = 0, K_CI = 1, K_R = 2, K_RI = 3 };

// Buffers an op reads or writes.  Data pointers are bound at execution.
enum BufId { B_SRC_RE = 0, B_SRC_IM, B_DST_RE, B_DST_IM, B_SCR, B_NBUF };

struct Ref {
  int buf = B_SRC_RE;
  long long off = 0;  // floats from the buffer base
};

struct IOSpec {
  Ref re, im;
  long long es = 1, lo = 0, hi = 0;
  int qshift = 0;
  long long qmask = 0;
};

enum OpType { OP_LINE = 0, OP_REAL = 1, OP_REAL1 = 2, OP_COPY = 3 };

struct Op {
  int type = OP_LINE;
  LineKernel k{};
  LineParams p{};
  RealPassParams rp{};
  CopyParams cp{};
  IOSpec in, out;
  long long real_L = 0;  // real twiddle length of a fused line op
  long long grid = 0;
  int threads = 0;
  size_t smem = 0;
};

// Error state of the calling thread.
void set_error(int code, const std::string& msg);
void clear_error();

// Form flags, OR-ed into the format argument of the batched and describe
// entry points: split-precision tensor-core butterflies where eligible
// (FORM_TC), or FP64 data and arithmetic (FORM_F64, the afft_64_* path).
constexpr int FORM_TC = 0x100;
constexpr int FORM_F64 = 0x200;

struct Plan {
  int kind = K_C;
  bool has_tma = false;        // some op may take its TMA-fed kernel (its waits report through the error word)
  int format = 0;              // afft_split / afft_interleaved
  int form = 0;                // 0 plain FP32, FORM_TC split-precision tensor cores, FORM_F64 FP64
  int ndim = 1;
  long long dims[64] = {0};
  long long batch = 1;
  long long in_elems = 0;      // complex (or real) elements per array, one transform
  long long out_elems = 0;
  int device = 0;
  int sm_count = 0;            // SMs of the device (the pipelined kernels' grid bound)
  std::vector<Op> ops;
  long long scratch_elems = 0;   // scratch elements (floats, doubles in FP64 plans)
  long long real_L_of_op = 0;
  float* scratch = nullptr;
  cudaStream_t stream = nullptr;
  // device staging for host-resident data
  float* stage = nullptr;
  size_t stage_bytes = 0;
  // host-data pipeline: a plan for a chunk of the batch, so copies of one
  // chunk overlap the transform of the previous one
  std::unique_ptr<Plan> chunk;
  long long nchunks = 1;
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  std::vector<cudaEvent_t> ev;
  std::mutex mu;

  ~Plan();
  bool f64() const { return (form & FORM_F64) != 0; }
  size_t esize() const { return f64() ? sizeof(double) : sizeof(float); }   // bytes per element
  // Launch all ops on `stream`; pointers must be device-accessible.
  int launch(const float* src_re, const float* src_im, float* dst_re, float* dst_im,
             cudaStream_t stream);
};

// Plan variants the autotuner chooses between (tune.cu).  split: 0 the
// built-in four-step split of long axes, 1 the other half first; real_inv:
// 0 the fused paired pre-pass for long 1D real inverses where it applies,
// 1 the standalone pre-pass; cols_lsu: 0 TMA-loaded input tiles for the
// cols passes that have them, 1 the LSU loads; tc: 1 the tensor-core form
// (plans of the plain form only); cols_c: 8 or 32 lines per CTA for
// 256-point, 16 for 512-point complex cols passes instead of the default.
struct Tuning {
  int split = 0;
  int real_inv = 0;
  int cols_lsu = 0;   // 1: cols passes load their tiles through the LSU even where TMA applies
  int tc = 0;         // 1: the split-precision tensor-core form where a pass has one
  int cols_c = 0;     // lines per CTA of the 256- and 512-point complex cols passes (0: the default)
  int passes = 0;     // 1D complex axes of 2^20 points and more: 0 the built-in rule (three passes
                      // from 2^21), 2 two passes, 3 three passes
  int no_pipe = 0;    // 1: 1024- and 2048-point cols passes keep their one-tile-per-CTA kernels
  int no_plane = 0;   // the last two axes of complex N-D transforms where a plane-fused pass applies:
                      // 0 the built-in rule, 1 a pass each, 2 the plane pass at any plane count
};
// The tuned choice for a shape on the current device, if the autotuner has
// one (tuning it first when AFFT_GB300_AUTOTUNE=1); else the defaults.
Tuning tuned_choice(int kind, int ndim, const long long* dims, long long batch, int format);
// The tuned choice for a queue's transforms of one shape (split format),
// tuning it first (at a batch of about 2^24 elements) when none is known.
Tuning tuned_for_queue(int kind, int ndim, const long long* dims);

// Build a plan; returns nullptr and sets the error on failure.
// dry: build the op list only (no device calls, twiddle pointers null), for
// describing a plan without a GPU.
// tune: the variant to build; nullptr = the tuned choice for device plans of
// the plain form, the defaults otherwise.
std::unique_ptr<Plan> build_plan(int kind, int ndim, const long long* dims, long long batch,
                                 int format, bool dry = false, int form = 0, const Tuning* tune = nullptr);
// TC form: the DFT-16 matrix tiles (Mh, Ml) and the per-device error word
const __half* tc_matrix_table();
int* tc_error_word();

// The tensor maps of a cols pass's TMA-fed kernel for the bound arrays, or
// false when they do not meet its alignment rules (launch k.fn instead).
bool tma_tile(const LineParams& p, const LineKernel& k, TmaTile* tm);
// the paired R2C pass's three maps over its input pairs, when the arrays allow them
bool tma_paired(const LineParams& p, const LineKernel& k, PairedTma* pt);

// Whether every table an op's kernel reads is present (device plans).
bool op_tables_ok(const Op& op);

// JSON description of a plan's ops (kernel shapes, grids, address specs).
std::string describe_plan(const Plan& P);

// Validation shared by memsize and create: 0 on success, else error code.
int validate_shape(int ndim, const size_t* dim, int* ndim_out, long long* dims_out);

// Device twiddle tables (FP64-computed, rounded once), cached per device.
const float2* stage_twiddles(int logl);
const float2* real_twiddles(long long L);         // W_{2L}^k, k < L
void fourstep_tables(long long N, const float2** hi, const float2** lo, int* lo_bits);
// The four-step twiddle as one matrix, W_N^{t2 k} at [t2 * L1 + k], for
// N <= kFullTableMax (nullptr above): one coalesced load per element.  It
// covers every four-step axis a plan builds (up to 2^22 points: 32 MB), so
// each plan's four-step twiddle is computed in FP64 and rounded once; the
// hi/lo product form remains for the no-allocation entry point's fixed
// arrays.
#ifndef AFFT_FULL_TABLE_LOG
#define AFFT_FULL_TABLE_LOG 22
#endif
constexpr long long kFullTableMax = 1LL << AFFT_FULL_TABLE_LOG;
const float2* fourstep_full_table(long long N, long long L2);
// FP64 tables (computed in FP64, no rounding): stage twiddles of the FP64
// line kernels, W_{2L}^k (k < L), and the four-step matrix W_N^{t2 k} at
// [t2 * L1 + k] for any N
const double2* stage_twiddles64(int logl);
const double2* real_twiddles64(long long L);
const double2* fourstep_full_table64(long long N, long long L2);
std::vector<double2> stage_table64_host(int logl);
std::vector<float2> fourstep_full_table_host(long long N, long long L2);
// The same tables on the host, without touching the device.
std::vector<float2> stage_table_host(int logl);
void fourstep_table_host(long long N, std::vector<float2>* hi, std::vector<float2>* lo, int* lo_bits);

}  // namespace agb
