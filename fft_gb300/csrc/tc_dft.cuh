// Split-precision tensor-core DFT-16 butterflies (tcgen05, TMEM) for the
// line-FFT kernel's "TC" form.
//
// In a radix-16 Stockham stage every thread owns one butterfly: 16 complex
// inputs x_n (already twiddled) whose DFT-16 it needs.  The TC form computes
// the butterflies of the whole CTA as one matrix product per 128-row tile:
//
//     [Yr | Yi] = [Xr | Xi] * M,   M = [[Wr, Wi], [-Wi, Wr]]  (32 x 32 real)
//
// with W_nk = exp(-2 pi i nk/16).  Operands are split into FP16 pairs to keep
// FP32-level accuracy: each row a (32 values) is scaled by a power of two s so
// that max|a s| is in [1, 2), then  a s = ah + al / 2048  with ah, al FP16;
// M = Mh + Ml / 2048 likewise.  Two FP32 accumulators in TMEM collect
//     D1 = ah Mh,    D2 = ah Ml + al Mh
// (six 128x32x16 tcgen05.mma per tile) and the butterfly outputs are
// y = (D1 + D2 / 2048) / s.  The dropped al Ml term is 2^-22 relative.
//
// Operand tiles are K-major without swizzle: 8x8 FP16 "core matrices" of 128
// bytes, K-adjacent core matrices 128 B apart (leading byte offset), 8-row
// groups 512 B apart (stride byte offset).  One elected thread issues the
// MMAs and commits them to an mbarrier; every wait on it is bounded, and a
// timeout sets the kernel's error word instead of hanging.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

namespace agb {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, k) of a K-major no-swizzle tile with K = 32
__device__ __forceinline__ uint32_t tc_core_off(int row, int k) {
  return (uint32_t)(((row >> 3) * 4 + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)(128 >> 4) << 16;   // K-adjacent core matrices
  d |= (uint64_t)(512 >> 4) << 32;   // 8-row groups
  d |= (uint64_t)1 << 46;            // descriptor version (sm_100 family)
  return d;                           // layout type 0: no swizzle
}

// kind::f16, D = F32, A = B = F16, K-major both, N = 32, M = 128
constexpr uint32_t kTcIdesc = (1u << 4) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t taddr, uint64_t ad, uint64_t bd, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
      "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait on an mbarrier phase: polls until the phase completes or
// limit_ns of wall time (the %globaltimer clock) has passed, with a poll
// count cap besides; returns false on timeout.
__device__ __forceinline__ bool mbar_wait_ns(uint32_t mbar, uint32_t parity, uint64_t limit_ns) {
  const uint64_t t0 = global_ns();
  for (uint32_t it = 0; it < (1u << 30); it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity));
    if (done) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
  return false;
}

// the kernels' waits (tensor-core results, TMA tiles) give up after one second
constexpr uint64_t kWaitLimitNs = 1000000000ull;
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) { return mbar_wait_ns(mbar, parity, kWaitLimitNs); }

#define AFFT_TMEM_LD8(taddr, r)                                                                          \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"                  \
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), \
                 "=r"(r[7])                                                                              \
               : "r"(taddr))

// Per-CTA tensor-core state.  Shared tiles: the A operands alias the
// kernel's Stockham exchange buffer (same bytes per butterfly); the B
// operands (Mh, Ml) live in their own 4 KB.
struct TcState {
  unsigned char* a;       // NT tiles x (Ah 8 KB | Al 8 KB), aliases the exchange buffer
  unsigned char* b;       // Mh 2 KB | Ml 2 KB
  uint32_t mbar;          // shared address of the mbarrier
  uint32_t tmem;          // TMEM base (64 columns per tile)
  uint32_t phase;         // parity of the next mbarrier phase
  int* err;               // error word (global), set on timeout
};

// Compute y = DFT16(x) for this thread's butterfly (row `row` of the CTA's
// butterfly list), cooperatively with the whole CTA.  All threads must call
// it at the same point.  NT = number of 128-row tiles (threads / 128).
template <int NT>
__device__ __forceinline__ void tc_dft16(float2 (&x)[16], int row, TcState& S) {
  // 1. row scale: a power of two with max|a s| in [1, 2)
  float m = 0.f;
#pragma unroll
  for (int n = 0; n < 16; n++) m = fmaxf(m, fmaxf(fabsf(x[n].x), fabsf(x[n].y)));
  int e = ((__float_as_int(m) >> 23) & 0xff) - 127;
  e = max(-100, min(100, e));
  const float s = __int_as_float((127 - e) << 23);
  const float inv_s = __int_as_float((127 + e) << 23);
  // 2. split and write the row into the A tiles (16-byte chunks of 8 values)
  const int tile = row >> 7, r = row & 127;
  unsigned char* ah = S.a + tile * 16384;
  unsigned char* al = ah + 8192;
#pragma unroll
  for (int g = 0; g < 4; g++) {
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
      uint32_t hp = 0, lp = 0;
#pragma unroll
      for (int h2 = 0; h2 < 2; h2++) {
        const int j = 8 * g + i + h2;
        const float a = (j < 16 ? x[j].x : x[j - 16].y) * s;
        const __half h = __float2half_rn(a);
        const __half l = __float2half_rn((a - __half2float(h)) * 2048.f);
        hp |= (uint32_t)__half_as_ushort(h) << (16 * h2);
        lp |= (uint32_t)__half_as_ushort(l) << (16 * h2);
      }
      hw[i >> 1] = hp;
      lw[i >> 1] = lp;
    }
    *(uint4*)(ah + tc_core_off(r, 8 * g)) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *(uint4*)(al + tc_core_off(r, 8 * g)) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  // 3. one thread issues 6 MMAs per tile and commits them
  if (threadIdx.x == 0) {
    const uint32_t a0 = smem_u32(S.a), b0 = smem_u32(S.b);
#pragma unroll
    for (int t = 0; t < NT; t++) {
      const uint32_t ahs = a0 + t * 16384, als = ahs + 8192;
      const uint32_t d1 = S.tmem + t * 64, d2 = d1 + 32;
      tc_mma(d1, tc_desc(ahs), tc_desc(b0), 0);
      tc_mma(d1, tc_desc(ahs + 256), tc_desc(b0 + 256), 1);
      tc_mma(d2, tc_desc(ahs), tc_desc(b0 + 2048), 0);
      tc_mma(d2, tc_desc(ahs + 256), tc_desc(b0 + 2048 + 256), 1);
      tc_mma(d2, tc_desc(als), tc_desc(b0), 1);
      tc_mma(d2, tc_desc(als + 256), tc_desc(b0 + 256), 1);
    }
    tc_commit(S.mbar);
  }
  const bool ok = tc_wait(S.mbar, S.phase);
  S.phase ^= 1u;
  if (!ok && S.err) atomicExch(S.err, 1);
  asm volatile("tcgen05.fence::after_thread_sync;");
  // 4. read this row's accumulators (warp w owns TMEM lanes 32 (w % 4) ..)
  const uint32_t lane_base = (uint32_t)(((threadIdx.x >> 5) & 3) * 32) << 16;
  const uint32_t t1 = S.tmem + lane_base + tile * 64, t2 = t1 + 32;
  float y[32];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    uint32_t a[8], b[8];
    AFFT_TMEM_LD8(t1 + 8 * c, a);
    AFFT_TMEM_LD8(t2 + 8 * c, b);
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int i = 0; i < 8; i++)
      y[8 * c + i] = ok ? fmaf(__uint_as_float(b[i]), 1.f / 2048.f, __uint_as_float(a[i])) * inv_s : 0.f;
  }
#pragma unroll
  for (int k = 0; k < 16; k++) x[k] = make_float2(y[k], y[16 + k]);
  // the next writer of the A tiles (this stage's Stockham scatter) waits
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
}

}  // namespace agb
