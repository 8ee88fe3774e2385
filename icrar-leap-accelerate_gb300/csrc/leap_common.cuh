// Shared device-side definitions for the LEAP calibration kernels (sm_103a).
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace leapgb {

// Speed of light in m/s (icrar::constants::speed_of_light, LA/common/constants.h:35).
constexpr double kSpeedOfLight = 299792458.0;
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kTwoPi = 6.283185307179586476925286766559005768;

// Device error word bits, set by kernels whose bounded waits give up.
constexpr int kDevErrTimeout = 1;
constexpr int kDevErrBadShape = 2;

// Upper bound on try_wait polls of one mbarrier phase before a kernel gives up.
// Each poll suspends for up to the hardware time hint, so this is seconds.
constexpr uint32_t kMaxWaitPolls = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- mbarrier helpers (PTX ISA "mbarrier") ----
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on one phase of an mbarrier.  Returns false if it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_polls = kMaxWaitPolls) {
  for (uint32_t i = 0; i < max_polls; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  return false;
}

// Self-test of the timeout path: an mbarrier phase that nothing completes,
// waited for with a bound of `polls`; the kernel records the timeout in the
// error word exactly as the production kernels do, and returns.
static __global__ void selftest_bounded_wait(uint32_t polls, int* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && !mbar_wait_bounded(&bar, 0, polls)) atomicOr(err, kDevErrTimeout);
}

// Two-dimensional tiled TMA load global -> shared through a tensor map,
// completing on an mbarrier.  x (the inner coordinate, in elements) times the
// element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void* smem_dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(smem_dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// One-dimensional bulk copy global -> shared, completing on an mbarrier
// (cp.async.bulk; both addresses 16-byte aligned, size a multiple of 16).
__device__ __forceinline__ void bulk_copy_g2s(void* smem_dst, const void* gmem_src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Twiddle table: kTwiddleBits-bit index of a turn -> (cos, sin) of 2*pi*i/2^kTwiddleBits,
// rounded to FP32 from FP64 values on the host.
constexpr int kTwiddleBits = 10;
constexpr int kTwiddleSize = 1 << kTwiddleBits;

// exp(2*pi*i*turns) for a 32-bit fixed-point fraction of a turn, to about 1e-7
// absolute: the top kTwiddleBits bits pick a table entry; the remaining 22 bits
// are an angle delta in [0, 2*pi/1024) (exact in a float mantissa), whose sine
// and cosine are the first Taylor terms (truncation below 6e-11); the table
// entry is then rotated by delta.  The table lives in shared memory.
__device__ __forceinline__ void twiddle_turns(uint32_t turns, const float2* __restrict__ tab, float& c, float& s) {
  constexpr float kStep = 6.28318530717958647692f / kTwiddleSize;
  const float2 t = tab[turns >> (32 - kTwiddleBits)];
  const uint32_t fbits = ((turns << kTwiddleBits) >> 9) | 0x3F800000u;
  const float d = fmaf(__uint_as_float(fbits), kStep, -kStep);
  const float d2 = d * d;
  const float cd = fmaf(d2, -0.5f, 1.0f);
  const float sd = d * fmaf(d2, -0.16666667f, 1.0f);
  c = fmaf(t.x, cd, -t.y * sd);
  s = fmaf(t.y, cd, t.x * sd);
}

// Knuth's TwoSum: a + b = s + e exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (ah + al) * (bh + bl) = p + e to about 2^-44 relative (TwoProd of the high parts).
__device__ __forceinline__ void df_prod(float ah, float al, float bh, float bl, float& p, float& e) {
  p = ah * bh;
  e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
}

// k[0..5] = (L, M, N) as (hi, lo) float pairs, x[0..5] = (u, v, w) likewise.
// Returns frac(L*u + M*v + N*w) as a 2^-32 fixed-point fraction of a turn,
// computed in double-float arithmetic (error ~1e-12 turns for |sum| < 1e4).
__device__ __forceinline__ uint32_t df_dot3_turns_u32(const float* k, const float* x) {
  float p1, e1, p2, e2, p3, e3, s, t1, t2;
  df_prod(k[0], k[1], x[0], x[1], p1, e1);
  df_prod(k[2], k[3], x[2], x[3], p2, e2);
  df_prod(k[4], k[5], x[4], x[5], p3, e3);
  two_sum(p1, p2, s, t1);
  two_sum(s, p3, s, t2);
  const float lo = (e1 + e2) + (e3 + (t1 + t2));
  const float f = s - rintf(s);  // exact, in [-0.5, 0.5]
  return static_cast<uint32_t>(__float2int_rn(f * 4294967296.0f)) +
         static_cast<uint32_t>(__float2int_rn(lo * 4294967296.0f));
}

// Fractional part of x (turns) as a rounded 2^-32 fixed-point value.
__device__ __forceinline__ uint32_t frac_turns_u32(double x) {
  const double f = x - rint(x);  // in [-0.5, 0.5]
  return static_cast<uint32_t>(static_cast<long long>(rint(f * 4294967296.0)));
}

}  // namespace leapgb
