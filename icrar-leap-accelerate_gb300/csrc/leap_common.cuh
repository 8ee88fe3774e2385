// Shared device-side definitions for the LEAP calibration kernels (sm_103a).
#pragma once

#include <cstdint>
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
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kMaxWaitPolls; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  return false;
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

// ---- packed FP32x2 arithmetic (sm_100+) ----
__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void unpack2(unsigned long long v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long ffma2(unsigned long long a, unsigned long long b,
                                                    unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// Phase in turns held as an unsigned 32-bit fraction of a turn -> angle in [-pi, pi).
// The top 23 bits (with the sign bit flipped, i.e. +half a turn) become the
// mantissa of a float in [1, 2); 2*pi*(f - 1.5) is then the angle.
__device__ __forceinline__ float turns_u32_to_angle(uint32_t turns) {
  const uint32_t bits = ((turns >> 9) ^ 0x00400000u) | 0x3F800000u;
  return fmaf(__uint_as_float(bits), 6.28318530717958647692f, -9.42477796076937971538f);
}

// Fractional part of x (turns) as a rounded 2^-32 fixed-point value.
__device__ __forceinline__ uint32_t frac_turns_u32(double x) {
  const double f = x - rint(x);  // in [-0.5, 0.5]
  return static_cast<uint32_t>(static_cast<long long>(rint(f * 4294967296.0)));
}

}  // namespace leapgb
