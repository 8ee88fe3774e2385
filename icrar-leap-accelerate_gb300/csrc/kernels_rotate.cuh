// Rotate + average kernels (the hot path).
//
// Reference semantics (CpuLeapCalibrator::RotateVisibilities,
// LA/algorithm/cpu/CpuLeapCalibrator.cc:181-217; g_RotateVisibilities,
// LA/algorithm/cuda/CudaLeapCalibrator.cu:305-400): for every row r of the
// integration and channel c
//     shift  = -2*pi*(w_rot[r] - w[r]) / lambda_c,   w_rot = (dd * uvw[r]).z
//     avg[r % nbl, p] += V[p, r, c] * exp(i*shift)   for every pol p
// where samples with a NaN in any pol are skipped.  Here NaN groups were
// zeroed when the integration was ingested, so they add exactly nothing.
//
// Differences in structure from the reference (same sums, new schedule):
//  * the visibilities are read-only and resident; nothing is written back;
//  * one launch handles many directions, so every visibility load is reused
//    by all the directions of a warp;
//  * lanes own baselines, loops run over (timestep, channel) in the
//    reference's order, and partial sums over (timestep, channel) slabs are
//    combined in a fixed order, so results are deterministic (no atomics).
#pragma once

#include "leap_common.cuh"
#include "kernels_pipe.cuh"

namespace leapgb {

struct RotateArgs {
  const void* vis;          // [channels][rows][pols] complex (float2 or double2)
  const double* uvw;        // [rows][3]
  const double* dd;         // [ndir][9] row-major direction matrices
  const double* lambda;     // [channels] c / (f0 + ch*df), as the reference computes it
  const double* inv_lambda; // [channels] 1 / lambda, rounded (all-FP64 form)
  const float2* twiddle;    // [kTwiddleSize] (cos, sin) table for the mixed form
  const float* uvw_f;       // [rows][6] (u, v, w) as (hi, lo) float pairs
  const float* dirk;        // [ndir][12] phase constants as (hi, lo) pairs: -(l, m, n-1)*f0/c, -(l, m, n-1)*df/c
  int64_t rows;
  int32_t channels, pols, nbl, timesteps, ndir;
  double f0, df;
  int32_t t_per_slab, c_per_slab, n_tslab, n_cslab;
  double2* out;             // nslab == 1: avg [ndir][pols][nbl]; else partial [nslab][ndir][pols][nbl]
  int* err;
};

template <typename T> struct VisScalar;
template <> struct VisScalar<float2> { using type = float; };
template <> struct VisScalar<double2> { using type = double; };

template <typename VisT>
__device__ __forceinline__ void load_sample(const VisT* __restrict__ p, double& re, double& im) {
  const VisT v = __ldg(p);
  re = static_cast<double>(v.x);
  im = static_cast<double>(v.y);
}

template <typename VisT>
__device__ __forceinline__ void load_sample_f(const VisT* __restrict__ p, float& re, float& im) {
  const VisT v = __ldg(p);
  re = static_cast<float>(v.x);
  im = static_cast<float>(v.y);
}

// ---------------------------------------------------------------------------
// All-FP64 form.  Lanes own baselines, a warp owns DPW directions, a block's
// warps share one baseline tile (so the visibility loads of one warp hit L1
// for the others).  The reference phase is shiftRad(c) = fl(shiftFactor /
// lambda_c) (CpuLeapCalibrator.cc:190-198), nearly linear in the channel index,
// so exp(i*shiftRad) is advanced channel to channel by one complex multiply with
// exp(i*shiftFactor*df/c_light) and re-seeded with an FP64 sincos every kSeed
// channels.  FP64 sincos runs at about 1/25 of the DFMA rate on GB300, so this
// removes it from the inner loop.
//
// The reference's own rounding matters here.  Its argument reaches thousands of
// radians for directions ~1 rad from the phase centre, where one unit in the last
// place is ~1e-12 rad, and lambda_c's rounding is the same for every row; the
// solve then moves the cal phases by ~5e-11 rad between two equally valid FP64
// roundings of the argument (shiftFactor * (1 / lambda_c) against shiftFactor /
// lambda_c).  So each channel's twiddle is corrected to the reference's own
// argument: fl(shiftFactor / lambda_c) from the rounded reciprocal and one
// FMA-exact remainder step (the correctly rounded quotient), minus the
// recurrence's phase seed + k * step, applied to first order (the difference is
// below 1e-11 rad, so its square is far below rounding).  shiftFactor itself is
// formed without fused operations, as the reference's expression is.
// ---------------------------------------------------------------------------
// kCheckNan: skip (row, channel) groups with a NaN in any pol inside the kernel
// (for callers whose visibilities did not go through the ingestion sanitiser).
template <typename VisT, int P, int DPW, bool kCheckNan = false>
__global__ void __launch_bounds__(128) rotate_average_fp64(RotateArgs a) {
  constexpr int NW = 4;
  constexpr int kSeed = 16;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int b = blockIdx.x * 32 + lane;
  const int d0 = (blockIdx.y * NW + warp) * DPW;
  const int slab = blockIdx.z;
  const int ts = slab / a.n_cslab, cs = slab % a.n_cslab;
  const int t_lo = ts * a.t_per_slab, t_hi = min(a.timesteps, t_lo + a.t_per_slab);
  const int c_lo = cs * a.c_per_slab, c_hi = min(a.channels, c_lo + a.c_per_slab);
  if (d0 >= a.ndir) return;
  const bool valid = b < a.nbl;

  double dd2[DPW][3];
#pragma unroll
  for (int j = 0; j < DPW; ++j) {
    const int d = min(d0 + j, a.ndir - 1);
    dd2[j][0] = __ldg(a.dd + 9 * d + 6);
    dd2[j][1] = __ldg(a.dd + 9 * d + 7);
    dd2[j][2] = __ldg(a.dd + 9 * d + 8);
  }
  double accr[DPW][P], acci[DPW][P];
#pragma unroll
  for (int j = 0; j < DPW; ++j)
#pragma unroll
    for (int p = 0; p < P; ++p) accr[j][p] = acci[j][p] = 0.0;

  const double inv_c = 1.0 / kSpeedOfLight;
  const VisT* vis = static_cast<const VisT*>(a.vis);
  if (valid) {
    for (int t = t_lo; t < t_hi; ++t) {
      const int64_t r = static_cast<int64_t>(t) * a.nbl + b;
      const double u = __ldg(a.uvw + 3 * r), v = __ldg(a.uvw + 3 * r + 1), w = __ldg(a.uvw + 3 * r + 2);
      double sf[DPW], st[DPW], wr[DPW], wi[DPW];
#pragma unroll
      for (int j = 0; j < DPW; ++j) {
        const double wrot =
            __dadd_rn(__dadd_rn(__dmul_rn(dd2[j][0], u), __dmul_rn(dd2[j][1], v)), __dmul_rn(dd2[j][2], w));
        sf[j] = __dmul_rn(-kTwoPi, __dadd_rn(wrot, -w));
        st[j] = sf[j] * (a.df * inv_c);
        sincos(st[j], &wi[j], &wr[j]);
      }
      for (int cb = c_lo; cb < c_hi; cb += kSeed) {
        const int ce = min(c_hi, cb + kSeed);
        double zr[DPW], zi[DPW], seed[DPW];
#pragma unroll
        for (int j = 0; j < DPW; ++j) {
          seed[j] = sf[j] / __ldg(a.lambda + cb);
          sincos(seed[j], &zi[j], &zr[j]);
        }
        for (int c = cb; c < ce; ++c) {
          const double lam = __ldg(a.lambda + c), rlam = __ldg(a.inv_lambda + c);
          const double k = static_cast<double>(c - cb);
          const VisT* src = vis + (static_cast<int64_t>(c) * a.rows + r) * P;
          double vr[P], vi[P];
#pragma unroll
          for (int p = 0; p < P; ++p) load_sample(src + p, vr[p], vi[p]);
          if (kCheckNan) {
            bool nan = false;
#pragma unroll
            for (int p = 0; p < P; ++p) nan |= isnan(vr[p]) || isnan(vi[p]);
            if (nan) {
#pragma unroll
              for (int p = 0; p < P; ++p) vr[p] = vi[p] = 0.0;
            }
          }
#pragma unroll
          for (int j = 0; j < DPW; ++j) {
            // The reference's argument fl(sf / lambda_c), and its difference from seed + k * step.
            const double q = sf[j] * rlam;
            const double arg = fma(fma(-q, lam, sf[j]), rlam, q);
            const double dlt = fma(-k, st[j], arg - seed[j]);
            const double tr = fma(-dlt, zi[j], zr[j]), ti = fma(dlt, zr[j], zi[j]);
#pragma unroll
            for (int p = 0; p < P; ++p) {
              accr[j][p] += vr[p] * tr - vi[p] * ti;
              acci[j][p] += vr[p] * ti + vi[p] * tr;
            }
            const double nr = zr[j] * wr[j] - zi[j] * wi[j];
            zi[j] = zr[j] * wi[j] + zi[j] * wr[j];
            zr[j] = nr;
          }
        }
      }
    }
  }
  if (!valid) return;
  const int64_t slab_off = static_cast<int64_t>(slab) * a.ndir * P * a.nbl;
#pragma unroll
  for (int j = 0; j < DPW; ++j) {
    const int d = d0 + j;
    if (d < a.ndir) {
#pragma unroll
      for (int p = 0; p < P; ++p)
        a.out[slab_off + (static_cast<int64_t>(d) * P + p) * a.nbl + b] = make_double2(accr[j][p], acci[j][p]);
    }
  }
}

// ---------------------------------------------------------------------------
// Mixed-precision form (direct loads).  Per (row, direction) the phase
//     turns(c) = -(w_rot - w) * (f0 + c*df) / c_light = A + c*B
// is formed in FP64 once per timestep and reduced to 32-bit fixed-point
// fractions of a turn; each channel then costs one integer multiply-add, the
// table twiddle of twiddle_turns (about 1e-7 absolute; the hardware sin/cos
// approximations, about 5e-7, are not accurate enough for nearly cancelling
// sums) and FP32 complex MACs.
// Sums run in FP32 over blocks of KB channels and are folded into Kahan
// (sum, compensation) pairs, written out as sum - compensation in FP64.
// ---------------------------------------------------------------------------
template <typename VisT, int P, int DPW>
__global__ void __launch_bounds__(128) rotate_average_mixed(RotateArgs a) {
  constexpr int NW = 4;
  constexpr int KB = 16;
  __shared__ float2 tab[kTwiddleSize];
  for (int i = threadIdx.x; i < kTwiddleSize; i += blockDim.x) tab[i] = __ldg(a.twiddle + i);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int b = blockIdx.x * 32 + lane;
  const int d0 = (blockIdx.y * NW + warp) * DPW;
  const int slab = blockIdx.z;
  const int ts = slab / a.n_cslab, cs = slab % a.n_cslab;
  const int t_lo = ts * a.t_per_slab, t_hi = min(a.timesteps, t_lo + a.t_per_slab);
  const int c_lo = cs * a.c_per_slab, c_hi = min(a.channels, c_lo + a.c_per_slab);
  if (d0 >= a.ndir) return;
  const bool valid = b < a.nbl;

  const double kA = a.f0 / kSpeedOfLight, kB = a.df / kSpeedOfLight;
  float sr[DPW][P], si[DPW][P], cr[DPW][P], ci[DPW][P];
#pragma unroll
  for (int j = 0; j < DPW; ++j)
#pragma unroll
    for (int p = 0; p < P; ++p) sr[j][p] = si[j][p] = cr[j][p] = ci[j][p] = 0.f;

  const VisT* vis = static_cast<const VisT*>(a.vis);
  if (valid) {
    for (int t = t_lo; t < t_hi; ++t) {
      const int64_t r = static_cast<int64_t>(t) * a.nbl + b;
      const double u = __ldg(a.uvw + 3 * r), v = __ldg(a.uvw + 3 * r + 1), w = __ldg(a.uvw + 3 * r + 2);
      uint32_t pa[DPW], pb[DPW];
#pragma unroll
      for (int j = 0; j < DPW; ++j) {
        const int d = min(d0 + j, a.ndir - 1);
        const double wrot = __ldg(a.dd + 9 * d + 6) * u + __ldg(a.dd + 9 * d + 7) * v + __ldg(a.dd + 9 * d + 8) * w;
        const double dw = wrot - w;
        pa[j] = frac_turns_u32(-dw * kA);
        pb[j] = frac_turns_u32(-dw * kB);
      }
      for (int cb = c_lo; cb < c_hi; cb += KB) {
        const int ce = min(c_hi, cb + KB);
        float pr[DPW][P], pi[DPW][P];
#pragma unroll
        for (int j = 0; j < DPW; ++j)
#pragma unroll
          for (int p = 0; p < P; ++p) pr[j][p] = pi[j][p] = 0.f;
        for (int c = cb; c < ce; ++c) {
          const VisT* src = vis + (static_cast<int64_t>(c) * a.rows + r) * P;
          float vr[P], vi[P];
#pragma unroll
          for (int p = 0; p < P; ++p) load_sample_f(src + p, vr[p], vi[p]);
#pragma unroll
          for (int j = 0; j < DPW; ++j) {
            float s, co;
            twiddle_turns(pa[j] + static_cast<uint32_t>(c) * pb[j], tab, co, s);
#pragma unroll
            for (int p = 0; p < P; ++p) {
              pr[j][p] = fmaf(vr[p], co, fmaf(-vi[p], s, pr[j][p]));
              pi[j][p] = fmaf(vr[p], s, fmaf(vi[p], co, pi[j][p]));
            }
          }
        }
#pragma unroll
        for (int j = 0; j < DPW; ++j)
#pragma unroll
          for (int p = 0; p < P; ++p) {
            float y = pr[j][p] - cr[j][p];
            float tt = sr[j][p] + y;
            cr[j][p] = (tt - sr[j][p]) - y;
            sr[j][p] = tt;
            y = pi[j][p] - ci[j][p];
            tt = si[j][p] + y;
            ci[j][p] = (tt - si[j][p]) - y;
            si[j][p] = tt;
          }
      }
    }
  }
  if (!valid) return;
  const int64_t slab_off = static_cast<int64_t>(slab) * a.ndir * P * a.nbl;
#pragma unroll
  for (int j = 0; j < DPW; ++j) {
    const int d = d0 + j;
    if (d < a.ndir) {
#pragma unroll
      for (int p = 0; p < P; ++p)
        a.out[slab_off + (static_cast<int64_t>(d) * P + p) * a.nbl + b] =
            make_double2(static_cast<double>(sr[j][p]) - static_cast<double>(cr[j][p]),
                         static_cast<double>(si[j][p]) - static_cast<double>(ci[j][p]));
    }
  }
}

// ---------------------------------------------------------------------------
// Reference-antenna baselines in FP64 (mixed form).  The solve reads pol 0 of
// the |I1| baselines through the reference antenna with weight one (cal1 =
// Ad1 * arg(avg[I1, 0])) and then multiplies cal1 by 2*pi, so an FP32 phase
// error on one of them reaches every antenna's cal phase ~7x amplified; on
// nearly cancelling sums FP32 products leave errors of 1e-6..1e-5 rad there.
// These rows are therefore accumulated in FP64 (the all-FP64 recurrence of
// rotate_average_fp64, pol 0 only), gathered by I1.  They are 1-2% of the rows
// and use the FP64 pipe, which the FP32 bulk kernel leaves idle, so the call
// launches this kernel on a second stream to overlap the two.
// Output: [nslab][ndir][nI1] double2 (nslab == 1: final).
// ---------------------------------------------------------------------------
template <typename VisT, int DPW>
__global__ void __launch_bounds__(128) refant_average_fp64(RotateArgs a, const int32_t* __restrict__ I1, int nI1,
                                                          double2* __restrict__ out) {
  constexpr int NW = 4;
  constexpr int kSeed = 16;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int k = blockIdx.x * 32 + lane;
  const int d0 = (blockIdx.y * NW + warp) * DPW;
  const int slab = blockIdx.z;
  const int ts = slab / a.n_cslab, cs = slab % a.n_cslab;
  const int t_lo = ts * a.t_per_slab, t_hi = min(a.timesteps, t_lo + a.t_per_slab);
  const int c_lo = cs * a.c_per_slab, c_hi = min(a.channels, c_lo + a.c_per_slab);
  if (d0 >= a.ndir || k >= nI1) return;
  int b = __ldg(I1 + k);
  if (b < 0) b += a.nbl;  // VectorRangeSelect wrap-around (LA/math/cpu/vector.h:97-104)

  double dd2[DPW][3];
#pragma unroll
  for (int j = 0; j < DPW; ++j) {
    const int d = min(d0 + j, a.ndir - 1);
    dd2[j][0] = __ldg(a.dd + 9 * d + 6);
    dd2[j][1] = __ldg(a.dd + 9 * d + 7);
    dd2[j][2] = __ldg(a.dd + 9 * d + 8);
  }
  double accr[DPW], acci[DPW];
#pragma unroll
  for (int j = 0; j < DPW; ++j) accr[j] = acci[j] = 0.0;
  const double inv_c = 1.0 / kSpeedOfLight;
  const VisT* vis = static_cast<const VisT*>(a.vis);
  for (int t = t_lo; t < t_hi; ++t) {
    const int64_t r = static_cast<int64_t>(t) * a.nbl + b;
    const double u = __ldg(a.uvw + 3 * r), v = __ldg(a.uvw + 3 * r + 1), w = __ldg(a.uvw + 3 * r + 2);
    double sf[DPW], wr[DPW], wi[DPW];
#pragma unroll
    for (int j = 0; j < DPW; ++j) {
      const double wrot = dd2[j][0] * u + dd2[j][1] * v + dd2[j][2] * w;
      sf[j] = -kTwoPi * (wrot - w);
      sincos(sf[j] * (a.df * inv_c), &wi[j], &wr[j]);
    }
    for (int cb = c_lo; cb < c_hi; cb += kSeed) {
      const int ce = min(c_hi, cb + kSeed);
      double zr[DPW], zi[DPW];
#pragma unroll
      for (int j = 0; j < DPW; ++j) sincos(sf[j] / __ldg(a.lambda + cb), &zi[j], &zr[j]);
      for (int c = cb; c < ce; ++c) {
        double vr, vi;
        load_sample(vis + (static_cast<int64_t>(c) * a.rows + r) * a.pols, vr, vi);
#pragma unroll
        for (int j = 0; j < DPW; ++j) {
          accr[j] += vr * zr[j] - vi * zi[j];
          acci[j] += vr * zi[j] + vi * zr[j];
          const double nr = zr[j] * wr[j] - zi[j] * wi[j];
          zi[j] = zr[j] * wi[j] + zi[j] * wr[j];
          zr[j] = nr;
        }
      }
    }
  }
  const int64_t slab_off = static_cast<int64_t>(slab) * a.ndir * nI1;
#pragma unroll
  for (int j = 0; j < DPW; ++j) {
    const int d = d0 + j;
    if (d < a.ndir) out[slab_off + static_cast<int64_t>(d) * nI1 + k] = make_double2(accr[j], acci[j]);
  }
}

// ---------------------------------------------------------------------------
// Reference-antenna baselines in compensated FP32 (mixed form, complex<float>
// input).  Same sums as refant_average_fp64, at about 1e-9 relative per term,
// on the FP32 pipe (GB300's FP64 rate is ~1/70 of FP32):
//  * phase: 64-bit fixed-point turns  pa + c*pb  (from FP64 A, B per timestep);
//  * twiddle: the top 10 bits pick a (cos, sin) entry held as (hi, lo) float
//    pairs (df_tab), the next 24 bits give delta < 2*pi/1024, and
//    z = entry * (1 - delta^2/2 + i*(delta - delta^3/6)) is formed as entry_hi
//    plus a correction (absolute error ~5e-10) and renormalised with TwoSum so
//    that the low part is below one FP32 ulp;
//  * product v*z_hi is exact (TwoProd), v*z_lo is rounded (error <= 4e-10 |v|),
//    and the running sum is a TwoSum pair, so the sum carries no FP32 rounding;
//  * a warp's two directions run as the two halves of paired FP32 instructions
//    (FFMA2, FADD2, FMUL2), which round each half exactly as the scalar
//    operation; a - b is formed as fma(b, -1, a) (one rounding, as the
//    subtraction) and a negated product as fma(a, -b, c) = fma(-a, b, c), so
//    each half carries the scalar sequence's sums bit for bit, at about half
//    the instructions.
// ---------------------------------------------------------------------------
struct DfAcc2 {
  float2 s, c;  // value = s + c, one direction per half
};

__device__ __forceinline__ float2 df_sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  const float2 bb = df_sub2(s, a);
  e = __fadd2_rn(df_sub2(a, df_sub2(s, bb)), df_sub2(b, bb));
}

// acc += x * (yh + yl) per half (nx = -x): x*yh = p + e exactly (TwoProd), TwoSum of
// acc.s and p, and err + (x*yl + e) into acc.c.
__device__ __forceinline__ void df_add_product2(DfAcc2& acc, float2 x, float2 nx, float2 yh, float2 yl) {
  const float2 p = __fmul2_rn(x, yh);
  const float2 en = __ffma2_rn(nx, yh, p);  // p - x*yh = -e, exact
  float2 sum, err;
  two_sum2(acc.s, p, sum, err);
  acc.s = sum;
  acc.c = __fadd2_rn(acc.c, df_sub2(err, __ffma2_rn(nx, yl, en)));  // -(x*yl + e) from nx, en
}

// Twiddles of two phases (one per half) as (hi, lo) pairs.
__device__ __forceinline__ void df_twiddle2(uint64_t t0, uint64_t t1, const float4* __restrict__ tab, float2& zrh,
                                            float2& zrl, float2& zih, float2& zil) {
  const float4 a = tab[t0 >> 54], b = tab[t1 >> 54];  // (cos_hi, cos_lo, sin_hi, sin_lo)
  const float2 tx = make_float2(a.x, b.x), ty = make_float2(a.y, b.y);
  const float2 tz = make_float2(a.z, b.z), tw = make_float2(a.w, b.w);
  const float2 r24 = make_float2(__uint2float_rn(static_cast<uint32_t>(t0 >> 30) & 0xFFFFFFu),
                                 __uint2float_rn(static_cast<uint32_t>(t1 >> 30) & 0xFFFFFFu));
  const float2 d = __fmul2_rn(r24, make_float2(3.657295198167899e-10f, 3.657295198167899e-10f));  // 2*pi / 2^34
  const float2 d2 = __fmul2_rn(d, d);
  const float2 nc2 = __fmul2_rn(make_float2(-0.5f, -0.5f), d2);  // cos(d) - 1 (d^4/24 < 6e-11 dropped)
  const float2 sd = __fmul2_rn(d, __ffma2_rn(d2, make_float2(-0.16666667f, -0.16666667f), make_float2(1.f, 1.f)));
  const float2 nsd = __fmul2_rn(sd, make_float2(-1.f, -1.f));      // -sin(d)
  const float2 lr = __ffma2_rn(tx, nc2, __ffma2_rn(tz, nsd, ty));  // z_re - entry_hi
  const float2 li = __ffma2_rn(tz, nc2, __ffma2_rn(tx, sd, tw));   // z_im - entry_hi
  two_sum2(tx, lr, zrh, zrl);
  two_sum2(tz, li, zih, zil);
}

// Fractional part of x (turns) as a 2^-64 fixed-point value.
__device__ __forceinline__ uint64_t frac_turns_u64(double x) {
  const double f = x - rint(x);  // in [-0.5, 0.5]
  return static_cast<uint64_t>(static_cast<long long>(rint(f * 9223372036854775808.0))) << 1;
}

// UVWs as (hi, lo) float pairs for the double-float phase set-up.
static __global__ void split_uvw(const double* __restrict__ uvw, int64_t rows, float* __restrict__ out) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < 3 * rows;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double x = uvw[i];
    const float hi = static_cast<float>(x);
    out[2 * i] = hi;
    out[2 * i + 1] = static_cast<float>(x - static_cast<double>(hi));
  }
}

// Per-direction phase constants: -(l, m, n-1) * f0/c and -(l, m, n-1) * df/c as
// (hi, lo) float pairs, from the third row of each direction matrix.  n-1 is
// exact in FP64 (Sterbenz), which removes the reference's w_rot - w cancellation.
static __global__ void direction_constants(const double* __restrict__ dd, int ndir, double f0, double df,
                                           float* __restrict__ out) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= ndir) return;
  const double kA = f0 / kSpeedOfLight, kB = df / kSpeedOfLight;
  const double lmn[3] = {dd[9 * d + 6], dd[9 * d + 7], dd[9 * d + 8] - 1.0};
  for (int s = 0; s < 2; ++s) {
    const double k = s == 0 ? kA : kB;
    for (int i = 0; i < 3; ++i) {
      const double x = -lmn[i] * k;
      const float hi = static_cast<float>(x);
      out[12 * d + 6 * s + 2 * i] = hi;
      out[12 * d + 6 * s + 2 * i + 1] = static_cast<float>(x - static_cast<double>(hi));
    }
  }
}

// One work item of the compensated reference-antenna pass (batched calls:
// one per integration chunk).  Blocks are numbered across items.
struct RefantItem {
  const float2* vis;       // [C][rows][pols]
  const double* uvw;       // [rows][3]
  const double* dd;        // the item's first direction matrix
  double2* out;            // [nslab][ndir][nI1]
  int64_t rows;
  int32_t T, C, pols, ndir;
  int32_t t_per_slab, c_per_slab, n_tslab, n_cslab;
  int32_t dgroups, block_begin, pad_[2];
};

constexpr int kRefantPrefetch = 16;  // channel loads in flight per lane in the compensated pass

// The compensated reference-antenna pass of one call: its work items, the reference
// baselines, and the number of warp tasks (4 per block of the standalone launch).
struct RefantParams {
  const RefantItem* items;
  const int32_t* I1;
  double f0, df;
  int32_t nitems, nbl, nI1, ntasks;
};

// One warp task of the compensated reference-antenna pass: task w is warp w % 4 of block
// w / 4 of the standalone launch, i.e. directions j0, j0 + 1 of one group of 4*DPW, for the
// 32 reference baselines of one tile (one per lane), over one (timestep, channel) slab.
// tab is the double-float twiddle table in shared memory.  Lanes without a baseline, and
// warps without a direction, have nothing to do (no warp-collective operations here).
template <int DPW>
__device__ __forceinline__ void refant_warp_task(const RefantParams& rp, int task, const float4* tab, int lane) {
  const RefantItem* items = rp.items;
  const int blk = task >> 2, warp = task & 3;
  int ii = 0;
  while (ii + 1 < rp.nitems && items[ii + 1].block_begin <= blk) ++ii;
  const RefantItem it = items[ii];
  constexpr int NW = 4;
  const int nslab = it.n_tslab * it.n_cslab;
  const int local = blk - it.block_begin;
  const int ktile = local / (it.dgroups * nslab);
  const int dg = (local / nslab) % it.dgroups;
  const int slab = local % nslab;
  const int k = ktile * 32 + lane;
  const int j0 = (dg * NW + warp) * DPW;
  const int ts = slab / it.n_cslab, cs = slab % it.n_cslab;
  const int t_lo = ts * it.t_per_slab, t_hi = min(it.T, t_lo + it.t_per_slab);
  const int c_lo = cs * it.c_per_slab, c_hi = min(it.C, c_lo + it.c_per_slab);
  const int nI1 = rp.nI1, nbl = rp.nbl;
  if (j0 >= it.ndir || k >= nI1) return;
  int b = __ldg(rp.I1 + k);
  if (b < 0) b += nbl;  // VectorRangeSelect wrap-around (LA/math/cpu/vector.h:97-104)
  const double kA = rp.f0 / kSpeedOfLight, kB = rp.df / kSpeedOfLight;
  static_assert(DPW == 2, "the two directions of a warp are the halves of paired instructions");
  DfAcc2 re{make_float2(0.f, 0.f), make_float2(0.f, 0.f)}, im = re;
  for (int t = t_lo; t < t_hi; ++t) {
    const int64_t r = static_cast<int64_t>(t) * nbl + b;
    const double uu = __ldg(it.uvw + 3 * r), vv = __ldg(it.uvw + 3 * r + 1), ww = __ldg(it.uvw + 3 * r + 2);
    uint64_t pa[DPW], pb[DPW];
#pragma unroll
    for (int j = 0; j < DPW; ++j) {
      const int d = min(j0 + j, it.ndir - 1);
      const double wrot = __ldg(it.dd + 9 * d + 6) * uu + __ldg(it.dd + 9 * d + 7) * vv + __ldg(it.dd + 9 * d + 8) * ww;
      const double dw = wrot - ww;
      pa[j] = frac_turns_u64(-dw * kA);
      pb[j] = frac_turns_u64(-dw * kB);
    }
    const float2* src = it.vis + r * it.pols;
    const int64_t cstride = static_cast<int64_t>(it.rows) * it.pols;
    // Blocks of kRefantPrefetch channels: all loads of a block are issued before any use,
    // so each lane keeps that many scattered 8-byte reads in flight (the rows of the
    // reference-antenna baselines are spread over the cube).
    for (int c0 = c_lo; c0 < c_hi; c0 += kRefantPrefetch) {
      float2 vb[kRefantPrefetch];
#pragma unroll
      for (int i = 0; i < kRefantPrefetch; ++i)
        vb[i] = c0 + i < c_hi ? __ldg(src + static_cast<int64_t>(c0 + i) * cstride) : make_float2(0.f, 0.f);
#pragma unroll
      for (int i = 0; i < kRefantPrefetch; ++i) {
        if (c0 + i >= c_hi) break;
        const float2 v = vb[i];
        const float2 vx = make_float2(v.x, v.x), nvx = make_float2(-v.x, -v.x);
        const float2 vy = make_float2(v.y, v.y), nvy = make_float2(-v.y, -v.y);
        float2 zrh, zrl, zih, zil;
        df_twiddle2(pa[0] + static_cast<uint64_t>(c0 + i) * pb[0], pa[1] + static_cast<uint64_t>(c0 + i) * pb[1], tab,
                    zrh, zrl, zih, zil);
        df_add_product2(re, vx, nvx, zrh, zrl);  // re += vr zr - vi zi
        df_add_product2(re, nvy, vy, zih, zil);
        df_add_product2(im, vx, nvx, zih, zil);  // im += vr zi + vi zr
        df_add_product2(im, vy, nvy, zrh, zrl);
      }
    }
  }
  double2* out = it.out + static_cast<int64_t>(slab) * it.ndir * nI1;
  out[static_cast<int64_t>(j0) * nI1 + k] = make_double2(static_cast<double>(re.s.x) + static_cast<double>(re.c.x),
                                                         static_cast<double>(im.s.x) + static_cast<double>(im.c.x));
  if (j0 + 1 < it.ndir)
    out[static_cast<int64_t>(j0 + 1) * nI1 + k] = make_double2(static_cast<double>(re.s.y) + static_cast<double>(re.c.y),
                                                               static_cast<double>(im.s.y) + static_cast<double>(im.c.y));
}

// The pass as its own launch: rp.ntasks / 4 blocks of 4 warps.
template <int DPW>
__global__ void __launch_bounds__(128, 5) refant_average_df_items(const RefantParams rp,
                                                                 const float4* __restrict__ df_tab) {
  __shared__ float4 tab[kTwiddleSize];
  for (int i = threadIdx.x; i < kTwiddleSize; i += blockDim.x) tab[i] = __ldg(df_tab + i);
  __syncthreads();
  refant_warp_task<DPW>(rp, static_cast<int>(blockIdx.x) * 4 + static_cast<int>(threadIdx.x >> 5), tab,
                        static_cast<int>(threadIdx.x & 31));
}

// Sum of slab partials in slab order: avg[i] = sum_s partial[s][i].
static __global__ void reduce_slabs(const double2* __restrict__ partial, int nslab, int64_t n, double2* __restrict__ avg) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double re = 0.0, im = 0.0;
    for (int s = 0; s < nslab; ++s) {
      const double2 v = partial[static_cast<int64_t>(s) * n + i];
      re += v.x;
      im += v.y;
    }
    avg[i] = make_double2(re, im);
  }
}

// Zero every (row, channel) group of P samples that holds a NaN in any pol,
// copying src -> dst (dst may equal src).  This applies the reference's
// per-sample NaN skip (CpuLeapCalibrator.cc:201-214) once, at ingestion.
template <typename VisT, int P>
__global__ void sanitize_nan_groups(const VisT* src, VisT* dst, int64_t groups) {  // src may equal dst
  using S = typename VisScalar<VisT>::type;
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < groups;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    VisT v[P];
    bool nan = false;
#pragma unroll
    for (int p = 0; p < P; ++p) {
      v[p] = src[g * P + p];
      nan |= isnan(v[p].x) || isnan(v[p].y);
    }
    if (!nan && src == dst) continue;  // in place: a clean group stays as it is
#pragma unroll
    for (int p = 0; p < P; ++p) {
      VisT o = v[p];
      if (nan) { o.x = S(0); o.y = S(0); }
      dst[g * P + p] = o;
    }
  }
}

// Runtime-P variant of the NaN sanitiser for pol counts without a template instance.
template <typename VisT>
__global__ void sanitize_nan_groups_generic(const VisT* src, VisT* dst, int64_t groups, int P) {
  using S = typename VisScalar<VisT>::type;
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < groups;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    bool nan = false;
    for (int p = 0; p < P; ++p) {
      const VisT v = src[g * P + p];
      nan |= isnan(v.x) || isnan(v.y);
    }
    if (!nan && src == dst) continue;
    for (int p = 0; p < P; ++p) {
      VisT o = src[g * P + p];
      if (nan) { o.x = S(0); o.y = S(0); }
      dst[g * P + p] = o;
    }
  }
}

// K1: rotated[d][r] = dd[d] * uvw[r]  (MetaData::CalcUVW, LA/model/cpu/MetaData.cc:220-229;
// g_RotateUVW, LA/algorithm/cuda/CudaLeapCalibrator.cu:271-282).
static __global__ void rotate_uvw(const double* __restrict__ dd, const double* __restrict__ uvw, int64_t rows, int ndir,
                           double* __restrict__ out) {
  const int64_t total = rows * ndir;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t d = i / rows, r = i % rows;
    const double* m = dd + 9 * d;
    const double x = uvw[3 * r], y = uvw[3 * r + 1], z = uvw[3 * r + 2];
#pragma unroll
    for (int k = 0; k < 3; ++k) out[3 * i + k] = m[3 * k] * x + m[3 * k + 1] * y + m[3 * k + 2] * z;
  }
}

}  // namespace leapgb
