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

namespace leapgb {

struct RotateArgs {
  const void* vis;          // [channels][rows][pols] complex (float2 or double2)
  const double* uvw;        // [rows][3]
  const double* dd;         // [ndir][9] row-major direction matrices
  const double* lambda;     // [channels] c / (f0 + ch*df), as the reference computes it
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
// for the others).  Arithmetic follows the reference expression by expression:
// shiftRad = shiftFactor / lambda_c with lambda_c = c / (f0 + ch*df), then
// exp(i*shiftRad) = (cos, sin) and a complex multiply.
// ---------------------------------------------------------------------------
template <typename VisT, int P, int DPW>
__global__ void __launch_bounds__(128) rotate_average_fp64(RotateArgs a) {
  constexpr int NW = 4;
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

  const VisT* vis = static_cast<const VisT*>(a.vis);
  if (valid) {
    for (int t = t_lo; t < t_hi; ++t) {
      const int64_t r = static_cast<int64_t>(t) * a.nbl + b;
      const double u = __ldg(a.uvw + 3 * r), v = __ldg(a.uvw + 3 * r + 1), w = __ldg(a.uvw + 3 * r + 2);
      double sf[DPW];
#pragma unroll
      for (int j = 0; j < DPW; ++j) {
        const double wrot = dd2[j][0] * u + dd2[j][1] * v + dd2[j][2] * w;
        sf[j] = -kTwoPi * (wrot - w);
      }
      for (int c = c_lo; c < c_hi; ++c) {
        const double lam = __ldg(a.lambda + c);
        const VisT* src = vis + (static_cast<int64_t>(c) * a.rows + r) * P;
        double vr[P], vi[P];
#pragma unroll
        for (int p = 0; p < P; ++p) load_sample(src + p, vr[p], vi[p]);
#pragma unroll
        for (int j = 0; j < DPW; ++j) {
          double s, co;
          sincos(sf[j] / lam, &s, &co);
#pragma unroll
          for (int p = 0; p < P; ++p) {
            accr[j][p] += vr[p] * co - vi[p] * s;
            acci[j][p] += vr[p] * s + vi[p] * co;
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
// fractions of a turn; each channel then costs one integer multiply-add, a
// bit-cast to an angle in [-pi, pi), FP32 sin/cos and FP32 complex MACs.
// Sums run in FP32 over blocks of KB channels and are folded into Kahan
// (sum, compensation) pairs, written out as sum - compensation in FP64.
// ---------------------------------------------------------------------------
template <typename VisT, int P, int DPW>
__global__ void __launch_bounds__(128) rotate_average_mixed(RotateArgs a) {
  constexpr int NW = 4;
  constexpr int KB = 16;
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
        // +256: round (instead of truncate) the 9 low bits dropped by turns_u32_to_angle.
        pa[j] = frac_turns_u32(-dw * kA) + 256u;
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
            const float ang = turns_u32_to_angle(pa[j] + static_cast<uint32_t>(c) * pb[j]);
            float s, co;
            __sincosf(ang, &s, &co);
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

// Sum of slab partials in slab order: avg[i] = sum_s partial[s][i].
__global__ void reduce_slabs(const double2* __restrict__ partial, int nslab, int64_t n, double2* __restrict__ avg) {
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
__global__ void sanitize_nan_groups(const VisT* __restrict__ src, VisT* __restrict__ dst, int64_t groups) {
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
__global__ void sanitize_nan_groups_generic(const VisT* __restrict__ src, VisT* __restrict__ dst, int64_t groups, int P) {
  using S = typename VisScalar<VisT>::type;
  for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < groups;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    bool nan = false;
    for (int p = 0; p < P; ++p) {
      const VisT v = src[g * P + p];
      nan |= isnan(v.x) || isnan(v.y);
    }
    for (int p = 0; p < P; ++p) {
      VisT o = src[g * P + p];
      if (nan) { o.x = S(0); o.y = S(0); }
      dst[g * P + p] = o;
    }
  }
}

// K1: rotated[d][r] = dd[d] * uvw[r]  (MetaData::CalcUVW, LA/model/cpu/MetaData.cc:220-229;
// g_RotateUVW, LA/algorithm/cuda/CudaLeapCalibrator.cu:271-282).
__global__ void rotate_uvw(const double* __restrict__ dd, const double* __restrict__ uvw, int64_t rows, int ndir,
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
