// Adjoint of the calibration chain rotate -> average -> arg -> solve (FP64).
//
// Forward, per direction (LA/algorithm/cpu/CpuLeapCalibrator.cc:159-217):
//   phase[r][c] = -2*pi*(l*u_r + m*v_r + (n-1)*w_r) / lambda_c,   (l, m, n) = row 2 of dd
//   avg[b]      = sum_{t, c} V[0][t*nbl + b][c] * exp(i*phase)    (pol 0; NaN groups skipped)
//   phi1[k]     = arg(avg[I1[k]]),  phi1[|I1|] = 0
//   cal1        = Ad1 * phi1
//   dInt[n]     = arg(exp(-2*pi*i*(A*cal1)[n]) * avg[n]),  n < |I|   (row n, not I[n])
//   cal         = Ad * (dInt ++ [0]) + cal1
//
// Gradients follow the convention of complex autograd: for a real loss L and a
// complex quantity z = x + iy, gz = dL/dx + i*dL/dy (so y = a*z gives
// gz = conj(a)*gy, and arg(z) has gradient i*z/|z|^2).  Given g_cal:
//   g_dphi  = Ad^T g_cal                               (entries n < |I|)
//   g_cal1  = g_cal + A^T (-2*pi * g_dphi)             (rows n < |I| of A)
//   g_phi1  = Ad1^T g_cal1                             (entries k < |I1|)
//   g_avg[b] = [b < |I|] g_dphi[b] i avg[b]/|avg[b]|^2 + sum_{k: I1[k] = b} g_phi1[k] i avg[b]/|avg[b]|^2
//   g_V[0][r][c] = g_avg[r mod nbl] * exp(-i*phase[r][c])  (zero for other pols and NaN groups)
//   dL/d(l, m, n) = sum_{r, c} Re(conj(g_avg[b]) * i * V[0][r][c] * exp(i*phase)) * (-2*pi/lambda_c) * (u, v, w)_r
// The rotated samples are recomputed here, not stored by the forward pass.
// Sums over (row, channel) go to per-block partials that one kernel adds in a
// fixed order: results do not depend on scheduling.
#pragma once

#include "leap_common.cuh"

namespace leapgb {

constexpr int kAdjChannels = 16;  // channels per thread item (phase re-seeded with sincos per item)

struct AdjointArgs {
  const void* vis;         // [C][rows][P], float2 (vis_c64) or double2
  int vis_c64;
  int check_nan;           // skip (row, channel) groups holding a NaN in any pol
  const double* uvw;       // [rows][3]
  const double* dd;        // [D][9]
  const double2* gavg;     // [D][nbl]
  int64_t rows;
  int32_t C, P, nbl, D;
  double f0, df;
  double* partial;         // [gridDim.x][D][3]
  void* gvis;              // [C][rows][P] same element type as vis, pol 0 written
};

__device__ __forceinline__ double2 adj_load(const AdjointArgs& a, int64_t idx) {
  if (a.vis_c64) {
    const float2 v = __ldg(static_cast<const float2*>(a.vis) + idx);
    return make_double2(v.x, v.y);
  }
  return __ldg(static_cast<const double2*>(a.vis) + idx);
}

// Pol-0 samples of one (row, 16-channel) item; zero where the group has a NaN or c >= C.
__device__ __forceinline__ void adj_item_samples(const AdjointArgs& a, int64_t r, int c0, double2 (&x)[kAdjChannels]) {
#pragma unroll
  for (int k = 0; k < kAdjChannels; ++k) {
    const int c = c0 + k;
    x[k] = make_double2(0.0, 0.0);
    if (c < a.C) {
      const int64_t base = (static_cast<int64_t>(c) * a.rows + r) * a.P;
      const double2 v0 = adj_load(a, base);
      bool nan = isnan(v0.x) || isnan(v0.y);
      if (a.check_nan)
        for (int p = 1; p < a.P; ++p) {
          const double2 v = adj_load(a, base + p);
          nan |= isnan(v.x) || isnan(v.y);
        }
      if (!nan) x[k] = v0;
    }
  }
}

// exp(i*phase) at channel c0 and the per-channel step exp(i*sf*df/c_light), sf = -2*pi*(w_rot - w).
__device__ __forceinline__ void adj_phasor(const AdjointArgs& a, int d, double u, double v, double w, int c0,
                                           double& zr, double& zi, double& wr, double& wi) {
  const double wrot = __ldg(a.dd + 9 * d + 6) * u + __ldg(a.dd + 9 * d + 7) * v + __ldg(a.dd + 9 * d + 8) * w;
  const double sf = -kTwoPi * (wrot - w);
  const double lambda0 = kSpeedOfLight / (a.f0 + c0 * a.df);
  sincos(sf / lambda0, &zi, &zr);
  sincos(sf * (a.df / kSpeedOfLight), &wi, &wr);
}

// dL/d(l, m, n) partial sums: blockIdx.y selects DPB directions, threads stride over (row, channel item).
template <int DPB>
__global__ void __launch_bounds__(256) adjoint_lmn(AdjointArgs a) {
  const int d0 = blockIdx.y * DPB;
  const int nitem = (a.C + kAdjChannels - 1) / kAdjChannels;
  const int64_t items = a.rows * nitem;
  double acc[DPB][3];
#pragma unroll
  for (int j = 0; j < DPB; ++j) acc[j][0] = acc[j][1] = acc[j][2] = 0.0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < items;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i % a.rows;
    const int c0 = static_cast<int>(i / a.rows) * kAdjChannels;
    const int b = static_cast<int>(r % a.nbl);
    double2 g[DPB];
    bool any = false;
#pragma unroll
    for (int j = 0; j < DPB; ++j) {
      g[j] = d0 + j < a.D ? a.gavg[static_cast<int64_t>(d0 + j) * a.nbl + b] : make_double2(0.0, 0.0);
      any |= g[j].x != 0.0 || g[j].y != 0.0;
    }
    if (!any) continue;
    double2 x[kAdjChannels];
    adj_item_samples(a, r, c0, x);
    const double u = __ldg(a.uvw + 3 * r), v = __ldg(a.uvw + 3 * r + 1), w = __ldg(a.uvw + 3 * r + 2);
#pragma unroll
    for (int j = 0; j < DPB; ++j) {
      if (g[j].x == 0.0 && g[j].y == 0.0) continue;
      double zr, zi, wr, wi;
      adj_phasor(a, d0 + j, u, v, w, c0, zr, zi, wr, wi);
      double s = 0.0;  // sum_c Re(conj(g) * i * x_c * z_c) / lambda_c
#pragma unroll
      for (int k = 0; k < kAdjChannels; ++k) {
        const double yr = x[k].x * zr - x[k].y * zi, yi = x[k].x * zi + x[k].y * zr;
        s += (g[j].y * yr - g[j].x * yi) * ((a.f0 + (c0 + k) * a.df) / kSpeedOfLight);
        const double nr = zr * wr - zi * wi;
        zi = zr * wi + zi * wr;
        zr = nr;
      }
      acc[j][0] += -kTwoPi * s * u;
      acc[j][1] += -kTwoPi * s * v;
      acc[j][2] += -kTwoPi * s * w;
    }
  }
  // Block reduction: warp tree, then warps in order.
  __shared__ double red[8][DPB * 3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < DPB; ++j)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double x = acc[j][q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) red[warp][j * 3 + q] = x;
    }
  __syncthreads();
  if (threadIdx.x < DPB * 3) {
    double x = 0.0;
    for (int wi = 0; wi < static_cast<int>(blockDim.x >> 5); ++wi) x += red[wi][threadIdx.x];
    const int j = threadIdx.x / 3, q = threadIdx.x % 3;
    if (d0 + j < a.D) a.partial[(static_cast<int64_t>(blockIdx.x) * a.D + d0 + j) * 3 + q] = x;
  }
}

// out[d][q] = sum over blocks (in order) of partial[blk][d][q].
static __global__ void adjoint_lmn_reduce(const double* __restrict__ partial, int nblk, int D, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * D) return;
  double x = 0.0;
  for (int k = 0; k < nblk; ++k) x += partial[static_cast<int64_t>(k) * 3 * D + i];
  out[i] = x;
}

// g_V[0][r][c] = sum_d g_avg[d][b] * exp(-i*phase_d[r][c]); zero at NaN groups.
// The other pols' gradients are zero (the caller clears the array first).
static __global__ void __launch_bounds__(256) adjoint_vis(AdjointArgs a) {
  const int nitem = (a.C + kAdjChannels - 1) / kAdjChannels;
  const int64_t items = a.rows * nitem;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < items;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i % a.rows;
    const int c0 = static_cast<int>(i / a.rows) * kAdjChannels;
    const int b = static_cast<int>(r % a.nbl);
    const double u = __ldg(a.uvw + 3 * r), v = __ldg(a.uvw + 3 * r + 1), w = __ldg(a.uvw + 3 * r + 2);
    double gr[kAdjChannels], gi[kAdjChannels];
#pragma unroll
    for (int k = 0; k < kAdjChannels; ++k) gr[k] = gi[k] = 0.0;
    for (int d = 0; d < a.D; ++d) {
      const double2 g = a.gavg[static_cast<int64_t>(d) * a.nbl + b];
      if (g.x == 0.0 && g.y == 0.0) continue;
      double zr, zi, wr, wi;
      adj_phasor(a, d, u, v, w, c0, zr, zi, wr, wi);
#pragma unroll
      for (int k = 0; k < kAdjChannels; ++k) {
        gr[k] += g.x * zr + g.y * zi;  // g * conj(z)
        gi[k] += g.y * zr - g.x * zi;
        const double nr = zr * wr - zi * wi;
        zi = zr * wi + zi * wr;
        zr = nr;
      }
    }
#pragma unroll
    for (int k = 0; k < kAdjChannels; ++k) {
      const int c = c0 + k;
      if (c >= a.C) break;
      const int64_t base = (static_cast<int64_t>(c) * a.rows + r) * a.P;
      bool nan = false;
      if (a.check_nan)
        for (int p = 0; p < a.P; ++p) {
          const double2 x = adj_load(a, base + p);
          nan |= isnan(x.x) || isnan(x.y);
        }
      const double outr = nan ? 0.0 : gr[k], outi = nan ? 0.0 : gi[k];
      if (a.vis_c64)
        static_cast<float2*>(a.gvis)[base] = make_float2(static_cast<float>(outr), static_cast<float>(outi));
      else
        static_cast<double2*>(a.gvis)[base] = make_double2(outr, outi);
    }
  }
}

// out[d * ldo + k] = sum_s M[s + S*k] * G[d*S + s] for k < kmax: one warp per k.
static __global__ void adjoint_contract_t(const double* __restrict__ M, int S, int kmax, const double* __restrict__ G,
                                          int D, double* __restrict__ out, int ldo) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (k >= kmax) return;
  const double* col = M + static_cast<int64_t>(S) * k;
  for (int d = 0; d < D; ++d) {
    double x = 0.0;
    for (int s = lane; s < S; s += 32) x += col[s] * G[static_cast<int64_t>(d) * S + s];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) out[static_cast<int64_t>(d) * ldo + k] = x;
  }
}

// g_cal1[d][s] = g_cal[d][s] - 2*pi * sum_{rows n of A with a non-zero in column s, n < |I|} A[n][s] * g_dphi[d][n].
// (at_ptr, at_idx, at_val) is A^T in compressed-row form over the first |I| rows.
static __global__ void adjoint_cal1(const double* __restrict__ gcal, const double* __restrict__ gdphi, int ld_dphi,
                                    const int32_t* __restrict__ at_ptr, const int32_t* __restrict__ at_idx,
                                    const double* __restrict__ at_val, int S, int D, double* __restrict__ gcal1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S * D) return;
  const int d = i / S, s = i % S;
  double x = 0.0;
  for (int j = at_ptr[s]; j < at_ptr[s + 1]; ++j) x += at_val[j] * gdphi[static_cast<int64_t>(d) * ld_dphi + at_idx[j]];
  gcal1[i] = gcal[i] - kTwoPi * x;
}

__device__ __forceinline__ double2 grad_arg(double2 z, double g) {
  const double n2 = z.x * z.x + z.y * z.y;
  if (n2 == 0.0) return make_double2(0.0, 0.0);
  return make_double2(-g * z.y / n2, g * z.x / n2);  // g * i * z / |z|^2
}

// g_avg[d][b] from the dInt term (b < |I|).
static __global__ void adjoint_avg_dint(const double2* __restrict__ avg0, const double* __restrict__ gdphi, int ld_dphi,
                                        int nI, int nbl, int D, double2* __restrict__ gavg) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < static_cast<int64_t>(nbl) * D;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int d = static_cast<int>(i / nbl), b = static_cast<int>(i % nbl);
    gavg[i] = b < nI ? grad_arg(avg0[i], gdphi[static_cast<int64_t>(d) * ld_dphi + b]) : make_double2(0.0, 0.0);
  }
}

// Adds the phi1 term: one thread per direction walks I1 in order (entries may repeat).
static __global__ void adjoint_avg_phi1(const double2* __restrict__ avg0, const double* __restrict__ gphi1,
                                        const int32_t* __restrict__ I1, int nI1, int nbl, int D,
                                        double2* __restrict__ gavg) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= D) return;
  for (int k = 0; k < nI1; ++k) {
    int idx = I1[k];
    if (idx < 0) idx += nbl;
    const int64_t o = static_cast<int64_t>(d) * nbl + idx;
    const double2 gz = grad_arg(avg0[o], gphi1[static_cast<int64_t>(d) * nI1 + k]);
    gavg[o].x += gz.x;
    gavg[o].y += gz.y;
  }
}

}  // namespace leapgb
