// Solve kernels: phase-angle extraction and the two pseudoinverse contractions.
//
// Reference (CpuLeapCalibrator::PhaseRotate, LA/algorithm/cpu/CpuLeapCalibrator.cc:159-178;
// CUDA: g_AvgDataToPhaseAngles, cublasGemmEx(Ad1), g_CalcDInt,
// g_GenerateDeltaPhaseColumn, cublasGemmEx(Ad, beta=1),
// LA/algorithm/cuda/CudaLeapCalibrator.cu:255-259,409-517):
//   phi1[k]  = arg(avg[I1[k], 0]), k < |I1|;  phi1[|I1|] = 0
//   cal1     = Ad1 * phi1
//   dInt[n]  = arg(exp(-2*pi*i * (A*cal1)[n]) * avg[n, 0]), n < |I|   (row n, not I[n])
//   dphi     = dInt ++ [0]
//   cal      = Ad * dphi + cal1
// Only pol 0 of avgData enters.  All directions of a call are solved together:
// the last contraction is one [S x K] * [K x D] product.
#pragma once

#include "leap_common.cuh"

namespace leapgb {

struct SolveArgs {
  const double2* avg;       // [ndir][pols][nbl]
  int32_t nbl, pols, ndir, S;
  const int32_t* I1;        // [A1rows - 1]
  const double* Ad1;        // [S x A1rows] column-major
  int32_t A1rows;
  const int4* arow;         // [Arows]: (col0, col1, -, -) of the non-zeros of each A row
  const double2* arow_val;  // [Arows]: (val0, val1)
  int32_t Arows;            // |I| + 1
  int32_t Kpad;             // padded length of dphi rows
  double* cal1;             // [ndir][S]
  void* dphi;               // [ndir][Kpad] double (FP64) or float (mixed)
  const double2* avg_i1;    // optional [ndir][A1rows-1]: FP64 pol-0 sums of the I1 baselines
};

// K3 + K4: phi1 and cal1 = Ad1 * phi1.  Grid (directions, ceil(S / kCal1Cols)): each block
// forms its direction's phi1 and kCal1Cols outputs of cal1, each output as 4 k-quarters of
// the dot product combined in a fixed order, so the FP64 work spreads over more SMs than
// one block per direction.  With FP64 sums of the I1 baselines (mixed form) those replace
// pol 0 of avgData first (written by the direction's first block; the others read avg_i1).
constexpr int kCal1Cols = 64;
static __global__ void __launch_bounds__(256) solve_cal1(SolveArgs a) {
  extern __shared__ double sphi[];  // [A1rows] phi1, then [4][kCal1Cols] partial sums
  double* part = sphi + a.A1rows;
  const int d = blockIdx.x;
  double2* avg0 = const_cast<double2*>(a.avg) + static_cast<int64_t>(d) * a.pols * a.nbl;  // pol 0 column
  for (int k = threadIdx.x; k < a.A1rows; k += blockDim.x) {
    double v = 0.0;
    if (k < a.A1rows - 1) {
      int idx = a.I1[k];
      if (idx < 0) idx += a.nbl;  // VectorRangeSelect wrap-around (LA/math/cpu/vector.h:97-104)
      double2 z;
      if (a.avg_i1) {
        z = a.avg_i1[static_cast<int64_t>(d) * (a.A1rows - 1) + k];
        if (blockIdx.y == 0) avg0[idx] = z;  // duplicate I1 entries carry the same value
      } else {
        z = avg0[idx];
      }
      v = atan2(z.y, z.x);
    }
    sphi[k] = v;
  }
  __syncthreads();
  const int col = threadIdx.x % kCal1Cols, qk = threadIdx.x / kCal1Cols;
  const int s = blockIdx.y * kCal1Cols + col;
  const int kq = (a.A1rows + 3) / 4, k0 = qk * kq, k1 = min(a.A1rows, k0 + kq);
  double acc = 0.0;
  if (s < a.S)
    for (int k = k0; k < k1; ++k) acc += a.Ad1[s + static_cast<int64_t>(a.S) * k] * sphi[k];
  part[qk * kCal1Cols + col] = acc;
  __syncthreads();
  if (qk == 0 && s < a.S)
    a.cal1[static_cast<int64_t>(d) * a.S + s] =
        ((part[col] + part[kCal1Cols + col]) + part[2 * kCal1Cols + col]) + part[3 * kCal1Cols + col];
}

// K5 + K6-prep: dphi[d][n] for n < Kpad (zero past |I|).  FP64 form.
static __global__ void solve_dint_fp64(SolveArgs a) {
  const int d = blockIdx.y;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.Kpad) return;
  double* out = static_cast<double*>(a.dphi) + static_cast<int64_t>(d) * a.Kpad;
  if (n >= a.Arows - 1) {
    out[n] = 0.0;
    return;
  }
  const double* cal1 = a.cal1 + static_cast<int64_t>(d) * a.S;
  const int4 c = a.arow[n];
  const double2 v = a.arow_val[n];
  const double acal = v.x * cal1[c.x] + v.y * cal1[c.y];
  const double th = -kTwoPi * acal;
  double s, co;
  sincos(th, &s, &co);
  const double2 z = a.avg[static_cast<int64_t>(d) * a.pols * a.nbl + n];
  out[n] = atan2(co * z.y + s * z.x, co * z.x - s * z.y);
}

// Mixed form: the same in FP32 after the FP64 reduction of A*cal1's argument.
static __global__ void solve_dint_mixed(SolveArgs a) {
  const int d = blockIdx.y;
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.Kpad) return;
  float* out = static_cast<float*>(a.dphi) + static_cast<int64_t>(d) * a.Kpad;
  if (n >= a.Arows - 1) {
    out[n] = 0.f;
    return;
  }
  const double* cal1 = a.cal1 + static_cast<int64_t>(d) * a.S;
  const int4 c = a.arow[n];
  const double2 v = a.arow_val[n];
  const double acal = v.x * cal1[c.x] + v.y * cal1[c.y];
  // exp(-2*pi*i*acal): reduce acal (turns) to [-0.5, 0.5] in FP64, then FP32 trig.
  const float th = static_cast<float>(-kTwoPi * (acal - rint(acal)));
  float s, co;
  sincosf(th, &s, &co);
  const double2 z = a.avg[static_cast<int64_t>(d) * a.pols * a.nbl + n];
  const float zr = static_cast<float>(z.x), zi = static_cast<float>(z.y);
  out[n] = atan2f(co * zi + s * zr, co * zr - s * zi);
}

// K6: partial[kc][d][s] = sum_{k in chunk kc} Ad[s, k] * dphi[d][k].
// Block tile: 64 stations x 16 directions, 256 threads, 4 outputs per thread.
template <typename T>
static __global__ void __launch_bounds__(256) gemm_ad_partial(const T* __restrict__ Ad, int S, int Arows,
                                                       const T* __restrict__ dphi, int Kpad, int ndir,
                                                       int kchunk, double* __restrict__ partial) {
  constexpr int TS = 64, TD = 16, TK = 32;
  __shared__ T sA[TK][TS + 1];
  __shared__ T sB[TD][TK + 1];
  const int s0 = blockIdx.x * TS, d0 = blockIdx.y * TD, kc = blockIdx.z;
  const int k_begin = kc * kchunk, k_end = min(Arows, k_begin + kchunk);
  const int tx = threadIdx.x & 63;   // station within tile
  const int ty = threadIdx.x >> 6;   // 0..3 -> directions ty, ty+4, ty+8, ty+12
  T acc[4] = {T(0), T(0), T(0), T(0)};
  for (int k0 = k_begin; k0 < k_end; k0 += TK) {
    for (int i = threadIdx.x; i < TK * TS; i += 256) {
      const int kk = i / TS, ss = i % TS;
      const int k = k0 + kk, s = s0 + ss;
      sA[kk][ss] = (k < k_end && s < S) ? Ad[s + static_cast<int64_t>(S) * k] : T(0);
    }
    for (int i = threadIdx.x; i < TD * TK; i += 256) {
      const int dd = i / TK, kk = i % TK;
      const int k = k0 + kk, d = d0 + dd;
      sB[dd][kk] = (k < k_end && d < ndir) ? dphi[static_cast<int64_t>(d) * Kpad + k] : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < TK; ++kk) {
      const T av = sA[kk][tx];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] += av * sB[ty + 4 * q][kk];
    }
    __syncthreads();
  }
  const int s = s0 + tx;
  if (s >= S) return;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int d = d0 + ty + 4 * q;
    if (d < ndir) partial[(static_cast<int64_t>(kc) * ndir + d) * S + s] = static_cast<double>(acc[q]);
  }
}

// cal[d][s] = sum_kc partial[kc][d][s] (fixed order) + cal1[d][s].
// A block covers kFinishCols consecutive outputs; its 8 warps sum interleaved k-chunks and
// the partial sums are combined in warp order (deterministic), so each dependent chain of
// FP64 adds is nk/8 long and the grid spans the SMs even for a few directions.
constexpr int kFinishCols = 32;
static __global__ void __launch_bounds__(256) gemm_ad_finish(const double* __restrict__ partial, int nk, int ndir,
                                                             int S, const double* __restrict__ cal1,
                                                             double* __restrict__ cal) {
  __shared__ double part[8][kFinishCols];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n = ndir * S;
  const int i = blockIdx.x * kFinishCols + lane;
  double acc = 0.0;
  if (i < n)
    for (int kc = w; kc < nk; kc += 8) acc += partial[static_cast<int64_t>(kc) * n + i];
  part[w][lane] = acc;
  __syncthreads();
  if (w == 0 && i < n) {
    double sum = part[0][lane];
    for (int j = 1; j < 8; ++j) sum += part[j][lane];
    cal[i] = sum + cal1[i];
  }
}

}  // namespace leapgb
