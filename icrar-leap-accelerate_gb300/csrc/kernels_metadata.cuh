// MetaData build on the device: the pseudo-inverse of a phase matrix A (m x n, two
// non-zeros per row) as Ad = G^-1 A^T with G = A^T A.
//
// The reference takes a thin SVD (LA/math/cpu/matrix_invert.h:49-74) and drops
// singular values at or below max(m,n)*eps*sigma_0.  For a phase matrix, G is an
// integer graph Laplacian plus the reference-antenna row: exact in FP64, with zero
// rows and columns for antennas that no kept baseline touches.  On the remaining
// columns G is positive definite whenever the baseline graph is connected.  The
// pseudo-inverse is unique, so there Ad = G^-1 A^T exactly, with exact zero rows for
// the untouched antennas, as the SVD gives them.
//
// Steps:
//  * G^-1 by Gauss-Jordan elimination without pivoting (stable for positive
//    definite matrices), one pivot per launch pair;
//  * two refinement steps X <- X + (I - X G) X, with the residual I - X G summed
//    in double-double (TwoProduct by FMA and TwoSum), which bring X to the
//    accuracy of an SVD of A;
//  * Ad[:, k] = sum over the non-zeros (k, j) of A of A[k, j] X[:, j].
// The host checks that every pivot was positive and that 1/||X||_F (a lower
// bound of the smallest eigenvalue of G) lies well above the reference's
// truncation threshold.  If either check fails, the SVD-style host path is used.
#pragma once

#include "leap_common.cuh"

namespace leapgb {

// Pivot k: r_j = M[k][j]/p (j != k), r_k = 1/p; f_i = M[i][k] (i != k), f_k = 0.  One block.
static __global__ void gj_pivot(const double* __restrict__ M, int n, int k, double* __restrict__ r,
                                double* __restrict__ f, int* __restrict__ bad) {
  const double p = M[static_cast<int64_t>(k) * n + k];
  if (threadIdx.x == 0 && !(p > 0.0)) atomicOr(bad, 1);
  const double inv = 1.0 / p;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    r[j] = j == k ? inv : M[static_cast<int64_t>(k) * n + j] * inv;
    f[j] = j == k ? 0.0 : M[static_cast<int64_t>(j) * n + k];
  }
}

// M[k][j] = r_j; M[i][j] = (j == k ? 0 : M[i][j]) - f_i r_j for i != k.
static __global__ void gj_update(double* __restrict__ M, int n, int k, const double* __restrict__ r,
                                 const double* __restrict__ f) {
  const int64_t total = static_cast<int64_t>(n) * n;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int i = static_cast<int>(e / n), j = static_cast<int>(e % n);
    if (i == k) M[e] = r[j];
    else M[e] = (j == k ? 0.0 : M[e]) - f[i] * r[j];
  }
}

// R = I - X G with every element summed in double-double (X, G row-major n x n).
static __global__ void residual_dd(const double* __restrict__ X, const double* __restrict__ G, int n,
                                   double* __restrict__ R) {
  const int64_t total = static_cast<int64_t>(n) * n;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int i = static_cast<int>(e / n), j = static_cast<int>(e % n);
    double s = i == j ? 1.0 : 0.0, c = 0.0;
    for (int l = 0; l < n; ++l) {
      const double g = G[static_cast<int64_t>(l) * n + j];
      if (g == 0.0) continue;
      const double x = X[static_cast<int64_t>(i) * n + l];
      const double pr = -x * g;
      const double pe = fma(-x, g, -pr);
      const double t = s + pr;
      const double bb = t - s;
      c += pe + ((s - (t - bb)) + (pr - bb));
      s = t;
    }
    R[e] = s + c;
  }
}

// Y = X + R X (row-major n x n).
static __global__ void refine_apply(const double* __restrict__ X, const double* __restrict__ R, int n,
                                    double* __restrict__ Y) {
  const int64_t total = static_cast<int64_t>(n) * n;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int i = static_cast<int>(e / n), j = static_cast<int>(e % n);
    double acc = 0.0;
    for (int l = 0; l < n; ++l) acc = fma(R[static_cast<int64_t>(i) * n + l], X[static_cast<int64_t>(l) * n + j], acc);
    Y[e] = X[e] + acc;
  }
}

// out[0] = sum of squares of x[0..len) (one block, fixed order per thread then tree).
static __global__ void sum_squares(const double* __restrict__ x, int64_t len, double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) s += x[i] * x[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

// Ad (S x Arows, column-major) = X_full A^T, where X_full[s][c] = X[cmp[s]][cmp[c]] for
// columns used by A (cmp >= 0) and 0 otherwise; rows of A as (c0, c1, v0, v1).
static __global__ void assemble_pinv(const double* __restrict__ X, int n, const int32_t* __restrict__ cmp,
                                     const int4* __restrict__ arow, const double2* __restrict__ aval, int S, int Arows,
                                     double* __restrict__ Ad) {
  const int64_t total = static_cast<int64_t>(S) * Arows;
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int s = static_cast<int>(e % S);
    const int k = static_cast<int>(e / S);
    const int si = cmp[s];
    double v = 0.0;
    if (si >= 0) {
      const int4 c = arow[k];
      const double2 a = aval[k];
      const int i0 = cmp[c.x], i1 = cmp[c.y];
      if (i0 >= 0) v += a.x * X[static_cast<int64_t>(si) * n + i0];
      if (i1 >= 0 && c.y != c.x) v += a.y * X[static_cast<int64_t>(si) * n + i1];
    }
    Ad[e] = v;
  }
}

// FP64 -> FP32 copy (the mixed form's Ad).
static __global__ void to_float(const double* __restrict__ x, int64_t len, float* __restrict__ y) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < len;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    y[i] = static_cast<float>(x[i]);
}

}  // namespace leapgb
