// Host-side FP64 set-up maths behind the C ABI: the direction matrix, the
// phase matrix and the pseudoinverse.  These run once per observation (or once
// per direction for the 3x3 matrix), never per visibility.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "leap_gb300.h"
#include "host_math.h"

namespace leapgb {

// dd = R3 * R2 * R1 with ang1 = pi/2 - dec0, ang2 = ra - ra0, ang3 = -pi/2 + dec
// (MetaData::GenerateDDMatrix, LA/model/cpu/MetaData.cc:166-203).  The three
// rotations are written out as the reference builds them and multiplied in the
// same order, so each element is formed from the same products.
void dd_matrix(double phase_ra, double phase_dec, double ra, double dec, double* dd) {
  const double pi = 3.141592653589793238462643383279502884;
  const double a1 = pi / 2.0 - phase_dec, a2 = ra - phase_ra, a3 = -pi / 2.0 + dec;
  const double r1[9] = {1, 0, 0, 0, std::cos(a1), -std::sin(a1), 0, std::sin(a1), std::cos(a1)};
  const double r2[9] = {std::cos(a2), std::sin(a2), 0, -std::sin(a2), std::cos(a2), 0, 0, 0, 1};
  const double r3[9] = {1, 0, 0, 0, std::cos(a3), -std::sin(a3), 0, std::sin(a3), std::cos(a3)};
  double t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t[3 * i + j] = r3[3 * i] * r2[j] + r3[3 * i + 1] * r2[3 + j] + r3[3 * i + 2] * r2[6 + j];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) dd[3 * i + j] = t[3 * i] * r1[j] + t[3 * i + 1] * r1[3 + j] + t[3 * i + 2] * r1[6 + j];
}

// PhaseMatrixFunction (LA/algorithm/cpu/PhaseMatrixFunction.cc:35-93): the checks, the
// number of antenna columns and the baselines kept (first-epoch cross baselines, not
// flagged, containing ref_ant when one is given), in baseline order.
static int phase_matrix_rows(const int32_t* a1, const int32_t* a2, const uint8_t* fg, int32_t n, int32_t ref_ant,
                             std::vector<int32_t>& keep, int32_t& cols, std::string& err) {
  if (ref_ant >= 0 && ref_ant >= n) {
    err = "refAnt " + std::to_string(ref_ant) + " is out of bounds";
    return LEAP_ERR_INVALID_ARGUMENT;
  }
  if (ref_ant >= 0 && fg[ref_ant]) {  // the reference indexes the baseline flags by antenna number
    err = "refAnt " + std::to_string(ref_ant) + " is flagged";
    return LEAP_ERR_INVALID_ARGUMENT;
  }
  if (n <= 0) {
    err = "a1 and a2 must not be empty";
    return LEAP_ERR_INVALID_ARGUMENT;
  }
  int32_t maxc = 0;
  for (int32_t i = 0; i < n; ++i) {
    if (a1[i] < 0 || a2[i] < 0) {
      err = "negative antenna index";
      return LEAP_ERR_INVALID_ARGUMENT;
    }
    maxc = std::max(maxc, std::max(a1[i], a2[i]));
  }
  cols = maxc + 1;
  keep.clear();
  keep.reserve(n);
  for (int32_t i = 0; i < n; ++i) {
    if (a1[i] == a2[i] || fg[i]) continue;
    if (ref_ant >= 0 && a1[i] != ref_ant && a2[i] != ref_ant) continue;
    keep.push_back(i);
  }
  return LEAP_OK;
}

int phase_matrix(const int32_t* a1, const int32_t* a2, const uint8_t* fg, int32_t n, int32_t ref_ant,
                 std::vector<double>& A, std::vector<int32_t>& I, int32_t& rows, int32_t& cols, std::string& err) {
  std::vector<int32_t> keep;
  const int rc = phase_matrix_rows(a1, a2, fg, n, ref_ant, keep, cols, err);
  if (rc != LEAP_OK) return rc;
  rows = static_cast<int32_t>(keep.size()) + 1;
  A.assign(static_cast<size_t>(rows) * cols, 0.0);
  I.assign(keep.begin(), keep.end());
  for (int32_t k = 0; k + 1 < rows; ++k) {
    A[k + static_cast<size_t>(rows) * a1[keep[k]]] = 1.0;
    A[k + static_cast<size_t>(rows) * a2[keep[k]]] = -1.0;
  }
  A[(rows - 1) + static_cast<size_t>(rows) * (ref_ant < 0 ? 0 : ref_ant)] = 1.0;
  return LEAP_OK;
}

int phase_matrix_sparse(const int32_t* a1, const int32_t* a2, const uint8_t* fg, int32_t n, int32_t ref_ant,
                        std::vector<SparseRow>& A, std::vector<int32_t>& I, int32_t& cols, std::string& err) {
  std::vector<int32_t> keep;
  const int rc = phase_matrix_rows(a1, a2, fg, n, ref_ant, keep, cols, err);
  if (rc != LEAP_OK) return rc;
  A.resize(keep.size() + 1);
  I.assign(keep.begin(), keep.end());
  for (size_t k = 0; k < keep.size(); ++k) {
    // column order, as the dense row of A lists its non-zeros
    const int32_t p = a1[keep[k]], q = a2[keep[k]];
    A[k] = p < q ? SparseRow{p, q, 1.0, -1.0} : SparseRow{q, p, -1.0, 1.0};
  }
  const int32_t r = ref_ant < 0 ? 0 : ref_ant;
  A[keep.size()] = SparseRow{r, r, 1.0, 0.0};
  return LEAP_OK;
}

// Pseudoinverse through the Gram matrix.
//
// A+ = (A^T A)+ A^T for any A.  G = A^T A is formed from the non-zeros of each
// row of A (two per row for a phase matrix, so G is an integer Laplacian plus
// the reference-antenna row and is formed exactly), diagonalised by cyclic
// Jacobi rotations (which keep exact zero rows and columns of G exact, so
// unobserved antennas get exactly zero weight), and applied to A^T row by row.
//
// Truncation: the reference drops singular values sigma <= max(m,n)*eps*sigma_0
// (LA/math/cpu/matrix_invert.h:54).  Eigenvalues of G are sigma^2 but are only
// resolved to about eps*lambda_0, so the rule is applied as
// lambda <= max(m,n)*eps*lambda_0; the two agree unless a singular value lies
// between max(m,n)*eps*sigma_0 and sqrt(max(m,n)*eps)*sigma_0, which the integer
// structure of phase matrices rules out.
int pseudo_inverse(const double* A, int32_t m, int32_t n, double* Ad, std::string& err) {
  if (m <= 0 || n <= 0) {
    err = "pseudo_inverse: empty matrix";
    return LEAP_ERR_INVALID_ARGUMENT;
  }
  // Row-wise non-zeros of A (column-major input).
  std::vector<int64_t> rowptr(static_cast<size_t>(m) + 1, 0);
  for (int32_t j = 0; j < n; ++j)
    for (int32_t i = 0; i < m; ++i)
      if (A[i + static_cast<size_t>(m) * j] != 0.0) rowptr[i + 1]++;
  for (int32_t i = 0; i < m; ++i) rowptr[i + 1] += rowptr[i];
  std::vector<int32_t> colidx(rowptr[m]);
  std::vector<double> val(rowptr[m]);
  {
    std::vector<int64_t> fill(rowptr.begin(), rowptr.end() - 1);
    for (int32_t j = 0; j < n; ++j)
      for (int32_t i = 0; i < m; ++i) {
        const double a = A[i + static_cast<size_t>(m) * j];
        if (a != 0.0) {
          colidx[fill[i]] = j;
          val[fill[i]] = a;
          fill[i]++;
        }
      }
  }
  // G = A^T A (row-major n x n, symmetric).
  std::vector<double> G(static_cast<size_t>(n) * n, 0.0);
  for (int32_t i = 0; i < m; ++i)
    for (int64_t p = rowptr[i]; p < rowptr[i + 1]; ++p)
      for (int64_t q = rowptr[i]; q < rowptr[i + 1]; ++q) G[static_cast<size_t>(colidx[p]) * n + colidx[q]] += val[p] * val[q];

  // Cyclic Jacobi: G <- J^T G J until the off-diagonal mass is negligible; V accumulates J.
  std::vector<double> V(static_cast<size_t>(n) * n, 0.0);
  for (int32_t i = 0; i < n; ++i) V[static_cast<size_t>(i) * n + i] = 1.0;
  auto g = [&](int32_t i, int32_t j) -> double& { return G[static_cast<size_t>(i) * n + j]; };
  const double eps = std::numeric_limits<double>::epsilon();
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int32_t i = 0; i < n; ++i) {
      diag += g(i, i) * g(i, i);
      for (int32_t j = i + 1; j < n; ++j) off += g(i, j) * g(i, j);
    }
    if (off <= eps * eps * diag * 1e-4 || off == 0.0) break;
    for (int32_t p = 0; p < n - 1; ++p) {
      for (int32_t q = p + 1; q < n; ++q) {
        const double apq = g(p, q);
        if (apq == 0.0) continue;
        const double app = g(p, p), aqq = g(q, q);
        // Skip rotations that cannot change the diagonal at working precision.
        if (std::fabs(apq) <= eps * 1e-3 * std::sqrt(std::fabs(app * aqq))) {
          g(p, q) = g(q, p) = 0.0;
          continue;
        }
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int32_t k = 0; k < n; ++k) {
          const double gkp = g(k, p), gkq = g(k, q);
          g(k, p) = c * gkp - s * gkq;
          g(k, q) = s * gkp + c * gkq;
        }
        for (int32_t k = 0; k < n; ++k) {
          const double gpk = g(p, k), gqk = g(q, k);
          g(p, k) = c * gpk - s * gqk;
          g(q, k) = s * gpk + c * gqk;
        }
        g(p, q) = g(q, p) = 0.0;
        for (int32_t k = 0; k < n; ++k) {
          double* vr = &V[static_cast<size_t>(k) * n];
          const double vkp = vr[p], vkq = vr[q];
          vr[p] = c * vkp - s * vkq;
          vr[q] = s * vkp + c * vkq;
        }
      }
    }
  }
  std::vector<double> lam(n);
  double lmax = 0.0;
  for (int32_t i = 0; i < n; ++i) {
    lam[i] = g(i, i);
    lmax = std::max(lmax, std::fabs(lam[i]));
  }
  const double tol = static_cast<double>(std::max(m, n)) * eps * lmax;
  // Gplus = V diag(1/lambda) V^T  (row-major n x n)
  std::vector<double> Gp(static_cast<size_t>(n) * n, 0.0);
  for (int32_t e = 0; e < n; ++e) {
    if (!(std::fabs(lam[e]) > tol)) continue;
    const double inv = 1.0 / lam[e];
    for (int32_t i = 0; i < n; ++i) {
      const double vie = V[static_cast<size_t>(i) * n + e] * inv;
      if (vie == 0.0) continue;
      double* row = &Gp[static_cast<size_t>(i) * n];
      for (int32_t j = 0; j < n; ++j) row[j] += vie * V[static_cast<size_t>(j) * n + e];
    }
  }
  // Iterative refinement Gplus <- Gplus + R Gplus with R = I - Gplus G, where
  // R is accumulated in double-double (Ogita-Rump-Oishi Dot2: FMA TwoProduct
  // and Knuth TwoSum).  The eigenvalue errors (about eps * lambda_0 each) leave
  // Gplus with a relative error near eps * kappa(G) = eps * kappa(A)^2; with an
  // accurately computed residual each step multiplies that error by itself, so
  // two steps bring it to the eps * kappa(A) level of an SVD of A.  Exact zero
  // rows and columns of G stay exact zeros.
  {
    // G was overwritten by the rotations; rebuild it from the rows of A.
    std::vector<double> G0(static_cast<size_t>(n) * n, 0.0);
    for (int32_t i = 0; i < m; ++i)
      for (int64_t p = rowptr[i]; p < rowptr[i + 1]; ++p)
        for (int64_t q = rowptr[i]; q < rowptr[i + 1]; ++q)
          G0[static_cast<size_t>(colidx[p]) * n + colidx[q]] += val[p] * val[q];
    std::vector<double> R(static_cast<size_t>(n) * n), U(static_cast<size_t>(n) * n);
    std::vector<double> Gcol(n);
    for (int step = 0; step < 2; ++step) {
      for (int32_t j = 0; j < n; ++j) {
        for (int32_t l = 0; l < n; ++l) Gcol[l] = G0[static_cast<size_t>(l) * n + j];
        for (int32_t i = 0; i < n; ++i) {
          const double* mrow = &Gp[static_cast<size_t>(i) * n];
          double s = (i == j) ? 1.0 : 0.0, c = 0.0;
          for (int32_t l = 0; l < n; ++l) {
            const double g = Gcol[l];
            if (g == 0.0) continue;
            const double p = -mrow[l] * g;
            const double pe = std::fma(-mrow[l], g, -p);
            const double t = s + p;
            const double bb = t - s;
            const double se = (s - (t - bb)) + (p - bb);
            s = t;
            c += pe + se;
          }
          R[static_cast<size_t>(i) * n + j] = s + c;
        }
      }
      std::fill(U.begin(), U.end(), 0.0);  // U = R * Gplus
      for (int32_t i = 0; i < n; ++i) {
        double* urow = &U[static_cast<size_t>(i) * n];
        for (int32_t l = 0; l < n; ++l) {
          const double x = R[static_cast<size_t>(i) * n + l];
          if (x == 0.0) continue;
          const double* prow = &Gp[static_cast<size_t>(l) * n];
          for (int32_t j = 0; j < n; ++j) urow[j] += x * prow[j];
        }
      }
      for (size_t i = 0; i < Gp.size(); ++i) Gp[i] += U[i];
    }
  }
  // Ad = Gplus A^T : column k of Ad = sum over non-zeros (k, j) of A of A[k,j] * Gplus[:, j].
  for (int32_t k = 0; k < m; ++k) {
    double* out = Ad + static_cast<size_t>(n) * k;
    std::fill(out, out + n, 0.0);
    for (int64_t p = rowptr[k]; p < rowptr[k + 1]; ++p) {
      const int32_t j = colidx[p];
      const double a = val[p];
      for (int32_t i = 0; i < n; ++i) out[i] += a * Gp[static_cast<size_t>(i) * n + j];
    }
  }
  return LEAP_OK;
}

}  // namespace leapgb

namespace leapgb {

std::vector<double> es_kernel_transform(int32_t taps, double beta, int32_t n, int32_t kmax) {
  // psi and all its derivatives are ~exp(-beta) at the ends of the support, so the
  // trapezoidal rule converges spectrally; 8192 panels give full FP64 accuracy.
  const int panels = 8192;
  const double half = 0.5 * taps, h = 2.0 * half / panels;
  std::vector<double> psi(panels + 1);
  for (int i = 0; i <= panels; ++i) {
    const double x = -half + i * h, z = x / half;
    const double q = std::max(0.0, 1.0 - z * z);
    psi[i] = std::exp(beta * (std::sqrt(q) - 1.0)) * ((i == 0 || i == panels) ? 0.5 : 1.0);
  }
  std::vector<double> out(kmax + 1);
  const double kTwoPiD = 6.283185307179586476925286766559;
  for (int k = 0; k <= kmax; ++k) {
    double s = 0.0;
    const double w = kTwoPiD * k / n;
    for (int i = 0; i <= panels; ++i) s += psi[i] * std::cos(w * (-half + i * h));
    out[k] = s * h;
  }
  return out;
}

void es_kernel_poly(int32_t taps, double beta, int32_t degree, float* out) {
  // h_m(f) = psi((f + taps/2 - 1 - m) * 2 / taps) for f in [0, 1): interpolate at the
  // degree + 1 Chebyshev points of x = 2 f - 1, then expand the Chebyshev series into
  // monomials of x (the Chebyshev coefficients c_n; T_{n+1} = 2 x T_n - T_{n-1}).
  const int np = degree + 1;
  const double kPiD = 3.141592653589793238462643383279;
  std::vector<double> tm(static_cast<size_t>(np) * np, 0.0);  // tm[n * np + j]: x^j coefficient of T_n
  tm[0] = 1.0;
  if (np > 1) tm[1 * np + 1] = 1.0;
  for (int n = 1; n + 1 < np; ++n)
    for (int j = 0; j < np; ++j)
      tm[(n + 1) * np + j] = (j > 0 ? 2.0 * tm[n * np + j - 1] : 0.0) - tm[(n - 1) * np + j];
  for (int m = 0; m < taps; ++m) {
    std::vector<double> val(np), mono(np, 0.0);
    for (int k = 0; k < np; ++k) {
      const double x = std::cos(kPiD * (k + 0.5) / np);
      const double z = ((x + 1.0) * 0.5 + 0.5 * taps - 1.0 - m) * 2.0 / taps;
      const double q = 1.0 - z * z;
      val[k] = q > 0.0 ? std::exp(beta * (std::sqrt(q) - 1.0)) : 0.0;
    }
    for (int n = 0; n < np; ++n) {
      double c = 0.0;
      for (int k = 0; k < np; ++k) c += val[k] * std::cos(kPiD * n * (k + 0.5) / np);
      c *= (n == 0 ? 1.0 : 2.0) / np;
      for (int j = 0; j < np; ++j) mono[j] += c * tm[n * np + j];
    }
    for (int j = 0; j < np; ++j) out[m * np + j] = static_cast<float>(mono[j]);
  }
}

namespace {
// IEEE binary16 bits of x rounded to nearest, ties to even (|x| < 65504), and its value.
uint16_t to_f16_bits(double x) {
  const uint16_t sign = x < 0 ? 0x8000u : 0u;
  const double a = std::fabs(x);
  if (a == 0.0) return sign;
  int e = 0;
  const double f = std::frexp(a, &e);  // a = f 2^e, f in [0.5, 1)
  const int E = e + 14;                // biased exponent of 2 f 2^(e - 1)
  if (E < 1) return static_cast<uint16_t>(sign | static_cast<uint16_t>(std::nearbyint(std::ldexp(a, 24))));
  const int mant = static_cast<int>(std::nearbyint((2.0 * f - 1.0) * 1024.0));
  return static_cast<uint16_t>(sign | ((E << 10) + mant));  // mant == 1024 carries into the exponent
}
double from_f16_bits(uint16_t h) {
  const int E = (h >> 10) & 31, mant = h & 1023;
  const double v = E == 0 ? std::ldexp(static_cast<double>(mant), -24) : std::ldexp(1.0 + mant / 1024.0, E - 15);
  return (h & 0x8000u) ? -v : v;
}
}  // namespace

float grid_table(int32_t C, int32_t taps, double beta, int32_t lbase, int32_t rows, std::vector<uint16_t>& out) {
  const int n = 2 * C, c0 = C / 2;
  const int nchunk = (C + 15) / 16, nrg = rows / 8;
  const std::vector<double> psi_hat = es_kernel_transform(taps, beta, n, std::max(c0, C - 1 - c0));
  // One power of two for the table: the largest |E| = max 1 / Psi(k) goes into [2^13, 2^14).
  double emax = 0.0;
  for (int c = 0; c < C; ++c) emax = std::max(emax, 1.0 / psi_hat[std::abs(c - c0)]);
  int e = 0;
  (void)std::frexp(emax, &e);
  const double scale = std::ldexp(1.0, 14 - e);
  out.assign(static_cast<size_t>(nchunk) * 2 * 2 * nrg * 128, 0);
  const double kTwoPiD = 6.283185307179586476925286766559;
  for (int c = 0; c < C; ++c) {
    const int k = c - c0;
    const double inv = scale / psi_hat[std::abs(k)];
    const int q = c / 16, kk = c % 16;
    for (int r = 0; r < rows; ++r) {
      const long long l = static_cast<long long>(r) - lbase;
      long long m = (static_cast<long long>(k) * l) % n;  // exact phase index
      if (m < 0) m += n;
      const double ang = kTwoPiD * static_cast<double>(m) / n;
      const double v[2] = {std::cos(ang) * inv, std::sin(ang) * inv};
      for (int ri = 0; ri < 2; ++ri) {
        const uint16_t hi = to_f16_bits(v[ri]);
        const uint16_t lo = to_f16_bits(v[ri] - from_f16_bits(hi));
        const int rr = 2 * r + ri;  // re and im rows of a grid point are neighbours
        for (int hl = 0; hl < 2; ++hl) {
          const size_t base = (static_cast<size_t>(q * 2 + hl) * 2 * nrg) * 128;
          // The kernel's K-major 16-bit block layout (grid_f16_offset), in 2-byte units.
          out[base + ((rr >> 3) * 2 + (kk >> 3)) * 64 + (rr & 7) * 8 + (kk & 7)] = hl == 0 ? hi : lo;
        }
      }
    }
  }
  return static_cast<float>(1.0 / scale);
}

}  // namespace leapgb
