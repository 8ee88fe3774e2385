// Host-side FP64 set-up maths shared by the C ABI and the C++ calibrator.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace leapgb {

// MetaData::GenerateDDMatrix (LA/model/cpu/MetaData.cc:166-203); dd is 3x3 row-major.
void dd_matrix(double phase_ra, double phase_dec, double ra, double dec, double* dd);

// PhaseMatrixFunction (LA/algorithm/cpu/PhaseMatrixFunction.cc:35-93).  ref_ant < 0 = none.
// A is returned column-major (rows x cols).  Returns a LEAP_* status.
int phase_matrix(const int32_t* a1, const int32_t* a2, const uint8_t* fg, int32_t n, int32_t ref_ant,
                 std::vector<double>& A, std::vector<int32_t>& I, int32_t& rows, int32_t& cols, std::string& err);

// One row of a phase matrix: the non-zeros (c0, v0), (c1, v1) in column order; a row with a
// single non-zero has c1 == c0 and v1 == 0.
struct SparseRow {
  int32_t c0, c1;
  double v0, v1;
};

// PhaseMatrixFunction in sparse row form (no dense rows x cols array).
int phase_matrix_sparse(const int32_t* a1, const int32_t* a2, const uint8_t* fg, int32_t n, int32_t ref_ant,
                        std::vector<SparseRow>& A, std::vector<int32_t>& I, int32_t& cols, std::string& err);

// SVDPseudoInverse (LA/math/cpu/matrix_invert.h:49-56): A (m x n, column-major) -> Ad (n x m, column-major).
int pseudo_inverse(const double* A, int32_t m, int32_t n, double* Ad, std::string& err);

// Grid matrix of the gridded rotate + average (kernels_grid.cuh) for C channels:
// E[l][c] = exp(2 pi i (c - C/2) l / (2C)) / Psi(c - C/2) for table rows r = l + lbase,
// r in [0, rows), with Psi the Fourier transform of the exponential-of-semicircle
// kernel of width `taps` and shape `beta` at frequency k / (2C).  Scaled by a power of
// two (its largest entry in [2^13, 2^14)) and written as FP16 (hi, lo) splits in the
// K-major layout the kernel copies from: [chunk of 16 channels][hi, lo][row group of 8]
// [2 k-halves][8 rows x 8 k], rows 2 l + (0: re, 1: im).  Returns the inverse scale.
float grid_table(int32_t C, int32_t taps, double beta, int32_t lbase, int32_t rows, std::vector<uint16_t>& out);

// Interpolation weights of the gridded rotate + average as polynomials: for m = 0 .. taps-1,
// out[m * (degree + 1) + j] is the x^j coefficient (x = 2 f - 1, f in [0, 1)) of the degree
// `degree` Chebyshev interpolant of psi((f + taps/2 - 1 - m) * 2 / taps), psi the
// exponential-of-semicircle kernel of width `taps` and shape `beta` (the piecewise-polynomial
// kernel evaluation of Barnett, Magland & af Klinteberg, SIAM J. Sci. Comput. 41 (2019) C479).
void es_kernel_poly(int32_t taps, double beta, int32_t degree, float* out);

// Psi(k) = integral over |x| < taps/2 of psi(x) cos(2 pi x k / n), for k = 0..kmax.
std::vector<double> es_kernel_transform(int32_t taps, double beta, int32_t n, int32_t kmax);

}  // namespace leapgb
