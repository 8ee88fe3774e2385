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
// kernel of width `taps` and shape `beta` at frequency k / (2C).  Written as 3xTF32
// (hi, lo) splits in the packed K-major layout the kernel copies from:
// [chunk of 16 channels][k-step][hi, lo][re, im][row group of 8][8 rows x 8 k].
void grid_table(int32_t C, int32_t taps, double beta, int32_t lbase, int32_t rows, std::vector<float>& out);

// Psi(k) = integral over |x| < taps/2 of psi(x) cos(2 pi x k / n), for k = 0..kmax.
std::vector<double> es_kernel_transform(int32_t taps, double beta, int32_t n, int32_t kmax);

}  // namespace leapgb
