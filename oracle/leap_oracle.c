/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C, all-FP64 restatement of the LEAP-Accelerate CPU calibration
 * path (the reference's Eigen implementation).  The GPU product's results are
 * compared against it: only the tests, the smoke check and the benchmark's CPU
 * baseline leg may load it, and never as the thing measured or shipped.
 *
 * Each function cites the reference file:line it follows (paths relative to
 * the reference project root, src/icrar/leap-accelerate/ abbreviated LA/).
 *
 * Data layouts are the reference's:
 *   vis     complex<double> tensor (pol, row, channel), column-major, i.e.
 *           element (p, r, c) at p + P*(r + rows*c)       (LA/ms/utils.h:133-145)
 *   uvw     rows x 3 doubles, row-major (u, v, w)        (LA/ms/utils.h:44-78)
 *   avgData nbl x P complex<double>, column-major        (LA/model/cpu/MetaData.h:127)
 *   A, Ad   column-major Eigen::MatrixXd                 (LA/algorithm/cpu/PhaseMatrixFunction.cc:59)
 *
 * Compiled with -ffp-contract=off so that x86-64 and aarch64 hosts give the
 * same rounding for the arithmetic written here.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_OK 0
#define ORACLE_ERR_INVALID_ARGUMENT 1

/* LA/common/constants.h:35 */
static const double kSpeedOfLight = 299792458.0;
/* boost::math::constants::two_pi<double>() / pi<double>() */
static const double kPi = 3.141592653589793238462643383279502884;
static const double kTwoPi = 6.283185307179586476925286766559005768;

/*
 * PhaseMatrixFunction (LA/algorithm/cpu/PhaseMatrixFunction.cc:35-93).
 *
 * a1, a2, fg have n entries (first-epoch baselines).  ref_ant < 0 means "no
 * reference antenna" (boost::none).  A_out must hold (n+1) * cols doubles and
 * is written column-major with leading dimension *rows_out (the compacted row
 * count), I_out must hold n ints.  cols = max(a1, a2) + 1.
 *
 * Returns ORACLE_ERR_INVALID_ARGUMENT where the reference throws
 * invalid_argument_exception: ref_ant >= n ("out of bounds", :46-51, which
 * also covers the empty-input case) or fg[ref_ant] set ("is flagged", :52-57;
 * note that the reference indexes the per-baseline flag vector with the
 * antenna number).
 */
int oracle_phase_matrix(const int32_t* a1, const int32_t* a2, const uint8_t* fg, int32_t n,
                        int32_t ref_ant, double* A_out, int32_t* I_out,
                        int32_t* rows_out, int32_t* cols_out)
{
    if (ref_ant >= 0 && ref_ant >= n) return ORACLE_ERR_INVALID_ARGUMENT;
    if (ref_ant >= 0 && fg[ref_ant]) return ORACLE_ERR_INVALID_ARGUMENT;
    if (n <= 0) return ORACLE_ERR_INVALID_ARGUMENT;

    int32_t maxc = a1[0];
    for (int32_t i = 0; i < n; ++i) {
        if (a1[i] > maxc) maxc = a1[i];
        if (a2[i] > maxc) maxc = a2[i];
    }
    const int32_t cols = maxc + 1;

    /* Rows are first built with leading dimension n + 1 (:59), then compacted
       by conservativeResize (:89), which keeps the top-left block. */
    const int32_t ld0 = n + 1;
    double* A = (double*)calloc((size_t)ld0 * cols, sizeof(double));
    if (!A) return ORACLE_ERR_INVALID_ARGUMENT;
    int32_t k = 0;
    for (int32_t i = 0; i < n; ++i) {
        if (a1[i] != a2[i]) {
            int use = !fg[i] && (ref_ant < 0 || a1[i] == ref_ant || a2[i] == ref_ant);
            if (use) {
                A[k + (size_t)ld0 * a1[i]] = 1.0;
                A[k + (size_t)ld0 * a2[i]] = -1.0;
                I_out[k] = i;
                k++;
            }
        }
    }
    const int32_t ref = ref_ant < 0 ? 0 : ref_ant; /* :81-84 */
    A[k + (size_t)ld0 * ref] = 1.0;               /* :86 */
    k++;
    for (int32_t c = 0; c < cols; ++c)
        for (int32_t r = 0; r < k; ++r) A_out[r + (size_t)k * c] = A[r + (size_t)ld0 * c];
    free(A);
    *rows_out = k;
    *cols_out = cols;
    return ORACLE_OK;
}

/*
 * MetaData::GenerateDDMatrix (LA/model/cpu/MetaData.cc:166-203):
 * dd = dd3 * dd2 * dd1, written row-major into dd[9].
 */
void oracle_dd_matrix(double phase_ra, double phase_dec, double ra, double dec, double* dd)
{
    const double ang1 = kPi / 2.0 - phase_dec;
    const double ang2 = ra - phase_ra;
    const double ang3 = -kPi / 2.0 + dec;
    const double d1[9] = {1, 0, 0, 0, cos(ang1), -sin(ang1), 0, sin(ang1), cos(ang1)};
    const double d2[9] = {cos(ang2), sin(ang2), 0, -sin(ang2), cos(ang2), 0, 0, 0, 1};
    const double d3[9] = {1, 0, 0, 0, cos(ang3), -sin(ang3), 0, sin(ang3), cos(ang3)};
    double t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int l = 0; l < 3; ++l) s += d3[3 * i + l] * d2[3 * l + j];
            t[3 * i + j] = s;
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int l = 0; l < 3; ++l) s += t[3 * i + l] * d1[3 * l + j];
            dd[3 * i + j] = s;
        }
}

/* MetaData::CalcUVW (LA/model/cpu/MetaData.cc:220-229): rotated = dd * uvw. */
void oracle_rotate_uvw(const double* dd, const double* uvw, int64_t rows, double* out)
{
    for (int64_t r = 0; r < rows; ++r) {
        const double* x = uvw + 3 * r;
        for (int i = 0; i < 3; ++i)
            out[3 * r + i] = dd[3 * i + 0] * x[0] + dd[3 * i + 1] * x[1] + dd[3 * i + 2] * x[2];
    }
}

/*
 * CpuLeapCalibrator::RotateVisibilities (LA/algorithm/cpu/CpuLeapCalibrator.cc:181-217).
 *
 * The reference rotates its per-direction copy of the integration in place
 * and accumulates into avgData; the oracle rotates each sample on the fly,
 * which is the same arithmetic without the copy.  avg (nbl x P, column-major,
 * interleaved re/im) is ADDED to, as in the reference, where the caller
 * zeroes it first (:137).
 *
 *   shiftFactor = -2*pi*(w_rot - w)                             (:190)
 *   shiftRad    = shiftFactor / lambda_c,
 *   lambda_c    = c / (f0 + ch*df)                               (:195; MetaData.h:95-98)
 *   V[p,r,ch]  *= exp(i*shiftRad)                                (:198)
 *   if no pol of the rotated V[:,r,ch] is NaN:
 *       avg[r % nbl, p] += V[p,r,ch]                             (:201-214)
 *
 * vis_f32 selects complex<float> input (widened to double as LA/ms/utils.h:141-142 does).
 */
void oracle_rotate_visibilities(const void* vis, int vis_f32, const double* uvw, const double* dd,
                                int64_t rows, int32_t channels, int32_t pols, int32_t nbl,
                                double f0, double df, double* avg)
{
    for (int64_t r = 0; r < rows; ++r) {
        const int32_t mdb = (int32_t)(r % nbl);
        const double* x = uvw + 3 * r;
        const double wrot = dd[6] * x[0] + dd[7] * x[1] + dd[8] * x[2];
        const double shiftFactor = -kTwoPi * (wrot - x[2]);
        for (int32_t ch = 0; ch < channels; ++ch) {
            const double lambda = kSpeedOfLight / (f0 + ch * df);
            const double shiftRad = shiftFactor / lambda;
            const double er = cos(shiftRad), ei = sin(shiftRad);
            double rot[2 * 16];
            int hasNaN = 0;
            for (int32_t p = 0; p < pols; ++p) {
                const size_t idx = (size_t)p + (size_t)pols * ((size_t)r + (size_t)rows * ch);
                double vr, vi;
                if (vis_f32) {
                    vr = ((const float*)vis)[2 * idx];
                    vi = ((const float*)vis)[2 * idx + 1];
                } else {
                    vr = ((const double*)vis)[2 * idx];
                    vi = ((const double*)vis)[2 * idx + 1];
                }
                rot[2 * p] = vr * er - vi * ei;
                rot[2 * p + 1] = vr * ei + vi * er;
                hasNaN |= isnan(rot[2 * p]) || isnan(rot[2 * p + 1]);
            }
            if (!hasNaN) {
                for (int32_t p = 0; p < pols; ++p) {
                    avg[2 * ((size_t)mdb + (size_t)nbl * p)] += rot[2 * p];
                    avg[2 * ((size_t)mdb + (size_t)nbl * p) + 1] += rot[2 * p + 1];
                }
            }
        }
    }
}

/*
 * CpuLeapCalibrator::PhaseRotate, solve part (LA/algorithm/cpu/CpuLeapCalibrator.cc:159-178):
 *
 *   phaseAnglesI1 = arg(avgData[I1, 0]) ++ [0]                  (:161-163)
 *   cal1  = Ad1 * phaseAnglesI1                                  (:165)
 *   ACal1 = A * cal1                                             (:166)
 *   dInt[n] = arg(exp(-2*pi*i*ACal1[n]) * avgData[n, 0]), n<|I|  (:168-172; row n, not I[n])
 *   deltaPhase = dInt ++ [0]                                     (:174-176)
 *   cal = Ad * deltaPhase + cal1                                 (:178)
 *
 * A is A_rows x S column-major (A_rows = |I|+1), Ad is S x A_rows column-major,
 * A1 likewise with A1_rows = |I1|+1.  Only pol 0 of avg enters (:161, :174).
 */
void oracle_solve(const double* avg, int32_t nbl, const double* A, int32_t A_rows, int32_t S,
                  const double* Ad, const int32_t* I1, const double* Ad1, int32_t A1_rows,
                  double* cal_out)
{
    double* phi1 = (double*)calloc((size_t)A1_rows, sizeof(double));
    double* cal1 = (double*)calloc((size_t)S, sizeof(double));
    double* dphi = (double*)calloc((size_t)A_rows, sizeof(double));
    for (int32_t k = 0; k < A1_rows - 1; ++k) {
        int32_t b = I1[k];
        if (b < 0) b += nbl; /* VectorRangeSelect wrap-around, LA/math/cpu/vector.h:97-104 */
        phi1[k] = atan2(avg[2 * (size_t)b + 1], avg[2 * (size_t)b]);
    }
    phi1[A1_rows - 1] = 0.0;
    for (int32_t s = 0; s < S; ++s) {
        double acc = 0.0;
        for (int32_t k = 0; k < A1_rows; ++k) acc += Ad1[s + (size_t)S * k] * phi1[k];
        cal1[s] = acc;
    }
    for (int32_t n = 0; n < A_rows - 1; ++n) {
        double acal = 0.0;
        for (int32_t s = 0; s < S; ++s) acal += A[n + (size_t)A_rows * s] * cal1[s];
        const double th = -kTwoPi * acal;
        const double er = cos(th), ei = sin(th);
        const double zr = avg[2 * (size_t)n], zi = avg[2 * (size_t)n + 1];
        const double pr = er * zr - ei * zi, pi = er * zi + ei * zr;
        dphi[n] = atan2(pi, pr);
    }
    dphi[A_rows - 1] = 0.0;
    for (int32_t s = 0; s < S; ++s) {
        double acc = 0.0;
        for (int32_t k = 0; k < A_rows; ++k) acc += Ad[s + (size_t)S * k] * dphi[k];
        cal_out[s] = acc + cal1[s];
    }
    free(phi1);
    free(cal1);
    free(dphi);
}

/*
 * One solution interval, all directions: the body of the direction loop of
 * CpuLeapCalibrator::Calibrate (LA/algorithm/cpu/CpuLeapCalibrator.cc:132-139):
 * SetDirection -> CalcUVW -> zero avgData -> RotateVisibilities -> solve.
 *
 * dd holds ndir row-major 3x3 matrices.  cal_out is ndir x S.  avg_out, when
 * not NULL, receives each direction's avgData (ndir x nbl x P complex,
 * column-major per direction).  Directions are independent, so with OpenMP
 * they run on separate threads (nthreads <= 0 means all available).
 */
int oracle_calibrate_interval(const void* vis, int vis_f32, const double* uvw, int64_t rows,
                              int32_t channels, int32_t pols, int32_t nbl, double f0, double df,
                              const double* dd, int32_t ndir,
                              const double* A, int32_t A_rows, int32_t S, const double* Ad,
                              const int32_t* I1, const double* Ad1, int32_t A1_rows,
                              double* cal_out, double* avg_out, int32_t nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    (void)nthreads;
    int err = ORACLE_OK;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
#endif
    for (int32_t d = 0; d < ndir; ++d) {
        double* avg = (double*)calloc((size_t)2 * nbl * pols, sizeof(double));
        if (!avg) {
            err = ORACLE_ERR_INVALID_ARGUMENT;
            continue;
        }
        oracle_rotate_visibilities(vis, vis_f32, uvw, dd + 9 * (size_t)d, rows, channels, pols, nbl,
                                   f0, df, avg);
        oracle_solve(avg, nbl, A, A_rows, S, Ad, I1, Ad1, A1_rows, cal_out + (size_t)S * d);
        if (avg_out) memcpy(avg_out + (size_t)2 * nbl * pols * d, avg, sizeof(double) * 2 * nbl * pols);
        free(avg);
    }
    return err;
}

/*
 * Several solution intervals (integration chunks of one array, so one set of A, Ad,
 * A1, Ad1), each with its own directions: the direction loop of
 * CpuLeapCalibrator::Calibrate (LA/algorithm/cpu/CpuLeapCalibrator.cc:132-139) for
 * every chunk, one (chunk, direction) pair per task, so that all host threads are busy
 * when each chunk has fewer directions than there are threads.  Each task is exactly
 * the per-direction work of oracle_calibrate_interval.
 *
 * Chunk i: vis[i] (channels[i] x rows[i] x pols), uvw[i] (rows[i] x 3), dd[i]
 * (ndir[i] row-major 3x3), cal_out[i] (ndir[i] x S), avg_out[i] (NULL, or ndir[i]
 * avgData blocks as in oracle_calibrate_interval).
 */
int oracle_calibrate_items(int32_t nitems, const void* const* vis, int vis_f32, const double* const* uvw,
                           const int64_t* rows, const int32_t* channels, int32_t pols, int32_t nbl, double f0,
                           double df, const double* const* dd, const int32_t* ndir,
                           const double* A, int32_t A_rows, int32_t S, const double* Ad,
                           const int32_t* I1, const double* Ad1, int32_t A1_rows,
                           double* const* cal_out, double* const* avg_out, int32_t nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
    (void)nthreads;
    int64_t ntask = 0;
    for (int32_t i = 0; i < nitems; ++i) ntask += ndir[i];
    int err = ORACLE_OK;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
#endif
    for (int64_t t = 0; t < ntask; ++t) {
        int32_t i = 0;
        int64_t d = t;
        while (d >= ndir[i]) d -= ndir[i++];
        double* avg = (double*)calloc((size_t)2 * nbl * pols, sizeof(double));
        if (!avg) {
            err = ORACLE_ERR_INVALID_ARGUMENT;
            continue;
        }
        oracle_rotate_visibilities(vis[i], vis_f32, uvw[i], dd[i] + 9 * (size_t)d, rows[i], channels[i], pols, nbl,
                                   f0, df, avg);
        oracle_solve(avg, nbl, A, A_rows, S, Ad, I1, Ad1, A1_rows, cal_out[i] + (size_t)S * d);
        if (avg_out && avg_out[i]) memcpy(avg_out[i] + (size_t)2 * nbl * pols * d, avg, sizeof(double) * 2 * nbl * pols);
        free(avg);
    }
    return err;
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
