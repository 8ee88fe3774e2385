/* Device-side generator of synthetic visibilities for the benchmark and test
 * workloads (not part of the calibration interface; no counterpart in the
 * reference, which reads a MeasurementSet).
 *
 * Fills a (channels, rows, pols) complex<float> cube, the reference
 * Integration layout (column-major (pol, row, channel),
 * LA/model/cpu/Integration.h:73), with
 *
 *   V[c][r][p] = gg[r mod nbl] * exp(+2 pi i delay[r] nu_c / c) + noise,
 *   nu_c = f0 + c df,
 *
 * where delay[r] = u l0 + v m0 + w (n0 - 1) in metres (the host computes it
 * in FP64 from the row's UVW), gg[b] = g_a conj(g_b) of baseline b, and each
 * noise component is N(0, sigma^2 / 2) from a counter-based generator keyed on
 * (seed, element index): the same inputs give the same cube on any GPU.
 */
#ifndef LEAP_SYNTH_H
#define LEAP_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* All pointers are device pointers; stream is a cudaStream_t (NULL = legacy
 * default stream).  Returns 0 on success, else a CUDA error code. */
int32_t leap_synth_fill_c64(void* vis, const double* delay, const double* gg /* nbl x (re, im) */, int64_t rows,
                            int32_t nbl, int32_t channels, int32_t pols, double f0, double df, double sigma,
                            uint64_t seed, void* stream);

#ifdef __cplusplus
}
#endif

#endif
