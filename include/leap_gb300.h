/*
 * leap_gb300.h — C ABI of the GB300-native LEAP calibration hot path.
 *
 * Plain C types only (pointers, sizes, POD structs); every entry point returns
 * an int32 status and never throws.  A context owns one CUDA device, one
 * stream and the device-resident buffers the reference keeps in its
 * ConstantBuffer / SolutionIntervalBuffer / DirectionBuffer / DeviceIntegration
 * objects (LA/model/cuda/DeviceMetaData.h:63-217, LA/model/cuda/DeviceIntegration.h:64-124).
 *
 * Citations name the reference interface each entry point replaces, as
 * path:line within the reference project (LA/ = src/icrar/leap-accelerate/).
 *
 * Layout conventions (all the reference's own):
 *   vis      (pol, row, channel) column-major complex tensor, i.e. a C array
 *            [channels][rows][pols] of (re, im)               (LA/ms/utils.h:133-145)
 *   uvw      [rows][3] doubles (u, v, w) in metres            (LA/ms/utils.h:44-78)
 *   A, Ad    column-major doubles, A is Arows x S, Ad is S x Arows
 *            (LA/algorithm/cpu/PhaseMatrixFunction.cc:59, LA/math/cpu/matrix_invert.h:55)
 *   dd       [ndirections][9] row-major 3x3 direction matrices
 *            (LA/model/cpu/MetaData.cc:166-203)
 *   cal      [ndirections][S] doubles, per-antenna phase calibration
 *            (LA/model/cpu/calibration/BeamCalibration.h:45-124)
 *   avgData  per direction [pols][nbl] complex doubles (nbl x pols column-major,
 *            LA/model/cpu/MetaData.h:127)
 */
#ifndef LEAP_GB300_H
#define LEAP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  LEAP_ERR_INVALID_ARGUMENT is where the reference throws
 * icrar::invalid_argument_exception (LA/exception/exception.h:35-92). */
#define LEAP_OK 0
#define LEAP_ERR_INVALID_ARGUMENT 1
#define LEAP_ERR_CUDA 2
#define LEAP_ERR_NOT_READY 3
#define LEAP_ERR_DEVICE_TIMEOUT 4
#define LEAP_ERR_OUT_OF_MEMORY 5
#define LEAP_ERR_INTERNAL 6

/* Visibility element types. */
#define LEAP_VIS_C64 0  /* complex<float>  (the MeasurementSet DATA type) */
#define LEAP_VIS_C128 1 /* complex<double> (the reference Integration type) */

/* Arithmetic forms. */
#define LEAP_PRECISION_FP64 0  /* all-FP64, matches the reference CPU path to <= 1e-10 rad */
#define LEAP_PRECISION_MIXED 1 /* FP64 phase arguments, FP32 rotation + Kahan averaging */

/* Where a pointer argument lives. */
#define LEAP_MEMORY_HOST 0
#define LEAP_MEMORY_DEVICE 1

typedef struct leap_ctx leap_ctx;

/* cpu::Constants (LA/model/cpu/MetaData.h:76-101), field for field. */
typedef struct leap_constants {
    uint32_t nbaselines;
    uint32_t referenceAntenna;
    uint32_t channels;
    uint32_t num_pols;
    uint32_t stations;
    uint32_t rows;
    double freq_start_hz;
    double freq_inc_hz;
    double phase_centre_ra_rad;
    double phase_centre_dec_rad;
    double dlm_ra;
    double dlm_dec;
} leap_constants;

/* One unit of a batched call: directions [first_direction, first_direction +
 * ndirections) of the dd array are calibrated against integration `slot`. */
typedef struct leap_work_item {
    int32_t slot;
    int32_t first_direction;
    int32_t ndirections;
    int32_t reserved;
} leap_work_item;

/* Device-side timings (CUDA events on the launching stream), summed over the
 * calibrate calls recorded since the last leap_timing_reset (at most 256). */
typedef struct leap_timings {
    float rotate_ms;   /* rotate + average (the hot kernel) */
    float solve_ms;    /* phase angles + both contractions */
    float total_ms;
    int32_t kernels;   /* kernels launched by one call (the last one) */
    int32_t calls;     /* calls summed */
} leap_timings;

/* Context lifetime.  Replaces CudaLeapCalibrator's constructor/destructor and
 * its cuBLAS handle (LA/algorithm/cuda/CudaLeapCalibrator.cu:73-92). */
int32_t leap_create(int32_t device, leap_ctx** out);
void leap_destroy(leap_ctx* ctx);

/* Message of the last failure on this context ("" if none).  Thread-local
 * message for failures without a context (ctx == NULL). */
const char* leap_last_error(const leap_ctx* ctx);

/* Upload the calibration constants; replaces ConstantBuffer construction
 * (LA/model/cuda/DeviceMetaData.h:63-112, DeviceMetaData.cu:33-47, called at
 * LA/algorithm/cuda/CudaLeapCalibrator.cu:140-148).  Every row of A must hold at
 * most two non-zeros (true of every PhaseMatrixFunction output). */
int32_t leap_set_metadata(leap_ctx* ctx, const leap_constants* constants, const double* A, int32_t A_rows,
                          int32_t A_cols, const int32_t* I, const double* Ad, const double* A1,
                          int32_t A1_rows, const int32_t* I1, const double* Ad1);

/* MetaData build on the device: from the first-epoch antenna columns a1/a2 and
 * the baseline flags fg (flagged or shorter than the minimum baseline, as
 * MeasurementSet::GetFilteredBaselines gives them, LA/ms/MeasurementSet.cc:181-240),
 * build A / I (no reference antenna) and A1 / I1 (constants->referenceAntenna) as
 * PhaseMatrixFunction does (LA/algorithm/cpu/PhaseMatrixFunction.cc:35-93), their
 * pseudo-inverses on the GPU, and install everything as leap_set_metadata would
 * (replaces the host MetaData construction, LA/model/cpu/MetaData.cc:84-136).
 * The pseudo-inverse is G^-1 A^T with G = A^T A inverted in FP64 and refined with
 * double-double residuals; when G is singular or too ill-conditioned for the
 * reference's truncation rule to leave it whole, the host SVD-style path runs
 * instead and bit 0 (A) / bit 1 (A1) of *used_host_path is set. */
int32_t leap_build_metadata(leap_ctx* ctx, const leap_constants* constants, const int32_t* a1, const int32_t* a2,
                            const uint8_t* fg, int32_t nbl, int32_t* used_host_path);

/* Copy Ad (which 0, S x Arows) or Ad1 (which 1, S x A1rows), column-major, to host
 * memory (e.g. for the reference's Ad file cache); out NULL only reports the shape. */
int32_t leap_get_metadata_matrix(leap_ctx* ctx, int32_t which, double* out, int64_t capacity, int32_t* rows_out,
                                 int32_t* cols_out);

/* Make an integration resident in HBM under `slot` (any int >= 0; a later
 * call with the same slot replaces it).  Replaces HostIntegration +
 * DeviceIntegration::Set and SolutionIntervalBuffer::SetUVW
 * (LA/model/cuda/DeviceIntegration.cu:69-84, LA/algorithm/cuda/CudaLeapCalibrator.cu:177-212).
 * `memory` says whether vis/uvw are host or device pointers; the data is
 * copied either way and groups of pols holding a NaN are zeroed on the copy. */
int32_t leap_set_integration(leap_ctx* ctx, int32_t slot, int32_t vis_type, const void* vis, const double* uvw,
                             int64_t rows, int32_t channels, int32_t pols, int32_t memory);

/* Same, from the MeasurementSet's own DATA order: ms_data is row-major
 * [rows][row_channels][pols] (the MS column layout that the reference transposes
 * and widens on the host, LA/ms/utils.h:81-146 via MeasurementSet::GetVis,
 * LA/ms/MeasurementSet.h:95-204); channels [start_channel, start_channel +
 * channels) of each row are taken.  The transpose to the Integration layout and
 * the NaN rule run on the device.  Device memory and page-locked host memory
 * are read directly by the transpose kernel, and so is pageable host memory on
 * devices that read it through the host's page tables (Grace hosts:
 * cudaDevAttrPageableMemoryAccessUsesHostPageTables); elsewhere pageable memory
 * goes through two pinned 64 MiB staging buffers, the host copy of one piece
 * overlapping the upload and transpose of the previous one. */
int32_t leap_set_integration_ms(leap_ctx* ctx, int32_t slot, int32_t vis_type, const void* ms_data,
                                int64_t row_channels, int32_t start_channel, const double* uvw, int64_t rows,
                                int32_t channels, int32_t pols, int32_t memory);

/* Asynchronous form of leap_set_integration_ms for device or page-locked host
 * memory, or pageable host memory on devices that read it in place (ms_data and
 * uvw; anything else is rejected): the upload is queued on the
 * context's copy stream, after every call already queued on the context's stream,
 * and the function returns at once.  Calibrate calls on the slot wait for it on the
 * device; rewriting or releasing the slot waits for it on the host.  The caller
 * keeps the source buffers unchanged until a call that reads the slot has
 * finished.  This overlaps the upload of the next integration chunk with the
 * calibration of the current one. */
int32_t leap_set_integration_ms_async(leap_ctx* ctx, int32_t slot, int32_t vis_type, const void* ms_data,
                                      int64_t row_channels, int32_t start_channel, const double* uvw, int64_t rows,
                                      int32_t channels, int32_t pols, int32_t memory);

/* Opt-in flagging (off unless called): zero every (row, channel) group of a resident
 * integration whose MeasurementSet FLAG is set for any pol, so flagged samples add
 * nothing to the averages.  The reference averages flagged samples and skips only
 * NaN (LA/algorithm/cpu/CpuLeapCalibrator.cc:201-214; flags enter only the phase
 * matrix, LA/ms/MeasurementSet.cc:181-240), so results match it only without this
 * call.  flags is MS order, [rows][row_channels][flag_pols] bytes (non-zero =
 * flagged), channel start_channel onwards; HOST or DEVICE memory.  The number of
 * groups zeroed is written to *flagged_groups when it is not NULL. */
int32_t leap_apply_flags(leap_ctx* ctx, int32_t slot, const uint8_t* flags, int64_t row_channels,
                         int32_t start_channel, int32_t flag_pols, int32_t memory, int64_t* flagged_groups);

/* Release the HBM held by one integration slot. */
int32_t leap_release_integration(leap_ctx* ctx, int32_t slot);

/* Calibrate ndirections directions against one resident integration: the body
 * of the direction loop of CudaLeapCalibrator::Calibrate
 * (LA/algorithm/cuda/CudaLeapCalibrator.cu:198-227, PhaseRotate :235-262).
 * dd and cal_out are HOST pointers; the call blocks until cal_out is written. */
int32_t leap_calibrate(leap_ctx* ctx, int32_t slot, const double* dd, int32_t ndirections, int32_t precision,
                       double* cal_out);

/* Same with DEVICE pointers, stream-ordered on `stream` (a cudaStream_t; NULL
 * selects the context's own non-blocking stream; pass cudaStreamLegacy to order
 * the call with work on the legacy default stream).  Does not synchronise; the context's scratch
 * buffers are shared by all calls, so calls on different streams must not overlap. */
int32_t leap_calibrate_async(leap_ctx* ctx, int32_t slot, const double* d_dd, int32_t ndirections,
                             int32_t precision, double* d_cal_out, void* stream);

/* Calibrate many (integration, direction range) work items in one call, e.g.
 * hundreds of directions spread over integration chunks of uneven timestep
 * and channel counts.  Replaces the reference's per-interval, per-direction
 * loop (LA/algorithm/cuda/CudaLeapCalibrator.cu:159-227) with one persistent
 * launch over all items and one Ad contraction for all directions.  dd holds
 * ndirections row-major 3x3 matrices (HOST), items[i] selects
 * dd[first_direction .. first_direction + ndirections); cal_out (HOST) is
 * [ndirections][S].  The first call of a new shape tunes the launch plan (see
 * leap_set_autotune) and records the launches as a CUDA graph, which later
 * calls of the same shape replay. */
int32_t leap_calibrate_batched(leap_ctx* ctx, const leap_work_item* items, int32_t nitems, const double* dd,
                               int32_t ndirections, int32_t precision, double* cal_out);

/* Failure-detection self-test (no counterpart in the reference): runs one kernel
 * whose mbarrier wait nothing completes, bounded to `polls` polls (1 .. 2^20),
 * through the same timeout path as the production kernels.  Returns
 * LEAP_ERR_DEVICE_TIMEOUT when that path works; the context stays usable. */
int32_t leap_selftest_bounded_wait(leap_ctx* ctx, int32_t polls);

/* Enable (default) or disable tuning of new batched shapes on first use. */
int32_t leap_set_autotune(leap_ctx* ctx, int32_t enable);

/* Context options (value 0 = off, 1 = on). */
#define LEAP_OPTION_AUTOTUNE 1                   /* as leap_set_autotune (default on) */
#define LEAP_OPTION_TENSOR_CORE_CONTRACTION 2    /* mixed form: Ad contraction as 3xTF32 tcgen05 MMAs (default on);
                                                    off: FP32 CUDA-core GEMM */
#define LEAP_OPTION_TENSOR_CORE_ROTATION 3       /* mixed form, 4-pol complex<float>: the rotate + average
                                                    multiply-accumulate as 3xTF32 mma.sync for items of >= 12
                                                    directions.  0: never; 1 (default): only where the batched
                                                    autotuner measures it faster; 2: always */
#define LEAP_OPTION_GRIDDED_ROTATION 4         /* mixed form, 4-pol complex<float>: evaluate each row's channel sum
                                                    at every direction's phase slope through a 2x-oversampled grid
                                                    (a type-2 non-uniform DFT): the grid values are one 3xFP16
                                                    tcgen05 product per tile, shared by all directions, then an
                                                    8-point interpolation per (row, direction).  0: never;
                                                    1: always; 2 (default): when every work item has at least
                                                    32 directions (unless the tensor-core rotation is forced) */
#define LEAP_OPTION_GRAPH_REPLAY 5             /* leap_calibrate_batched: 1 (default) records a call's launches as
                                                    a CUDA graph and replays it for later calls of the same shape;
                                                    0 launches every call eagerly, so that its timing events (and
                                                    leap_get_timings' rotate_ms) bracket the rotate + average stage */
#define LEAP_OPTION_GRID_SHARED_GROUPS 6        /* gridded rotate + average with more than 64 directions per item:
                                                    0 (default) each group of 64 directions runs its own grid
                                                    product; 1 one grid product per tile serves every group */
int32_t leap_set_option(leap_ctx* ctx, int32_t option, int32_t value);

/* Copy the avgData of `direction` from the last calibrate call to host memory
 * (pols x nbl complex doubles): MetaData::GetAvgData after RotateVisibilities
 * (LA/model/cpu/MetaData.h:127; DeviceMetaData::ToHost). */
int32_t leap_get_avgdata(leap_ctx* ctx, int32_t direction, double* out);

/* Device-side copy of pol `pol` of the avgData of every direction of the last
 * calibrate call: d_out is [ndirections][nbl] complex doubles (DEVICE), written
 * on `stream` (NULL: the context's stream).  In the mixed form the
 * reference-antenna rows hold the compensated sums the solve used. */
int32_t leap_get_avgdata_device(leap_ctx* ctx, int32_t pol, double* d_out, void* stream);

/* Adjoint of one calibrate call (rotate -> average -> arg -> solve), in FP64.
 * Replaces nothing in the reference (its path has no gradient); it is the
 * backward of the differentiable form for the Python leap_drops layer.
 * Inputs (DEVICE, on `stream`; NULL: the context's stream):
 *   d_dd        [ndirections][9] the direction matrices of the forward call
 *   d_avg0      [ndirections][nbl] complex: pol 0 of the forward's avgData
 *               (leap_get_avgdata_device right after the forward call)
 *   d_grad_cal  [ndirections][S] dL/dcal
 *   d_vis       the caller's own visibilities of slot `slot` (same type and
 *               layout as given to leap_set_integration), used to recompute the
 *               rotated samples and to find NaN groups; NULL: the slot's copy
 *               (same dL/d(l,m,n); NaN groups then receive a vis gradient)
 * Outputs:
 *   d_grad_lmn  [ndirections][3] dL/d(third row of dd) = dL/d(l, m, n)
 *   d_grad_vis  [channels][rows][pols] dL/dV as complex gradients
 *               (dL/dRe + i dL/dIm), element type of the slot; only pol 0 is
 *               non-zero; NULL: not computed.
 * The chain rule ignores arg()'s 2*pi jumps: gradients hold on the smooth
 * branch, away from angles at +-pi. */
int32_t leap_backward(leap_ctx* ctx, int32_t slot, const double* d_dd, int32_t ndirections, const double* d_avg0,
                      const double* d_grad_cal, const void* d_vis, double* d_grad_lmn, void* d_grad_vis,
                      void* stream);

/* Rotate the UVWs of a resident integration by ndirections direction matrices
 * (host dd, host out [ndirections][rows][3]).  Replaces MetaData::CalcUVW /
 * g_RotateUVW (LA/model/cpu/MetaData.cc:220-229, LA/algorithm/cuda/CudaLeapCalibrator.cu:271-293). */
int32_t leap_rotate_uvw(leap_ctx* ctx, int32_t slot, const double* dd, int32_t ndirections, double* out);

/* Timings summed over the calls since the last reset; waits for the last
 * recorded call to finish on its stream. */
int32_t leap_get_timings(leap_ctx* ctx, leap_timings* out);

/* Forget the recorded calls. */
int32_t leap_timing_reset(leap_ctx* ctx);

/* Block until the context's stream is idle and report any device-side error. */
int32_t leap_synchronize(leap_ctx* ctx);

/* ---- entry point that allocates no device memory ---- */

/* Size of the library's built-in scratch array (16 MiB), held on every GPU that
 * loads the library until the process exits. */
#define LEAP_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)

/* This entry point has no counterpart in the reference.  It is for callers that
 * must not allocate device memory while they run: code that builds or replays a
 * CUDA graph (cudaMalloc is not allowed between stream-capture begin and end),
 * hosts whose device memory is owned by another runtime's pool or arena and
 * hands this library only pre-allocated buffers, and real-time pipelines that
 * cannot take the latency or fragmentation of an allocation.
 *
 * It computes the all-FP64 rotate + average stage (RotateVisibilities,
 * LA/algorithm/cpu/CpuLeapCalibrator.cc:181-217) of one integration for
 * ndirections directions into avg_out, [ndirections][pols][nbl] complex
 * doubles (the layout of leap_get_avgdata).  vis, uvw, dd and avg_out are
 * DEVICE pointers on the current device, in the layouts above; (row, channel)
 * groups with a NaN in any pol are skipped inside the kernel.  The call only
 * launches kernels on `stream` (NULL: the default stream) and does not wait.
 *
 * Its scratch (wavelength table and partial sums) is one array of
 * LEAP_NOALLOC_SCRATCH_BYTES per device; sizes that cannot fit (more than
 * about one million channels) are rejected with LEAP_ERR_INVALID_ARGUMENT, and
 * large workloads use fewer partial-sum slabs.  All calls on a device share the
 * array, so calls that overlap on the GPU (different streams, or several host
 * threads) race and must be serialised by the caller.  The first call on each
 * device, with that device current, looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * Error text: leap_noalloc_last_error(). */
int32_t leap_rotate_average_noalloc(int32_t vis_type, const void* vis, const double* uvw, int64_t rows,
                                    int32_t channels, int32_t pols, int32_t nbl, double freq_start_hz,
                                    double freq_inc_hz, const double* dd, int32_t ndirections, double* avg_out,
                                    void* stream);

/* Message of the last failure of leap_rotate_average_noalloc on this thread. */
const char* leap_noalloc_last_error(void);

/* ---- host helpers (FP64, no device needed) ---- */

/* MetaData::GenerateDDMatrix (LA/model/cpu/MetaData.cc:166-203). */
void leap_dd_matrix(double phase_ra, double phase_dec, double ra, double dec, double* dd_out);

/* PhaseMatrixFunction (LA/algorithm/cpu/PhaseMatrixFunction.cc:35-93).  ref_ant < 0 = none.
 * A_out holds (n+1) * (max(a1, a2) + 1) doubles, written column-major with leading
 * dimension *rows_out; I_out holds n ints. */
int32_t leap_phase_matrix(const int32_t* a1, const int32_t* a2, const uint8_t* fg, int32_t n, int32_t ref_ant,
                          double* A_out, int32_t* I_out, int32_t* rows_out, int32_t* cols_out);

/* SVDPseudoInverse (LA/math/cpu/matrix_invert.h:49-56): A is rows x cols
 * column-major, Ad_out cols x rows column-major. */
int32_t leap_pseudo_inverse(const double* A, int32_t rows, int32_t cols, double* Ad_out);

#ifdef __cplusplus
}
#endif

#endif /* LEAP_GB300_H */
