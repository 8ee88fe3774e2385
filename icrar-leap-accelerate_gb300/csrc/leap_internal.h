// Internal declarations shared by the translation units of the C ABI (leap_context.cu,
// leap_metadata.cu, leap_ingest.cu, leap_calibrate.cu, leap_adjoint.cu): the context
// and its resident buffers, and the helpers every entry point uses.  Not installed;
// include/leap_gb300.h is the contract of each entry point and names the reference
// interface it replaces.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <queue>
#include <memory>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "leap_gb300.h"
#include "host_math.h"
#include "kernels_rotate.cuh"
#include "kernels_grid.cuh"



namespace leapabi {

using namespace leapgb;

extern thread_local std::string g_last_error;

// Bumped whenever any device buffer is (re)allocated: captured CUDA graphs
// hold raw pointers, so a graph recorded before the bump is stale.
extern uint64_t g_alloc_epoch;

// Grow-only device buffer: steady-state calls reuse it and never allocate.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t need) {
    if (need <= bytes) return cudaSuccess;
    ++g_alloc_epoch;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&ptr, need);
    if (e == cudaSuccess) bytes = need;
    return e;
  }
  void release() {
    if (ptr) {
      cudaFree(ptr);
      ++g_alloc_epoch;
    }
    ptr = nullptr;
    bytes = 0;
  }
  template <typename T> T* as() const { return static_cast<T*>(ptr); }
};

struct Integration {
  DeviceBuffer vis, uvw, uvw_f;
  int32_t vis_type = LEAP_VIS_C64;
  int64_t rows = 0;
  int32_t channels = 0, pols = 0;
  bool has_map = false;
  CUtensorMap map16, map8;  // [channel][row*8 floats] views of a 4-pol complex<float> integration, box heights 16 / 8
  // Split grid operand of the gridded kernel (scaled FP16 hi/lo tiles in the MMA layout, then
  // the inverse scales), built on the first gridded call after the visibilities change;
  // op_nbl: the baseline count it was built for (0: none).
  DeviceBuffer op;
  int32_t op_nbl = 0;
  // Asynchronous ingestion: the upload runs on the context's copy stream and `ready`
  // marks its end; calibrate calls make their stream wait for it.
  cudaEvent_t ready = nullptr;
  bool pending = false;
};

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link).
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

struct Metadata {
  bool set = false;
  leap_constants k{};
  int32_t S = 0, Arows = 0, A1rows = 0, Kpad = 0;
  int32_t tc_mtiles = 0, tc_kblocks = 0;
  DeviceBuffer I1, Ad1, Ad, Ad_f32, arow, arow_val, Ad_tc;
  DeviceBuffer at_ptr, at_idx, at_val;  // A^T (rows n < |I|) in compressed-row form, for the adjoint
};

}  // namespace leapabi

using namespace leapgb;
using namespace leapabi;

// Launch choices the autotuner may set (0 = built-in heuristic).
struct TuneChoice {
  int tpb = 0;    // tiles per block of the pipelined kernel (1 or 4)
  int waves = 0;  // target rounds of the persistent grid when planning slabs
  int mma = -1;   // 1: tensor-core (mma.sync) bulk kernel, 0: CUDA-core kernel, -1: by direction count
};

struct leap_ctx {
  int device = 0;
  int sms = 152;
  bool pageable_direct = false;       // kernels can read pageable host memory in place (ATS / HMM)
  bool pipe_attr_set = false, pipe_attr_set4 = false;
  TuneChoice tune;
  bool capturing = false;             // recording a CUDA graph: skip host-side uploads and timing events
  bool autotune = true;               // tune new batched shapes on first use
  bool graph_replay = true;           // batched calls: record and replay a CUDA graph per shape
  bool tc_gemm = true;                // mixed form: Ad contraction on the tensor cores (3xTF32)
  int mma_rotate = 1;                 // tensor-core rotate + average: 0 never, 1 autotuner candidate, 2 always
  int gridded = 2;                    // gridded rotate + average (tcgen05 grid product): 0 never, 1 always,
                                      // 2 when every item has >= kGridAutoDirs directions
  bool grid_attr = false;
  bool grid_shared_groups = false;    // gridded kernel: one grid product per tile for all direction groups
  std::map<int, DeviceBuffer> grid_tabs;  // grid matrix per channel count
  std::map<int, float> grid_einv;         // ... and the inverse of its scale
  std::vector<GridItem> grid_items_host;
  std::vector<int32_t> grid_order_host;
  DeviceBuffer grid_items, grid_order, grid_win;
  bool pipe_attr_mma = false;
  int tc_attr_set = 0;                // bit per N tile whose shared-memory size was raised
  DeviceBuffer dphi_tc;               // packed dphi operand of the tensor-core contraction
  DeviceBuffer adj_dphi, adj_cal1, adj_phi1, adj_gavg, adj_partial;  // adjoint scratch
  DeviceBuffer flag_count;
  // MeasurementSet-order ingestion from pageable host memory: two pinned staging
  // buffers and their device twins, each reused once its piece has been transposed.
  static constexpr size_t kStageBytes = size_t(64) << 20;
  void* stage_host[2] = {nullptr, nullptr};
  DeviceBuffer stage_dev[2];
  cudaEvent_t stage_done[2] = {nullptr, nullptr};
  std::map<std::string, TuneChoice> tuned;
  std::string graph_key;
  cudaGraphExec_t graph_exec = nullptr;
  uint64_t graph_epoch = 0;
  std::vector<PipeItem> pipe_items_host;
  std::vector<int32_t> pipe_order_host;
  std::vector<ReduceItem> reduce_items_host, refant_reduce_host;
  std::vector<RefantItem> refant_items_host;
  DeviceBuffer pipe_items, pipe_order, reduce_items, refant_items, refant_reduce;
  cudaStream_t stream = nullptr;
  std::string err;
  Metadata md;
  std::map<int32_t, Integration> integ;
  // scratch, shared by calls on this context
  DeviceBuffer partial, avg, cal1, dphi, gemm_partial, dd, cal, dev_err, lambda, twiddle, twiddle_df, partial_i1, avg_i1,
      dirk;
  cudaStream_t aux = nullptr;           // second stream for the FP64 reference-antenna pass
  cudaStream_t copy = nullptr;          // asynchronous ingestion
  cudaEvent_t copy_fence = nullptr;     // orders an asynchronous upload after earlier calls
  cudaEvent_t fork = nullptr, join = nullptr;
  int last_ndir = 0, last_pols = 0, last_nbl = 0;
  std::vector<double> lambda_host;
  double lambda_f0 = 0.0, lambda_df = 0.0;
  // Ring of (start, after rotate, end) events, one triple per recorded call.
  static constexpr int kRing = 256;
  cudaEvent_t ring[kRing][3] = {};
  int ring_count = 0;
  int kernels_last = 0;
};

namespace leapabi {

inline int fail(leap_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  g_last_error = msg;
  return code;
}

inline int cuda_fail(leap_ctx* ctx, cudaError_t e, const char* what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? LEAP_ERR_OUT_OF_MEMORY : LEAP_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define LEAP_CUDA(call, what)                         \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
  } while (0)

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

constexpr int kPipeNC = 8;   // warps of the pipelined kernel
// Directions per item from which the gridded kernel is the default: its grid product costs
// about as much as ~25 directions of the pipelined kernel's per-direction work (measured on
// 128 antennas x 384 channels: 64 directions 1.29 vs 2.86 ms; 8 per item 35 vs 14 ms).
constexpr int kGridAutoDirs = 32;
constexpr int kPipeDPW = 4;  // directions per warp

inline int grid_1d(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return static_cast<int>(std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 32));
}

// Slab split of (timestep, channel) space so that the grid reaches `target` blocks.
inline void choose_slabs_target(int timesteps, int channels, int64_t base_blocks, int64_t target, int& t_per, int& c_per,
                         int& nts, int& ncs) {
  int64_t want = std::max<int64_t>(1, (target + base_blocks - 1) / base_blocks);
  // Keep at least 64 (timestep, channel) pairs per slab.
  const int64_t max_slabs = std::max<int64_t>(1, (static_cast<int64_t>(timesteps) * channels) / 64);
  want = std::min(want, max_slabs);
  nts = static_cast<int>(std::min<int64_t>(want, timesteps));
  t_per = (timesteps + nts - 1) / nts;
  nts = (timesteps + t_per - 1) / t_per;
  int64_t rest = (want + nts - 1) / nts;
  ncs = static_cast<int>(std::min<int64_t>(rest, std::max(1, channels / 16)));
  c_per = (channels + ncs - 1) / ncs;
  ncs = (channels + c_per - 1) / c_per;
}

// Slab split for the direct-load kernels: about 8 blocks per SM.
inline void choose_slabs(int timesteps, int channels, int64_t base_blocks, int& t_per, int& c_per, int& nts, int& ncs) {
  choose_slabs_target(timesteps, channels, base_blocks, 152 * 8, t_per, c_per, nts, ncs);
}

// Timestep slabs for the persistent pipelined kernel: the smallest split whose
// unit count fills the persistent grid to >= 95% on the last round.
inline void choose_pipe_slabs(int timesteps, int64_t base_units, int grid, int& t_per, int& nts) {
  int best = 1;
  double best_eff = 0.0;
  for (int n = 1; n <= std::min(timesteps, 16); ++n) {
    const int tp = (timesteps + n - 1) / n;
    const int nn = (timesteps + tp - 1) / tp;
    const int64_t u = base_units * nn;
    const double eff = static_cast<double>(u) / (static_cast<double>(grid) * ((u + grid - 1) / grid));
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = nn;
    }
    if (eff >= 0.95) break;
  }
  t_per = (timesteps + best - 1) / best;
  nts = (timesteps + t_per - 1) / t_per;
}

// A unit of a calibrate call: directions [dir0, dir0 + ndir) against integration `slot`.
struct WorkItem {
  int32_t slot, dir0, ndir;
};

// Defined in leap_context.cu.
int check_device_error(leap_ctx* ctx);
int fill_timings(leap_ctx* ctx, leap_timings* out);
// Defined in leap_ingest.cu.
void finish_upload(Integration& in);
// Defined in leap_calibrate.cu.
void wait_for_uploads(leap_ctx* ctx, const std::vector<WorkItem>& items, cudaStream_t s);

}  // namespace leapabi
