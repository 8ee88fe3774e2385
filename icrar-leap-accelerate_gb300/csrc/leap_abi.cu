// C ABI of the GB300 LEAP calibration hot path: context, resident buffers,
// launch configuration.  See include/leap_gb300.h for the contract of each
// entry point and the reference interface it replaces.
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
#include "kernels_solve.cuh"
#include "kernels_tc.cuh"
#include "kernels_adjoint.cuh"
#include "kernels_ingest.cuh"
#include "kernels_metadata.cuh"
#include "kernels_mma.cuh"
#include "kernels_grid.cuh"

using namespace leapgb;

namespace {

thread_local std::string g_last_error;

// Bumped whenever any device buffer is (re)allocated: captured CUDA graphs
// hold raw pointers, so a graph recorded before the bump is stale.
uint64_t g_alloc_epoch = 0;

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
  // Split grid operand of the gridded kernel (TF32 hi/lo tiles in the MMA layout), built on
  // the first gridded call after the visibilities change; op_nbl: the baseline count it was
  // built for (0: none).
  DeviceBuffer op;
  int32_t op_nbl = 0;
  // Asynchronous ingestion: the upload runs on the context's copy stream and `ready`
  // marks its end; calibrate calls make their stream wait for it.
  cudaEvent_t ready = nullptr;
  bool pending = false;
};

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
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

}  // namespace

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

namespace {

int fail(leap_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  g_last_error = msg;
  return code;
}

int cuda_fail(leap_ctx* ctx, cudaError_t e, const char* what) {
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

int grid_1d(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return static_cast<int>(std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 32));
}

// Slab split of (timestep, channel) space so that the grid reaches `target` blocks.
void choose_slabs_target(int timesteps, int channels, int64_t base_blocks, int64_t target, int& t_per, int& c_per,
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
void choose_slabs(int timesteps, int channels, int64_t base_blocks, int& t_per, int& c_per, int& nts, int& ncs) {
  choose_slabs_target(timesteps, channels, base_blocks, 152 * 8, t_per, c_per, nts, ncs);
}

// Timestep slabs for the persistent pipelined kernel: the smallest split whose
// unit count fills the persistent grid to >= 95% on the last round.
void choose_pipe_slabs(int timesteps, int64_t base_units, int grid, int& t_per, int& nts) {
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

template <typename VisT, int P>
void launch_rotate(const RotateArgs& a, dim3 grid, int precision, cudaStream_t s) {
  if (precision == LEAP_PRECISION_FP64) {
    rotate_average_fp64<VisT, P, 2><<<grid, 128, 0, s>>>(a);
  } else {
    rotate_average_mixed<VisT, P, 4><<<grid, 128, 0, s>>>(a);
  }
}

template <typename VisT>
int dispatch_pols(const RotateArgs& a, dim3 grid, int precision, cudaStream_t s) {
  switch (a.pols) {
    case 1: launch_rotate<VisT, 1>(a, grid, precision, s); return 0;
    case 2: launch_rotate<VisT, 2>(a, grid, precision, s); return 0;
    case 4: launch_rotate<VisT, 4>(a, grid, precision, s); return 0;
    default: return -1;
  }
}

// A unit of a calibrate call: directions [dir0, dir0 + ndir) against integration `slot`.
struct WorkItem {
  int32_t slot, dir0, ndir;
};

// Grid matrix of the gridded kernel for C channels (built once per channel count).
const float* grid_table_for(leap_ctx* ctx, int C) {
  auto it = ctx->grid_tabs.find(C);
  if (it != ctx->grid_tabs.end()) return it->second.as<float>();
  if (ctx->capturing) return nullptr;
  std::vector<float> tab;
  grid_table(C, kGrTaps, kGrBeta, grid_lbase(C), grid_rows(C), tab);
  DeviceBuffer& b = ctx->grid_tabs[C];
  if (b.ensure(sizeof(float) * tab.size()) != cudaSuccess) return nullptr;
  if (cudaMemcpy(b.ptr, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
  return b.as<float>();
}

// Rotate + average of every item through the gridded kernel (4-pol complex<float>
// integrations with a tensor map): a window pass over the units, then one
// persistent launch, then the slab reduction where items were split.
int gridded_stage(leap_ctx* ctx, const std::vector<WorkItem>& items, const double* d_dd, int32_t D, cudaStream_t s,
                  int& kernels) {
  Metadata& md = ctx->md;
  const int32_t nbl = static_cast<int32_t>(md.k.nbaselines);
  const int nquad = (nbl + 3) / 4;
  std::vector<GridItem>& git = ctx->grid_items_host;
  std::vector<ReduceItem>& red = ctx->reduce_items_host;
  git.assign(items.size(), GridItem{});
  red.clear();
  // A unit is a quad of baselines over a timestep slab, for one direction group, or for all of
  // them (one grid product per tile) with LEAP_OPTION_GRID_SHARED_GROUPS.
  auto unit_groups = [&](int dgroups) { return ctx->grid_shared_groups ? dgroups : 1; };
  int64_t base_units = 0;
  for (const auto& w : items) {
    const int dgroups = (w.ndir + kGrDirs - 1) / kGrDirs;
    base_units += static_cast<int64_t>(nquad) * ((dgroups + unit_groups(dgroups) - 1) / unit_groups(dgroups));
  }
  // Timestep slabs only when the (quad, direction group) units alone would leave blocks idle.
  const int64_t want_slabs = std::max<int64_t>(1, (4 * static_cast<int64_t>(ctx->sms) + base_units - 1) / base_units);
  int units = 0;
  int64_t partial_elems = 0;
  std::vector<int64_t> partial_off(items.size(), -1);
  for (size_t i = 0; i < items.size(); ++i) {
    const WorkItem& w = items[i];
    Integration& in = ctx->integ.at(w.slot);
    const int T = static_cast<int>(in.rows / nbl);
    const int C = in.channels;
    if (in.op_nbl != nbl) {
      // The split grid operand: built once per upload (the visibilities read once, hi and lo
      // written), then read by every gridded call on this integration.
      if (ctx->capturing) return fail(ctx, LEAP_ERR_INTERNAL, "grid operand missing while recording a graph");
      LEAP_CUDA(in.op.ensure(static_cast<size_t>(grid_operand_bytes(nbl, T, C))), "alloc grid operand");
      const dim3 og((nbl + 3) / 4, (T + 3) / 4, grid_chunks(C));
      grid_split_operand<<<og, 128, 0, s>>>(in.vis.as<float>(), in.rows, nbl, T, C, (T + 3) / 4, in.op.as<float>());
      LEAP_CUDA(cudaGetLastError(), "grid operand launch");
      ++kernels;
      in.op_nbl = nbl;
    }
    const float* tab = grid_table_for(ctx, C);
    if (!tab) return fail(ctx, LEAP_ERR_CUDA, "grid matrix unavailable for this channel count");
    GridItem& it = git[i];
    it.op = in.op.as<float>();
    it.ntb = (T + 3) / 4;
    it.uvw_f = in.uvw_f.as<float>();
    it.etab = tab;
    it.T = T;
    it.C = C;
    it.nchunk = grid_chunks(C);
    const int ntb = (T + 3) / 4;
    it.dgroups = (w.ndir + kGrDirs - 1) / kGrDirs;
    it.udg = unit_groups(it.dgroups);
    it.uparts = (it.dgroups + it.udg - 1) / it.udg;
    // With several direction groups in a unit the epilogue cannot hold every group's sums
    // across the unit's tiles, so such a unit is one tile (a slab per timestep block) and its
    // sums are stored once; the fixed-order slab reduction adds the tiles.
    const int nslab_want = it.udg > 1 ? ntb : static_cast<int>(std::min<int64_t>(ntb, want_slabs));
    it.tb_per_slab = (ntb + nslab_want - 1) / nslab_want;
    it.nslab = (ntb + it.tb_per_slab - 1) / it.tb_per_slab;
    it.nquad = nquad;
    it.dir0 = w.dir0;
    it.ndir = w.ndir;
    it.unit_begin = units;
    it.nrg = grid_rows(C) / 8;
    it.lbase = grid_lbase(C);
    units += it.nquad * it.uparts * it.nslab;
    if (it.nslab > 1) {
      partial_off[i] = partial_elems;
      partial_elems += static_cast<int64_t>(it.nslab) * w.ndir * 4 * nbl;
    }
  }
  if (units == 0) return LEAP_OK;
  if (partial_elems) LEAP_CUDA(ctx->partial.ensure(sizeof(double2) * partial_elems), "alloc partial sums");
  for (size_t i = 0; i < items.size(); ++i) {
    GridItem& it = git[i];
    if (it.nslab > 1) {
      it.out = ctx->partial.as<double2>() + partial_off[i];
      red.push_back(ReduceItem{it.out, static_cast<int64_t>(it.dir0) * 4 * nbl, it.nslab, it.ndir});
    } else {
      it.out = ctx->avg.as<double2>() + static_cast<int64_t>(it.dir0) * 4 * nbl;
    }
  }
  // Longest unit first, each to the least-loaded block (cost: timestep blocks x chunks).
  const int grid = std::min(units, ctx->sms);
  {
    std::vector<std::pair<int64_t, int>> cost;
    cost.reserve(units);
    for (const GridItem& it : git) {
      const int per_item = it.nquad * it.uparts * it.nslab;
      for (int l = 0; l < per_item; ++l) {
        const int slab = l % it.nslab;
        const int t_lo = slab * it.tb_per_slab * 4, t_hi = std::min(it.T, t_lo + it.tb_per_slab * 4);
        cost.emplace_back(-static_cast<int64_t>((t_hi - t_lo + 3) / 4) * (it.nchunk + 2 * it.udg),
                          it.unit_begin + l);
      }
    }
    std::stable_sort(cost.begin(), cost.end());
    std::vector<std::vector<int32_t>> lists(grid);
    std::priority_queue<std::pair<int64_t, int>, std::vector<std::pair<int64_t, int>>, std::greater<>> load;
    for (int b = 0; b < grid; ++b) load.emplace(0, b);
    for (const auto& c : cost) {
      auto [l, b] = load.top();
      load.pop();
      lists[b].push_back(c.second);
      load.emplace(l - c.first, b);
    }
    size_t rounds = 0;
    for (const auto& l : lists) rounds = std::max(rounds, l.size());
    std::vector<int32_t>& order = ctx->grid_order_host;
    order.assign(rounds * grid + grid, -1);
    for (int b = 0; b < grid; ++b)
      for (size_t k = 0; k < lists[b].size(); ++k) order[k * grid + b] = lists[b][k];
    LEAP_CUDA(ctx->grid_order.ensure(sizeof(int32_t) * order.size()), "alloc unit order");
    if (!ctx->capturing)
      LEAP_CUDA(cudaMemcpyAsync(ctx->grid_order.ptr, order.data(), sizeof(int32_t) * order.size(),
                                cudaMemcpyHostToDevice, s),
                "upload unit order");
  }
  LEAP_CUDA(ctx->grid_items.ensure(sizeof(GridItem) * git.size()), "alloc item table");
  LEAP_CUDA(ctx->grid_win.ensure(sizeof(GridWindow) * units), "alloc grid windows");
  if (!ctx->capturing)
    LEAP_CUDA(cudaMemcpyAsync(ctx->grid_items.ptr, git.data(), sizeof(GridItem) * git.size(), cudaMemcpyHostToDevice, s),
              "upload item table");
  if (!red.empty() && !ctx->capturing) {
    LEAP_CUDA(ctx->reduce_items.ensure(sizeof(ReduceItem) * red.size()), "alloc reduce table");
    LEAP_CUDA(cudaMemcpyAsync(ctx->reduce_items.ptr, red.data(), sizeof(ReduceItem) * red.size(),
                              cudaMemcpyHostToDevice, s),
              "upload reduce table");
  }
  direction_constants<<<(D + 63) / 64, 64, 0, s>>>(d_dd, D, md.k.freq_start_hz, md.k.freq_inc_hz,
                                                   ctx->dirk.as<float>());
  ++kernels;
  GridParams gp{};
  gp.items = ctx->grid_items.as<GridItem>();
  gp.order = ctx->grid_order.as<int32_t>();
  gp.win = ctx->grid_win.as<GridWindow>();
  gp.dirk = ctx->dirk.as<float>();
  gp.twiddle = ctx->twiddle.as<float2>();
  gp.err = ctx->dev_err.as<int>();
  gp.nslots = static_cast<int32_t>(ctx->grid_order_host.size());
  gp.nitems = static_cast<int32_t>(git.size());
  gp.units = units;
  gp.nbl = nbl;
  grid_windows<<<static_cast<unsigned>((static_cast<int64_t>(units) * 32 + 255) / 256), 256, 0, s>>>(gp);
  ++kernels;
  if (!ctx->grid_attr) {
    LEAP_CUDA(cudaFuncSetAttribute(rotate_average_gridded<kGrTaps>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   grid_smem_bytes()),
              "set shared memory size");
    ctx->grid_attr = true;
  }
  rotate_average_gridded<kGrTaps><<<grid, kGrThreads, grid_smem_bytes(), s>>>(gp);
  ++kernels;
  if (!red.empty()) {
    int64_t maxn = 0;
    for (const auto& r : red) maxn = std::max<int64_t>(maxn, static_cast<int64_t>(r.ndir) * 4 * nbl);
    const dim3 rg(static_cast<unsigned>(std::min<int64_t>((maxn + 255) / 256, 1024)), static_cast<unsigned>(red.size()));
    reduce_item_slabs<<<rg, 256, 0, s>>>(ctx->reduce_items.as<ReduceItem>(), static_cast<int>(red.size()), 4 * nbl,
                                          ctx->avg.as<double2>());
    ++kernels;
  }
  return LEAP_OK;
}

// The gridded kernel runs when it is forced on, or by default when every item has enough
// directions to amortise the grid product (the tensor-core rotation option, when forced, wins);
// it needs the 4-pol complex<float> mixed form with TMA maps on every item.
bool uses_gridded(const leap_ctx* ctx, const std::vector<WorkItem>& items, int32_t D, int32_t precision, int P) {
  if (precision != LEAP_PRECISION_MIXED || P != 4 || ctx->gridded == 0) return false;
  int min_ndir = D;
  for (const auto& w : items) {
    const Integration& in = ctx->integ.at(w.slot);
    if (in.vis_type != LEAP_VIS_C64 || !in.has_map) return false;
    min_ndir = std::min(min_ndir, w.ndir);
  }
  return ctx->gridded == 1 || (ctx->mma_rotate != 2 && min_ndir >= kGridAutoDirs);
}

// Rotate + average of every item into ctx->avg ([D][P][nbl]).
int rotate_stage(leap_ctx* ctx, const std::vector<WorkItem>& items, const double* d_dd, int32_t D, int32_t precision,
                 int P, cudaStream_t s, int& kernels) {
  Metadata& md = ctx->md;
  const int32_t nbl = static_cast<int32_t>(md.k.nbaselines);
  const int tiles = (nbl + 31) / 32;
  bool all_pipe = precision == LEAP_PRECISION_MIXED && P == 4;
  int maxC = 0;
  int min_ndir = D;
  for (const auto& w : items) {
    const Integration& in = ctx->integ.at(w.slot);
    all_pipe = all_pipe && in.vis_type == LEAP_VIS_C64 && in.has_map;
    maxC = std::max(maxC, in.channels);
    min_ndir = std::min(min_ndir, w.ndir);
  }
  // Channel wavelengths, computed exactly as Constants::GetChannelWavelength does;
  // uploaded only when the channel count or the spectral window changes.
  LEAP_CUDA(ctx->lambda.ensure(sizeof(double) * 2 * maxC), "alloc wavelengths");
  if (ctx->lambda_host.size() != static_cast<size_t>(2 * maxC) || ctx->lambda_f0 != md.k.freq_start_hz ||
      ctx->lambda_df != md.k.freq_inc_hz) {
    // [wavelengths][their reciprocals]: c / (f0 + ch*df) with each operation rounded on its own,
    // as the reference's Constants::GetChannelWavelength (no fused multiply-add).
    ctx->lambda_host.resize(2 * maxC);
    for (int c = 0; c < maxC; ++c) {
      volatile double prod = static_cast<double>(c) * md.k.freq_inc_hz;
      const double lam = kSpeedOfLight / (md.k.freq_start_hz + prod);
      ctx->lambda_host[c] = lam;
      ctx->lambda_host[maxC + c] = 1.0 / lam;
    }
    ctx->lambda_f0 = md.k.freq_start_hz;
    ctx->lambda_df = md.k.freq_inc_hz;
    LEAP_CUDA(cudaMemcpyAsync(ctx->lambda.ptr, ctx->lambda_host.data(), sizeof(double) * 2 * maxC,
                              cudaMemcpyHostToDevice, s),
              "upload wavelengths");
  }

  if (uses_gridded(ctx, items, D, precision, P)) return gridded_stage(ctx, items, d_dd, D, s, kernels);
  if (all_pipe) {
    // Kernel: the tensor-core one (16 directions per unit) when the autotuner chose it or the
    // option forces it (items of at least 12 directions); else the CUDA-core one with 4 tiles
    // per block when items hold at most 8 directions (one block covers 128 baselines x 8
    // directions), else 1 tile (32 baselines x 32 directions).
    const bool mma = ctx->mma_rotate > 0 && (ctx->tune.mma >= 0 ? ctx->tune.mma == 1
                                                                : ctx->mma_rotate == 2 && min_ndir >= 12);
    const int tpb = mma ? 1 : (ctx->tune.tpb > 0) ? ctx->tune.tpb : (min_ndir <= 8 ? 4 : 1);
    const int wpt = kPipeNC / tpb;
    const int dirs_per_unit = mma ? kMmaDirs : wpt * kPipeDPW;
    const int tgroups = (tiles + tpb - 1) / tpb;
    int64_t work = 0;  // timestep-channels x unit multiplicity, for the slab plan
    for (const auto& w : items) {
      const Integration& in = ctx->integ.at(w.slot);
      work += (in.rows / nbl) * in.channels * static_cast<int64_t>(tgroups) * ((w.ndir + dirs_per_unit - 1) / dirs_per_unit);
    }
    // Target work per unit: enough units for ~target_waves rounds of the persistent grid.
    const int waves = ctx->tune.waves > 0 ? ctx->tune.waves : 4;
    const int64_t per_unit = std::max<int64_t>(1, work / (static_cast<int64_t>(ctx->sms) * waves));
    std::vector<PipeItem>& pit = ctx->pipe_items_host;
    std::vector<ReduceItem>& red = ctx->reduce_items_host;
    pit.assign(items.size(), PipeItem{});
    red.clear();
    int units = 0;
    int64_t partial_elems = 0;
    std::vector<int64_t> partial_off(items.size(), -1);
    for (size_t i = 0; i < items.size(); ++i) {
      const WorkItem& w = items[i];
      Integration& in = ctx->integ.at(w.slot);
      const int T = static_cast<int>(in.rows / nbl);
      const int C = in.channels;
      PipeItem& it = pit[i];
      it.map = tpb == 4 ? in.map8 : in.map16;
      it.uvw_f = in.uvw_f.as<float>();
      it.rows = in.rows;
      it.T = T;
      it.C = C;
      int tps;
      if (items.size() == 1 && ctx->tune.waves <= 0) {
        int nts;
        choose_pipe_slabs(T, static_cast<int64_t>(tgroups) * ((w.ndir + dirs_per_unit - 1) / dirs_per_unit), ctx->sms,
                          tps, nts);
      } else {
        tps = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(T, (per_unit + C - 1) / C)));
      }
      it.t_per_slab = tps;
      it.nslab = (T + tps - 1) / tps;
      it.tgroups = tgroups;
      it.dgroups = (w.ndir + dirs_per_unit - 1) / dirs_per_unit;
      it.dir0 = w.dir0;
      it.ndir = w.ndir;
      it.unit_begin = units;
      units += it.tgroups * it.dgroups * it.nslab;
      if (it.nslab > 1) {
        partial_off[i] = partial_elems;
        partial_elems += static_cast<int64_t>(it.nslab) * w.ndir * 4 * nbl;
      }
    }
    if (units == 0) return LEAP_OK;
    if (partial_elems) LEAP_CUDA(ctx->partial.ensure(sizeof(double2) * partial_elems), "alloc partial sums");
    for (size_t i = 0; i < items.size(); ++i) {
      PipeItem& it = pit[i];
      if (it.nslab > 1) {
        it.out = ctx->partial.as<double2>() + partial_off[i];
        red.push_back(ReduceItem{it.out, static_cast<int64_t>(it.dir0) * 4 * nbl, it.nslab, it.ndir});
      } else {
        it.out = ctx->avg.as<double2>() + static_cast<int64_t>(it.dir0) * 4 * nbl;
      }
    }
    // Unit schedule: longest unit first, each to the least-loaded block (cost in channel
    // steps: timesteps x (padded channels + a per-timestep set-up allowance)).
    const int grid = std::min(units, ctx->sms);
    {
      const int CH = tpb == 4 ? PipeShape<4>::CH : PipeShape<1>::CH;
      std::vector<std::pair<int64_t, int>> cost;
      cost.reserve(units);
      for (const PipeItem& it : pit) {
        const int64_t per_t = static_cast<int64_t>((it.C + CH - 1) / CH) * CH + 8;
        const int per_item = it.tgroups * it.dgroups * it.nslab;
        for (int l = 0; l < per_item; ++l) {
          const int slab = l % it.nslab;
          const int t_lo = slab * it.t_per_slab, t_hi = std::min(it.T, t_lo + it.t_per_slab);
          cost.emplace_back(-(t_hi - t_lo) * per_t, it.unit_begin + l);
        }
      }
      std::stable_sort(cost.begin(), cost.end());
      std::vector<std::vector<int32_t>> lists(grid);
      std::priority_queue<std::pair<int64_t, int>, std::vector<std::pair<int64_t, int>>, std::greater<>> load;
      for (int b = 0; b < grid; ++b) load.emplace(0, b);
      for (const auto& c : cost) {
        auto [l, b] = load.top();
        load.pop();
        lists[b].push_back(c.second);
        load.emplace(l - c.first, b);
      }
      size_t rounds = 0;
      for (const auto& l : lists) rounds = std::max(rounds, l.size());
      std::vector<int32_t>& order = ctx->pipe_order_host;
      order.assign(rounds * grid + grid, -1);  // one extra round of -1 ends every block
      for (int b = 0; b < grid; ++b)
        for (size_t k = 0; k < lists[b].size(); ++k) order[k * grid + b] = lists[b][k];
      LEAP_CUDA(ctx->pipe_order.ensure(sizeof(int32_t) * order.size()), "alloc unit order");
      if (!ctx->capturing)
        LEAP_CUDA(cudaMemcpyAsync(ctx->pipe_order.ptr, order.data(), sizeof(int32_t) * order.size(),
                                  cudaMemcpyHostToDevice, s),
                  "upload unit order");
    }
    LEAP_CUDA(ctx->pipe_items.ensure(sizeof(PipeItem) * pit.size()), "alloc item table");
    if (!ctx->capturing)
      LEAP_CUDA(cudaMemcpyAsync(ctx->pipe_items.ptr, pit.data(), sizeof(PipeItem) * pit.size(), cudaMemcpyHostToDevice, s),
                "upload item table");
    if (!red.empty() && !ctx->capturing) {
      LEAP_CUDA(ctx->reduce_items.ensure(sizeof(ReduceItem) * red.size()), "alloc reduce table");
      LEAP_CUDA(cudaMemcpyAsync(ctx->reduce_items.ptr, red.data(), sizeof(ReduceItem) * red.size(),
                                cudaMemcpyHostToDevice, s),
                "upload reduce table");
    }
    direction_constants<<<(D + 63) / 64, 64, 0, s>>>(d_dd, D, md.k.freq_start_hz, md.k.freq_inc_hz,
                                                     ctx->dirk.as<float>());
    ++kernels;
    PipeParams pp{};
    pp.items = ctx->pipe_items.as<PipeItem>();
    pp.order = ctx->pipe_order.as<int32_t>();
    pp.nslots = static_cast<int32_t>(ctx->pipe_order_host.size());
    pp.nitems = static_cast<int32_t>(pit.size());
    pp.units = units;
    pp.nbl = nbl;
    pp.dirk = ctx->dirk.as<float>();
    pp.twiddle = ctx->twiddle.as<float2>();
    pp.err = ctx->dev_err.as<int>();
    if (mma) {
      if (!ctx->pipe_attr_mma) {
        LEAP_CUDA(cudaFuncSetAttribute(rotate_average_mma_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       pipe_smem_bytes<1>()),
                  "set shared memory size");
        ctx->pipe_attr_mma = true;
      }
      rotate_average_mma_pipe<<<grid, kPipeNC * 32, pipe_smem_bytes<1>(), s>>>(pp);
    } else if (tpb == 4) {
      if (!ctx->pipe_attr_set4) {
        LEAP_CUDA(cudaFuncSetAttribute(rotate_average_mixed_pipe<kPipeNC, kPipeDPW, 4>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, pipe_smem_bytes<4>()),
                  "set shared memory size");
        ctx->pipe_attr_set4 = true;
      }
      rotate_average_mixed_pipe<kPipeNC, kPipeDPW, 4><<<grid, kPipeNC * 32, pipe_smem_bytes<4>(), s>>>(pp);
    } else {
      if (!ctx->pipe_attr_set) {
        LEAP_CUDA(cudaFuncSetAttribute(rotate_average_mixed_pipe<kPipeNC, kPipeDPW, 1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, pipe_smem_bytes<1>()),
                  "set shared memory size");
        ctx->pipe_attr_set = true;
      }
      rotate_average_mixed_pipe<kPipeNC, kPipeDPW, 1><<<grid, kPipeNC * 32, pipe_smem_bytes<1>(), s>>>(pp);
    }
    ++kernels;
    if (!red.empty()) {
      int64_t maxn = 0;
      for (const auto& r : red) maxn = std::max<int64_t>(maxn, static_cast<int64_t>(r.ndir) * 4 * nbl);
      const dim3 rg(static_cast<unsigned>(std::min<int64_t>((maxn + 255) / 256, 1024)), static_cast<unsigned>(red.size()));
      reduce_item_slabs<<<rg, 256, 0, s>>>(ctx->reduce_items.as<ReduceItem>(), static_cast<int>(red.size()), 4 * nbl,
                                            ctx->avg.as<double2>());
      ++kernels;
    }
    return LEAP_OK;
  }

  // Direct-load kernels, one launch per item.
  for (const auto& w : items) {
    Integration& in = ctx->integ.at(w.slot);
    const int T = static_cast<int>(in.rows / nbl);
    const int C = in.channels;
    const int dpw = precision == LEAP_PRECISION_FP64 ? 2 : 4;
    const int dgroups = (w.ndir + 4 * dpw - 1) / (4 * dpw);
    int t_per, c_per, nts, ncs;
    choose_slabs(T, C, static_cast<int64_t>(tiles) * dgroups, t_per, c_per, nts, ncs);
    const int nslab = nts * ncs;
    const int64_t n = static_cast<int64_t>(w.ndir) * P * nbl;
    if (nslab > 1) LEAP_CUDA(ctx->partial.ensure(sizeof(double2) * n * nslab), "alloc partial sums");
    RotateArgs ra{};
    ra.vis = in.vis.ptr;
    ra.uvw = in.uvw.as<double>();
    ra.dd = d_dd + 9 * static_cast<int64_t>(w.dir0);
    ra.lambda = ctx->lambda.as<double>();
    ra.inv_lambda = ctx->lambda.as<double>() + ctx->lambda_host.size() / 2;
    ra.twiddle = ctx->twiddle.as<float2>();
    ra.rows = in.rows;
    ra.channels = C;
    ra.pols = P;
    ra.nbl = nbl;
    ra.timesteps = T;
    ra.ndir = w.ndir;
    ra.f0 = md.k.freq_start_hz;
    ra.df = md.k.freq_inc_hz;
    ra.t_per_slab = t_per;
    ra.c_per_slab = c_per;
    ra.n_tslab = nts;
    ra.n_cslab = ncs;
    double2* avg_item = ctx->avg.as<double2>() + static_cast<int64_t>(w.dir0) * P * nbl;
    ra.out = nslab > 1 ? ctx->partial.as<double2>() : avg_item;
    ra.err = ctx->dev_err.as<int>();
    const dim3 grid(tiles, dgroups, nslab);
    int rc = in.vis_type == LEAP_VIS_C64 ? dispatch_pols<float2>(ra, grid, precision, s)
                                         : dispatch_pols<double2>(ra, grid, precision, s);
    if (rc != 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "unsupported polarisation count (1, 2 or 4)");
    ++kernels;
    if (nslab > 1) {
      reduce_slabs<<<grid_1d(n, 256), 256, 0, s>>>(ctx->partial.as<double2>(), nslab, n, avg_item);
      ++kernels;
    }
  }
  return LEAP_OK;
}

// Mixed form: compensated sums of pol 0 of the reference-antenna baselines into
// ctx->avg_i1 ([D][nI1]), on the aux stream.  complex<float> items go through
// one item-table launch; complex<double> items keep the FP64 kernel.
int refant_stage(leap_ctx* ctx, const std::vector<WorkItem>& items, const double* d_dd, int32_t D, int& kernels) {
  Metadata& md = ctx->md;
  const int32_t nbl = static_cast<int32_t>(md.k.nbaselines);
  const int nI1 = md.A1rows - 1;
  const int rtiles = (nI1 + 31) / 32;
  cudaStream_t a = ctx->aux;
  LEAP_CUDA(ctx->avg_i1.ensure(sizeof(double2) * static_cast<int64_t>(D) * nI1), "alloc I1 sums");
  std::vector<RefantItem>& rit = ctx->refant_items_host;
  std::vector<ReduceItem>& red = ctx->refant_reduce_host;
  rit.clear();
  red.clear();
  int64_t partial_elems = 0;
  std::vector<int64_t> off;
  int blocks = 0;
  // Each block sums 4*DPW directions of 32 reference baselines over a slab of
  // (timestep, channel) pairs.  Slabs are sized to one budget across items (about
  // 32 blocks per SM in total, several waves of the 5 resident blocks), so that chunks
  // of 1 x 48 and 64 x 384 samples give blocks of similar length instead of the same
  // number of blocks each, and the last wave is a small part of the pass.
  int64_t work_total = 0;
  for (const auto& w : items) {
    const Integration& in = ctx->integ.at(w.slot);
    work_total += (in.rows / nbl) * in.channels * rtiles * ((w.ndir + 7) / 8);
  }
  const int64_t slab_budget = std::max<int64_t>(64, (work_total + 32 * ctx->sms - 1) / (32 * ctx->sms));
  for (const auto& w : items) {
    Integration& in = ctx->integ.at(w.slot);
    const int T = static_cast<int>(in.rows / nbl);
    if (in.vis_type != LEAP_VIS_C64) {
      // FP64 kernel for complex<double> input, one launch per item.
      int rt_per, rc_per, rnts, rncs;
      const int rdg = (w.ndir + 7) / 8;
      choose_slabs_target(T, in.channels, static_cast<int64_t>(rtiles) * rdg, ctx->sms, rt_per, rc_per, rnts, rncs);
      const int rslab = rnts * rncs;
      const int64_t n = static_cast<int64_t>(w.ndir) * nI1;
      LEAP_CUDA(ctx->partial_i1.ensure(sizeof(double2) * n * rslab), "alloc I1 partials");
      RotateArgs rr{};
      rr.vis = in.vis.ptr;
      rr.uvw = in.uvw.as<double>();
      rr.dd = d_dd + 9 * static_cast<int64_t>(w.dir0);
      rr.lambda = ctx->lambda.as<double>();
      rr.inv_lambda = ctx->lambda.as<double>() + ctx->lambda_host.size() / 2;
      rr.rows = in.rows;
      rr.channels = in.channels;
      rr.pols = in.pols;
      rr.nbl = nbl;
      rr.timesteps = T;
      rr.ndir = w.ndir;
      rr.f0 = md.k.freq_start_hz;
      rr.df = md.k.freq_inc_hz;
      rr.t_per_slab = rt_per;
      rr.c_per_slab = rc_per;
      rr.n_tslab = rnts;
      rr.n_cslab = rncs;
      double2* dst = ctx->avg_i1.as<double2>() + static_cast<int64_t>(w.dir0) * nI1;
      const dim3 rgrid(rtiles, rdg, rslab);
      refant_average_fp64<double2, 2><<<rgrid, 128, 0, a>>>(rr, md.I1.as<int32_t>(), nI1,
                                                             rslab > 1 ? ctx->partial_i1.as<double2>() : dst);
      ++kernels;
      if (rslab > 1) {
        reduce_slabs<<<grid_1d(n, 256), 256, 0, a>>>(ctx->partial_i1.as<double2>(), rslab, n, dst);
        ++kernels;
      }
      continue;
    }
    RefantItem r{};
    r.vis = in.vis.as<float2>();
    r.uvw = in.uvw.as<double>();
    r.dd = d_dd + 9 * static_cast<int64_t>(w.dir0);
    r.rows = in.rows;
    r.T = T;
    r.C = in.channels;
    r.pols = in.pols;
    r.ndir = w.ndir;
    r.dgroups = (w.ndir + 7) / 8;  // 4 warps x 2 directions
    const int64_t want =
        std::max<int64_t>(1, (static_cast<int64_t>(T) * in.channels + slab_budget - 1) / slab_budget);
    r.n_tslab = static_cast<int>(std::min<int64_t>(T, want));
    r.t_per_slab = (T + r.n_tslab - 1) / r.n_tslab;
    r.n_tslab = (T + r.t_per_slab - 1) / r.t_per_slab;
    const int64_t rest = (want + r.n_tslab - 1) / r.n_tslab;
    r.n_cslab = static_cast<int>(std::min<int64_t>(rest, std::max(1, in.channels / 16)));
    r.c_per_slab = (in.channels + r.n_cslab - 1) / r.n_cslab;
    if (r.n_cslab > 1) r.c_per_slab = (r.c_per_slab + 15) / 16 * 16;  // whole blocks of kRefantPrefetch loads
    r.n_cslab = (in.channels + r.c_per_slab - 1) / r.c_per_slab;
    r.block_begin = blocks;
    blocks += rtiles * r.dgroups * r.n_tslab * r.n_cslab;
    off.push_back(partial_elems);
    partial_elems += static_cast<int64_t>(r.n_tslab) * r.n_cslab * w.ndir * nI1;
    rit.push_back(r);
    red.push_back(ReduceItem{nullptr, static_cast<int64_t>(w.dir0) * nI1, r.n_tslab * r.n_cslab, w.ndir});
  }
  if (rit.empty()) return LEAP_OK;
  LEAP_CUDA(ctx->partial_i1.ensure(sizeof(double2) * partial_elems), "alloc I1 partials");
  for (size_t i = 0; i < rit.size(); ++i) {
    rit[i].out = ctx->partial_i1.as<double2>() + off[i];
    red[i].partial = rit[i].out;
  }
  LEAP_CUDA(ctx->refant_items.ensure(sizeof(RefantItem) * rit.size()), "alloc refant table");
  LEAP_CUDA(ctx->refant_reduce.ensure(sizeof(ReduceItem) * red.size()), "alloc refant reduce table");
  if (!ctx->capturing) {
    LEAP_CUDA(cudaMemcpyAsync(ctx->refant_items.ptr, rit.data(), sizeof(RefantItem) * rit.size(), cudaMemcpyHostToDevice,
                              a),
              "upload refant table");
    LEAP_CUDA(cudaMemcpyAsync(ctx->refant_reduce.ptr, red.data(), sizeof(ReduceItem) * red.size(),
                              cudaMemcpyHostToDevice, a),
              "upload refant reduce table");
  }
  refant_average_df_items<2><<<blocks, 128, 0, a>>>(ctx->refant_items.as<RefantItem>(), static_cast<int>(rit.size()), nbl,
                                                    md.k.freq_start_hz, md.k.freq_inc_hz, md.I1.as<int32_t>(), nI1,
                                                    ctx->twiddle_df.as<float4>());
  ++kernels;
  int64_t maxn = 0;
  for (const auto& r : red) maxn = std::max<int64_t>(maxn, static_cast<int64_t>(r.ndir) * nI1);
  const dim3 rg(static_cast<unsigned>(std::min<int64_t>((maxn + 255) / 256, 1024)), static_cast<unsigned>(red.size()));
  reduce_item_slabs<<<rg, 256, 0, a>>>(ctx->refant_reduce.as<ReduceItem>(), static_cast<int>(red.size()), nI1,
                                        ctx->avg_i1.as<double2>());
  ++kernels;
  return LEAP_OK;
}

template <int N>
int launch_tc_gemm(leap_ctx* ctx, int D, int ntiles, int nkc, int kb_per_cta, cudaStream_t s, int bit) {
  Metadata& md = ctx->md;
  if (!(ctx->tc_attr_set & bit)) {
    LEAP_CUDA(cudaFuncSetAttribute(tc_gemm_ad<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_gemm_smem_bytes<N>()),
              "set shared memory size");
    ctx->tc_attr_set |= bit;
  }
  const dim3 grid(md.tc_mtiles, ntiles, nkc);
  tc_gemm_ad<N><<<grid, 128, tc_gemm_smem_bytes<N>(), s>>>(md.Ad_tc.as<float>(), ctx->dphi_tc.as<float>(), md.S, D,
                                                             md.tc_kblocks, kb_per_cta, ctx->gemm_partial.as<double>(),
                                                             ctx->dev_err.as<int>());
  return LEAP_OK;
}

// cal = Ad * dphi + cal1 for all directions on the tensor cores (3xTF32, FP32
// accumulate in TMEM), split over K across CTAs and finished in FP64.
int tc_contraction(leap_ctx* ctx, int32_t D, double* d_cal, cudaStream_t s, int& kernels) {
  Metadata& md = ctx->md;
  const int N = D <= 32 ? 32 : (D <= 64 ? 64 : (D <= 128 ? 128 : 256));
  const int ntiles = (D + N - 1) / N;
  const int tiles = md.tc_mtiles * ntiles;
  const int nkc_want = std::max(1, std::min(md.tc_kblocks, (ctx->sms + tiles - 1) / tiles));
  const int kb_per_cta = (md.tc_kblocks + nkc_want - 1) / nkc_want;
  const int nkc = (md.tc_kblocks + kb_per_cta - 1) / kb_per_cta;
  const size_t bbytes = static_cast<size_t>(ntiles) * md.tc_kblocks * 2 * tc_block_bytes(N);
  LEAP_CUDA(ctx->dphi_tc.ensure(bbytes), "alloc packed dphi");
  LEAP_CUDA(ctx->gemm_partial.ensure(sizeof(double) * static_cast<size_t>(nkc) * D * md.S), "alloc gemm partial");
  tc_pack_operand<float><<<grid_1d(static_cast<int64_t>(ntiles) * N * md.tc_kblocks * kTcKB, 256), 256, 0, s>>>(
      static_cast<const float*>(ctx->dphi.ptr), D, md.Kpad, md.Kpad, N, ntiles, md.tc_kblocks, ctx->dphi_tc.as<float>());
  int rc;
  switch (N) {
    case 32: rc = launch_tc_gemm<32>(ctx, D, ntiles, nkc, kb_per_cta, s, 1); break;
    case 64: rc = launch_tc_gemm<64>(ctx, D, ntiles, nkc, kb_per_cta, s, 2); break;
    case 128: rc = launch_tc_gemm<128>(ctx, D, ntiles, nkc, kb_per_cta, s, 4); break;
    default: rc = launch_tc_gemm<256>(ctx, D, ntiles, nkc, kb_per_cta, s, 8); break;
  }
  if (rc != LEAP_OK) return rc;
  gemm_ad_finish<<<(D * md.S + kFinishCols - 1) / kFinishCols, 256, 0, s>>>(ctx->gemm_partial.as<double>(), nkc, D,
                                                                          md.S, ctx->cal1.as<double>(), d_cal);
  kernels += 5;  // solve_dint, pack, gemm, finish (+ solve_cal1 counted by the caller)
  return LEAP_OK;
}

// Phase angles + both contractions for all D directions: avg -> cal.
int solve_stage(leap_ctx* ctx, int32_t D, int32_t precision, int P, bool refant, double* d_cal, cudaStream_t s,
                int& kernels) {
  Metadata& md = ctx->md;
  const int32_t nbl = static_cast<int32_t>(md.k.nbaselines);
  const int kchunk = 512;
  const int nk = (md.Arows + kchunk - 1) / kchunk;
  SolveArgs sa{};
  sa.avg = ctx->avg.as<double2>();
  sa.nbl = nbl;
  sa.pols = P;
  sa.ndir = D;
  sa.S = md.S;
  sa.I1 = md.I1.as<int32_t>();
  sa.Ad1 = md.Ad1.as<double>();
  sa.A1rows = md.A1rows;
  sa.arow = md.arow.as<int4>();
  sa.arow_val = md.arow_val.as<double2>();
  sa.Arows = md.Arows;
  sa.Kpad = md.Kpad;
  sa.cal1 = ctx->cal1.as<double>();
  sa.dphi = ctx->dphi.ptr;
  sa.avg_i1 = refant ? ctx->avg_i1.as<double2>() : nullptr;
  solve_cal1<<<dim3(D, (md.S + kCal1Cols - 1) / kCal1Cols), 4 * kCal1Cols, sizeof(double) * (md.A1rows + 4 * kCal1Cols),
               s>>>(sa);
  ++kernels;
  const dim3 gd((md.Kpad + 255) / 256, D);
  const dim3 gg((md.S + 63) / 64, (D + 15) / 16, nk);
  if (precision == LEAP_PRECISION_FP64) {
    solve_dint_fp64<<<gd, 256, 0, s>>>(sa);
    gemm_ad_partial<double><<<gg, 256, 0, s>>>(md.Ad.as<double>(), md.S, md.Arows, static_cast<double*>(sa.dphi), md.Kpad,
                                                D, kchunk, ctx->gemm_partial.as<double>());
  } else if (!ctx->tc_gemm) {
    solve_dint_mixed<<<gd, 256, 0, s>>>(sa);
    gemm_ad_partial<float><<<gg, 256, 0, s>>>(md.Ad_f32.as<float>(), md.S, md.Arows, static_cast<float*>(sa.dphi),
                                               md.Kpad, D, kchunk, ctx->gemm_partial.as<double>());
  } else {
    solve_dint_mixed<<<gd, 256, 0, s>>>(sa);
    return tc_contraction(ctx, D, d_cal, s, kernels);
  }
  gemm_ad_finish<<<(D * md.S + kFinishCols - 1) / kFinishCols, 256, 0, s>>>(ctx->gemm_partial.as<double>(), nk, D,
                                                                          md.S, ctx->cal1.as<double>(), d_cal);
  kernels += 3;
  return LEAP_OK;
}

// The whole calibration of a list of work items with D directions in total.
// Make stream s wait for the asynchronous uploads of the items' slots.
void wait_for_uploads(leap_ctx* ctx, const std::vector<WorkItem>& items, cudaStream_t s) {
  for (const auto& w : items) {
    auto it = ctx->integ.find(w.slot);
    if (it != ctx->integ.end() && it->second.pending) cudaStreamWaitEvent(s, it->second.ready, 0);
  }
}

// Before a slot is rewritten or freed: its asynchronous upload must be over.
void finish_upload(Integration& in) {
  if (in.pending) {
    cudaEventSynchronize(in.ready);
    in.pending = false;
  }
}

int calibrate_items(leap_ctx* ctx, const std::vector<WorkItem>& items, const double* d_dd, int32_t D, int32_t precision,
                    double* d_cal, cudaStream_t s) {
  if (!ctx->md.set) return fail(ctx, LEAP_ERR_NOT_READY, "metadata not set");
  if (D <= 0 || items.empty()) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "ndirections must be positive");
  if (precision != LEAP_PRECISION_FP64 && precision != LEAP_PRECISION_MIXED)
    return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "unknown precision");
  Metadata& md = ctx->md;
  const int32_t nbl = static_cast<int32_t>(md.k.nbaselines);
  int P = -1;
  for (const auto& w : items) {
    auto it = ctx->integ.find(w.slot);
    if (it == ctx->integ.end()) return fail(ctx, LEAP_ERR_NOT_READY, "integration slot not set");
    if (w.ndir <= 0 || w.dir0 < 0 || w.dir0 + w.ndir > D)
      return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "work item directions out of range");
    if (it->second.rows % nbl != 0)
      return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "integration rows not a multiple of the baseline count");
    if (P >= 0 && it->second.pols != P) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "work items differ in pols");
    P = it->second.pols;
  }
  const int64_t avg_elems = static_cast<int64_t>(D) * P * nbl;
  const int kchunk = 512;
  const int nk = (md.Arows + kchunk - 1) / kchunk;
  LEAP_CUDA(ctx->avg.ensure(sizeof(double2) * avg_elems), "alloc avgData");
  LEAP_CUDA(ctx->dirk.ensure(sizeof(float) * 12 * D), "alloc direction constants");
  LEAP_CUDA(ctx->cal1.ensure(sizeof(double) * D * md.S), "alloc cal1");
  LEAP_CUDA(ctx->dphi.ensure(sizeof(double) * static_cast<size_t>(D) * md.Kpad), "alloc dphi");
  LEAP_CUDA(ctx->gemm_partial.ensure(sizeof(double) * static_cast<size_t>(nk) * D * md.S), "alloc gemm partial");

  int kernels = 0;
  if (!ctx->capturing) wait_for_uploads(ctx, items, s);
  cudaEvent_t* ev = ctx->ring[ctx->ring_count % leap_ctx::kRing];
  if (!ctx->capturing) cudaEventRecord(ev[0], s);
  const bool refant = precision == LEAP_PRECISION_MIXED && md.A1rows > 1;
  if (refant) {
    LEAP_CUDA(cudaEventRecord(ctx->fork, s), "fork");
    LEAP_CUDA(cudaStreamWaitEvent(ctx->aux, ctx->fork, 0), "fork");
  }
  // The reference-antenna pass cannot share an SM with either bulk kernel (registers or shared
  // memory).  Beside the gridded kernel it goes first, so that it overlaps the small kernels
  // that set up the grid windows; beside the pipelined kernel it goes after it, so that the
  // persistent blocks, whose unit schedule assumes they start together, take the SMs first.
  const bool refant_first = refant && uses_gridded(ctx, items, D, precision, P);
  int rc = LEAP_OK;
  if (refant_first) {
    rc = refant_stage(ctx, items, d_dd, D, kernels);
    if (rc != LEAP_OK) return rc;
    LEAP_CUDA(cudaEventRecord(ctx->join, ctx->aux), "join");
  }
  rc = rotate_stage(ctx, items, d_dd, D, precision, P, s, kernels);
  if (rc != LEAP_OK) return rc;
  if (refant && !refant_first) {
    rc = refant_stage(ctx, items, d_dd, D, kernels);
    if (rc != LEAP_OK) return rc;
    LEAP_CUDA(cudaEventRecord(ctx->join, ctx->aux), "join");
  }
  if (!ctx->capturing) cudaEventRecord(ev[1], s);
  if (refant) LEAP_CUDA(cudaStreamWaitEvent(s, ctx->join, 0), "join");
  rc = solve_stage(ctx, D, precision, P, refant, d_cal, s, kernels);
  if (rc != LEAP_OK) return rc;
  if (!ctx->capturing) {
    cudaEventRecord(ev[2], s);
    ctx->ring_count++;
  }
  LEAP_CUDA(cudaGetLastError(), "kernel launch");
  ctx->last_ndir = D;
  ctx->last_pols = P;
  ctx->last_nbl = nbl;
  ctx->kernels_last = kernels;
  return LEAP_OK;
}

int calibrate_impl(leap_ctx* ctx, int32_t slot, const double* d_dd, int32_t ndir, int32_t precision, double* d_cal,
                   cudaStream_t s) {
  if (ndir <= 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "ndirections must be positive");
  return calibrate_items(ctx, {WorkItem{slot, 0, ndir}}, d_dd, ndir, precision, d_cal, s);
}

std::string batch_key(const leap_ctx* ctx, const std::vector<WorkItem>& items, int32_t D, int32_t precision) {
  std::string k = std::to_string(D) + ":" + std::to_string(precision) + (ctx->tc_gemm ? ":tc" : ":cc") +
                  ":mma" + std::to_string(ctx->mma_rotate) + ":grid" + std::to_string(ctx->gridded) +
                  (ctx->grid_shared_groups ? "s" : "");
  for (const auto& w : items) k += "|" + std::to_string(w.slot) + "," + std::to_string(w.dir0) + "," + std::to_string(w.ndir);
  return k;
}

// Autotuner: time each candidate launch plan of the batched call with CUDA
// events (after one warm-up run) and keep the fastest for this shape.
int autotune_batch(leap_ctx* ctx, const std::vector<WorkItem>& items, int32_t D, int32_t precision,
                   const std::string& key) {
  int min_ndir = D;
  for (const auto& w : items) min_ndir = std::min(min_ndir, w.ndir);
  std::vector<TuneChoice> cands;
  const int tpbs[2] = {1, 4};
  for (int tpb : tpbs) {
    if (tpb == 4 && min_ndir > 8) continue;
    for (int waves : {2, 4, 8}) cands.push_back(TuneChoice{tpb, waves, 0});
  }
  if (ctx->mma_rotate > 0 && precision == LEAP_PRECISION_MIXED && min_ndir >= 12)
    for (int waves : {2, 4, 8}) cands.push_back(TuneChoice{1, waves, 1});
  cudaEvent_t e0, e1;
  LEAP_CUDA(cudaEventCreate(&e0), "tuning event");
  LEAP_CUDA(cudaEventCreate(&e1), "tuning event");
  float best = 1e30f;
  TuneChoice choice{};
  for (const auto& c : cands) {
    ctx->tune = c;
    int rc = calibrate_items(ctx, items, ctx->dd.as<double>(), D, precision, ctx->cal.as<double>(), ctx->stream);
    if (rc != LEAP_OK) break;
    cudaEventRecord(e0, ctx->stream);
    rc = calibrate_items(ctx, items, ctx->dd.as<double>(), D, precision, ctx->cal.as<double>(), ctx->stream);
    cudaEventRecord(e1, ctx->stream);
    if (rc != LEAP_OK) break;
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      choice = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->tune = choice;
  ctx->tuned[key] = choice;
  return LEAP_OK;
}

int calibrate_batched_impl(leap_ctx* ctx, const leap_work_item* witems, int32_t nitems, int32_t D, int32_t precision) {
  if (!witems || nitems <= 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "no work items");
  std::vector<WorkItem> items(nitems);
  for (int i = 0; i < nitems; ++i) items[i] = WorkItem{witems[i].slot, witems[i].first_direction, witems[i].ndirections};
  const std::string key = batch_key(ctx, items, D, precision);
  cudaStream_t s = ctx->stream;
  if (ctx->graph_replay && ctx->graph_exec && ctx->graph_key == key && ctx->graph_epoch == g_alloc_epoch) {
    wait_for_uploads(ctx, items, s);
    cudaEvent_t* ev = ctx->ring[ctx->ring_count % leap_ctx::kRing];
    cudaEventRecord(ev[0], s);
    cudaEventRecord(ev[1], s);
    LEAP_CUDA(cudaGraphLaunch(ctx->graph_exec, s), "graph launch");
    cudaEventRecord(ev[2], s);
    ctx->ring_count++;
    return LEAP_OK;
  }
  auto t = ctx->tuned.find(key);
  if (t != ctx->tuned.end()) {
    ctx->tune = t->second;
  } else if (ctx->autotune) {
    int rc = autotune_batch(ctx, items, D, precision, key);
    if (rc != LEAP_OK) return rc;
  } else {
    ctx->tune = TuneChoice{};
  }
  // Eager run: allocates and uploads the launch tables, produces this call's result.
  int rc = calibrate_items(ctx, items, ctx->dd.as<double>(), D, precision, ctx->cal.as<double>(), s);
  if (rc != LEAP_OK) return rc;
  if (!ctx->graph_replay) return LEAP_OK;
  // Record the same launches once as a CUDA graph for the next calls of this shape.
  if (ctx->graph_exec) {
    cudaGraphExecDestroy(ctx->graph_exec);
    ctx->graph_exec = nullptr;
  }
  cudaGraph_t graph = nullptr;
  LEAP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
  ctx->capturing = true;
  const int kernels = ctx->kernels_last;
  rc = calibrate_items(ctx, items, ctx->dd.as<double>(), D, precision, ctx->cal.as<double>(), s);
  ctx->capturing = false;
  const cudaError_t ec = cudaStreamEndCapture(s, &graph);
  ctx->kernels_last = kernels;
  if (rc != LEAP_OK) return rc;
  if (ec != cudaSuccess) return cuda_fail(ctx, ec, "end capture");
  const cudaError_t ei = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) return cuda_fail(ctx, ei, "instantiate graph");
  ctx->graph_key = key;
  ctx->graph_epoch = g_alloc_epoch;
  return LEAP_OK;
}

int check_device_error(leap_ctx* ctx) {
  int h = 0;
  LEAP_CUDA(cudaMemcpy(&h, ctx->dev_err.ptr, sizeof(int), cudaMemcpyDeviceToHost), "read device error word");
  if (h != 0) {
    cudaMemset(ctx->dev_err.ptr, 0, sizeof(int));
    if (h & kDevErrTimeout) return fail(ctx, LEAP_ERR_DEVICE_TIMEOUT, "a bounded device wait gave up");
    return fail(ctx, LEAP_ERR_INTERNAL, "device reported an inconsistent shape");
  }
  return LEAP_OK;
}

int fill_timings(leap_ctx* ctx, leap_timings* out) {
  *out = leap_timings{};
  const int n = std::min(ctx->ring_count, leap_ctx::kRing);
  if (n == 0) return LEAP_OK;
  LEAP_CUDA(cudaEventSynchronize(ctx->ring[(ctx->ring_count - 1) % leap_ctx::kRing][2]), "wait for timing events");
  for (int i = 0; i < n; ++i) {
    float a = 0, b = 0;
    LEAP_CUDA(cudaEventElapsedTime(&a, ctx->ring[i][0], ctx->ring[i][1]), "elapsed time");
    LEAP_CUDA(cudaEventElapsedTime(&b, ctx->ring[i][1], ctx->ring[i][2]), "elapsed time");
    out->rotate_ms += a;
    out->solve_ms += b;
  }
  out->total_ms = out->rotate_ms + out->solve_ms;
  out->kernels = ctx->kernels_last;
  out->calls = n;
  return LEAP_OK;
}

// Split UVWs, record the shape and build the TMA views of a freshly written integration.
int finish_integration(leap_ctx* ctx, Integration& in, int32_t vis_type, int64_t rows, int32_t channels, int32_t pols) {
  LEAP_CUDA(in.uvw_f.ensure(sizeof(float) * 6 * rows), "alloc split uvw");
  split_uvw<<<grid_1d(3 * rows, 256), 256, 0, ctx->stream>>>(in.uvw.as<double>(), rows, in.uvw_f.as<float>());
  LEAP_CUDA(cudaGetLastError(), "ingestion launch");
  LEAP_CUDA(cudaStreamSynchronize(ctx->stream), "set integration");
  in.vis_type = vis_type;
  in.rows = rows;
  in.channels = channels;
  in.pols = pols;
  in.has_map = false;
  in.op_nbl = 0;
  if (vis_type == LEAP_VIS_C64 && pols == 4 && rows * 8 < (int64_t(1) << 31)) {
    // The pipelined kernels' view: 2-D floats [channels][rows*8], box 256 floats x 16 channels.
    auto enc = tensor_map_encoder();
    if (!enc) return fail(ctx, LEAP_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {static_cast<cuuint64_t>(rows) * 8, static_cast<cuuint64_t>(channels)};
    cuuint64_t strides[1] = {static_cast<cuuint64_t>(rows) * 32};
    cuuint32_t estr[2] = {1, 1};
    for (int which = 0; which < 2; ++which) {
      cuuint32_t box[2] = {256, static_cast<cuuint32_t>(which == 0 ? PipeShape<1>::CH : PipeShape<4>::CH)};
      CUresult r = enc(which == 0 ? &in.map16 : &in.map8, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, in.vis.ptr, dims, strides,
                       box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS) return fail(ctx, LEAP_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string(r));
    }
    in.has_map = true;
  }
  return LEAP_OK;
}

template <typename VisT>
int launch_ingest(leap_ctx* ctx, const void* src, int64_t row_channels, int32_t start_channel, int64_t nrows,
                  int32_t channels, int32_t pols, void* dst, int64_t rows_total, int64_t row0, cudaStream_t s,
                  int max_blocks) {
  const int TC = IngestTile<VisT>::TC;
  const int64_t tiles = ((nrows + 31) / 32) * ((channels + TC - 1) / TC);
  const int grid = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(tiles, max_blocks)));
  // Beside a running calibration (one block per SM) the blocks are 128 threads, small
  // enough in registers to share an SM with the bulk kernel's 256 x 223.
  const int threads = max_blocks <= ctx->sms ? 128 : 256;
  const VisT* sp = static_cast<const VisT*>(src);
  VisT* dp = static_cast<VisT*>(dst);
  switch (pols) {
    case 1: ingest_ms_transpose<VisT, 1><<<grid, threads, 0, s>>>(sp, row_channels, start_channel, nrows, channels, dp, rows_total, row0); break;
    case 2: ingest_ms_transpose<VisT, 2><<<grid, threads, 0, s>>>(sp, row_channels, start_channel, nrows, channels, dp, rows_total, row0); break;
    default: ingest_ms_transpose<VisT, 4><<<grid, threads, 0, s>>>(sp, row_channels, start_channel, nrows, channels, dp, rows_total, row0); break;
  }
  LEAP_CUDA(cudaGetLastError(), "ingestion kernel");
  return LEAP_OK;
}

// max_blocks: the synchronous path fills the GPU (8 blocks per SM); the asynchronous one
// keeps to one block per SM so that a calibration kernel running beside it stays resident.
int ingest(leap_ctx* ctx, int32_t vis_type, const void* src, int64_t row_channels, int32_t start_channel, int64_t nrows,
           int32_t channels, int32_t pols, void* dst, int64_t rows_total, int64_t row0, cudaStream_t s,
           int max_blocks = 0) {
  if (max_blocks <= 0) max_blocks = ctx->sms * 8;
  return vis_type == LEAP_VIS_C64
             ? launch_ingest<float2>(ctx, src, row_channels, start_channel, nrows, channels, pols, dst, rows_total, row0,
                                     s, max_blocks)
             : launch_ingest<double2>(ctx, src, row_channels, start_channel, nrows, channels, pols, dst, rows_total,
                                      row0, s, max_blocks);
}

// Install a metadata set: constants, sparse rows of A, I1, and Ad / Ad1 from host
// memory (kind HostToDevice) or device memory (DeviceToDevice).
int install_metadata(leap_ctx* ctx, const leap_constants* k, const std::vector<int4>& arow,
                     const std::vector<double2>& aval, int32_t A_cols, const int32_t* I1, int32_t A1_rows,
                     const double* Ad, const double* Ad1, cudaMemcpyKind kind) {
  const int32_t A_rows = static_cast<int32_t>(arow.size());
  for (int32_t i = 0; i + 1 < A1_rows; ++i) {
    const int64_t idx = I1[i] < 0 ? static_cast<int64_t>(I1[i]) + k->nbaselines : I1[i];
    if (idx < 0 || idx >= static_cast<int64_t>(k->nbaselines))
      return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "I1 index out of range");
  }
  Metadata& md = ctx->md;
  md.set = false;
  md.k = *k;
  md.S = A_cols;
  md.Arows = A_rows;
  md.A1rows = A1_rows;
  md.Kpad = ((A_rows + 127) / 128) * 128;
  const size_t nI1 = static_cast<size_t>(std::max(A1_rows - 1, 0));
  const size_t nad = static_cast<size_t>(A_cols) * A_rows;
  LEAP_CUDA(md.I1.ensure(sizeof(int32_t) * std::max<size_t>(nI1, 1)), "alloc I1");
  LEAP_CUDA(md.Ad1.ensure(sizeof(double) * A_cols * A1_rows), "alloc Ad1");
  LEAP_CUDA(md.Ad.ensure(sizeof(double) * nad), "alloc Ad");
  LEAP_CUDA(md.Ad_f32.ensure(sizeof(float) * nad), "alloc Ad f32");
  LEAP_CUDA(md.arow.ensure(sizeof(int4) * A_rows), "alloc A rows");
  LEAP_CUDA(md.arow_val.ensure(sizeof(double2) * A_rows), "alloc A values");
  if (nI1) LEAP_CUDA(cudaMemcpy(md.I1.ptr, I1, sizeof(int32_t) * nI1, cudaMemcpyHostToDevice), "upload I1");
  if (Ad1 != md.Ad1.as<double>())
    LEAP_CUDA(cudaMemcpy(md.Ad1.ptr, Ad1, sizeof(double) * A_cols * A1_rows, kind), "upload Ad1");
  if (Ad != md.Ad.as<double>()) LEAP_CUDA(cudaMemcpy(md.Ad.ptr, Ad, sizeof(double) * nad, kind), "upload Ad");
  to_float<<<grid_1d(static_cast<int64_t>(nad), 256), 256, 0, ctx->stream>>>(md.Ad.as<double>(), nad, md.Ad_f32.as<float>());
  LEAP_CUDA(cudaMemcpy(md.arow.ptr, arow.data(), sizeof(int4) * A_rows, cudaMemcpyHostToDevice), "upload A rows");
  LEAP_CUDA(cudaMemcpy(md.arow_val.ptr, aval.data(), sizeof(double2) * A_rows, cudaMemcpyHostToDevice), "upload A vals");
  // A^T over the rows n < |I| (the rows dInt reads), compressed by column, for the adjoint.
  {
    const int32_t nI = A_rows - 1;
    std::vector<int32_t> ptr(A_cols + 1, 0);
    for (int32_t n = 0; n < nI; ++n) {
      ++ptr[arow[n].x + 1];
      if (arow[n].y != arow[n].x) ++ptr[arow[n].y + 1];
    }
    for (int32_t c = 0; c < A_cols; ++c) ptr[c + 1] += ptr[c];
    std::vector<int32_t> idx(std::max(ptr[A_cols], 1));
    std::vector<double> val(std::max(ptr[A_cols], 1));
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int32_t n = 0; n < nI; ++n) {
      idx[fill[arow[n].x]] = n;
      val[fill[arow[n].x]++] = aval[n].x;
      if (arow[n].y != arow[n].x) {
        idx[fill[arow[n].y]] = n;
        val[fill[arow[n].y]++] = aval[n].y;
      }
    }
    LEAP_CUDA(md.at_ptr.ensure(sizeof(int32_t) * ptr.size()), "alloc A^T");
    LEAP_CUDA(md.at_idx.ensure(sizeof(int32_t) * idx.size()), "alloc A^T");
    LEAP_CUDA(md.at_val.ensure(sizeof(double) * val.size()), "alloc A^T");
    LEAP_CUDA(cudaMemcpy(md.at_ptr.ptr, ptr.data(), sizeof(int32_t) * ptr.size(), cudaMemcpyHostToDevice), "upload A^T");
    LEAP_CUDA(cudaMemcpy(md.at_idx.ptr, idx.data(), sizeof(int32_t) * idx.size(), cudaMemcpyHostToDevice), "upload A^T");
    LEAP_CUDA(cudaMemcpy(md.at_val.ptr, val.data(), sizeof(double) * val.size(), cudaMemcpyHostToDevice), "upload A^T");
  }
  // Ad split into TF32 hi/lo and packed once for the tensor-core contraction.
  md.tc_mtiles = (A_cols + kTcM - 1) / kTcM;
  md.tc_kblocks = md.Kpad / kTcKB;
  LEAP_CUDA(md.Ad_tc.ensure(static_cast<size_t>(md.tc_mtiles) * md.tc_kblocks * 2 * kTcBlockBytesA), "alloc packed Ad");
  tc_pack_ad<<<grid_1d(static_cast<int64_t>(md.tc_mtiles) * kTcM * md.tc_kblocks * kTcKB, 256), 256, 0, ctx->stream>>>(
      md.Ad.as<double>(), A_cols, A_rows, md.tc_mtiles, md.tc_kblocks, md.Ad_tc.as<float>());
  LEAP_CUDA(cudaGetLastError(), "pack Ad");
  LEAP_CUDA(cudaStreamSynchronize(ctx->stream), "pack Ad");
  md.set = true;
  return LEAP_OK;
}

// Sparse rows (column order) of a column-major dense phase matrix.
int sparse_rows(leap_ctx* ctx, const double* A, int32_t A_rows, int32_t A_cols, std::vector<int4>& arow,
                std::vector<double2>& aval) {
  arow.resize(A_rows);
  aval.resize(A_rows);
  for (int32_t r = 0; r < A_rows; ++r) {
    int nz = 0;
    int cidx[2] = {0, 0};
    double v[2] = {0.0, 0.0};
    for (int32_t c = 0; c < A_cols; ++c) {
      const double x = A[r + static_cast<size_t>(A_rows) * c];
      if (x != 0.0) {
        if (nz == 2) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "A row has more than two non-zeros");
        cidx[nz] = c;
        v[nz] = x;
        ++nz;
      }
    }
    arow[r] = make_int4(cidx[0], nz > 1 ? cidx[1] : cidx[0], 0, 0);
    aval[r] = make_double2(v[0], v[1]);
  }
  return LEAP_OK;
}

// Pseudo-inverse of a phase matrix on the device (see kernels_metadata.cuh) into
// Ad_out (device, S x Arows column-major).  Returns LEAP_OK, or LEAP_ERR_NOT_READY
// when the Gram matrix is not safely invertible (the caller then uses the host path).
int device_pinv(leap_ctx* ctx, const std::vector<int4>& arow, const std::vector<double2>& aval, int32_t S,
                double* Ad_out) {
  const int32_t m = static_cast<int32_t>(arow.size());
  // Exact integer Gram matrix and the columns A uses.
  std::vector<double> G(static_cast<size_t>(S) * S, 0.0);
  for (int32_t r = 0; r < m; ++r) {
    const int c[2] = {arow[r].x, arow[r].y};
    const double v[2] = {aval[r].x, aval[r].y};
    const int nz = c[1] != c[0] ? 2 : 1;
    for (int a = 0; a < nz; ++a)
      for (int b = 0; b < nz; ++b) G[static_cast<size_t>(c[a]) * S + c[b]] += v[a] * v[b];
  }
  std::vector<int32_t> cmp(S, -1);
  int n = 0;
  for (int32_t c = 0; c < S; ++c)
    if (G[static_cast<size_t>(c) * S + c] != 0.0) cmp[c] = n++;
  if (n == 0) return LEAP_ERR_NOT_READY;
  std::vector<double> Gc(static_cast<size_t>(n) * n);
  double gf = 0.0;
  for (int32_t i = 0; i < S; ++i)
    for (int32_t j = 0; j < S; ++j)
      if (cmp[i] >= 0 && cmp[j] >= 0) {
        const double x = G[static_cast<size_t>(i) * S + j];
        Gc[static_cast<size_t>(cmp[i]) * n + cmp[j]] = x;
        gf += x * x;
      }
  const size_t nn = static_cast<size_t>(n) * n;
  DeviceBuffer dG, dX, dR, dY, dr, df, dbad, dnorm, dcmp, darow, daval;
  struct Release {  // scratch goes on every return path
    std::initializer_list<DeviceBuffer*> bufs;
    ~Release() {
      for (DeviceBuffer* b : bufs) b->release();
    }
  } release_all{{&dG, &dX, &dR, &dY, &dr, &df, &dbad, &dnorm, &dcmp, &darow, &daval}};
  LEAP_CUDA(dG.ensure(sizeof(double) * nn), "alloc pinv");
  LEAP_CUDA(dX.ensure(sizeof(double) * nn), "alloc pinv");
  LEAP_CUDA(dR.ensure(sizeof(double) * nn), "alloc pinv");
  LEAP_CUDA(dY.ensure(sizeof(double) * nn), "alloc pinv");
  LEAP_CUDA(dr.ensure(sizeof(double) * n), "alloc pinv");
  LEAP_CUDA(df.ensure(sizeof(double) * n), "alloc pinv");
  LEAP_CUDA(dbad.ensure(sizeof(int)), "alloc pinv");
  LEAP_CUDA(dnorm.ensure(sizeof(double)), "alloc pinv");
  LEAP_CUDA(dcmp.ensure(sizeof(int32_t) * S), "alloc pinv");
  LEAP_CUDA(darow.ensure(sizeof(int4) * m), "alloc pinv");
  LEAP_CUDA(daval.ensure(sizeof(double2) * m), "alloc pinv");
  cudaStream_t s = ctx->stream;
  LEAP_CUDA(cudaMemcpyAsync(dG.ptr, Gc.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, s), "upload G");
  LEAP_CUDA(cudaMemcpyAsync(dX.ptr, dG.ptr, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s), "copy G");
  LEAP_CUDA(cudaMemcpyAsync(dcmp.ptr, cmp.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice, s), "upload columns");
  LEAP_CUDA(cudaMemcpyAsync(darow.ptr, arow.data(), sizeof(int4) * m, cudaMemcpyHostToDevice, s), "upload rows");
  LEAP_CUDA(cudaMemcpyAsync(daval.ptr, aval.data(), sizeof(double2) * m, cudaMemcpyHostToDevice, s), "upload rows");
  LEAP_CUDA(cudaMemsetAsync(dbad.ptr, 0, sizeof(int), s), "clear");
  const int ug = grid_1d(static_cast<int64_t>(nn), 256);
  for (int k = 0; k < n; ++k) {
    gj_pivot<<<1, 512, 0, s>>>(dX.as<double>(), n, k, dr.as<double>(), df.as<double>(), dbad.as<int>());
    gj_update<<<ug, 256, 0, s>>>(dX.as<double>(), n, k, dr.as<double>(), df.as<double>());
  }
  for (int step = 0; step < 2; ++step) {
    residual_dd<<<ug, 256, 0, s>>>(dX.as<double>(), dG.as<double>(), n, dR.as<double>());
    refine_apply<<<ug, 256, 0, s>>>(dX.as<double>(), dR.as<double>(), n, dY.as<double>());
    std::swap(dX.ptr, dY.ptr);
    std::swap(dX.bytes, dY.bytes);
  }
  sum_squares<<<1, 256, 0, s>>>(dX.as<double>(), static_cast<int64_t>(nn), dnorm.as<double>());
  LEAP_CUDA(cudaGetLastError(), "pinv kernels");
  int bad = 0;
  double xf2 = 0.0;
  LEAP_CUDA(cudaMemcpyAsync(&bad, dbad.ptr, sizeof(int), cudaMemcpyDeviceToHost, s), "read pivot check");
  LEAP_CUDA(cudaMemcpyAsync(&xf2, dnorm.ptr, sizeof(double), cudaMemcpyDeviceToHost, s), "read norm");
  LEAP_CUDA(cudaStreamSynchronize(s), "pinv");
  // lambda_min(G) >= 1/||X||_F; the reference truncates at max(m,n)*eps*sigma_0 on sigma,
  // i.e. at about max(m,n)*eps*lambda_0 on lambda (lambda_0 <= ||G||_F).  Keep a margin of 1e3.
  const double tol = static_cast<double>(std::max(m, S)) * std::numeric_limits<double>::epsilon() * std::sqrt(gf);
  if (bad || !(xf2 > 0.0) || !std::isfinite(xf2) || 1.0 / std::sqrt(xf2) <= 1e3 * tol) return LEAP_ERR_NOT_READY;
  assemble_pinv<<<grid_1d(static_cast<int64_t>(S) * m, 256), 256, 0, s>>>(
      dX.as<double>(), n, dcmp.as<int32_t>(), darow.as<int4>(), daval.as<double2>(), S, m, Ad_out);
  LEAP_CUDA(cudaGetLastError(), "assemble pinv");
  LEAP_CUDA(cudaStreamSynchronize(s), "assemble pinv");
  return LEAP_OK;
}

}  // namespace

extern "C" {

int32_t leap_create(int32_t device, leap_ctx** out) {
  if (!out) return fail(nullptr, LEAP_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(nullptr, LEAP_ERR_CUDA, "no CUDA device available");
  if (device < 0 || device >= n) return fail(nullptr, LEAP_ERR_INVALID_ARGUMENT, "device index out of range");
  leap_ctx* ctx = new leap_ctx();
  ctx->device = device;
  int rc = [&]() -> int {
    DeviceGuard g(device);
    LEAP_CUDA(cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device), "query SM count");
    {
      // On Grace hosts the GPU reads pageable host memory through the host's page tables
      // at the rate of page-locked memory, so ingestion reads such sources in place.
      int pageable = 0, host_tables = 0;
      LEAP_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device), "query pageable access");
      LEAP_CUDA(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device),
                "query pageable access");
      ctx->pageable_direct = pageable != 0 && host_tables != 0;
    }
    LEAP_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "create stream");
    LEAP_CUDA(cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking), "create aux stream");
    {
      // Uploads queue behind calibration work: the copy stream has the lowest priority.
      int least = 0, greatest = 0;
      LEAP_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
      LEAP_CUDA(cudaStreamCreateWithPriority(&ctx->copy, cudaStreamNonBlocking, least), "create copy stream");
    }
    LEAP_CUDA(cudaEventCreateWithFlags(&ctx->copy_fence, cudaEventDisableTiming), "create event");
    LEAP_CUDA(cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming), "create event");
    LEAP_CUDA(cudaEventCreateWithFlags(&ctx->join, cudaEventDisableTiming), "create event");
    for (auto& tri : ctx->ring)
      for (auto& ev : tri) LEAP_CUDA(cudaEventCreate(&ev), "create event");
    LEAP_CUDA(ctx->dev_err.ensure(sizeof(int)), "alloc error word");
    LEAP_CUDA(cudaMemset(ctx->dev_err.ptr, 0, sizeof(int)), "clear error word");
    // (cos, sin) of 2*pi*i/kTwiddleSize, FP64 rounded once to FP32.
    std::vector<float2> tw(kTwiddleSize);
    for (int i = 0; i < kTwiddleSize; ++i) {
      const double ang = kTwoPi * static_cast<double>(i) / kTwiddleSize;
      tw[i] = make_float2(static_cast<float>(std::cos(ang)), static_cast<float>(std::sin(ang)));
    }
    // The same angles as (hi, lo) float pairs of cos and sin for the compensated kernel.
    std::vector<float4> twd(kTwiddleSize);
    for (int i = 0; i < kTwiddleSize; ++i) {
      const double ang = kTwoPi * static_cast<double>(i) / kTwiddleSize;
      const double c = std::cos(ang), sn = std::sin(ang);
      const float ch = static_cast<float>(c), sh = static_cast<float>(sn);
      twd[i] = make_float4(ch, static_cast<float>(c - ch), sh, static_cast<float>(sn - sh));
    }
    LEAP_CUDA(ctx->twiddle_df.ensure(sizeof(float4) * kTwiddleSize), "alloc twiddle table");
    LEAP_CUDA(cudaMemcpy(ctx->twiddle_df.ptr, twd.data(), sizeof(float4) * kTwiddleSize, cudaMemcpyHostToDevice),
              "upload twiddle table");
    LEAP_CUDA(ctx->twiddle.ensure(sizeof(float2) * kTwiddleSize), "alloc twiddle table");
    LEAP_CUDA(cudaMemcpy(ctx->twiddle.ptr, tw.data(), sizeof(float2) * kTwiddleSize, cudaMemcpyHostToDevice),
              "upload twiddle table");
    return LEAP_OK;
  }();
  if (rc != LEAP_OK) {
    g_last_error = ctx->err;
    leap_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return LEAP_OK;
}

void leap_destroy(leap_ctx* ctx) {
  if (!ctx) return;
  {
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->integ) {
      kv.second.vis.release();
      kv.second.uvw.release();
      kv.second.uvw_f.release();
    }
    Metadata& md = ctx->md;
    md.I1.release(); md.Ad1.release(); md.Ad.release(); md.Ad_f32.release(); md.arow.release(); md.arow_val.release();
    md.Ad_tc.release();
    md.at_ptr.release(); md.at_idx.release(); md.at_val.release();
    ctx->dphi_tc.release();
    ctx->partial.release(); ctx->avg.release(); ctx->cal1.release(); ctx->dphi.release();
    ctx->gemm_partial.release(); ctx->dd.release(); ctx->cal.release(); ctx->dev_err.release(); ctx->lambda.release();
    ctx->dirk.release();
    ctx->twiddle.release();
    ctx->twiddle_df.release();
    for (auto& kv : ctx->grid_tabs) kv.second.release();
    ctx->grid_items.release(); ctx->grid_order.release(); ctx->grid_win.release();
    for (auto& tri : ctx->ring)
      for (auto& ev : tri)
        if (ev) cudaEventDestroy(ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->aux) cudaStreamDestroy(ctx->aux);
    if (ctx->copy) {
      cudaStreamSynchronize(ctx->copy);
      cudaStreamDestroy(ctx->copy);
    }
    if (ctx->copy_fence) cudaEventDestroy(ctx->copy_fence);
    for (auto& kv : ctx->integ)
      if (kv.second.ready) cudaEventDestroy(kv.second.ready);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    if (ctx->join) cudaEventDestroy(ctx->join);
    ctx->partial_i1.release();
    ctx->avg_i1.release();
    ctx->pipe_items.release();
    ctx->pipe_order.release();
    ctx->reduce_items.release();
    ctx->refant_items.release();
    ctx->refant_reduce.release();
    ctx->adj_dphi.release(); ctx->adj_cal1.release(); ctx->adj_phi1.release(); ctx->adj_gavg.release();
    ctx->adj_partial.release();
    ctx->flag_count.release();
    for (int b = 0; b < 2; ++b) {
      ctx->stage_dev[b].release();
      if (ctx->stage_host[b]) cudaFreeHost(ctx->stage_host[b]);
      if (ctx->stage_done[b]) cudaEventDestroy(ctx->stage_done[b]);
    }
  }
  delete ctx;
}

const char* leap_last_error(const leap_ctx* ctx) { return ctx ? ctx->err.c_str() : g_last_error.c_str(); }

int32_t leap_set_metadata(leap_ctx* ctx, const leap_constants* k, const double* A, int32_t A_rows, int32_t A_cols,
                          const int32_t* I, const double* Ad, const double* A1, int32_t A1_rows, const int32_t* I1,
                          const double* Ad1) {
  if (!ctx || !k || !A || !Ad || !A1 || !I1 || !Ad1) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  (void)I;
  if (A_rows < 1 || A_cols < 1 || A1_rows < 1) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "empty phase matrix");
  if (k->nbaselines == 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "nbaselines must be positive");
  if (static_cast<int64_t>(A_rows) - 1 > static_cast<int64_t>(k->nbaselines))
    return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "A has more rows than baselines + 1");
  DeviceGuard g(ctx->device);
  std::vector<int4> arow;
  std::vector<double2> aval;
  int rc = sparse_rows(ctx, A, A_rows, A_cols, arow, aval);
  if (rc != LEAP_OK) return rc;
  return install_metadata(ctx, k, arow, aval, A_cols, I1, A1_rows, Ad, Ad1, cudaMemcpyHostToDevice);
}

int32_t leap_build_metadata(leap_ctx* ctx, const leap_constants* k, const int32_t* a1, const int32_t* a2,
                            const uint8_t* fg, int32_t nbl, int32_t* used_host_path) {
  if (!ctx || !k || !a1 || !a2 || !fg) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (nbl <= 0 || static_cast<uint32_t>(nbl) != k->nbaselines)
    return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "nbl must equal constants.nbaselines");
  DeviceGuard g(ctx->device);
  std::string err;
  std::vector<SparseRow> sA, sA1;
  std::vector<int32_t> I, I1;
  int32_t cols = 0, cols1 = 0;
  int rc = phase_matrix_sparse(a1, a2, fg, nbl, -1, sA, I, cols, err);
  if (rc != LEAP_OK) return fail(ctx, rc, err);
  rc = phase_matrix_sparse(a1, a2, fg, nbl, static_cast<int32_t>(k->referenceAntenna), sA1, I1, cols1, err);
  if (rc != LEAP_OK) return fail(ctx, rc, err);
  auto to_dev = [](const std::vector<SparseRow>& r, std::vector<int4>& ar, std::vector<double2>& av) {
    ar.resize(r.size());
    av.resize(r.size());
    for (size_t i = 0; i < r.size(); ++i) {
      ar[i] = make_int4(r[i].c0, r[i].c1, 0, 0);
      av[i] = make_double2(r[i].v0, r[i].v1);
    }
  };
  std::vector<int4> arow, arow1;
  std::vector<double2> aval, aval1;
  to_dev(sA, arow, aval);
  to_dev(sA1, arow1, aval1);
  const int32_t A_rows = static_cast<int32_t>(arow.size()), A1_rows = static_cast<int32_t>(arow1.size());
  Metadata& md = ctx->md;
  md.set = false;
  LEAP_CUDA(md.Ad.ensure(sizeof(double) * cols * A_rows), "alloc Ad");
  LEAP_CUDA(md.Ad1.ensure(sizeof(double) * cols * A1_rows), "alloc Ad1");
  int host = 0;
  for (int which = 0; which < 2; ++which) {
    const auto& ar = which == 0 ? arow : arow1;
    const auto& av = which == 0 ? aval : aval1;
    double* out = which == 0 ? md.Ad.as<double>() : md.Ad1.as<double>();
    rc = device_pinv(ctx, ar, av, cols, out);
    if (rc == LEAP_ERR_NOT_READY) {
      // Rank-deficient or ill-conditioned Gram matrix: the SVD-style host path, as the reference truncates.
      host |= 1 << which;
      const int32_t rows = static_cast<int32_t>(ar.size());
      std::vector<double> A(static_cast<size_t>(rows) * cols, 0.0), Ad(static_cast<size_t>(rows) * cols);
      for (int32_t r = 0; r < rows; ++r) {
        A[r + static_cast<size_t>(rows) * ar[r].x] = av[r].x;
        if (ar[r].y != ar[r].x) A[r + static_cast<size_t>(rows) * ar[r].y] = av[r].y;
      }
      rc = pseudo_inverse(A.data(), rows, cols, Ad.data(), err);
      if (rc != LEAP_OK) return fail(ctx, rc, err);
      LEAP_CUDA(cudaMemcpy(out, Ad.data(), sizeof(double) * Ad.size(), cudaMemcpyHostToDevice), "upload Ad");
    } else if (rc != LEAP_OK) {
      return rc;
    }
  }
  if (used_host_path) *used_host_path = host;
  return install_metadata(ctx, k, arow, aval, cols, I1.data(), A1_rows, md.Ad.as<double>(), md.Ad1.as<double>(),
                          cudaMemcpyDeviceToDevice);
}

int32_t leap_get_metadata_matrix(leap_ctx* ctx, int32_t which, double* out, int64_t capacity, int32_t* rows_out,
                                 int32_t* cols_out) {
  if (!ctx) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL context");
  if (!ctx->md.set) return fail(ctx, LEAP_ERR_NOT_READY, "metadata not set");
  const Metadata& md = ctx->md;
  if (which != 0 && which != 1) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "which must be 0 (Ad) or 1 (Ad1)");
  const int32_t cols = which == 0 ? md.Arows : md.A1rows;
  if (rows_out) *rows_out = md.S;
  if (cols_out) *cols_out = cols;
  if (!out) return LEAP_OK;
  const int64_t n = static_cast<int64_t>(md.S) * cols;
  if (capacity < n) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "output capacity too small");
  DeviceGuard g(ctx->device);
  LEAP_CUDA(cudaMemcpy(out, which == 0 ? md.Ad.ptr : md.Ad1.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost), "copy Ad");
  return LEAP_OK;
}

int32_t leap_set_integration(leap_ctx* ctx, int32_t slot, int32_t vis_type, const void* vis, const double* uvw,
                             int64_t rows, int32_t channels, int32_t pols, int32_t memory) {
  if (!ctx || !vis || !uvw) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (slot < 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "slot must be >= 0");
  if (vis_type != LEAP_VIS_C64 && vis_type != LEAP_VIS_C128) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "unknown vis type");
  if (rows <= 0 || channels <= 0 || pols <= 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "empty integration");
  if (pols != 1 && pols != 2 && pols != 4) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "pols must be 1, 2 or 4");
  if (memory != LEAP_MEMORY_HOST && memory != LEAP_MEMORY_DEVICE) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "unknown memory kind");
  DeviceGuard g(ctx->device);
  Integration& in = ctx->integ[slot];
  finish_upload(in);
  const size_t esz = vis_type == LEAP_VIS_C64 ? sizeof(float2) : sizeof(double2);
  const int64_t groups = rows * channels;
  const size_t vbytes = esz * static_cast<size_t>(groups) * pols;
  LEAP_CUDA(in.vis.ensure(vbytes), "alloc vis");
  LEAP_CUDA(in.uvw.ensure(sizeof(double) * 3 * rows), "alloc uvw");
  const cudaMemcpyKind kind = memory == LEAP_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  LEAP_CUDA(cudaMemcpyAsync(in.vis.ptr, vis, vbytes, kind, ctx->stream), "copy vis");
  LEAP_CUDA(cudaMemcpyAsync(in.uvw.ptr, uvw, sizeof(double) * 3 * rows, kind, ctx->stream), "copy uvw");
  const int grid = grid_1d(groups, 256);
  if (vis_type == LEAP_VIS_C64) {
    float2* p = in.vis.as<float2>();
    if (pols == 4) sanitize_nan_groups<float2, 4><<<grid, 256, 0, ctx->stream>>>(p, p, groups);
    else sanitize_nan_groups_generic<float2><<<grid, 256, 0, ctx->stream>>>(p, p, groups, pols);
  } else {
    double2* p = in.vis.as<double2>();
    if (pols == 4) sanitize_nan_groups<double2, 4><<<grid, 256, 0, ctx->stream>>>(p, p, groups);
    else sanitize_nan_groups_generic<double2><<<grid, 256, 0, ctx->stream>>>(p, p, groups, pols);
  }
  return finish_integration(ctx, in, vis_type, rows, channels, pols);
}


int32_t leap_set_integration_ms(leap_ctx* ctx, int32_t slot, int32_t vis_type, const void* ms_data, int64_t row_channels,
                                int32_t start_channel, const double* uvw, int64_t rows, int32_t channels, int32_t pols,
                                int32_t memory) {
  if (!ctx || !ms_data || !uvw) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (slot < 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "slot must be >= 0");
  if (vis_type != LEAP_VIS_C64 && vis_type != LEAP_VIS_C128) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "unknown vis type");
  if (rows <= 0 || channels <= 0 || pols <= 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "empty integration");
  if (pols != 1 && pols != 2 && pols != 4) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "pols must be 1, 2 or 4");
  if (start_channel < 0 || static_cast<int64_t>(start_channel) + channels > row_channels)
    return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "channel range outside the MeasurementSet row");
  if (memory != LEAP_MEMORY_HOST && memory != LEAP_MEMORY_DEVICE) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "unknown memory kind");
  DeviceGuard g(ctx->device);
  Integration& in = ctx->integ[slot];
  finish_upload(in);
  const size_t esz = vis_type == LEAP_VIS_C64 ? sizeof(float2) : sizeof(double2);
  LEAP_CUDA(in.vis.ensure(esz * static_cast<size_t>(rows) * channels * pols), "alloc vis");
  LEAP_CUDA(in.uvw.ensure(sizeof(double) * 3 * rows), "alloc uvw");
  cudaStream_t s = ctx->stream;
  LEAP_CUDA(cudaMemcpyAsync(in.uvw.ptr, uvw, sizeof(double) * 3 * rows,
                            memory == LEAP_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s),
            "copy uvw");
  // A source the kernel can read directly: device memory, or page-locked host memory
  // through its device mapping (read over the host link, no staging copy).
  const void* direct = memory == LEAP_MEMORY_DEVICE ? ms_data : nullptr;
  if (!direct) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, ms_data) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
      direct = at.devicePointer;
    else
      cudaGetLastError();  // pageable memory: not an error
    if (!direct && ctx->pageable_direct) direct = ms_data;  // pageable, read in place
  }
  if (direct) {
    int rc = ingest(ctx, vis_type, direct, row_channels, start_channel, rows, channels, pols, in.vis.ptr, rows, 0, s);
    if (rc != LEAP_OK) return rc;
  } else {
    // Pageable host memory: pieces of whole rows go through the pinned staging buffers.
    // The host copy of piece k overlaps the upload and transpose of piece k-1.
    const size_t row_bytes = esz * static_cast<size_t>(channels) * pols;
    const int64_t piece_rows = std::max<int64_t>(1, static_cast<int64_t>(leap_ctx::kStageBytes / row_bytes));
    const size_t stage_bytes = row_bytes * static_cast<size_t>(std::min<int64_t>(piece_rows, rows));
    for (int b = 0; b < 2; ++b) {
      if (!ctx->stage_host[b]) {
        LEAP_CUDA(cudaHostAlloc(&ctx->stage_host[b], std::max(stage_bytes, leap_ctx::kStageBytes), cudaHostAllocDefault),
                  "alloc pinned staging");
        LEAP_CUDA(cudaEventCreateWithFlags(&ctx->stage_done[b], cudaEventDisableTiming), "staging event");
      }
      LEAP_CUDA(ctx->stage_dev[b].ensure(std::max(stage_bytes, leap_ctx::kStageBytes)), "alloc device staging");
    }
    const unsigned char* base = static_cast<const unsigned char*>(ms_data);
    const size_t src_row_bytes = esz * static_cast<size_t>(row_channels) * pols;
    int k = 0;
    for (int64_t r0 = 0; r0 < rows; r0 += piece_rows, ++k) {
      const int b = k & 1;
      const int64_t nr = std::min(piece_rows, rows - r0);
      if (k >= 2) LEAP_CUDA(cudaEventSynchronize(ctx->stage_done[b]), "staging wait");
      unsigned char* h = static_cast<unsigned char*>(ctx->stage_host[b]);
      for (int64_t r = 0; r < nr; ++r)
        std::memcpy(h + r * row_bytes, base + (r0 + r) * src_row_bytes + esz * static_cast<size_t>(start_channel) * pols,
                    row_bytes);
      LEAP_CUDA(cudaMemcpyAsync(ctx->stage_dev[b].ptr, h, row_bytes * nr, cudaMemcpyHostToDevice, s), "upload piece");
      int rc = ingest(ctx, vis_type, ctx->stage_dev[b].ptr, channels, 0, nr, channels, pols, in.vis.ptr, rows, r0, s);
      if (rc != LEAP_OK) return rc;
      LEAP_CUDA(cudaEventRecord(ctx->stage_done[b], s), "staging event");
    }
  }
  return finish_integration(ctx, in, vis_type, rows, channels, pols);
}

int32_t leap_set_integration_ms_async(leap_ctx* ctx, int32_t slot, int32_t vis_type, const void* ms_data,
                                      int64_t row_channels, int32_t start_channel, const double* uvw, int64_t rows,
                                      int32_t channels, int32_t pols, int32_t memory) {
  if (!ctx || !ms_data || !uvw) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (slot < 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "slot must be >= 0");
  if (vis_type != LEAP_VIS_C64 && vis_type != LEAP_VIS_C128) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "unknown vis type");
  if (rows <= 0 || channels <= 0 || pols <= 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "empty integration");
  if (pols != 1 && pols != 2 && pols != 4) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "pols must be 1, 2 or 4");
  if (start_channel < 0 || static_cast<int64_t>(start_channel) + channels > row_channels)
    return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "channel range outside the MeasurementSet row");
  if (memory != LEAP_MEMORY_HOST && memory != LEAP_MEMORY_DEVICE) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "unknown memory kind");
  DeviceGuard g(ctx->device);
  // The kernel reads the source directly: device memory or page-locked host memory only.
  const void* direct = memory == LEAP_MEMORY_DEVICE ? ms_data : nullptr;
  bool uvw_pinned = memory == LEAP_MEMORY_DEVICE;
  if (memory == LEAP_MEMORY_HOST) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, ms_data) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
      direct = at.devicePointer;
    cudaGetLastError();
    cudaPointerAttributes au{};
    uvw_pinned = cudaPointerGetAttributes(&au, uvw) == cudaSuccess && au.type == cudaMemoryTypeHost;
    cudaGetLastError();
    if (!direct && ctx->pageable_direct) direct = ms_data;  // pageable, read in place
    if (!uvw_pinned && ctx->pageable_direct) uvw_pinned = true;
  }
  if (!direct || !uvw_pinned)
    return fail(ctx, LEAP_ERR_INVALID_ARGUMENT,
                "asynchronous ingestion needs device memory, page-locked host memory, or a device that reads "
                "pageable host memory");
  Integration& in = ctx->integ[slot];
  finish_upload(in);
  const size_t esz = vis_type == LEAP_VIS_C64 ? sizeof(float2) : sizeof(double2);
  LEAP_CUDA(in.vis.ensure(esz * static_cast<size_t>(rows) * channels * pols), "alloc vis");
  LEAP_CUDA(in.uvw.ensure(sizeof(double) * 3 * rows), "alloc uvw");
  LEAP_CUDA(in.uvw_f.ensure(sizeof(float) * 6 * rows), "alloc split uvw");
  if (!in.ready) LEAP_CUDA(cudaEventCreateWithFlags(&in.ready, cudaEventDisableTiming), "create event");
  cudaStream_t c = ctx->copy;
  // After every earlier call on the context's stream (which may still read this slot).
  LEAP_CUDA(cudaEventRecord(ctx->copy_fence, ctx->stream), "fence");
  LEAP_CUDA(cudaStreamWaitEvent(c, ctx->copy_fence, 0), "fence");
  LEAP_CUDA(cudaMemcpyAsync(in.uvw.ptr, uvw, sizeof(double) * 3 * rows,
                            memory == LEAP_MEMORY_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, c),
            "copy uvw");
  int rc = ingest(ctx, vis_type, direct, row_channels, start_channel, rows, channels, pols, in.vis.ptr, rows, 0, c,
                  ctx->sms);
  if (rc != LEAP_OK) return rc;
  split_uvw<<<grid_1d(3 * rows, 256), 256, 0, c>>>(in.uvw.as<double>(), rows, in.uvw_f.as<float>());
  LEAP_CUDA(cudaGetLastError(), "ingestion launch");
  LEAP_CUDA(cudaEventRecord(in.ready, c), "upload event");
  in.pending = true;
  in.vis_type = vis_type;
  in.rows = rows;
  in.channels = channels;
  in.pols = pols;
  in.has_map = false;
  in.op_nbl = 0;
  if (vis_type == LEAP_VIS_C64 && pols == 4 && rows * 8 < (int64_t(1) << 31)) {
    auto enc = tensor_map_encoder();
    if (!enc) return fail(ctx, LEAP_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {static_cast<cuuint64_t>(rows) * 8, static_cast<cuuint64_t>(channels)};
    cuuint64_t strides[1] = {static_cast<cuuint64_t>(rows) * 32};
    cuuint32_t estr[2] = {1, 1};
    for (int which = 0; which < 2; ++which) {
      cuuint32_t box[2] = {256, static_cast<cuuint32_t>(which == 0 ? PipeShape<1>::CH : PipeShape<4>::CH)};
      CUresult r = enc(which == 0 ? &in.map16 : &in.map8, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, in.vis.ptr, dims, strides,
                       box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS) return fail(ctx, LEAP_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string(r));
    }
    in.has_map = true;
  }
  return LEAP_OK;
}

int32_t leap_apply_flags(leap_ctx* ctx, int32_t slot, const uint8_t* flags, int64_t row_channels, int32_t start_channel,
                         int32_t flag_pols, int32_t memory, int64_t* flagged_groups) {
  if (!ctx || !flags) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  auto it = ctx->integ.find(slot);
  if (it == ctx->integ.end()) return fail(ctx, LEAP_ERR_NOT_READY, "integration slot not set");
  Integration& in = it->second;
  finish_upload(in);
  if (flag_pols < 1 || start_channel < 0 || static_cast<int64_t>(start_channel) + in.channels > row_channels)
    return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "flag array shape does not cover the integration");
  if (memory != LEAP_MEMORY_HOST && memory != LEAP_MEMORY_DEVICE) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "unknown memory kind");
  DeviceGuard g(ctx->device);
  cudaStream_t s = ctx->stream;
  const size_t fbytes = static_cast<size_t>(in.rows) * row_channels * flag_pols;
  const uint8_t* dflags = flags;
  DeviceBuffer tmp;
  if (memory == LEAP_MEMORY_HOST) {
    LEAP_CUDA(tmp.ensure(fbytes), "alloc flags");
    LEAP_CUDA(cudaMemcpyAsync(tmp.ptr, flags, fbytes, cudaMemcpyHostToDevice, s), "upload flags");
    dflags = tmp.as<uint8_t>();
  }
  LEAP_CUDA(ctx->flag_count.ensure(sizeof(unsigned long long)), "alloc flag count");
  LEAP_CUDA(cudaMemsetAsync(ctx->flag_count.ptr, 0, sizeof(unsigned long long), s), "clear flag count");
  in.op_nbl = 0;  // the visibilities change: rebuild the split grid operand on its next use
  const int grid = grid_1d(in.rows * in.channels, 256);
  if (in.vis_type == LEAP_VIS_C64)
    apply_flag_groups<float2><<<grid, 256, 0, s>>>(in.vis.as<float2>(), dflags, in.rows, in.channels, in.pols, row_channels,
                                                   start_channel, flag_pols, ctx->flag_count.as<unsigned long long>());
  else
    apply_flag_groups<double2><<<grid, 256, 0, s>>>(in.vis.as<double2>(), dflags, in.rows, in.channels, in.pols,
                                                    row_channels, start_channel, flag_pols,
                                                    ctx->flag_count.as<unsigned long long>());
  LEAP_CUDA(cudaGetLastError(), "flag kernel");
  unsigned long long n = 0;
  LEAP_CUDA(cudaMemcpyAsync(&n, ctx->flag_count.ptr, sizeof(n), cudaMemcpyDeviceToHost, s), "read flag count");
  LEAP_CUDA(cudaStreamSynchronize(s), "apply flags");
  tmp.release();
  if (flagged_groups) *flagged_groups = static_cast<int64_t>(n);
  return LEAP_OK;
}

int32_t leap_release_integration(leap_ctx* ctx, int32_t slot) {
  if (!ctx) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL context");
  auto it = ctx->integ.find(slot);
  if (it == ctx->integ.end()) return fail(ctx, LEAP_ERR_NOT_READY, "integration slot not set");
  DeviceGuard g(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  finish_upload(it->second);
  if (it->second.ready) cudaEventDestroy(it->second.ready);
  it->second.vis.release();
  it->second.uvw.release();
  it->second.uvw_f.release();
  it->second.op.release();
  ctx->integ.erase(it);
  return LEAP_OK;
}

int32_t leap_calibrate(leap_ctx* ctx, int32_t slot, const double* dd, int32_t ndir, int32_t precision, double* cal_out) {
  if (!ctx || !dd || !cal_out) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (ndir <= 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "ndirections must be positive");
  if (!ctx->md.set) return fail(ctx, LEAP_ERR_NOT_READY, "metadata not set");
  DeviceGuard g(ctx->device);
  const int S = ctx->md.S;
  LEAP_CUDA(ctx->dd.ensure(sizeof(double) * 9 * ndir), "alloc dd");
  LEAP_CUDA(ctx->cal.ensure(sizeof(double) * S * ndir), "alloc cal");
  LEAP_CUDA(cudaMemcpyAsync(ctx->dd.ptr, dd, sizeof(double) * 9 * ndir, cudaMemcpyHostToDevice, ctx->stream), "upload dd");
  int rc = calibrate_impl(ctx, slot, ctx->dd.as<double>(), ndir, precision, ctx->cal.as<double>(), ctx->stream);
  if (rc != LEAP_OK) return rc;
  LEAP_CUDA(cudaMemcpyAsync(cal_out, ctx->cal.ptr, sizeof(double) * S * ndir, cudaMemcpyDeviceToHost, ctx->stream), "download cal");
  LEAP_CUDA(cudaStreamSynchronize(ctx->stream), "calibrate");
  return check_device_error(ctx);
}

int32_t leap_calibrate_async(leap_ctx* ctx, int32_t slot, const double* d_dd, int32_t ndir, int32_t precision,
                             double* d_cal_out, void* stream) {
  if (!ctx || !d_dd || !d_cal_out) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard g(ctx->device);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  return calibrate_impl(ctx, slot, d_dd, ndir, precision, d_cal_out, s);
}

int32_t leap_calibrate_batched(leap_ctx* ctx, const leap_work_item* items, int32_t nitems, const double* dd,
                               int32_t ndirections, int32_t precision, double* cal_out) {
  if (!ctx || !items || !dd || !cal_out) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (ndirections <= 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "ndirections must be positive");
  if (!ctx->md.set) return fail(ctx, LEAP_ERR_NOT_READY, "metadata not set");
  DeviceGuard g(ctx->device);
  const int S = ctx->md.S;
  LEAP_CUDA(ctx->dd.ensure(sizeof(double) * 9 * ndirections), "alloc dd");
  LEAP_CUDA(ctx->cal.ensure(sizeof(double) * S * ndirections), "alloc cal");
  LEAP_CUDA(cudaMemcpyAsync(ctx->dd.ptr, dd, sizeof(double) * 9 * ndirections, cudaMemcpyHostToDevice, ctx->stream),
            "upload dd");
  int rc = calibrate_batched_impl(ctx, items, nitems, ndirections, precision);
  if (rc != LEAP_OK) return rc;
  LEAP_CUDA(cudaMemcpyAsync(cal_out, ctx->cal.ptr, sizeof(double) * S * ndirections, cudaMemcpyDeviceToHost, ctx->stream),
            "download cal");
  LEAP_CUDA(cudaStreamSynchronize(ctx->stream), "calibrate batched");
  return check_device_error(ctx);
}

int32_t leap_get_avgdata_device(leap_ctx* ctx, int32_t pol, double* d_out, void* stream) {
  if (!ctx || !d_out) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (ctx->last_ndir <= 0) return fail(ctx, LEAP_ERR_NOT_READY, "no calibrate call yet");
  if (pol < 0 || pol >= ctx->last_pols) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "pol out of range");
  DeviceGuard g(ctx->device);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  const size_t nbl = static_cast<size_t>(ctx->last_nbl);
  // avg is [ndir][pols][nbl]: one strided 2-D copy gathers pol `pol` of every direction.
  LEAP_CUDA(cudaMemcpy2DAsync(d_out, sizeof(double2) * nbl, ctx->avg.as<double2>() + pol * nbl,
                              sizeof(double2) * nbl * ctx->last_pols, sizeof(double2) * nbl, ctx->last_ndir,
                              cudaMemcpyDeviceToDevice, s),
            "copy avgData");
  return LEAP_OK;
}

int32_t leap_backward(leap_ctx* ctx, int32_t slot, const double* d_dd, int32_t ndir, const double* d_avg0,
                      const double* d_grad_cal, const void* d_vis, double* d_grad_lmn, void* d_grad_vis,
                      void* stream) {
  if (!ctx || !d_dd || !d_avg0 || !d_grad_cal || !d_grad_lmn) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (ndir <= 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "ndirections must be positive");
  if (!ctx->md.set) return fail(ctx, LEAP_ERR_NOT_READY, "metadata not set");
  auto it = ctx->integ.find(slot);
  if (it == ctx->integ.end()) return fail(ctx, LEAP_ERR_NOT_READY, "integration slot not set");
  DeviceGuard g(ctx->device);
  Metadata& md = ctx->md;
  const Integration& in = it->second;
  const int nbl = static_cast<int>(md.k.nbaselines);
  const int S = md.S, D = ndir, nI = md.Arows - 1, nI1 = md.A1rows - 1;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  if (in.pending) cudaStreamWaitEvent(s, in.ready, 0);
  LEAP_CUDA(ctx->adj_dphi.ensure(sizeof(double) * std::max(nI, 1) * D), "alloc adjoint scratch");
  LEAP_CUDA(ctx->adj_cal1.ensure(sizeof(double) * S * D), "alloc adjoint scratch");
  LEAP_CUDA(ctx->adj_phi1.ensure(sizeof(double) * std::max(nI1, 1) * D), "alloc adjoint scratch");
  LEAP_CUDA(ctx->adj_gavg.ensure(sizeof(double2) * static_cast<size_t>(nbl) * D), "alloc adjoint scratch");
  // Solve adjoint: g_dphi, g_cal1, g_phi1, g_avg.
  if (nI > 0)
    adjoint_contract_t<<<(nI * 32 + 255) / 256, 256, 0, s>>>(md.Ad.as<double>(), S, nI, d_grad_cal, D,
                                                             ctx->adj_dphi.as<double>(), nI);
  else
    LEAP_CUDA(cudaMemsetAsync(ctx->adj_dphi.ptr, 0, sizeof(double) * D, s), "clear");
  adjoint_cal1<<<(S * D + 255) / 256, 256, 0, s>>>(d_grad_cal, ctx->adj_dphi.as<double>(), std::max(nI, 1),
                                                   md.at_ptr.as<int32_t>(), md.at_idx.as<int32_t>(),
                                                   md.at_val.as<double>(), S, D, ctx->adj_cal1.as<double>());
  if (nI1 > 0)
    adjoint_contract_t<<<(nI1 * 32 + 255) / 256, 256, 0, s>>>(md.Ad1.as<double>(), S, nI1, ctx->adj_cal1.as<double>(),
                                                              D, ctx->adj_phi1.as<double>(), nI1);
  const double2* avg0 = reinterpret_cast<const double2*>(d_avg0);
  adjoint_avg_dint<<<grid_1d(static_cast<int64_t>(nbl) * D, 256), 256, 0, s>>>(
      avg0, ctx->adj_dphi.as<double>(), std::max(nI, 1), nI, nbl, D, ctx->adj_gavg.as<double2>());
  if (nI1 > 0)
    adjoint_avg_phi1<<<(D + 127) / 128, 128, 0, s>>>(avg0, ctx->adj_phi1.as<double>(), md.I1.as<int32_t>(), nI1, nbl,
                                                     D, ctx->adj_gavg.as<double2>());
  // Rotate + average adjoint over the integration, recomputing the rotated samples.
  AdjointArgs aa{};
  aa.vis = d_vis ? d_vis : in.vis.ptr;
  aa.vis_c64 = in.vis_type == LEAP_VIS_C64;
  aa.check_nan = d_vis != nullptr;
  aa.uvw = in.uvw.as<double>();
  aa.dd = d_dd;
  aa.gavg = ctx->adj_gavg.as<double2>();
  aa.rows = in.rows;
  aa.C = in.channels;
  aa.P = in.pols;
  aa.nbl = nbl;
  aa.D = D;
  aa.f0 = md.k.freq_start_hz;
  aa.df = md.k.freq_inc_hz;
  constexpr int kDPB = 4;
  const int64_t items = in.rows * ((in.channels + kAdjChannels - 1) / kAdjChannels);
  const int dgroups = (D + kDPB - 1) / kDPB;
  const int64_t want = (items + 255) / 256;
  const int bx = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(want, std::max(1, ctx->sms * 8 / dgroups))));
  LEAP_CUDA(ctx->adj_partial.ensure(sizeof(double) * 3 * static_cast<size_t>(bx) * D), "alloc adjoint partials");
  aa.partial = ctx->adj_partial.as<double>();
  adjoint_lmn<kDPB><<<dim3(bx, dgroups), 256, 0, s>>>(aa);
  adjoint_lmn_reduce<<<(3 * D + 127) / 128, 128, 0, s>>>(aa.partial, bx, D, d_grad_lmn);
  if (d_grad_vis) {
    const size_t esz = aa.vis_c64 ? sizeof(float2) : sizeof(double2);
    LEAP_CUDA(cudaMemsetAsync(d_grad_vis, 0, esz * static_cast<size_t>(in.rows) * in.channels * in.pols, s),
              "clear vis gradient");
    aa.gvis = d_grad_vis;
    adjoint_vis<<<grid_1d(items, 256), 256, 0, s>>>(aa);
  }
  LEAP_CUDA(cudaGetLastError(), "adjoint launch");
  return LEAP_OK;
}

int32_t leap_selftest_bounded_wait(leap_ctx* ctx, int32_t polls) {
  if (!ctx) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL context");
  if (polls < 1 || polls > (1 << 20)) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "polls must be in [1, 2^20]");
  DeviceGuard g(ctx->device);
  selftest_bounded_wait<<<1, 32, 0, ctx->stream>>>(static_cast<uint32_t>(polls), ctx->dev_err.as<int>());
  LEAP_CUDA(cudaGetLastError(), "self-test launch");
  LEAP_CUDA(cudaStreamSynchronize(ctx->stream), "self-test");
  return check_device_error(ctx);
}

int32_t leap_set_option(leap_ctx* ctx, int32_t option, int32_t value) {
  if (!ctx) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL context");
  switch (option) {
    case LEAP_OPTION_AUTOTUNE: ctx->autotune = value != 0; return LEAP_OK;
    case LEAP_OPTION_TENSOR_CORE_CONTRACTION: ctx->tc_gemm = value != 0; return LEAP_OK;
    case LEAP_OPTION_TENSOR_CORE_ROTATION:
      if (value < 0 || value > 2) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "rotation option must be 0, 1 or 2");
      ctx->mma_rotate = value;
      return LEAP_OK;
    case LEAP_OPTION_GRIDDED_ROTATION:
      if (value < 0 || value > 2) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "gridded option must be 0, 1 or 2");
      ctx->gridded = value;
      return LEAP_OK;
    case LEAP_OPTION_GRAPH_REPLAY: ctx->graph_replay = value != 0; return LEAP_OK;
    case LEAP_OPTION_GRID_SHARED_GROUPS: ctx->grid_shared_groups = value != 0; return LEAP_OK;
    default: return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "unknown option");
  }
}

int32_t leap_set_autotune(leap_ctx* ctx, int32_t enable) {
  if (!ctx) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL context");
  ctx->autotune = enable != 0;
  return LEAP_OK;
}

int32_t leap_get_avgdata(leap_ctx* ctx, int32_t direction, double* out) {
  if (!ctx || !out) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  if (direction < 0 || direction >= ctx->last_ndir) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "direction out of range");
  DeviceGuard g(ctx->device);
  const size_t n = static_cast<size_t>(ctx->last_pols) * ctx->last_nbl;
  LEAP_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
  LEAP_CUDA(cudaMemcpy(out, ctx->avg.as<double2>() + n * direction, sizeof(double2) * n, cudaMemcpyDeviceToHost), "download avgData");
  return LEAP_OK;
}

int32_t leap_rotate_uvw(leap_ctx* ctx, int32_t slot, const double* dd, int32_t ndir, double* out) {
  if (!ctx || !dd || !out) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  auto it = ctx->integ.find(slot);
  if (it == ctx->integ.end()) return fail(ctx, LEAP_ERR_NOT_READY, "integration slot not set");
  if (ndir <= 0) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "ndirections must be positive");
  DeviceGuard g(ctx->device);
  finish_upload(it->second);
  const int64_t rows = it->second.rows;
  DeviceBuffer d_dd, d_out;
  LEAP_CUDA(d_dd.ensure(sizeof(double) * 9 * ndir), "alloc dd");
  LEAP_CUDA(d_out.ensure(sizeof(double) * 3 * rows * ndir), "alloc rotated uvw");
  LEAP_CUDA(cudaMemcpyAsync(d_dd.ptr, dd, sizeof(double) * 9 * ndir, cudaMemcpyHostToDevice, ctx->stream), "upload dd");
  rotate_uvw<<<grid_1d(rows * ndir, 256), 256, 0, ctx->stream>>>(d_dd.as<double>(), it->second.uvw.as<double>(), rows, ndir,
                                                                d_out.as<double>());
  LEAP_CUDA(cudaGetLastError(), "rotate_uvw launch");
  LEAP_CUDA(cudaMemcpyAsync(out, d_out.ptr, sizeof(double) * 3 * rows * ndir, cudaMemcpyDeviceToHost, ctx->stream), "download");
  LEAP_CUDA(cudaStreamSynchronize(ctx->stream), "rotate_uvw");
  d_dd.release();
  d_out.release();
  return LEAP_OK;
}

int32_t leap_get_timings(leap_ctx* ctx, leap_timings* out) {
  if (!ctx || !out) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  DeviceGuard g(ctx->device);
  return fill_timings(ctx, out);
}

int32_t leap_timing_reset(leap_ctx* ctx) {
  if (!ctx) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL context");
  ctx->ring_count = 0;
  return LEAP_OK;
}

int32_t leap_synchronize(leap_ctx* ctx) {
  if (!ctx) return fail(ctx, LEAP_ERR_INVALID_ARGUMENT, "NULL context");
  DeviceGuard g(ctx->device);
  LEAP_CUDA(cudaStreamSynchronize(ctx->stream), "synchronize");
  LEAP_CUDA(cudaDeviceSynchronize(), "synchronize device");
  return check_device_error(ctx);
}

void leap_dd_matrix(double phase_ra, double phase_dec, double ra, double dec, double* dd_out) {
  if (dd_out) dd_matrix(phase_ra, phase_dec, ra, dec, dd_out);
}

int32_t leap_phase_matrix(const int32_t* a1, const int32_t* a2, const uint8_t* fg, int32_t n, int32_t ref_ant,
                          double* A_out, int32_t* I_out, int32_t* rows_out, int32_t* cols_out) {
  if (n > 0 && (!a1 || !a2 || !fg || !A_out || !I_out || !rows_out || !cols_out))
    return fail(nullptr, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  std::vector<double> A;
  std::vector<int32_t> I;
  int32_t rows = 0, cols = 0;
  std::string err;
  int rc = phase_matrix(a1, a2, fg, n, ref_ant, A, I, rows, cols, err);
  if (rc != LEAP_OK) return fail(nullptr, rc, err);
  std::memcpy(A_out, A.data(), sizeof(double) * A.size());
  if (!I.empty()) std::memcpy(I_out, I.data(), sizeof(int32_t) * I.size());
  *rows_out = rows;
  *cols_out = cols;
  return LEAP_OK;
}

int32_t leap_pseudo_inverse(const double* A, int32_t rows, int32_t cols, double* Ad_out) {
  if (!A || !Ad_out) return fail(nullptr, LEAP_ERR_INVALID_ARGUMENT, "NULL argument");
  std::string err;
  int rc = pseudo_inverse(A, rows, cols, Ad_out, err);
  if (rc != LEAP_OK) return fail(nullptr, rc, err);
  return LEAP_OK;
}

}  // extern "C"
