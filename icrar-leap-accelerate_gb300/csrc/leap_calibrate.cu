// C ABI: the calibration itself -- rotate + average (pipelined, gridded, tensor-core, FP64
// kernels), the compensated reference-antenna pass, the solve and the contraction, the
// batched call with its autotuner and graph replay, and the avgData / UVW getters.
#include "leap_internal.h"
#include "kernels_solve.cuh"
#include "kernels_mma.cuh"

namespace leapabi {

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

// Grid matrix of the gridded kernel for C channels (built once per channel count) and the
// inverse of its scale.
const unsigned char* grid_table_for(leap_ctx* ctx, int C, float& einv) {
  auto it = ctx->grid_tabs.find(C);
  if (it != ctx->grid_tabs.end()) {
    einv = ctx->grid_einv.at(C);
    return it->second.as<unsigned char>();
  }
  if (ctx->capturing) return nullptr;
  std::vector<uint16_t> tab;
  einv = grid_table(C, kGrTaps, kGrBeta, grid_lbase(C), grid_rows(C), tab);
  DeviceBuffer& b = ctx->grid_tabs[C];
  if (b.ensure(sizeof(uint16_t) * tab.size()) != cudaSuccess) return nullptr;
  if (cudaMemcpy(b.ptr, tab.data(), sizeof(uint16_t) * tab.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return nullptr;
  ctx->grid_einv[C] = einv;
  return b.as<unsigned char>();
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
    const int64_t op_bytes = grid_operand_bytes(nbl, T, C);
    if (in.op_nbl != nbl) {
      // The split grid operand and its scales: built once per upload (the visibilities read
      // twice, hi and lo written), then read by every gridded call on this integration.
      if (ctx->capturing) return fail(ctx, LEAP_ERR_INTERNAL, "grid operand missing while recording a graph");
      LEAP_CUDA(in.op.ensure(static_cast<size_t>(op_bytes + grid_scale_bytes(nbl, T))), "alloc grid operand");
      const dim3 og((nbl + 3) / 4, (T + 3) / 4);
      grid_split_operand<<<og, 128, 0, s>>>(in.vis.as<float>(), in.rows, nbl, T, C, (T + 3) / 4,
                                            in.op.as<unsigned char>(),
                                            reinterpret_cast<float*>(in.op.as<unsigned char>() + op_bytes));
      LEAP_CUDA(cudaGetLastError(), "grid operand launch");
      ++kernels;
      in.op_nbl = nbl;
    }
    float einv = 1.f;
    const unsigned char* tab = grid_table_for(ctx, C, einv);
    if (!tab) return fail(ctx, LEAP_ERR_CUDA, "grid matrix unavailable for this channel count");
    GridItem& it = git[i];
    it.op = in.op.as<unsigned char>();
    it.vinv = reinterpret_cast<const float*>(in.op.as<unsigned char>() + op_bytes);
    it.einv = einv;
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
  es_kernel_poly(kGrTaps, kGrBeta, kGrPolyDeg, &gp.wpoly[0][0]);
  grid_windows<<<static_cast<unsigned>(units), kGrWinThreads, 0, s>>>(gp);
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

// Sum of the reference-antenna pass's slab partials into ctx->avg_i1, on stream st (fixed order).
int refant_reduce(leap_ctx* ctx, cudaStream_t st, int& kernels) {
  const std::vector<ReduceItem>& red = ctx->refant_reduce_host;
  if (red.empty()) return LEAP_OK;
  const int nI1 = ctx->md.A1rows - 1;
  int64_t maxn = 0;
  for (const auto& r : red) maxn = std::max<int64_t>(maxn, static_cast<int64_t>(r.ndir) * nI1);
  const dim3 rg(static_cast<unsigned>(std::min<int64_t>((maxn + 255) / 256, 1024)), static_cast<unsigned>(red.size()));
  reduce_item_slabs<<<rg, 256, 0, st>>>(ctx->refant_reduce.as<ReduceItem>(), static_cast<int>(red.size()), nI1,
                                         ctx->avg_i1.as<double2>());
  ++kernels;
  return LEAP_OK;
}

// Mixed form: compensated sums of pol 0 of the reference-antenna baselines into
// ctx->avg_i1 ([D][nI1]), on the aux stream.  complex<float> items go through one
// item-table launch; complex<double> items keep the FP64 kernel.
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
  // 10 blocks per SM in total, two waves of the 5 resident blocks), so that chunks
  // of 1 x 48 and 64 x 384 samples give blocks of similar length instead of the same
  // number of blocks each; fewer, longer slabs also keep the partial sums (and their
  // reduction) small.
  int64_t work_total = 0;
  for (const auto& w : items) {
    const Integration& in = ctx->integ.at(w.slot);
    work_total += (in.rows / nbl) * in.channels * rtiles * ((w.ndir + 7) / 8);
  }
  const int64_t slab_budget = std::max<int64_t>(64, (work_total + 10 * ctx->sms - 1) / (10 * ctx->sms));
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
  RefantParams rp{};
  rp.items = ctx->refant_items.as<RefantItem>();
  rp.I1 = md.I1.as<int32_t>();
  rp.f0 = md.k.freq_start_hz;
  rp.df = md.k.freq_inc_hz;
  rp.nitems = static_cast<int32_t>(rit.size());
  rp.nbl = nbl;
  rp.nI1 = nI1;
  rp.ntasks = blocks * 4;
  refant_average_df_items<2><<<blocks, 128, 0, a>>>(rp, ctx->twiddle_df.as<float4>());
  ++kernels;
  return refant_reduce(ctx, a, kernels);
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
  // memory; running it on extra warps of the gridded kernel measured slower than two launches).
  // Beside the gridded kernel it goes first, so that it overlaps the small kernels that set up
  // the grid windows; beside the pipelined kernel it goes after it, so that the persistent
  // blocks, whose unit schedule assumes they start together, take the SMs first.
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

}  // namespace leapabi

extern "C" {

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

}  // extern "C"
