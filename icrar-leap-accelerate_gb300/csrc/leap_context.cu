// C ABI: context lifetime, options, timings, error text, the self-test and the host
// set-up maths (include/leap_gb300.h).
#include "leap_internal.h"

namespace leapabi {

thread_local std::string g_last_error;

// Bumped whenever any device buffer is (re)allocated: captured CUDA graphs
// hold raw pointers, so a graph recorded before the bump is stale.
uint64_t g_alloc_epoch = 0;

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

}  // namespace leapabi

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
      kv.second.op.release();
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
