// C ABI: leap_backward, the FP64 adjoint of one calibrate call (differentiable form).
#include "leap_internal.h"
#include "kernels_solve.cuh"
#include "kernels_adjoint.cuh"

extern "C" {

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

}  // extern "C"
