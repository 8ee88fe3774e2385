// C ABI: integration slots -- uploads in the Integration layout or in MeasurementSet order
// (transposed on the device, synchronously or on the copy stream), opt-in flags, release.
#include "leap_internal.h"
#include "kernels_ingest.cuh"

namespace leapabi {

// Before a slot is rewritten or freed: its asynchronous upload must be over.
void finish_upload(Integration& in) {
  if (in.pending) {
    cudaEventSynchronize(in.ready);
    in.pending = false;
  }
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

}  // namespace leapabi

extern "C" {

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
  LEAP_CUDA(cudaMemcpyAsync(in.uvw.ptr, uvw, sizeof(double) * 3 * rows, kind, ctx->stream), "copy uvw");
  // A source the kernels can read (device memory, page-locked host memory, or pageable host
  // memory read in place through the host page tables) is copied and cleaned in one pass by
  // 16-byte vectors.  Measured on a Grace host, uploading 52.5 GB from page-locked memory: 201
  // GB/s, against 182 GB/s for a copy-engine transfer followed by the NaN pass in place, which
  // is what other sources still take.
  const void* direct = memory == LEAP_MEMORY_DEVICE ? vis : nullptr;
  if (!direct) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, vis) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
      direct = at.devicePointer;
    else
      cudaGetLastError();  // pageable memory: not an error
    if (!direct && ctx->pageable_direct) direct = vis;
  }
  const size_t group_bytes = esz * static_cast<size_t>(pols);
  if (direct && reinterpret_cast<uintptr_t>(direct) % 16 == 0 && group_bytes % 16 == 0) {
    const int64_t n16 = static_cast<int64_t>(vbytes / 16);
    const int V = static_cast<int>(group_bytes / 16);
    const int grid = static_cast<int>(std::min<int64_t>((n16 + 255) / 256, static_cast<int64_t>(ctx->sms) * 8));
    const uint4* sp = static_cast<const uint4*>(direct);
    uint4* dp = in.vis.as<uint4>();
    if (vis_type == LEAP_VIS_C64) {
      if (V == 1) copy_sanitize_groups<float, 1><<<grid, 256, 0, ctx->stream>>>(sp, dp, n16);
      else copy_sanitize_groups<float, 2><<<grid, 256, 0, ctx->stream>>>(sp, dp, n16);
    } else {
      if (V == 1) copy_sanitize_groups<double, 1><<<grid, 256, 0, ctx->stream>>>(sp, dp, n16);
      else if (V == 2) copy_sanitize_groups<double, 2><<<grid, 256, 0, ctx->stream>>>(sp, dp, n16);
      else copy_sanitize_groups<double, 4><<<grid, 256, 0, ctx->stream>>>(sp, dp, n16);
    }
    return finish_integration(ctx, in, vis_type, rows, channels, pols);
  }
  LEAP_CUDA(cudaMemcpyAsync(in.vis.ptr, vis, vbytes, kind, ctx->stream), "copy vis");
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

}  // extern "C"
