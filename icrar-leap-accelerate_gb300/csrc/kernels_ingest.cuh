// MeasurementSet ingestion on the device: the MS DATA column is row-major
// [row][channel][pol] (LA/ms/utils.h:81-146, where the reference transposes and
// widens it on the host); the Integration layout is [channel][row][pol]
// (column-major (pol, row, channel), LA/model/cpu/Integration.h:73).  One
// kernel does the transpose through a shared-memory tile and applies the NaN
// rule on the way (a (row, channel) group with a NaN in any pol is zeroed, so
// it adds nothing to the averages, as CpuLeapCalibrator.cc:201-214 skips it).
//
// The source may be device memory or page-locked host memory (read directly
// over the host link, no staging copy).  Tile: 32 rows x TC channels of
// (pol group) elements; reads are contiguous along channels, writes along rows.
#pragma once

#include "leap_common.cuh"

namespace leapgb {

// Integration-layout upload in one pass from a source the device can read (device memory,
// page-locked host memory, or pageable host memory on hosts whose GPU uses the host page
// tables): 16-byte vectors, one per lane, so that every load and store instruction of a warp
// covers 512 contiguous bytes; the V lanes that hold one (row, channel) group of pols agree
// on its NaN flag by shuffles and zero it together (the NaN rule of the transpose above).
// n16: 16-byte vectors in all, a multiple of V (V = 1, 2 or 4 vectors per group).
template <typename S, int V>
__global__ void __launch_bounds__(256) copy_sanitize_groups(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                                            int64_t n16) {
  static_assert(V == 1 || V == 2 || V == 4, "a group is 16, 32 or 64 bytes");
  const int lane = threadIdx.x & 31;
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  for (int64_t w = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; w * 32 < n16; w += warps) {
    const int64_t i = w * 32 + lane;
    const bool act = i < n16;  // the same for all V lanes of a group (n16 is a multiple of V)
    uint4 v = act ? src[i] : make_uint4(0u, 0u, 0u, 0u);
    bool nan;
    if (sizeof(S) == 4)
      nan = isnan(__uint_as_float(v.x)) || isnan(__uint_as_float(v.y)) || isnan(__uint_as_float(v.z)) ||
            isnan(__uint_as_float(v.w));
    else
      nan = isnan(__hiloint2double(static_cast<int>(v.y), static_cast<int>(v.x))) ||
            isnan(__hiloint2double(static_cast<int>(v.w), static_cast<int>(v.z)));
#pragma unroll
    for (int o = 1; o < V; o <<= 1) nan |= __shfl_xor_sync(0xffffffffu, nan, o) != 0;
    if (nan) v = make_uint4(0u, 0u, 0u, 0u);
    if (act) dst[i] = v;
  }
}

template <typename VisT, int P>
struct IngestGroup {
  VisT v[P];
};

template <typename VisT> struct IngestTile;
template <> struct IngestTile<float2> { static constexpr int TC = 32; };
template <> struct IngestTile<double2> { static constexpr int TC = 16; };

// src: element (r, c, p) of the selected block at src[(r * row_channels + start_channel + c) * P + p],
// r in [0, nrows); dst: the integration [channels][rows_total][P], rows [row0, row0 + nrows).
template <typename VisT, int P>
__global__ void __launch_bounds__(256) ingest_ms_transpose(const VisT* __restrict__ src, int64_t row_channels,
                                                           int start_channel, int64_t nrows, int channels,
                                                           VisT* __restrict__ dst, int64_t rows_total, int64_t row0) {
  constexpr int TR = 32, TC = IngestTile<VisT>::TC;
  using G = IngestGroup<VisT, P>;
  __shared__ G tile[TC][TR + 1];
  const int64_t r_tiles = (nrows + TR - 1) / TR;
  const int c_tiles = (channels + TC - 1) / TC;
  for (int64_t t = blockIdx.x; t < r_tiles * c_tiles; t += gridDim.x) {
    const int64_t rt = t % r_tiles;
    const int ct = static_cast<int>(t / r_tiles);
    const int64_t rbase = rt * TR;
    const int cbase = ct * TC;
    // load: threads run along channels (contiguous in the MS row)
    for (int i = threadIdx.x; i < TR * TC; i += blockDim.x) {
      const int lc = i % TC, lr = i / TC;
      const int64_t r = rbase + lr;
      const int c = cbase + lc;
      G g;
      if (r < nrows && c < channels) {
        const VisT* s = src + (r * row_channels + start_channel + c) * P;
        bool nan = false;
#pragma unroll
        for (int p = 0; p < P; ++p) {
          g.v[p] = s[p];
          nan |= isnan(g.v[p].x) || isnan(g.v[p].y);
        }
        if (nan) {
#pragma unroll
          for (int p = 0; p < P; ++p) g.v[p].x = g.v[p].y = 0;
        }
        tile[lc][lr] = g;
      }
    }
    __syncthreads();
    // store: threads run along rows (contiguous in the integration)
    for (int i = threadIdx.x; i < TR * TC; i += blockDim.x) {
      const int lr = i % TR, lc = i / TR;
      const int64_t r = rbase + lr;
      const int c = cbase + lc;
      if (r < nrows && c < channels) {
        VisT* d = dst + (static_cast<int64_t>(c) * rows_total + row0 + r) * P;
        const G g = tile[lc][lr];
#pragma unroll
        for (int p = 0; p < P; ++p) d[p] = g.v[p];
      }
    }
    __syncthreads();
  }
}

// Opt-in flagging: zero every (row, channel) group whose MeasurementSet FLAG is set
// for any pol.  flags is MS order, [rows][row_channels][flag_pols] bytes (non-zero =
// flagged); threads run along channels so the flag reads are contiguous, and only
// flagged groups are written.  The reference averages flagged samples (it skips only
// NaN, CpuLeapCalibrator.cc:201-214), so this is off unless a caller asks for it.
template <typename VisT>
__global__ void apply_flag_groups(VisT* __restrict__ vis, const uint8_t* __restrict__ flags, int64_t rows, int channels,
                                  int pols, int64_t row_channels, int start_channel, int flag_pols,
                                  unsigned long long* __restrict__ count) {
  unsigned long long mine = 0;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < rows * channels;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = static_cast<int>(i % channels);
    const int64_t r = i / channels;
    const uint8_t* f = flags + (r * row_channels + start_channel + c) * flag_pols;
    bool flagged = false;
    for (int p = 0; p < flag_pols; ++p) flagged |= f[p] != 0;
    if (flagged) {
      VisT* v = vis + (static_cast<int64_t>(c) * rows + r) * pols;
      for (int p = 0; p < pols; ++p) v[p].x = v[p].y = 0;
      ++mine;
    }
  }
  if (mine) atomicAdd(count, mine);
}

}  // namespace leapgb
