// Mixed-precision rotate + average, pipelined (4 pols, complex<float>): the hot kernel.
//
// Work comes from a table of items; an item is one resident integration and a
// contiguous range of directions (the single-integration call is one item; a
// batched call has one item per integration chunk).  An item is cut into units
// = (group of TPB 32-baseline tiles, group of (NC/TPB)*DPW directions,
// timestep slab); units of all items are numbered consecutively, so uneven
// chunks share one launch.  The host assigns units to the persistent blocks
// longest first, each to the least-loaded block, and passes the result as an
// order table (block b visits order[b], order[b + grid], ... up to a -1), so
// blocks finish together even when unit sizes differ by 100x.
//
// A unit is a sequence of chunks = (timestep, CH channels).  The visibility
// tensor of an item is viewed as a 2-D array [channel][row*8 floats]; a chunk
// is one TMA box of 256 floats (32 baselines x 4 pols x complex) by CH
// channels per tile, loaded with cp.async.bulk.tensor from the item's tensor
// map into a shared-memory stage, completing on the stage's "full" mbarrier.
// Boxes past the last row or channel are zero-filled by the TMA unit; rows of
// a partial tile that belong to the next timestep are loaded but not used.
// Every warp releases a stage through its "empty" mbarrier; lane 0 of warp 0
// then refills it with the chunk one ring length ahead.  (A separate producer
// warp would make 9 warps, 3 on one SM sub-partition, and cap registers at
// 168.)  All waits are bounded and report a device error instead of hanging.
//
// Per (row, direction) the phase turns(c) = A + c*B is formed once per
// timestep in double-float arithmetic (~1e-12 turns) as 32-bit fixed-point
// fractions of a turn: no FP64 instructions in this kernel (GB300 runs them
// at ~1/70 of the FP32 rate).  The twiddle is table-accurate (twiddle_turns)
// every kPipeReseed channels and advanced by one FP32 complex multiply per
// channel in between (drift over 16 steps ~1e-6; it reaches the cal phases
// only through baselines that the reference-antenna pass does not cover, with
// weight ~1/S).  Sums: FP32 over 64 channels, folded into Kahan pairs.
// Reseeding every 16 rather than 8 channels and folding every 32 rather than 16
// cut the 128-antenna call from 3.00 to 2.85 ms and moved its cal-phase
// difference from the FP64 form from 5.5e-7 to 2.1e-6 rad (bar: 1e-5); the
// paired multiply-accumulate below and folds every 64 then took it to 2.49 ms
// and 1.6e-6 rad.
//
// Shared-memory reads: lane i reads its 32 bytes as two 16-byte halves; lanes
// with bit 2 set read the upper half first so that each quarter-warp covers
// all 32 banks (conflict-free).  Those lanes hold pols (2,3,0,1) in register
// slots (0,1,2,3) and swap back when writing out.
#pragma once

#include "leap_common.cuh"

namespace leapgb {

// One item of a pipelined launch (device memory; the tensor map needs 128-byte alignment).
struct alignas(128) PipeItem {
  CUtensorMap map;        // [channel][rows*8 floats], box 256 x CH
  const float* uvw_f;     // [rows][6] split UVWs
  double2* out;           // nslab == 1: avg + dir0*4*nbl; else this item's [nslab][ndir][4][nbl] partials
  int64_t rows;
  int32_t T, C, t_per_slab, nslab;
  int32_t tgroups, dgroups, dir0, ndir;
  int32_t unit_begin, pad_[3];
};

struct PipeParams {
  const PipeItem* items;
  const int32_t* order;    // [nslots]: block b visits units order[b], order[b + grid], ... until -1
  int32_t nslots;
  int32_t nitems, units;
  int32_t nbl;
  const float* dirk;       // [ndir_total][12]
  const float2* twiddle;   // [kTwiddleSize]
  int* err;
};

constexpr int kPipeMaxItems = 128;
constexpr int kPipeReseed = 16;         // channels between table-accurate twiddles
// Channels summed in FP32 before a Kahan fold.  At 32 the fold was ~6% of the FMA-pipe work;
// FP32 partial sums over 64 channels (~2e-8 of the sum of |terms|) stay far below the phasor
// drift between reseeds (~1e-6).  Measured: 32-chunk batched workload 11.47 -> 11.10 ms per
// call (cal-phase difference from the FP64 form over 256 directions: median 1.1e-7 -> 1.2e-7
// rad, maximum 4.7e-6 -> 4.2e-6); 128-antenna 1-tile call 2.58 -> 2.49 ms.
constexpr int kPipeFold = 64;
constexpr int kPipeItemBytes = 32 * 4 * 8;  // one channel of one tile: 32 baselines x 4 pols x complex<float>

// Channels per chunk and ring depth: 1 tile x 16 channels = 16 KB stages, 4 deep; 4 tiles x
// 16 channels = 64 KB stages, 3 deep (192 KB of the 227 KB of shared memory).
template <int TPB> struct PipeShape;
template <> struct PipeShape<1> { static constexpr int CH = 16, STAGES = 4; };
template <> struct PipeShape<4> { static constexpr int CH = 16, STAGES = 3; };

template <int TPB>
__host__ __device__ constexpr int pipe_stage_bytes() { return TPB * PipeShape<TPB>::CH * kPipeItemBytes; }

template <int TPB>
__host__ __device__ constexpr int pipe_smem_bytes() {
  return PipeShape<TPB>::STAGES * (pipe_stage_bytes<TPB>() + 16) + kTwiddleSize * 8 + kPipeMaxItems * 4;
}

// Position in a block's chunk sequence: slot s of the order table, unit u = order[s].
struct ChunkCursor {
  int s, u, item, t, cb;
  int t_hi;
};

// Item holding unit u: the last item whose first unit is <= u (binary search; units of
// an item are consecutive and items are in unit order).
__device__ __forceinline__ int find_item(const int* unit_begin, int nitems, int u) {
  int lo = 0, hi = nitems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (unit_begin[mid] <= u) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int slot_unit(const PipeParams& p, int s) { return s < p.nslots ? __ldg(p.order + s) : -1; }

__device__ __forceinline__ void cursor_unit(ChunkCursor& k, const PipeParams& p, const int* unit_begin) {
  k.item = find_item(unit_begin, p.nitems, k.u);
  const PipeItem& it = p.items[k.item];
  const int slab = (k.u - it.unit_begin) % it.nslab;
  k.t = slab * it.t_per_slab;
  k.t_hi = min(it.T, k.t + it.t_per_slab);
  k.cb = 0;
}

template <int TPB>
__device__ __forceinline__ void cursor_next(ChunkCursor& k, const PipeParams& p, const int* unit_begin) {
  k.cb += PipeShape<TPB>::CH;
  if (k.cb < p.items[k.item].C) return;
  k.cb = 0;
  if (++k.t < k.t_hi) return;
  k.s += gridDim.x;
  k.u = slot_unit(p, k.s);
  if (k.u >= 0) cursor_unit(k, p, unit_begin);
}

template <int TPB>
__device__ __forceinline__ void issue_chunk(const ChunkCursor& k, const PipeParams& p, unsigned char* stage_mem,
                                           uint64_t* full, int st) {
  constexpr int CH = PipeShape<TPB>::CH;
  const PipeItem& it = p.items[k.item];
  const int l = k.u - it.unit_begin;
  const int tg = l / (it.dgroups * it.nslab);
  mbar_arrive_expect_tx(&full[st], pipe_stage_bytes<TPB>());
  unsigned char* dst = stage_mem + st * pipe_stage_bytes<TPB>();
#pragma unroll
  for (int ts = 0; ts < TPB; ++ts)
    tma_load_2d(dst + ts * CH * kPipeItemBytes, &it.map, (k.t * p.nbl + (tg * TPB + ts) * 32) * 8, k.cb, &full[st]);
}

// One channel of the complex multiply-accumulate for DPW directions and 4 pols, on paired
// FP32 FMAs (FFMA2): each visibility enters as its natural (re, im) register pair v from the
// shared-memory load and once swapped, vs = (im, re), shared by the DPW directions; the
// phasor stays a natural (zr, zi) pair advanced by 4 scalar FMAs.  Then
//     acc_a += v * z = (vr zr, vi zi),   acc_b += vs * z = (vi zr, vr zi),
// and the fold takes re = acc_a.x - acc_a.y, im = acc_b.x + acc_b.y: 8 paired FMAs (16
// FMA-pipe cycles) and 4 scalar ones per direction and channel, no per-direction moves.
template <int DPW>
__device__ __forceinline__ void mac_channel(const unsigned char* src, int h, float2 (&acc_a)[DPW][4],
                                            float2 (&acc_b)[DPW][4], float2 (&z)[DPW], const float2 (&w)[DPW]) {
  const float4 x0 = *reinterpret_cast<const float4*>(src + 16 * h);
  const float4 x1 = *reinterpret_cast<const float4*>(src + 16 * (1 - h));
  const float2 v[4] = {make_float2(x0.x, x0.y), make_float2(x0.z, x0.w), make_float2(x1.x, x1.y),
                       make_float2(x1.z, x1.w)};
  const float2 vs[4] = {make_float2(x0.y, x0.x), make_float2(x0.w, x0.z), make_float2(x1.y, x1.x),
                        make_float2(x1.w, x1.z)};
#pragma unroll
  for (int j = 0; j < DPW; ++j) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      acc_a[j][q] = __ffma2_rn(v[q], z[j], acc_a[j][q]);
      acc_b[j][q] = __ffma2_rn(vs[q], z[j], acc_b[j][q]);
    }
    const float nr = fmaf(z[j].x, w[j].x, -z[j].y * w[j].y);
    z[j].y = fmaf(z[j].x, w[j].y, z[j].y * w[j].x);
    z[j].x = nr;
  }
}

template <int NC, int DPW, int TPB>
__global__ void __launch_bounds__(NC * 32, 1) rotate_average_mixed_pipe(const PipeParams p) {
  constexpr int CH = PipeShape<TPB>::CH;
  constexpr int NS = PipeShape<TPB>::STAGES;
  constexpr int WPT = NC / TPB;  // warps (direction groups of DPW) per tile
  static_assert(NC % TPB == 0, "warps must divide among tiles");
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* stage_mem = smem;
  float2* tab = reinterpret_cast<float2*>(smem + NS * pipe_stage_bytes<TPB>());
  uint64_t* full = reinterpret_cast<uint64_t*>(tab + kTwiddleSize);
  uint64_t* empty = full + NS;
  int* unit_begin = reinterpret_cast<int*>(empty + NS);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool producer = threadIdx.x == 0;
  for (int i = threadIdx.x; i < kTwiddleSize; i += blockDim.x) tab[i] = __ldg(p.twiddle + i);
  for (int i = threadIdx.x; i < p.nitems; i += blockDim.x) unit_begin[i] = p.items[i].unit_begin;
  __syncthreads();
  ChunkCursor pc{};  // producer cursor, NS chunks ahead of the consumers
  uint32_t issued = 0;
  if (producer) {
    for (int i = 0; i < NS; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], NC);
    }
    fence_mbar_init();
    pc.s = blockIdx.x;
    pc.u = slot_unit(p, pc.s);
    pc.item = 0;
    if (pc.u >= 0) cursor_unit(pc, p, unit_begin);
    for (; issued < NS && pc.u >= 0; ++issued) {
      issue_chunk<TPB>(pc, p, stage_mem, full, issued);
      cursor_next<TPB>(pc, p, unit_begin);
    }
  }
  __syncthreads();

  const int h = (lane >> 2) & 1;  // read order of the two 16-byte halves
  const int ts = warp / WPT, dsub = warp % WPT;
  uint32_t it = 0;
  bool ok = true;
  int item = 0;
  for (int sl = blockIdx.x; ok; sl += gridDim.x) {
    const int u = slot_unit(p, sl);
    if (u < 0) break;
    item = find_item(unit_begin, p.nitems, u);
    const PipeItem& I = p.items[item];
    const int l = u - I.unit_begin;
    const int tg = l / (I.dgroups * I.nslab);
    const int dg = (l / I.nslab) % I.dgroups;
    const int slab = l % I.nslab;
    const int t_lo = slab * I.t_per_slab, t_hi = min(I.T, t_lo + I.t_per_slab);
    const int C = I.C;
    const int b = (tg * TPB + ts) * 32 + lane;
    const bool valid = b < p.nbl;
    const int jd0 = (dg * WPT + dsub) * DPW;  // first direction of this warp within the item
    // A tile wholly past the last baseline (the last tile group when nbl is not a multiple
    // of 32 * TPB) only takes part in the stage hand-over.
    const bool active = jd0 < I.ndir && (tg * TPB + ts) * 32 < p.nbl;

    float sr[DPW][4], si[DPW][4], cr[DPW][4], ci[DPW][4];
#pragma unroll
    for (int j = 0; j < DPW; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) sr[j][q] = si[j][q] = cr[j][q] = ci[j][q] = 0.f;

    // The row's split UVWs are loaded one timestep ahead, so that the set-up of a
    // timestep does not wait on a global load.
    float xn[6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
      xn[i] = active ? __ldg(I.uvw_f + 6 * (static_cast<int64_t>(t_lo) * p.nbl + (valid ? b : 0)) + i) : 0.f;
    for (int t = t_lo; t < t_hi && ok; ++t) {
      uint32_t pa[DPW], pb[DPW];
      float2 w[DPW];
      if (active) {
        // turns(c) = A + c*B, A = -(l*u + m*v + (n-1)*w)*f0/c, B likewise with df.
        float x[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) x[i] = xn[i];
        if (t + 1 < t_hi) {
          const int64_t rn = static_cast<int64_t>(t + 1) * p.nbl + (valid ? b : 0);
#pragma unroll
          for (int i = 0; i < 6; ++i) xn[i] = __ldg(I.uvw_f + 6 * rn + i);
        }
#pragma unroll
        for (int j = 0; j < DPW; ++j) {
          const int d = I.dir0 + min(jd0 + j, I.ndir - 1);
          float ka[6], kb[6];
#pragma unroll
          for (int i = 0; i < 6; ++i) {
            ka[i] = __ldg(p.dirk + 12 * d + i);
            kb[i] = __ldg(p.dirk + 12 * d + 6 + i);
          }
          pa[j] = df_dot3_turns_u32(ka, x);
          pb[j] = df_dot3_turns_u32(kb, x);
          float wr, wi;
          twiddle_turns(pb[j], tab, wr, wi);
          w[j] = make_float2(wr, wi);
        }
      }
      // FP32 partial sums of up to kPipeFold channels, then a Kahan fold.
      // acc holds (vr zr, vi zi) and acc_b (vi zr, vr zi) per direction and pol.
      float2 acc[DPW][4], acc_b[DPW][4];
#pragma unroll
      for (int j = 0; j < DPW; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[j][q] = acc_b[j][q] = make_float2(0.f, 0.f);
      for (int cb = 0; cb < C; cb += CH, ++it) {
        const int n = min(CH, C - cb);
        const int st = it % NS;
        if (!mbar_wait_bounded(&full[st], (it / NS) & 1)) {
          atomicOr(p.err, kDevErrTimeout);
          ok = false;
          break;
        }
        if (active) {
          float2 z[DPW];
          const unsigned char* src = stage_mem + st * pipe_stage_bytes<TPB>() + ts * CH * kPipeItemBytes + lane * 32;
          if (n == CH) {
#pragma unroll
            for (int sub = 0; sub < CH; sub += kPipeReseed) {
#pragma unroll
              for (int j = 0; j < DPW; ++j)
                twiddle_turns(pa[j] + static_cast<uint32_t>(cb + sub) * pb[j], tab, z[j].x, z[j].y);
#pragma unroll
              for (int k = 0; k < kPipeReseed; ++k) {
                mac_channel<DPW>(src + (sub + k) * kPipeItemBytes, h, acc, acc_b, z, w);
              }
            }
          } else {
            for (int k = 0; k < n; ++k) {
              if (k % kPipeReseed == 0) {
#pragma unroll
                for (int j = 0; j < DPW; ++j)
                  twiddle_turns(pa[j] + static_cast<uint32_t>(cb + k) * pb[j], tab, z[j].x, z[j].y);
              }
              mac_channel<DPW>(src + k * kPipeItemBytes, h, acc, acc_b, z, w);
            }
          }
          if ((cb + CH) % kPipeFold == 0 || cb + CH >= C) {
#pragma unroll
            for (int j = 0; j < DPW; ++j)
#pragma unroll
              for (int q = 0; q < 4; ++q) {
                const float re = acc[j][q].x - acc[j][q].y;
                const float im = acc_b[j][q].x + acc_b[j][q].y;
                float y = re - cr[j][q];
                float tt = sr[j][q] + y;
                cr[j][q] = (tt - sr[j][q]) - y;
                sr[j][q] = tt;
                y = im - ci[j][q];
                tt = si[j][q] + y;
                ci[j][q] = (tt - si[j][q]) - y;
                si[j][q] = tt;
                acc[j][q] = acc_b[j][q] = make_float2(0.f, 0.f);
              }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);
        if (producer && pc.u >= 0) {
          // Refill this stage with the chunk NS ahead once every warp released it.
          if (!mbar_wait_bounded(&empty[st], (it / NS) & 1)) {
            atomicOr(p.err, kDevErrTimeout);
            ok = false;
          } else {
            issue_chunk<TPB>(pc, p, stage_mem, full, st);
            cursor_next<TPB>(pc, p, unit_begin);
            ++issued;
          }
        }
        __syncwarp();
      }
    }
    if (ok && active && valid) {
      // nslab == 1: out points at avg[dir0]; else at this item's partials.
      double2* out = I.out + static_cast<int64_t>(I.nslab > 1 ? slab : 0) * I.ndir * 4 * p.nbl;
#pragma unroll
      for (int j = 0; j < DPW; ++j) {
        const int jd = jd0 + j;
        if (jd < I.ndir) {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int pol = q ^ (2 * h);
            out[(static_cast<int64_t>(jd) * 4 + pol) * p.nbl + b] =
                make_double2(static_cast<double>(sr[j][q]) - static_cast<double>(cr[j][q]),
                             static_cast<double>(si[j][q]) - static_cast<double>(ci[j][q]));
          }
        }
      }
    }
  }
  if (producer) {
    // Do not leave while copies issued by this block may still land in shared memory.
    for (uint32_t j = (issued > NS ? issued - NS : 0); j < issued; ++j)
      if (!mbar_wait_bounded(&full[j % NS], (j / NS) & 1)) atomicOr(p.err, kDevErrTimeout);
  }
}

// Per-item slab reduction: out[begin + i] = sum over the item's slabs of partial[s][i],
// i < ndir * per_dir (per_dir = pols * nbl for avgData, nI1 for the reference rows).
struct ReduceItem {
  const double2* partial;  // [nslab][ndir][per_dir]
  int64_t begin;           // first flat output index of the item
  int32_t nslab, ndir;
};

static __global__ void reduce_item_slabs(const ReduceItem* __restrict__ items, int nitems, int per_dir,
                                         double2* __restrict__ avg) {
  const ReduceItem r = items[blockIdx.y];
  const int64_t n = static_cast<int64_t>(r.ndir) * per_dir;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    // Four partial sums (slabs s = j mod 4), added in a fixed order: four loads in flight.
    double re[4] = {0.0, 0.0, 0.0, 0.0}, im[4] = {0.0, 0.0, 0.0, 0.0};
    int s = 0;
    for (; s + 4 <= r.nslab; s += 4) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const double2 v = r.partial[static_cast<int64_t>(s + j) * n + i];
        re[j] += v.x;
        im[j] += v.y;
      }
    }
    for (int j = 0; s < r.nslab; ++s, ++j) {
      const double2 v = r.partial[static_cast<int64_t>(s) * n + i];
      re[j] += v.x;
      im[j] += v.y;
    }
    avg[r.begin + i] = make_double2((re[0] + re[1]) + (re[2] + re[3]), (im[0] + im[1]) + (im[2] + im[3]));
  }
}

}  // namespace leapgb
