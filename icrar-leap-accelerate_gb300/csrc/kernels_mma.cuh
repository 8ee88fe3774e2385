// Mixed-precision rotate + average with the complex multiply-accumulate on the
// tensor cores (4 pols, complex<float>).
//
// For one baseline row r and a block of channels, the averages of 16 directions
// and 4 pols form a small matrix product
//     avg[d][p] += sum_c z[d][c] * V[c][p],   z[d][c] = exp(2*pi*i*turns(r, d, c)),
// whose real form is a 16 x 8 x 8 MMA per 4 channels (mma.sync m16n8k8, TF32):
//     A[d][k]   k = (part, c): Re z (part 0), Im z (part 1)     16 directions x 8
//     B[k][n]   n = (p, re/im): (Re V, -Im V ; Im V, Re V)       8 x (4 pols x 2)
//     D[d][n]   (Re, Im) of the 4-pol sums of the 16 directions
// The phasors are generated in registers directly in the A-fragment layout:
// lane (g = lane/4, q = lane%4) holds z for directions g and g+8 at channel q of
// each 4-channel step, and advances both by exp(2*pi*i*4B) per step.  B comes from
// the TMA-staged tile with one 8-byte shared load per lane.  FP32 accuracy from
// TF32 units: every operand is split as hi = x rounded to TF32, lo = x - hi, and the
// step issues hi*hi + hi*lo + lo*hi into one FP32 accumulator.
//
// Measured on GB300 (128-antenna workload, 14 timesteps, 64 directions): 3.49 ms
// against 2.96 ms for the CUDA-core kernel, at 5.3e-6 rad cal-phase error against the
// FP64 form (CUDA-core kernel: 5.5e-7); splitting with cvt.rna.tf32 instead costs
// 4.6 ms, and truncating splits (3.1 ms) exceed the 1e-5 rad bar.  The 16x8x8 MMAs are small, their accumulators form
// dependent chains, the per-lane phasor recurrence and operand splits still run on
// the FP32 pipe, and the B loads of one step hit the same shared-memory banks for
// the four channels.  It is therefore an autotuner candidate for batched calls
// (LEAP_OPTION_TENSOR_CORE_ROTATION) rather than the default.
//
// Block: 8 warps share one 32-baseline tile (the TMA ring and producer of the
// CUDA-core kernel, 16-channel chunks); warp w owns baselines 4w .. 4w+3 of the
// tile for the unit's 16 directions, with FP32 accumulators folded into Kahan
// pairs every 32 channels.  Phasors are reseeded table-accurately (twiddle_turns)
// every 32 channels, i.e. after 8 recurrence steps, as in the CUDA-core kernel.
// Units (tile, 16-direction group, timestep slab) follow the host's order table.
#pragma once

#include "kernels_pipe.cuh"

namespace leapgb {

constexpr int kMmaDirs = 16;          // directions per unit: the M of one MMA
constexpr int kMmaBaselines = 4;      // baselines per warp
constexpr int kMmaReseedChunks = 2;   // table-accurate phasors every 2 chunks (32 channels)
constexpr int kMmaFoldChunks = 2;     // Kahan fold every 2 chunks

// x = hi + lo with hi = x rounded to TF32 (nearest, ties away from zero: add half an ulp
// of the 10-bit mantissa to the bits, clear the low 13) and lo = x - hi, exact in FP32 and
// at most 2^-11 |x|; the tensor core reads lo to TF32, which leaves x - hi - lo below
// about 2^-22 |x|.  Two integer operations instead of a conversion instruction; the
// operands here are finite and far from the overflow threshold.
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  const uint32_t h = (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u;
  hi = h;
  lo = __float_as_uint(x - __uint_as_float(h));
}

__device__ __forceinline__ void mma_16x8x8_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                                uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

static __global__ void __launch_bounds__(256, 1) rotate_average_mma_pipe(const PipeParams p) {
  constexpr int TPB = 1;
  constexpr int CH = PipeShape<TPB>::CH;
  constexpr int NS = PipeShape<TPB>::STAGES;
  constexpr int NC = 8;
  constexpr int NB = kMmaBaselines;
  static_assert(NC * NB == 32, "8 warps x 4 baselines cover a 32-baseline tile");
  static_assert(CH == 16, "4 MMA steps of 4 channels per chunk");
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* stage_mem = smem;
  float2* tab = reinterpret_cast<float2*>(smem + NS * pipe_stage_bytes<TPB>());
  uint64_t* full = reinterpret_cast<uint64_t*>(tab + kTwiddleSize);
  uint64_t* empty = full + NS;
  int* unit_begin = reinterpret_cast<int*>(empty + NS);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, q = lane & 3;
  const bool producer = threadIdx.x == 0;
  for (int i = threadIdx.x; i < kTwiddleSize; i += blockDim.x) tab[i] = __ldg(p.twiddle + i);
  for (int i = threadIdx.x; i < p.nitems; i += blockDim.x) unit_begin[i] = p.items[i].unit_begin;
  __syncthreads();
  ChunkCursor pc{};
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

  uint32_t it = 0;
  bool ok = true;
  for (int sl = blockIdx.x; ok; sl += gridDim.x) {
    const int u = slot_unit(p, sl);
    if (u < 0) break;
    const int item = find_item(unit_begin, p.nitems, u);
    const PipeItem& I = p.items[item];
    const int l = u - I.unit_begin;
    const int tg = l / (I.dgroups * I.nslab);
    const int dg = (l / I.nslab) % I.dgroups;
    const int slab = l % I.nslab;
    const int t_lo = slab * I.t_per_slab, t_hi = min(I.T, t_lo + I.t_per_slab);
    const int C = I.C;
    const int b0 = tg * 32 + warp * NB;           // first baseline of this warp
    const int e[2] = {dg * kMmaDirs + g, dg * kMmaDirs + g + 8};  // directions (within the item) of rows g, g+8
    int dglob[2];
#pragma unroll
    for (int x = 0; x < 2; ++x) dglob[x] = I.dir0 + min(e[x], I.ndir - 1);

    float acc[NB][4], sum[NB][4], cmp[NB][4];
#pragma unroll
    for (int j = 0; j < NB; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[j][k] = sum[j][k] = cmp[j][k] = 0.f;

    for (int t = t_lo; t < t_hi && ok; ++t) {
      // Per (baseline, direction): turns(c) = pa + c*pb as 2^-32 fixed point; step of 4 channels.
      uint32_t pa[NB][2], pb[NB][2];
      float wr[NB][2], wi[NB][2], zr[NB][2], zi[NB][2];
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const int b = min(b0 + j, p.nbl - 1);
        const int64_t r = static_cast<int64_t>(t) * p.nbl + b;
        float xu[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) xu[i] = __ldg(I.uvw_f + 6 * r + i);
#pragma unroll
        for (int x = 0; x < 2; ++x) {
          float ka[6], kb[6];
#pragma unroll
          for (int i = 0; i < 6; ++i) {
            ka[i] = __ldg(p.dirk + 12 * dglob[x] + i);
            kb[i] = __ldg(p.dirk + 12 * dglob[x] + 6 + i);
          }
          pa[j][x] = df_dot3_turns_u32(ka, xu);
          pb[j][x] = df_dot3_turns_u32(kb, xu);
          twiddle_turns(pb[j][x] * 4u, tab, wr[j][x], wi[j][x]);
          zr[j][x] = 1.f;
          zi[j][x] = 0.f;
        }
      }
      for (int cb = 0; cb < C; cb += CH, ++it) {
        const int st = it % NS;
        if (!mbar_wait_bounded(&full[st], (it / NS) & 1)) {
          atomicOr(p.err, kDevErrTimeout);
          ok = false;
          break;
        }
        const int chunk = cb / CH;
        if (chunk % kMmaReseedChunks == 0) {
#pragma unroll
          for (int j = 0; j < NB; ++j)
#pragma unroll
            for (int x = 0; x < 2; ++x)
              twiddle_turns(pa[j][x] + static_cast<uint32_t>(cb + q) * pb[j][x], tab, zr[j][x], zi[j][x]);
        }
        // Channels past C are zero in the tile (TMA fill) and add nothing.
        const unsigned char* src = stage_mem + st * pipe_stage_bytes<TPB>() + (g >> 1) * 8;
#pragma unroll
        for (int s = 0; s < CH / 4; ++s) {
#pragma unroll
          for (int j = 0; j < NB; ++j) {
            const float2 v = *reinterpret_cast<const float2*>(src + ((4 * s + q) * 32 + warp * NB + j) * 32);
            const float bf0 = (g & 1) ? v.y : v.x;
            const float bf1 = (g & 1) ? v.x : -v.y;
            uint32_t b0h, b0l, b1h, b1l;
            split_tf32(bf0, b0h, b0l);
            split_tf32(bf1, b1h, b1l);
            uint32_t a0h, a0l, a1h, a1l, a2h, a2l, a3h, a3l;
            split_tf32(zr[j][0], a0h, a0l);
            split_tf32(zr[j][1], a1h, a1l);
            split_tf32(zi[j][0], a2h, a2l);
            split_tf32(zi[j][1], a3h, a3l);
            mma_16x8x8_tf32(acc[j], a0h, a1h, a2h, a3h, b0h, b1h);
            mma_16x8x8_tf32(acc[j], a0h, a1h, a2h, a3h, b0l, b1l);
            mma_16x8x8_tf32(acc[j], a0l, a1l, a2l, a3l, b0h, b1h);
#pragma unroll
            for (int x = 0; x < 2; ++x) {
              const float nr = fmaf(zr[j][x], wr[j][x], -zi[j][x] * wi[j][x]);
              zi[j][x] = fmaf(zr[j][x], wi[j][x], zi[j][x] * wr[j][x]);
              zr[j][x] = nr;
            }
          }
        }
        if (chunk % kMmaFoldChunks == kMmaFoldChunks - 1 || cb + CH >= C) {
#pragma unroll
          for (int j = 0; j < NB; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const float y = acc[j][k] - cmp[j][k];
              const float tt = sum[j][k] + y;
              cmp[j][k] = (tt - sum[j][k]) - y;
              sum[j][k] = tt;
              acc[j][k] = 0.f;
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);
        if (producer && pc.u >= 0) {
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
    if (ok) {
      // Lane (g, q) holds pol q of directions e[0] (elements 0, 1) and e[1] (2, 3).
      double2* out = I.out + static_cast<int64_t>(I.nslab > 1 ? slab : 0) * I.ndir * 4 * p.nbl;
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const int b = b0 + j;
        if (b >= p.nbl) continue;
#pragma unroll
        for (int x = 0; x < 2; ++x) {
          if (e[x] >= I.ndir) continue;
          out[(static_cast<int64_t>(e[x]) * 4 + q) * p.nbl + b] =
              make_double2(static_cast<double>(sum[j][2 * x]) - static_cast<double>(cmp[j][2 * x]),
                           static_cast<double>(sum[j][2 * x + 1]) - static_cast<double>(cmp[j][2 * x + 1]));
        }
      }
    }
  }
  if (producer) {
    for (uint32_t j = (issued > NS ? issued - NS : 0); j < issued; ++j)
      if (!mbar_wait_bounded(&full[j % NS], (j / NS) & 1)) atomicOr(p.err, kDevErrTimeout);
  }
}

}  // namespace leapgb
