// Gridded rotate + average (mixed form, 4 pols, complex<float>) on the tensor cores.
//
// For one row r and one direction the averaging sums (LA/algorithm/cpu/
// CpuLeapCalibrator.cc:181-217) are
//   sum_c V[p, r, c] exp(2 pi i (A + c B)),   A, B in turns (A: f0 term, B: df term).
// With c = c0 + k (c0 = C/2) that is exp(2 pi i (A + c0 B)) G(B) where
//   G(B) = sum_k f_k exp(2 pi i k B),  f_k = V[p, r, c0 + k],
// a trigonometric polynomial in B that does not depend on the direction.  G is
// evaluated as a type-2 non-uniform DFT: on the grid B_l = l / n (n = 2C, twice
// oversampled) the values
//   b_l = sum_k f_k exp(2 pi i k l / n) / Psi(k)
// are one dense product of the visibility tile with a fixed matrix E[l, k], and
//   G(B) ~= sum_l b_l psi(n B - l)
// over the W grid points nearest n B, with psi the "exponential of semicircle"
// kernel psi(x) = exp(beta (sqrt(1 - (2x/W)^2) - 1)) and Psi its Fourier
// transform at frequency k / n (Barnett, Magland & af Klinteberg, SIAM J. Sci.
// Comput. 41 (2019) C479).  With W = 10, beta = 2.3 W the interpolation error is
// about 1e-9 of the l2 norm of f (their rule for a 2x grid: W = log10(1/eps) + 1).
// W = 8 (error ~1e-7) was measured too coarse for long integrations: the error of a
// bright source's fringe adds coherently over timesteps while the averages of
// directions away from it do not, and a 47-timestep chunk reached 2e-5 rad.
// Per (row, direction) the work is W + 1 complex multiply-adds instead of C, so the
// direction count no longer multiplies the channel work; the channel work moves to
// the tensor cores.
//
// Tile: M = 128 rows of the product = 4 baselines x 4 timesteps x 4 pols x
// (re, im).  TMEM lane m = 32 q + 8 t + 2 p + s holds baseline q of the quad, so
// each 32-lane quarter is one baseline at 4 neighbouring timesteps, whose grid
// positions differ by far less than a grid step: one warp-uniform 16-column
// tcgen05.ld per accumulator half serves all 32 lanes of a direction.
//
// The product runs in 3xFP16 (V E ~ V_hi E_hi + V_lo E_hi + V_hi E_lo with hi = f16(x),
// lo = f16(x - hi): 22 significant bits, as 3xTF32, at half the operand bytes and MMAs).
// Each (baseline, pol) of a tile is scaled by a power of two that puts its largest
// component near 2^14 and the grid matrix by one for the whole table, so both splits stay
// in FP16's normal range; the epilogue undoes the scales exactly.  The tensor cores
// accumulate FP32 with truncation, whose error
// grows with the number of accumulation steps and the size of the accumulator, and is
// biased (toward zero), so it too adds coherently over timesteps; so the large hi*hi
// products restart in a fresh accumulator every 64 channels (a "segment") and the small
// corrections go to an accumulator of their own.  Fold warps add the segments together
// with rounded FP32 adds.  Emulated on a 47-timestep, 384-channel chunk of 128
// antennas, the truncation is then the largest error left, ~1e-7 of the sum of |terms|.
// (32-channel segments measured 5% slower at 128 antennas, with no lower maximum error.)
//
// TMEM (512 columns, one block per SM): RS[0], RS[1] (running sums, double
// buffered: the epilogue reads one while the next tile accumulates into the
// other), IS (segments 1.. of the current tile), AC (corrections).  Column 2j of
// a region holds sum V_s Re E at window grid point j, column 2j + 1 sum V_s Im E
// (the grid matrix interleaves its re and im rows), so the W + 1 taps of one
// stencil are 2 (W + 1) = 22 adjacent columns: a 16-, a 4- and a 2-column tcgen05.ld.
//
// Operands.  The tile's visibilities reach shared memory already scaled and split into
// FP16 hi and lo parts in the MMA's canonical K-major layout: grid_split_operand builds
// that copy of an integration once (8 KB per tile and 16-channel chunk, the bytes of the
// visibilities), and each chunk is then one bulk copy, so no warp converts operands
// between the copy and the MMAs.
//
// Warp roles (14 warps): 0 = producer (bulk copies of the split operand and of the E
// window), 1 = MMA issuer (+ TMEM owner), 2-5 = fold warps (add the finished hi*hi
// segments and the corrections into the running sums), 6-13 = epilogue (warp w reads
// TMEM lanes 32 (w % 4) ..; two warps per quarter take 32 directions each).  One ring of
// kGrStages stages of {A hi, A lo, E window}, handed over in rounds of kGrMacro (one 64-channel
// segment) and released by one MMA commit per round.  A round issues its 8 correction MMAs
// before its 4 hi*hi MMAs, so the fold that frees IS overlaps the corrections (a round's
// stages all land before it starts).  Every wait is bounded; a timeout sets the error word, stops every
// role, and the block still waits (bounded) for its copies and MMAs and frees its TMEM.
#pragma once

#include <cuda_fp16.h>

#include "leap_common.cuh"
#include "kernels_tc.cuh"

namespace leapgb {

constexpr int kGrTaps = 10;           // W, grid points per interpolation
constexpr float kGrBeta = 23.0f;      // 2.3 W
constexpr int kGrChunk = 16;          // channels per stage
constexpr int kGrSegChunks = 4;       // chunks per hi*hi accumulation segment (64 channels)
constexpr int kGrStages = 8;          // {A hi, A lo, E window} ring: two rounds in flight
constexpr int kGrMacro = 4;           // chunks handed over per barrier round: one hi*hi segment
// One MMA commit per round releases the round's stages to the producer and tells the fold warps
// that the segment is complete: a commit makes the issuing thread wait for the MMAs before it
// (measured: 72 MMAs issue in 12.3K cycles without commits, 24.6K with one every 6), so the
// kernel commits once per segment rather than per stage pair, per segment and per tile.
constexpr int kGrMacroStages = kGrStages / kGrMacro;
constexpr int kGrJwMax = 64;          // grid points per pass (MMA N = 2 Jw <= 128)
constexpr int kGrPassStride = 48;     // grid points between pass windows (multiple of 8)
constexpr int kGrLoadCols = kGrTaps + 1;  // grid points one interpolation load reads (2 TMEM columns each)
constexpr int kGrPolyDeg = 8;         // degree of the per-tap weight polynomials
constexpr int kGrBatch = 4;           // directions per timestep reduce-scatter (loads go in pairs)
constexpr int kGrDirs = 64;           // directions per unit (8 epilogue warps x 32 / 4 quarters)
constexpr int kGrEpiWarps = 8;
constexpr int kGrWarpDirs = kGrDirs * 4 / kGrEpiWarps;  // directions per epilogue warp
constexpr int kGrWarps = 6 + kGrEpiWarps;
constexpr int kGrThreads = kGrWarps * 32;
constexpr int kGrAHalf = 128 * kGrChunk * 2;            // one split of A: 128 rows x 16 f16 (32 B)
constexpr int kGrOpBytes = 2 * kGrAHalf;                 // hi + lo of one chunk of one tile
constexpr int kGrEBytes = 2 * 2 * kGrJwMax * kGrChunk * 2;  // [hl][2 Jw rows x 32 B]
// Stage: [A hi][A lo][E hi][E lo]
constexpr int kGrStageBytes = kGrOpBytes + kGrEBytes;
constexpr int kGrEOffset = kGrOpBytes;
constexpr int kGrRecWords = 16;                          // per (direction, timestep) record: 4 16-byte rows
constexpr int kGrCodeWord = kGrTaps + 3;                 // record: W + 1 weights, cr, sr, then the load code
constexpr int kGrRecDirs = 16;                           // directions whose records a warp holds at a time
constexpr int kGrRecBytes = kGrEpiWarps * 4 * kGrRecDirs * kGrRecWords * 4;  // [warps][4 t][16 dirs][12]
constexpr uint32_t kGrRegion = 128;                      // TMEM columns per region
constexpr uint32_t kGrIS = 2 * kGrRegion, kGrAC = 3 * kGrRegion;
constexpr int kGrWide = 1 << 16;                         // record flag: the 4 timesteps need separate loads
constexpr int kGrNumBars = 2 * kGrMacroStages + 8;

// A pass window must hold every stencil whose start falls in its stride, plus the
// columns one load reads past the stencil.
static_assert(kGrPassStride % 8 == 0 && kGrPassStride - 1 + kGrLoadCols <= kGrJwMax, "pass windows");
static_assert(kGrMacro == kGrSegChunks, "a barrier round is a segment");
static_assert(kGrStages % kGrMacro == 0 && kGrStages / kGrMacro >= 2, "at least two rounds in flight");
static_assert(kGrTaps + 1 <= kGrLoadCols, "one load per stencil");
static_assert(kGrCodeWord < kGrRecWords, "record layout");

__host__ __device__ constexpr int grid_smem_bytes() {
  return kGrStages * kGrStageBytes + kTwiddleSize * 8 + kGrRecBytes + kGrNumBars * 8 + 16;
}
static_assert(grid_smem_bytes() <= 227 * 1024, "one block's dynamic shared memory (227 KB on sm_103)");

// Rows of the E table of channel count C: row r is grid point l = r - lbase.
__host__ __device__ constexpr int grid_lbase(int C) { return ((C + kGrTaps + 8 + 7) / 8) * 8; }
__host__ __device__ constexpr int grid_rows(int C) { return ((grid_lbase(C) + C + kGrJwMax + 8 + 7) / 8) * 8; }
__host__ __device__ constexpr int grid_chunks(int C) { return (C + kGrChunk - 1) / kGrChunk; }
// Split grid operand of an integration: per (quad, timestep block, 16-channel chunk) the
// tile's scaled visibilities as FP16 hi and lo parts in the MMA's canonical K-major layout,
// [hi: 16 row groups x 2 k-halves x 8 rows x 16 B][lo: the same], 8 KB, exactly what the
// shared-memory stage holds before the MMAs of a chunk; then the inverse scales, one float
// per (quad, timestep block, baseline of the quad, pol).
__host__ __device__ constexpr int64_t grid_operand_bytes(int nbl, int T, int C) {
  return static_cast<int64_t>((nbl + 3) / 4) * ((T + 3) / 4) * ((C + 15) / 16) * kGrOpBytes;
}
__host__ __device__ constexpr int64_t grid_scale_bytes(int nbl, int T) {
  return static_cast<int64_t>((nbl + 3) / 4) * ((T + 3) / 4) * 16 * 4;
}

// Byte offset of element (row, k) of a K-major operand block of 16-bit values without
// swizzle: 8-row core matrices of 16 B rows, k-halves 128 B apart, row groups 256 B apart.
__host__ __device__ constexpr int grid_f16_offset(int row, int k) {
  return ((row >> 3) * 2 + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// Builds the split grid operand of a 4-pol complex<float> integration [C][rows][8 floats]:
// one 128-thread block per (quad, timestep block); warp w takes timestep w of the block and
// lane = 8 q + 2 p + s, the baseline q of the quad, pol p, (re, im) s.  The power of two
// of each (baseline, pol) brings its largest |component| over the block's 4 timesteps and
// all channels into [2^13, 2^14); vinv holds its inverse (1 for an all-zero one).  hi is
// the scaled visibility rounded to FP16, lo the remainder rounded to FP16.  Rows and
// channels past the integration are zero, as a tensor-map load fills them.
static __global__ void __launch_bounds__(128) grid_split_operand(const float* __restrict__ vis, int64_t rows, int nbl,
                                                                 int T, int C, int ntb, unsigned char* __restrict__ out,
                                                                 float* __restrict__ vinv) {
  __shared__ float smax[4][32];
  const int q = blockIdx.x, tb = blockIdx.y, nchunk = (C + kGrChunk - 1) / kGrChunk;
  const int lane = threadIdx.x & 31, tl = threadIdx.x >> 5;
  const int t = tb * 4 + tl, b = q * 4 + (lane >> 3);
  const bool rv = t < T && b < nbl;
  const float* src = vis + (static_cast<int64_t>(t) * nbl + b) * 8 + (lane & 7);
  const int64_t cstride = rows * 8;
  float m = 0.f;
  if (rv)
    for (int c = 0; c < C; ++c) m = fmaxf(m, fabsf(__ldg(src + c * cstride)));
  m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));  // re and im
  smax[tl][lane] = m;
  __syncthreads();
  m = fmaxf(fmaxf(smax[0][lane], smax[1][lane]), fmaxf(smax[2][lane], smax[3][lane]));
  int e = 0;
  (void)frexpf(m, &e);  // m < 2^e
  const float scale = m > 0.f ? ldexpf(1.f, 14 - e) : 1.f;
  if (tl == 0 && !(lane & 1)) vinv[(static_cast<int64_t>(q) * ntb + tb) * 16 + (lane >> 1)] = 1.f / scale;
  const int mrow = (lane >> 3) * 32 + tl * 8 + (lane & 7);  // TMEM lane: baseline, timestep, pol, re/im
  for (int chunk = 0; chunk < nchunk; ++chunk) {
    unsigned char* dst = out + ((static_cast<int64_t>(q) * ntb + tb) * nchunk + chunk) * kGrOpBytes;
#pragma unroll
    for (int kh = 0; kh < 2; ++kh) {
      uint32_t hw[4], lw[4];
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        float x[2];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const int c = chunk * kGrChunk + kh * 8 + j + i;
          x[i] = (rv && c < C) ? __ldg(src + c * cstride) * scale : 0.f;
        }
        const __half2 h = __floats2half2_rn(x[0], x[1]);
        const __half2 l = __floats2half2_rn(x[0] - __low2float(h), x[1] - __high2float(h));
        hw[j >> 1] = *reinterpret_cast<const uint32_t*>(&h);
        lw[j >> 1] = *reinterpret_cast<const uint32_t*>(&l);
      }
      const int off = grid_f16_offset(mrow, kh * 8);
      *reinterpret_cast<uint4*>(dst + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
      *reinterpret_cast<uint4*>(dst + kGrAHalf + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
    }
  }
}

// One item of a gridded launch (device memory).
struct alignas(16) GridItem {
  const unsigned char* op;  // split grid operand: [quad][timestep block][chunk][kGrOpBytes]
  const float* vinv;     // [quad][timestep block][16]: inverse scales of the operand's (baseline, pol)s
  const float* uvw_f;    // [rows][6] split UVWs
  const unsigned char* etab;  // E table of this channel count (FP16 hi/lo, scaled by 1 / einv)
  double2* out;          // nslab == 1: avg + dir0*4*nbl; else this item's [nslab][ndir][4][nbl] partials
  int32_t T, C, nchunk, tb_per_slab;
  int32_t nslab, nquad, dgroups, dir0;
  int32_t ndir, unit_begin, nrg, lbase;
  int32_t udg, uparts;   // direction groups per unit, units per (quad, slab): ceil(dgroups / udg)
  int32_t ntb;           // timestep blocks of the integration (the operand's second dimension)
  float einv;            // inverse scale of the E table
};

// Grid window of one unit, written by grid_windows: table rows [8 rg0, 8 rg0 + jw)
// in pass 0, shifted by kGrPassStride per pass.  npass == 0: nothing to do.
struct GridWindow {
  int32_t rg0, jw, npass, pad;
};

struct GridParams {
  const GridItem* items;
  const int32_t* order;    // [nslots]: block b visits units order[b], order[b + grid], ... until -1
  GridWindow* win;         // [units]
  const float* dirk;       // [ndir_total][12]
  const float2* twiddle;   // [kTwiddleSize]
  int* err;
  int32_t nslots, nitems, units, nbl;
  // Weight polynomials: tap m of a stencil at fractional grid position f has weight
  // sum_j wpoly[m][j] x^j, x = 2 f - 1 (es_kernel_poly on the host; the kernel reads the
  // rows m < W / 2 and mirrors them).
  float wpoly[kGrTaps][kGrPolyDeg + 1];
};

// A unit: one quad of baselines over one timestep slab, for direction groups [dg_lo, dg_hi)
// of its item (the grid product of a tile serves all of them).
struct GridUnit {
  int item, quad, slab, t_lo, t_hi, ntb, dg_lo, dg_hi;
};

__device__ __forceinline__ int grid_find_item(const GridItem* items, int nitems, int u) {
  int lo = 0, hi = nitems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&items[mid].unit_begin) <= u) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ GridUnit grid_unit(const GridParams& p, int u) {
  GridUnit g;
  g.item = grid_find_item(p.items, p.nitems, u);
  const GridItem& I = p.items[g.item];
  const int l = u - I.unit_begin;
  g.quad = l / (I.uparts * I.nslab);
  const int part = (l / I.nslab) % I.uparts;
  g.slab = l % I.nslab;
  g.dg_lo = part * I.udg;
  g.dg_hi = min(I.dgroups, g.dg_lo + I.udg);
  g.t_lo = g.slab * I.tb_per_slab * 4;
  g.t_hi = min(I.T, g.t_lo + I.tb_per_slab * 4);
  g.ntb = (g.t_hi - g.t_lo + 3) / 4;
  return g;
}

// Grid position n*B of a phase slope B given as a 2^-32 fixed-point fraction of a
// turn (its signed value is B reduced to [-1/2, 1/2), which leaves exp(2 pi i k B)
// unchanged for integer k): returns floor(n B), and the fraction in f.
__device__ __forceinline__ int grid_position(uint32_t pb, int n, float& f) {
  const long long prod = static_cast<long long>(static_cast<int>(pb)) * n;
  f = static_cast<float>(static_cast<uint32_t>(prod)) * 2.3283064365386963e-10f;
  return static_cast<int>(prod >> 32);
}

// First grid point of the W-point stencil (W even) around x = i0 + f: the points within
// W/2 of x are i0 - W/2 + 1 .. i0 + W/2.  A load reads W + 1 points from the earliest
// start of a quarter's 4 timesteps, which covers starts that differ by one.
static_assert(kGrTaps % 2 == 0, "the stencil start is floor(x) - W/2 + 1 for even W");
__device__ __forceinline__ int grid_stencil_start(int i0, float) { return i0 - kGrTaps / 2 + 1; }

__device__ __forceinline__ void tma_load_3d(void* smem_dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(smem_dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait that also gives up once another role has raised the abort flag.
// (mbarrier.try_wait itself suspends the thread for a while when the phase is not complete.)
__device__ __forceinline__ bool grid_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
  for (uint32_t i = 0; i < kMaxWaitPolls; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63u) == 63u && *abort_flag) return false;
  }
  return false;
}

__device__ __forceinline__ void grid_fail(const GridParams& p, volatile int* abort_flag) {
  atomicOr(p.err, kDevErrTimeout);
  *abort_flag = 1;
}

// Grid window of each unit: the range of stencil starts over the unit's rows and its
// direction groups.  One 64-thread block per unit: thread r takes rows r, r + 64, ... of the
// unit (baseline r % 4 of the quad, timestep t_lo + r / 4), loads its UVWs once and walks the
// directions, whose slopes the block stages in shared memory 64 at a time.
constexpr int kGrWinThreads = 64;
static __global__ void __launch_bounds__(kGrWinThreads) grid_windows(const GridParams p) {
  __shared__ float kbs[kGrDirs][6];
  __shared__ int red[2][kGrWinThreads / 32];
  const int u = blockIdx.x;
  const GridUnit g = grid_unit(p, u);
  const GridItem& I = p.items[g.item];
  const int n = 2 * I.C;
  const int nrow = (g.t_hi - g.t_lo) * 4;
  int smin = 0x7fffffff, smax = -0x7fffffff;
  for (int dg = g.dg_lo; dg < g.dg_hi; ++dg) {
    const int nd = min(kGrDirs, I.ndir - dg * kGrDirs);
    __syncthreads();  // the previous group's slopes are no longer read
    for (int i = threadIdx.x; i < nd * 6; i += kGrWinThreads)
      kbs[i / 6][i % 6] = __ldg(p.dirk + 12 * (I.dir0 + dg * kGrDirs + i / 6) + 6 + i % 6);
    __syncthreads();
    for (int rr = threadIdx.x; rr < nrow; rr += kGrWinThreads) {
      const int b = g.quad * 4 + (rr & 3), t = g.t_lo + (rr >> 2);
      if (b >= p.nbl) continue;
      const int64_t r = static_cast<int64_t>(t) * p.nbl + b;
      float x[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) x[i] = __ldg(I.uvw_f + 6 * r + i);
      for (int d = 0; d < nd; ++d) {
        float f;
        const int i0 = grid_position(df_dot3_turns_u32(kbs[d], x), n, f);
        const int st = grid_stencil_start(i0, f);
        smin = min(smin, st);
        smax = max(smax, st);
      }
    }
  }
  smin = __reduce_min_sync(0xffffffffu, smin);
  smax = __reduce_max_sync(0xffffffffu, smax);
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = smin;
    red[1][threadIdx.x >> 5] = smax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 1; w < kGrWinThreads / 32; ++w) {
      smin = min(smin, red[0][w]);
      smax = max(smax, red[1][w]);
    }
    GridWindow w{0, 16, 0, 0};
    if (smin <= smax) {
      w.rg0 = (smin + I.lbase) >> 3;
      const int r0 = w.rg0 * 8;
      // Stencil starts lie in [smin, smax]; a load reads kGrLoadCols grid points from a start.
      const int need = smax + kGrLoadCols + I.lbase - r0;
      if (need <= kGrJwMax) {
        w.jw = max(8, (need + 7) & ~7);
        w.npass = 1;
      } else {
        w.jw = kGrJwMax;
        w.npass = (smax + I.lbase - r0) / kGrPassStride + 1;
      }
    }
    p.win[u] = w;
  }
}

// The W + 1 weights of a shared load for a stencil at fractional grid position f that starts
// `shifted` (0 or 1) columns after the load: w[k] = h_{k - shifted}(f), 0 outside the W taps,
// with h_m the tap polynomials of c (degree kGrPolyDeg in x = 2 f - 1).  psi is even, so tap
// W - 1 - m is tap m mirrored, h_{W-1-m}(x) = h_m(-x): each pair is evaluated from the even and
// odd parts of h_m in y = x^2 (half the multiply-adds of W separate Horner chains, and chains
// half as long).  Only rows m < W / 2 of c are read.  The weight error is about 8e-8 of the
// largest weight, FP32 rounding included.
template <int W>
__device__ __forceinline__ void grid_weights(float f, bool shifted, const float (&c)[W][kGrPolyDeg + 1],
                                             float (&w)[W + 1]) {
  static_assert(W % 2 == 0 && kGrPolyDeg % 2 == 0, "tap pairs; even and odd parts of an even degree");
  const float x = fmaf(2.0f, f, -1.0f);
  const float y = x * x;
  float h[W];
#pragma unroll
  for (int m = 0; m < W / 2; ++m) {
    float e = c[m][kGrPolyDeg];
#pragma unroll
    for (int j = kGrPolyDeg - 2; j >= 0; j -= 2) e = fmaf(e, y, c[m][j]);
    float o = c[m][kGrPolyDeg - 1];
#pragma unroll
    for (int j = kGrPolyDeg - 3; j >= 1; j -= 2) o = fmaf(o, y, c[m][j]);
    h[m] = fmaf(x, o, e);
    h[W - 1 - m] = fmaf(-x, o, e);
  }
  w[0] = shifted ? 0.f : h[0];
#pragma unroll
  for (int k = 1; k < W; ++k) w[k] = shifted ? h[k - 1] : h[k];
  w[W] = shifted ? h[W - 1] : 0.f;
}

// Two directions' stencils from TMEM: a 16-, a 4- and a 2-column load each (the W + 1 = 11
// taps, re and im interleaved) at columns c0 and c1 of this warp's lanes, and one wait for both.
constexpr int kGrLoadRegs = 2 * kGrLoadCols;
static_assert(kGrLoadRegs == 22, "22 columns per stencil: x16 + x4 + x2 loads");
__device__ __forceinline__ void grid_load_pair(uint32_t tbase, uint32_t c0, uint32_t c1,
                                               uint32_t (&v)[2][kGrLoadRegs]) {
  // All loads and the wait in one statement: the results are defined only after the wait.
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%44];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16,%17,%18,%19}, [%45];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%20,%21}, [%46];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37}, [%47];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%38,%39,%40,%41}, [%48];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%42,%43}, [%49];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(v[0][0]), "=r"(v[0][1]), "=r"(v[0][2]), "=r"(v[0][3]), "=r"(v[0][4]), "=r"(v[0][5]), "=r"(v[0][6]),
        "=r"(v[0][7]), "=r"(v[0][8]), "=r"(v[0][9]), "=r"(v[0][10]), "=r"(v[0][11]), "=r"(v[0][12]), "=r"(v[0][13]),
        "=r"(v[0][14]), "=r"(v[0][15]), "=r"(v[0][16]), "=r"(v[0][17]), "=r"(v[0][18]), "=r"(v[0][19]),
        "=r"(v[0][20]), "=r"(v[0][21]),
        "=r"(v[1][0]), "=r"(v[1][1]), "=r"(v[1][2]), "=r"(v[1][3]), "=r"(v[1][4]), "=r"(v[1][5]), "=r"(v[1][6]),
        "=r"(v[1][7]), "=r"(v[1][8]), "=r"(v[1][9]), "=r"(v[1][10]), "=r"(v[1][11]), "=r"(v[1][12]), "=r"(v[1][13]),
        "=r"(v[1][14]), "=r"(v[1][15]), "=r"(v[1][16]), "=r"(v[1][17]), "=r"(v[1][18]), "=r"(v[1][19]),
        "=r"(v[1][20]), "=r"(v[1][21])
      : "r"(tbase + c0), "r"(tbase + c0 + 16u), "r"(tbase + c0 + 20u), "r"(tbase + c1), "r"(tbase + c1 + 16u),
        "r"(tbase + c1 + 20u));
}

// One stencil from TMEM (a 16-, a 4- and a 2-column load) and its wait.
__device__ __forceinline__ void grid_load_one(uint32_t a0, uint32_t (&v)[kGrLoadRegs]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%22];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16,%17,%18,%19}, [%23];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%20,%21}, [%24];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21])
      : "r"(a0), "r"(a0 + 16u), "r"(a0 + 20u));
}

// One direction of one lane: the W + 1 taps v (re, im interleaved) weighted by the
// lane's record (weights, then the rotation (cr, sr)), rotated and combined with the
// partner lane (the other component of the same visibility); returns this lane's
// component of the rotated sum.  sgn is -1 on the real lane (comp 0), +1 on the imaginary.
template <int W>
__device__ __forceinline__ float grid_tap_combine(const uint32_t (&v)[kGrLoadRegs], const float* rec, float sgn) {
  static_assert(W + 1 == kGrLoadCols && kGrRecWords == 16, "record layout: W + 1 weights, then cr, sr, code");
  float r[16];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float4 q = reinterpret_cast<const float4*>(rec)[i];
    r[4 * i] = q.x;
    r[4 * i + 1] = q.y;
    r[4 * i + 2] = q.z;
    r[4 * i + 3] = q.w;
  }
  // Two chains per sum (even and odd taps) halve the dependent FMA latency.
  float P0 = 0.f, P1 = 0.f, Q0 = 0.f, Q1 = 0.f;
#pragma unroll
  for (int k = 0; k <= W; ++k) {
    if (k & 1) {
      P1 = fmaf(r[k], __uint_as_float(v[2 * k]), P1);
      Q1 = fmaf(r[k], __uint_as_float(v[2 * k + 1]), Q1);
    } else {
      P0 = fmaf(r[k], __uint_as_float(v[2 * k]), P0);
      Q0 = fmaf(r[k], __uint_as_float(v[2 * k + 1]), Q0);
    }
  }
  const float P = P0 + P1, Q = Q0 + Q1;
  const float cr = r[W + 1], sr = r[W + 2];
  // Lane re: P = sum Vr ReE, Q = sum Vr ImE; lane im: P = sum Vi ReE, Q = sum Vi ImE.
  // G = (P_r - Q_i) + i (Q_r + P_i), and G (cr + i sr) has
  //   re = (P_r cr - Q_r sr) - (P_i sr + Q_i cr),  im = (P_i cr - Q_i sr) + (P_r sr + Q_r cr):
  // each lane keeps P cr - Q sr and hands P sr + Q cr to its partner (one shuffle).
  const float keep = fmaf(P, cr, -Q * sr);
  const float send = fmaf(P, sr, Q * cr);
  return fmaf(sgn, __shfl_xor_sync(0xffffffffu, send, 1), keep);
}

// A direction whose 4 timesteps need separate grid windows: one load per timestep
// (rare; kept out of line so that the common path stays small).  rec_dir is the
// direction's record at timestep 0; timestep t's is t * kGrRecDirs records further.
template <int W>
__device__ __noinline__ float grid_wide_sum(const float* rec_dir, uint32_t tbase, float sgn, int tl, int pp) {
  float acc = 0.f;
  for (int tt = 0; tt < 4; ++tt) {
    const float* r = rec_dir + tt * kGrRecDirs * kGrRecWords;
    const int ct = __float_as_int(r[kGrCodeWord]);
    if ((ct & 0xFFFF) == 0xFFFF || ((ct >> 8) & 255) != pp) continue;  // same in every lane
    uint32_t v[kGrLoadRegs];
    grid_load_one(tbase + 2u * static_cast<uint32_t>(ct & 255), v);
    const float g = grid_tap_combine<W>(v, r, sgn);
    if (tl == tt) acc += g;
  }
  return acc;
}

// The record of one (timestep, direction) for this lane's row of the tile: the W + 1
// interpolation weights of the quarter's shared stencil, the rotation at the centre
// channel, and the load code: the pass and the column of the quarter's shared load, with
// kGrWide when the 4 timesteps need loads of their own (0xFFFF in the column field for a
// row outside the data), or -1 when the direction reads nothing.  Every lane of the warp
// calls it together (the 4 timesteps of a direction exchange their stencil starts).
template <int W>
__device__ __forceinline__ void grid_record(const GridParams& p, const float (&x)[6], const float2* tab, int d,
                                            bool dv, bool rval, int n, int c0, int lbase, int r0, int npass,
                                            float* dst) {
  float ka[6], kb[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    ka[i] = __ldg(p.dirk + 12 * d + i);
    kb[i] = __ldg(p.dirk + 12 * d + 6 + i);
  }
  const uint32_t pa = df_dot3_turns_u32(ka, x);
  const uint32_t pb = df_dot3_turns_u32(kb, x);
  float f;
  const int i0 = grid_position(pb, n, f);
  const int st = grid_stencil_start(i0, f);  // this row's stencil start
  const int sl0 = rval ? st : 0x7fffffff, sh0 = rval ? st : -0x7fffffff;
  int cw = min(sl0, __shfl_xor_sync(0xffffffffu, sl0, 8));
  cw = min(cw, __shfl_xor_sync(0xffffffffu, cw, 16));
  int cm = max(sh0, __shfl_xor_sync(0xffffffffu, sh0, 8));
  cm = max(cm, __shfl_xor_sync(0xffffffffu, cm, 16));
  const bool any = cw != 0x7fffffff;
  // Normally the 4 timesteps' stencils start within one grid point of each other and
  // share one load from the earliest start; otherwise each timestep loads its own.
  const bool wide = any && cm - cw > 1;  // W + 1 taps from cw cover starts cw and cw + 1
  const int base = wide ? st : cw;
  int code = -1;
  if (dv && any) {
    if (wide && !rval) {
      code = kGrWide | 0xFFFF;
    } else {
      const int rr = base + lbase - r0;
      const int pass = npass == 1 ? 0 : rr / kGrPassStride;
      code = (wide ? kGrWide : 0) | (pass << 8) | (rr - pass * kGrPassStride);
    }
  }
  float wt[W + 1];
  grid_weights<W>(f, st - base == 1, p.wpoly, wt);  // starts differ by at most one without kGrWide
  float cr, sr;
  twiddle_turns(pa + static_cast<uint32_t>(c0) * pb, tab, cr, sr);
  static_assert(W == 10 && kGrCodeWord == 13 && kGrRecWords == 16, "record layout");
  float4* my = reinterpret_cast<float4*>(dst);
  my[0] = make_float4(wt[0], wt[1], wt[2], wt[3]);
  my[1] = make_float4(wt[4], wt[5], wt[6], wt[7]);
  my[2] = make_float4(wt[8], wt[9], wt[10], cr);
  my[3] = make_float4(sr, __int_as_float(code), 0.f, 0.f);
}

// Sum of TMEM regions into the first one, for this warp's 32 lanes and columns
// [0, ncols): dst = a (+ b) (+ c), rounded FP32 adds.
__device__ __forceinline__ void grid_fold(uint32_t lanes, uint32_t dst, uint32_t b, uint32_t c, bool use_b, bool use_c,
                                          int ncols) {
  for (int c0 = 0; c0 < ncols; c0 += 16) {
    uint32_t x[16], y[16], z[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(x[0]), "=r"(x[1]), "=r"(x[2]), "=r"(x[3]), "=r"(x[4]), "=r"(x[5]), "=r"(x[6]), "=r"(x[7]), "=r"(x[8]),
          "=r"(x[9]), "=r"(x[10]), "=r"(x[11]), "=r"(x[12]), "=r"(x[13]), "=r"(x[14]), "=r"(x[15])
        : "r"(lanes + dst + c0)
        : "memory");
    if (use_b)
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(y[0]), "=r"(y[1]), "=r"(y[2]), "=r"(y[3]), "=r"(y[4]), "=r"(y[5]), "=r"(y[6]), "=r"(y[7]), "=r"(y[8]),
            "=r"(y[9]), "=r"(y[10]), "=r"(y[11]), "=r"(y[12]), "=r"(y[13]), "=r"(y[14]), "=r"(y[15])
          : "r"(lanes + b + c0)
          : "memory");
    if (use_c)
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(z[0]), "=r"(z[1]), "=r"(z[2]), "=r"(z[3]), "=r"(z[4]), "=r"(z[5]), "=r"(z[6]), "=r"(z[7]), "=r"(z[8]),
            "=r"(z[9]), "=r"(z[10]), "=r"(z[11]), "=r"(z[12]), "=r"(z[13]), "=r"(z[14]), "=r"(z[15])
          : "r"(lanes + c + c0)
          : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      float v = __uint_as_float(x[i]);
      if (use_b) v += __uint_as_float(y[i]);
      if (use_c) v += __uint_as_float(z[i]);
      x[i] = __float_as_uint(v);
    }
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
            lanes + dst + c0),
        "r"(x[0]), "r"(x[1]), "r"(x[2]), "r"(x[3]), "r"(x[4]), "r"(x[5]), "r"(x[6]), "r"(x[7]), "r"(x[8]), "r"(x[9]),
        "r"(x[10]), "r"(x[11]), "r"(x[12]), "r"(x[13]), "r"(x[14]), "r"(x[15])
        : "memory");
  }
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// Instruction descriptor, kind::f16: D = F32, A = B = F16, both K-major, dense.
__host__ __device__ constexpr uint32_t grid_idesc_f16(int M, int N) {
  return (1u << 4) | (static_cast<uint32_t>(N >> 3) << 17) | (static_cast<uint32_t>(M >> 4) << 24);
}

// The two correction MMAs of a 16-channel chunk (lo*hi and hi*lo) into one accumulator, from
// one statement: acc0 = 0 overwrites the accumulator with the first.
__device__ __forceinline__ void grid_mma_corrections(uint32_t d, uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl,
                                                     uint32_t idesc, uint32_t acc0) {
  asm volatile(
      "{\n\t.reg .pred p, t;\n\t"
      "setp.ne.b32 p, %6, 0;\n\t"
      "setp.eq.b32 t, %6, %6;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %5, p;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %3, %4, %5, t;\n\t}" ::"r"(d),
      "l"(al), "l"(bh), "l"(ah), "l"(bl), "r"(idesc), "r"(acc0)
      : "memory");
}

// The hi*hi MMA of a chunk.
__device__ __forceinline__ void grid_mma_hihi(uint32_t d, uint64_t ah, uint64_t bh, uint32_t idesc, uint32_t acc0) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(ah), "l"(bh), "r"(idesc), "r"(acc0)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// The 4 timestep lanes of a quad lane's row (lane bits 3 and 4) each hold one value per
// direction of a batch (g[bb], direction jb + bb); sum them over the 4 timesteps and leave
// direction jb + tl's sum in timestep lane tl (a reduce-scatter: 3 shuffles for 4 directions).
__device__ __forceinline__ float grid_sum_timesteps(const float (&g)[kGrBatch], int tl) {
  static_assert(kGrBatch == 4, "one direction per timestep lane");
  const bool h = tl & 2, l = tl & 1;
  float ka = h ? g[2] : g[0], kb = h ? g[3] : g[1];
  ka += __shfl_xor_sync(0xffffffffu, h ? g[0] : g[2], 16);
  kb += __shfl_xor_sync(0xffffffffu, h ? g[1] : g[3], 16);
  return (l ? kb : ka) + __shfl_xor_sync(0xffffffffu, l ? ka : kb, 8);
}

// Store (first) or add a warp's sums to the unit's output: acc[k] is this lane's component
// of direction 4 k + tl of the warp (summed over the 4 timesteps), directions dbase .. dbase
// + nd of the item, out[direction][pol][nbl] complex doubles.  Each output element has one
// writer lane.
__device__ __forceinline__ void grid_flush(const float (&acc)[kGrWarpDirs / kGrBatch], double2* out, int dbase, int nd,
                                           int b, bool bval, int tl, int ps, int comp, int nbl, bool first) {
#pragma unroll
  for (int k = 0; k < kGrWarpDirs / kGrBatch; ++k) {
    const int j = k * kGrBatch + tl;
    if (bval && j < nd) {
      double* o = reinterpret_cast<double*>(out + (static_cast<int64_t>(dbase + j) * 4 + (ps >> 1)) * nbl + b);
      o[comp] = first ? static_cast<double>(acc[k]) : o[comp] + static_cast<double>(acc[k]);
    }
  }
}

template <int W>
__global__ void __launch_bounds__(kGrThreads, 1) rotate_average_gridded(const GridParams p) {
  extern __shared__ __align__(128) unsigned char grid_smem[];
  unsigned char* smem = grid_smem;
  unsigned char* ve = smem;                                          // [kGrStages][V then A hi | A lo | E]
  float2* tab = reinterpret_cast<float2*>(smem + kGrStages * kGrStageBytes);
  float* rec_all = reinterpret_cast<float*>(tab + kTwiddleSize);
  uint64_t* bars = reinterpret_cast<uint64_t*>(rec_all + kGrRecBytes / 4);
  uint64_t* vfull = bars;                      // [kGrMacroStages] bytes of a round's stages landed
  uint64_t* sdone = vfull + kGrMacroStages;    // [kGrMacroStages] MMAs that read it completed
  uint64_t* is_empty = sdone + kGrMacroStages;  // a middle segment was folded into RS (sdone: its MMAs completed)
  uint64_t* ac_free = is_empty + 1;             // final fold of a tile done: IS and AC reusable
  uint64_t* rs_full = ac_free + 1;             // [2] running sum final: epilogue may read
  uint64_t* rs_free = rs_full + 2;             // [2] epilogue finished reading
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kGrNumBars);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < kTwiddleSize; i += blockDim.x) tab[i] = __ldg(p.twiddle + i);
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)), "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < kGrMacroStages; ++i) {
      mbar_init(&vfull[i], 1);
      mbar_init(&sdone[i], 1);
    }
    mbar_init(is_empty, 4);
    mbar_init(ac_free, 4);
    for (int i = 0; i < 2; ++i) {
      mbar_init(&rs_full[i], 4);
      mbar_init(&rs_free[i], kGrEpiWarps);
    }
    fence_mbar_init();
    *abort_flag = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- producer ----------------
    if (lane == 0) {
      uint32_t ctr = 0;
      bool ok = true;
      for (int sl = blockIdx.x; ok; sl += gridDim.x) {
        const int u = sl < p.nslots ? __ldg(p.order + sl) : -1;
        if (u < 0) break;
        const GridUnit g = grid_unit(p, u);
        const GridItem& I = p.items[g.item];
        const GridWindow w = p.win[u];
        for (int tb = 0; tb < g.ntb && ok; ++tb)
          for (int ps = 0; ps < w.npass && ok; ++ps)
            for (int q0 = 0; q0 < I.nchunk; q0 += kGrMacro, ++ctr) {
              const int m = ctr % kGrMacroStages;
              const int nq = min(kGrMacro, I.nchunk - q0);
              if (ctr >= kGrMacroStages && !grid_wait(&sdone[m], ((ctr / kGrMacroStages) - 1) & 1, abort_flag)) {
                grid_fail(p, abort_flag);
                ok = false;
                break;
              }
              mbar_arrive_expect_tx(&vfull[m], nq * (kGrOpBytes + 4 * w.jw * 32));
              const int rg = w.rg0 + ps * (kGrPassStride / 8);
              const int tbi = g.t_lo / 4 + tb;  // the tile's timestep block in the integration
              for (int i = 0; i < nq; ++i) {
                const int q = q0 + i;
                unsigned char* st = ve + (m * kGrMacro + i) * kGrStageBytes;
                // The chunk's A operand, hi and lo, already in the MMA layout.
                bulk_copy_g2s(st, I.op + ((static_cast<int64_t>(g.quad) * I.ntb + tbi) * I.nchunk + q) * kGrOpBytes,
                              kGrOpBytes, &vfull[m]);
#pragma unroll
                for (int hl = 0; hl < 2; ++hl) {
                  // Window grid points [8 rg, 8 rg + jw): 2 jw interleaved (re, im) rows.
                  const unsigned char* src = I.etab + (static_cast<int64_t>(q * 2 + hl) * 2 * I.nrg + 2 * rg) * 256;
                  bulk_copy_g2s(st + kGrEOffset + hl * 2 * w.jw * 32, src, 2 * w.jw * 32, &vfull[m]);
                }
              }
            }
      }
      // Do not leave while copies issued by this block may still land.
      for (uint32_t j = (ctr > kGrMacroStages ? ctr - kGrMacroStages : 0); j < ctr; ++j)
        if (!mbar_wait_bounded(&vfull[j % kGrMacroStages], (j / kGrMacroStages) & 1)) atomicOr(p.err, kDevErrTimeout);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      uint32_t ctr = 0, blk = 0, mids = 0;
      bool ok = true, issued = false;
      for (int sl = blockIdx.x; ok; sl += gridDim.x) {
        const int u = sl < p.nslots ? __ldg(p.order + sl) : -1;
        if (u < 0) break;
        const GridUnit g = grid_unit(p, u);
        const GridItem& I = p.items[g.item];
        const GridWindow w = p.win[u];
        const uint32_t idesc = grid_idesc_f16(128, 2 * w.jw);
        const uint64_t adesc0 = tc_smem_desc(ve, kTcLbo, kTcSbo);
        const uint64_t edesc0 = tc_smem_desc(ve + kGrEOffset, kTcLbo, kTcSbo);
        for (int tb = 0; tb < g.ntb && ok; ++tb)
          for (int ps = 0; ps < w.npass && ok; ++ps, ++blk) {
            const uint32_t b = blk & 1;
            if ((blk >= 2 && !grid_wait(&rs_free[b], ((blk >> 1) - 1) & 1, abort_flag)) ||
                (blk >= 1 && !grid_wait(ac_free, (blk - 1) & 1, abort_flag))) {
              grid_fail(p, abort_flag);
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t rs = tmem + b * kGrRegion;
            for (int q0 = 0; q0 < I.nchunk && ok; q0 += kGrMacro, ++ctr) {
              const int m = ctr % kGrMacroStages;
              const int nq = min(kGrMacro, I.nchunk - q0);
              if (!grid_wait(&vfull[m], (ctr / kGrMacroStages) & 1, abort_flag)) {
                grid_fail(p, abort_flag);
                ok = false;
                break;
              }
              asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
              // A round is one segment.  Its correction MMAs go first: they give the fold of the
              // previous segment time to finish before the hi*hi MMAs restart IS.
              const int seg = q0 / kGrSegChunks;
              // Descriptors of stage i: A hi/lo at +0 / +kGrAHalf, E hi/lo at +0 / +2*jw*32 from their
              // bases (address field >> 4).
              const uint64_t so0 = static_cast<uint64_t>(m * kGrMacro * (kGrStageBytes >> 4));
              const uint64_t sst = static_cast<uint64_t>(kGrStageBytes >> 4);
              for (int i = 0; i < nq; ++i) {
                const uint64_t ah = adesc0 + so0 + i * sst, bh = edesc0 + so0 + i * sst;
                const uint64_t al = ah + (kGrAHalf >> 4), bl = bh + static_cast<uint64_t>(2 * w.jw * 2);
                grid_mma_corrections(tmem + kGrAC, ah, al, bh, bl, idesc, q0 + i > 0 ? 1u : 0u);
              }
              issued = true;
              if (seg >= 2 && !grid_wait(is_empty, (mids - 1) & 1, abort_flag)) {
                grid_fail(p, abort_flag);
                ok = false;
              } else {
                const uint32_t dst = seg == 0 ? rs : tmem + kGrIS;
                for (int i = 0; i < nq; ++i)
                  grid_mma_hihi(dst, adesc0 + so0 + i * sst, edesc0 + so0 + i * sst, idesc, i > 0 ? 1u : 0u);
                if (seg >= 1 && q0 + nq < I.nchunk) ++mids;  // a middle segment, folded
              }
              if (issued) tc_commit(&sdone[m]);
            }
          }
      }
      // No MMA of this block may be in flight when its TMEM is freed.
      if (issued) {
        const uint32_t j = ctr - 1;
        if (!mbar_wait_bounded(&sdone[j % kGrMacroStages], (j / kGrMacroStages) & 1)) atomicOr(p.err, kDevErrTimeout);
      }
    }
  } else if (warp < 6) {
    // ---------------- fold warps: segments and corrections into the running sums ----------------
    const uint32_t lanes = static_cast<uint32_t>((warp & 3) * 32) << 16;
    uint32_t blk = 0, rnd = 0;  // tiles (x passes) and barrier rounds (segments), as the MMA issuer counts them
    bool ok = true;
    for (int sl = blockIdx.x; ok; sl += gridDim.x) {
      const int u = sl < p.nslots ? __ldg(p.order + sl) : -1;
      if (u < 0) break;
      const GridUnit g = grid_unit(p, u);
      const GridItem& I = p.items[g.item];
      const GridWindow w = p.win[u];
      const int nseg = (I.nchunk + kGrSegChunks - 1) / kGrSegChunks;
      for (int tb = 0; tb < g.ntb && ok; ++tb)
        for (int ps = 0; ps < w.npass && ok; ++ps, ++blk, rnd += nseg) {
          const uint32_t b = blk & 1;
          // Middle segments 1 .. nseg - 2 complete in IS one after another (round rnd + sg of the
          // stage ring): each is added to RS as soon as its MMAs have completed, so that the next
          // segment can restart IS.  (Segment 0 accumulates in RS itself.)
          for (int sg = 1; sg <= nseg - 2; ++sg) {
            const uint32_t r = rnd + sg;
            if (!grid_wait(&sdone[r % kGrMacroStages], (r / kGrMacroStages) & 1, abort_flag)) {
              grid_fail(p, abort_flag);
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            grid_fold(lanes, tmem + b * kGrRegion, tmem + kGrIS, 0, true, false, 2 * w.jw);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(is_empty);
          }
          if (!ok) break;
          // Final fold: RS += last segment (if any beyond the first) + corrections.
          const uint32_t rl = rnd + nseg - 1;  // the tile's last round: every MMA of the tile completed
          if ((blk >= 2 && !grid_wait(&rs_free[b], ((blk >> 1) - 1) & 1, abort_flag)) ||
              !grid_wait(&sdone[rl % kGrMacroStages], (rl / kGrMacroStages) & 1, abort_flag)) {
            grid_fail(p, abort_flag);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          grid_fold(lanes, tmem + b * kGrRegion, tmem + kGrIS, tmem + kGrAC, nseg >= 2, true, 2 * w.jw);
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) {
            mbar_arrive(ac_free);
            mbar_arrive(&rs_full[b]);
          }
        }
    }
  } else {
    // ---------------- epilogue: interpolate, rotate, accumulate ----------------
    const int e = warp - 6;
    const int half = e >> 2;       // which kGrWarpDirs directions of the unit
    const int quarter = warp & 3;  // TMEM lanes 32*quarter .. (hardware rule: warp id mod 4)
    const int tl = lane >> 3, ps = lane & 7, comp = lane & 1;
    const float sgn = comp ? 1.f : -1.f;
    // Records of kGrRecDirs of the warp's directions at a time: record (t, j) at
    // (t * kGrRecDirs + j % kGrRecDirs) * kGrRecWords.
    float* rec = rec_all + e * (4 * kGrRecDirs * kGrRecWords);
    float* rec_t = rec + tl * kGrRecDirs * kGrRecWords;  // this lane's timestep
    uint32_t blk = 0;
    bool ok = true;
    for (int sl = blockIdx.x; ok; sl += gridDim.x) {
      const int u = sl < p.nslots ? __ldg(p.order + sl) : -1;
      if (u < 0) break;
      const GridUnit g = grid_unit(p, u);
      const GridItem& I = p.items[g.item];
      const GridWindow w = p.win[u];
      if (w.npass == 0) continue;
      const int n = 2 * I.C, c0 = I.C / 2;
      const int r0 = w.rg0 * 8;
      const int b = g.quad * 4 + quarter;
      const bool bval = b < p.nbl;
      double2* out = I.out + static_cast<int64_t>(I.nslab > 1 ? g.slab : 0) * I.ndir * 4 * p.nbl;
      // With one direction group the warp's sums stay in registers over the unit's tiles and
      // passes; with several, each (tile, pass, group) adds its sums to the unit's output in
      // order (the first stores), since every group's sums do not fit in registers.
      const bool keep = g.dg_hi - g.dg_lo == 1;
      float acc[kGrWarpDirs / kGrBatch];  // acc[k]: direction k * kGrBatch + tl, summed over timesteps
#pragma unroll
      for (int k = 0; k < kGrWarpDirs / kGrBatch; ++k) acc[k] = 0.f;
      for (int tb = 0; tb < g.ntb && ok; ++tb) {
        const int t = g.t_lo + tb * 4 + tl;
        const bool rval = bval && t < g.t_hi;
        const int64_t r = rval ? static_cast<int64_t>(t) * p.nbl + b : 0;
        // Undoes the operand's and the E table's scales of this lane's (baseline, pol).
        const float sc =
            __ldg(I.vinv + (static_cast<int64_t>(g.quad) * I.ntb + g.t_lo / 4 + tb) * 16 + quarter * 4 + (ps >> 1)) *
            I.einv;
        for (int pp = 0; pp < w.npass; ++pp, ++blk) {
          const uint32_t rb = blk & 1;
          if (!grid_wait(&rs_full[rb], (blk >> 1) & 1, abort_flag)) {
            grid_fail(p, abort_flag);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t tbase = tmem + (static_cast<uint32_t>(quarter * 32) << 16) + rb * kGrRegion;
          for (int dg = g.dg_lo; dg < g.dg_hi; ++dg) {
            const int dbase = dg * kGrDirs + half * kGrWarpDirs;  // item-relative first direction of this warp
            const int nd = max(0, min(kGrWarpDirs, I.ndir - dbase));
            if (!keep) {
#pragma unroll
              for (int k = 0; k < kGrWarpDirs / kGrBatch; ++k) acc[k] = 0.f;
            }
#pragma unroll
            for (int hr = 0; hr < kGrWarpDirs; hr += kGrRecDirs) {
              if (hr >= nd) break;  // the same in every lane
              {
                // Lane (t, ps) computes the records of directions hr + ps and hr + 8 + ps at
                // timestep t; the records past nd say "no load".  (Written as a loop, the two
                // records take fewer registers than two inlined calls: the kernel does not spill.)
                float x[6];
#pragma unroll
                for (int i = 0; i < 6; ++i) x[i] = __ldg(I.uvw_f + 6 * r + i);
                __syncwarp();
#pragma unroll 1
                for (int jj = 0; jj < 2; ++jj) {
                  const int j = hr + ps + 8 * jj;
                  grid_record<W>(p, x, tab, I.dir0 + dbase + min(j, nd - 1), j < nd, rval, n, c0, I.lbase, r0,
                                 w.npass, rec_t + (ps + 8 * jj) * kGrRecWords);
                }
                __syncwarp();
              }
#pragma unroll
              for (int jb = hr; jb < hr + kGrRecDirs; jb += kGrBatch) {
                if (jb >= nd) break;  // the same in every lane
                // The batch's directions that read this pass with one shared load (codes are the
                // same in every lane for those): loads and one wait per pair, then their sums.
                const float* rb = rec_t + (jb - hr) * kGrRecWords;
                uint32_t col[kGrBatch];
                int code[kGrBatch];
                int live = 0;
#pragma unroll
                for (int bb = 0; bb < kGrBatch; ++bb) {
                  code[bb] = __float_as_int(rb[bb * kGrRecWords + kGrCodeWord]);
                  const bool use = code[bb] >= 0 && !(code[bb] & kGrWide) && ((code[bb] >> 8) & 255) == pp;
                  col[bb] = use ? 2u * static_cast<uint32_t>(code[bb] & 255) : 0u;
                  live |= (use ? 1 : 0) << bb;
                }
                float gs[kGrBatch] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int bp = 0; bp < kGrBatch; bp += 2) {
                  if ((live >> bp) & 3) {
                    uint32_t v[2][kGrLoadRegs];
                    grid_load_pair(tbase, col[bp], col[bp + 1], v);
#pragma unroll
                    for (int bb = 0; bb < 2; ++bb) {
                      const float gsum = grid_tap_combine<W>(v[bb], rb + (bp + bb) * kGrRecWords, sgn);
                      gs[bp + bb] = ((live >> (bp + bb)) & 1) ? gsum : 0.f;
                    }
                  }
                }
#pragma unroll
                for (int bb = 0; bb < kGrBatch; ++bb)
                  if (code[bb] >= 0 && (code[bb] & kGrWide))  // the kGrWide bit is the same in every lane
                    gs[bb] += grid_wide_sum<W>(rec + (jb - hr + bb) * kGrRecWords, tbase, sgn, tl, pp);
                acc[jb / kGrBatch] = fmaf(sc, grid_sum_timesteps(gs, tl), acc[jb / kGrBatch]);
              }
            }
            if (!keep) grid_flush(acc, out, dbase, nd, b, bval, tl, ps, comp, p.nbl, tb == 0 && pp == 0);
          }
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(&rs_free[rb]);
        }
      }
      if (!ok) break;
      if (keep) {
        const int dbase = g.dg_lo * kGrDirs + half * kGrWarpDirs;
        grid_flush(acc, out, dbase, max(0, min(kGrWarpDirs, I.ndir - dbase)), b, bval, tl, ps, comp, p.nbl, true);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  }
}

}  // namespace leapgb
