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
// Comput. 41 (2019) C479).  With W = 8, beta = 2.3 W the interpolation error is
// about 1e-7 of the l2 norm of f (their rule for a 2x grid: W = log10(1/eps) + 1;
// W = 7 was measured too coarse for 16-station arrays, whose solve averages little).
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
// The product runs in 3xTF32 (V E ~ V_hi E_hi + V_lo E_hi + V_hi E_lo with hi = tf32(x),
// lo = tf32(x - hi)).  The tensor cores accumulate FP32 with truncation, whose error
// grows with the number of accumulation steps and the size of the accumulator; so the
// large hi*hi products restart in a fresh accumulator every 64 channels (a "segment")
// and the small corrections go to an accumulator of their own.  Converter warps add
// the segments together with rounded FP32 adds.  Measured on 128 antennas x 384
// channels this keeps the averages within ~5e-7 of the FP64 sums (relative to the
// sum of |terms|).
//
// TMEM (512 columns, one block per SM): RS[0], RS[1] (running sums, double
// buffered: the epilogue reads one while the next tile accumulates into the
// other), IS (segments 1.. of the current tile), AC (corrections).  Column 2j of
// a region holds sum V_s Re E at window grid point j, column 2j + 1 sum V_s Im E
// (the grid matrix interleaves its re and im rows), so the W + 1 taps of one
// stencil are 2 (W + 1) = 18 adjacent columns: a 16- and a 2-column tcgen05.ld.
//
// Operands.  The tile's visibilities reach shared memory already split into TF32 hi
// and lo parts in the MMA's canonical K-major layout: grid_split_operand builds that
// copy of an integration once (16 KB per tile and 16-channel chunk, twice the bytes of
// the visibilities), and each chunk is then one bulk copy, so no warp converts
// operands between the copy and the MMAs.
//
// Warp roles (14 warps): 0 = producer (bulk copies of the split operand and of the E
// window), 1 = MMA issuer (+ TMEM owner), 2-5 = fold warps (add the finished hi*hi
// segments and the corrections into the running sums), 6-13 = epilogue (warp w reads
// TMEM lanes 32 (w % 4) ..; two warps per quarter take 32 directions each).  One ring of
// kGrStages stages of {A hi, A lo, E window}, handed over in pairs and released by one
// MMA commit per pair.  Every wait is bounded; a timeout sets the error word, stops every
// role, and the block still waits (bounded) for its copies and MMAs and frees its TMEM.
#pragma once

#include "leap_common.cuh"
#include "kernels_tc.cuh"

namespace leapgb {

constexpr int kGrTaps = 8;            // W, grid points per interpolation
constexpr float kGrBeta = 18.4f;      // 2.3 W
constexpr int kGrChunk = 16;          // channels per stage
constexpr int kGrSegChunks = 4;       // chunks per hi*hi accumulation segment (64 channels)
constexpr int kGrStages = 6;          // {visibility box / A hi, A lo, E window} ring
constexpr int kGrMacro = 2;           // chunks handed over per barrier round (stages go in pairs)
constexpr int kGrMacroStages = kGrStages / kGrMacro;
constexpr int kGrJwMax = 64;          // grid points per pass (MMA N = 2 Jw <= 128)
constexpr int kGrPassStride = 56;     // grid points between pass windows (multiple of 8)
constexpr int kGrLoadCols = 9;        // grid points one interpolation load reads (2 TMEM columns each)
constexpr int kGrBatch = 4;           // directions whose loads share one tcgen05.wait::ld
constexpr int kGrDirs = 64;           // directions per unit (8 epilogue warps x 32 / 4 quarters)
constexpr int kGrEpiWarps = 8;
constexpr int kGrWarpDirs = kGrDirs * 4 / kGrEpiWarps;  // directions per epilogue warp
constexpr int kGrWarps = 6 + kGrEpiWarps;
constexpr int kGrThreads = kGrWarps * 32;
constexpr int kGrVBytes = 32 * 4 * kGrChunk * 4;         // one chunk of a tile: 16 ch x 4 t x 32 floats
constexpr int kGrEBytes = 2 * 2 * 2 * kGrJwMax * 32;     // [hl][ks][2 Jw rows x 32 B]
constexpr int kGrAHalf = 2 * 128 * 32;                   // one split of A: [ks][128 rows x 32 B]
static_assert(kGrAHalf == kGrVBytes, "one split of A holds one chunk of a tile");
// Stage: [A hi][A lo][E]
constexpr int kGrStageBytes = kGrVBytes + kGrAHalf + kGrEBytes;
constexpr int kGrEOffset = kGrVBytes + kGrAHalf;
constexpr int kGrRecWords = 12;                          // per (direction, timestep) record: 3 16-byte rows
constexpr int kGrRecBytes = kGrEpiWarps * 32 * kGrRecWords * 4;  // [warps][4 t][8 dirs][12]
constexpr uint32_t kGrRegion = 128;                      // TMEM columns per region
constexpr uint32_t kGrIS = 2 * kGrRegion, kGrAC = 3 * kGrRegion;
constexpr int kGrWide = 1 << 16;                         // record flag: the 4 timesteps need separate loads
constexpr int kGrNumBars = 2 * kGrMacroStages + 8;

// A pass window must hold every stencil whose start falls in its stride, plus the
// columns one load reads past the stencil.
static_assert(kGrPassStride % 8 == 0 && kGrPassStride - 1 + kGrLoadCols <= kGrJwMax, "pass windows");
static_assert(kGrTaps + 1 <= kGrLoadCols, "one load per stencil");

__host__ __device__ constexpr int grid_smem_bytes() {
  return kGrStages * kGrStageBytes + kTwiddleSize * 8 + kGrRecBytes + kGrNumBars * 8 + 16;
}

// Rows of the E table of channel count C: row r is grid point l = r - lbase.
__host__ __device__ constexpr int grid_lbase(int C) { return ((C + kGrTaps + 8 + 7) / 8) * 8; }
__host__ __device__ constexpr int grid_rows(int C) { return ((grid_lbase(C) + C + kGrJwMax + 8 + 7) / 8) * 8; }
__host__ __device__ constexpr int grid_chunks(int C) { return (C + kGrChunk - 1) / kGrChunk; }
// Floats of the E table: [chunk][ks][hl][row group][8 rows x 8 k], rows 2 l + (0: re, 1: im) of grid
// point l (relative to -lbase).
__host__ __device__ constexpr int64_t grid_table_floats(int C) {
  return static_cast<int64_t>(grid_chunks(C)) * 2 * 2 * 2 * grid_rows(C) * 8;
}

// Split grid operand of an integration: per (quad, timestep block, 16-channel chunk) the
// tile's visibilities as TF32 hi and lo parts in the MMA's canonical K-major layout,
// [hi: 2 k-steps x 16 row groups x 2 k-halves x 8 rows x 16 B][lo: the same], 16 KB,
// exactly what the shared-memory stage holds before the MMAs of a chunk.
constexpr int kGrOpBytes = 2 * 2 * 128 * 32;  // hi + lo blocks of one chunk of one tile
__host__ __device__ constexpr int64_t grid_operand_bytes(int nbl, int T, int C) {
  return static_cast<int64_t>((nbl + 3) / 4) * ((T + 3) / 4) * ((C + 15) / 16) * kGrOpBytes;
}

// Builds the split grid operand of a 4-pol complex<float> integration [C][rows][8 floats]:
// one 128-thread block per (chunk, timestep block, quad); warp w takes timestep w of the
// block and lane = 8 q + 2 p + s, the baseline q of the quad, pol p, (re, im) s.  Rows and
// channels past the integration are zero, as a tensor-map load fills them.  hi is the
// visibility rounded to TF32, lo the remainder rounded to TF32.
static __global__ void __launch_bounds__(128) grid_split_operand(const float* __restrict__ vis, int64_t rows, int nbl,
                                                                 int T, int C, int ntb, float* __restrict__ out) {
  const int q = blockIdx.x, tb = blockIdx.y, chunk = blockIdx.z;
  const int lane = threadIdx.x & 31, tl = threadIdx.x >> 5;
  const int t = tb * 4 + tl, b = q * 4 + (lane >> 3);
  const bool rv = t < T && b < nbl;
  const int64_t row = static_cast<int64_t>(t) * nbl + b;
  unsigned char* dst = reinterpret_cast<unsigned char*>(out) +
                       ((static_cast<int64_t>(q) * ntb + tb) * gridDim.z + chunk) * kGrOpBytes;
  const int mrow = (lane >> 3) * 32 + tl * 8 + (lane & 7);  // TMEM lane: baseline, timestep, pol, re/im
#pragma unroll
  for (int cg = 0; cg < 4; ++cg) {
    float x[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = chunk * kGrChunk + cg * 4 + j;
      x[j] = (rv && c < C) ? __ldg(vis + (static_cast<int64_t>(c) * rows + row) * 8 + (lane & 7)) : 0.f;
    }
    float4 hi, lo;
    hi.x = to_tf32(x[0]);
    hi.y = to_tf32(x[1]);
    hi.z = to_tf32(x[2]);
    hi.w = to_tf32(x[3]);
    lo.x = to_tf32(x[0] - hi.x);
    lo.y = to_tf32(x[1] - hi.y);
    lo.z = to_tf32(x[2] - hi.z);
    lo.w = to_tf32(x[3] - hi.w);
    const int k = cg * 4;
    const int off = (k >> 3) * 4096 + (((mrow >> 3) << 1) + ((k >> 2) & 1)) * 128 + (mrow & 7) * 16;
    *reinterpret_cast<float4*>(dst + off) = hi;
    *reinterpret_cast<float4*>(dst + kGrAHalf + off) = lo;
  }
}

// One item of a gridded launch (device memory).
struct alignas(16) GridItem {
  const float* op;       // split grid operand: [quad][timestep block][chunk][kGrOpBytes]
  const float* uvw_f;    // [rows][6] split UVWs
  const float* etab;     // E table of this channel count
  double2* out;          // nslab == 1: avg + dir0*4*nbl; else this item's [nslab][ndir][4][nbl] partials
  int32_t T, C, nchunk, tb_per_slab;
  int32_t nslab, nquad, dgroups, dir0;
  int32_t ndir, unit_begin, nrg, lbase;
  int32_t udg, uparts;   // direction groups per unit, units per (quad, slab): ceil(dgroups / udg)
  int32_t ntb, pad_;     // timestep blocks of the integration (the operand's second dimension)
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

// Per unit: the range of interpolation stencil starts over its valid rows and
// directions, as a window of E-table rows (one warp per unit).
static __global__ void grid_windows(const GridParams p) {
  const int u = static_cast<int>((blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (u >= p.units) return;
  const GridUnit g = grid_unit(p, u);
  const GridItem& I = p.items[g.item];
  const int n = 2 * I.C;
  int smin = 0x7fffffff, smax = -0x7fffffff;
  // Every direction group of the item: lanes hold the slopes of directions lane and
  // lane + 32 of the group and walk the unit's rows; a row's UVWs are one broadcast load.
  static_assert(kGrDirs == 64, "two directions per lane");
  for (int dg = g.dg_lo; dg < g.dg_hi; ++dg) {
    const int nd = min(kGrDirs, I.ndir - dg * kGrDirs);
    float kb[2][6];
    bool has[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int dj = lane + 32 * h;
      has[h] = dj < nd;
      const int d = I.dir0 + dg * kGrDirs + min(dj, nd - 1);
#pragma unroll
      for (int i = 0; i < 6; ++i) kb[h][i] = __ldg(p.dirk + 12 * d + 6 + i);
    }
    for (int t = g.t_lo; t < g.t_hi; ++t) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int b = g.quad * 4 + q;
        if (b >= p.nbl) continue;
        const int64_t r = static_cast<int64_t>(t) * p.nbl + b;
        float x[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) x[i] = __ldg(I.uvw_f + 6 * r + i);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (!has[h]) continue;
          float f;
          const int i0 = grid_position(df_dot3_turns_u32(kb[h], x), n, f);
          const int s = grid_stencil_start(i0, f);
          smin = min(smin, s);
          smax = max(smax, s);
        }
      }
    }
  }
  smin = __reduce_min_sync(0xffffffffu, smin);
  smax = __reduce_max_sync(0xffffffffu, smax);
  if (lane == 0) {
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

template <int W>
__device__ __forceinline__ void grid_weights(float y, float (&w)[W + 1]) {
  constexpr float kInvHalf = 2.0f / W;
  constexpr float kBeta2 = kGrBeta * 1.4426950408889634f;  // beta / ln 2
#pragma unroll
  for (int k = 0; k <= W; ++k) {
    // sqrt(1 - z^2) - 1 = -z^2 / (1 + sqrt(1 - z^2)): no cancellation near the centre.
    // Hardware reciprocal square root and exp2 (~2 ulp): weight error below 1e-7 of the
    // largest weight.
    const float z = (y - static_cast<float>(k)) * kInvHalf;
    const float z2 = z * z;
    const float q = fmaxf(1e-30f, 1.0f - z2);
    const float v = exp2f(-kBeta2 * __fdividef(z2, fmaf(q, rsqrtf(q), 1.0f)));
    w[k] = z2 < 1.0f ? v : 0.0f;  // psi vanishes outside its support (the load's spare tap)
  }
}

// kGrBatch directions' stencils from TMEM: a 16- and a 2-column load each (the W + 1
// taps, re and im interleaved) at columns col[b] of this warp's lanes, and one wait for all.
__device__ __forceinline__ void grid_load_batch(uint32_t tbase, const uint32_t (&col)[kGrBatch],
                                                uint32_t (&v)[kGrBatch][18]) {
  static_assert(kGrBatch == 4 && kGrLoadCols == 9, "four 18-column loads per batch");
  // All loads and the wait in one statement: the results are defined only after the wait.
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%72];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%16,%17}, [%73];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33}, [%74];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%34,%35}, [%75];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51}, [%76];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%52,%53}, [%77];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%54,%55,%56,%57,%58,%59,%60,%61,%62,%63,%64,%65,%66,%67,%68,%69}, [%78];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%70,%71}, [%79];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(v[0][0]), "=r"(v[0][1]), "=r"(v[0][2]), "=r"(v[0][3]), "=r"(v[0][4]), "=r"(v[0][5]), "=r"(v[0][6]),
        "=r"(v[0][7]), "=r"(v[0][8]), "=r"(v[0][9]), "=r"(v[0][10]), "=r"(v[0][11]), "=r"(v[0][12]), "=r"(v[0][13]),
        "=r"(v[0][14]), "=r"(v[0][15]), "=r"(v[0][16]), "=r"(v[0][17]),
        "=r"(v[1][0]), "=r"(v[1][1]), "=r"(v[1][2]), "=r"(v[1][3]), "=r"(v[1][4]), "=r"(v[1][5]), "=r"(v[1][6]),
        "=r"(v[1][7]), "=r"(v[1][8]), "=r"(v[1][9]), "=r"(v[1][10]), "=r"(v[1][11]), "=r"(v[1][12]), "=r"(v[1][13]),
        "=r"(v[1][14]), "=r"(v[1][15]), "=r"(v[1][16]), "=r"(v[1][17]),
        "=r"(v[2][0]), "=r"(v[2][1]), "=r"(v[2][2]), "=r"(v[2][3]), "=r"(v[2][4]), "=r"(v[2][5]), "=r"(v[2][6]),
        "=r"(v[2][7]), "=r"(v[2][8]), "=r"(v[2][9]), "=r"(v[2][10]), "=r"(v[2][11]), "=r"(v[2][12]), "=r"(v[2][13]),
        "=r"(v[2][14]), "=r"(v[2][15]), "=r"(v[2][16]), "=r"(v[2][17]),
        "=r"(v[3][0]), "=r"(v[3][1]), "=r"(v[3][2]), "=r"(v[3][3]), "=r"(v[3][4]), "=r"(v[3][5]), "=r"(v[3][6]),
        "=r"(v[3][7]), "=r"(v[3][8]), "=r"(v[3][9]), "=r"(v[3][10]), "=r"(v[3][11]), "=r"(v[3][12]), "=r"(v[3][13]),
        "=r"(v[3][14]), "=r"(v[3][15]), "=r"(v[3][16]), "=r"(v[3][17])
      : "r"(tbase + col[0]), "r"(tbase + col[0] + 16u), "r"(tbase + col[1]), "r"(tbase + col[1] + 16u),
        "r"(tbase + col[2]), "r"(tbase + col[2] + 16u), "r"(tbase + col[3]), "r"(tbase + col[3] + 16u));
}

// One direction of one lane: the W + 1 taps v (re, im interleaved) weighted by the
// lane's record (weights, then the rotation (cr, sr)), combined with the partner
// lane's component, rotated; returns this lane's component of the rotated sum.
template <int W>
__device__ __forceinline__ float grid_tap_combine(const uint32_t (&v)[18], const float* rec, int comp) {
  static_assert(W + 1 == 9, "record layout: 9 weights, then cr, sr, code");
  const float4 q0 = reinterpret_cast<const float4*>(rec)[0], q1 = reinterpret_cast<const float4*>(rec)[1];
  const float4 q2 = reinterpret_cast<const float4*>(rec)[2];
  const float2 rot = make_float2(q2.y, q2.z);
  const float w[9] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x};
  float P = 0.f, Q = 0.f;
#pragma unroll
  for (int k = 0; k <= W; ++k) {
    P = fmaf(w[k], __uint_as_float(v[2 * k]), P);
    Q = fmaf(w[k], __uint_as_float(v[2 * k + 1]), Q);
  }
  // Lane re (comp 0): P = sum Vr ReE, Q = sum Vr ImE; lane im: P = sum Vi ReE, Q = sum Vi ImE.
  // G = (P_re - Q_im) + i (Q_re + P_im); the lane's component of G * (cr + i sr).
  const float o = __shfl_xor_sync(0xffffffffu, Q, 1);
  const float gown = comp ? (o + P) : (P - o);
  const float o2 = __shfl_xor_sync(0xffffffffu, gown, 1);
  return comp ? fmaf(o2, rot.y, gown * rot.x) : fmaf(-o2, rot.y, gown * rot.x);
}

// A direction whose 4 timesteps need separate grid windows: one load per timestep
// (rare; kept out of line so that the common path stays small).
template <int W>
__device__ __noinline__ float grid_wide_sum(const float* rec_dir, uint32_t tbase, int comp, int tl, int pp) {
  float acc = 0.f;
  for (int tt = 0; tt < 4; ++tt) {
    const float* r = rec_dir + tt * 8 * kGrRecWords;
    const int ct = __float_as_int(r[11]);
    if ((ct & 0xFFFF) == 0xFFFF || ((ct >> 8) & 255) != pp) continue;  // same in every lane
    uint32_t v[18];
    const uint32_t a0 = tbase + 2u * static_cast<uint32_t>(ct & 255);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%18];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%16,%17}, [%19];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17])
        : "r"(a0), "r"(a0 + 16u));
    const float g = grid_tap_combine<W>(v, r, comp);
    if (tl == tt) acc += g;
  }
  return acc;
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

// The four correction MMAs of a 16-channel chunk (lo*hi and hi*lo of both k-steps) into one
// accumulator, from one statement: acc0 = 0 overwrites the accumulator with the first.
__device__ __forceinline__ void grid_mma_corrections(uint32_t d, uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl,
                                                     uint64_t ka, uint64_t kb, uint32_t idesc, uint32_t acc0) {
  asm volatile(
      "{\n\t.reg .pred p, t;\n\t"
      "setp.ne.b32 p, %9, 0;\n\t"
      "setp.eq.b32 t, %9, %9;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %8, p;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %3, %4, %8, t;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %5, %6, %8, t;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %7, %10, %8, t;\n\t}" ::"r"(d),
      "l"(al), "l"(bh), "l"(ah), "l"(bl), "l"(al + ka), "l"(bh + kb), "l"(ah + ka), "r"(idesc), "r"(acc0), "l"(bl + kb)
      : "memory");
}

// The two hi*hi MMAs (both k-steps) of a chunk.
__device__ __forceinline__ void grid_mma_hihi(uint32_t d, uint64_t ah, uint64_t bh, uint64_t ka, uint64_t kb,
                                              uint32_t idesc, uint32_t acc0) {
  asm volatile(
      "{\n\t.reg .pred p, t;\n\t"
      "setp.ne.b32 p, %6, 0;\n\t"
      "setp.eq.b32 t, %6, %6;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %5, p;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %3, %4, %5, t;\n\t}" ::"r"(d),
      "l"(ah), "l"(bh), "l"(ah + ka), "l"(bh + kb), "r"(idesc), "r"(acc0)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Sum a warp's per-lane sums over the 4 timesteps of its quad lanes and store them
// (first) or add them to the unit's output: directions dbase .. dbase + nd of the item,
// out[direction][pol][nbl] complex doubles.  Each output element has one writer lane.
__device__ __forceinline__ void grid_flush(const float (&acc)[kGrWarpDirs], double2* out, int dbase, int nd, int b,
                                           bool bval, int tl, int ps, int comp, int nbl, bool first) {
#pragma unroll
  for (int j = 0; j < kGrWarpDirs; ++j) {
    float v = acc[j] + __shfl_xor_sync(0xffffffffu, acc[j], 8);
    v += __shfl_xor_sync(0xffffffffu, v, 16);
    if (tl == 0 && bval && j < nd) {
      double* o = reinterpret_cast<double*>(out + (static_cast<int64_t>(dbase + j) * 4 + (ps >> 1)) * nbl + b);
      o[comp] = first ? static_cast<double>(v) : o[comp] + static_cast<double>(v);
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
  uint64_t* vfull = bars;                      // [kGrMacroStages] bytes of a stage pair landed
  uint64_t* sdone = vfull + kGrMacroStages;    // [kGrMacroStages] MMAs that read it completed
  uint64_t* is_full = sdone + kGrMacroStages;  // a middle segment is complete in IS
  uint64_t* is_empty = is_full + 1;            // ... and was folded into RS
  uint64_t* blk_full = is_empty + 1;           // every MMA of a tile completed
  uint64_t* ac_free = blk_full + 1;            // final fold of a tile done: IS and AC reusable
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
    mbar_init(is_full, 1);
    mbar_init(is_empty, 4);
    mbar_init(blk_full, 1);
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
              mbar_arrive_expect_tx(&vfull[m], nq * (kGrOpBytes + 8 * w.jw * 32));
              const int rg = w.rg0 + ps * (kGrPassStride / 8);
              const int tbi = g.t_lo / 4 + tb;  // the tile's timestep block in the integration
              for (int i = 0; i < nq; ++i) {
                const int q = q0 + i;
                unsigned char* st = ve + (m * kGrMacro + i) * kGrStageBytes;
                // The chunk's A operand, hi and lo, already in the MMA layout.
                bulk_copy_g2s(st, reinterpret_cast<const unsigned char*>(I.op) +
                                      ((static_cast<int64_t>(g.quad) * I.ntb + tbi) * I.nchunk + q) * kGrOpBytes,
                              kGrOpBytes, &vfull[m]);
#pragma unroll
                for (int ks = 0; ks < 2; ++ks)
#pragma unroll
                  for (int hl = 0; hl < 2; ++hl) {
                    // Window grid points [8 rg, 8 rg + jw): 2 jw interleaved (re, im) rows.
                    const float* src = I.etab + (static_cast<int64_t>((q * 2 + ks) * 2 + hl) * 2 * I.nrg + 2 * rg) * 64;
                    bulk_copy_g2s(st + kGrEOffset + (hl * 2 + ks) * 2 * w.jw * 32, src, 2 * w.jw * 32, &vfull[m]);
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
        const uint32_t idesc = tc_idesc_tf32(128, 2 * w.jw);
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
              for (int i = 0; i < nq; ++i) {
                const int q = q0 + i;
                const int seg = q / kGrSegChunks, qs = q % kGrSegChunks;
                // Descriptors of this stage: A hi/lo at +0 / +2*4096, E hi/lo at +0 / +4*jw*32 from
                // their bases; k-step 1 is 4096 (A) or 2*jw*32 (E) bytes further (address field >> 4).
                const uint64_t so = static_cast<uint64_t>((m * kGrMacro + i) * (kGrStageBytes >> 4));
                const uint64_t ah = adesc0 + so, bh = edesc0 + so;
                const uint64_t al = ah + (2 * 4096 >> 4), bl = bh + static_cast<uint64_t>(4 * w.jw * 2);
                const uint64_t ka = 4096 >> 4, kb = static_cast<uint64_t>(2 * w.jw * 2);
                // Corrections first: they give the fold of the previous segment time to finish.
                grid_mma_corrections(tmem + kGrAC, ah, al, bh, bl, ka, kb, idesc, q > 0 ? 1u : 0u);
                if (seg >= 2 && qs == 0 && !grid_wait(is_empty, (mids - 1) & 1, abort_flag)) {
                  grid_fail(p, abort_flag);
                  ok = false;
                  break;
                }
                const uint32_t dst = seg == 0 ? rs : tmem + kGrIS;
                grid_mma_hihi(dst, ah, bh, ka, kb, idesc, qs > 0 ? 1u : 0u);
                issued = true;
                if (seg >= 1 && qs == kGrSegChunks - 1 && q != I.nchunk - 1) {
                  tc_commit(is_full);  // a middle segment, folded by the converters
                  ++mids;
                }
              }
              if (issued) tc_commit(&sdone[m]);
            }
            if (ok) tc_commit(blk_full);
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
    uint32_t blk = 0, mids = 0;
    bool ok = true;
    for (int sl = blockIdx.x; ok; sl += gridDim.x) {
      const int u = sl < p.nslots ? __ldg(p.order + sl) : -1;
      if (u < 0) break;
      const GridUnit g = grid_unit(p, u);
      const GridItem& I = p.items[g.item];
      const GridWindow w = p.win[u];
      const int nseg = (I.nchunk + kGrSegChunks - 1) / kGrSegChunks;
      for (int tb = 0; tb < g.ntb && ok; ++tb)
        for (int ps = 0; ps < w.npass && ok; ++ps, ++blk) {
          const uint32_t b = blk & 1;
          // Middle segments 1 .. nseg - 2 complete in IS one after another: each is added to RS
          // as soon as its MMAs have completed, so that the next segment can restart IS.
          for (int sg = 1; sg <= nseg - 2; ++sg) {
            if (!grid_wait(is_full, mids & 1, abort_flag)) {
              grid_fail(p, abort_flag);
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            grid_fold(lanes, tmem + b * kGrRegion, tmem + kGrIS, 0, true, false, 2 * w.jw);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(is_empty);
            ++mids;
          }
          if (!ok) break;
          // Final fold: RS += last segment (if any beyond the first) + corrections.
          if ((blk >= 2 && !grid_wait(&rs_free[b], ((blk >> 1) - 1) & 1, abort_flag)) ||
              !grid_wait(blk_full, blk & 1, abort_flag)) {
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
    float* rec = rec_all + e * (32 * kGrRecWords);  // record (t, direction jj) at (8 t + jj) * kGrRecWords
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
      float acc[kGrWarpDirs];
#pragma unroll
      for (int j = 0; j < kGrWarpDirs; ++j) acc[j] = 0.f;
      for (int tb = 0; tb < g.ntb && ok; ++tb) {
        const int t = g.t_lo + tb * 4 + tl;
        const bool rval = bval && t < g.t_hi;
        const int64_t r = rval ? static_cast<int64_t>(t) * p.nbl + b : 0;
        float x[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) x[i] = __ldg(I.uvw_f + 6 * r + i);
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
            for (int j = 0; j < kGrWarpDirs; ++j) acc[j] = 0.f;
          }
#pragma unroll
          for (int gi = 0; gi < kGrWarpDirs / 8; ++gi) {
            if (gi * 8 >= nd) break;
            {
              // This lane's record: direction gi*8 + ps at timestep tl.
              const int dj = gi * 8 + ps;
              const bool dv = dj < nd;
              const int d = I.dir0 + dbase + min(dj, nd - 1);
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
                  const int rr = base + I.lbase - r0;
                  const int pass = w.npass == 1 ? 0 : rr / kGrPassStride;
                  code = (wide ? kGrWide : 0) | (pass << 8) | (rr - pass * kGrPassStride);
                }
              }
              float wt[W + 1];
              grid_weights<W>(any ? static_cast<float>(i0 - base) + f : 0.f, wt);
              float cr, sr;
              twiddle_turns(pa + static_cast<uint32_t>(c0) * pb, tab, cr, sr);
              // Record: weights 0-8, then cr, sr, code.
              float4* my = reinterpret_cast<float4*>(rec + (tl * 8 + ps) * kGrRecWords);
              my[0] = make_float4(wt[0], wt[1], wt[2], wt[3]);
              my[1] = make_float4(wt[4], wt[5], wt[6], wt[7]);
              my[2] = make_float4(wt[8], cr, sr, __int_as_float(code));
            }
            __syncwarp();
#pragma unroll
            for (int jb = 0; jb < 8; jb += kGrBatch) {
              // The batch's directions that read this pass with one shared load (codes are the
              // same in every lane for those): their loads, one wait, then their sums.
              uint32_t col[kGrBatch];
              int live = 0;
#pragma unroll
              for (int bb = 0; bb < kGrBatch; ++bb) {
                const int code = __float_as_int(rec[(tl * 8 + jb + bb) * kGrRecWords + 11]);
                const bool use = code >= 0 && !(code & kGrWide) && ((code >> 8) & 255) == pp;
                col[bb] = use ? 2u * static_cast<uint32_t>(code & 255) : 0u;
                live |= (use ? 1 : 0) << bb;
              }
              if (live) {
                uint32_t v[kGrBatch][18];
                grid_load_batch(tbase, col, v);
#pragma unroll
                for (int bb = 0; bb < kGrBatch; ++bb)
                  if (live & (1 << bb))
                    acc[gi * 8 + jb + bb] += grid_tap_combine<W>(v[bb], rec + (tl * 8 + jb + bb) * kGrRecWords, comp);
              }
#pragma unroll
              for (int bb = 0; bb < kGrBatch; ++bb) {
                const int code = __float_as_int(rec[(tl * 8 + jb + bb) * kGrRecWords + 11]);
                if (code >= 0 && (code & kGrWide))  // the kGrWide bit is the same in every lane
                  acc[gi * 8 + jb + bb] += grid_wide_sum<W>(rec + (jb + bb) * kGrRecWords, tbase, comp, tl, pp);
              }
            }
            __syncwarp();
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
