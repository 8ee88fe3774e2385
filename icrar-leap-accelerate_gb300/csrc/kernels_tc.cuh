// Ad contraction on the 5th-generation tensor cores (tcgen05, sm_103a).
//
//   partial[kb][d][s] = sum_{k in K block kb} Ad[s][k] * dphi[d][k]
//
// as D[m=s][n=d] += A[m][k] * B[n][k] with both operands K-major in shared
// memory and the accumulator in tensor memory.  FP32 precision from TF32
// units ("3xTF32"): every operand is split into hi = tf32(x) and
// lo = tf32(x - hi), and the block issues hi*hi + hi*lo + lo*hi into the same
// FP32 accumulator (the lo*lo term is below 2^-22 relative).
//
// Operand layout ("canonical" K-major, no swizzle): a block of R rows x 64 k
// is cut into core matrices of 8 rows x 4 elements (16 bytes per row, 128
// bytes each).  The block is 8 k-steps of 8 elements; k-step ks starts at byte
// ks*R*32 and holds its 2 x R/8 core matrices with the two k halves of a row
// group side by side: core (g = row/8, j = (k/4)&1) at (2g + j)*128.  So the
// leading byte offset (next core matrix along k) is 128 and the stride byte
// offset (next 8-row group) is 256.  Every byte one MMA can address under
// either reading of those two fields lies inside its own k-step slab.  Ad is
// packed this way once per metadata upload, dphi once per call; a CTA moves
// its two blocks in with plain bulk copies.
//
// One CTA = one (128-row M tile, N-column tile, run of 64-k blocks); 128
// threads.  Warp 0 allocates (and finally frees) N TMEM columns; thread 0
// streams the run through a ring of half-block stages (4 k-steps: the hi and
// lo halves of both operands, four bulk copies), issues 12 MMAs (4 k-steps x
// 3) per stage and commits them to the stage's mbarrier, and refills a stage
// once its MMAs have completed while the next stage's MMAs run; the four warps
// then read their 32 accumulator rows (TMEM lanes) with tcgen05.ld and write
// FP64 partial sums.  Waits are bounded: on a timeout the CTA sets the error
// word, still waits (bounded) for its copies and MMAs, frees its TMEM and
// returns.
#pragma once

#include "leap_common.cuh"

namespace leapgb {

constexpr int kTcM = 128;   // rows of an M tile (stations)
constexpr int kTcKB = 64;   // k per block
constexpr int kTcBlockBytesA = kTcM * kTcKB * 4;  // one split (hi or lo) of an A block

__host__ __device__ constexpr int tc_block_bytes(int rows) { return rows * kTcKB * 4; }

// Byte offset of element (row r, k) inside one packed block of R rows.
__host__ __device__ inline int tc_packed_offset(int r, int k, int R) {
  return (k >> 3) * (R * 32) + (((r >> 3) << 1) + ((k >> 2) & 1)) * 128 + (r & 7) * 16 + (k & 3) * 4;
}
constexpr uint32_t kTcLbo = 128;  // next core matrix along k
constexpr uint32_t kTcSbo = 256;  // next group of 8 rows

__device__ __forceinline__ float to_tf32(float x) {
  uint32_t y;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(y) : "f"(x));
  return __uint_as_float(y);
}

// Pack a [rows][K] operand (row stride ld, element (r, k) at src[r*ld + k]) into
// [row tile][k block][hi, lo][packed block] with R rows per tile (zero padded).
template <typename T>
__global__ void tc_pack_operand(const T* __restrict__ src, int rows, int K, int64_t ld, int R, int row_tiles,
                                int kblocks, float* __restrict__ dst) {
  const int64_t total = static_cast<int64_t>(row_tiles) * R * kblocks * kTcKB;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int k = static_cast<int>(i % (static_cast<int64_t>(kblocks) * kTcKB));
    const int r = static_cast<int>(i / (static_cast<int64_t>(kblocks) * kTcKB));
    const int tile = r / R, rr = r % R, kb = k / kTcKB, kk = k % kTcKB;
    const float x = (r < rows && k < K) ? static_cast<float>(src[static_cast<int64_t>(r) * ld + k]) : 0.f;
    const float hi = to_tf32(x);
    const float lo = to_tf32(x - hi);
    float* blk = dst + (static_cast<int64_t>(tile) * kblocks + kb) * 2 * (static_cast<int64_t>(R) * kTcKB);
    const int off = tc_packed_offset(rr, kk, R) / 4;
    blk[off] = hi;
    blk[static_cast<int64_t>(R) * kTcKB + off] = lo;
  }
}

// Ad is stored column-major S x K (element (s, k) at s + S*k): rows are s with
// row stride 1 and k stride S.  Pack it with an explicit k stride.
static __global__ void tc_pack_ad(const double* __restrict__ Ad, int S, int K, int row_tiles, int kblocks,
                           float* __restrict__ dst) {
  const int R = kTcM;
  const int64_t total = static_cast<int64_t>(row_tiles) * R * kblocks * kTcKB;
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int r = static_cast<int>(i % (static_cast<int64_t>(row_tiles) * R));  // s fastest: coalesced reads
    const int k = static_cast<int>(i / (static_cast<int64_t>(row_tiles) * R));
    const int tile = r / R, rr = r % R, kb = k / kTcKB, kk = k % kTcKB;
    const float x = (r < S && k < K) ? static_cast<float>(Ad[r + static_cast<int64_t>(S) * k]) : 0.f;
    const float hi = to_tf32(x);
    const float lo = to_tf32(x - hi);
    float* blk = dst + (static_cast<int64_t>(tile) * kblocks + kb) * 2 * (static_cast<int64_t>(R) * kTcKB);
    const int off = tc_packed_offset(rr, kk, R) / 4;
    blk[off] = hi;
    blk[static_cast<int64_t>(R) * kTcKB + off] = lo;
  }
}

__device__ __forceinline__ uint64_t tc_smem_desc(const void* p, uint32_t lbo, uint32_t sbo) {
  const uint64_t a = (smem_u32(p) >> 4) & 0x3FFFu;
  return a | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) | (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) |
         (1ull << 46);  // descriptor version 1 (sm_100 family); base offset 0; no swizzle
}

// Instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major, dense.
__host__ __device__ constexpr uint32_t tc_idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(N >> 3) << 17) | (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma_tf32(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}

// Ring of the Ad contraction: stages of half a K block (4 k-steps of 8), sized so that the ring
// holds about 192 KB of operands whatever N.
template <int N>
__host__ __device__ constexpr int tc_half_bytes() { return 2 * (kTcM + N) * (kTcKB / 2) * 4; }  // A, B: hi + lo
template <int N>
__host__ __device__ constexpr int tc_stages() { return N >= 256 ? 2 : (N >= 128 ? 3 : 4); }

// N columns of FP32 accumulator per CTA; N is a multiple of 16 in [16, 256].
// CTA (mt, nt, kc) accumulates K blocks [kc*kb_per_cta, ...) in TMEM through a ring of
// tc_stages<N>() half-block stages: thread 0 keeps the copies of the next stages in flight
// while the MMAs of the current one run (a stage is refilled once the MMAs that read it
// have completed), then the four warps write partial[kc][d][s].
template <int N>
__global__ void __launch_bounds__(128, 1) tc_gemm_ad(const float* __restrict__ A_packed, const float* __restrict__ B_packed,
                                                     int S, int D, int kblocks, int kb_per_cta,
                                                     double* __restrict__ partial, int* __restrict__ err) {
  static_assert(N % 16 == 0 && N >= 16 && N <= 256, "N tile");
  constexpr int kCols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));  // power of two >= 32
  constexpr int kBlockA = tc_block_bytes(kTcM), kBlockB = tc_block_bytes(N);  // one split (hi or lo) of a block
  constexpr int kHalfA = kBlockA / 2, kHalfB = kBlockB / 2;                   // 4 of its 8 k-step slabs
  constexpr int kStage = tc_half_bytes<N>(), kStages = tc_stages<N>();
  static_assert(kStage == 2 * kHalfA + 2 * kHalfB, "stage layout: [A hi][A lo][B hi][B lo]");
  extern __shared__ __align__(128) unsigned char tc_smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(tc_smem + kStages * kStage);  // [kStages] copies landed
  uint64_t* empty = full + kStages;                                          // [kStages] MMAs that read it done
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(empty + kStages);
  int* status = reinterpret_cast<int*>(tmem_slot + 1);  // 0 = MMAs of every block issued and completed

  const int mt = blockIdx.x, nt = blockIdx.y, kc = blockIdx.z;
  const int kb0 = kc * kb_per_cta, kb1 = min(kblocks, kb0 + kb_per_cta);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    fence_mbar_init();
    *status = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (threadIdx.x == 0) {
    constexpr uint32_t idesc = tc_idesc_tf32(kTcM, N);
    const int nu = 2 * (kb1 - kb0);  // half blocks
    const unsigned char* ga0 = reinterpret_cast<const unsigned char*>(A_packed) +
                               static_cast<int64_t>(mt) * kblocks * (2 * static_cast<int64_t>(kBlockA));
    const unsigned char* gb0 = reinterpret_cast<const unsigned char*>(B_packed) +
                               static_cast<int64_t>(nt) * kblocks * (2 * static_cast<int64_t>(kBlockB));
    // Half block u of this CTA: k-step slabs 4h .. 4h + 3 of block kb0 + u / 2, from the hi and lo
    // parts of each operand (a packed block is [hi: 8 slabs][lo: 8 slabs]).
    auto issue = [&](int u) {
      unsigned char* st = tc_smem + (u % kStages) * kStage;
      const int64_t kb = kb0 + u / 2, h = u & 1;
      const unsigned char* ga = ga0 + kb * (2 * kBlockA) + h * kHalfA;
      const unsigned char* gb = gb0 + kb * (2 * kBlockB) + h * kHalfB;
      mbar_arrive_expect_tx(&full[u % kStages], kStage);
      bulk_copy_g2s(st, ga, kHalfA, &full[u % kStages]);
      bulk_copy_g2s(st + kHalfA, ga + kBlockA, kHalfA, &full[u % kStages]);
      bulk_copy_g2s(st + 2 * kHalfA, gb, kHalfB, &full[u % kStages]);
      bulk_copy_g2s(st + 2 * kHalfA + kHalfB, gb + kBlockB, kHalfB, &full[u % kStages]);
    };
    int issued = 0, waited = 0, committed = 0;  // units copied / landed / whose MMAs were committed
    for (; issued < min(kStages, nu); ++issued) issue(issued);
    bool ok = true;
    for (int u = 0; u < nu && ok; ++u) {
      const int sidx = u % kStages;
      if (!mbar_wait_bounded(&full[sidx], (u / kStages) & 1)) {
        ok = false;
        break;
      }
      waited = u + 1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const unsigned char* st = tc_smem + sidx * kStage;
#pragma unroll
      for (int ks = 0; ks < kTcKB / 16; ++ks) {
        const uint64_t ah = tc_smem_desc(st + ks * kTcM * 32, kTcLbo, kTcSbo);
        const uint64_t al = tc_smem_desc(st + kHalfA + ks * kTcM * 32, kTcLbo, kTcSbo);
        const uint64_t bh = tc_smem_desc(st + 2 * kHalfA + ks * N * 32, kTcLbo, kTcSbo);
        const uint64_t bl = tc_smem_desc(st + 2 * kHalfA + kHalfB + ks * N * 32, kTcLbo, kTcSbo);
        tc_mma_tf32(tmem, ah, bh, idesc, (u > 0 || ks > 0) ? 1u : 0u);
        tc_mma_tf32(tmem, ah, bl, idesc, 1u);
        tc_mma_tf32(tmem, al, bh, idesc, 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&empty[sidx]))
                   : "memory");
      committed = u + 1;
      // The previous unit's stage is refilled once its MMAs have completed (this unit's run meanwhile).
      const int v = u - 1;
      if (v >= 0 && v + kStages < nu) {
        if (!mbar_wait_bounded(&empty[v % kStages], (v / kStages) & 1)) {
          ok = false;
          break;
        }
        issue(v + kStages);
        ++issued;
      }
    }
    if (!ok) {
      atomicOr(err, kDevErrTimeout);
      *status = 1;
      // Do not leave while copies may still land in shared memory.
      for (int j = waited; j < issued; ++j) mbar_wait_bounded(&full[j % kStages], (j / kStages) & 1);
    }
    // No MMA may be in flight when the accumulator is read or TMEM is freed (commits complete in order).
    if (committed > 0) {
      const int c = committed - 1;
      if (!mbar_wait_bounded(&empty[c % kStages], (c / kStages) & 1)) {
        atomicOr(err, kDevErrTimeout);
        *status = 1;
      }
    }
  }
  __syncthreads();
  __syncwarp();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (*status == 0 && kb1 > kb0) {
    // Warp w owns TMEM lanes (accumulator rows) 32w .. 32w+31.
    const int m = mt * kTcM + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (m < S) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = nt * N + c0 + j;
          if (n < D) partial[(static_cast<int64_t>(kc) * D + n) * S + m] = static_cast<double>(__uint_as_float(v[j]));
        }
      }
    }
  } else if (kb1 <= kb0) {
    // No K blocks for this CTA (only when the grid over-covers K): contribute zeros.
    const int m = mt * kTcM + warp * 32 + lane;
    if (m < S)
      for (int n = nt * N; n < min(D, nt * N + N); ++n) partial[(static_cast<int64_t>(kc) * D + n) * S + m] = 0.0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
  }
}

template <int N>
__host__ __device__ constexpr int tc_gemm_smem_bytes() {
  return tc_stages<N>() * tc_half_bytes<N>() + 16 * tc_stages<N>() + 16;
}
static_assert(tc_gemm_smem_bytes<256>() <= 227 * 1024 && tc_gemm_smem_bytes<128>() <= 227 * 1024 &&
                  tc_gemm_smem_bytes<64>() <= 227 * 1024 && tc_gemm_smem_bytes<32>() <= 227 * 1024,
              "ring of the Ad contraction within one block's shared memory");

}  // namespace leapgb
