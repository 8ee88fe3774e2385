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
// One CTA = one (128-row M tile, N-column tile, 64-k block); 128 threads.
// Warp 0 allocates (and finally frees) N TMEM columns; thread 0 issues the
// copies and the 24 MMAs (8 k-steps x 3) and commits them to an mbarrier; the
// four warps then read their 32 accumulator rows (TMEM lanes) with
// tcgen05.ld and write FP64 partial sums.  Waits are bounded: on a timeout
// the CTA sets the error word, still waits (bounded) for its copies, frees its
// TMEM and returns.
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

// N columns of FP32 accumulator per CTA; N is a multiple of 16 in [16, 256].
// CTA (mt, nt, kc) accumulates K blocks [kc*kb_per_cta, ...) in TMEM, one
// block at a time (load, 24 MMAs, wait), then writes partial[kc][d][s].
template <int N>
__global__ void __launch_bounds__(128, 1) tc_gemm_ad(const float* __restrict__ A_packed, const float* __restrict__ B_packed,
                                                     int S, int D, int kblocks, int kb_per_cta,
                                                     double* __restrict__ partial, int* __restrict__ err) {
  static_assert(N % 16 == 0 && N >= 16 && N <= 256, "N tile");
  constexpr int kCols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));  // power of two >= 32
  constexpr int kBytesA = 2 * tc_block_bytes(kTcM);
  constexpr int kBytesB = 2 * tc_block_bytes(N);
  extern __shared__ __align__(128) unsigned char tc_smem[];
  unsigned char* sA = tc_smem;                 // [hi | lo], 128 rows
  unsigned char* sB = tc_smem + kBytesA;       // [hi | lo], N rows
  uint64_t* bars = reinterpret_cast<uint64_t*>(tc_smem + kBytesA + kBytesB);  // [0] loads, [1] MMAs
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2);
  int* status = reinterpret_cast<int*>(tmem_slot + 1);  // 0 = MMAs of every block issued

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
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
    *status = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (threadIdx.x == 0) {
    constexpr uint32_t idesc = tc_idesc_tf32(kTcM, N);
    constexpr uint32_t lboA = kTcLbo, lboB = kTcLbo, sbo = kTcSbo;
    const unsigned char* aparts[2] = {sA, sA + tc_block_bytes(kTcM)};
    const unsigned char* bparts[2] = {sB, sB + tc_block_bytes(N)};
    for (int kb = kb0; kb < kb1; ++kb) {
      const uint32_t phase = static_cast<uint32_t>(kb - kb0) & 1u;
      const unsigned char* ga = reinterpret_cast<const unsigned char*>(A_packed) +
                                (static_cast<int64_t>(mt) * kblocks + kb) * static_cast<int64_t>(kBytesA);
      const unsigned char* gb = reinterpret_cast<const unsigned char*>(B_packed) +
                                (static_cast<int64_t>(nt) * kblocks + kb) * static_cast<int64_t>(kBytesB);
      mbar_arrive_expect_tx(&bars[0], kBytesA + kBytesB);
      for (int off = 0; off < kBytesA; off += 16384)
        bulk_copy_g2s(sA + off, ga + off, min(16384, kBytesA - off), &bars[0]);
      for (int off = 0; off < kBytesB; off += 16384)
        bulk_copy_g2s(sB + off, gb + off, min(16384, kBytesB - off), &bars[0]);
      if (!mbar_wait_bounded(&bars[0], phase)) {
        atomicOr(err, kDevErrTimeout);
        *status = 1;
        mbar_wait_bounded(&bars[0], phase);  // do not leave while the copies may still land
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int ks = 0; ks < kTcKB / 8; ++ks) {
        const int ao = ks * kTcM * 32, bo = ks * N * 32;
        tc_mma_tf32(tmem, tc_smem_desc(aparts[0] + ao, lboA, sbo), tc_smem_desc(bparts[0] + bo, lboB, sbo), idesc,
                    (kb > kb0 || ks > 0) ? 1u : 0u);
        tc_mma_tf32(tmem, tc_smem_desc(aparts[0] + ao, lboA, sbo), tc_smem_desc(bparts[1] + bo, lboB, sbo), idesc, 1u);
        tc_mma_tf32(tmem, tc_smem_desc(aparts[1] + ao, lboA, sbo), tc_smem_desc(bparts[0] + bo, lboB, sbo), idesc, 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bars[1]))
                   : "memory");
      // The next block's copies overwrite the operands: wait for these MMAs first.
      if (!mbar_wait_bounded(&bars[1], phase)) {
        atomicOr(err, kDevErrTimeout);
        *status = 1;
        mbar_wait_bounded(&bars[1], phase);  // one more bounded chance before TMEM is freed
        break;
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
  return 2 * tc_block_bytes(kTcM) + 2 * tc_block_bytes(N) + 64;
}

}  // namespace leapgb
