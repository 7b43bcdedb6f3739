// Small-K matrix products C[b] (=|+=) A @ B[b] on the 5th-generation tensor cores (tcgen05), BF16 inputs with a
// split-precision correction and FP32 accumulation in tensor memory.
//
// Each float32 operand x is split into x_hi = bf16(x) and x_lo = bf16(x - x_hi); the product is formed as
// A_hi B_hi + A_hi B_lo + A_lo B_hi (the A_lo B_lo term is below the float32 rounding of the sum), which keeps about
// sixteen bits of every input: relative errors near 1e-5 instead of bfloat16's 4e-3. The contraction of the
// scattering source has a short inner dimension (K <= 128) and a very long column dimension J, so the kernel streams
// J in tiles of 128 columns:
//
//   * A (M <= 128 rows, zero-padded to 128) is split once per CTA into shared memory in the K-major canonical layout
//     without swizzle: 8-row x 16-byte core matrices, adjacent in K 128 bytes apart (leading byte offset) and in M 256
//     bytes apart (stride byte offset), one region per 16-wide K step.
//   * Per tile, thread t reads column t of B in groups of 8 rows (coalesced across the warp), splits it and writes
//     one 16-byte core-matrix row of B_hi and of B_lo: the same K-major layout with N in place of M.
//   * One thread issues the 3 x (K / 16) MMAs (kind::f16 with bf16 operands) with the tile's 128 columns as the MMA's
//     M and the rows of C (rounded up to 16) as its N, so that the float32 accumulator in tensor memory holds C[:,
//     tile] transposed, and commits them to an mbarrier; every wait on it is bounded by a wall-clock limit, after
//     which the CTA records the error and leaves.
//   * Accumulator lane l is column l of the tile: each thread reads its lane (tcgen05.ld 32x32b) and stores (or adds
//     to) its column of C, 32 consecutive columns of one row per warp store.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>
#include <stdlib.h>
#include <string.h>

#include "tcgen05.cuh"

namespace citrus {
namespace {

constexpr int kTcThreads = 128;  // four warps: warp w owns accumulator lanes 32w .. 32w + 31
constexpr int kTcN = 128;        // MMA columns per tile (B columns)
constexpr int kTcMaxK = 128;     // inner dimension, padded to a multiple of 16

// D = C[:, tile]^T: the tile's 128 columns are the MMA's rows and the (M rounded up to 16) rows of C its N, so each
// accumulator lane is one column of C, stored directly. F (the first-collision means of the source expansion,
// [M, J / 4] per batch, ldf floats per row and stride_f floats between batches) is added to the first of every four
// columns of C when not null (with accumulate 0).
__global__ void __launch_bounds__(kTcThreads) gemm_tc_kernel(const float* __restrict__ A, int64_t lda,
                                                             const float* __restrict__ B, int64_t ldb,
                                                             float* __restrict__ C, int64_t ldc, int M, int K,
                                                             int64_t J, int64_t stride_b, int64_t stride_c,
                                                             int accumulate, int64_t tiles_per_batch,
                                                             int64_t num_tiles, uint32_t* __restrict__ error_word,
                                                             const float* __restrict__ F, int64_t ldf,
                                                             int64_t stride_f) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int KS = (K + 15) / 16;            // K steps
  const uint32_t a_step = kTcM * 16 * 2;   // bytes of one K step of A (4 KB)
  const uint32_t b_step = kTcN * 16 * 2;   // bytes of one K step of B (4 KB)
  uint8_t* a_hi = smem;
  uint8_t* a_lo = a_hi + KS * a_step;
  uint8_t* b_hi = a_lo + KS * a_step;
  uint8_t* b_lo = b_hi + KS * b_step;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;

  // A, split once: thread t packs rows t of all K steps, 8 columns (one core-matrix row) at a time
  for (int s = 0; s < KS; ++s) {
    for (int k8 = 0; k8 < 16; k8 += 8) {
      float x[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int k = s * 16 + k8 + q;
        x[q] = (tid < M && k < K) ? A[(int64_t)tid * lda + k] : 0.f;
      }
      uint4 hi, lo;
      split_pair(x[0], x[1], hi.x, lo.x);
      split_pair(x[2], x[3], hi.y, lo.y);
      split_pair(x[4], x[5], hi.z, lo.z);
      split_pair(x[6], x[7], hi.w, lo.w);
      const uint32_t off = s * a_step + core_offset(tid, k8);
      *reinterpret_cast<uint4*>(a_hi + off) = hi;
      *reinterpret_cast<uint4*>(a_lo + off) = lo;
    }
  }
  if (tid == 0) {
    abort_flag = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const int n_t = ((M + 15) / 16) * 16;                   // MMA N: the rows of C rounded up to 16
  const uint32_t acc_cols = n_t <= 64 ? 64u : 128u;       // accumulator columns (a power of two >= 32)
  const uint32_t idesc = idesc_bf16(n_t);
  if (warp == 0) {  // the accumulator: 128 lanes x acc_cols float32 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(acc_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  const uint32_t mbar_addr = smem_u32(&mbar);
  uint32_t phase = 0;

  for (int64_t tile = blockIdx.x; tile < num_tiles; tile += gridDim.x) {
    const int64_t bz = tile / tiles_per_batch;
    const int64_t n0 = (tile - bz * tiles_per_batch) * kTcN;
    const float* Bz = B + bz * stride_b;
    float* Cz = C + bz * stride_c;
    const float* Fz = F != nullptr ? F + bz * stride_f : nullptr;
    // B tile: column n0 + tid, split into the K-major layout
    const int64_t col = n0 + tid;
    const bool cvalid = col < J;
    for (int s = 0; s < KS; ++s) {
      for (int k8 = 0; k8 < 16; k8 += 8) {
        float x[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int k = s * 16 + k8 + q;
          x[q] = (cvalid && k < K) ? __ldg(Bz + (int64_t)k * ldb + col) : 0.f;
        }
        uint4 hi, lo;
        split_pair(x[0], x[1], hi.x, lo.x);
        split_pair(x[2], x[3], hi.y, lo.y);
        split_pair(x[4], x[5], hi.z, lo.z);
        split_pair(x[6], x[7], hi.w, lo.w);
        const uint32_t off = s * b_step + core_offset(tid, k8);
        *reinterpret_cast<uint4*>(b_hi + off) = hi;
        *reinterpret_cast<uint4*>(b_lo + off) = lo;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the operands, visible to the tensor cores
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int s = 0; s < KS; ++s) {
        const uint64_t ah = smem_desc(smem_u32(a_hi + s * a_step), 128, 256);
        const uint64_t al = smem_desc(smem_u32(a_lo + s * a_step), 128, 256);
        const uint64_t bh = smem_desc(smem_u32(b_hi + s * b_step), 128, 256);
        const uint64_t bl = smem_desc(smem_u32(b_lo + s * b_step), 128, 256);
        mma_bf16(tmem, bh, ah, idesc, s > 0 ? 1u : 0u);
        mma_bf16(tmem, bh, al, idesc, 1u);
        mma_bf16(tmem, bl, ah, idesc, 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_addr)
                   : "memory");
    }
    const bool ok = mbar_wait(mbar_addr, phase, global_timer_ns());
    phase ^= 1u;
    if (!ok) {
      if (error_word != nullptr) atomicExch(error_word, 1u);
      abort_flag = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (abort_flag) break;
    {
      // epilogue: lane 32 warp + lane is column n0 + 32 warp + lane of C, its accumulator
      // columns the rows of C; every store covers 32 consecutive columns of one row
      const int64_t col = n0 + warp * 32 + lane;
#pragma unroll 1
      for (int m0 = 0; m0 < n_t; m0 += 16) {
        uint32_t r[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)m0)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (col < J) {
          const int rows = min(16, M - m0);
          float* out = Cz + (int64_t)m0 * ldc + col;
          float prev[16];
          if (accumulate) {
#pragma unroll
            for (int q = 0; q < 16; ++q) prev[q] = q < rows ? out[(int64_t)q * ldc] : 0.f;
          } else if (Fz != nullptr && (col & 3) == 0) {  // the mean of the quadruple's first column
#pragma unroll
            for (int q = 0; q < 16; ++q) prev[q] = q < rows ? __ldg(Fz + (int64_t)(m0 + q) * ldf + (col >> 2)) : 0.f;
          }
          const bool add = accumulate || (Fz != nullptr && (col & 3) == 0);
#pragma unroll
          for (int q = 0; q < 16; ++q)
            if (q < rows) out[(int64_t)q * ldc] = add ? prev[q] + __uint_as_float(r[q]) : __uint_as_float(r[q]);
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // the accumulator and the B tile are free for the next tile
  }
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(acc_cols) : "memory");
}

// ---- the warp-specialised form ------------------------------------------------------------------------------------
// The same product as gemm_tc_kernel with its stages overlapped, one CTA per SM walking its tiles in order:
//
//   * loader (one thread of warp 13): the [K x 128] float32 tile of B comes in one tensor copy (cp.async.bulk.tensor
//     through a tensor map of B as [batch][K][J], completing on the stage's mbarrier with the box's byte count;
//     columns past J read as zeros), or, where the map cannot be made, as K bulk copies of its 512-byte row runs, into
//     a ring of float32 stages (as many as the shared memory holds, up to kWsRawMax). One request per tile instead of
//     K: the per-request cost of K small copies held the loads near 1.3 TB/s;
//   * converters (warps 8 to 11): thread t splits column t of a raw stage into the bfloat16 high and low operand
//     tiles in the K-major core-matrix layout (kWsOps stages), then frees the raw stage;
//   * MMA issuer (one thread of warp 12): 3 x (K / 16) tcgen05.mma per tile into one of two float32 accumulators in
//     tensor memory, committed to the operand stage (freed once read) and to the accumulator (full);
//   * epilogue (warps 0 to 7): warp w reads accumulator lanes 32 (w % 4) .. + 31 (columns of C) and every other
//     16 of its rows, and writes (or adds to) C, so that the stores of one tile overlap the loads, splits and MMAs
//     of the next; the means come from their own two-stage ring (one tensor copy of [M][32] per tile).
//
// The MMAs run in gemm_tc_kernel's order and the epilogue adds in its order: the two forms give the same bits. Every
// mbarrier wait is bounded by kTcTimeoutNs; a role whose wait runs out records the error and stops, the others then
// stop at their own bounded waits, the issuer waits (bounded) for its last MMAs, and the CTA frees its tensor memory.
constexpr int kWsRawMax = 3;              // float32 stages of B (deeper rings measured no faster with tensor copies)
constexpr int kWsOps = 2;                 // bf16 hi/lo operand stages
constexpr int kWsThreads = 14 * 32;       // 8 epilogue, 4 converter, 1 MMA and 1 loader warps
constexpr int kWsEpilogueWarps = 8;
constexpr int kWsConverterWarp0 = 8;
constexpr int kWsMmaWarp = 12;
constexpr int kWsLoaderWarp = 13;
constexpr size_t kWsMeansBytes = 2 * kTcM * 32 * 4;  // two [M <= 128][32] float32 tiles of the means

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__global__ void __launch_bounds__(kWsThreads, 1) gemm_ws_kernel(const float* __restrict__ A, int64_t lda,
                                                                const float* __restrict__ B, int64_t ldb,
                                                                float* __restrict__ C, int64_t ldc, int M, int K,
                                                                int64_t J, int64_t stride_b, int64_t stride_c,
                                                                int accumulate, int64_t tiles_per_batch,
                                                                int64_t num_tiles, uint32_t* __restrict__ error_word,
                                                                const float* __restrict__ F, int64_t ldf,
                                                                int64_t stride_f, int raw_stages,
                                                                const __grid_constant__ CUtensorMap b_map,
                                                                int use_map,
                                                                const __grid_constant__ CUtensorMap f_map,
                                                                int use_f_map) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int KS = (K + 15) / 16;
  const uint32_t a_step = kTcM * 16 * 2, b_step = kTcN * 16 * 2;
  const uint32_t raw_bytes = (uint32_t)K * kTcN * 4;
  const uint32_t raw_stride = (raw_bytes + 1023u) & ~1023u;
  uint8_t* a_hi = smem;
  uint8_t* a_lo = a_hi + KS * a_step;
  uint8_t* ops = a_lo + KS * a_step;                                 // kWsOps x (hi, lo)
  const uint32_t op_bytes = 2u * KS * b_step;
  float* raw = reinterpret_cast<float*>(ops + kWsOps * op_bytes);   // raw_stages x [K][128]
  __shared__ __align__(8) uint64_t bar[2 * kWsRawMax + 2 * kWsOps + 9];
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  uint64_t* raw_full = bar;
  uint64_t* raw_empty = bar + kWsRawMax;
  uint64_t* op_full = bar + 2 * kWsRawMax;
  uint64_t* op_empty = op_full + kWsOps;
  uint64_t* acc_full = op_empty + kWsOps;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* mma_done = acc_empty + 2;  // the issuer's last commit: its MMAs are complete before the CTA frees TMEM
  // the first-collision means come as [M][32] tiles (the tile's 128 columns / 4) in two stages after the float32 ring
  uint64_t* f_full = mma_done + 1;
  uint64_t* f_empty = f_full + 2;
  float* f_stage = reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(raw) + raw_stages * raw_stride);
  const bool f_tma = F != nullptr && use_f_map != 0;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;

  // A, split once (threads 0..127), rows r of every K step, 8 columns at a time
  for (int r = tid; r < kTcM; r += kWsThreads)
    for (int s = 0; s < KS; ++s)
      for (int k8 = 0; k8 < 16; k8 += 8) {
        float x[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int k = s * 16 + k8 + q;
          x[q] = (r < M && k < K) ? A[(int64_t)r * lda + k] : 0.f;
        }
        uint4 hi, lo;
        split_pair(x[0], x[1], hi.x, lo.x);
        split_pair(x[2], x[3], hi.y, lo.y);
        split_pair(x[4], x[5], hi.z, lo.z);
        split_pair(x[6], x[7], hi.w, lo.w);
        const uint32_t off = s * a_step + core_offset(r, k8);
        *reinterpret_cast<uint4*>(a_hi + off) = hi;
        *reinterpret_cast<uint4*>(a_lo + off) = lo;
      }
  if (tid == 0) {
    abort_flag = 0;
    for (int i = 0; i < raw_stages; ++i) {
      mbar_init(smem_u32(raw_full + i), 1);
      mbar_init(smem_u32(raw_empty + i), 128);
    }
    for (int i = 0; i < kWsOps; ++i) {
      mbar_init(smem_u32(op_full + i), 128);
      mbar_init(smem_u32(op_empty + i), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_u32(acc_full + i), 1);
      mbar_init(smem_u32(acc_empty + i), 32 * kWsEpilogueWarps);
    }
    mbar_init(smem_u32(mma_done), 1);
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_u32(f_full + i), 1);
      mbar_init(smem_u32(f_empty + i), 32 * kWsEpilogueWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const int n_t = ((M + 15) / 16) * 16;
  const uint32_t acc_cols = n_t <= 64 ? 64u : 128u;  // one accumulator; two are allocated
  const uint32_t idesc = idesc_bf16(n_t);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(2 * acc_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the split A, visible to the tensor cores
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  const int64_t my_tiles = num_tiles > (int64_t)blockIdx.x ? (num_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const auto fail = [&]() {
    if (error_word != nullptr) atomicExch(error_word, 1u);
    abort_flag = 1;
  };

  if (warp == kWsLoaderWarp) {
    if (lane == 1 && f_tma) {  // the means: one tensor copy of [M][32] per tile, two stages ahead of the epilogue
      for (int64_t i = 0; i < my_tiles && !abort_flag; ++i) {
        const int fs = (int)(i & 1);
        if (!mbar_wait(smem_u32(f_empty + fs), (uint32_t)((i >> 1) & 1) ^ 1u, global_timer_ns())) {
          fail();
          break;
        }
        const int64_t tile = blockIdx.x + i * gridDim.x;
        const int64_t bz = tile / tiles_per_batch;
        const int64_t n0 = (tile - bz * tiles_per_batch) * kTcN;
        const uint32_t mb = smem_u32(f_full + fs);
        mbar_expect_tx(mb, (uint32_t)M * 32u * 4u);
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
            "%4}], [%5];" ::"r"(smem_u32(f_stage + fs * M * 32)),
            "l"(reinterpret_cast<uint64_t>(&f_map)), "r"((int)(n0 / 4)), "r"(0), "r"((int)bz), "r"(mb)
            : "memory");
      }
    }
    if (lane == 0) {
      for (int64_t i = 0; i < my_tiles && !abort_flag; ++i) {
        const int st = (int)(i % raw_stages);
        if (!mbar_wait(smem_u32(raw_empty + st), (uint32_t)((i / raw_stages) & 1) ^ 1u, global_timer_ns())) {
          fail();
          break;
        }
        const int64_t tile = blockIdx.x + i * gridDim.x;
        const int64_t bz = tile / tiles_per_batch;
        const int64_t n0 = (tile - bz * tiles_per_batch) * kTcN;
        const uint32_t bytes = (uint32_t)((J - n0 < kTcN ? J - n0 : (int64_t)kTcN) * 4);
        const uint32_t mb = smem_u32(raw_full + st);
        const uint32_t dst = smem_u32(reinterpret_cast<uint8_t*>(raw) + st * raw_stride);
        if (use_map) {
          mbar_expect_tx(mb, (uint32_t)K * kTcN * 4);  // the whole box, its columns past J filled with zeros
          asm volatile(
              "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
              "%4}], [%5];" ::"r"(dst),
              "l"(reinterpret_cast<uint64_t>(&b_map)), "r"((int)n0), "r"(0), "r"((int)bz), "r"(mb)
              : "memory");
        } else {
          mbar_expect_tx(mb, bytes * (uint32_t)K);
          const float* src = B + bz * stride_b + n0;
          for (int k = 0; k < K; ++k) bulk_copy_g2s(dst + (uint32_t)k * kTcN * 4, src + (int64_t)k * ldb, bytes, mb);
        }
      }
    }
  } else if (warp >= kWsConverterWarp0 && warp < kWsConverterWarp0 + 4) {
    const int t = tid - kWsConverterWarp0 * 32;  // the tile column this thread splits
    for (int64_t i = 0; i < my_tiles && !abort_flag; ++i) {
      const int st = (int)(i % raw_stages), op = (int)(i % kWsOps);
      if (!mbar_wait(smem_u32(raw_full + st), (uint32_t)((i / raw_stages) & 1), global_timer_ns()) ||
          !mbar_wait(smem_u32(op_empty + op), (uint32_t)((i / kWsOps) & 1) ^ 1u, global_timer_ns())) {
        fail();
        break;
      }
      const float* col = reinterpret_cast<const float*>(reinterpret_cast<uint8_t*>(raw) + st * raw_stride) + t;
      uint8_t* o_hi = ops + op * op_bytes;
      uint8_t* o_lo = o_hi + KS * b_step;
      for (int s = 0; s < KS; ++s)
        for (int k8 = 0; k8 < 16; k8 += 8) {
          float x[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int k = s * 16 + k8 + q;
            x[q] = k < K ? col[k * kTcN] : 0.f;
          }
          uint4 hi, lo;
          split_pair(x[0], x[1], hi.x, lo.x);
          split_pair(x[2], x[3], hi.y, lo.y);
          split_pair(x[4], x[5], hi.z, lo.z);
          split_pair(x[6], x[7], hi.w, lo.w);
          const uint32_t off = s * b_step + core_offset(t, k8);
          *reinterpret_cast<uint4*>(o_hi + off) = hi;
          *reinterpret_cast<uint4*>(o_lo + off) = lo;
        }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the operands, visible to the tensor cores
      mbar_arrive(smem_u32(raw_empty + st));
      mbar_arrive(smem_u32(op_full + op));
    }
  } else if (warp == kWsMmaWarp) {
    if (lane == 0) {
      for (int64_t i = 0; i < my_tiles && !abort_flag; ++i) {
        const int op = (int)(i % kWsOps), ac = (int)(i & 1);
        if (!mbar_wait(smem_u32(op_full + op), (uint32_t)((i / kWsOps) & 1), global_timer_ns()) ||
            !mbar_wait(smem_u32(acc_empty + ac), (uint32_t)((i >> 1) & 1) ^ 1u, global_timer_ns())) {
          fail();
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + (uint32_t)ac * acc_cols;
        uint8_t* o_hi = ops + op * op_bytes;
        uint8_t* o_lo = o_hi + KS * b_step;
        for (int s = 0; s < KS; ++s) {
          const uint64_t ah = smem_desc(smem_u32(a_hi + s * a_step), 128, 256);
          const uint64_t al = smem_desc(smem_u32(a_lo + s * a_step), 128, 256);
          const uint64_t bh = smem_desc(smem_u32(o_hi + s * b_step), 128, 256);
          const uint64_t bl = smem_desc(smem_u32(o_lo + s * b_step), 128, 256);
          mma_bf16(d, bh, ah, idesc, s > 0 ? 1u : 0u);
          mma_bf16(d, bh, al, idesc, 1u);
          mma_bf16(d, bl, ah, idesc, 1u);
        }
        tc_commit(smem_u32(op_empty + op));
        tc_commit(smem_u32(acc_full + ac));
      }
      tc_commit(smem_u32(mma_done));  // tracks every MMA issued above
      if (!mbar_wait(smem_u32(mma_done), 0u, global_timer_ns())) fail();
    }
  } else {  // epilogue warps 0 .. 7
    const int quarter = warp % 4, half = warp / 4;
    for (int64_t i = 0; i < my_tiles && !abort_flag; ++i) {
      const int ac = (int)(i & 1);
      if (!mbar_wait(smem_u32(acc_full + ac), (uint32_t)((i >> 1) & 1), global_timer_ns())) {
        fail();
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int64_t tile = blockIdx.x + i * gridDim.x;
      const int64_t bz = tile / tiles_per_batch;
      const int64_t n0 = (tile - bz * tiles_per_batch) * kTcN;
      float* Cz = C + bz * stride_c;
      const float* Fz = F != nullptr ? F + bz * stride_f : nullptr;
      const uint32_t taddr = tmem + (uint32_t)ac * acc_cols + ((uint32_t)(quarter * 32) << 16);
      const float* fst = f_stage + (int)(i & 1) * M * 32;
      if (f_tma && !mbar_wait(smem_u32(f_full + (int)(i & 1)), (uint32_t)((i >> 1) & 1), global_timer_ns())) {
        fail();
        break;
      }
      {
        // accumulator lane 32 quarter + lane is column n0 + 32 quarter + lane of C; its columns are the rows of C,
        // split in 16-row steps between the two halves of the epilogue warps
        const int64_t col = n0 + quarter * 32 + lane;
        const bool add = accumulate || (Fz != nullptr && (col & 3) == 0);
        for (int m0 = half * 16; m0 < n_t; m0 += 32) {
          const int rows = min(16, M - m0);
          float* out = Cz + (int64_t)m0 * ldc + col;
          // the loads of C (accumulating) or of the means are issued before the tensor-memory load, so that the two
          // latencies overlap
          float prev[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) prev[q] = 0.f;
          if (col < J) {
            if (accumulate) {
#pragma unroll
              for (int q = 0; q < 16; ++q)
                if (q < rows) prev[q] = out[(int64_t)q * ldc];
            } else if (add && f_tma) {
              const int fc = (quarter * 32 + lane) >> 2;  // the tile's column / 4
#pragma unroll
              for (int q = 0; q < 16; ++q)
                if (q < rows) prev[q] = fst[(m0 + q) * 32 + fc];
            } else if (add) {
#pragma unroll
              for (int q = 0; q < 16; ++q)
                if (q < rows) prev[q] = __ldg(Fz + (int64_t)(m0 + q) * ldf + (col >> 2));
            }
          }
          uint32_t r[16];
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
              "%14, %15}, [%16];"
              : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
              : "r"(taddr + (uint32_t)m0)
              : "memory");
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (col < J) {
#pragma unroll
            for (int q = 0; q < 16; ++q)
              if (q < rows) out[(int64_t)q * ldc] = add ? prev[q] + __uint_as_float(r[q]) : __uint_as_float(r[q]);
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(smem_u32(acc_empty + ac));
      if (f_tma) mbar_arrive(smem_u32(f_empty + (int)(i & 1)));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * acc_cols) : "memory");
}

// shared memory of the warp-specialised form: A hi/lo, kWsOps operand stages, the float32 stages (1 KB aligned),
// the two stages of the means; ws_raw_stages: as many float32 stages as fit 227 KB with the rest, up to kWsRawMax
constexpr size_t kWsSmemLimit = 227 * 1024;
size_t ws_raw_stride(int K) { return (((size_t)K * kTcN * 4) + 1023) & ~(size_t)1023; }
size_t ws_fixed_bytes(int K) {
  const size_t KS = (size_t)(K + 15) / 16;
  return KS * 2 * kTcM * 16 * 2 + kWsOps * KS * 2 * kTcN * 16 * 2 + kWsMeansBytes;
}
int ws_raw_stages(int K) {
  const size_t fixed = ws_fixed_bytes(K), stride = ws_raw_stride(K);
  const size_t n = fixed < kWsSmemLimit ? (kWsSmemLimit - fixed) / stride : 0;
  return (int)std::min<size_t>(n, kWsRawMax);
}
size_t ws_smem_bytes(int K) { return ws_fixed_bytes(K) + (size_t)std::max(ws_raw_stages(K), 2) * ws_raw_stride(K); }

}  // namespace
}  // namespace citrus

using namespace citrus;

namespace citrus {
namespace {

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against the driver library); null when the
// driver does not provide it
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// B as a float32 tensor [batch][K][J] (J innermost, rows ldb floats apart, batches stride_b floats apart) with a
// [1][K][128] box: one tensor copy per tile. The launcher has checked the 16-byte alignment of B, ldb and stride_b.
// the means F as [batch][M][J / 4] with a [1][M][32] box (the 128 columns of a tile / 4); false when F's alignment,
// row or batch strides do not allow a tensor map (the epilogue then reads F from global memory)
bool encode_f_map(CUtensorMap* map, const float* F, int64_t M, int64_t J, int64_t ldf, int64_t batch,
                  int64_t stride_f) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (enc == nullptr || F == nullptr || ((uintptr_t)F % 16) != 0 || ldf % 4 != 0 || (batch > 1 && stride_f % 4 != 0) ||
      J / 4 > 0x7fffffffLL || batch > 0x7fffffffLL)
    return false;
  const cuuint64_t dims[3] = {(cuuint64_t)(J / 4), (cuuint64_t)M, (cuuint64_t)batch};
  const cuuint64_t strides[2] = {(cuuint64_t)ldf * 4, (cuuint64_t)(batch > 1 ? stride_f : ldf * M) * 4};
  const cuuint32_t box[3] = {32u, (cuuint32_t)M, 1u};
  const cuuint32_t elem[3] = {1u, 1u, 1u};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(F), dims, strides, box, elem,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_b_map(CUtensorMap* map, const float* B, int64_t K, int64_t J, int64_t ldb, int64_t batch,
                  int64_t stride_b) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (enc == nullptr || J > 0x7fffffffLL || batch > 0x7fffffffLL) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)J, (cuuint64_t)K, (cuuint64_t)batch};
  const cuuint64_t strides[2] = {(cuuint64_t)ldb * 4, (cuuint64_t)(batch > 1 ? stride_b : ldb * K) * 4};
  const cuuint32_t box[3] = {(cuuint32_t)kTcN, (cuuint32_t)K, 1u};
  const cuuint32_t elem[3] = {1u, 1u, 1u};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(B), dims, strides, box, elem,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// CITRUS_TC_FORM=single keeps the single-stage kernel (measurements, and the check that both forms agree); read at
// every call
inline bool ws_disabled() {
  const char* v = getenv("CITRUS_TC_FORM");
  return v != nullptr && v[0] == 's';
}

int launch_gemm_tc(const char* name, const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
                   int64_t M, int64_t K, int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c,
                   int32_t accumulate, uint32_t* error_word, const float* F, int64_t ldf, int64_t stride_f,
                   void* stream) {
  CITRUS_REQUIRE(A && B && C, "%s: null pointer argument", name);
  CITRUS_REQUIRE(M >= 1 && M <= kTcM && K >= 1 && K <= kTcMaxK && J >= 0 && batch >= 1,
                 "%s: M %lld (<= %d) or K %lld (<= %d) out of range", name, (long long)M, kTcM, (long long)K,
                 kTcMaxK);
  CITRUS_REQUIRE(lda >= K && ldb >= J && ldc >= J, "%s: leading dimensions too small", name);
  if (J == 0) return CITRUS_OK;
  const int KS = (int)((K + 15) / 16);
  // A and B operands (the epilogue's staging, 128 x 33 floats, reuses the B region), and at least 50 KB so that no
  // more than four CTAs (4 x 128 of the 512 tensor-memory columns) share an SM: every allocation succeeds at once
  const size_t b_bytes = (size_t)KS * 2 * kTcN * 16 * 2;
  const size_t smem = std::max<size_t>((size_t)KS * 2 * kTcM * 16 * 2 + b_bytes, 50 * 1024);
  // the warp-specialised form when B's rows are runs of 16-byte units (bulk copies) and its stages fit one CTA
  const size_t ws_smem = ws_smem_bytes((int)K);
  const int raw_stages = ws_raw_stages((int)K);
  if (J % 4 == 0 && ldb % 4 == 0 && stride_b % 4 == 0 && ((uintptr_t)B % 16) == 0 && raw_stages >= 2 &&
      ws_smem <= kWsSmemLimit && !ws_disabled()) {
    const void* wfn = (const void*)gemm_ws_kernel;
    cudaError_t we = cudaFuncSetAttribute(wfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ws_smem);
    if (we != cudaSuccess) return set_error(CITRUS_ECUDA, "%s: %s", name, cudaGetErrorString(we));
    const int64_t tiles_per_batch = cdiv(J, kTcN);
    const int64_t num_tiles = tiles_per_batch * batch;
    const int64_t grid = std::min<int64_t>(num_tiles, (int64_t)num_sms());
    CUtensorMap b_map;
    memset(&b_map, 0, sizeof(b_map));
    const int use_map = encode_b_map(&b_map, B, K, J, ldb, batch, stride_b) ? 1 : 0;
    CUtensorMap f_map;
    memset(&f_map, 0, sizeof(f_map));
    const int use_f_map = F != nullptr && encode_f_map(&f_map, F, M, J, ldf, batch, stride_f) ? 1 : 0;
    gemm_ws_kernel<<<(unsigned)grid, kWsThreads, ws_smem, as_stream(stream)>>>(
        A, lda, B, ldb, C, ldc, (int)M, (int)K, J, stride_b, stride_c, accumulate, tiles_per_batch, num_tiles,
        error_word, F, ldf, stride_f, raw_stages, b_map, use_map, f_map, use_f_map);
    note_launches();
    return launch_status(name);
  }
  const void* fn = (const void*)gemm_tc_kernel;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  // all of the unified L1 / shared-memory capacity as shared memory, so that four CTAs fit an SM
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "%s: %s", name, cudaGetErrorString(e));
  const int64_t tiles_per_batch = cdiv(J, kTcN);
  const int64_t num_tiles = tiles_per_batch * batch;
  // four CTAs per SM: the shared-memory floor keeps a fifth from becoming resident (tensor memory holds four
  // 128-column accumulators), and CTAs beyond what fits simply wait for a free slot
  const int64_t grid = std::min<int64_t>(num_tiles, 4 * (int64_t)num_sms());
  gemm_tc_kernel<<<(unsigned)grid, kTcThreads, smem, as_stream(stream)>>>(
      A, lda, B, ldb, C, ldc, (int)M, (int)K, J, stride_b, stride_c, accumulate, tiles_per_batch, num_tiles,
      error_word, F, ldf, stride_f);
  note_launches();
  return launch_status(name);
}

}  // namespace
}  // namespace citrus

extern "C" int citrus_small_k_gemm_bf16x3(const float* A, int64_t lda, const float* B, int64_t ldb, float* C,
                                          int64_t ldc, int64_t M, int64_t K, int64_t J, int64_t batch,
                                          int64_t stride_b, int64_t stride_c, int32_t accumulate,
                                          uint32_t* error_word, void* stream) {
  return launch_gemm_tc("citrus_small_k_gemm_bf16x3", A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c,
                        accumulate, error_word, nullptr, 0, 0, stream);
}

extern "C" int citrus_source_expansion_first_bf16x3(const float* A, int64_t lda, const float* B, int64_t ldb,
                                                    float* C, int64_t ldc, const float* F, int64_t ldf, int64_t M,
                                                    int64_t K, int64_t J, int64_t batch, int64_t stride_b,
                                                    int64_t stride_c, int64_t stride_f, uint32_t* error_word,
                                                    void* stream) {
  CITRUS_REQUIRE(F != nullptr, "citrus_source_expansion_first_bf16x3: null means");
  CITRUS_REQUIRE(J % 4 == 0 && ldf >= J / 4, "citrus_source_expansion_first_bf16x3: the columns must come in "
                 "quadruples (J %lld) and ldf >= J / 4", (long long)J);
  return launch_gemm_tc("citrus_source_expansion_first_bf16x3", A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b,
                        stride_c, 0, error_word, F, ldf, stride_f, stream);
}
