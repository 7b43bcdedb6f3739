// Small-K matrix products C[b] (=|+=) A @ B[b] of the sweep and of the image.
//
// The contractions of the scattering source (Y [D x N_sh] @ T [N_sh x J]), of the moment accumulation
// (Yw^T [N_sh x D] @ psi [D x J]) and of the multiple-collision source all have a short inner dimension
// (N_sh <= 64, D <= 240) and a very long column dimension J (cells x groups x 4), so they are streaming products: each
// block keeps A in shared memory, streams a 128-column slab of B through shared memory in 32-row chunks, and holds
// an (8 R) x 128 tile of C in registers, R rows and one float4 of columns per thread. B and C move once through HBM.
#include "common.cuh"

namespace citrus {
namespace {

constexpr int kThreads = 256;  // 8 warps; warp w owns rows w, w + 8, ... of the block's row tile
constexpr int kCols = 128;     // columns per block: 32 lanes x float4
constexpr int kChunk = 32;     // rows of B per shared-memory chunk

template <int R, bool kAligned>
__global__ void __launch_bounds__(kThreads) small_k_gemm_kernel(const float* __restrict__ A, int64_t lda,
                                                                const float* __restrict__ B, int64_t ldb,
                                                                float* __restrict__ C, int64_t ldc, int M, int K,
                                                                int64_t J, int64_t stride_b, int64_t stride_c,
                                                                int accumulate) {
  extern __shared__ float smem[];
  float* As = smem;                       // [8R][K] rows of this block's row tile
  float* Bs = smem + (size_t)8 * R * K;   // [kChunk][kCols]
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int64_t col0 = (int64_t)blockIdx.x * kCols;
  const int row0 = blockIdx.y * 8 * R;
  const int64_t batch = blockIdx.z;
  B += batch * stride_b;
  C += batch * stride_c;
  for (int i = threadIdx.x; i < 8 * R * K; i += kThreads) {
    const int r = i / K, k = i % K;
    As[i] = (row0 + r < M) ? A[(int64_t)(row0 + r) * lda + k] : 0.f;
  }
  float4 acc[R];
#pragma unroll
  for (int i = 0; i < R; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  const int64_t col = col0 + 4 * lane;
  for (int k0 = 0; k0 < K; k0 += kChunk) {
    const int kc = min(kChunk, K - k0);
    __syncthreads();
    for (int i = threadIdx.x; i < kc * (kCols / 4); i += kThreads) {
      const int r = i / (kCols / 4), c4 = i % (kCols / 4);
      const int64_t gc = col0 + 4 * c4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      const float* row = B + (int64_t)(k0 + r) * ldb;
      if (kAligned) {
        if (gc < J) v = *reinterpret_cast<const float4*>(row + gc);
      } else {
        if (gc < J) v.x = row[gc];
        if (gc + 1 < J) v.y = row[gc + 1];
        if (gc + 2 < J) v.z = row[gc + 2];
        if (gc + 3 < J) v.w = row[gc + 3];
      }
      *reinterpret_cast<float4*>(Bs + r * kCols + 4 * c4) = v;
    }
    __syncthreads();
    for (int kk = 0; kk < kc; ++kk) {
      const float4 b = *reinterpret_cast<const float4*>(Bs + kk * kCols + 4 * lane);
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const float a = As[(warp + 8 * i) * K + k0 + kk];
        acc[i].x = fmaf(a, b.x, acc[i].x);
        acc[i].y = fmaf(a, b.y, acc[i].y);
        acc[i].z = fmaf(a, b.z, acc[i].z);
        acc[i].w = fmaf(a, b.w, acc[i].w);
      }
    }
  }
  if (col >= J) return;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int row = row0 + warp + 8 * i;
    if (row >= M) break;
    float4 v = acc[i];
    if (kAligned) {
      float4* out = reinterpret_cast<float4*>(C + (int64_t)row * ldc + col);
      if (accumulate) {
        const float4 o = *out;
        v.x += o.x;
        v.y += o.y;
        v.z += o.z;
        v.w += o.w;
      }
      *out = v;
    } else {
      float* out = C + (int64_t)row * ldc + col;
      const float vals[4] = {v.x, v.y, v.z, v.w};
      for (int q = 0; q < 4; ++q)
        if (col + q < J) out[q] = accumulate ? out[q] + vals[q] : vals[q];
    }
  }
}

// ---- streaming forms for a short inner dimension -----------------------------------------------------------------
//
// Column-stationary (K <= 64): a thread keeps the K values of its two columns of B in registers and walks the rows of
// A (shared memory, read as float4 broadcasts), writing each output row as it goes; B is read once, C once.
// Row-stationary (M <= 64, any K): a thread keeps the M outputs of its two columns in registers and streams the rows
// of B past the columns of A (A^T in shared memory). Both add the products over k in increasing order with fused
// multiply-adds, as the tiled kernel above does.
constexpr int kStreamThreads = 128;
constexpr int kStreamRows = 128;  // rows of A per block of the column-stationary form

// kMode: 0 C = A B, 1 C += A B, 2 C = A B plus, in the first of every four columns, the matching element of F (the
// means [M, J / 4] of a store of LD moment quadruples, the others zero), i.e. C = A B + the quadruples (F, 0, 0, 0)
// without reading C (pairs of columns only)
template <int kKP, bool kPair, int kMode>
__global__ void __launch_bounds__(kStreamThreads) gemm_cols_kernel(const float* __restrict__ A, int64_t lda,
                                                                  const float* __restrict__ B, int64_t ldb,
                                                                  float* __restrict__ C, int64_t ldc, int M, int K,
                                                                  int64_t J, int64_t stride_b, int64_t stride_c,
                                                                  const float* __restrict__ F, int64_t ldf,
                                                                  int64_t stride_f) {
  constexpr bool kAccumulate = kMode == 1;
  extern __shared__ float4 s_a4[];
  float (*As)[kKP] = reinterpret_cast<float (*)[kKP]>(s_a4);  // [kStreamRows + 3][kKP], zero past the tile
  constexpr int kCols = kPair ? 2 : 1;
  const int row0 = blockIdx.y * kStreamRows;
  const int rows = min(kStreamRows, M - row0);
  for (int i = threadIdx.x; i < (kStreamRows + 3) * kKP; i += kStreamThreads) {
    const int r = i / kKP, k = i % kKP;
    As[r][k] = (r < rows && k < K) ? A[(int64_t)(row0 + r) * lda + k] : 0.f;
  }
  B += blockIdx.z * stride_b;
  C += blockIdx.z * stride_c;
  if (kMode == 2) F += blockIdx.z * stride_f;
  const int64_t col = ((int64_t)blockIdx.x * kStreamThreads + threadIdx.x) * kCols;
  const bool valid = col < J;
  float b0[kKP], b1[kKP];
#pragma unroll
  for (int k = 0; k < kKP; ++k) {
    b0[k] = 0.f;
    b1[k] = 0.f;
    if (valid && k < K) {
      if (kPair) {
        const float2 v = *reinterpret_cast<const float2*>(B + (int64_t)k * ldb + col);
        b0[k] = v.x;
        b1[k] = v.y;
      } else {
        b0[k] = B[(int64_t)k * ldb + col];
      }
    }
  }
  __syncthreads();
  if (!valid) return;
  // four rows at a time: eight independent multiply-add chains per thread
  for (int r0 = 0; r0 < rows; r0 += 4) {
    float a0[4] = {0.f, 0.f, 0.f, 0.f}, a1[4] = {0.f, 0.f, 0.f, 0.f};
    // the four means (first column of each quadruple) are loaded before the products, which hide their latency
    float f[4] = {0.f, 0.f, 0.f, 0.f};
    if (kMode == 2 && (col & 3) == 0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) f[q] = r0 + q < rows ? F[(int64_t)(row0 + r0 + q) * ldf + (col >> 2)] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kKP; k += 4) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 a = *reinterpret_cast<const float4*>(&As[r0 + q][k]);  // rows past the tile are zero
        a0[q] = fmaf(a.x, b0[k], a0[q]);
        a0[q] = fmaf(a.y, b0[k + 1], a0[q]);
        a0[q] = fmaf(a.z, b0[k + 2], a0[q]);
        a0[q] = fmaf(a.w, b0[k + 3], a0[q]);
        if (kPair) {
          a1[q] = fmaf(a.x, b1[k], a1[q]);
          a1[q] = fmaf(a.y, b1[k + 1], a1[q]);
          a1[q] = fmaf(a.z, b1[k + 2], a1[q]);
          a1[q] = fmaf(a.w, b1[k + 3], a1[q]);
        }
      }
    }
    float* out = C + (int64_t)(row0 + r0) * ldc + col;
    if (kAccumulate) {  // the four loads before the first store
      float2 o[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        o[q] = make_float2(0.f, 0.f);
        if (r0 + q < rows) {
          if (kPair) o[q] = *reinterpret_cast<const float2*>(out + (int64_t)q * ldc);
          else o[q].x = out[(int64_t)q * ldc];
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a0[q] += o[q].x;
        a1[q] += o[q].y;
      }
    }
    if (kMode == 2 && (col & 3) == 0) {  // the means added before the first store
#pragma unroll
      for (int q = 0; q < 4; ++q) a0[q] += f[q];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (r0 + q >= rows) break;
      if (kPair) *reinterpret_cast<float2*>(out + (int64_t)q * ldc) = make_float2(a0[q], a1[q]);
      else out[(int64_t)q * ldc] = a0[q];
    }
  }
}

template <int kMP, bool kPair, bool kAccumulate>
__global__ void __launch_bounds__(kStreamThreads) gemm_rows_kernel(const float* __restrict__ A, int64_t lda,
                                                                  const float* __restrict__ B, int64_t ldb,
                                                                  float* __restrict__ C, int64_t ldc, int M, int K,
                                                                  int64_t J, int64_t stride_b, int64_t stride_c) {
  extern __shared__ float4 s_at4[];
  float* At = reinterpret_cast<float*>(s_at4);  // [K][kMP], A transposed, zero rows past M
  constexpr int kCols = kPair ? 2 : 1;
  for (int i = threadIdx.x; i < K * kMP; i += kStreamThreads) {
    const int k = i / kMP, r = i % kMP;
    At[i] = r < M ? A[(int64_t)r * lda + k] : 0.f;
  }
  B += blockIdx.z * stride_b;
  C += blockIdx.z * stride_c;
  const int64_t col = ((int64_t)blockIdx.x * kStreamThreads + threadIdx.x) * kCols;
  const bool valid = col < J;
  __syncthreads();
  if (!valid) return;
  float c0[kMP], c1[kMP];
#pragma unroll
  for (int r = 0; r < kMP; ++r) c0[r] = c1[r] = 0.f;
  // the loads of kU consecutive rows of B are issued before their products, so that every warp keeps kU loads in
  // flight instead of one (the sums still run over k in order)
  constexpr int kU = 8;
  auto load_b = [&](int k, float& x0, float& x1) {
    if (kPair) {
      const float2 v = __ldg(reinterpret_cast<const float2*>(B + (int64_t)k * ldb + col));
      x0 = v.x;
      x1 = v.y;
    } else {
      x0 = __ldg(B + (int64_t)k * ldb + col);
      x1 = 0.f;
    }
  };
  auto product = [&](int k, float x0, float x1) {
    const float* at = At + k * kMP;
#pragma unroll
    for (int r = 0; r < kMP; r += 4) {
      const float4 a = *reinterpret_cast<const float4*>(at + r);
      c0[r] = fmaf(a.x, x0, c0[r]);
      c0[r + 1] = fmaf(a.y, x0, c0[r + 1]);
      c0[r + 2] = fmaf(a.z, x0, c0[r + 2]);
      c0[r + 3] = fmaf(a.w, x0, c0[r + 3]);
      if (kPair) {
        c1[r] = fmaf(a.x, x1, c1[r]);
        c1[r + 1] = fmaf(a.y, x1, c1[r + 1]);
        c1[r + 2] = fmaf(a.z, x1, c1[r + 2]);
        c1[r + 3] = fmaf(a.w, x1, c1[r + 3]);
      }
    }
  };
  int k = 0;
  for (; k + kU <= K; k += kU) {
    float x0[kU], x1[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) load_b(k + u, x0[u], x1[u]);
#pragma unroll
    for (int u = 0; u < kU; ++u) product(k + u, x0[u], x1[u]);
  }
  for (; k < K; ++k) {
    float x0, x1;
    load_b(k, x0, x1);
    product(k, x0, x1);
  }
  if (kAccumulate) {  // eight rows' loads before their stores
#pragma unroll
    for (int r8 = 0; r8 < kMP; r8 += 8) {
      float2 o[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        o[q] = make_float2(0.f, 0.f);
        if (r8 + q < M) {
          const float* in = C + (int64_t)(r8 + q) * ldc + col;
          if (kPair) o[q] = *reinterpret_cast<const float2*>(in);
          else o[q].x = *in;
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        if (r8 + q < kMP) {
          c0[r8 + q] += o[q].x;
          c1[r8 + q] += o[q].y;
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < kMP; ++r) {
    if (r >= M) break;
    float* out = C + (int64_t)r * ldc + col;
    if (kPair) *reinterpret_cast<float2*>(out) = make_float2(c0[r], c1[r]);
    else *out = c0[r];
  }
}

template <int kKP, bool kPair, int kMode>
int launch_cols(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int M, int K,
                int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c, cudaStream_t s,
                const float* F = nullptr, int64_t ldf = 0, int64_t stride_f = 0) {
  const int64_t cols_per_block = (int64_t)kStreamThreads * (kPair ? 2 : 1);
  const size_t smem = (size_t)(kStreamRows + 3) * kKP * sizeof(float);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(gemm_cols_kernel<kKP, kPair, kMode>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "citrus_small_k_gemm: %s", cudaGetErrorString(e));
  }
  dim3 grid((unsigned)cdiv(J, cols_per_block), (unsigned)cdiv(M, kStreamRows), (unsigned)batch);
  gemm_cols_kernel<kKP, kPair, kMode><<<grid, kStreamThreads, smem, s>>>(A, lda, B, ldb, C, ldc, M, K, J, stride_b,
                                                                        stride_c, F, ldf, stride_f);
  note_launches();
  return launch_status("citrus_small_k_gemm");
}

template <int kMP, bool kPair, bool kAcc>
int launch_rows(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int M, int K,
                int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c, cudaStream_t s) {
  const size_t smem = (size_t)K * kMP * sizeof(float);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(gemm_rows_kernel<kMP, kPair, kAcc>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "citrus_small_k_gemm: %s", cudaGetErrorString(e));
  }
  const int64_t cols_per_block = (int64_t)kStreamThreads * (kPair ? 2 : 1);
  dim3 grid((unsigned)cdiv(J, cols_per_block), 1, (unsigned)batch);
  gemm_rows_kernel<kMP, kPair, kAcc><<<grid, kStreamThreads, smem, s>>>(A, lda, B, ldb, C, ldc, M, K, J, stride_b,
                                                                       stride_c);
  note_launches();
  return launch_status("citrus_small_k_gemm");
}

template <bool kPair, bool kAcc>
int launch_stream(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int M, int K,
                  int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c, cudaStream_t s) {
  if (K <= 16) return launch_cols<16, kPair, kAcc>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, s);
  if (K <= 32) return launch_cols<32, kPair, kAcc>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, s);
  if (K <= 36) return launch_cols<36, kPair, kAcc>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, s);
  if (K <= 48) return launch_cols<48, kPair, kAcc>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, s);
  if (K <= 64) return launch_cols<64, kPair, kAcc>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, s);
  if (M <= 16) return launch_rows<16, kPair, kAcc>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, s);
  if (M <= 32) return launch_rows<32, kPair, kAcc>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, s);
  if (M <= 36) return launch_rows<36, kPair, kAcc>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, s);
  if (M <= 48) return launch_rows<48, kPair, kAcc>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, s);
  return launch_rows<64, kPair, kAcc>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, s);
}

template <int R, bool kAligned>
int launch_variant(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int M, int K,
                   int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c, int accumulate, cudaStream_t stream) {
  const size_t smem = ((size_t)8 * R * K + (size_t)kChunk * kCols) * sizeof(float);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(small_k_gemm_kernel<R, kAligned>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "citrus_small_k_gemm: %s", cudaGetErrorString(e));
  }
  dim3 grid((unsigned)cdiv(J, kCols), (unsigned)cdiv(M, 8 * R), (unsigned)batch);
  small_k_gemm_kernel<R, kAligned><<<grid, kThreads, smem, stream>>>(A, lda, B, ldb, C, ldc, M, K, J, stride_b,
                                                                     stride_c, accumulate);
  note_launches();
  return launch_status("citrus_small_k_gemm");
}

template <int R>
int launch(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int M, int K, int64_t J,
           int64_t batch, int64_t stride_b, int64_t stride_c, int accumulate, cudaStream_t stream) {
  const bool aligned = J % 4 == 0 && ldb % 4 == 0 && ldc % 4 == 0 && stride_b % 4 == 0 && stride_c % 4 == 0 &&
                       ((uintptr_t)B % 16) == 0 && ((uintptr_t)C % 16) == 0;
  if (aligned) return launch_variant<R, true>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, accumulate,
                                              stream);
  return launch_variant<R, false>(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, accumulate, stream);
}

}  // namespace
}  // namespace citrus

using namespace citrus;

namespace {

int launch_tiled(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int m, int k,
                 int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c, int accumulate, int tile_rows,
                 cudaStream_t s) {
  switch (tile_rows) {
    case 1: return launch<1>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, accumulate, s);
    case 2: return launch<2>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, accumulate, s);
    case 3: return launch<3>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, accumulate, s);
    case 4: return launch<4>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, accumulate, s);
    case 5: return launch<5>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, accumulate, s);
    case 6: return launch<6>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, accumulate, s);
    case 8: return launch<8>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, accumulate, s);
    case 12: return launch<12>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, accumulate, s);
    case 16: return launch<16>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, accumulate, s);
    default: return set_error(CITRUS_EINVAL, "citrus_small_k_gemm: tile of %d row groups (1-6, 8, 12 or 16)",
                              tile_rows);
  }
}

}  // namespace

extern "C" int citrus_small_k_gemm_config(const float* A, int64_t lda, const float* B, int64_t ldb, float* C,
                                          int64_t ldc, int64_t M, int64_t K, int64_t J, int64_t batch,
                                          int64_t stride_b, int64_t stride_c, int32_t accumulate, int32_t variant,
                                          int32_t tile_rows, void* stream) {
  CITRUS_REQUIRE(A && B && C, "citrus_small_k_gemm: null pointer argument");
  CITRUS_REQUIRE(M >= 1 && K >= 1 && J >= 0 && batch >= 1 && batch <= 65535,
                 "citrus_small_k_gemm: bad sizes M %lld K %lld J %lld batch %lld", (long long)M, (long long)K,
                 (long long)J, (long long)batch);
  CITRUS_REQUIRE(K <= 1024 && M <= (1 << 20), "citrus_small_k_gemm: K %lld or M %lld too large", (long long)K,
                 (long long)M);
  CITRUS_REQUIRE(lda >= K && ldb >= J && ldc >= J, "citrus_small_k_gemm: leading dimensions too small");
  CITRUS_REQUIRE(variant >= 0 && variant <= 2, "citrus_small_k_gemm: variant %d (0 auto, 1 streaming, 2 tiled)",
                 variant);
  if (J == 0) return CITRUS_OK;
  const int m = (int)M, k = (int)K;
  const int rows = (m + 7) / 8;
  cudaStream_t s = as_stream(stream);
  const bool streaming_fits = K <= 64 || (M <= 64 && K * 64 * 4 <= 200 * 1024);
  CITRUS_REQUIRE(variant != 1 || streaming_fits,
                 "citrus_small_k_gemm: the streaming forms need K <= 64, or M <= 64 with K <= 800");
  if (variant == 1 || (variant == 0 && streaming_fits)) {
    const bool pair = J % 2 == 0 && ldb % 2 == 0 && ldc % 2 == 0 && stride_b % 2 == 0 && stride_c % 2 == 0 &&
                      ((uintptr_t)B % 8) == 0 && ((uintptr_t)C % 8) == 0;
    if (pair && accumulate)
      return launch_stream<true, true>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, s);
    if (pair) return launch_stream<true, false>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, s);
    if (accumulate) return launch_stream<false, true>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, s);
    return launch_stream<false, false>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, s);
  }
  int tile = tile_rows;
  if (tile == 0) {
    static const int kTiles[] = {1, 2, 3, 4, 5, 6, 8, 12, 16};
    tile = 16;
    for (int t : kTiles)
      if (rows <= t) {
        tile = t;
        break;
      }
  }
  if (8ll * tile * K * 4 + kChunk * kCols * 4 > 200 * 1024)
    return set_error(CITRUS_EINVAL, "citrus_small_k_gemm: K %lld too large for a shared-memory tile of %d row groups",
                     (long long)K, tile);
  return launch_tiled(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, accumulate, tile, s);
}

extern "C" int citrus_source_expansion_first(const float* A, int64_t lda, const float* B, int64_t ldb, float* C,
                                             int64_t ldc, const float* F, int64_t ldf, int64_t M, int64_t K,
                                             int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c,
                                             int64_t stride_f, void* stream) {
  CITRUS_REQUIRE(A && B && C && F, "citrus_source_expansion_first: null pointer argument");
  CITRUS_REQUIRE(M >= 1 && K >= 1 && K <= 64 && J >= 0 && batch >= 1 && batch <= 65535 && M <= (1 << 20),
                 "citrus_source_expansion_first: bad sizes M %lld K %lld (at most 64) J %lld batch %lld",
                 (long long)M, (long long)K, (long long)J, (long long)batch);
  CITRUS_REQUIRE(lda >= K && ldb >= J && ldc >= J && ldf >= J / 4,
                 "citrus_source_expansion_first: leading dimensions too small");
  CITRUS_REQUIRE(J % 4 == 0 && ldb % 2 == 0 && ldc % 2 == 0 && stride_b % 2 == 0 && stride_c % 2 == 0 &&
                     ((uintptr_t)B % 8) == 0 && ((uintptr_t)C % 8) == 0,
                 "citrus_source_expansion_first: columns must come in quadruples of 8-byte aligned pairs");
  if (J == 0) return CITRUS_OK;
  const int m = (int)M, k = (int)K;
  cudaStream_t s = as_stream(stream);
#define CITRUS_EXPAND(KP) \
  launch_cols<KP, true, 2>(A, lda, B, ldb, C, ldc, m, k, J, batch, stride_b, stride_c, s, F, ldf, stride_f)
  if (K <= 16) return CITRUS_EXPAND(16);
  if (K <= 32) return CITRUS_EXPAND(32);
  if (K <= 36) return CITRUS_EXPAND(36);
  if (K <= 48) return CITRUS_EXPAND(48);
  return CITRUS_EXPAND(64);
#undef CITRUS_EXPAND
}

extern "C" int citrus_small_k_gemm(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
                                   int64_t M, int64_t K, int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c,
                                   int32_t accumulate, void* stream) {
  return citrus_small_k_gemm_config(A, lda, B, ldb, C, ldc, M, K, J, batch, stride_b, stride_c, accumulate, 0, 0,
                                    stream);
}
