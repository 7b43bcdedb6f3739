// Training and inference kernels of the learned higher-order proposal: a 3D U-Net on the transport cells that maps
// (densities, first-collided scalar flux) to the scalar flux of the higher collision orders.
//
// Tensors are NCDHW float32 [B, C, D, H, W]; convolution weights are bfloat16 [C_out, C_in, k, k, k] (k = 1 or 3,
// zero padding k / 2, stride 1) with float32 biases; every sum is accumulated in float32.
//
//   * conv_kernel: out = act(bias + w * [A, up(B)]) with the channel concatenation of the decoder and its nearest
//     2x upsampling fused into the input staging (B is read at half resolution), and an optional ReLU. The same kernel
//     runs the input gradient of a convolution (the transposed convolution: flipped taps, swapped channel roles,
//     outputs split back into the A and B parts and the A part masked by its ReLU activation).
//     A CTA computes a 4 x 8 x 8 brick of voxels x 16 output channels; per chunk of 4 input channels the haloed input
//     brick and the chunk's weights (tap-major, 16 output channels contiguous for float4 broadcasts) are staged in
//     shared memory.
//   * wgrad_kernel: weight gradients as fixed-order reductions over (batch, voxel bricks), split over CTAs into
//     partial sums that wgrad_reduce_kernel adds in split order (deterministic).
//   * pooling (2x average), the upsampling's backward pass, MSE and Adam.
#include <cuda_bf16.h>

#include <algorithm>

#include "tcgen05.cuh"

namespace citrus {
namespace {

constexpr int kConvThreads = 256;
constexpr int kTZ = 4, kTY = 8, kTX = 8;  // voxel brick of one CTA (kTZ * kTY * kTX == kConvThreads)
constexpr int kCoT = 16;                  // output channels of one CTA
constexpr int kCiT = 4;                   // input channels per staging step
constexpr int kLearnThreads = 256;

__device__ __forceinline__ float bf16_bits_to_float(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

struct ConvArgs {
  const float* in_a;      // [B, ca, D, H, W]
  const float* in_b;      // [B, cb, D, H, W], or [B, cb, D/2, H/2, W/2] when b_up
  int ca, cb, b_up;
  const uint16_t* w;      // weight element (o, i, t) at w_base + o w_o + i w_i + t w_t
  long long w_o, w_i, w_t, w_base;
  const float* bias;      // [oa + ob] or null
  float* out_a;           // output channels [0, oa)
  float* out_b;           // output channels [oa, oa + ob)
  int oa, ob;
  const float* mask_a;    // out_a *= (mask_a > 0) when set
  int relu;
  int B, D, H, W;
};

template <int kK>
__global__ void __launch_bounds__(kConvThreads) conv_kernel(const ConvArgs a) {
  constexpr int kH = kK / 2;
  constexpr int SZ = kTZ + 2 * kH, SY = kTY + 2 * kH, SX = kTX + 2 * kH, S3 = SZ * SY * SX;
  constexpr int K3 = kK * kK * kK;
  __shared__ float s_in[kCiT * S3];
  __shared__ __align__(16) float s_w[kCiT * K3 * kCoT];

  const int tid = threadIdx.x;
  const int ntx = (a.W + kTX - 1) / kTX, nty = (a.H + kTY - 1) / kTY;
  const int tile = blockIdx.x;
  const int x0 = (tile % ntx) * kTX, y0 = ((tile / ntx) % nty) * kTY, z0 = (tile / (ntx * nty)) * kTZ;
  const int co0 = blockIdx.y * kCoT, b = blockIdx.z;
  const int lx = tid % kTX, ly = (tid / kTX) % kTY, lz = tid / (kTX * kTY);
  const int O = a.oa + a.ob, Ci = a.ca + a.cb;
  const int64_t V = (int64_t)a.D * a.H * a.W;
  const int Dc = a.D >> 1, Hc = a.H >> 1, Wc = a.W >> 1;

  float acc[kCoT];
#pragma unroll
  for (int j = 0; j < kCoT; ++j) acc[j] = (a.bias != nullptr && co0 + j < O) ? a.bias[co0 + j] : 0.f;

  for (int ci0 = 0; ci0 < Ci; ci0 += kCiT) {
    __syncthreads();
    for (int e = tid; e < kCiT * S3; e += kConvThreads) {
      const int c = e / S3, r = e % S3;
      const int gz = z0 + r / (SY * SX) - kH, gy = y0 + (r / SX) % SY - kH, gx = x0 + r % SX - kH;
      const int ci = ci0 + c;
      float v = 0.f;
      if (ci < Ci && gz >= 0 && gz < a.D && gy >= 0 && gy < a.H && gx >= 0 && gx < a.W) {
        if (ci < a.ca) {
          v = __ldg(a.in_a + ((int64_t)b * a.ca + ci) * V + ((int64_t)gz * a.H + gy) * a.W + gx);
        } else if (a.b_up) {
          v = __ldg(a.in_b + (((int64_t)b * a.cb + (ci - a.ca)) * Dc + (gz >> 1)) * Hc * Wc + (int64_t)(gy >> 1) * Wc +
                    (gx >> 1));
        } else {
          v = __ldg(a.in_b + ((int64_t)b * a.cb + (ci - a.ca)) * V + ((int64_t)gz * a.H + gy) * a.W + gx);
        }
      }
      s_in[e] = v;
    }
    for (int e = tid; e < kCiT * K3 * kCoT; e += kConvThreads) {
      const int j = e % kCoT, t = (e / kCoT) % K3, c = e / (kCoT * K3);
      const int o = co0 + j, i = ci0 + c;
      s_w[e] = (o < O && i < Ci) ? bf16_bits_to_float(a.w[a.w_base + o * a.w_o + i * a.w_i + t * a.w_t]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < kCiT; ++c) {
#pragma unroll
      for (int tz = 0; tz < kK; ++tz)
#pragma unroll
        for (int ty = 0; ty < kK; ++ty)
#pragma unroll
          for (int tx = 0; tx < kK; ++tx) {
            const float v = s_in[c * S3 + ((lz + tz) * SY + (ly + ty)) * SX + lx + tx];
            const float4* w4 = reinterpret_cast<const float4*>(s_w + (c * K3 + (tz * kK + ty) * kK + tx) * kCoT);
#pragma unroll
            for (int q = 0; q < kCoT / 4; ++q) {
              const float4 wq = w4[q];
              acc[4 * q + 0] = fmaf(wq.x, v, acc[4 * q + 0]);
              acc[4 * q + 1] = fmaf(wq.y, v, acc[4 * q + 1]);
              acc[4 * q + 2] = fmaf(wq.z, v, acc[4 * q + 2]);
              acc[4 * q + 3] = fmaf(wq.w, v, acc[4 * q + 3]);
            }
          }
    }
  }

  const int x = x0 + lx, y = y0 + ly, z = z0 + lz;
  if (x >= a.W || y >= a.H || z >= a.D) return;
  const int64_t vox = ((int64_t)z * a.H + y) * a.W + x;
#pragma unroll
  for (int j = 0; j < kCoT; ++j) {
    const int o = co0 + j;
    if (o >= O) break;
    float r = a.relu ? fmaxf(acc[j], 0.f) : acc[j];
    if (o < a.oa) {
      const int64_t idx = ((int64_t)b * a.oa + o) * V + vox;
      if (a.mask_a != nullptr && !(a.mask_a[idx] > 0.f)) r = 0.f;
      a.out_a[idx] = r;
    } else {
      a.out_b[((int64_t)b * a.ob + (o - a.oa)) * V + vox] = r;
    }
  }
}

// The same convolution as an implicit GEMM on the tcgen05 tensor cores: D[voxel, o] = sum_k A[voxel, k] B[o, k] with
// k = tap C_in + input channel (tap-major, so that a run of k shares one spatial offset and its bounds test). A CTA
// takes a tile of 128 consecutive voxels (the MMA's M) x n_tile output channels (its N, a multiple of 16 up to 256)
// and walks k in chunks of 64 through two shared-memory stages:
//   * two threads per voxel row gather 32 inputs each (all loads issued before the first store; the concatenation and
//     the upsampling read in place, zero padding outside the volume), split every float32 value into bfloat16 high
//     and low parts and write them in the K-major canonical layout (8-row x 16-byte core matrices, no swizzle);
//   * the chunk's weights, already bfloat16, fill the B operand as they are;
//   * one thread issues 2 x 4 MMAs (M = 128, N = n_tile, K = 16, kind::f16: A_hi B + A_lo B, exact weights, so the
//     product keeps about sixteen bits of every input) into a float32 accumulator in tensor memory and commits them
//     to the stage's mbarrier, while the threads build the other stage;
//   * every wait on an mbarrier is bounded by a wall-clock limit (the CTA records the error and leaves).
// The epilogue reads the accumulator (lane = voxel, column = output channel; the two warp groups take half the
// columns each) and stores 32 consecutive voxels of one channel per warp instruction, with the bias, the ReLU and the
// mask applied.
constexpr int kCvThreads = 256;
constexpr int kCvKC = 64;                     // inner dimension of one stage (four MMA K-steps)
constexpr uint32_t kCvAStep = kTcM * 16 * 2;  // bytes of one K-step of A: 128 rows x 16 bfloat16

inline uint32_t tc_columns(int n_tile) {
  uint32_t c = 32;
  while (c < (uint32_t)n_tile) c <<= 1;
  return c;
}

inline size_t tc_stage_bytes(int n_tile) { return 2 * 4 * (size_t)kCvAStep + 4 * (size_t)n_tile * 32; }

template <int kK>
__global__ void __launch_bounds__(kCvThreads) conv_tc_kernel(const ConvArgs a, int n_tile, int co_tiles,
                                                            int vox_tiles, int64_t num_tiles,
                                                            uint32_t* __restrict__ error_word) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr int K3 = kK * kK * kK;
  constexpr int kH = kK / 2;
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid / 32;
  const int row = tid & (kTcM - 1), half = tid >> 7;   // voxel row of the tile, half of the chunk's k range
  const int O = a.oa + a.ob, Ci = a.ca + a.cb;
  const int Ktot = Ci * K3;
  const int nchunks = (Ktot + kCvKC - 1) / kCvKC;
  const int64_t V = (int64_t)a.D * a.H * a.W;
  const int64_t Vc = (int64_t)(a.D >> 1) * (a.H >> 1) * (a.W >> 1);
  const int Hc = a.H >> 1, Wc = a.W >> 1;
  const uint32_t a_bytes = 4 * kCvAStep;
  const uint32_t b_step = (uint32_t)n_tile * 32;
  const uint32_t stage_bytes = 2 * a_bytes + 4 * b_step;
  const uint32_t cols = n_tile <= 32 ? 32u : n_tile <= 64 ? 64u : n_tile <= 128 ? 128u : 256u;
  const uint32_t idesc = idesc_bf16(n_tile);
  const int n_half = ((n_tile / 16 + 1) / 2) * 16;     // accumulator columns of the first warp group

  if (tid == 0) {
    abort_flag = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  uint32_t phase0 = 0, phase1 = 0;
  bool pending0 = false, pending1 = false;
  bool failed = false;

  for (int64_t tile = blockIdx.x; tile < num_tiles && !failed; tile += gridDim.x) {
    const int vt = (int)(tile % vox_tiles);
    const int64_t rest = tile / vox_tiles;
    const int ct = (int)(rest % co_tiles);
    const int b = (int)(rest / co_tiles);
    const int co0 = ct * n_tile;
    const int64_t vox = (int64_t)vt * kTcM + row;
    const bool vvalid = vox < V;
    const int x = vvalid ? (int)(vox % a.W) : 0;
    const int y = vvalid ? (int)((vox / a.W) % a.H) : 0;
    const int z = vvalid ? (int)(vox / ((int64_t)a.W * a.H)) : 0;
    const float* src_a = a.in_a + (int64_t)b * a.ca * V;
    const float* src_b = a.in_b + (int64_t)b * a.cb * (a.b_up ? Vc : V);
    for (int c = 0; c < nchunks; ++c) {
      const int st = c & 1;
      uint8_t* sa_hi = smem + st * stage_bytes;
      uint8_t* sa_lo = sa_hi + a_bytes;
      uint8_t* sb = sa_lo + a_bytes;
      // the stage's previous MMAs must be done before its operands are overwritten
      if (st == 0 ? pending0 : pending1) {
        const bool ok = mbar_wait(smem_u32(&mbar[st]), st == 0 ? phase0 : phase1, global_timer_ns());
        if (st == 0) { phase0 ^= 1u; pending0 = false; } else { phase1 ^= 1u; pending1 = false; }
        if (!ok) abort_flag = 1;
      }
      // A: this thread's 32 inputs of the chunk, k = tap Ci + ci
      {
        const int k0 = c * kCvKC + half * 32;
        int t = k0 / Ci, ci = k0 - t * Ci;
        int64_t off_a = 0, off_b = 0;
        bool inb = false;
        int t_cur = -1;
        float xv[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          float v = 0.f;
          if (t < K3) {
            if (t != t_cur) {  // a new tap: its spatial offset and bounds test, shared by the run of channels
              t_cur = t;
              const int gz = z + t / (kK * kK) - kH, gy = y + (t / kK) % kK - kH, gx = x + t % kK - kH;
              inb = vvalid && gz >= 0 && gz < a.D && gy >= 0 && gy < a.H && gx >= 0 && gx < a.W;
              off_a = ((int64_t)gz * a.H + gy) * a.W + gx;
              off_b = a.b_up ? ((int64_t)(gz >> 1) * Hc + (gy >> 1)) * Wc + (gx >> 1) : off_a;
            }
            if (inb)
              v = ci < a.ca ? __ldg(src_a + (int64_t)ci * V + off_a)
                            : __ldg(src_b + (int64_t)(ci - a.ca) * (a.b_up ? Vc : V) + off_b);
          }
          xv[q] = v;
          if (++ci == Ci) {
            ci = 0;
            ++t;
          }
        }
#pragma unroll
        for (int g8 = 0; g8 < 4; ++g8) {
          uint4 hi, lo;
          split_pair(xv[8 * g8 + 0], xv[8 * g8 + 1], hi.x, lo.x);
          split_pair(xv[8 * g8 + 2], xv[8 * g8 + 3], hi.y, lo.y);
          split_pair(xv[8 * g8 + 4], xv[8 * g8 + 5], hi.z, lo.z);
          split_pair(xv[8 * g8 + 6], xv[8 * g8 + 7], hi.w, lo.w);
          const int kk8 = half * 32 + g8 * 8;
          const uint32_t off = (uint32_t)(kk8 >> 4) * kCvAStep + core_offset(row, kk8 & 15);
          *reinterpret_cast<uint4*>(sa_hi + off) = hi;
          *reinterpret_cast<uint4*>(sa_lo + off) = lo;
        }
      }
      // B: n_tile output channels x the chunk's 64 weights, 8 at a time
      for (int u = tid; u < n_tile * 8; u += kCvThreads) {
        const int brow = u >> 3, g8 = u & 7;
        const int o = co0 + brow;
        const int k0 = c * kCvKC + g8 * 8;
        int t = k0 / Ci, i = k0 - t * Ci;
        uint32_t w2[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint32_t pair = 0;
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            uint32_t bits = 0;
            if (o < O && t < K3) bits = a.w[a.w_base + o * a.w_o + i * a.w_i + t * a.w_t];
            pair |= bits << (16 * h);
            if (++i == Ci) {
              i = 0;
              ++t;
            }
          }
          w2[q] = pair;
        }
        const uint32_t off = (uint32_t)(g8 >> 1) * b_step + core_offset(brow, (g8 & 1) * 8);
        *reinterpret_cast<uint4*>(sb + off) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (abort_flag) {
        failed = true;
        break;
      }
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int s4 = 0; s4 < 4; ++s4) {
          const uint64_t ah = smem_desc(smem_u32(sa_hi + s4 * kCvAStep), 128, 256);
          const uint64_t al = smem_desc(smem_u32(sa_lo + s4 * kCvAStep), 128, 256);
          const uint64_t bd = smem_desc(smem_u32(sb + s4 * b_step), 128, 256);
          mma_bf16(tmem, ah, bd, idesc, (c > 0 || s4 > 0) ? 1u : 0u);
          mma_bf16(tmem, al, bd, idesc, 1u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&mbar[st]))
                     : "memory");
      }
      if (st == 0) pending0 = true; else pending1 = true;
    }
    // every MMA of the tile done (both stages drained)
    if (pending0) {
      if (!mbar_wait(smem_u32(&mbar[0]), phase0, global_timer_ns())) abort_flag = 1;
      phase0 ^= 1u;
      pending0 = false;
    }
    if (pending1) {
      if (!mbar_wait(smem_u32(&mbar[1]), phase1, global_timer_ns())) abort_flag = 1;
      phase1 ^= 1u;
      pending1 = false;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (abort_flag || failed) {
      failed = true;
      break;
    }
    // epilogue: accumulator lane = voxel row, columns = output channels; warps 0-3 take columns [0, n_half), warps
    // 4-7 the rest, each warp its own 32 lanes
    {
      const int j_lo = half == 0 ? 0 : n_half, j_hi = half == 0 ? n_half : n_tile;
#pragma unroll 1
      for (int j0 = j_lo; j0 < j_hi; j0 += 16) {
        uint32_t r[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
            "%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)j0)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (vvalid) {
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int o = co0 + j0 + q;
            if (o < O) {
              float val = __uint_as_float(r[q]) + (a.bias != nullptr ? a.bias[o] : 0.f);
              if (a.relu) val = fmaxf(val, 0.f);
              if (o < a.oa) {
                const int64_t idx = ((int64_t)b * a.oa + o) * V + vox;
                if (a.mask_a != nullptr && !(a.mask_a[idx] > 0.f)) val = 0.f;
                a.out_a[idx] = val;
              } else {
                a.out_b[((int64_t)b * a.ob + (o - a.oa)) * V + vox] = val;
              }
            }
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // the accumulator is free for the next tile
  }
  if (failed && tid == 0 && error_word != nullptr) atomicExch(error_word, 1u);
  // leave only after the tensor cores are done with this CTA's shared memory and tensor memory
  if (pending0) mbar_wait(smem_u32(&mbar[0]), phase0, global_timer_ns());
  if (pending1) mbar_wait(smem_u32(&mbar[1]), phase1, global_timer_ns());
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols) : "memory");
}

// grad_w[o, i, t] partial sums over the bricks s, s + S, s + 2S, ... of (batch x voxel bricks):
// sum g[b, o](x) in_i(x + off(t)); in_i is the concatenation [A, up(B)] of the forward pass.
template <int kK, int kCiW>
__global__ void __launch_bounds__(kConvThreads) wgrad_kernel(const float* __restrict__ g, int Co,
                                                            const float* __restrict__ in_a, int ca,
                                                            const float* __restrict__ in_b, int cb, int b_up,
                                                            float* __restrict__ partial, int splits, int B, int D,
                                                            int H, int W) {
  constexpr int kH = kK / 2;
  constexpr int SZ = kTZ + 2 * kH, SY = kTY + 2 * kH, SX = kTX + 2 * kH, S3 = SZ * SY * SX;
  constexpr int K3 = kK * kK * kK;
  constexpr int kVox = kTZ * kTY * kTX;
  static_assert(kCiW * K3 <= kConvThreads, "one thread per (input channel, tap)");
  __shared__ __align__(16) float s_g[kVox * kCoT];
  __shared__ float s_in[kCiW * S3];

  const int tid = threadIdx.x;
  const int co0 = blockIdx.x * kCoT, ci0 = blockIdx.y * kCiW, split = blockIdx.z;
  const int Ci = ca + cb;
  const int c_own = tid / K3, t_own = tid % K3;
  const int tz = t_own / (kK * kK), ty = (t_own / kK) % kK, tx = t_own % kK;
  const bool active = tid < kCiW * K3;
  const int ntx = (W + kTX - 1) / kTX, nty = (H + kTY - 1) / kTY, ntz = (D + kTZ - 1) / kTZ;
  const int tiles = ntx * nty * ntz;
  const int64_t V = (int64_t)D * H * W;
  const int Dc = D >> 1, Hc = H >> 1, Wc = W >> 1;

  float acc[kCoT];
#pragma unroll
  for (int j = 0; j < kCoT; ++j) acc[j] = 0.f;

  for (int brick = split; brick < B * tiles; brick += splits) {
    const int b = brick / tiles, tile = brick % tiles;
    const int x0 = (tile % ntx) * kTX, y0 = ((tile / ntx) % nty) * kTY, z0 = (tile / (ntx * nty)) * kTZ;
    __syncthreads();
    for (int e = tid; e < kVox * kCoT; e += kConvThreads) {
      const int j = e / kVox, v = e % kVox;
      const int x = x0 + v % kTX, y = y0 + (v / kTX) % kTY, z = z0 + v / (kTX * kTY);
      const int o = co0 + j;
      float val = 0.f;
      if (o < Co && x < W && y < H && z < D) val = __ldg(g + ((int64_t)b * Co + o) * V + ((int64_t)z * H + y) * W + x);
      s_g[v * kCoT + j] = val;
    }
    for (int e = tid; e < kCiW * S3; e += kConvThreads) {
      const int c = e / S3, r = e % S3;
      const int gz = z0 + r / (SY * SX) - kH, gy = y0 + (r / SX) % SY - kH, gx = x0 + r % SX - kH;
      const int ci = ci0 + c;
      float v = 0.f;
      if (ci < Ci && gz >= 0 && gz < D && gy >= 0 && gy < H && gx >= 0 && gx < W) {
        if (ci < ca) {
          v = __ldg(in_a + ((int64_t)b * ca + ci) * V + ((int64_t)gz * H + gy) * W + gx);
        } else if (b_up) {
          v = __ldg(in_b + (((int64_t)b * cb + (ci - ca)) * Dc + (gz >> 1)) * Hc * Wc + (int64_t)(gy >> 1) * Wc +
                    (gx >> 1));
        } else {
          v = __ldg(in_b + ((int64_t)b * cb + (ci - ca)) * V + ((int64_t)gz * H + gy) * W + gx);
        }
      }
      s_in[e] = v;
    }
    __syncthreads();
    if (active) {
      const float* src = s_in + c_own * S3 + (tz * SY + ty) * SX + tx;
#pragma unroll 4
      for (int v = 0; v < kVox; ++v) {
        const int lx = v % kTX, ly = (v / kTX) % kTY, lz = v / (kTX * kTY);
        const float val = src[(lz * SY + ly) * SX + lx];
        const float4* g4 = reinterpret_cast<const float4*>(s_g + v * kCoT);
#pragma unroll
        for (int q = 0; q < kCoT / 4; ++q) {
          const float4 gq = g4[q];
          acc[4 * q + 0] = fmaf(gq.x, val, acc[4 * q + 0]);
          acc[4 * q + 1] = fmaf(gq.y, val, acc[4 * q + 1]);
          acc[4 * q + 2] = fmaf(gq.z, val, acc[4 * q + 2]);
          acc[4 * q + 3] = fmaf(gq.w, val, acc[4 * q + 3]);
        }
      }
    }
  }
  const int i = ci0 + c_own;
  if (!active || i >= Ci) return;
  const int64_t nW = (int64_t)Co * Ci * K3;
#pragma unroll
  for (int j = 0; j < kCoT; ++j) {
    const int o = co0 + j;
    if (o < Co) partial[(int64_t)split * nW + ((int64_t)o * Ci + i) * K3 + t_own] = acc[j];
  }
}

__global__ void wgrad_reduce_kernel(const float* __restrict__ partial, int splits, int64_t n,
                                    float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * kLearnThreads + threadIdx.x;
  if (i >= n) return;
  float s = 0.f;
  for (int k = 0; k < splits; ++k) s += partial[(int64_t)k * n + i];
  out[i] = s;
}

// grad_bias[o] = sum over batch and voxels of g[b, o] (one block per output channel, fixed order)
__global__ void __launch_bounds__(kLearnThreads) bias_grad_kernel(const float* __restrict__ g, int Co, int B,
                                                                 int64_t V, float* __restrict__ out) {
  const int o = blockIdx.x;
  float s = 0.f;
  for (int b = 0; b < B; ++b) {
    const float* src = g + ((int64_t)b * Co + o) * V;
    for (int64_t t = threadIdx.x; t < V; t += kLearnThreads) s += src[t];
  }
  __shared__ float red[kLearnThreads];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = kLearnThreads / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[o] = red[0];
}

// out[bc](z, y, x) = mean of the 2 x 2 x 2 children of in[bc] (D, H, W even)
__global__ void pool_kernel(const float* __restrict__ in, float* __restrict__ out, int64_t BC, int D, int H, int W) {
  const int Dc = D / 2, Hc = H / 2, Wc = W / 2;
  const int64_t n = BC * Dc * Hc * Wc;
  const int64_t i = (int64_t)blockIdx.x * kLearnThreads + threadIdx.x;
  if (i >= n) return;
  const int x = (int)(i % Wc), y = (int)((i / Wc) % Hc), z = (int)((i / ((int64_t)Wc * Hc)) % Dc);
  const int64_t bc = i / ((int64_t)Wc * Hc * Dc);
  const float* src = in + bc * D * H * W;
  float s = 0.f;
  for (int dz = 0; dz < 2; ++dz)
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) s += src[((int64_t)(2 * z + dz) * H + 2 * y + dy) * W + 2 * x + dx];
  out[i] = 0.125f * s;
}

// grad_in[bc](fine) = ((accumulate ? grad_in : 0) + grad_out[bc](fine / 2) / 8) * (mask > 0 when set)
__global__ void pool_backward_kernel(const float* __restrict__ grad_out, float* __restrict__ grad_in,
                                     const float* __restrict__ mask, int accumulate, int64_t BC, int D, int H, int W) {
  const int64_t n = BC * D * H * W;
  const int64_t i = (int64_t)blockIdx.x * kLearnThreads + threadIdx.x;
  if (i >= n) return;
  const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)((i / ((int64_t)W * H)) % D);
  const int64_t bc = i / ((int64_t)W * H * D);
  const int Dc = D / 2, Hc = H / 2, Wc = W / 2;
  float r = 0.125f * grad_out[((bc * Dc + z / 2) * Hc + y / 2) * Wc + x / 2];
  if (accumulate) r += grad_in[i];
  if (mask != nullptr && !(mask[i] > 0.f)) r = 0.f;
  grad_in[i] = r;
}

// grad_coarse[bc](p) = (sum of grad_fine over the 8 children of p) * (mask_coarse(p) > 0 when set)
__global__ void upsample_backward_kernel(const float* __restrict__ grad_fine, const float* __restrict__ mask,
                                         float* __restrict__ grad_coarse, int64_t BC, int Dc, int Hc, int Wc) {
  const int64_t n = BC * Dc * Hc * Wc;
  const int64_t i = (int64_t)blockIdx.x * kLearnThreads + threadIdx.x;
  if (i >= n) return;
  const int x = (int)(i % Wc), y = (int)((i / Wc) % Hc), z = (int)((i / ((int64_t)Wc * Hc)) % Dc);
  const int64_t bc = i / ((int64_t)Wc * Hc * Dc);
  const int D = 2 * Dc, H = 2 * Hc, W = 2 * Wc;
  const float* src = grad_fine + bc * D * H * W;
  float s = 0.f;
  for (int dz = 0; dz < 2; ++dz)
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) s += src[((int64_t)(2 * z + dz) * H + 2 * y + dy) * W + 2 * x + dx];
  if (mask != nullptr && !(mask[i] > 0.f)) s = 0.f;
  grad_coarse[i] = s;
}

// grad = 2 (pred - target) / n; partial[block] = sum of the block's squared errors
__global__ void __launch_bounds__(kLearnThreads) mse_kernel(const float* __restrict__ pred,
                                                           const float* __restrict__ target, int64_t n,
                                                           float* __restrict__ grad, float* __restrict__ partial) {
  const int64_t i = (int64_t)blockIdx.x * kLearnThreads + threadIdx.x;
  float e = 0.f;
  if (i < n) {
    const float d = pred[i] - target[i];
    grad[i] = 2.f * d / (float)n;
    e = d * d;
  }
  __shared__ float red[kLearnThreads];
  red[threadIdx.x] = e;
  __syncthreads();
  for (int s = kLearnThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, uint16_t* __restrict__ p_bf16, int64_t n, float lr, float beta1,
                            float beta2, float eps, float c1, float c2) {
  const int64_t i = (int64_t)blockIdx.x * kLearnThreads + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = beta1 * m[i] + (1.f - beta1) * gi;
  const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  p[i] = pi;
  if (p_bf16 != nullptr) p_bf16[i] = __bfloat16_as_ushort(__float2bfloat16_rn(pi));
}

__global__ void to_bf16_kernel(const float* __restrict__ src, uint16_t* __restrict__ dst, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * kLearnThreads + threadIdx.x;
  if (i < n) dst[i] = __bfloat16_as_ushort(__float2bfloat16_rn(src[i]));
}

int check_volume(int64_t batch, int64_t depth, int64_t height, int64_t width, const char* name) {
  CITRUS_REQUIRE(batch >= 1 && batch <= 65535 && depth >= 1 && height >= 1 && width >= 1 &&
                     depth * height * width < (1ll << 31),
                 "%s: bad volume sizes", name);
  return CITRUS_OK;
}

template <int kK>
int launch_conv_tc_k(const ConvArgs& a, uint32_t* error_word, cudaStream_t s) {
  const int O = a.oa + a.ob;
  const int co_tiles = (int)cdiv(O, 256);
  const int n_tile = (int)(cdiv(cdiv(O, co_tiles), 16) * 16);
  const int64_t V = (int64_t)a.D * a.H * a.W;
  const int64_t vox_tiles = cdiv(V, kTcM);
  CITRUS_REQUIRE(vox_tiles < (1ll << 30), "conv3d: too many voxel tiles");
  const int64_t num_tiles = vox_tiles * co_tiles * a.B;
  const size_t smem = 2 * tc_stage_bytes(n_tile);
  cudaError_t e = cudaFuncSetAttribute(conv_tc_kernel<kK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "conv3d (tensor cores): %s", cudaGetErrorString(e));
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, conv_tc_kernel<kK>, kCvThreads, smem);
  if (e != cudaSuccess || per_sm < 1) return set_error(CITRUS_ECUDA, "conv3d (tensor cores): occupancy query failed");
  const int by_tmem = (int)(512 / tc_columns(n_tile));  // tensor-memory columns of the SM
  if (per_sm > by_tmem) per_sm = by_tmem;
  const int64_t grid = std::min<int64_t>(num_tiles, (int64_t)per_sm * num_sms());
  conv_tc_kernel<kK><<<(unsigned)grid, kCvThreads, smem, s>>>(a, n_tile, co_tiles, (int)vox_tiles, num_tiles,
                                                               error_word);
  note_launches();
  return CITRUS_OK;
}

// variant 1: the FP32 SIMT kernel; variant 2 (and 0): the tcgen05 implicit GEMM
int launch_conv(const ConvArgs& a, int kernel_size, int variant, uint32_t* error_word, cudaStream_t s) {
  if (variant != 1) {
    return kernel_size == 3 ? launch_conv_tc_k<3>(a, error_word, s) : launch_conv_tc_k<1>(a, error_word, s);
  }
  const int64_t tiles = cdiv(a.W, kTX) * cdiv(a.H, kTY) * cdiv(a.D, kTZ);
  CITRUS_REQUIRE(tiles < (1ll << 31), "conv3d: too many voxel bricks");
  dim3 grid((unsigned)tiles, (unsigned)cdiv(a.oa + a.ob, kCoT), (unsigned)a.B);
  if (kernel_size == 3) conv_kernel<3><<<grid, kConvThreads, 0, s>>>(a);
  else conv_kernel<1><<<grid, kConvThreads, 0, s>>>(a);
  note_launches();
  return CITRUS_OK;
}

}  // namespace
}  // namespace citrus

using namespace citrus;

extern "C" int citrus_conv3d_forward_config(const float* in_a, int64_t channels_a, const float* in_b,
                                            int64_t channels_b, int32_t b_upsampled, const uint16_t* weight,
                                            const float* bias, float* out, int64_t channels_out, int64_t batch,
                                            int64_t depth, int64_t height, int64_t width, int32_t kernel_size,
                                            int32_t relu, int32_t variant, uint32_t* error_word, void* stream) {
  int st = check_volume(batch, depth, height, width, "citrus_conv3d_forward");
  if (st) return st;
  CITRUS_REQUIRE(in_a && weight && out, "citrus_conv3d_forward: null pointer argument");
  CITRUS_REQUIRE(kernel_size == 1 || kernel_size == 3, "citrus_conv3d_forward: kernel size %d (1 or 3)", kernel_size);
  CITRUS_REQUIRE(channels_a >= 1 && channels_b >= 0 && channels_a + channels_b <= 4096 && channels_out >= 1 &&
                     channels_out <= 65535 * kCoT,
                 "citrus_conv3d_forward: bad channel counts");
  CITRUS_REQUIRE(channels_b == 0 || in_b != nullptr, "citrus_conv3d_forward: null second input");
  CITRUS_REQUIRE(!b_upsampled || (depth % 2 == 0 && height % 2 == 0 && width % 2 == 0),
                 "citrus_conv3d_forward: an upsampled input needs even sizes");
  const int64_t k3 = (int64_t)kernel_size * kernel_size * kernel_size;
  ConvArgs a{in_a, in_b, (int)channels_a, (int)channels_b, b_upsampled ? 1 : 0,
             weight, (channels_a + channels_b) * k3, k3, 1, 0,
             bias, out, nullptr, (int)channels_out, 0, nullptr, relu ? 1 : 0,
             (int)batch, (int)depth, (int)height, (int)width};
  CITRUS_REQUIRE(variant >= 0 && variant <= 2, "citrus_conv3d_forward: variant %d (0 auto, 1 SIMT, 2 tensor cores)",
                 variant);
  st = launch_conv(a, kernel_size, variant, error_word, as_stream(stream));
  if (st) return st;
  return launch_status("citrus_conv3d_forward");
}

extern "C" int citrus_conv3d_forward(const float* in_a, int64_t channels_a, const float* in_b, int64_t channels_b,
                                     int32_t b_upsampled, const uint16_t* weight, const float* bias, float* out,
                                     int64_t channels_out, int64_t batch, int64_t depth, int64_t height,
                                     int64_t width, int32_t kernel_size, int32_t relu, void* stream) {
  return citrus_conv3d_forward_config(in_a, channels_a, in_b, channels_b, b_upsampled, weight, bias, out,
                                      channels_out, batch, depth, height, width, kernel_size, relu, 0, nullptr,
                                      stream);
}

extern "C" int citrus_conv3d_backward_input_config(const float* grad_out, int64_t channels_out,
                                                   const uint16_t* weight, float* grad_a, int64_t channels_a,
                                                   const float* mask_a, float* grad_b, int64_t channels_b,
                                                   int64_t batch, int64_t depth, int64_t height, int64_t width,
                                                   int32_t kernel_size, int32_t variant, uint32_t* error_word,
                                                   void* stream) {
  int st = check_volume(batch, depth, height, width, "citrus_conv3d_backward_input");
  if (st) return st;
  CITRUS_REQUIRE(grad_out && weight && grad_a, "citrus_conv3d_backward_input: null pointer argument");
  CITRUS_REQUIRE(kernel_size == 1 || kernel_size == 3, "citrus_conv3d_backward_input: kernel size %d (1 or 3)",
                 kernel_size);
  CITRUS_REQUIRE(channels_out >= 1 && channels_out <= 4096 && channels_a >= 1 && channels_b >= 0 &&
                     channels_a + channels_b <= 65535 * kCoT,
                 "citrus_conv3d_backward_input: bad channel counts");
  CITRUS_REQUIRE(channels_b == 0 || grad_b != nullptr, "citrus_conv3d_backward_input: null second gradient");
  const int64_t k3 = (int64_t)kernel_size * kernel_size * kernel_size;
  const int64_t ci = channels_a + channels_b;
  // transposed convolution: output channel = forward input channel, input channel = forward output channel,
  // taps flipped
  ConvArgs a{grad_out, nullptr, (int)channels_out, 0, 0,
             weight, k3, ci * k3, -1, k3 - 1,
             nullptr, grad_a, grad_b, (int)channels_a, (int)channels_b, mask_a, 0,
             (int)batch, (int)depth, (int)height, (int)width};
  CITRUS_REQUIRE(variant >= 0 && variant <= 2,
                 "citrus_conv3d_backward_input: variant %d (0 auto, 1 SIMT, 2 tensor cores)", variant);
  st = launch_conv(a, kernel_size, variant, error_word, as_stream(stream));
  if (st) return st;
  return launch_status("citrus_conv3d_backward_input");
}

extern "C" int citrus_conv3d_backward_input(const float* grad_out, int64_t channels_out, const uint16_t* weight,
                                            float* grad_a, int64_t channels_a, const float* mask_a, float* grad_b,
                                            int64_t channels_b, int64_t batch, int64_t depth, int64_t height,
                                            int64_t width, int32_t kernel_size, void* stream) {
  return citrus_conv3d_backward_input_config(grad_out, channels_out, weight, grad_a, channels_a, mask_a, grad_b,
                                             channels_b, batch, depth, height, width, kernel_size, 0, nullptr,
                                             stream);
}

extern "C" int64_t citrus_conv3d_weight_grad_splits(int64_t channels_out, int64_t channels_a, int64_t channels_b,
                                                    int64_t batch, int64_t depth, int64_t height, int64_t width,
                                                    int32_t kernel_size) {
  if (kernel_size != 1 && kernel_size != 3) return 1;
  const int64_t ciw = kernel_size == 3 ? 8 : 16;
  const int64_t blocks = cdiv(channels_out, kCoT) * cdiv(channels_a + channels_b, ciw);
  const int64_t bricks = batch * cdiv(width, kTX) * cdiv(height, kTY) * cdiv(depth, kTZ);
  int64_t splits = cdiv(4 * (int64_t)num_sms(), blocks);
  if (splits > bricks) splits = bricks;
  if (splits > 65535) splits = 65535;
  return splits < 1 ? 1 : splits;
}

extern "C" int citrus_conv3d_backward_weight(const float* grad_out, int64_t channels_out, const float* in_a,
                                             int64_t channels_a, const float* in_b, int64_t channels_b,
                                             int32_t b_upsampled, float* grad_weight, float* grad_bias, int64_t batch,
                                             int64_t depth, int64_t height, int64_t width, int32_t kernel_size,
                                             float* partial, int64_t partial_capacity, void* stream) {
  int st = check_volume(batch, depth, height, width, "citrus_conv3d_backward_weight");
  if (st) return st;
  CITRUS_REQUIRE(grad_out && in_a && grad_weight, "citrus_conv3d_backward_weight: null pointer argument");
  CITRUS_REQUIRE(kernel_size == 1 || kernel_size == 3, "citrus_conv3d_backward_weight: kernel size %d (1 or 3)",
                 kernel_size);
  CITRUS_REQUIRE(channels_out >= 1 && channels_out <= 65535 * kCoT && channels_a >= 1 && channels_b >= 0 &&
                     channels_a + channels_b <= 4096,
                 "citrus_conv3d_backward_weight: bad channel counts");
  CITRUS_REQUIRE(channels_b == 0 || in_b != nullptr, "citrus_conv3d_backward_weight: null second input");
  CITRUS_REQUIRE(!b_upsampled || (depth % 2 == 0 && height % 2 == 0 && width % 2 == 0),
                 "citrus_conv3d_backward_weight: an upsampled input needs even sizes");
  cudaStream_t s = as_stream(stream);
  const int64_t k3 = (int64_t)kernel_size * kernel_size * kernel_size;
  const int64_t nW = channels_out * (channels_a + channels_b) * k3;
  int64_t splits = citrus_conv3d_weight_grad_splits(channels_out, channels_a, channels_b, batch, depth, height, width,
                                                    kernel_size);
  if (partial == nullptr || partial_capacity < 2 * nW) splits = 1;
  else if (splits * nW > partial_capacity) splits = partial_capacity / nW;
  float* dst = splits == 1 ? grad_weight : partial;
  const int ciw = kernel_size == 3 ? 8 : 16;
  dim3 grid((unsigned)cdiv(channels_out, kCoT), (unsigned)cdiv(channels_a + channels_b, ciw), (unsigned)splits);
  if (kernel_size == 3)
    wgrad_kernel<3, 8><<<grid, kConvThreads, 0, s>>>(grad_out, (int)channels_out, in_a, (int)channels_a, in_b,
                                                     (int)channels_b, b_upsampled ? 1 : 0, dst, (int)splits,
                                                     (int)batch, (int)depth, (int)height, (int)width);
  else
    wgrad_kernel<1, 16><<<grid, kConvThreads, 0, s>>>(grad_out, (int)channels_out, in_a, (int)channels_a, in_b,
                                                      (int)channels_b, b_upsampled ? 1 : 0, dst, (int)splits,
                                                      (int)batch, (int)depth, (int)height, (int)width);
  note_launches();
  if (splits > 1) {
    wgrad_reduce_kernel<<<(unsigned)cdiv(nW, kLearnThreads), kLearnThreads, 0, s>>>(partial, (int)splits, nW,
                                                                                   grad_weight);
    note_launches();
  }
  if (grad_bias != nullptr) {
    bias_grad_kernel<<<(unsigned)channels_out, kLearnThreads, 0, s>>>(grad_out, (int)channels_out, (int)batch,
                                                                     depth * height * width, grad_bias);
    note_launches();
  }
  return launch_status("citrus_conv3d_backward_weight");
}

extern "C" int citrus_avg_pool2(const float* in, float* out, int64_t batch_channels, int64_t depth, int64_t height,
                                int64_t width, void* stream) {
  CITRUS_REQUIRE(in && out, "citrus_avg_pool2: null pointer argument");
  CITRUS_REQUIRE(batch_channels >= 1 && depth >= 2 && height >= 2 && width >= 2 && depth % 2 == 0 &&
                     height % 2 == 0 && width % 2 == 0 && depth * height * width < (1ll << 31),
                 "citrus_avg_pool2: sizes must be even");
  const int64_t n = batch_channels * (depth / 2) * (height / 2) * (width / 2);
  pool_kernel<<<(unsigned)cdiv(n, kLearnThreads), kLearnThreads, 0, as_stream(stream)>>>(
      in, out, batch_channels, (int)depth, (int)height, (int)width);
  note_launches();
  return launch_status("citrus_avg_pool2");
}

extern "C" int citrus_avg_pool2_backward(const float* grad_out, float* grad_in, const float* mask, int32_t accumulate,
                                         int64_t batch_channels, int64_t depth, int64_t height, int64_t width,
                                         void* stream) {
  CITRUS_REQUIRE(grad_out && grad_in, "citrus_avg_pool2_backward: null pointer argument");
  CITRUS_REQUIRE(batch_channels >= 1 && depth >= 2 && height >= 2 && width >= 2 && depth % 2 == 0 &&
                     height % 2 == 0 && width % 2 == 0 && depth * height * width < (1ll << 31),
                 "citrus_avg_pool2_backward: sizes must be even");
  const int64_t n = batch_channels * depth * height * width;
  pool_backward_kernel<<<(unsigned)cdiv(n, kLearnThreads), kLearnThreads, 0, as_stream(stream)>>>(
      grad_out, grad_in, mask, accumulate ? 1 : 0, batch_channels, (int)depth, (int)height, (int)width);
  note_launches();
  return launch_status("citrus_avg_pool2_backward");
}

extern "C" int citrus_upsample2_backward(const float* grad_fine, const float* mask_coarse, float* grad_coarse,
                                         int64_t batch_channels, int64_t depth, int64_t height, int64_t width,
                                         void* stream) {
  CITRUS_REQUIRE(grad_fine && grad_coarse, "citrus_upsample2_backward: null pointer argument");
  CITRUS_REQUIRE(batch_channels >= 1 && depth >= 1 && height >= 1 && width >= 1 &&
                     8 * depth * height * width < (1ll << 31),
                 "citrus_upsample2_backward: bad sizes");
  const int64_t n = batch_channels * depth * height * width;
  upsample_backward_kernel<<<(unsigned)cdiv(n, kLearnThreads), kLearnThreads, 0, as_stream(stream)>>>(
      grad_fine, mask_coarse, grad_coarse, batch_channels, (int)depth, (int)height, (int)width);
  note_launches();
  return launch_status("citrus_upsample2_backward");
}

extern "C" int citrus_mse(const float* pred, const float* target, int64_t n, float* grad, float* partial,
                          int64_t partial_capacity, void* stream) {
  CITRUS_REQUIRE(pred && target && grad && partial && n >= 1, "citrus_mse: bad arguments");
  CITRUS_REQUIRE(partial_capacity >= cdiv(n, kLearnThreads), "citrus_mse: partial buffer holds %lld floats, needs %lld",
                 (long long)partial_capacity, (long long)cdiv(n, kLearnThreads));
  mse_kernel<<<(unsigned)cdiv(n, kLearnThreads), kLearnThreads, 0, as_stream(stream)>>>(pred, target, n, grad,
                                                                                        partial);
  note_launches();
  return launch_status("citrus_mse");
}

extern "C" int citrus_adam(float* param, const float* grad, float* m, float* v, uint16_t* param_bf16, int64_t n,
                           double lr, double beta1, double beta2, double eps, int64_t step, void* stream) {
  CITRUS_REQUIRE(param && grad && m && v && n >= 0 && step >= 1, "citrus_adam: bad arguments");
  if (n == 0) return CITRUS_OK;
  const float c1 = (float)(1.0 - pow(beta1, (double)step)), c2 = (float)(1.0 - pow(beta2, (double)step));
  adam_kernel<<<(unsigned)cdiv(n, kLearnThreads), kLearnThreads, 0, as_stream(stream)>>>(
      param, grad, m, v, param_bf16, n, (float)lr, (float)beta1, (float)beta2, (float)eps, c1, c2);
  note_launches();
  return launch_status("citrus_adam");
}

extern "C" int citrus_to_bf16(const float* src, uint16_t* dst, int64_t n, void* stream) {
  CITRUS_REQUIRE(src && dst && n >= 0, "citrus_to_bf16: bad arguments");
  if (n == 0) return CITRUS_OK;
  to_bf16_kernel<<<(unsigned)cdiv(n, kLearnThreads), kLearnThreads, 0, as_stream(stream)>>>(src, dst, n);
  note_launches();
  return launch_status("citrus_to_bf16");
}
