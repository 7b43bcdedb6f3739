// Finite-cone footprint and accumulation of the collapsed-cone scatter image
// (citrus/scatter_solver/scatter_image.py:897-1135, 1234-1323).
//
// The footprint of direction k is a box blur of its single-ray image with a width of hbar_k W_k / pitch pixels along
// the channels and the rows, hbar_k the emission-weighted mean panel height (from the emission kernel's sums). The
// reference applies it as dense [N, N] overlap matrices in batched products (box_matrix, :952-1007); here each output
// pixel sums only the input pixels its window overlaps, with the same overlap weights
// B[c, j] = |[j, j + 1] n W_c| / |W_c|, W_c = [c + 1/2 - w/2, c + 1/2 + w/2] n [0, N], so the cost is O(N w) instead of
// O(N^2). The width is computed in the kernel from the height sums, so no host round trip sits between the emission
// and the blur.
#include <math.h>

#include "common.cuh"

namespace citrus {
namespace {

struct WidthArgs {
  const float* fixed;        // [K] widths in pixels, or null
  const float* height_sums;  // [K, 2] (sum e, sum e h), with cell widths
  const float* cell_width;   // [K, 2] gnomonic widths (channels, rows)
  int axis;                  // 0: channels, 1: rows
  float inv_pitch;           // 1 / pixel pitch along the axis
  float center_height;       // mean height where the emission vanishes
};

__device__ __forceinline__ float blur_width(const WidthArgs& w, int k) {
  if (w.fixed) return w.fixed[k];
  const float den = w.height_sums[2 * k], num = w.height_sums[2 * k + 1];
  const float hbar = den > 0.f ? num / fmaxf(den, 1.17549435e-38f) : w.center_height;
  return hbar * w.cell_width[2 * k + w.axis] * w.inv_pitch;
}

// out[k, line, c] = sum_j B_k[c, j] in[k, line, j] along an axis of N pixels; lines and pixels through strides.
__global__ void box_blur_kernel(const float* __restrict__ in, float* __restrict__ out, int K, int64_t lines, int N,
                                int64_t is_k, int64_t is_l, int64_t is_p, int64_t os_k, int64_t os_l, int64_t os_p,
                                WidthArgs wa) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (t >= lines * N || k >= K) return;
  const int64_t line = t / N;
  const int c = (int)(t - line * N);
  const float half = 0.5f * fmaxf(blur_width(wa, k), 1e-3f);
  const float nf = (float)N;
  const float center = (float)c + 0.5f;
  const float lo = fminf(fmaxf(center - half, 0.f), nf), hi = fminf(fmaxf(center + half, 0.f), nf);
  const float* src = in + k * is_k + line * is_l;
  const int j0 = max(0, (int)floorf(lo)), j1 = min(N - 1, (int)ceilf(hi) - 1);
  float acc = 0.f;
  for (int j = j0; j <= j1; ++j) {
    const float ov = fmaxf(fminf(hi, (float)j + 1.f) - fmaxf(lo, (float)j), 0.f);
    acc = fmaf(ov, src[j * is_p], acc);
  }
  out[k * os_k + line * os_l + (int64_t)c * os_p] = acc / (hi - lo);
}

// The same filter with O(1) work per output pixel (box_blur_warp_kernel below): a warp owns one line, stages its N
// pixels in shared memory with their prefix sums (a warp scan, float32 pairs), and each output pixel is its partial
// first pixel, the prefix-sum difference over the fully covered pixels and its partial last pixel, divided by the
// window length.
constexpr int kScanMaxN = 1024;

// A float32 pair (hi, lo) that carries a sum to about 2^-40 of its magnitude: the prefix sums of the scan below are
// kept this way instead of in float64, whose rate on this GPU is a small fraction of float32's.
struct F2 {
  float hi, lo;
};

// hi + lo of a + b exactly (Knuth's two-sum), then the pair renormalised
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bp = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(b.hi, bp));
  const float t = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  const float hi = __fadd_rn(s, t);
  return F2{hi, __fsub_rn(t, __fsub_rn(hi, s))};
}

__device__ __forceinline__ F2 f2_neg(F2 a) { return F2{-a.hi, -a.lo}; }

// One warp per line and kBlurLines lines per block: a lane sums a contiguous run of ceil(N / 32) pixels, a
// warp-level scan of the run sums gives the prefix sums, and no block barrier is needed, so a block's eight lines
// proceed independently (a block of 256 threads per line, as before, left most of its threads waiting at the
// scan's barriers). Lines of strided pixels (the row blur) are adjacent in memory across the block's warps, so
// the eight warps share the sectors of their loads and stores.
constexpr int kBlurLines = 8;

__global__ void __launch_bounds__(32 * kBlurLines) box_blur_warp_kernel(const float* __restrict__ in,
                                                                        float* __restrict__ out, int64_t lines, int N,
                                                                        int64_t is_k, int64_t is_l, int64_t is_p,
                                                                        int64_t os_k, int64_t os_l, int64_t os_p,
                                                                        WidthArgs wa) {
  extern __shared__ float s_blur[];  // per warp: x [N], P_hi [N + 1], P_lo [N + 1]
  const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
  const int k = blockIdx.y;
  const int64_t line = (int64_t)blockIdx.x * kBlurLines + warp;
  if (line >= lines) return;  // the whole warp: no block barrier follows
  float* x = s_blur + (int64_t)warp * (3 * N + 2);
  float* P_hi = x + N;
  float* P_lo = P_hi + N + 1;
  const float* src = in + k * is_k + line * is_l;
  for (int j = lane; j < N; j += 32) x[j] = src[j * is_p];
  __syncwarp();
  const int per = (N + 31) / 32;
  const int j0 = min(N, lane * per), j1 = min(N, j0 + per);
  F2 run{0.f, 0.f};
  for (int j = j0; j < j1; ++j) run = f2_add(run, F2{x[j], 0.f});
  F2 incl = run;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const F2 y{__shfl_up_sync(0xffffffffu, incl.hi, off), __shfl_up_sync(0xffffffffu, incl.lo, off)};
    if (lane >= off) incl = f2_add(incl, y);
  }
  F2 acc = f2_add(incl, f2_neg(run));  // exclusive prefix of this lane's run
  if (lane == 0) {
    P_hi[0] = 0.f;
    P_lo[0] = 0.f;
  }
  for (int j = j0; j < j1; ++j) {
    acc = f2_add(acc, F2{x[j], 0.f});
    P_hi[j + 1] = acc.hi;
    P_lo[j + 1] = acc.lo;
  }
  __syncwarp();
  const float half = 0.5f * fmaxf(blur_width(wa, k), 1e-3f);
  const float nf = (float)N;
  float* dst = out + k * os_k + line * os_l;
  for (int c = lane; c < N; c += 32) {
    const float center = (float)c + 0.5f;
    const float lo = fminf(fmaxf(center - half, 0.f), nf), hi = fminf(fmaxf(center + half, 0.f), nf);
    const int a = max(0, (int)floorf(lo)), b = min(N - 1, (int)ceilf(hi) - 1);
    float sum;
    if (a >= b) {
      sum = fmaxf(hi - lo, 0.f) * x[a];
    } else {
      const float first = ((float)a + 1.f - lo) * x[a], last = (hi - (float)b) * x[b];
      const F2 interior = f2_add(F2{P_hi[b], P_lo[b]}, F2{-P_hi[a + 1], -P_lo[a + 1]});
      const F2 total = f2_add(f2_add(interior, F2{first, 0.f}), F2{last, 0.f});
      sum = total.hi + total.lo;
    }
    dst[(int64_t)c * os_p] = sum / (hi - lo);
  }
}

// the dense overlap matrices of the same filter, [K, N, N] (scatter_image.py:952-981)
__global__ void box_matrix_kernel(const float* __restrict__ widths, int N, float* __restrict__ out) {
  const int k = blockIdx.y;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)N * N) return;
  const int c = (int)(t / N), j = (int)(t - (int64_t)c * N);
  const float half = 0.5f * fmaxf(widths[k], 1e-3f);
  const float nf = (float)N, center = (float)c + 0.5f;
  const float lo = fminf(fmaxf(center - half, 0.f), nf), hi = fminf(fmaxf(center + half, 0.f), nf);
  out[(int64_t)k * N * N + t] = fmaxf(fminf(hi, (float)j + 1.f) - fmaxf(lo, (float)j), 0.f) / (hi - lo);
}

// out[k, r, c] = sum_g img[k, r, g, c] W[k, g, c or 0] for rows-outer images [K, R, G, C]
__global__ void weighted_group_sum_kernel(const float* __restrict__ img, const float* __restrict__ W, int K, int R,
                                          int G, int C, int w_channels, float* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (t >= (int64_t)R * C) return;
  const int r = (int)(t / C), c = (int)(t - (int64_t)r * C);
  const float* src = img + (((int64_t)k * R + r) * G) * C + c;
  const float* w = W + (int64_t)k * G * w_channels + (w_channels > 1 ? c : 0);
  float acc = 0.f;
  for (int g = 0; g < G; ++g) acc = fmaf(src[(int64_t)g * C], w[(int64_t)g * w_channels], acc);
  out[((int64_t)k * R + r) * C + c] = acc;
}

// acc[p] (+)= sum_k img[k, p], directions summed in order
__global__ void sum_directions_kernel(const float* __restrict__ img, int K, int64_t P, int64_t stride_k,
                                      float* __restrict__ acc, int accumulate) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  float s = 0.f;
  for (int k = 0; k < K; ++k) s += img[k * stride_k + p];
  acc[p] = accumulate ? acc[p] + s : s;
}

// acc[g, r, c] (+)= sum_k W[k, g, r | 0, c | 0] img[k, g, r, c], images through strides (the accumulation of the full
// images, DirectionSetContext.accumulate, scatter_image.py:340-371)
__global__ void weighted_direction_sum_kernel(const float* __restrict__ img, int K, int G, int R, int C, int64_t is_k,
                                              int64_t is_g, int64_t is_r, int64_t is_c, const float* __restrict__ W,
                                              int w_rows, int w_cols, float* __restrict__ acc, int accumulate) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)G * R * C) return;
  const int g = (int)(t / ((int64_t)R * C));
  const int64_t rc = t - (int64_t)g * R * C;
  const int r = (int)(rc / C), c = (int)(rc - (int64_t)r * C);
  const int64_t w_k = (int64_t)G * w_rows * w_cols;
  const float* w = W + ((int64_t)g * w_rows + (w_rows > 1 ? r : 0)) * w_cols + (w_cols > 1 ? c : 0);
  const float* src = img + g * is_g + r * is_r + c * is_c;
  float s = 0.f;
  for (int k = 0; k < K; ++k) s = fmaf(w[k * w_k], src[k * is_k], s);
  acc[t] = accumulate ? acc[t] + s : s;
}

}  // namespace
}  // namespace citrus

using namespace citrus;

extern "C" int citrus_weighted_direction_sum(const float* image, int64_t num_directions, int64_t groups,
                                             int64_t rows, int64_t cols, int64_t is_k, int64_t is_g, int64_t is_r,
                                             int64_t is_c, const float* weights, int64_t weight_rows,
                                             int64_t weight_cols, float* accumulator, int32_t accumulate,
                                             void* stream) {
  CITRUS_REQUIRE(image && weights && accumulator, "citrus_weighted_direction_sum: null pointer");
  CITRUS_REQUIRE((weight_rows == 1 || weight_rows == rows) && (weight_cols == 1 || weight_cols == cols),
                 "citrus_weighted_direction_sum: weights must be [K, G, rows | 1, cols | 1]");
  const int64_t total = groups * rows * cols;
  if (total == 0) return CITRUS_OK;
  weighted_direction_sum_kernel<<<(unsigned)cdiv(total, 256), 256, 0, as_stream(stream)>>>(
      image, (int)num_directions, (int)groups, (int)rows, (int)cols, is_k, is_g, is_r, is_c, weights,
      (int)weight_rows, (int)weight_cols, accumulator, accumulate);
  note_launches();
  return launch_status("citrus_weighted_direction_sum");
}

extern "C" int citrus_box_blur(const float* in, float* out, int64_t num_directions, int64_t lines, int64_t length,
                               int64_t is_k, int64_t is_l, int64_t is_p, int64_t os_k, int64_t os_l, int64_t os_p,
                               const float* widths, const float* height_sums, const float* cell_width, int32_t axis,
                               double pitch, double center_height, void* stream) {
  CITRUS_REQUIRE(in && out, "citrus_box_blur: null pointer");
  CITRUS_REQUIRE(widths || (height_sums && cell_width && pitch > 0), "citrus_box_blur: give widths or height sums");
  CITRUS_REQUIRE(num_directions >= 0 && num_directions <= 65535 && lines >= 0 && length >= 1 && (axis == 0 || axis == 1),
                 "citrus_box_blur: bad sizes");
  CITRUS_REQUIRE(in != out, "citrus_box_blur: in and out must not alias");
  if (num_directions == 0 || lines == 0) return CITRUS_OK;
  WidthArgs wa{widths, height_sums, cell_width, axis, (float)(pitch > 0 ? 1.0 / pitch : 0.0), (float)center_height};
  if (length <= kScanMaxN && cdiv(lines, kBlurLines) <= 0x7fffffff) {
    const size_t smem = (size_t)kBlurLines * (3 * length + 2) * sizeof(float);  // 96 KB at the longest lines
    cudaError_t e = cudaFuncSetAttribute(box_blur_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)((size_t)kBlurLines * (3 * kScanMaxN + 2) * sizeof(float)));
    if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "citrus_box_blur: %s", cudaGetErrorString(e));
    dim3 grid((unsigned)cdiv(lines, kBlurLines), (unsigned)num_directions);
    box_blur_warp_kernel<<<grid, 32 * kBlurLines, smem, as_stream(stream)>>>(in, out, lines, (int)length, is_k, is_l,
                                                                             is_p, os_k, os_l, os_p, wa);
  } else {
    dim3 grid((unsigned)cdiv(lines * length, 256), (unsigned)num_directions);
    box_blur_kernel<<<grid, 256, 0, as_stream(stream)>>>(in, out, (int)num_directions, lines, (int)length, is_k,
                                                         is_l, is_p, os_k, os_l, os_p, wa);
  }
  note_launches();
  return launch_status("citrus_box_blur");
}

extern "C" int citrus_box_matrix(const float* widths, int64_t num_directions, int64_t length, float* out,
                                 void* stream) {
  CITRUS_REQUIRE(widths && out && num_directions >= 0 && num_directions <= 65535 && length >= 1,
                 "citrus_box_matrix: bad arguments");
  if (num_directions == 0) return CITRUS_OK;
  dim3 grid((unsigned)cdiv(length * length, 256), (unsigned)num_directions);
  box_matrix_kernel<<<grid, 256, 0, as_stream(stream)>>>(widths, (int)length, out);
  note_launches();
  return launch_status("citrus_box_matrix");
}

extern "C" int citrus_weighted_group_sum(const float* image, const float* weights, int64_t num_directions,
                                         int64_t rows, int64_t groups, int64_t cols, int64_t weight_cols, float* out,
                                         void* stream) {
  CITRUS_REQUIRE(image && weights && out, "citrus_weighted_group_sum: null pointer");
  CITRUS_REQUIRE(num_directions >= 0 && num_directions <= 65535 && (weight_cols == 1 || weight_cols == cols),
                 "citrus_weighted_group_sum: bad sizes");
  if (num_directions == 0) return CITRUS_OK;
  dim3 grid((unsigned)cdiv(rows * cols, 256), (unsigned)num_directions);
  weighted_group_sum_kernel<<<grid, 256, 0, as_stream(stream)>>>(image, weights, (int)num_directions, (int)rows,
                                                                 (int)groups, (int)cols, (int)weight_cols, out);
  note_launches();
  return launch_status("citrus_weighted_group_sum");
}

extern "C" int citrus_sum_directions(const float* image, int64_t num_directions, int64_t pixels, int64_t stride_k,
                                     float* accumulator, int32_t accumulate, void* stream) {
  CITRUS_REQUIRE(image && accumulator && num_directions >= 0 && pixels >= 0, "citrus_sum_directions: bad arguments");
  if (pixels == 0) return CITRUS_OK;
  sum_directions_kernel<<<(unsigned)cdiv(pixels, 256), 256, 0, as_stream(stream)>>>(image, (int)num_directions, pixels,
                                                                                   stride_k, accumulator, accumulate);
  note_launches();
  return launch_status("citrus_sum_directions");
}
