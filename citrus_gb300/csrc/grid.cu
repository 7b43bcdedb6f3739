// Signal accumulation behind an anti-scatter grid whose transmission varies over the panel
// (citrus/scatter_solver/scatter_image.py:340-389, 437-486 with detector.py:704-756).
//
// The signal of a direction chunk is sum_k W[k, g, r, c] image[k, g, r, c], where the weight is the product of the
// factors the direction set keeps: one per direction and group (quadrature weight, incidence and detector response on
// a flat panel; septa that vary only with the direction), one per direction, group and channel (a curved panel's
// incidence; septa along the rows), one per direction, group and row (septa along the channels on a flat panel), and
// the septa whose grid angles vary along the rows and the channels together. Those angles are a part per direction
// and channel plus a part per pixel, theta(k, r, c) = theta(k, 0, c) + (theta(0, r, c) - theta(0, 0, c)), so one thread
// per pixel adds the two float32 parts, brackets |theta1| and |theta2| in the table's nodes once per (direction,
// pixel), and interpolates the table (at the group energies) bilinearly for every group. The weights never touch
// memory: a [K, G, Rd, Cd] weight tensor of a 512 x 384 panel with 16 groups and 32 directions would be 400 MB per
// chunk. The reference multiplies the same factors into per-pixel weights and reduces over the directions.
#include <math.h>

#include "common.cuh"

namespace citrus {
namespace {

constexpr int kGridMaxG = 32;
constexpr int kGridMaxSepta = 2;

struct PixelSepta {
  const float* theta_channels;  // [2, K, Cd] theta1 and theta2 along the first row (chunk directions from 0)
  const float* theta_pixels;    // [2, Rd, Cd] their change from the first row, the same for every direction
  const float* table;           // [G, T1, T2] transmission at the group energies
  const float* nodes1;          // [T1] ascending theta1 nodes
  const float* nodes2;          // [T2] ascending theta2 nodes
  int T1, T2;
};

struct GridSignalArgs {
  PixelSepta septa[kGridMaxSepta];
  int num_septa;
};

// i0, i1 and the weight of i1 of x in ascending nodes, clamped to the end nodes (detector.py:147-170)
__device__ __forceinline__ void bracket(const float* __restrict__ nodes, int n, float x, int& i0, int& i1, float& w) {
  if (n == 1) {
    i0 = i1 = 0;
    w = 0.f;
    return;
  }
  const float lo = __ldg(nodes), hi = __ldg(nodes + n - 1);
  const float xc = fminf(fmaxf(x, lo), hi);
  int a = 0, b = n;  // first node > xc
  while (a < b) {
    const int m = (a + b) >> 1;
    if (__ldg(nodes + m) <= xc) a = m + 1;
    else b = m;
  }
  i1 = min(max(a, 1), n - 1);
  i0 = i1 - 1;
  const float n0 = __ldg(nodes + i0), n1 = __ldg(nodes + i1);
  w = fminf(fmaxf((xc - n0) / (n1 - n0), 0.f), 1.f);
}

// acc[g, r, c] (or acc[r, c], the groups summed) (+)= sum_k W[k, g, r, c] img[k, g, r, c]; one thread per pixel.
__global__ void grid_signal_sum_kernel(const float* __restrict__ img, int K, int G, int R, int C, int64_t is_k,
                                       int64_t is_g, int64_t is_r, int64_t is_c, const float* __restrict__ W,
                                       int w_cols, const float* __restrict__ row_w, GridSignalArgs ga,
                                       float* __restrict__ acc, int per_group, int accumulate) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)R * C) return;
  const int r = (int)(t / C), c = (int)(t - (int64_t)r * C);
  float sum[kGridMaxG];
#pragma unroll
  for (int g = 0; g < kGridMaxG; ++g) sum[g] = 0.f;
  float th1[kGridMaxSepta], th2[kGridMaxSepta];
  for (int s = 0; s < ga.num_septa; ++s) {
    th1[s] = __ldg(ga.septa[s].theta_pixels + t);
    th2[s] = __ldg(ga.septa[s].theta_pixels + (int64_t)R * C + t);
  }
  for (int k = 0; k < K; ++k) {
    int i10[kGridMaxSepta], i11[kGridMaxSepta], i20[kGridMaxSepta], i21[kGridMaxSepta];
    float w1[kGridMaxSepta], w2[kGridMaxSepta];
    for (int s = 0; s < ga.num_septa; ++s) {
      const PixelSepta& ps = ga.septa[s];
      const float a1 = __ldg(ps.theta_channels + (int64_t)k * C + c) + th1[s];
      const float a2 = __ldg(ps.theta_channels + ((int64_t)K + k) * C + c) + th2[s];
      bracket(ps.nodes1, ps.T1, fabsf(a1), i10[s], i11[s], w1[s]);
      bracket(ps.nodes2, ps.T2, fabsf(a2), i20[s], i21[s], w2[s]);
    }
    const float* src = img + k * is_k + r * is_r + c * is_c;
#pragma unroll
    for (int g = 0; g < kGridMaxG; ++g) {
      if (g >= G) break;
      float w = __ldg(W + ((int64_t)k * G + g) * w_cols + (w_cols > 1 ? c : 0));
      if (row_w) w *= __ldg(row_w + ((int64_t)k * G + g) * R + r);
      for (int s = 0; s < ga.num_septa; ++s) {
        const PixelSepta& ps = ga.septa[s];
        const float* tg = ps.table + (int64_t)g * ps.T1 * ps.T2;
        const float a00 = __ldg(tg + i10[s] * ps.T2 + i20[s]), a01 = __ldg(tg + i10[s] * ps.T2 + i21[s]);
        const float a10 = __ldg(tg + i11[s] * ps.T2 + i20[s]), a11 = __ldg(tg + i11[s] * ps.T2 + i21[s]);
        const float a0 = a00 + (a01 - a00) * w2[s];
        const float a1 = a10 + (a11 - a10) * w2[s];
        w *= a0 + (a1 - a0) * w1[s];
      }
      sum[g] = fmaf(w, __ldg(src + g * is_g), sum[g]);
    }
  }
  if (per_group) {
#pragma unroll
    for (int g = 0; g < kGridMaxG; ++g) {
      if (g >= G) break;
      float* o = acc + (int64_t)g * R * C + t;
      *o = accumulate ? *o + sum[g] : sum[g];
    }
  } else {
    float total = 0.f;
#pragma unroll
    for (int g = 0; g < kGridMaxG; ++g)
      if (g < G) total += sum[g];
    acc[t] = accumulate ? acc[t] + total : total;
  }
}

}  // namespace
}  // namespace citrus

using namespace citrus;

extern "C" int citrus_grid_signal_sum(const float* image, int64_t num_directions, int64_t groups, int64_t rows,
                                      int64_t cols, int64_t is_k, int64_t is_g, int64_t is_r, int64_t is_c,
                                      const float* weights, int64_t weight_cols, const float* row_weights,
                                      int64_t num_septa, const float* const* theta_channels,
                                      const float* const* theta_pixels, const float* const* tables,
                                      const float* const* theta1_nodes, const int64_t* num_theta1,
                                      const float* const* theta2_nodes, const int64_t* num_theta2,
                                      float* accumulator, int32_t per_group, int32_t accumulate, void* stream) {
  CITRUS_REQUIRE(image && weights && accumulator, "citrus_grid_signal_sum: null pointer");
  CITRUS_REQUIRE(num_directions >= 0 && groups >= 1 && groups <= kGridMaxG && rows >= 0 && cols >= 0,
                 "citrus_grid_signal_sum: need 1 <= groups <= 32 and non-negative sizes");
  CITRUS_REQUIRE(weight_cols == 1 || weight_cols == cols, "citrus_grid_signal_sum: weights must be [K, G, cols | 1]");
  CITRUS_REQUIRE(num_septa >= 0 && num_septa <= kGridMaxSepta, "citrus_grid_signal_sum: at most two sets of septa");
  GridSignalArgs ga{};
  ga.num_septa = (int)num_septa;
  for (int s = 0; s < ga.num_septa; ++s) {
    CITRUS_REQUIRE(theta_channels && theta_pixels && tables && theta1_nodes && num_theta1 && theta2_nodes &&
                       num_theta2,
                   "citrus_grid_signal_sum: septa arrays missing");
    CITRUS_REQUIRE(theta_channels[s] && theta_pixels[s] && tables[s] && theta1_nodes[s] && theta2_nodes[s] &&
                       num_theta1[s] >= 1 && num_theta2[s] >= 1,
                   "citrus_grid_signal_sum: septa set %d incomplete", s);
    ga.septa[s] = PixelSepta{theta_channels[s], theta_pixels[s], tables[s], theta1_nodes[s], theta2_nodes[s],
                             (int)num_theta1[s], (int)num_theta2[s]};
  }
  const int64_t P = rows * cols;
  if (P == 0) return CITRUS_OK;
  grid_signal_sum_kernel<<<(unsigned)cdiv(P, 128), 128, 0, as_stream(stream)>>>(
      image, (int)num_directions, (int)groups, (int)rows, (int)cols, is_k, is_g, is_r, is_c, weights,
      (int)weight_cols, row_weights, ga, accumulator, per_group, accumulate);
  note_launches();
  return launch_status("citrus_grid_signal_sum");
}
