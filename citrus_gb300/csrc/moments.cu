// Spherical-harmonic moments of the scattering source, T[g, n, k, x] = sum_g' transfer[g', g, l(n), x] phi[g', n, k, x]
// (citrus/scatter_solver/angular_quadrature.py:600-677 and kernels/scattering_kernels.py:159-252), summed over the
// incoming groups in ascending order. Two thread mappings over the same arithmetic:
//  * linear-discontinuous layouts with the 4 moments contiguous (the sweep's cell-major storage): one thread per
//    (moment n, point x) moves the 4 moments of every group as float4;
//  * any other strides (the image's cell means, moment-major): one thread per (n, k, x), points fastest.
#include "common.cuh"

namespace citrus {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxGroups = 32;

__device__ __forceinline__ int degree_of(int n) {
  int l = (int)sqrtf((float)n);
  while ((l + 1) * (l + 1) <= n) ++l;
  while (l * l > n) --l;
  return l;
}

template <int kMax>
__global__ void __launch_bounds__(kThreads) moments_vec4_kernel(const float* __restrict__ transfer,
                                                               const float* __restrict__ phi, float* __restrict__ out,
                                                               int GI, int GO, int num_legendre, int64_t X,
                                                               int64_t ps_g, int64_t ps_n, int64_t ps_x, int64_t os_g,
                                                               int64_t os_n, int64_t os_x) {
  // the moments are the fastest block index: the blocks of one range of points run back to back over all moments,
  // so the transfer rows of a degree, shared by its 2l + 1 moments, are read from DRAM once and then from L2
  const int64_t x = (int64_t)blockIdx.y * kThreads + threadIdx.x;
  const int n = blockIdx.x;
  if (x >= X) return;
  const int l = degree_of(n);
  float4 ph[kMax];
#pragma unroll
  for (int gi = 0; gi < kMax; ++gi)
    if (gi < GI) ph[gi] = *reinterpret_cast<const float4*>(phi + gi * ps_g + n * ps_n + x * ps_x);
  const float* tr = transfer + (int64_t)l * X + x;
  const int64_t pair = (int64_t)num_legendre * X;
  for (int go = 0; go < GO; ++go) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int gi = 0; gi < kMax; ++gi) {
      if (gi < GI) {
        const float m = __ldg(tr + (int64_t)(gi * GO + go) * pair);
        acc.x = fmaf(m, ph[gi].x, acc.x);
        acc.y = fmaf(m, ph[gi].y, acc.y);
        acc.z = fmaf(m, ph[gi].z, acc.z);
        acc.w = fmaf(m, ph[gi].w, acc.w);
      }
    }
    *reinterpret_cast<float4*>(out + go * os_g + n * os_n + x * os_x) = acc;
  }
}

template <int kMax>
__global__ void __launch_bounds__(kThreads) moments_scalar_kernel(const float* __restrict__ transfer,
                                                                 const float* __restrict__ phi,
                                                                 float* __restrict__ out, int GI, int GO,
                                                                 int num_legendre, int64_t X, int64_t ps_g,
                                                                 int64_t ps_n, int64_t ps_k, int64_t ps_x,
                                                                 int64_t os_g, int64_t os_n, int64_t os_k,
                                                                 int64_t os_x) {
  const int64_t x = (int64_t)blockIdx.y * kThreads + threadIdx.x;  // the moments fastest, as above
  const int n = blockIdx.x, k = blockIdx.z;
  if (x >= X) return;
  const int l = degree_of(n);
  float ph[kMax];
#pragma unroll
  for (int gi = 0; gi < kMax; ++gi)
    if (gi < GI) ph[gi] = phi[gi * ps_g + n * ps_n + k * ps_k + x * ps_x];
  const float* tr = transfer + (int64_t)l * X + x;
  const int64_t pair = (int64_t)num_legendre * X;
  for (int go = 0; go < GO; ++go) {
    float acc = 0.f;
#pragma unroll
    for (int gi = 0; gi < kMax; ++gi)
      if (gi < GI) acc = fmaf(__ldg(tr + (int64_t)(gi * GO + go) * pair), ph[gi], acc);
    out[go * os_g + n * os_n + k * os_k + x * os_x] = acc;
  }
}

}  // namespace
}  // namespace citrus

using namespace citrus;

extern "C" int citrus_scattering_moments(const float* transfer, const float* phi, float* out, int64_t g_in,
                                         int64_t g_out, int64_t num_legendre, int64_t num_moments, int64_t k_count,
                                         int64_t num_points, int64_t ps_g, int64_t ps_n, int64_t ps_k, int64_t ps_x,
                                         int64_t os_g, int64_t os_n, int64_t os_k, int64_t os_x, void* stream) {
  CITRUS_REQUIRE(transfer && phi && out, "citrus_scattering_moments: null pointer argument");
  CITRUS_REQUIRE(g_in >= 1 && g_in <= kMaxGroups && g_out >= 1 && g_out <= 4096,
                 "citrus_scattering_moments: groups in %lld / out %lld outside [1, %d]", (long long)g_in,
                 (long long)g_out, kMaxGroups);
  CITRUS_REQUIRE(num_moments >= 1 && num_moments <= 65535 && num_points >= 0 && (k_count == 1 || k_count == 4),
                 "citrus_scattering_moments: bad sizes");
  int L = 0;
  while ((L + 1) * (L + 1) < num_moments) ++L;
  CITRUS_REQUIRE((L + 1) * (L + 1) == num_moments && L + 1 <= num_legendre,
                 "citrus_scattering_moments: %lld moments is not (L+1)^2 with L < %lld Legendre orders",
                 (long long)num_moments, (long long)num_legendre);
  if (num_points == 0) return CITRUS_OK;
  cudaStream_t s = as_stream(stream);
  const bool vec = k_count == 4 && ps_k == 1 && os_k == 1 && ps_g % 4 == 0 && ps_n % 4 == 0 && ps_x % 4 == 0 &&
                   os_g % 4 == 0 && os_n % 4 == 0 && os_x % 4 == 0 && ((uintptr_t)phi % 16) == 0 &&
                   ((uintptr_t)out % 16) == 0;
  CITRUS_REQUIRE(cdiv(num_points, kThreads) <= 65535, "citrus_scattering_moments: %lld points exceed the grid",
                 (long long)num_points);
  const unsigned bx = (unsigned)cdiv(num_points, kThreads);
  const int GI = (int)g_in, GO = (int)g_out, NL = (int)num_legendre;
#define CITRUS_MOMENTS_LAUNCH(KMAX)                                                                                   \
  if (vec) {                                                                                                          \
    moments_vec4_kernel<KMAX><<<dim3((unsigned)num_moments, bx), kThreads, 0, s>>>(                                   \
        transfer, phi, out, GI, GO, NL, num_points, ps_g, ps_n, ps_x, os_g, os_n, os_x);                              \
  } else {                                                                                                            \
    moments_scalar_kernel<KMAX><<<dim3((unsigned)num_moments, bx, (unsigned)k_count), kThreads, 0, s>>>(              \
        transfer, phi, out, GI, GO, NL, num_points, ps_g, ps_n, ps_k, ps_x, os_g, os_n, os_k, os_x);                  \
  }
  if (GI <= 4) {
    CITRUS_MOMENTS_LAUNCH(4)
  } else if (GI <= 8) {
    CITRUS_MOMENTS_LAUNCH(8)
  } else if (GI <= 16) {
    CITRUS_MOMENTS_LAUNCH(16)
  } else {
    CITRUS_MOMENTS_LAUNCH(32)
  }
#undef CITRUS_MOMENTS_LAUNCH
  note_launches();
  return launch_status("citrus_scattering_moments");
}
