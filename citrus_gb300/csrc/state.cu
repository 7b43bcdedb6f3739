// Compact per-view storage of the CITRUS accumulator: the linear-discontinuous cell mean in scaled float16
// (citrus/citrus.py:620-720, StateStore.put / get).
//
// Encoding: for every (group, moment) the largest |cell mean| over the cells is mapped to 2^14, scale = max / 2^14
// (1 where the maximum is 0), and each cell mean is stored as float16(mean / scale) with IEEE division and
// round-to-nearest-even conversion, as the reference's float32 tensor arithmetic does. The maximum carries a NaN as
// the reference's abs().amax() does; "maximum > 0" is then false and that (group, moment) takes the scale 1, its
// other cells stored unscaled, exactly as the reference stores them. Decoding multiplies back in
// float32 and writes zero slopes. One block per (group, moment) reduces the maximum in a fixed order, so the codec is
// bit-exact and deterministic.
#include <cuda_fp16.h>

#include "common.cuh"

namespace citrus {
namespace {

constexpr int kStateThreads = 256;
constexpr float kFloat16Target = 16384.0f;  // 2^14: |q| <= 16384 < 65504

// max that returns a NaN operand (fmaxf drops it)
__device__ __forceinline__ float max_keep_nan(float a, float b) { return isnan(a) ? a : (isnan(b) ? b : fmaxf(a, b)); }

// element (g, n, cell) of the cell-mean component at g * s_g + n * s_n + cell * s_x
__global__ void __launch_bounds__(kStateThreads) state_encode_kernel(const float* __restrict__ acc, int N,
                                                                     int64_t cells, int64_t s_g, int64_t s_n,
                                                                     int64_t s_x, __half* __restrict__ data,
                                                                     float* __restrict__ scale) {
  const int gn = blockIdx.x;  // g * N + n
  const int g = gn / N, n = gn - g * N;
  const float* src = acc + g * s_g + n * s_n;
  __shared__ float red[kStateThreads];
  float m = 0.f;
  for (int64_t x = threadIdx.x; x < cells; x += kStateThreads) m = max_keep_nan(m, fabsf(__ldg(src + x * s_x)));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = kStateThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = max_keep_nan(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  const float maximum = red[0];
  const float sc = maximum > 0.f ? __fdiv_rn(maximum, kFloat16Target) : 1.f;
  if (threadIdx.x == 0) scale[gn] = sc;
  __half* dst = data + (int64_t)gn * cells;
  for (int64_t x = threadIdx.x; x < cells; x += kStateThreads) dst[x] = __float2half_rn(__fdiv_rn(src[x * s_x], sc));
}

// full accumulator element (g, n, k, cell) at g * o_g + n * o_n + k * o_k + cell * o_x: k = 0 the decoded mean, else 0
__global__ void __launch_bounds__(kStateThreads) state_decode_kernel(const __half* __restrict__ data,
                                                                     const float* __restrict__ scale, int N,
                                                                     int64_t cells, float* __restrict__ out,
                                                                     int64_t o_g, int64_t o_n, int64_t o_k,
                                                                     int64_t o_x) {
  const int gn = blockIdx.y;
  const int g = gn / N, n = gn - g * N;
  const int64_t x = (int64_t)blockIdx.x * kStateThreads + threadIdx.x;
  if (x >= cells) return;
  const float v = __half2float(data[(int64_t)gn * cells + x]) * __ldg(scale + gn);
  float* o = out + g * o_g + n * o_n + x * o_x;
  o[0] = v;
  o[o_k] = 0.f;
  o[2 * o_k] = 0.f;
  o[3 * o_k] = 0.f;
}

}  // namespace
}  // namespace citrus

using namespace citrus;

extern "C" int citrus_state_encode(const float* accumulator, int64_t groups, int64_t moments, int64_t cells,
                                   int64_t s_g, int64_t s_n, int64_t s_x, uint16_t* data, float* scale,
                                   void* stream) {
  CITRUS_REQUIRE(accumulator && data && scale, "citrus_state_encode: null pointer argument");
  CITRUS_REQUIRE(groups >= 1 && moments >= 1 && cells >= 1 && groups * moments <= (1 << 30),
                 "citrus_state_encode: bad sizes (groups %lld, moments %lld, cells %lld)", (long long)groups,
                 (long long)moments, (long long)cells);
  state_encode_kernel<<<(unsigned)(groups * moments), kStateThreads, 0, as_stream(stream)>>>(
      accumulator, (int)moments, cells, s_g, s_n, s_x, reinterpret_cast<__half*>(data), scale);
  note_launches();
  return launch_status("citrus_state_encode");
}

extern "C" int citrus_state_decode(const uint16_t* data, const float* scale, int64_t groups, int64_t moments,
                                   int64_t cells, float* accumulator, int64_t o_g, int64_t o_n, int64_t o_k,
                                   int64_t o_x, void* stream) {
  CITRUS_REQUIRE(accumulator && data && scale, "citrus_state_decode: null pointer argument");
  CITRUS_REQUIRE(groups >= 1 && moments >= 1 && cells >= 1 && groups * moments <= 65535,
                 "citrus_state_decode: bad sizes (groups %lld, moments %lld, cells %lld)", (long long)groups,
                 (long long)moments, (long long)cells);
  dim3 grid((unsigned)cdiv(cells, kStateThreads), (unsigned)(groups * moments));
  state_decode_kernel<<<grid, kStateThreads, 0, as_stream(stream)>>>(reinterpret_cast<const __half*>(data), scale,
                                                                     (int)moments, cells, accumulator, o_g, o_n,
                                                                     o_k, o_x);
  note_launches();
  return launch_status("citrus_state_decode");
}
