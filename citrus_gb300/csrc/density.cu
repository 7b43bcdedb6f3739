// Interpolating density model: the density of one reference material from an attenuation volume X in 1/cm
// (citrus/utilities.py:710-799, attenuation_to_density).
//
// The materials, sorted by nominal attenuation mu_s = rho_s^nom m_s at the model energy, bracket X: on [mu_{s-1},
// mu_s) material s gets f rho_s^nom with f = (X - mu_{s-1}) / (mu_s - mu_{s-1}); on [mu_s, mu_{s+1}) it gets
// (1 - f) rho_s^nom with f = (X - mu_s) / (mu_{s+1} - mu_s); below mu_0 the first material alone gets max(X, 0) / m_0,
// from mu_{M-1} on the last material alone gets X / m_{M-1}; elsewhere 0. The float32 operations are those of the
// reference's tensor expressions (IEEE division, one rounding per operation), so the maps agree bit for bit.
#include "common.cuh"

namespace citrus {
namespace {

constexpr int kDensityThreads = 256;

__global__ void __launch_bounds__(kDensityThreads) density_kernel(const float* __restrict__ X, int64_t V,
                                                                  const float* __restrict__ mu,
                                                                  const float* __restrict__ mass,
                                                                  const float* __restrict__ nominal, int M, int slot,
                                                                  float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * kDensityThreads + threadIdx.x;
  if (i >= V) return;
  const float x = X[i];
  float r = 0.f;
  if (slot >= 1 && x >= mu[slot - 1] && x < mu[slot])
    r = __fmul_rn(__fdiv_rn(__fsub_rn(x, mu[slot - 1]), __fsub_rn(mu[slot], mu[slot - 1])), nominal[slot]);
  if (slot <= M - 2 && x >= mu[slot] && x < mu[slot + 1]) {
    const float f = __fdiv_rn(__fsub_rn(x, mu[slot]), __fsub_rn(mu[slot + 1], mu[slot]));
    r = __fmul_rn(__fadd_rn(-f, 1.0f), nominal[slot]);
  }
  if (slot == 0 && x < mu[0]) r = __fdiv_rn(fmaxf(x, 0.f), mass[0]);
  if (slot == M - 1 && x >= mu[M - 1]) r = __fdiv_rn(x, mass[M - 1]);
  out[i] = r;
}

}  // namespace
}  // namespace citrus

using namespace citrus;

extern "C" int citrus_attenuation_to_density(const float* X, int64_t num_voxels, const float* mu, const float* mass,
                                             const float* nominal, int64_t num_materials, int64_t slot, float* out,
                                             void* stream) {
  CITRUS_REQUIRE(X && mu && mass && nominal && out, "citrus_attenuation_to_density: null pointer argument");
  CITRUS_REQUIRE(num_materials >= 1 && slot >= 0 && slot < num_materials && num_voxels >= 0,
                 "citrus_attenuation_to_density: slot %lld outside %lld materials", (long long)slot,
                 (long long)num_materials);
  if (num_voxels == 0) return CITRUS_OK;
  density_kernel<<<(unsigned)cdiv(num_voxels, kDensityThreads), kDensityThreads, 0, as_stream(stream)>>>(
      X, num_voxels, mu, mass, nominal, (int)num_materials, (int)slot, out);
  note_launches();
  return launch_status("citrus_attenuation_to_density");
}
