// Uncollided fluence and first-collision source of one view.
//
//  * group transmission, T_g = sum_{e in g} w_e exp(-sum_m mu_m(e) P_m - mu_f(e) P_f)
//    (citrus/scatter_solver/cross_sections.py:797-883, kernels/transmission_kernels.py:187-226), optionally times a
//    per-point factor (the source weight b / |r - r0|^2 of uncollided.py:160-197);
//  * the focal-spot weight b(Omega) / |r - r0|^2 at points (source.py:289-382: 1 where the ray from the focal spot
//    meets the collimated field on the panel);
//  * the first-collision source S_FC,g(r, omega) = sum_m rho_m sum_{g' <= g} T_m^{g' -> g}(Omega_UC . omega) phi_g'
//    with the transfer interpolated linearly in eta (uncollided.py:200-308, cross_sections.py:905-1021), and three
//    fused forms of it: the LD moments of the corrected source per transport cell, written cell-major into the
//    sweep's store (uncollided.py:464-511, uncollided_kernels.py:552-634); the quadrature sums I0, I1, I2 with the
//    exact moments E0, E1 and the float64 correction factors (uncollided.py:357-461, 538-636); and the attenuated
//    total emission of the collapsed-cone image with per-block sums of its mean panel height
//    (scatter_image.py:829-874, uncollided_kernels.py:712-795).
//
// Thread layout of the point kernels: a block is 32 points (threadIdx.x) by the outgoing groups (threadIdx.y), so a
// warp reads and writes 32 consecutive points of one group. The transfer table is laid out [M, N_eta, G_out, G_in]
// (downscatter only, zero above the diagonal), so the 32 B row of one outgoing group at one node is one vector load.
#include <math.h>

#include "common.cuh"

namespace citrus {
namespace {

constexpr int kPoints = 32;
constexpr int kMaxG = 32;
constexpr int kMaxM = 8;

struct PointGrid {
  int R, C, S;            // points of the quadrature grid
  int f;                  // points per cell axis (q)
  int Rc, Cc, Sc;         // transport cells
};

__device__ __forceinline__ void point_rcs(int64_t v, const PointGrid& g, int& i, int& j, int& k) {
  const int64_t cs = (int64_t)g.C * g.S;
  i = (int)(v / cs);
  const int64_t rem = v - (int64_t)i * cs;
  j = (int)(rem / g.S);
  k = (int)(rem - (int64_t)j * g.S);
}

// unit primary direction from the focal spot to point (x, y, z), IEEE sqrt and division
__device__ __forceinline__ void primary_direction(float x, float y, float z, float r0x, float r0y, float r0z,
                                                  float& ux, float& uy, float& uz) {
  const float dx = x - r0x, dy = y - r0y, dz = z - r0z;
  const float n = __fsqrt_rn(dx * dx + dy * dy + dz * dz);
  ux = __fdiv_rn(dx, n);
  uy = __fdiv_rn(dy, n);
  uz = __fdiv_rn(dz, n);
}

struct Table {
  const float* t;    // [M, N, G, G] transfer by (node, g_out, g_in)
  int M, N, G;
  float eta_lo, eta_hi;
};

// table position of a cosine (cross_sections.py:905-938, uniform table)
__device__ __forceinline__ void table_position(const Table& tb, float cosine, int& i0, float& w) {
  const float eta = fminf(fmaxf(cosine, tb.eta_lo), tb.eta_hi);
  const float pos = __fdiv_rn(eta - tb.eta_lo, tb.eta_hi - tb.eta_lo) * (float)(tb.N - 1);
  float f0 = floorf(pos);
  f0 = fminf(fmaxf(f0, 0.f), (float)(tb.N - 2));
  i0 = (int)f0;
  w = fminf(fmaxf(pos - f0, 0.f), 1.f);
}

// S_FC of group go at one point for one direction: sum_m rho_m [(1 - w) T_m[i0] + w T_m[i0 + 1]] . phi
template <int kG>
__device__ __forceinline__ float fc_value(const Table& tb, int i0, float w, int go, const float* rho,
                                          const float* phi) {
  const int G = kG > 0 ? kG : tb.G;
  float acc = 0.f;
  for (int m = 0; m < tb.M; ++m) {
    const float r = rho[m];
    if (r == 0.f) continue;
    const float* row0 = tb.t + (((int64_t)m * tb.N + i0) * G + go) * G;
    const float* row1 = row0 + (int64_t)G * G;
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int gi = 0; gi < (kG > 0 ? kG : kMaxG); ++gi) {
      if (gi > go || gi >= G) break;
      a0 = fmaf(__ldg(row0 + gi), phi[gi], a0);
      a1 = fmaf(__ldg(row1 + gi), phi[gi], a1);
    }
    acc = fmaf(r, a0 + (a1 - a0) * w, acc);
  }
  return acc;
}

// ---- group transmission -------------------------------------------------------------------------------------
__global__ void transmission_kernel(const float* __restrict__ path, int Mp, int64_t P,
                                    const float* __restrict__ fine_mu /*[Mp, E]*/, const float* __restrict__ weight,
                                    const int* __restrict__ group, int E, int G, const float* __restrict__ filter_path,
                                    const float* __restrict__ filter_mu, const float* __restrict__ factor,
                                    float* __restrict__ out) {
  extern __shared__ float sm[];
  float* s_mu = sm;                        // [Mp, E]
  float* s_w = sm + Mp * E;                // [E]
  float* s_f = s_w + E;                    // [E]
  int* s_g = reinterpret_cast<int*>(s_f + E);
  for (int i = threadIdx.x; i < Mp * E; i += blockDim.x) s_mu[i] = fine_mu[i];
  for (int i = threadIdx.x; i < E; i += blockDim.x) {
    s_w[i] = weight[i];
    s_f[i] = filter_mu ? filter_mu[i] : 0.f;
    s_g[i] = group[i];
  }
  __syncthreads();
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  float pm[kMaxM];
#pragma unroll
  for (int m = 0; m < kMaxM; ++m) pm[m] = m < Mp ? path[(int64_t)m * P + p] : 0.f;
  const float pf = filter_path ? filter_path[p] : 0.f;
  float acc[kMaxG];
#pragma unroll
  for (int g = 0; g < kMaxG; ++g) acc[g] = 0.f;
  for (int e = 0; e < E; ++e) {
    float tau = s_mu[e] * pm[0];
    for (int m = 1; m < Mp; ++m) tau = fmaf(s_mu[m * E + e], pm[m], tau);
    if (filter_path) tau = fmaf(s_f[e], pf, tau);  // the filter after the materials, as the reference adds it
    const float t = s_w[e] * expf(-tau);
    const int g = s_g[e];
#pragma unroll
    for (int q = 0; q < kMaxG; ++q)
      if (q == g) acc[q] += t;
  }
  const float fac = factor ? factor[p] : 1.f;
#pragma unroll
  for (int g = 0; g < kMaxG; ++g)
    if (g < G) out[(int64_t)g * P + p] = acc[g] * fac;
}

// ---- focal-spot weight b / |r - r0|^2 -----------------------------------------------------------------------
struct Field {
  int curved;
  double r0[3];
  double center[3], u_hat[3], v_hat[3], n_hat[3];
  double sdd;
  double off_u, off_v, half_u, half_v, margin_u, margin_v;
};

__device__ __forceinline__ float source_weight(const Field& fd, float x, float y, float z, int squared) {
  const double dx = x - fd.r0[0], dy = y - fd.r0[1], dz = z - fd.r0[2];
  double t;
  if (!fd.curved) {
    const double den = dx * fd.n_hat[0] + dy * fd.n_hat[1] + dz * fd.n_hat[2];
    const double num = (fd.center[0] - fd.r0[0]) * fd.n_hat[0] + (fd.center[1] - fd.r0[1]) * fd.n_hat[1] +
                       (fd.center[2] - fd.r0[2]) * fd.n_hat[2];
    t = num / den;
  } else {  // from the cylinder's axis: |h(t d)| = SDD -> t = SDD / |h(d)|
    const double a = dx * dx + dy * dy;
    t = a > 0 ? fd.sdd / sqrt(a) : INFINITY;
  }
  double w = 0.0;
  if (isfinite(t) && t > 0) {
    const double hx = fd.r0[0] + t * dx, hy = fd.r0[1] + t * dy, hz = fd.r0[2] + t * dz;
    double u, v;
    if (!fd.curved) {
      u = (hx - fd.center[0]) * fd.u_hat[0] + (hy - fd.center[1]) * fd.u_hat[1] + (hz - fd.center[2]) * fd.u_hat[2];
      v = (hx - fd.center[0]) * fd.v_hat[0] + (hy - fd.center[1]) * fd.v_hat[1] + (hz - fd.center[2]) * fd.v_hat[2];
    } else {
      const double ex = hx - fd.r0[0], ey = hy - fd.r0[1], ez = hz - fd.r0[2];
      const double depth = -(ex * fd.n_hat[0] + ey * fd.n_hat[1] + ez * fd.n_hat[2]);
      u = fd.sdd * atan2(ex * fd.u_hat[0] + ey * fd.u_hat[1] + ez * fd.u_hat[2], depth);
      v = fd.sdd * (ex * fd.v_hat[0] + ey * fd.v_hat[1] + ez * fd.v_hat[2]) / depth;
    }
    const bool inside = fabs(u + fd.off_u) <= fd.half_u + fd.margin_u && fabs(v + fd.off_v) <= fd.half_v + fd.margin_v;
    w = inside ? 1.0 : 0.0;
  }
  if (!squared) return (float)w;
  const float fx = x - (float)fd.r0[0], fy = y - (float)fd.r0[1], fz = z - (float)fd.r0[2];
  return (float)w / (fx * fx + fy * fy + fz * fz);
}

__global__ void source_weight_kernel(Field fd, const double* __restrict__ pts, const double* __restrict__ ax_x,
                                     const double* __restrict__ ax_y, const double* __restrict__ ax_z, int gc, int gs,
                                     int64_t P, int squared, float* __restrict__ out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  float x, y, z;
  if (pts) {
    x = (float)pts[3 * p];
    y = (float)pts[3 * p + 1];
    z = (float)pts[3 * p + 2];
  } else {
    const int64_t row = p / ((int64_t)gc * gs), rem = p - row * (int64_t)gc * gs, col = rem / gs;
    x = (float)ax_x[col];
    y = (float)ax_y[row];
    z = (float)ax_z[rem - col * gs];
  }
  out[p] = source_weight(fd, x, y, z, squared);
}

// ---- shared point inputs of the first-collision kernels ---------------------------------------------------------
struct FCInputs {
  const float* rho;   // [M, V]
  const float* phi;   // [G, V]
  const float* ax_x;  // [C] point coordinates (float32, as the reference's float32 path)
  const float* ax_y;  // [R]
  const float* ax_z;  // [S]
  float r0x, r0y, r0z;
  int64_t V;
};

template <int kG>
__device__ __forceinline__ void load_point(const FCInputs& in, const Table& tb, int64_t v, float* rho, float* phi) {
  const int G = kG > 0 ? kG : tb.G;
  for (int m = 0; m < tb.M; ++m) rho[m] = __ldg(in.rho + (int64_t)m * in.V + v);
#pragma unroll
  for (int g = 0; g < (kG > 0 ? kG : kMaxG); ++g)
    if (g < G) phi[g] = __ldg(in.phi + (int64_t)g * in.V + v);
}

// ---- first-collision source [K, G, V] ------------------------------------------------------------------------
template <int kG>
__global__ void fc_source_kernel(FCInputs in, Table tb, PointGrid pg, const float* __restrict__ omegas, int K,
                                 int KB, float* __restrict__ out) {
  const int64_t v = (int64_t)blockIdx.x * kPoints + threadIdx.x;
  const int go = threadIdx.y;
  if (v >= in.V) return;
  int i, j, k;
  point_rcs(v, pg, i, j, k);
  float ux, uy, uz;
  primary_direction(__ldg(in.ax_x + j), __ldg(in.ax_y + i), __ldg(in.ax_z + k), in.r0x, in.r0y, in.r0z, ux, uy, uz);
  float rho[kMaxM], phi[kG > 0 ? kG : kMaxG];
  load_point<kG>(in, tb, v, rho, phi);
  const int G = kG > 0 ? kG : tb.G;
  for (int kb = 0; kb < KB; ++kb) {
    const int d = blockIdx.y * KB + kb;
    if (d >= K) break;
    const float cosine = ux * __ldg(omegas + 3 * d) + uy * __ldg(omegas + 3 * d + 1) + uz * __ldg(omegas + 3 * d + 2);
    int i0;
    float w;
    table_position(tb, cosine, i0, w);
    out[((int64_t)d * G + go) * in.V + v] = fc_value<kG>(tb, i0, w, go, rho, phi);
  }
}

// ---- LD moments of the corrected source per transport cell, cell-major [K, NC, G, 4] ---------------------------
template <int kG>
__global__ void fc_moments_kernel(FCInputs in, Table tb, PointGrid pg, const float* __restrict__ omegas, int K,
                                  const float* __restrict__ scale, const float* __restrict__ beta, float slope_scale,
                                  float* __restrict__ out, int64_t out_k_stride) {
  const int64_t NC = (int64_t)pg.Rc * pg.Cc * pg.Sc;
  const int64_t c = (int64_t)blockIdx.x * kPoints + threadIdx.x;
  const int go = threadIdx.y;
  const int d = blockIdx.y;
  if (c >= NC || d >= K) return;
  const int G = kG > 0 ? kG : tb.G;
  const int64_t csc = (int64_t)pg.Cc * pg.Sc;
  const int ic = (int)(c / csc);
  const int jc = (int)((c - (int64_t)ic * csc) / pg.Sc);
  const int kc = (int)(c - (int64_t)ic * csc - (int64_t)jc * pg.Sc);
  const float ox = __ldg(omegas + 3 * d), oy = __ldg(omegas + 3 * d + 1), oz = __ldg(omegas + 3 * d + 2);
  const int F = pg.f;
  float m0 = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
  for (int a = 0; a < F; ++a) {      // rows (y)
    for (int b = 0; b < F; ++b) {    // cols (x)
      for (int e = 0; e < F; ++e) {  // slices (z)
        const int i = ic * F + a, j = jc * F + b, k = kc * F + e;
        const int64_t v = ((int64_t)i * pg.C + j) * pg.S + k;
        float ux, uy, uz;
        primary_direction(__ldg(in.ax_x + j), __ldg(in.ax_y + i), __ldg(in.ax_z + k), in.r0x, in.r0y, in.r0z, ux, uy,
                          uz);
        float rho[kMaxM], phi[kG > 0 ? kG : kMaxG];
        load_point<kG>(in, tb, v, rho, phi);
        const float cosine = ux * ox + uy * oy + uz * oz;
        int i0;
        float w;
        table_position(tb, cosine, i0, w);
        const float src = fc_value<kG>(tb, i0, w, go, rho, phi);
        const int64_t gv = (int64_t)go * in.V + v;
        const float s = src * __ldg(scale + gv) * (1.f + __ldg(beta + gv) * cosine);
        m0 += s;
        mx += s * ((2.f * b + 1.f) / F - 1.f);
        my += s * ((2.f * a + 1.f) / F - 1.f);
        mz += s * ((2.f * e + 1.f) / F - 1.f);
      }
    }
  }
  const float inv = 1.f / (float)(F * F * F);
  float4 r;
  r.x = m0 * inv;
  r.y = mx * (inv * slope_scale);
  r.z = my * (inv * slope_scale);
  r.w = mz * (inv * slope_scale);
  *reinterpret_cast<float4*>(out + d * out_k_stride + (c * G + go) * 4) = r;
}

// ---- quadrature sums, exact moments and the float64 correction factors -----------------------------------------
template <int kG>
__global__ void fc_sums_kernel(FCInputs in, Table tb, PointGrid pg, const float* __restrict__ omegas,
                               const float* __restrict__ weights, int K, const float* __restrict__ moments /*[M,2,G,G]*/,
                               float* __restrict__ sums /*[5, G, V] or null*/, float* __restrict__ scale,
                               float* __restrict__ beta) {
  const int64_t v = (int64_t)blockIdx.x * kPoints + threadIdx.x;
  const int go = threadIdx.y;
  if (v >= in.V) return;
  const int G = kG > 0 ? kG : tb.G;
  int i, j, k;
  point_rcs(v, pg, i, j, k);
  float ux, uy, uz;
  primary_direction(__ldg(in.ax_x + j), __ldg(in.ax_y + i), __ldg(in.ax_z + k), in.r0x, in.r0y, in.r0z, ux, uy, uz);
  float rho[kMaxM], phi[kG > 0 ? kG : kMaxG];
  load_point<kG>(in, tb, v, rho, phi);
  float E0 = 0.f, E1 = 0.f;
  for (int m = 0; m < tb.M; ++m) {
    const float* r0 = moments + (((int64_t)m * 2 + 0) * G + go) * G;
    const float* r1 = moments + (((int64_t)m * 2 + 1) * G + go) * G;
    float a0 = 0.f, a1 = 0.f;
    for (int gi = 0; gi <= go; ++gi) {
      a0 = fmaf(__ldg(r0 + gi), phi[gi], a0);
      a1 = fmaf(__ldg(r1 + gi), phi[gi], a1);
    }
    E0 = fmaf(rho[m], a0, E0);
    E1 = fmaf(rho[m], a1, E1);
  }
  float I0 = 0.f, I1 = 0.f, I2 = 0.f;
  for (int d = 0; d < K; ++d) {
    const float cosine = ux * __ldg(omegas + 3 * d) + uy * __ldg(omegas + 3 * d + 1) + uz * __ldg(omegas + 3 * d + 2);
    int i0;
    float w;
    table_position(tb, cosine, i0, w);
    const float ws = fc_value<kG>(tb, i0, w, go, rho, phi) * __ldg(weights + d);
    I0 += ws;
    I1 += ws * cosine;
    I2 += ws * (cosine * cosine);
  }
  const int64_t gv = (int64_t)go * in.V + v;
  if (sums) {
    const int64_t GV = (int64_t)G * in.V;
    sums[gv] = I0;
    sums[GV + gv] = I1;
    sums[2 * GV + gv] = I2;
    sums[3 * GV + gv] = E0;
    sums[4 * GV + gv] = E1;
  }
  // factors in float64 (uncollided.py:611-636)
  const double i0d = I0, i1d = I1, i2d = I2, e0 = E0, e1 = E1;
  const bool pos = e0 > 0;
  const double c = pos ? e1 / e0 : 0.0;
  const double den = i2d - c * i1d;
  const bool ok = pos && fabs(den) > 1e-12 * fabs(i0d);
  double b = ok ? (c * i0d - i1d) / den : 0.0;
  b = fmin(fmax(b, -1.0), 1.0);
  const double d0 = i0d + b * i1d;
  scale[gv] = (float)(d0 > 0 ? e0 / d0 : 1.0);
  beta[gv] = (float)b;
}

// ---- attenuated total emission of the image ---------------------------------------------------------------------
// e = (S_FC + S_MC,cell) exp(-max(0, tau_cell - mu_cell omega . (r - r_cell))), written voxel-major [k, V, G] (or the
// weighted group sum [k, V] with signal weights), and per block the sums of e and e h (h = panel height of the point).
template <int kG>
__global__ void emission_kernel(FCInputs in, Table tb, PointGrid pg, const float* __restrict__ omegas, int K,
                                const float* __restrict__ tau /*[K, G, NC]*/, const float* __restrict__ mu /*[G, NC]*/,
                                const float* __restrict__ multiple /*[K, G, NC]*/, const float* __restrict__ heights,
                                const float* __restrict__ signal_weight /*[K, G] or null*/, float dx, float dy,
                                float dz, float* __restrict__ out, float* __restrict__ partial /*[K, nblocks, 2]*/) {
  __shared__ float tile[kPoints * kMaxG];
  __shared__ float red[2][kMaxG][kPoints + 1];
  const int64_t v = (int64_t)blockIdx.x * kPoints + threadIdx.x;
  const int go = threadIdx.y;
  const int G = kG > 0 ? kG : tb.G;
  const bool valid = v < in.V;
  const int64_t NC = (int64_t)pg.Rc * pg.Cc * pg.Sc;
  float rho[kMaxM], phi[kG > 0 ? kG : kMaxG];
  float ux = 0.f, uy = 0.f, uz = 0.f, h = 0.f, muc = 0.f, offx = 0.f, offy = 0.f, offz = 0.f;
  int64_t cell = 0;
  if (valid) {
    int i, j, k;
    point_rcs(v, pg, i, j, k);
    primary_direction(__ldg(in.ax_x + j), __ldg(in.ax_y + i), __ldg(in.ax_z + k), in.r0x, in.r0y, in.r0z, ux, uy, uz);
    load_point<kG>(in, tb, v, rho, phi);
    const int F = pg.f, ic = i / F, jc = j / F, kc = k / F;
    cell = ((int64_t)ic * pg.Cc + jc) * pg.Sc + kc;
    const float half = (F - 1) * 0.5f;
    offy = dy * ((float)(i - ic * F) - half);
    offx = dx * ((float)(j - jc * F) - half);
    offz = dz * ((float)(k - kc * F) - half);
    h = heights ? __ldg(heights + v) : 0.f;
    muc = __ldg(mu + (int64_t)go * NC + cell);
  }
  const int64_t base_v = (int64_t)blockIdx.x * kPoints;
  const int npts = (int)min((int64_t)kPoints, in.V - base_v);
  const int KB = (K + gridDim.y - 1) / gridDim.y;
  for (int kb = 0; kb < KB; ++kb) {
    const int d = blockIdx.y * KB + kb;
    if (d >= K) break;
    float e = 0.f;
    if (valid) {
      const float ox = __ldg(omegas + 3 * d), oy = __ldg(omegas + 3 * d + 1), oz = __ldg(omegas + 3 * d + 2);
      const float cosine = ux * ox + uy * oy + uz * oz;
      int i0;
      float w;
      table_position(tb, cosine, i0, w);
      const float src = fc_value<kG>(tb, i0, w, go, rho, phi);
      const int64_t kc = ((int64_t)d * G + go) * NC + cell;
      const float offset = oy * offy + ox * offx + oz * offz;
      const float depth = fmaxf(__ldg(tau + kc) - muc * offset, 0.f);
      e = (src + __ldg(multiple + kc)) * expf(-depth);
    }
    __syncthreads();
    red[0][go][threadIdx.x] = e;
    red[1][go][threadIdx.x] = e * h;
    if (signal_weight == nullptr) tile[threadIdx.x * G + go] = e;
    __syncthreads();
    if (signal_weight == nullptr) {
      // the block's [points, G] tile is contiguous in the voxel-major output
      float* o = out + ((int64_t)d * in.V + base_v) * G;
      for (int q = threadIdx.y * kPoints + threadIdx.x; q < npts * G; q += kPoints * G) o[q] = tile[q];
    } else if (threadIdx.y == 0 && valid) {
      float s = 0.f;
      for (int g = 0; g < G; ++g) s = fmaf(__ldg(signal_weight + (int64_t)d * G + g), red[0][g][threadIdx.x], s);
      out[(int64_t)d * in.V + v] = s;
    }
    if (threadIdx.y == 0 && threadIdx.x < 2) {  // fixed-order block sums: deterministic
      const int which = threadIdx.x;
      float s = 0.f;
      for (int g = 0; g < G; ++g)
        for (int p = 0; p < kPoints; ++p) s += red[which][g][p];
      partial[((int64_t)d * gridDim.x + blockIdx.x) * 2 + which] = s;
    }
  }
}

// sums over the blocks of the emission's partial sums, in block order: [K, nblocks, 2] -> [K, 2]
__global__ void reduce_partials_kernel(const float* __restrict__ partial, int64_t nblocks, int K,
                                       float* __restrict__ out) {
  const int d = blockIdx.x;
  const int which = threadIdx.y;
  __shared__ double s[2][256];
  double acc = 0.0;
  for (int64_t b = threadIdx.x; b < nblocks; b += blockDim.x) acc += partial[((int64_t)d * nblocks + b) * 2 + which];
  s[which][threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w /= 2) {
    if (threadIdx.x < w) s[which][threadIdx.x] += s[which][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[d * 2 + which] = (float)s[which][0];
}

int check_table(const float* table, int64_t M, int64_t N, int64_t G) {
  CITRUS_REQUIRE(table != nullptr, "first collision: null transfer table");
  CITRUS_REQUIRE(M >= 1 && M <= kMaxM, "first collision: %lld materials outside [1, %d]", (long long)M, kMaxM);
  CITRUS_REQUIRE(N >= 2 && G >= 1 && G <= kMaxG, "first collision: bad table (N %lld, G %lld)", (long long)N,
                 (long long)G);
  return CITRUS_OK;
}

FCInputs make_inputs(const float* rho, const float* phi, const float* ax, int64_t V, const double* r0,
                     const int64_t* pdims) {
  FCInputs in;
  in.rho = rho;
  in.phi = phi;
  in.ax_x = ax;                    // x [C] then y [R] then z [S]
  in.ax_y = ax + pdims[1];
  in.ax_z = ax + pdims[1] + pdims[0];
  in.r0x = (float)r0[0];
  in.r0y = (float)r0[1];
  in.r0z = (float)r0[2];
  in.V = V;
  return in;
}

PointGrid make_grid(const int64_t* pdims, int64_t f) {
  PointGrid pg;
  pg.R = (int)pdims[0];
  pg.C = (int)pdims[1];
  pg.S = (int)pdims[2];
  pg.f = (int)f;
  pg.Rc = pg.R / pg.f;
  pg.Cc = pg.C / pg.f;
  pg.Sc = pg.S / pg.f;
  return pg;
}

#define CITRUS_G_DISPATCH(G, KERNEL, GRID, BLOCK, SMEM, STREAM, ...)                         \
  switch (G) {                                                                                \
    case 1: KERNEL<1><<<GRID, BLOCK, SMEM, STREAM>>>(__VA_ARGS__); break;                    \
    case 4: KERNEL<4><<<GRID, BLOCK, SMEM, STREAM>>>(__VA_ARGS__); break;                    \
    case 8: KERNEL<8><<<GRID, BLOCK, SMEM, STREAM>>>(__VA_ARGS__); break;                    \
    case 16: KERNEL<16><<<GRID, BLOCK, SMEM, STREAM>>>(__VA_ARGS__); break;                  \
    default: KERNEL<0><<<GRID, BLOCK, SMEM, STREAM>>>(__VA_ARGS__); break;                   \
  }

}  // namespace
}  // namespace citrus

using namespace citrus;

extern "C" int citrus_group_transmission(const float* path, int64_t num_materials, int64_t num_points,
                                         const float* fine_mu, const float* fine_weight, const int32_t* fine_group,
                                         int64_t num_fine, int64_t num_groups, const float* filter_path,
                                         const float* filter_mu, const float* factor, float* out, void* stream) {
  CITRUS_REQUIRE(path && fine_mu && fine_weight && fine_group && out, "citrus_group_transmission: null pointer");
  CITRUS_REQUIRE(num_materials >= 1 && num_materials <= kMaxM && num_groups >= 1 && num_groups <= kMaxG &&
                     num_fine >= 1 && num_points >= 0,
                 "citrus_group_transmission: bad sizes (materials %lld, groups %lld, fine %lld)",
                 (long long)num_materials, (long long)num_groups, (long long)num_fine);
  CITRUS_REQUIRE((filter_path == nullptr) == (filter_mu == nullptr),
                 "citrus_group_transmission: filter_path and filter_mu go together");
  const size_t smem = (size_t)(num_materials * num_fine + 2 * num_fine) * sizeof(float) + num_fine * sizeof(int);
  CITRUS_REQUIRE(smem <= 96 * 1024, "citrus_group_transmission: %lld fine energies too many", (long long)num_fine);
  if (num_points == 0) return CITRUS_OK;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(transmission_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  transmission_kernel<<<(unsigned)cdiv(num_points, 128), 128, smem, as_stream(stream)>>>(
      path, (int)num_materials, num_points, fine_mu, fine_weight, fine_group, (int)num_fine, (int)num_groups,
      filter_path, filter_mu, factor, out);
  return launch_status("citrus_group_transmission");
}

extern "C" int citrus_source_weight(const double* field, const double* points, const double* axis_x,
                                    const double* axis_y, const double* axis_z, const int64_t* point_dims,
                                    int64_t num_points, int32_t divide_by_distance_squared, float* out, void* stream) {
  CITRUS_REQUIRE(field && out, "citrus_source_weight: null pointer");
  CITRUS_REQUIRE(points || (axis_x && axis_y && axis_z && point_dims), "citrus_source_weight: no points");
  Field fd;
  fd.curved = field[0] != 0.0;
  for (int a = 0; a < 3; ++a) {
    fd.r0[a] = field[1 + a];
    fd.center[a] = field[4 + a];
    fd.u_hat[a] = field[7 + a];
    fd.v_hat[a] = field[10 + a];
    fd.n_hat[a] = field[13 + a];
  }
  fd.sdd = field[16];
  fd.off_u = field[17];
  fd.off_v = field[18];
  fd.half_u = field[19];
  fd.half_v = field[20];
  fd.margin_u = field[21];
  fd.margin_v = field[22];
  int gc = 1, gs = 1;
  if (!points) {
    gc = (int)point_dims[1];
    gs = (int)point_dims[2];
  }
  if (num_points == 0) return CITRUS_OK;
  source_weight_kernel<<<(unsigned)cdiv(num_points, 128), 128, 0, as_stream(stream)>>>(
      fd, points, axis_x, axis_y, axis_z, gc, gs, num_points, divide_by_distance_squared, out);
  return launch_status("citrus_source_weight");
}

extern "C" int citrus_first_collision_source(const float* rho, int64_t num_materials, const float* phi,
                                             int64_t num_groups, const float* axes, const int64_t* point_dims,
                                             const double* focal_spot, const float* table, int64_t num_eta,
                                             double eta_lo, double eta_hi, const float* omegas,
                                             int64_t num_directions, float* out, void* stream) {
  int st = check_table(table, num_materials, num_eta, num_groups);
  if (st) return st;
  CITRUS_REQUIRE(rho && phi && axes && point_dims && focal_spot && omegas && out,
                 "citrus_first_collision_source: null pointer");
  const int64_t V = point_dims[0] * point_dims[1] * point_dims[2];
  if (V == 0 || num_directions == 0) return CITRUS_OK;
  const FCInputs in = make_inputs(rho, phi, axes, V, focal_spot, point_dims);
  const Table tb{table, (int)num_materials, (int)num_eta, (int)num_groups, (float)eta_lo, (float)eta_hi};
  const PointGrid pg = make_grid(point_dims, 1);
  const int G = (int)num_groups, K = (int)num_directions, KB = 4;
  dim3 grid((unsigned)cdiv(V, kPoints), (unsigned)cdiv(K, KB)), block(kPoints, G);
  CITRUS_G_DISPATCH(G, fc_source_kernel, grid, block, 0, as_stream(stream), in, tb, pg, omegas, K, KB, out)
  return launch_status("citrus_first_collision_source");
}

extern "C" int citrus_first_collision_moments(const float* rho, int64_t num_materials, const float* phi,
                                              int64_t num_groups, const float* axes, const int64_t* point_dims,
                                              int64_t points_per_cell, const double* focal_spot, const float* table,
                                              int64_t num_eta, double eta_lo, double eta_hi, const float* omegas,
                                              int64_t num_directions, const float* scale, const float* beta,
                                              float* out, int64_t out_direction_stride, void* stream) {
  int st = check_table(table, num_materials, num_eta, num_groups);
  if (st) return st;
  CITRUS_REQUIRE(rho && phi && axes && point_dims && focal_spot && omegas && scale && beta && out,
                 "citrus_first_collision_moments: null pointer");
  const int64_t f = points_per_cell;
  CITRUS_REQUIRE(f >= 1 && point_dims[0] % f == 0 && point_dims[1] % f == 0 && point_dims[2] % f == 0,
                 "citrus_first_collision_moments: the point grid is not cells x %lld", (long long)f);
  CITRUS_REQUIRE(((uintptr_t)out % 16) == 0 && out_direction_stride % 4 == 0,
                 "citrus_first_collision_moments: out must be 16-byte aligned");
  CITRUS_REQUIRE(num_directions <= 65535, "citrus_first_collision_moments: too many directions");
  const int64_t V = point_dims[0] * point_dims[1] * point_dims[2];
  if (V == 0 || num_directions == 0) return CITRUS_OK;
  const FCInputs in = make_inputs(rho, phi, axes, V, focal_spot, point_dims);
  const Table tb{table, (int)num_materials, (int)num_eta, (int)num_groups, (float)eta_lo, (float)eta_hi};
  const PointGrid pg = make_grid(point_dims, f);
  double mean_u2 = 0;
  for (int j = 0; j < f; ++j) {
    const double u = (2.0 * j + 1.0) / f - 1.0;
    mean_u2 += u * u / f;
  }
  const float slope_scale = f > 1 ? (float)(1.0 / mean_u2) : 0.f;
  const int64_t NC = V / (f * f * f);
  const int G = (int)num_groups, K = (int)num_directions;
  dim3 grid((unsigned)cdiv(NC, kPoints), (unsigned)K), block(kPoints, G);
  CITRUS_G_DISPATCH(G, fc_moments_kernel, grid, block, 0, as_stream(stream), in, tb, pg, omegas, K, scale, beta,
                    slope_scale, out, out_direction_stride)
  return launch_status("citrus_first_collision_moments");
}

extern "C" int citrus_first_collision_correction(const float* rho, int64_t num_materials, const float* phi,
                                                 int64_t num_groups, const float* axes, const int64_t* point_dims,
                                                 const double* focal_spot, const float* table, int64_t num_eta,
                                                 double eta_lo, double eta_hi, const float* omegas,
                                                 const float* weights, int64_t num_directions, const float* moments,
                                                 float* sums, float* scale, float* beta, void* stream) {
  int st = check_table(table, num_materials, num_eta, num_groups);
  if (st) return st;
  CITRUS_REQUIRE(rho && phi && axes && point_dims && focal_spot && omegas && weights && moments && scale && beta,
                 "citrus_first_collision_correction: null pointer");
  const int64_t V = point_dims[0] * point_dims[1] * point_dims[2];
  if (V == 0) return CITRUS_OK;
  const FCInputs in = make_inputs(rho, phi, axes, V, focal_spot, point_dims);
  const Table tb{table, (int)num_materials, (int)num_eta, (int)num_groups, (float)eta_lo, (float)eta_hi};
  const PointGrid pg = make_grid(point_dims, 1);
  const int G = (int)num_groups, K = (int)num_directions;
  dim3 grid((unsigned)cdiv(V, kPoints)), block(kPoints, G);
  CITRUS_G_DISPATCH(G, fc_sums_kernel, grid, block, 0, as_stream(stream), in, tb, pg, omegas, weights, K, moments,
                    sums, scale, beta)
  return launch_status("citrus_first_collision_correction");
}

extern "C" int citrus_attenuated_emission(const float* rho, int64_t num_materials, const float* phi,
                                          int64_t num_groups, const float* axes, const int64_t* point_dims,
                                          int64_t points_per_cell, const double* point_deltas,
                                          const double* focal_spot, const float* table, int64_t num_eta,
                                          double eta_lo, double eta_hi, const float* omegas, int64_t num_directions,
                                          const float* tau, const float* mu, const float* multiple,
                                          const float* heights, const float* signal_weight, float* out,
                                          float* partial, int64_t partial_capacity, float* height_sums,
                                          void* stream) {
  int st = check_table(table, num_materials, num_eta, num_groups);
  if (st) return st;
  CITRUS_REQUIRE(rho && phi && axes && point_dims && point_deltas && focal_spot && omegas && tau && mu && multiple &&
                     out && partial && height_sums,
                 "citrus_attenuated_emission: null pointer");
  const int64_t f = points_per_cell;
  CITRUS_REQUIRE(f >= 1 && point_dims[0] % f == 0 && point_dims[1] % f == 0 && point_dims[2] % f == 0,
                 "citrus_attenuated_emission: the point grid is not cells x %lld", (long long)f);
  CITRUS_REQUIRE(num_directions >= 0 && num_directions <= 65535, "citrus_attenuated_emission: bad direction count");
  const int64_t V = point_dims[0] * point_dims[1] * point_dims[2];
  const int64_t nblocks = cdiv(V, kPoints);
  CITRUS_REQUIRE(partial_capacity >= nblocks * num_directions * 2,
                 "citrus_attenuated_emission: partial buffer holds %lld floats, needs %lld",
                 (long long)partial_capacity, (long long)(nblocks * num_directions * 2));
  if (V == 0 || num_directions == 0) return CITRUS_OK;
  const FCInputs in = make_inputs(rho, phi, axes, V, focal_spot, point_dims);
  const Table tb{table, (int)num_materials, (int)num_eta, (int)num_groups, (float)eta_lo, (float)eta_hi};
  const PointGrid pg = make_grid(point_dims, f);
  const int G = (int)num_groups, K = (int)num_directions;
  const int ky = K;  // one direction per block row: the point data is reused from registers across none; simple
  dim3 grid((unsigned)nblocks, (unsigned)ky), block(kPoints, G);
  cudaStream_t s = as_stream(stream);
  CITRUS_G_DISPATCH(G, emission_kernel, grid, block, 0, s, in, tb, pg, omegas, K, tau, mu, multiple, heights,
                    signal_weight, (float)point_deltas[0], (float)point_deltas[1], (float)point_deltas[2], out,
                    partial)
  reduce_partials_kernel<<<K, dim3(256, 2), 0, s>>>(partial, nblocks, K, height_sums);
  return launch_status("citrus_attenuated_emission");
}
