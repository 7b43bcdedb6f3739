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
#include <type_traits>
#include <stdlib.h>

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
  float inv_span;    // 1 / (eta_hi - eta_lo) when the span is a power of two (the product is then the quotient), else 0
};

Table make_table(const float* t, int64_t M, int64_t N, int64_t G, double eta_lo, double eta_hi) {
  Table tb{t, (int)M, (int)N, (int)G, (float)eta_lo, (float)eta_hi, 0.f};
  const float span = tb.eta_hi - tb.eta_lo;
  int e = 0;
  if (span > 0.f && frexpf(span, &e) == 0.5f) tb.inv_span = ldexpf(1.f, 1 - e);
  return tb;
}

// table position of a cosine (cross_sections.py:905-938, uniform table)
__device__ __forceinline__ void table_position(const Table& tb, float cosine, int& i0, float& w) {
  const float eta = fminf(fmaxf(cosine, tb.eta_lo), tb.eta_hi);
  const float q = tb.inv_span != 0.f ? (eta - tb.eta_lo) * tb.inv_span : __fdiv_rn(eta - tb.eta_lo, tb.eta_hi - tb.eta_lo);
  const float pos = q * (float)(tb.N - 1);
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

// Emission profile, off-focal table and beam filter of the source (all optional; float64 tables on the device).
struct SourceExtras {
  const double* profile;    // [rows, channels] relative emission toward each pixel centre, or null
  const double* thickness;  // [t_rows, channels] filter thickness in cm at the pixel centres, or null
  int t_rows;
  const double* off_nodes;  // [n_off] ascending distances past the field edge in cm, or null
  const double* off_values; // [n_off] emission there relative to the field edge
  int n_off;
  int rows, channels;
  double d_row, d_ch, off_row, off_ch;
  double filter_density;
};

// Bilinear at panel coordinates, held at the outermost pixel centres (source.py:484-510)
__device__ double panel_interpolate(const double* __restrict__ img, int img_rows, const SourceExtras& ex, double u,
                                    double v) {
  const double xc = fmin(fmax((u + ex.off_ch) / ex.d_ch + (ex.channels - 1) * 0.5, 0.0), ex.channels - 1.0);
  const double xr = fmin(fmax((v + ex.off_row) / ex.d_row + (ex.rows - 1) * 0.5, 0.0), ex.rows - 1.0);
  const int c0 = min(max((int)floor(xc), 0), max(ex.channels - 2, 0)), c1 = min(c0 + 1, ex.channels - 1);
  int r0 = min(max((int)floor(xr), 0), max(ex.rows - 2, 0)), r1 = min(r0 + 1, ex.rows - 1);
  if (img_rows == 1) r0 = r1 = 0;
  const double wc = fmin(fmax(xc - c0, 0.0), 1.0), wr = fmin(fmax(xr - r0, 0.0), 1.0);
  const double* a = img + (int64_t)r0 * ex.channels;
  const double* b = img + (int64_t)r1 * ex.channels;
  const double top = a[c0] + (a[c1] - a[c0]) * wc;
  const double bottom = b[c0] + (b[c1] - b[c0]) * wc;
  return top + (bottom - top) * wr;
}

// b(Omega) (/ |r - r0|^2) and the filter path rho_f t(Omega) of the ray from the focal spot through (x, y, z)
// (source.py:289-430)
__device__ __forceinline__ float source_field(const Field& fd, const SourceExtras& ex, float x, float y, float z,
                                              int squared, float* filter_path) {
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
  double w = 0.0, path = 0.0;
  if (isfinite(t) && t > 0) {
    const double hx = fd.r0[0] + t * dx, hy = fd.r0[1] + t * dy, hz = fd.r0[2] + t * dz;
    double u, v;
    if (!fd.curved) {
      u = (hx - fd.center[0]) * fd.u_hat[0] + (hy - fd.center[1]) * fd.u_hat[1] + (hz - fd.center[2]) * fd.u_hat[2];
      v = (hx - fd.center[0]) * fd.v_hat[0] + (hy - fd.center[1]) * fd.v_hat[1] + (hz - fd.center[2]) * fd.v_hat[2];
    } else {
      const double ex_ = hx - fd.r0[0], ey = hy - fd.r0[1], ez = hz - fd.r0[2];
      const double depth = -(ex_ * fd.n_hat[0] + ey * fd.n_hat[1] + ez * fd.n_hat[2]);
      u = fd.sdd * atan2(ex_ * fd.u_hat[0] + ey * fd.u_hat[1] + ez * fd.u_hat[2], depth);
      v = fd.sdd * (ex_ * fd.v_hat[0] + ey * fd.v_hat[1] + ez * fd.v_hat[2]) / depth;
    }
    const double edge_u = fd.half_u + fd.margin_u, edge_v = fd.half_v + fd.margin_v;
    const double au = fabs(u + fd.off_u), av = fabs(v + fd.off_v);
    if (au <= edge_u && av <= edge_v) {
      w = 1.0;
    } else if (ex.n_off > 0) {  // past the field edge: the off-focal fraction of the distance to the field rectangle
      const double pu = fmax(au - edge_u, 0.0), pv = fmax(av - edge_v, 0.0);
      const double dist = sqrt(pu * pu + pv * pv);
      if (dist <= ex.off_nodes[ex.n_off - 1]) {
        int above = 0;  // nodes <= dist
        while (above < ex.n_off && ex.off_nodes[above] <= dist) ++above;
        const int i0 = min(max(above - 1, 0), ex.n_off - 1), i1 = min(above, ex.n_off - 1);
        const double span = ex.off_nodes[i1] - ex.off_nodes[i0];
        const double f = span > 0 ? fmin(fmax((dist - ex.off_nodes[i0]) / span, 0.0), 1.0) : 0.0;
        w = ex.off_values[i0] + (ex.off_values[i1] - ex.off_values[i0]) * f;
      }
    }
    if (w != 0.0 && ex.profile) w *= panel_interpolate(ex.profile, ex.rows, ex, u, v);
    if (ex.thickness) path = panel_interpolate(ex.thickness, ex.t_rows, ex, u, v) * ex.filter_density;
  }
  if (filter_path) *filter_path = (float)path;
  if (!squared) return (float)w;
  const float fx = x - (float)fd.r0[0], fy = y - (float)fd.r0[1], fz = z - (float)fd.r0[2];
  return (float)w / (fx * fx + fy * fy + fz * fz);
}

__global__ void source_weight_kernel(Field fd, SourceExtras ex, const double* __restrict__ pts,
                                     const double* __restrict__ ax_x, const double* __restrict__ ax_y,
                                     const double* __restrict__ ax_z, int gc, int gs, int64_t P, int squared,
                                     float* __restrict__ out, float* __restrict__ filter_out) {
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
  float path;
  out[p] = source_field(fd, ex, x, y, z, squared, filter_out ? &path : nullptr);
  if (filter_out) filter_out[p] = path;
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
//
// A block is 32 points by the G groups (a warp holds 32 / G points with their groups in adjacent lanes) by 16, 32 or
// 64 directions (emission_dirs): the [K, NC, G] loads of a warp are coalesced, the point's inputs are loaded once for
// all of the block's directions, and the transfer rows of the eta nodes that the block's points and directions touch are staged
// in shared memory (the window). S_MC is either read ([K, G, NC], the reference's interface) or formed from the
// scattering-source moments of the point's cell held in registers, T[n, g, cell] for n < N_sh, and the harmonics of
// the block's directions in shared memory. The per-block sums are a fixed-order warp butterfly and a fixed-order sum
// over the groups: deterministic.
constexpr int kEmitPoints = 32;
constexpr int kMaxMoments = 64;
constexpr int kRegMoments = 36;  // scattering-source moments held in registers (P5); more are read per direction

// row . phi over the incoming groups (upscatter entries of the table are zero); the row in global memory (read-only
// path) or in shared memory
template <int kGP, bool kShared>
__device__ __forceinline__ float row_dot(const float* __restrict__ row, const float* phi, int G) {
  float a = 0.f;
  if (kGP % 4 == 0 && G == kGP) {
#pragma unroll
    for (int q = 0; q < kGP / 4; ++q) {
      const float4 t = kShared ? reinterpret_cast<const float4*>(row)[q] : __ldg(reinterpret_cast<const float4*>(row) + q);
      a = fmaf(t.x, phi[4 * q], a);
      a = fmaf(t.y, phi[4 * q + 1], a);
      a = fmaf(t.z, phi[4 * q + 2], a);
      a = fmaf(t.w, phi[4 * q + 3], a);
    }
  } else {
#pragma unroll
    for (int gi = 0; gi < kGP; ++gi)
      if (gi < G) a = fmaf(kShared ? row[gi] : __ldg(row + gi), phi[gi], a);
  }
  return a;
}

// The window of table nodes a block needs: its points' cosines with its directions span a few dozen of the eta nodes,
// so the rows of those nodes ([node][m][g][g'], each (node, m) block padded by 4 floats against bank conflicts) are
// staged in shared memory once and every interpolation of the block reads them there.
constexpr int kWindowBytes = 32 * 1024;

__host__ __device__ inline int window_row_stride(int G) { return G * G + 4; }
__host__ __device__ inline int window_nodes(int M, int G, int bytes = kWindowBytes) {
  const int n = bytes / (4 * M * window_row_stride(G));
  return n < 96 ? n : 96;
}


// Stages the table window of a block for the directions s_om[0..n): the eta nodes [lo, hi + 1] that its valid points
// touch, if they fit, else s_window[0] = -1 (rows read from global memory). Each thread evaluates the directions
// first_dir, first_dir + dir_step, ... for its point; s_range holds one (lo, hi) per warp. Ends with a block barrier;
// every thread of the block must call it.
__device__ void stage_window(const Table& tb, bool valid, float ux, float uy, float uz, const float (*s_om)[3], int n,
                             int first_dir, int dir_step, int warp, int nwarps, int tid, int nthreads,
                             int (*s_range)[32], int* s_window, float* s_tab, int window_bytes = kWindowBytes) {
  const int G = tb.G;
  int lo = 1 << 30, hi = -1;
  if (valid) {
    for (int dd = first_dir; dd < n; dd += dir_step) {
      int i0;
      float w;
      table_position(tb, ux * s_om[dd][0] + uy * s_om[dd][1] + uz * s_om[dd][2], i0, w);
      lo = min(lo, i0);
      hi = max(hi, i0);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, off));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, off));
  }
  if ((tid & 31) == 0) {
    s_range[0][warp] = lo;
    s_range[1][warp] = hi;
  }
  __syncthreads();
  if (tid == 0) {
    for (int q = 1; q < nwarps; ++q) {
      lo = min(lo, s_range[0][q]);
      hi = max(hi, s_range[1][q]);
    }
    const bool fits = hi >= lo && hi + 2 - lo <= window_nodes(tb.M, G, window_bytes);
    s_window[0] = fits ? lo : -1;
    s_window[1] = fits ? hi + 2 - lo : 0;
  }
  __syncthreads();
  const int win_lo = s_window[0], win_n = s_window[1];
  if (win_lo >= 0 && G % 4 == 0 && ((uintptr_t)tb.t % 16) == 0) {
    // whole (node, material) blocks of G x G floats as float4, one block per warp at a time: no index division per
    // element (the padded stride G G + 4 keeps every block 16-byte aligned)
    const int RS = window_row_stride(G), GG4 = G * G / 4;
    for (int nm = warp; nm < win_n * tb.M; nm += nwarps) {
      const int node = nm / tb.M, m = nm - node * tb.M;
      const float4* src = reinterpret_cast<const float4*>(tb.t + ((int64_t)m * tb.N + win_lo + node) * G * G);
      float4* dst = reinterpret_cast<float4*>(s_tab + (node * tb.M + m) * RS);
      for (int r = tid & 31; r < GG4; r += 32) dst[r] = __ldg(src + r);
    }
  } else if (win_lo >= 0) {
    const int RS = window_row_stride(G);
    const int per = tb.M * G * G;
    for (int q = tid; q < win_n * per; q += nthreads) {
      const int node = q / per, rem = q - node * per;
      const int m = rem / (G * G), r = rem - m * G * G;
      s_tab[(node * tb.M + m) * RS + r] = __ldg(tb.t + ((int64_t)m * tb.N + win_lo + node) * G * G + r);
    }
  }
  __syncthreads();
}

// S_FC of group g at one point for one direction, rows from the window (win_lo >= 0) or from global memory
// kWindow: 1 the rows are in the block's shared-memory window, 2 in global memory, 0 decided by win_lo >= 0
template <int kGP, int kMM, int kWindow = 0>
__device__ __forceinline__ float fc_group(const Table& tb, const float* s_tab, int win_lo, int i0, float w, int g,
                                          const float* rho, const float* phi) {
  const int G = tb.G, RS = window_row_stride(G);
  float src = 0.f;
#pragma unroll
  for (int m = 0; m < kMM; ++m) {
    const float r = rho[m];
    if (m >= tb.M || r == 0.f) continue;
    float a0, a1;
    if (kWindow == 1 || (kWindow == 0 && win_lo >= 0)) {
      const float* row0 = s_tab + ((i0 - win_lo) * tb.M + m) * RS + g * G;
      a0 = row_dot<kGP, true>(row0, phi, G);
      a1 = row_dot<kGP, true>(row0 + tb.M * RS, phi, G);
    } else {
      const float* row0 = tb.t + (((int64_t)m * tb.N + i0) * G + g) * G;
      a0 = row_dot<kGP, false>(row0, phi, G);
      a1 = row_dot<kGP, false>(row0 + (int64_t)G * G, phi, G);
    }
    src = fmaf(r, a0 + (a1 - a0) * w, src);
  }
  return src;
}

// window bytes of an emission block with kDirs directions (more directions span more table nodes)
__host__ __device__ constexpr int emission_window_bytes(int dirs) {
  return dirs > 32 ? 64 * 1024 : dirs > 16 ? 48 * 1024 : kWindowBytes;
}

template <int kGP, int kMM, bool kFused, int kDirs>
__global__ void __launch_bounds__(kEmitPoints * kGP) emission_kernel(
    FCInputs in, Table tb, PointGrid pg, const float* __restrict__ omegas, int K,
    const float* __restrict__ tau /*[K, NC, G], or [K, NC, TM] path lengths with tau_mu*/,
    const float* __restrict__ tau_mu /*[TM, G] or null*/, int TM, const float* __restrict__ mu /*[G, NC]*/,
    const float* __restrict__ multiple /*[K, NC, G], read when not fused*/,
    const float* __restrict__ harmonics /*[K, NS], fused*/, const float* __restrict__ moments /*[NS, NC, G], fused*/,
    int NS, const float* __restrict__ heights, const float* __restrict__ signal_weight /*[K, G] or null*/, float dx,
    float dy, float dz, float* __restrict__ out, float* __restrict__ partial /*[K, nblocks, 2]*/) {
  constexpr int kPW = 32 / kGP;                 // points per warp
  constexpr int kWarps = kEmitPoints / kPW;     // = kGP
  extern __shared__ float4 s_dyn4[];
  float* s_tab = reinterpret_cast<float*>(s_dyn4);  // the table window (dynamic, kWindowBytes)
  __shared__ float s_om[kDirs][3];
  __shared__ float s_sw[kDirs][kGP];          // signal weights of the block's directions
  __shared__ __align__(16) float s_y[kFused ? kDirs : 1][kFused ? kMaxMoments : 4];
  __shared__ float s_sum[kDirs][kWarps][2];   // per-direction, per-warp sums of e and e h
  __shared__ int s_range[2][32];
  __shared__ int s_window[2];
  const int G = tb.G;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const int g = lane % kGP, p = warp * kPW + lane / kGP;   // the thread's group and point of the block
  const bool gvalid = g < G;
  const int d0 = blockIdx.y * kDirs;
  const int nd = min(kDirs, K - d0);
  constexpr int nthreads = kEmitPoints * kGP;
  for (int i = tid; i < kDirs * 3; i += nthreads) s_om[i / 3][i % 3] = i < nd * 3 ? omegas[3 * d0 + i] : 0.f;
  if (signal_weight != nullptr)
    for (int i = tid; i < kDirs * kGP; i += nthreads) {
      const int dd = i / kGP, q = i % kGP;
      s_sw[dd][q] = (dd < nd && q < G) ? signal_weight[(int64_t)(d0 + dd) * G + q] : 0.f;
    }
  if (kFused)
    for (int i = tid; i < kDirs * NS; i += nthreads)
      s_y[i / NS][i % NS] = i < nd * NS ? harmonics[(int64_t)d0 * NS + i] : 0.f;

  const int64_t v = (int64_t)blockIdx.x * kEmitPoints + p;
  const bool valid = v < in.V;
  const int64_t NC = (int64_t)pg.Rc * pg.Cc * pg.Sc;
  float rho[kMM], phi[kGP];
  float ux = 0.f, uy = 0.f, uz = 0.f, h = 0.f, offx = 0.f, offy = 0.f, offz = 0.f, muc = 0.f;
  int64_t cell = 0;
#pragma unroll
  for (int q = 0; q < kGP; ++q) phi[q] = 0.f;
#pragma unroll
  for (int m = 0; m < kMM; ++m) rho[m] = 0.f;
  float tmom[kFused ? kRegMoments : 1];
  if (valid) {
    int i, j, k;
    point_rcs(v, pg, i, j, k);
    primary_direction(__ldg(in.ax_x + j), __ldg(in.ax_y + i), __ldg(in.ax_z + k), in.r0x, in.r0y, in.r0z, ux, uy, uz);
#pragma unroll
    for (int m = 0; m < kMM; ++m)
      if (m < tb.M) rho[m] = __ldg(in.rho + (int64_t)m * in.V + v);
#pragma unroll
    for (int q = 0; q < kGP; ++q)
      if (q < G) phi[q] = __ldg(in.phi + (int64_t)q * in.V + v);
    const int F = pg.f, ic = i / F, jc = j / F, kc = k / F;
    cell = ((int64_t)ic * pg.Cc + jc) * pg.Sc + kc;
    const float half = (F - 1) * 0.5f;
    offy = dy * ((float)(i - ic * F) - half);
    offx = dx * ((float)(j - jc * F) - half);
    offz = dz * ((float)(k - kc * F) - half);
    h = heights ? __ldg(heights + v) : 0.f;
    if (gvalid) muc = __ldg(mu + (int64_t)g * NC + cell);
  }
  float tmu[kMM];  // the group's attenuation per traced material, when tau holds material path lengths
#pragma unroll
  for (int m = 0; m < kMM; ++m) tmu[m] = (tau_mu != nullptr && m < TM && gvalid) ? __ldg(tau_mu + m * G + g) : 0.f;
  if (kFused) {
#pragma unroll
    for (int n = 0; n < (kFused ? kRegMoments : 1); ++n)
      tmom[n] = (valid && gvalid && n < NS) ? __ldg(moments + ((int64_t)n * NC + cell) * G + g) : 0.f;
  }
  __syncthreads();  // s_om and s_y are complete
  stage_window(tb, valid, ux, uy, uz, s_om, nd, g, kGP, warp, kWarps, tid, nthreads, s_range, s_window, s_tab,
               emission_window_bytes(kDirs));
  const int win_lo = s_window[0];

  // running pointers to this lane's element of direction d0 + dd (advanced once per direction)
  const float* mp = kFused ? nullptr : multiple + ((int64_t)d0 * NC + cell) * G + g;
  const float* tp = tau_mu != nullptr ? tau + ((int64_t)d0 * NC + cell) * TM : tau + ((int64_t)d0 * NC + cell) * G + g;
  const int64_t mp_step = NC * G, tp_step = tau_mu != nullptr ? NC * TM : NC * G;
  float* op = signal_weight != nullptr ? out + (int64_t)d0 * in.V + v : out + ((int64_t)d0 * in.V + v) * G + g;
  const int64_t op_step = signal_weight != nullptr ? in.V : in.V * G;
  // the table window (or, where a block's nodes do not fit it, the table in global memory) is fixed for the block:
  // the direction loop is compiled for each case, with no test of it per direction
  auto directions = [&](auto windowed) {
    constexpr bool kWin = decltype(windowed)::value;
    for (int dd = 0; dd < nd; ++dd) {
      float e = 0.f;
      if (valid && gvalid) {
        const float ox = s_om[dd][0], oy = s_om[dd][1], oz = s_om[dd][2];
        const float cosine = ux * ox + uy * oy + uz * oz;
        int i0;
        float w;
        table_position(tb, cosine, i0, w);
        const float offset = pg.f > 1 ? oy * offy + ox * offx + oz * offz : 0.f;  // one point per cell: its centre
        const float src = fc_group<kGP, kMM, kWin ? 1 : 2>(tb, s_tab, win_lo, i0, w, g, rho, phi);
        float smc = 0.f;
        if (kFused) {
#pragma unroll
          for (int n = 0; n < (kFused ? kRegMoments : 1); n += 4) {
            const float4 y = *reinterpret_cast<const float4*>(&s_y[kFused ? dd : 0][n]);
            smc = fmaf(y.x, tmom[n], smc);
            if (n + 1 < kRegMoments) smc = fmaf(y.y, tmom[n + 1], smc);
            if (n + 2 < kRegMoments) smc = fmaf(y.z, tmom[n + 2], smc);
            if (n + 3 < kRegMoments) smc = fmaf(y.w, tmom[n + 3], smc);
          }
          for (int n = kRegMoments; n < NS; ++n)
            smc = fmaf(s_y[kFused ? dd : 0][n], __ldg(moments + ((int64_t)n * NC + cell) * G + g), smc);
        } else {
          smc = __ldg(mp);
        }
        float t;
        if (tau_mu != nullptr) {  // sum_m mu[m, g] P_m, in material order
          t = 0.f;
#pragma unroll
          for (int m = 0; m < kMM; ++m)
            if (m < TM) t = fmaf(tmu[m], __ldg(tp + m), t);
        } else {
          t = __ldg(tp);
        }
        const float depth = pg.f > 1 ? fmaxf(t - muc * offset, 0.f) : fmaxf(t, 0.f);
        e = (src + smc) * __expf(-depth);  // the fast exponential: within a few ulp for these depths
      }
      // group sums over the kGP lanes of the point (in group order), then the warp's points
      float tot = e, sgl = signal_weight != nullptr ? s_sw[dd][g] * e : 0.f;
#pragma unroll
      for (int off = 1; off < kGP; off <<= 1) {
        tot += __shfl_xor_sync(0xffffffffu, tot, off);
        sgl += __shfl_xor_sync(0xffffffffu, sgl, off);
      }
      if (signal_weight != nullptr) {
        if (g == 0 && valid) *op = sgl;
      } else if (valid && gvalid) {
        *op = e;
      }
      float a = (g == 0) ? tot : 0.f, b = (g == 0) ? tot * h : 0.f;
#pragma unroll
      for (int off = kGP; off < 32; off <<= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
      }
      if (lane == 0) {
        s_sum[dd][warp][0] = a;
        s_sum[dd][warp][1] = b;
      }
      if (!kFused) mp += mp_step;
      tp += tp_step;
      op += op_step;
    }
  };
  if (win_lo >= 0) directions(std::true_type{});
  else directions(std::false_type{});
  __syncthreads();
  if (tid < 2 * nd) {
    const int dd = tid / 2, which = tid % 2;
    float acc = 0.f;
    for (int q = 0; q < kWarps; ++q) acc += s_sum[dd][q][which];
    partial[((int64_t)(d0 + dd) * gridDim.x + blockIdx.x) * 2 + which] = acc;
  }
}

// ---- attenuated emission, one thread per (point, direction) with all of its groups ---------------------------------
// A block is 32 points (the lanes, consecutive points and, for one point per cell, consecutive cells) by kEmitWarps
// warps; warp w takes the block's directions w, w + kEmitWarps, ... . The cosine, the table position, the traced path
// lengths, the signal sum and the write happen once per (point, direction), where the group lanes of emission_kernel
// repeat them G times; the multiple-collision source (and per-group optical depths) of a cell are G contiguous floats,
// read as float4 and coalesced over the warp. Only the transfer entries of incoming groups at or above the outgoing
// one enter the sum (the reference's first-collision table is downscatter only, uncollided_kernels.py:488-550).
// Every group value, the group sums and the per-block partial sums are formed in emission_kernel's order (its
// sequential incoming-group sums, its xor-butterfly group sums, its warp-then-block point sums), so the two kernels
// give the same bits on a table without upscatter entries.
constexpr int kEmitWarps = 8;

// x[0] + ... + x[n-1] in the order of an xor butterfly over n lanes read at lane 0: pairwise halves, each addition
// rounded on its own (a butterfly's shuffles keep a product from fusing into the next addition; here __fadd_rn does)
template <int n>
__device__ __forceinline__ float tree_sum(const float* x) {
  if constexpr (n == 1) {
    return x[0];
  } else {
    return __fadd_rn(tree_sum<n / 2>(x), tree_sum<n / 2>(x + n / 2));
  }
}

// sum_{gi <= g} row[gi] phi[gi], in incoming-group order; the row in shared or global memory, float4 reads when the
// rows are 16-byte aligned (kVec)
template <int kGP, bool kVec, bool kShared>
__device__ __forceinline__ float dot_lower(const float* __restrict__ row, const float* phi, int g) {
  float a = 0.f;
  if constexpr (kVec) {
#pragma unroll
    for (int q = 0; q < kGP / 4; ++q) {
      if (4 * q > g) break;
      const float4 t = kShared ? reinterpret_cast<const float4*>(row)[q]
                               : __ldg(reinterpret_cast<const float4*>(row) + q);
      a = fmaf(t.x, phi[4 * q], a);
      if (4 * q + 1 <= g) a = fmaf(t.y, phi[4 * q + 1], a);
      if (4 * q + 2 <= g) a = fmaf(t.z, phi[4 * q + 2], a);
      if (4 * q + 3 <= g) a = fmaf(t.w, phi[4 * q + 3], a);
    }
  } else {
#pragma unroll
    for (int gi = 0; gi < kGP; ++gi) {
      if (gi > g) break;
      a = fmaf(kShared ? row[gi] : __ldg(row + gi), phi[gi], a);
    }
  }
  return a;
}

template <int kGP, bool kVec>
__device__ __forceinline__ void load_groups(const float* __restrict__ p, int G, float* x) {
  if constexpr (kVec) {
#pragma unroll
    for (int q = 0; q < kGP / 4; ++q) {
      if (4 * q < G) {
        const float4 t = __ldg(reinterpret_cast<const float4*>(p) + q);
        x[4 * q] = t.x;
        x[4 * q + 1] = t.y;
        x[4 * q + 2] = t.z;
        x[4 * q + 3] = t.w;
      } else {
        x[4 * q] = x[4 * q + 1] = x[4 * q + 2] = x[4 * q + 3] = 0.f;
      }
    }
  } else {
#pragma unroll
    for (int q = 0; q < kGP; ++q) x[q] = q < G ? __ldg(p + q) : 0.f;
  }
}

// kQ1: one point per cell (the point is the cell's centre: no in-cell offsets, no cell attenuation needed). A warp's
// loads of its next direction's multiple-collision source and path lengths are issued before the table sums of the
// current one, so their latency hides behind that arithmetic; 3 blocks of 256 threads per SM (80 registers, the
// 64 KB table window).
template <int kGP, int kMM, int kDirs, bool kVec, bool kQ1>
__global__ void __launch_bounds__(32 * kEmitWarps, 3) emission_warps_kernel(
    FCInputs in, Table tb, PointGrid pg, const float* __restrict__ omegas, int K,
    const float* __restrict__ tau /*[K, NC, G], or [K, NC, TM] path lengths with tau_mu*/,
    const float* __restrict__ tau_mu /*[TM, G] or null*/, int TM, const float* __restrict__ mu /*[G, NC]*/,
    const float* __restrict__ multiple /*[K, NC, G]*/, const float* __restrict__ heights,
    const float* __restrict__ signal_weight /*[K, G] or null*/, float dx, float dy, float dz,
    float* __restrict__ out, float* __restrict__ partial /*[K, nblocks, 2]*/) {
  constexpr int kPW = 32 / kGP;  // points per warp of emission_kernel, whose partial-sum order is kept
  constexpr int nthreads = 32 * kEmitWarps;
  extern __shared__ float4 s_dyn4[];
  float* s_tab = reinterpret_cast<float*>(s_dyn4);
  __shared__ float s_om[kDirs][3];
  __shared__ float s_sw[kDirs][kGP];
  __shared__ float s_tmu[kMM][kGP];
  __shared__ int s_range[2][32];
  __shared__ int s_window[2];
  const int G = tb.G;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int d0 = blockIdx.y * kDirs;
  const int nd = min(kDirs, K - d0);
  for (int i = tid; i < kDirs * 3; i += nthreads) s_om[i / 3][i % 3] = i < nd * 3 ? omegas[3 * d0 + i] : 0.f;
  if (signal_weight != nullptr)
    for (int i = tid; i < kDirs * kGP; i += nthreads) {
      const int dd = i / kGP, q = i % kGP;
      s_sw[dd][q] = (dd < nd && q < G) ? signal_weight[(int64_t)(d0 + dd) * G + q] : 0.f;
    }
  for (int i = tid; i < kMM * kGP; i += nthreads) {
    const int m = i / kGP, q = i % kGP;
    s_tmu[m][q] = (tau_mu != nullptr && m < TM && q < G) ? tau_mu[m * G + q] : 0.f;
  }

  const int64_t v = (int64_t)blockIdx.x * 32 + lane;
  const bool valid = v < in.V;
  const int64_t NC = (int64_t)pg.Rc * pg.Cc * pg.Sc;
  float rho[kMM], phi[kGP], muc[kGP];
  float ux = 0.f, uy = 0.f, uz = 0.f, h = 0.f, offx = 0.f, offy = 0.f, offz = 0.f;
  int64_t cell = 0;
#pragma unroll
  for (int q = 0; q < kGP; ++q) phi[q] = muc[q] = 0.f;
#pragma unroll
  for (int m = 0; m < kMM; ++m) rho[m] = 0.f;
  if (valid) {
    int i, j, k;
    point_rcs(v, pg, i, j, k);
    primary_direction(__ldg(in.ax_x + j), __ldg(in.ax_y + i), __ldg(in.ax_z + k), in.r0x, in.r0y, in.r0z, ux, uy, uz);
#pragma unroll
    for (int m = 0; m < kMM; ++m)
      if (m < tb.M) rho[m] = __ldg(in.rho + (int64_t)m * in.V + v);
#pragma unroll
    for (int q = 0; q < kGP; ++q)
      if (q < G) phi[q] = __ldg(in.phi + (int64_t)q * in.V + v);
    const int F = pg.f, ic = i / F, jc = j / F, kc = k / F;
    cell = ((int64_t)ic * pg.Cc + jc) * pg.Sc + kc;
    const float half = (F - 1) * 0.5f;
    offy = dy * ((float)(i - ic * F) - half);
    offx = dx * ((float)(j - jc * F) - half);
    offz = dz * ((float)(k - kc * F) - half);
    h = heights ? __ldg(heights + v) : 0.f;
    if (!kQ1) {
#pragma unroll
      for (int q = 0; q < kGP; ++q)
        if (q < G) muc[q] = __ldg(mu + (int64_t)q * NC + cell);
    }
  }
  __syncthreads();  // s_om, s_sw and s_tmu are complete
  stage_window(tb, valid, ux, uy, uz, s_om, nd, warp, kEmitWarps, warp, kEmitWarps, tid, nthreads, s_range, s_window,
               s_tab, emission_window_bytes(kDirs));
  const int win_lo = s_window[0];
  const int RS = window_row_stride(G);

  auto directions = [&](auto windowed) {
    constexpr bool kWin = decltype(windowed)::value;
    float smc_n[kGP], P_n[kMM];
    auto fetch = [&](int dd) {
      if (valid && dd < nd) {
        const int64_t dc = (d0 + dd) * NC + cell;
        load_groups<kGP, kVec>(multiple + dc * G, G, smc_n);
        if (tau_mu != nullptr) {
#pragma unroll
          for (int m = 0; m < kMM; ++m) P_n[m] = m < TM ? __ldg(tau + dc * TM + m) : 0.f;
        }
      }
    };
    fetch(warp);
    for (int dd = warp; dd < nd; dd += kEmitWarps) {
      const int64_t d = d0 + dd;
      float e[kGP];
#pragma unroll
      for (int q = 0; q < kGP; ++q) e[q] = 0.f;
      float smc[kGP], P[kMM];
#pragma unroll
      for (int q = 0; q < kGP; ++q) smc[q] = smc_n[q];
#pragma unroll
      for (int m = 0; m < kMM; ++m) P[m] = P_n[m];
      fetch(dd + kEmitWarps);  // the next direction's loads in flight during this one's table sums
      if (valid) {
        const int64_t dc = d * NC + cell;
        float t[kGP];
        if (tau_mu != nullptr) {  // sum_m mu[m, g] P_m, in material order
#pragma unroll
          for (int q = 0; q < kGP; ++q) t[q] = 0.f;
#pragma unroll
          for (int m = 0; m < kMM; ++m)
            if (m < TM) {
#pragma unroll
              for (int q = 0; q < kGP; ++q) t[q] = fmaf(s_tmu[m][q], P[m], t[q]);
            }
        } else {
          load_groups<kGP, kVec>(tau + dc * G, G, t);
        }
        const float ox = s_om[dd][0], oy = s_om[dd][1], oz = s_om[dd][2];
        const float cosine = ux * ox + uy * oy + uz * oz;
        int i0;
        float w;
        table_position(tb, cosine, i0, w);
        const float offset = kQ1 ? 0.f : oy * offy + ox * offx + oz * offz;
        float src[kGP];
#pragma unroll
        for (int q = 0; q < kGP; ++q) src[q] = 0.f;
#pragma unroll
        for (int m = 0; m < kMM; ++m) {
          const float r = rho[m];
          if (m >= tb.M || r == 0.f) continue;
          const float* row0 = kWin ? s_tab + ((i0 - win_lo) * tb.M + m) * RS
                                   : tb.t + ((int64_t)m * tb.N + i0) * G * G;
          const float* row1 = row0 + (kWin ? tb.M * RS : G * G);
#pragma unroll
          for (int g = 0; g < kGP; ++g) {
            if (g >= G) break;
            const float a0 = dot_lower<kGP, kVec, kWin>(row0 + g * G, phi, g);
            const float a1 = dot_lower<kGP, kVec, kWin>(row1 + g * G, phi, g);
            src[g] = fmaf(r, a0 + (a1 - a0) * w, src[g]);
          }
        }
#pragma unroll
        for (int g = 0; g < kGP; ++g) {
          if (g >= G) break;
          const float depth = kQ1 ? fmaxf(t[g], 0.f) : fmaxf(t[g] - muc[g] * offset, 0.f);
          e[g] = (src[g] + smc[g]) * __expf(-depth);  // the fast exponential: within a few ulp for these depths
        }
      }
      const float tot = tree_sum<kGP>(e);
      if (signal_weight != nullptr) {
        float sg[kGP];
#pragma unroll
        for (int q = 0; q < kGP; ++q) sg[q] = __fmul_rn(s_sw[dd][q], e[q]);
        if (valid) out[d * in.V + v] = tree_sum<kGP>(sg);
      } else if (valid) {
        float* o = out + (d * in.V + v) * G;
        if (kVec) {
#pragma unroll
          for (int q = 0; q < kGP / 4; ++q)
            if (4 * q < G) reinterpret_cast<float4*>(o)[q] = make_float4(e[4 * q], e[4 * q + 1], e[4 * q + 2], e[4 * q + 3]);
        } else {
#pragma unroll
          for (int q = 0; q < kGP; ++q)
            if (q < G) o[q] = e[q];
        }
      }
      // emission_kernel's order: a butterfly over its kPW points per warp, then its warps in sequence
      float a = tot, b = __fmul_rn(tot, h);
#pragma unroll
      for (int off = 1; off < kPW; off <<= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
      }
      float sa = 0.f, sb = 0.f;
#pragma unroll
      for (int q = 0; q < kGP; ++q) {
        sa += __shfl_sync(0xffffffffu, a, q * kPW);
        sb += __shfl_sync(0xffffffffu, b, q * kPW);
      }
      if (lane == 0) {
        partial[(d * gridDim.x + blockIdx.x) * 2] = sa;
        partial[(d * gridDim.x + blockIdx.x) * 2 + 1] = sb;
      }
    }
  };
  if (win_lo >= 0) directions(std::true_type{});
  else directions(std::false_type{});
}

// ---- sampling correction over the sweep directions, with the source values kept -----------------------------------
// A block is 32 points by the G groups and walks all K sweep directions, in the order of their cosine with the
// block's first point so that each batch of kFcBatch directions touches few table nodes (the window); it sums
// I0, I1, I2 per (point, group), stores S_FC(direction, group, point) in cache [K, G, V] when given (the LD moments
// of the sweep's source read it back instead of evaluating the table again), and forms E0, E1 and the float64
// factors as the reference does.
constexpr int kFcBatch = 16;
constexpr int kMaxSorted = 1024;

template <int kGP, int kMM>
__global__ void __launch_bounds__(kEmitPoints * kGP) fc_correction_kernel(
    FCInputs in, Table tb, PointGrid pg, const float* __restrict__ omegas, const float* __restrict__ weights, int K,
    const float* __restrict__ moments /*[M, 2, G, G]*/, float* __restrict__ sums /*[5, G, V] or null*/,
    float* __restrict__ scale, float* __restrict__ beta, float* __restrict__ cache /*[K, G, V] or null*/) {
  extern __shared__ float4 s_dyn4[];
  float* s_tab = reinterpret_cast<float*>(s_dyn4);
  __shared__ float s_key[kMaxSorted];
  __shared__ int s_order[kMaxSorted];
  __shared__ float s_om[kFcBatch][3];
  __shared__ float s_w[kFcBatch];
  __shared__ int s_d[kFcBatch];
  __shared__ int s_range[2][32];
  __shared__ int s_window[2];
  __shared__ float s_u0[3];
  const int G = tb.G;
  const int g = threadIdx.y, lane = threadIdx.x;
  const int nthreads = kEmitPoints * G, tid = g * kEmitPoints + lane;
  const int64_t v = (int64_t)blockIdx.x * kEmitPoints + lane;
  const bool valid = v < in.V;
  float rho[kMM], phi[kGP];
  float ux = 0.f, uy = 0.f, uz = 0.f;
#pragma unroll
  for (int q = 0; q < kGP; ++q) phi[q] = 0.f;
#pragma unroll
  for (int m = 0; m < kMM; ++m) rho[m] = 0.f;
  if (valid) {
    int i, j, k;
    point_rcs(v, pg, i, j, k);
    primary_direction(__ldg(in.ax_x + j), __ldg(in.ax_y + i), __ldg(in.ax_z + k), in.r0x, in.r0y, in.r0z, ux, uy, uz);
#pragma unroll
    for (int m = 0; m < kMM; ++m)
      if (m < tb.M) rho[m] = __ldg(in.rho + (int64_t)m * in.V + v);
#pragma unroll
    for (int q = 0; q < kGP; ++q)
      if (q < G) phi[q] = __ldg(in.phi + (int64_t)q * in.V + v);
  }
  // exact l = 0, 1 moments of the source (downscatter rows of the moment table)
  float E0 = 0.f, E1 = 0.f;
  for (int m = 0; m < tb.M; ++m) {
    const float* r0 = moments + (((int64_t)m * 2 + 0) * G + g) * G;
    const float* r1 = moments + (((int64_t)m * 2 + 1) * G + g) * G;
    float a0 = 0.f, a1 = 0.f;
    for (int gi = 0; gi <= g; ++gi) {
      a0 = fmaf(__ldg(r0 + gi), phi[gi < kGP ? gi : 0], a0);
      a1 = fmaf(__ldg(r1 + gi), phi[gi < kGP ? gi : 0], a1);
    }
    E0 = fmaf(rho[m], a0, E0);
    E1 = fmaf(rho[m], a1, E1);
  }
  // directions in the order of their cosine with the block's first point
  if (tid == 0) {
    s_u0[0] = ux;
    s_u0[1] = uy;
    s_u0[2] = uz;
  }
  __syncthreads();
  const bool sorted = K <= kMaxSorted;
  if (sorted) {
    for (int d = tid; d < K; d += nthreads)
      s_key[d] = s_u0[0] * __ldg(omegas + 3 * d) + s_u0[1] * __ldg(omegas + 3 * d + 1) +
                 s_u0[2] * __ldg(omegas + 3 * d + 2);
    __syncthreads();
    for (int d = tid; d < K; d += nthreads) {
      const float key = s_key[d];
      int rank = 0;
      for (int q = 0; q < K; ++q) {
        const float other = s_key[q];
        rank += (other < key) || (other == key && q < d);
      }
      s_order[rank] = d;
    }
    __syncthreads();
  }
  float I0 = 0.f, I1 = 0.f, I2 = 0.f;
  for (int b0 = 0; b0 < K; b0 += kFcBatch) {
    const int nb = min(kFcBatch, K - b0);
    if (tid < nb) {
      const int d = sorted ? s_order[b0 + tid] : b0 + tid;
      s_d[tid] = d;
      s_om[tid][0] = __ldg(omegas + 3 * d);
      s_om[tid][1] = __ldg(omegas + 3 * d + 1);
      s_om[tid][2] = __ldg(omegas + 3 * d + 2);
      s_w[tid] = __ldg(weights + d);
    }
    __syncthreads();
    stage_window(tb, valid, ux, uy, uz, s_om, nb, g, G, g, G, tid, nthreads, s_range, s_window, s_tab);
    const int win_lo = s_window[0];
    if (valid) {
      for (int i = 0; i < nb; ++i) {
        const float cosine = ux * s_om[i][0] + uy * s_om[i][1] + uz * s_om[i][2];
        int i0;
        float w;
        table_position(tb, cosine, i0, w);
        const float S = fc_group<kGP, kMM>(tb, s_tab, win_lo, i0, w, g, rho, phi);
        const float ws = S * s_w[i];
        I0 += ws;
        I1 += ws * cosine;
        I2 += ws * (cosine * cosine);
        if (cache != nullptr) cache[((int64_t)s_d[i] * G + g) * in.V + v] = S;
      }
    }
    __syncthreads();  // the batch's directions and window are replaced next
  }
  if (!valid) return;
  const int64_t gv = (int64_t)g * in.V + v;
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

// ---- sampling correction, one thread per (point, direction) with all of its groups --------------------------------
// The correction of fc_correction_kernel with the emission's thread layout: a block is 32 points (the lanes) by
// kFcWarps warps; per batch of kFcDirBatch directions (in the order of their cosine with the block's first point, so
// that a batch touches few table nodes) warp w takes the batch's directions w, w + kFcWarps, ... . A thread forms the
// cosine and the table position of its (point, direction) once and the source of every group from float4 rows
// (incoming groups at or above the outgoing one), adds the weighted source to its own partial sums I0, I1, I2 and
// writes the source values to the cache; the warps' partial sums are then added in warp order, and the float64
// factors formed as fc_correction_kernel forms them. The sums differ from fc_correction_kernel's at rounding level
// (another order of the same terms).
// 3 blocks of 256 threads per SM (80 registers): at 2 (128 registers) the table gathers' latency went unhidden
constexpr int kFcWarps = 8;
constexpr int kFcDirBatch = 32;

template <int kGP, int kMM, bool kVec>
__global__ void __launch_bounds__(32 * kFcWarps, 3) fc_correction_warps_kernel(
    FCInputs in, Table tb, PointGrid pg, const float* __restrict__ omegas, const float* __restrict__ weights, int K,
    const float* __restrict__ moments /*[M, 2, G, G]*/, float* __restrict__ sums /*[5, G, V] or null*/,
    float* __restrict__ scale, float* __restrict__ beta, float* __restrict__ cache /*[K, G, V] or null*/) {
  constexpr int nthreads = 32 * kFcWarps;
  extern __shared__ float4 s_dyn4[];
  float* s_tab = reinterpret_cast<float*>(s_dyn4);
  __shared__ float s_key[kMaxSorted];
  __shared__ int s_order[kMaxSorted];
  __shared__ float s_om[kFcDirBatch][3];
  __shared__ float s_w[kFcDirBatch];
  __shared__ int s_d[kFcDirBatch];
  __shared__ int s_range[2][32];
  __shared__ int s_window[2];
  __shared__ float s_u0[3];
  // after the direction loop the window's shared memory holds the warps' partial sums [kFcWarps][3][kGP][32]
  static_assert(kFcWarps * 3 * kGP * 32 * 4 <= emission_window_bytes(kFcDirBatch), "partial sums exceed the window");
  const int G = tb.G;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t v = (int64_t)blockIdx.x * 32 + lane;
  const bool valid = v < in.V;
  float rho[kMM], phi[kGP];
  float ux = 0.f, uy = 0.f, uz = 0.f;
#pragma unroll
  for (int q = 0; q < kGP; ++q) phi[q] = 0.f;
#pragma unroll
  for (int m = 0; m < kMM; ++m) rho[m] = 0.f;
  if (valid) {
    int i, j, k;
    point_rcs(v, pg, i, j, k);
    primary_direction(__ldg(in.ax_x + j), __ldg(in.ax_y + i), __ldg(in.ax_z + k), in.r0x, in.r0y, in.r0z, ux, uy, uz);
#pragma unroll
    for (int m = 0; m < kMM; ++m)
      if (m < tb.M) rho[m] = __ldg(in.rho + (int64_t)m * in.V + v);
#pragma unroll
    for (int q = 0; q < kGP; ++q)
      if (q < G) phi[q] = __ldg(in.phi + (int64_t)q * in.V + v);
  }
  if (tid == 0) {
    s_u0[0] = ux;
    s_u0[1] = uy;
    s_u0[2] = uz;
  }
  __syncthreads();
  const bool sorted = K <= kMaxSorted;
  if (sorted) {
    for (int d = tid; d < K; d += nthreads)
      s_key[d] = s_u0[0] * __ldg(omegas + 3 * d) + s_u0[1] * __ldg(omegas + 3 * d + 1) +
                 s_u0[2] * __ldg(omegas + 3 * d + 2);
    __syncthreads();
    for (int d = tid; d < K; d += nthreads) {
      const float key = s_key[d];
      int rank = 0;
      for (int q = 0; q < K; ++q) {
        const float other = s_key[q];
        rank += (other < key) || (other == key && q < d);
      }
      s_order[rank] = d;
    }
    __syncthreads();
  }
  float I0[kGP], I1[kGP], I2[kGP];
#pragma unroll
  for (int q = 0; q < kGP; ++q) I0[q] = I1[q] = I2[q] = 0.f;
  const int RS = window_row_stride(G);
  for (int b0 = 0; b0 < K; b0 += kFcDirBatch) {
    const int nb = min(kFcDirBatch, K - b0);
    if (tid < nb) {
      const int d = sorted ? s_order[b0 + tid] : b0 + tid;
      s_d[tid] = d;
      s_om[tid][0] = __ldg(omegas + 3 * d);
      s_om[tid][1] = __ldg(omegas + 3 * d + 1);
      s_om[tid][2] = __ldg(omegas + 3 * d + 2);
      s_w[tid] = __ldg(weights + d);
    }
    __syncthreads();
    stage_window(tb, valid, ux, uy, uz, s_om, nb, warp, kFcWarps, warp, kFcWarps, tid, nthreads, s_range, s_window,
                 s_tab, emission_window_bytes(kFcDirBatch));
    const int win_lo = s_window[0];
    if (valid) {
      for (int i = warp; i < nb; i += kFcWarps) {
        const float cosine = ux * s_om[i][0] + uy * s_om[i][1] + uz * s_om[i][2];
        int i0;
        float w;
        table_position(tb, cosine, i0, w);
        float S[kGP];
#pragma unroll
        for (int q = 0; q < kGP; ++q) S[q] = 0.f;
        const bool win = win_lo >= 0;
#pragma unroll
        for (int m = 0; m < kMM; ++m) {
          const float r = rho[m];
          if (m >= tb.M || r == 0.f) continue;
          const float* row0 = win ? s_tab + ((i0 - win_lo) * tb.M + m) * RS : tb.t + ((int64_t)m * tb.N + i0) * G * G;
          const float* row1 = row0 + (win ? tb.M * RS : G * G);
#pragma unroll
          for (int g = 0; g < kGP; ++g) {
            if (g >= G) break;
            float a0, a1;
            if (win) {
              a0 = dot_lower<kGP, kVec, true>(row0 + g * G, phi, g);
              a1 = dot_lower<kGP, kVec, true>(row1 + g * G, phi, g);
            } else {
              a0 = dot_lower<kGP, kVec, false>(row0 + g * G, phi, g);
              a1 = dot_lower<kGP, kVec, false>(row1 + g * G, phi, g);
            }
            S[g] = fmaf(r, a0 + (a1 - a0) * w, S[g]);
          }
        }
        const float wt = s_w[i], c2 = cosine * cosine;
        const int64_t d = s_d[i];
#pragma unroll
        for (int g = 0; g < kGP; ++g) {
          if (g >= G) break;
          const float ws = S[g] * wt;
          I0[g] += ws;
          I1[g] += ws * cosine;
          I2[g] += ws * c2;
          if (cache != nullptr) cache[(d * G + g) * in.V + v] = S[g];
        }
      }
    }
    __syncthreads();  // the batch's directions and window are replaced next
  }
  float* s_part = s_tab;  // free: the last batch's barrier above ended every read of the window
#pragma unroll
  for (int q = 0; q < kGP; ++q) {
    s_part[((warp * 3 + 0) * kGP + q) * 32 + lane] = I0[q];
    s_part[((warp * 3 + 1) * kGP + q) * 32 + lane] = I1[q];
    s_part[((warp * 3 + 2) * kGP + q) * 32 + lane] = I2[q];
  }
  __syncthreads();
  // warp g forms the factors of group g of its lane's point (every warp holds the point's densities and fluence)
  for (int g = warp; g < G && g < kGP; g += kFcWarps) {
    if (!valid) break;
    float i0s = 0.f, i1s = 0.f, i2s = 0.f;
#pragma unroll
    for (int q = 0; q < kFcWarps; ++q) {
      i0s += s_part[((q * 3 + 0) * kGP + g) * 32 + lane];
      i1s += s_part[((q * 3 + 1) * kGP + g) * 32 + lane];
      i2s += s_part[((q * 3 + 2) * kGP + g) * 32 + lane];
    }
    // exact l = 0, 1 moments of the source (downscatter rows of the moment table)
    float E0 = 0.f, E1 = 0.f;
    for (int m = 0; m < tb.M && m < kMM; ++m) {
      const float* r0 = moments + (((int64_t)m * 2 + 0) * G + g) * G;
      const float* r1 = moments + (((int64_t)m * 2 + 1) * G + g) * G;
      float a0 = 0.f, a1 = 0.f;
      for (int gi = 0; gi <= g; ++gi) {
        a0 = fmaf(__ldg(r0 + gi), phi[gi], a0);
        a1 = fmaf(__ldg(r1 + gi), phi[gi], a1);
      }
      E0 = fmaf(rho[m], a0, E0);
      E1 = fmaf(rho[m], a1, E1);
    }
    const int64_t gv = (int64_t)g * in.V + v;
    if (sums) {
      const int64_t GV = (int64_t)G * in.V;
      sums[gv] = i0s;
      sums[GV + gv] = i1s;
      sums[2 * GV + gv] = i2s;
      sums[3 * GV + gv] = E0;
      sums[4 * GV + gv] = E1;
    }
    // factors in float64 (uncollided.py:611-636)
    const double i0d = i0s, i1d = i1s, i2d = i2s, e0 = E0, e1 = E1;
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
}

// ---- LD moments of the corrected source from the kept source values ---------------------------------------------
// A block is 32 cells by the G groups by kFcBatch directions of the chunk: S_FC read from cache [K, G, V] at the
// chunk direction's cache_index, corrected (scale (1 + beta cos)) and restricted to the cell's LD moments; the
// block's [cells, G, 4] tile goes out through shared memory as contiguous float4 rows.
template <int kGP>
__global__ void __launch_bounds__(kEmitPoints * kGP) fc_moments_cached_kernel(
    FCInputs in, PointGrid pg, const float* __restrict__ omegas, int K, const float* __restrict__ cache,
    const int32_t* __restrict__ cache_index, const float* __restrict__ scale, const float* __restrict__ beta,
    float slope_scale, float* __restrict__ out, int64_t out_k_stride) {
  // thread (cell, group) with the group fastest: a warp's float4 outputs [cell, group, 4] are contiguous
  const int G = (int)(blockDim.y);
  const int tid = threadIdx.y * kEmitPoints + threadIdx.x;
  const int lane = tid / G, g = tid - lane * G;
  const int64_t NC = (int64_t)pg.Rc * pg.Cc * pg.Sc;
  const int64_t c0 = (int64_t)blockIdx.x * kEmitPoints;
  const int64_t c = c0 + lane;
  const bool valid = c < NC;
  const int F = pg.f;
  int ic = 0, jc = 0, kc = 0;
  if (valid) {
    const int64_t csc = (int64_t)pg.Cc * pg.Sc;
    ic = (int)(c / csc);
    jc = (int)((c - (int64_t)ic * csc) / pg.Sc);
    kc = (int)(c - (int64_t)ic * csc - (int64_t)jc * pg.Sc);
  }
  const float inv = 1.f / (float)(F * F * F);
  const int dlast = min(K, (int)(blockIdx.y + 1) * kFcBatch);
  // one point per cell (the common case): its primary direction and correction factors once for all directions
  float u1x = 0.f, u1y = 0.f, u1z = 0.f, sc1 = 0.f, be1 = 0.f;
  int64_t v1 = 0;
  if (F == 1 && valid) {
    v1 = ((int64_t)ic * pg.C + jc) * pg.S + kc;
    primary_direction(__ldg(in.ax_x + jc), __ldg(in.ax_y + ic), __ldg(in.ax_z + kc), in.r0x, in.r0y, in.r0z, u1x,
                      u1y, u1z);
    sc1 = __ldg(scale + (int64_t)g * in.V + v1);
    be1 = __ldg(beta + (int64_t)g * in.V + v1);
  }
  for (int d = blockIdx.y * kFcBatch; d < dlast; ++d) {
    if (!valid) break;
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    const float ox = __ldg(omegas + 3 * d), oy = __ldg(omegas + 3 * d + 1), oz = __ldg(omegas + 3 * d + 2);
    const float* src = cache + (int64_t)__ldg(cache_index + d) * G * in.V + (int64_t)g * in.V;
    if (F == 1) {
      const float cosine = u1x * ox + u1y * oy + u1z * oz;
      r.x = __ldg(src + v1) * sc1 * (1.f + be1 * cosine) * inv;
    } else {
      float m0 = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
      for (int a = 0; a < F; ++a) {      // rows (y)
        for (int b = 0; b < F; ++b) {    // cols (x)
          for (int e = 0; e < F; ++e) {  // slices (z)
            const int i = ic * F + a, j = jc * F + b, k = kc * F + e;
            const int64_t v = ((int64_t)i * pg.C + j) * pg.S + k;
            float ux, uy, uz;
            primary_direction(__ldg(in.ax_x + j), __ldg(in.ax_y + i), __ldg(in.ax_z + k), in.r0x, in.r0y, in.r0z,
                              ux, uy, uz);
            const float cosine = ux * ox + uy * oy + uz * oz;
            const int64_t gv = (int64_t)g * in.V + v;
            const float s = __ldg(src + v) * __ldg(scale + gv) * (1.f + __ldg(beta + gv) * cosine);
            m0 += s;
            mx += s * ((2.f * b + 1.f) / F - 1.f);
            my += s * ((2.f * a + 1.f) / F - 1.f);
            mz += s * ((2.f * e + 1.f) / F - 1.f);
          }
        }
      }
      r.x = m0 * inv;
      r.y = mx * (inv * slope_scale);
      r.z = my * (inv * slope_scale);
      r.w = mz * (inv * slope_scale);
    }
    reinterpret_cast<float4*>(out + d * out_k_stride)[c * G + g] = r;
  }
}

// The means alone, for one point per cell (whose LD slopes vanish): out [K, NC, G] with out_k_stride floats between
// directions. A block is 32 cells by the G groups and 16 directions: it reads the cached source rows [g][cells] whole
// (a warp per group) and writes each direction's [cells, G] run whole, through shared memory.
template <int kGP>
__global__ void __launch_bounds__(kEmitPoints * kGP) fc_means_kernel(
    FCInputs in, PointGrid pg, const float* __restrict__ omegas, int K, const float* __restrict__ cache,
    const int32_t* __restrict__ cache_index, const float* __restrict__ scale, const float* __restrict__ beta,
    float* __restrict__ out, int64_t out_k_stride) {
  constexpr int kPass = kGP >= 16 ? 128 / kGP : kFcBatch;  // directions per shared-memory pass (16 KB)
  __shared__ float s_out[kPass][kEmitPoints * kGP];
  const int G = (int)blockDim.y;
  const int x = threadIdx.x, g = threadIdx.y, tid = g * kEmitPoints + x;
  const int64_t c0 = (int64_t)blockIdx.x * kEmitPoints;
  const int64_t c = c0 + x;  // one point per cell: the cell is the point
  const int n = (int)min((int64_t)kEmitPoints, in.V - c0);  // cells of this block
  float ux = 0.f, uy = 0.f, uz = 0.f, sc = 0.f, be = 0.f;
  if (x < n) {
    int i, j, k;
    point_rcs(c, pg, i, j, k);
    primary_direction(__ldg(in.ax_x + j), __ldg(in.ax_y + i), __ldg(in.ax_z + k), in.r0x, in.r0y, in.r0z, ux, uy, uz);
    sc = __ldg(scale + (int64_t)g * in.V + c);
    be = __ldg(beta + (int64_t)g * in.V + c);
  }
  const int d0 = blockIdx.y * kFcBatch, dlast = min(K, d0 + kFcBatch);
  for (int p0 = d0; p0 < dlast; p0 += kPass) {
    const int np = min(kPass, dlast - p0);
    // eight directions' cache loads in flight per thread before their products and shared-memory stores
    constexpr int kU = 8;
    for (int q0 = 0; q0 < np; q0 += kU) {
      float v[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u)
        v[u] = (x < n && q0 + u < np)
                   ? __ldg(cache + ((int64_t)__ldg(cache_index + p0 + q0 + u) * G + g) * in.V + c)
                   : 0.f;
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        if (q0 + u >= np) break;
        const int d = p0 + q0 + u;
        float r = 0.f;
        if (x < n) {
          const float ox = __ldg(omegas + 3 * d), oy = __ldg(omegas + 3 * d + 1), oz = __ldg(omegas + 3 * d + 2);
          const float cosine = ux * ox + uy * oy + uz * oz;
          r = v[u] * sc * (1.f + be * cosine);
        }
        s_out[q0 + u][x * G + g] = r;
      }
    }
    __syncthreads();
    for (int q = 0; q < np; ++q)
      if (tid < n * G) out[(int64_t)(p0 + q) * out_k_stride + c0 * G + tid] = s_out[q][tid];
    __syncthreads();
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
  }                                                                                           \
  note_launches();

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
  note_launches();
  return launch_status("citrus_group_transmission");
}

extern "C" int citrus_source_field(const double* field, const double* panel, const double* profile,
                                   const double* thickness, int64_t thickness_rows, double filter_density,
                                   const double* off_focal_nodes, const double* off_focal_values,
                                   int64_t num_off_focal, const double* points, const double* axis_x,
                                   const double* axis_y, const double* axis_z, const int64_t* point_dims,
                                   int64_t num_points, int32_t divide_by_distance_squared, float* out,
                                   float* filter_path_out, void* stream) {
  CITRUS_REQUIRE(field && out, "citrus_source_field: null pointer");
  CITRUS_REQUIRE(points || (axis_x && axis_y && axis_z && point_dims), "citrus_source_field: no points");
  CITRUS_REQUIRE(num_points >= 0 && num_off_focal >= 0, "citrus_source_field: negative size");
  CITRUS_REQUIRE((num_off_focal == 0) == (off_focal_nodes == nullptr) &&
                     (off_focal_nodes == nullptr) == (off_focal_values == nullptr),
                 "citrus_source_field: the off-focal nodes and values go together with their count");
  CITRUS_REQUIRE((thickness == nullptr) == (filter_path_out == nullptr),
                 "citrus_source_field: the filter thickness and the filter-path output go together");
  CITRUS_REQUIRE(!(profile || thickness) || panel, "citrus_source_field: a profile or a filter needs the panel");
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
  SourceExtras ex{};
  ex.profile = profile;
  ex.thickness = thickness;
  ex.off_nodes = off_focal_nodes;
  ex.off_values = off_focal_values;
  ex.n_off = (int)num_off_focal;
  ex.filter_density = filter_density;
  if (panel) {
    ex.rows = (int)panel[0];
    ex.channels = (int)panel[1];
    ex.d_row = panel[2];
    ex.d_ch = panel[3];
    ex.off_row = panel[4];
    ex.off_ch = panel[5];
    CITRUS_REQUIRE(ex.rows >= 1 && ex.channels >= 1 && ex.d_row > 0 && ex.d_ch > 0,
                   "citrus_source_field: bad panel");
  }
  ex.t_rows = (int)thickness_rows;
  CITRUS_REQUIRE(!thickness || thickness_rows == 1 || thickness_rows == ex.rows,
                 "citrus_source_field: the filter thickness must have 1 or all rows");
  int gc = 1, gs = 1;
  if (!points) {
    gc = (int)point_dims[1];
    gs = (int)point_dims[2];
  }
  if (num_points == 0) return CITRUS_OK;
  source_weight_kernel<<<(unsigned)cdiv(num_points, 128), 128, 0, as_stream(stream)>>>(
      fd, ex, points, axis_x, axis_y, axis_z, gc, gs, num_points, divide_by_distance_squared, out, filter_path_out);
  note_launches();
  return launch_status("citrus_source_field");
}

extern "C" int citrus_source_weight(const double* field, const double* points, const double* axis_x,
                                    const double* axis_y, const double* axis_z, const int64_t* point_dims,
                                    int64_t num_points, int32_t divide_by_distance_squared, float* out, void* stream) {
  return citrus_source_field(field, nullptr, nullptr, nullptr, 0, 0.0, nullptr, nullptr, 0, points, axis_x, axis_y,
                             axis_z, point_dims, num_points, divide_by_distance_squared, out, nullptr, stream);
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
  const Table tb = make_table(table, num_materials, num_eta, num_groups, eta_lo, eta_hi);
  const PointGrid pg = make_grid(point_dims, 1);
  const int G = (int)num_groups, K = (int)num_directions, KB = 4;
  dim3 grid((unsigned)cdiv(V, kPoints), (unsigned)cdiv(K, KB)), block(kPoints, G);
  CITRUS_G_DISPATCH(G, fc_source_kernel, grid, block, 0, as_stream(stream), in, tb, pg, omegas, K, KB, out)
  return launch_status("citrus_first_collision_source");
}

namespace citrus {
namespace {

template <int kGP, int kMM>
int launch_fc_correction_m(dim3 grid, int G, cudaStream_t s, const FCInputs& in, const Table& tb,
                           const PointGrid& pg, const float* omegas, const float* weights, int K,
                           const float* moments, float* sums, float* scale, float* beta, float* cache) {
  cudaError_t e = cudaFuncSetAttribute(fc_correction_kernel<kGP, kMM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kWindowBytes);
  if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "first-collision window: %s", cudaGetErrorString(e));
  fc_correction_kernel<kGP, kMM><<<grid, dim3(kEmitPoints, G), kWindowBytes, s>>>(in, tb, pg, omegas, weights, K,
                                                                                 moments, sums, scale, beta, cache);
  note_launches();
  return CITRUS_OK;
}

template <int kGP, int kMM, bool kVec>
int launch_fc_correction_warps(dim3 grid, cudaStream_t s, const FCInputs& in, const Table& tb, const PointGrid& pg,
                               const float* omegas, const float* weights, int K, const float* moments, float* sums,
                               float* scale, float* beta, float* cache) {
  constexpr int bytes = emission_window_bytes(kFcDirBatch);
  cudaError_t e = cudaFuncSetAttribute(fc_correction_warps_kernel<kGP, kMM, kVec>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "first-collision window: %s", cudaGetErrorString(e));
  fc_correction_warps_kernel<kGP, kMM, kVec><<<grid, 32 * kFcWarps, bytes, s>>>(in, tb, pg, omegas, weights, K,
                                                                                moments, sums, scale, beta, cache);
  note_launches();
  return CITRUS_OK;
}

// CITRUS_FC_KERNEL=groups selects the group-lane correction kernel (fc_correction_kernel); read at every call
inline bool fc_by_groups() {
  const char* v = getenv("CITRUS_FC_KERNEL");
  return v != nullptr && v[0] == 'g';
}

// materials held in registers: two (the common water and bone case) or up to eight; G <= 16 takes the (point,
// direction) kernel
template <int kGP>
int launch_fc_correction(dim3 grid, int G, cudaStream_t s, const FCInputs& in, const Table& tb, const PointGrid& pg,
                         const float* omegas, const float* weights, int K, const float* moments, float* sums,
                         float* scale, float* beta, float* cache) {
  if constexpr (kGP <= 16) {
    if (!fc_by_groups()) {
      const bool vec = kGP >= 4 && G % 4 == 0 && ((uintptr_t)tb.t % 16) == 0;
      constexpr bool kCanVec = kGP >= 4;
      if (tb.M <= 2)
        return vec ? launch_fc_correction_warps<kGP, 2, kCanVec>(grid, s, in, tb, pg, omegas, weights, K, moments,
                                                                 sums, scale, beta, cache)
                   : launch_fc_correction_warps<kGP, 2, false>(grid, s, in, tb, pg, omegas, weights, K, moments,
                                                               sums, scale, beta, cache);
      return vec ? launch_fc_correction_warps<kGP, kMaxM, kCanVec>(grid, s, in, tb, pg, omegas, weights, K, moments,
                                                                   sums, scale, beta, cache)
                 : launch_fc_correction_warps<kGP, kMaxM, false>(grid, s, in, tb, pg, omegas, weights, K, moments,
                                                                 sums, scale, beta, cache);
    }
  }
  if (tb.M <= 2)
    return launch_fc_correction_m<kGP, 2>(grid, G, s, in, tb, pg, omegas, weights, K, moments, sums, scale, beta,
                                          cache);
  return launch_fc_correction_m<kGP, kMaxM>(grid, G, s, in, tb, pg, omegas, weights, K, moments, sums, scale, beta,
                                            cache);
}

template <int kGP>
void launch_fc_moments_cached(int64_t NC, int G, int K, cudaStream_t s, const FCInputs& in, const PointGrid& pg,
                              const float* omegas, const float* cache, const int32_t* cache_index,
                              const float* scale, const float* beta, float slope_scale, float* out,
                              int64_t out_k_stride) {
  dim3 grid((unsigned)cdiv(NC, kEmitPoints), (unsigned)cdiv(K, kFcBatch));
  fc_moments_cached_kernel<kGP><<<grid, dim3(kEmitPoints, G), 0, s>>>(in, pg, omegas, K, cache, cache_index, scale,
                                                                      beta, slope_scale, out, out_k_stride);
  note_launches();
}

template <int kGP>
void launch_fc_means(int G, int K, cudaStream_t s, const FCInputs& in, const PointGrid& pg, const float* omegas,
                     const float* cache, const int32_t* cache_index, const float* scale, const float* beta, float* out,
                     int64_t out_k_stride) {
  dim3 grid((unsigned)cdiv(in.V, kEmitPoints), (unsigned)cdiv(K, kFcBatch));
  fc_means_kernel<kGP><<<grid, dim3(kEmitPoints, G), 0, s>>>(in, pg, omegas, K, cache, cache_index, scale, beta, out,
                                                             out_k_stride);
  note_launches();
}

}  // namespace
}  // namespace citrus

#define CITRUS_GP_DISPATCH(G, CALL) \
  ((G) <= 1 ? CALL(1) : (G) <= 2 ? CALL(2) : (G) <= 4 ? CALL(4) : (G) <= 8 ? CALL(8) : (G) <= 16 ? CALL(16) : CALL(32))

extern "C" int citrus_first_collision_moments(const float* rho, int64_t num_materials, const float* phi,
                                              int64_t num_groups, const float* axes, const int64_t* point_dims,
                                              int64_t points_per_cell, const double* focal_spot, const float* table,
                                              int64_t num_eta, double eta_lo, double eta_hi, const float* omegas,
                                              int64_t num_directions, const float* scale, const float* beta,
                                              const float* cache, const int32_t* cache_index, float* out,
                                              int64_t out_direction_stride, void* stream) {
  int st = check_table(table, num_materials, num_eta, num_groups);
  if (st) return st;
  CITRUS_REQUIRE(rho && phi && axes && point_dims && focal_spot && omegas && scale && beta && out,
                 "citrus_first_collision_moments: null pointer");
  CITRUS_REQUIRE((cache == nullptr) == (cache_index == nullptr),
                 "citrus_first_collision_moments: cache and cache_index go together");
  const int64_t f = points_per_cell;
  CITRUS_REQUIRE(f >= 1 && point_dims[0] % f == 0 && point_dims[1] % f == 0 && point_dims[2] % f == 0,
                 "citrus_first_collision_moments: the point grid is not cells x %lld", (long long)f);
  CITRUS_REQUIRE(((uintptr_t)out % 16) == 0 && out_direction_stride % 4 == 0,
                 "citrus_first_collision_moments: out must be 16-byte aligned");
  CITRUS_REQUIRE(num_directions <= 65535, "citrus_first_collision_moments: too many directions");
  const int64_t V = point_dims[0] * point_dims[1] * point_dims[2];
  if (V == 0 || num_directions == 0) return CITRUS_OK;
  const FCInputs in = make_inputs(rho, phi, axes, V, focal_spot, point_dims);
  const Table tb = make_table(table, num_materials, num_eta, num_groups, eta_lo, eta_hi);
  const PointGrid pg = make_grid(point_dims, f);
  double mean_u2 = 0;
  for (int j = 0; j < f; ++j) {
    const double u = (2.0 * j + 1.0) / f - 1.0;
    mean_u2 += u * u / f;
  }
  const float slope_scale = f > 1 ? (float)(1.0 / mean_u2) : 0.f;
  const int64_t NC = V / (f * f * f);
  const int G = (int)num_groups, K = (int)num_directions;
  cudaStream_t s = as_stream(stream);
  if (cache != nullptr) {
#define CITRUS_FCM(GP) \
  (launch_fc_moments_cached<GP>(NC, G, K, s, in, pg, omegas, cache, cache_index, scale, beta, slope_scale, out, \
                                out_direction_stride), 0)
    (void)CITRUS_GP_DISPATCH(G, CITRUS_FCM);
#undef CITRUS_FCM
    return launch_status("citrus_first_collision_moments");
  }
  dim3 grid((unsigned)cdiv(NC, kPoints), (unsigned)K), block(kPoints, G);
  CITRUS_G_DISPATCH(G, fc_moments_kernel, grid, block, 0, s, in, tb, pg, omegas, K, scale, beta, slope_scale, out,
                    out_direction_stride)
  return launch_status("citrus_first_collision_moments");
}

extern "C" int citrus_first_collision_means(int64_t num_groups, const float* axes, const int64_t* point_dims,
                                            const double* focal_spot, const float* omegas, int64_t num_directions,
                                            const float* scale, const float* beta, const float* cache,
                                            const int32_t* cache_index, float* out, int64_t out_direction_stride,
                                            void* stream) {
  CITRUS_REQUIRE(axes && point_dims && focal_spot && omegas && scale && beta && cache && cache_index && out,
                 "citrus_first_collision_means: null pointer");
  CITRUS_REQUIRE(num_groups >= 1 && num_groups <= 32 && num_directions <= 65535,
                 "citrus_first_collision_means: bad sizes");
  const int64_t V = point_dims[0] * point_dims[1] * point_dims[2];
  CITRUS_REQUIRE(out_direction_stride >= V * num_groups, "citrus_first_collision_means: direction stride too small");
  if (V == 0 || num_directions == 0) return CITRUS_OK;
  const FCInputs in = make_inputs(nullptr, nullptr, axes, V, focal_spot, point_dims);  // points only
  const PointGrid pg = make_grid(point_dims, 1);
  const int G = (int)num_groups, K = (int)num_directions;
  cudaStream_t s = as_stream(stream);
#define CITRUS_FCM(GP) \
  (launch_fc_means<GP>(G, K, s, in, pg, omegas, cache, cache_index, scale, beta, out, out_direction_stride), 0)
  (void)CITRUS_GP_DISPATCH(G, CITRUS_FCM);
#undef CITRUS_FCM
  return launch_status("citrus_first_collision_means");
}

extern "C" int citrus_first_collision_correction(const float* rho, int64_t num_materials, const float* phi,
                                                 int64_t num_groups, const float* axes, const int64_t* point_dims,
                                                 const double* focal_spot, const float* table, int64_t num_eta,
                                                 double eta_lo, double eta_hi, const float* omegas,
                                                 const float* weights, int64_t num_directions, const float* moments,
                                                 float* sums, float* scale, float* beta, float* cache, void* stream) {
  int st = check_table(table, num_materials, num_eta, num_groups);
  if (st) return st;
  CITRUS_REQUIRE(rho && phi && axes && point_dims && focal_spot && omegas && weights && moments && scale && beta,
                 "citrus_first_collision_correction: null pointer");
  if (num_groups % 4 == 0)
    CITRUS_REQUIRE(((uintptr_t)table % 16) == 0, "citrus_first_collision_correction: table must be 16-byte aligned");
  const int64_t V = point_dims[0] * point_dims[1] * point_dims[2];
  if (V == 0) return CITRUS_OK;
  const FCInputs in = make_inputs(rho, phi, axes, V, focal_spot, point_dims);
  const Table tb = make_table(table, num_materials, num_eta, num_groups, eta_lo, eta_hi);
  const PointGrid pg = make_grid(point_dims, 1);
  const int G = (int)num_groups, K = (int)num_directions;
  dim3 grid((unsigned)cdiv(V, kEmitPoints));
  cudaStream_t s = as_stream(stream);
#define CITRUS_FCC(GP) launch_fc_correction<GP>(grid, G, s, in, tb, pg, omegas, weights, K, moments, sums, scale, beta, cache)
  st = CITRUS_GP_DISPATCH(G, CITRUS_FCC);
#undef CITRUS_FCC
  if (st) return st;
  return launch_status("citrus_first_collision_correction");
}

namespace citrus {
namespace {

template <int kGP, int kMM, bool kFused, int kDirs>
int launch_emission_d(dim3 grid, cudaStream_t s, const FCInputs& in, const Table& tb, const PointGrid& pg,
                      const float* omegas, int K, const float* tau, const float* tau_mu, int TM, const float* mu,
                      const float* multiple, const float* harmonics, const float* moments, int NS,
                      const float* heights, const float* signal_weight, const double* deltas, float* out,
                      float* partial) {
  constexpr int bytes = emission_window_bytes(kDirs);
  cudaError_t e = cudaFuncSetAttribute(emission_kernel<kGP, kMM, kFused, kDirs>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "emission window: %s", cudaGetErrorString(e));
  grid.y = (unsigned)cdiv(K, kDirs);
  emission_kernel<kGP, kMM, kFused, kDirs><<<grid, kEmitPoints * kGP, bytes, s>>>(
      in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple, harmonics, moments, NS, heights, signal_weight, (float)deltas[0],
      (float)deltas[1], (float)deltas[2], out, partial);
  note_launches();
  return CITRUS_OK;
}

// directions per emission block: 32 amortise the block's set-up (point geometry, table window) over twice as many
// directions once there are enough of them; CITRUS_EMISSION_DIRS (16, 32 or 64) overrides, for measurements
inline int emission_dirs(int K) {
  static const int forced = [] {
    const char* v = getenv("CITRUS_EMISSION_DIRS");
    return v ? atoi(v) : 0;
  }();
  if (forced == 16 || forced == 32 || forced == 64) return forced;
  return K >= 64 ? 32 : 16;
}

template <int kGP, int kMM, bool kFused>
int launch_emission_m(dim3 grid, int G, cudaStream_t s, const FCInputs& in, const Table& tb, const PointGrid& pg,
                      const float* omegas, int K, const float* tau, const float* tau_mu, int TM, const float* mu,
                      const float* multiple, const float* harmonics, const float* moments, int NS,
                      const float* heights, const float* signal_weight, const double* deltas, float* out,
                      float* partial) {
  (void)G;
  const int dirs = emission_dirs(K);
  if (dirs == 64)
    return launch_emission_d<kGP, kMM, kFused, 64>(grid, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple,
                                                   harmonics, moments, NS, heights, signal_weight, deltas, out,
                                                   partial);
  if (dirs == 32)
    return launch_emission_d<kGP, kMM, kFused, 32>(grid, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple,
                                                   harmonics, moments, NS, heights, signal_weight, deltas, out,
                                                   partial);
  return launch_emission_d<kGP, kMM, kFused, 16>(grid, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple,
                                                 harmonics, moments, NS, heights, signal_weight, deltas, out, partial);
}

template <int kGP, bool kFused>
int launch_emission(dim3 grid, int G, cudaStream_t s, const FCInputs& in, const Table& tb, const PointGrid& pg,
                    const float* omegas, int K, const float* tau, const float* tau_mu, int TM, const float* mu,
                    const float* multiple, const float* harmonics, const float* moments, int NS,
                    const float* heights, const float* signal_weight, const double* deltas, float* out,
                    float* partial) {
  if (tb.M <= 2 && TM <= 2)
    return launch_emission_m<kGP, 2, kFused>(grid, G, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple,
                                             harmonics, moments, NS, heights, signal_weight, deltas, out, partial);
  return launch_emission_m<kGP, kMaxM, kFused>(grid, G, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple,
                                               harmonics, moments, NS, heights, signal_weight, deltas, out, partial);
}

template <int kGP, int kMM, int kDirs, bool kVec, bool kQ1>
int launch_emission_warps_q(dim3 grid, cudaStream_t s, const FCInputs& in, const Table& tb, const PointGrid& pg,
                            const float* omegas, int K, const float* tau, const float* tau_mu, int TM,
                            const float* mu, const float* multiple, const float* heights, const float* signal_weight,
                            const double* deltas, float* out, float* partial) {
  constexpr int bytes = emission_window_bytes(kDirs);
  cudaError_t e = cudaFuncSetAttribute(emission_warps_kernel<kGP, kMM, kDirs, kVec, kQ1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "emission window: %s", cudaGetErrorString(e));
  grid.y = (unsigned)cdiv(K, kDirs);
  emission_warps_kernel<kGP, kMM, kDirs, kVec, kQ1><<<grid, 32 * kEmitWarps, bytes, s>>>(
      in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple, heights, signal_weight, (float)deltas[0],
      (float)deltas[1], (float)deltas[2], out, partial);
  note_launches();
  return CITRUS_OK;
}

template <int kGP, int kMM, int kDirs, bool kVec>
int launch_emission_warps_d(dim3 grid, cudaStream_t s, const FCInputs& in, const Table& tb, const PointGrid& pg,
                            const float* omegas, int K, const float* tau, const float* tau_mu, int TM,
                            const float* mu, const float* multiple, const float* heights, const float* signal_weight,
                            const double* deltas, float* out, float* partial) {
  if (pg.f == 1)
    return launch_emission_warps_q<kGP, kMM, kDirs, kVec, true>(grid, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu,
                                                                multiple, heights, signal_weight, deltas, out,
                                                                partial);
  return launch_emission_warps_q<kGP, kMM, kDirs, kVec, false>(grid, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu,
                                                               multiple, heights, signal_weight, deltas, out, partial);
}

template <int kGP, int kMM, bool kVec>
int launch_emission_warps_v(dim3 grid, cudaStream_t s, const FCInputs& in, const Table& tb, const PointGrid& pg,
                            const float* omegas, int K, const float* tau, const float* tau_mu, int TM,
                            const float* mu, const float* multiple, const float* heights, const float* signal_weight,
                            const double* deltas, float* out, float* partial) {
  if (K >= 64)
    return launch_emission_warps_d<kGP, kMM, 64, kVec>(grid, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple,
                                                       heights, signal_weight, deltas, out, partial);
  return launch_emission_warps_d<kGP, kMM, 32, kVec>(grid, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple,
                                                     heights, signal_weight, deltas, out, partial);
}

// the (point, direction) kernel for G <= 16 with the multiple-collision source read (not fused); float4 group rows
// when G is a multiple of 4 and the table, the per-group inputs and the output are 16-byte aligned
template <int kGP>
int launch_emission_warps(dim3 grid, cudaStream_t s, const FCInputs& in, const Table& tb, const PointGrid& pg,
                          const float* omegas, int K, const float* tau, const float* tau_mu, int TM, const float* mu,
                          const float* multiple, const float* heights, const float* signal_weight,
                          const double* deltas, float* out, float* partial) {
  const auto aligned = [](const void* p) { return ((uintptr_t)p % 16) == 0; };
  const bool vec = tb.G % 4 == 0 && aligned(tb.t) && aligned(multiple) && (tau_mu != nullptr || aligned(tau)) &&
                   (signal_weight != nullptr || aligned(out));
  constexpr bool kCanVec = kGP >= 4;  // G < 4 has no float4 rows
#define CITRUS_EW(MM, VEC)                                                                                         \
  launch_emission_warps_v<kGP, MM, VEC>(grid, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple, heights,    \
                                        signal_weight, deltas, out, partial)
  if (tb.M <= 2 && TM <= 2) return vec ? CITRUS_EW(2, kCanVec) : CITRUS_EW(2, false);
  return vec ? CITRUS_EW(kMaxM, kCanVec) : CITRUS_EW(kMaxM, false);
#undef CITRUS_EW
}

// CITRUS_EMISSION_KERNEL=groups selects the group-lane kernel (emission_kernel) for the product form too; read at
// every call, for measurements and for the test that the two kernels agree
inline bool emission_by_groups() {
  const char* v = getenv("CITRUS_EMISSION_KERNEL");
  return v != nullptr && v[0] == 'g';
}

template <int kGP>
int emission_for(int64_t V, int K, cudaStream_t s, const FCInputs& in, const Table& tb, const PointGrid& pg,
                 const float* omegas, const float* tau, const float* tau_mu, int TM, const float* mu,
                 const float* multiple,
                 const float* harmonics, const float* moments, int NS, const float* heights,
                 const float* signal_weight, const double* deltas, float* out, float* partial,
                 float* height_sums) {
  const int64_t nblocks = cdiv(V, kEmitPoints);
  dim3 grid((unsigned)nblocks, 1u);  // grid.y: the direction blocks, set by the launcher
  int st;
  if (moments == nullptr && kGP <= 16 && !emission_by_groups())
    st = launch_emission_warps<(kGP <= 16 ? kGP : 16)>(grid, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple,
                                                       heights, signal_weight, deltas, out, partial);
  else
    st = moments != nullptr
             ? launch_emission<kGP, true>(grid, tb.G, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple,
                                          harmonics, moments, NS, heights, signal_weight, deltas, out, partial)
             : launch_emission<kGP, false>(grid, tb.G, s, in, tb, pg, omegas, K, tau, tau_mu, TM, mu, multiple,
                                           harmonics, moments, NS, heights, signal_weight, deltas, out, partial);
  if (st) return st;
  reduce_partials_kernel<<<K, dim3(256, 2), 0, s>>>(partial, nblocks, K, height_sums);
  note_launches();
  return CITRUS_OK;
}

// shared by the two entry points: multiple [K, G, NC] (moments NULL), or harmonics [K, NS] and moments [NS, G, NC]
int attenuated_emission(const char* name, const float* rho, int64_t num_materials, const float* phi,
                        int64_t num_groups, const float* axes, const int64_t* point_dims, int64_t points_per_cell,
                        const double* point_deltas, const double* focal_spot, const float* table, int64_t num_eta,
                        double eta_lo, double eta_hi, const float* omegas, int64_t num_directions, const float* tau,
                        const float* tau_mu, int64_t tau_materials, const float* mu, const float* multiple,
                        const float* harmonics, const float* moments,
                        int64_t num_moments, const float* heights, const float* signal_weight, float* out,
                        float* partial, int64_t partial_capacity, float* height_sums, void* stream) {
  int st = check_table(table, num_materials, num_eta, num_groups);
  if (st) return st;
  CITRUS_REQUIRE(rho && phi && axes && point_dims && point_deltas && focal_spot && omegas && tau && mu && out &&
                     partial && height_sums && (multiple || (harmonics && moments)),
                 "%s: null pointer", name);
  CITRUS_REQUIRE(tau_mu == nullptr || (tau_materials >= 1 && tau_materials <= kMaxM),
                 "%s: %lld traced materials outside [1, %d]", name, (long long)tau_materials, kMaxM);
  CITRUS_REQUIRE(moments == nullptr || (num_moments >= 1 && num_moments <= kMaxMoments),
                 "%s: %lld moments outside [1, %d]", name, (long long)num_moments, kMaxMoments);
  const int64_t f = points_per_cell;
  CITRUS_REQUIRE(f >= 1 && point_dims[0] % f == 0 && point_dims[1] % f == 0 && point_dims[2] % f == 0,
                 "%s: the point grid is not cells x %lld", name, (long long)f);
  CITRUS_REQUIRE(num_directions >= 0 && num_directions <= 65535, "%s: bad direction count", name);
  if (num_groups % 4 == 0)
    CITRUS_REQUIRE(((uintptr_t)table % 16) == 0 && ((uintptr_t)out % 16) == 0,
                   "%s: table and out must be 16-byte aligned", name);
  const int64_t V = point_dims[0] * point_dims[1] * point_dims[2];
  const int64_t nblocks = cdiv(V, kEmitPoints);
  CITRUS_REQUIRE(partial_capacity >= nblocks * num_directions * 2, "%s: partial buffer holds %lld floats, needs %lld",
                 name, (long long)partial_capacity, (long long)(nblocks * num_directions * 2));
  if (V == 0 || num_directions == 0) return CITRUS_OK;
  const FCInputs in = make_inputs(rho, phi, axes, V, focal_spot, point_dims);
  const Table tb = make_table(table, num_materials, num_eta, num_groups, eta_lo, eta_hi);
  const PointGrid pg = make_grid(point_dims, f);
  const int G = (int)num_groups, K = (int)num_directions, NS = (int)num_moments;
  cudaStream_t s = as_stream(stream);
#define CITRUS_EMISSION(GP)                                                                                        \
  emission_for<GP>(V, K, s, in, tb, pg, omegas, tau, tau_mu, (int)tau_materials, mu, multiple, harmonics, moments,  \
                   NS, heights, signal_weight, \
                   point_deltas, out, partial, height_sums)
  if (G <= 1) st = CITRUS_EMISSION(1);
  else if (G <= 2) st = CITRUS_EMISSION(2);
  else if (G <= 4) st = CITRUS_EMISSION(4);
  else if (G <= 8) st = CITRUS_EMISSION(8);
  else if (G <= 16) st = CITRUS_EMISSION(16);
  else st = CITRUS_EMISSION(32);
#undef CITRUS_EMISSION
  if (st) return st;
  return launch_status(name);
}

}  // namespace
}  // namespace citrus

extern "C" int citrus_attenuated_emission(const float* rho, int64_t num_materials, const float* phi,
                                          int64_t num_groups, const float* axes, const int64_t* point_dims,
                                          int64_t points_per_cell, const double* point_deltas,
                                          const double* focal_spot, const float* table, int64_t num_eta,
                                          double eta_lo, double eta_hi, const float* omegas, int64_t num_directions,
                                          const float* tau, const float* tau_mu, int64_t tau_materials,
                                          const float* mu, const float* multiple, const float* heights,
                                          const float* signal_weight, float* out, float* partial,
                                          int64_t partial_capacity, float* height_sums, void* stream) {
  CITRUS_REQUIRE(multiple != nullptr, "citrus_attenuated_emission: null multiple-collision source");
  return attenuated_emission("citrus_attenuated_emission", rho, num_materials, phi, num_groups, axes, point_dims,
                             points_per_cell, point_deltas, focal_spot, table, num_eta, eta_lo, eta_hi, omegas,
                             num_directions, tau, tau_mu, tau_materials, mu, multiple, nullptr, nullptr, 0, heights,
                             signal_weight, out, partial, partial_capacity, height_sums, stream);
}

extern "C" int citrus_attenuated_emission_moments(const float* rho, int64_t num_materials, const float* phi,
                                                  int64_t num_groups, const float* axes, const int64_t* point_dims,
                                                  int64_t points_per_cell, const double* point_deltas,
                                                  const double* focal_spot, const float* table, int64_t num_eta,
                                                  double eta_lo, double eta_hi, const float* omegas,
                                                  int64_t num_directions, const float* tau, const float* tau_mu,
                                                  int64_t tau_materials, const float* mu, const float* harmonics,
                                                  const float* moments, int64_t num_moments,
                                                  const float* heights, const float* signal_weight, float* out,
                                                  float* partial, int64_t partial_capacity, float* height_sums,
                                                  void* stream) {
  CITRUS_REQUIRE(harmonics != nullptr && moments != nullptr,
                 "citrus_attenuated_emission_moments: null harmonics or moments");
  return attenuated_emission("citrus_attenuated_emission_moments", rho, num_materials, phi, num_groups, axes,
                             point_dims, points_per_cell, point_deltas, focal_spot, table, num_eta, eta_lo, eta_hi,
                             omegas, num_directions, tau, tau_mu, tau_materials, mu, nullptr, harmonics, moments,
                             num_moments, heights,
                             signal_weight, out, partial, partial_capacity, height_sums, stream);
}
