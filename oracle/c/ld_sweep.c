/*
 * CPU restatement of the linear-discontinuous wavefront sweep of one direction chunk, float64, OpenMP over the entries
 * of a plane. Test infrastructure (the oracle and the timed CPU baseline); it follows
 * citrus/scatter_solver/transport_sweep.py:271-357 (plane step, zero vacuum neighbour) and
 * linear_discontinuous_cell.py:14-87 (right-hand sides and closed-form solve), the same arithmetic as oracle/sweep.py.
 *
 * store   [8, Dc, N, G, 4] float64: the chunk's source moments, overwritten with the angular-fluence moments.
 * mu      [N, G] float64 total attenuation per cell; c [8, Dc, 3] |Omega_a| / Delta_a.
 * octant, cell [E], upstream [E, 3] (-1 or N: vacuum) and offsets [P + 1]: the plane-sorted plan (int64).
 */
#include <stdint.h>

static void solve_one(const double* c, double sx, double sy, double sz, double m, const double* s, const double* X,
                      const double* Y, const double* Z, double* out) {
  const double cx = c[0], cy = c[1], cz = c[2];
  const double pbx = X[0] + sx * X[1], pby = Y[0] + sy * Y[2], pbz = Z[0] + sz * Z[3];
  const double r0 = s[0] + (cx * pbx + cy * pby + cz * pbz);
  const double rx = s[1] - 3.0 * sx * cx * pbx + (cy * Y[1] + cz * Z[1]);
  const double ry = s[2] - 3.0 * sy * cy * pby + (cx * X[2] + cz * Z[2]);
  const double rz = s[3] - 3.0 * sz * cz * pbz + (cx * X[3] + cy * Y[3]);
  const double csum = cx + cy + cz;
  const double dx = 3.0 * cx + (csum - cx) + m, dy = 3.0 * cy + (csum - cy) + m, dz = 3.0 * cz + (csum - cz) + m;
  const double qx = cx / dx, qy = cy / dy, qz = cz / dz;
  const double den = csum + m + 3.0 * (cx * qx + cy * qy + cz * qz);
  const double p0 = (r0 - (sx * qx * rx + sy * qy * ry + sz * qz * rz)) / den;
  out[0] = p0;
  out[1] = (rx + 3.0 * sx * cx * p0) / dx;
  out[2] = (ry + 3.0 * sy * cy * p0) / dy;
  out[3] = (rz + 3.0 * sz * cz * p0) / dz;
}

int oracle_ld_sweep_chunk(double* store, const double* mu, const double* c, const int64_t* octant,
                          const int64_t* cell, const int64_t* upstream, const int64_t* offsets, int64_t num_planes,
                          int64_t N, int64_t G, int64_t Dc) {
  static const double zero[4] = {0.0, 0.0, 0.0, 0.0};
  const int64_t Q = 4 * G;
  for (int64_t p = 0; p < num_planes; ++p) {
    const int64_t start = offsets[p], end = offsets[p + 1];
    const int64_t work = (end - start) * Dc;
#pragma omp parallel for schedule(static)
    for (int64_t w = 0; w < work; ++w) {
      const int64_t e = start + w / Dc, d = w % Dc;
      const int64_t o = octant[e], n = cell[e];
      const int64_t u[3] = {upstream[3 * e], upstream[3 * e + 1], upstream[3 * e + 2]};
      const double sx = (o & 4) ? -1.0 : 1.0, sy = (o & 2) ? -1.0 : 1.0, sz = (o & 1) ? -1.0 : 1.0;
      const double* cc = c + 3 * (o * Dc + d);
      double* base = store + (o * Dc + d) * N * Q;
      for (int64_t g = 0; g < G; ++g) {
        const double* X = (u[0] >= 0 && u[0] < N) ? base + u[0] * Q + 4 * g : zero;
        const double* Y = (u[1] >= 0 && u[1] < N) ? base + u[1] * Q + 4 * g : zero;
        const double* Z = (u[2] >= 0 && u[2] < N) ? base + u[2] * Q + 4 * g : zero;
        double* s = base + n * Q + 4 * g;
        double out[4];
        solve_one(cc, sx, sy, sz, mu[n * G + g], s, X, Y, Z, out);
        s[0] = out[0];
        s[1] = out[1];
        s[2] = out[2];
        s[3] = out[3];
      }
    }
  }
  return 0;
}
