// Exact line integrals of voxel fields (Siddon / Amanatides-Woo traversal), the five ray operations of the
// reference's Projectors protocol (citrus/scatter_solver/ray_tracing.py:27-115, 141-202 and the Triton kernels of
// kernels/ray_tracing_kernels.py:215-639).
//
// Each ray is clipped to the grid box (the segment parameters of ray_tracing.py:160-173), then walked voxel by voxel.
// The walk keeps the ray's position as integer voxel indices plus a fractional position inside the current voxel, so
// every segment length is computed from quantities of voxel size (relative error ~ float epsilon per segment), and the
// travelled distance is summed with a compensated (Kahan) sum, so the end of the ray is placed to float epsilon of its
// total length, and it crosses along each axis only as many planes as lie between the entry and exit voxels. Rays that
// must meet 1e-6 relative path lengths (upstream to points, primary) do their set-up in float64; the oblique rays
// through the pixel centres, some of which run along a face of the box, do it in float pairs with float64 for the
// lines near a face; the downstream rays do it in float32.
//
// Volumes are read voxel-major, [V, C] with the C channels (groups or materials) of a voxel contiguous, so one voxel
// visit is one or two 16-byte loads for every channel at once.
#include <math.h>

#include "common.cuh"

namespace citrus {
namespace {

constexpr int kThreads = 128;
constexpr int kMaxChannels = 32;

struct Box {
  double lo[3];     // lower corner (x, y, z) in cm
  double delta[3];  // voxel sizes (x, y, z) in cm
  int n[3];         // voxel counts (x = columns, y = rows, z = slices)
  float lof[3], deltaf[3];  // the same rounded to float (float64 runs at a small fraction of float32 on this GPU)
};

Box make_box(const double* box, const int64_t* dims) {
  Box b;
  for (int a = 0; a < 3; ++a) {
    b.lo[a] = box[a];
    b.delta[a] = box[3 + a];
    b.n[a] = (int)dims[a];
    b.lof[a] = (float)b.lo[a];
    b.deltaf[a] = (float)b.delta[a];
  }
  return b;
}

// the centre of voxel i along axis a, in float
__device__ __forceinline__ float voxel_centre(const Box& b, int a, int i) {
  return b.lof[a] + b.deltaf[a] * ((float)i + 0.5f);
}

template <typename T>
struct Setup {
  bool hit;
  float total;      // length of the clipped segment in cm
  float v[3];       // direction in voxel units per cm
  int idx[3];       // voxel index at the entry point
  float f[3];       // fractional position inside that voxel, in [0, 1]
  int cross[3];     // plane crossings along each axis between the entry and exit voxels
};

// Rounded add and multiply that the compiler may not fuse, for the set-up steps whose rounding decides which voxels a
// line touches (the reference evaluates them as separate float64 tensor operations).
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }

// Clip p0 -> p1 to the box and locate the entry voxel. T is the arithmetic type of the set-up (double or float).
template <typename T>
__device__ __forceinline__ Setup<T> ray_setup(const Box& b, const T p0[3], const T p1[3]) {
  Setup<T> s;
  T d[3];
  T a_lo = 0, a_hi = 1;
  for (int a = 0; a < 3; ++a) {
    d[a] = p1[a] - p0[a];
    const T lo = (T)b.lo[a], hi = add_rn(lo, mul_rn((T)b.delta[a], (T)b.n[a]));
    if (d[a] != 0) {
      const T inv = (T)1 / d[a];
      const T t1 = (lo - p0[a]) * inv, t2 = (hi - p0[a]) * inv;
      a_lo = fmax(a_lo, fmin(t1, t2));
      a_hi = fmin(a_hi, fmax(t1, t2));
    } else if (!(p0[a] >= lo && p0[a] <= hi)) {
      a_hi = -1;  // parallel to this slab and outside it
    }
  }
  const T len = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  s.hit = a_hi > a_lo && len > 0;
  if (!s.hit) {
    s.total = 0.f;
    return s;
  }
  s.total = (float)((a_hi - a_lo) * len);
  for (int a = 0; a < 3; ++a) {
    const T u = d[a] / len;
    s.v[a] = (float)(u / (T)b.delta[a]);
    const T q = (p0[a] + a_lo * d[a] - (T)b.lo[a]) / (T)b.delta[a];
    T fl = floor(q);
    int i = (int)fl;
    if (i < 0) i = 0;
    if (i > b.n[a] - 1) i = b.n[a] - 1;
    T fr = q - (T)i;
    if (fr < 0) fr = 0;
    if (fr > 1) fr = 1;
    s.idx[a] = i;
    s.f[a] = (float)fr;
    // exit voxel along this axis, clamped like the entry one: a line that runs along a face of the box (within
    // rounding) stays in the boundary layer for its whole clipped length, as the segment midpoints of
    // ray_tracing.py:186-192 place it, instead of stepping out through that face at once
    int ie = (int)floor((p0[a] + a_hi * d[a] - (T)b.lo[a]) / (T)b.delta[a]);
    if (ie < 0) ie = 0;
    if (ie > b.n[a] - 1) ie = b.n[a] - 1;
    s.cross[a] = ie > i ? ie - i : i - ie;
  }
  return s;
}

// The constants of one oblique direction, shared by a block's rays (float64, formed once per block): the direction,
// the segment d = 2 h omega / |omega| that every ray of the direction spans, its reciprocal components, the far
// corner of the box and 1 / |omega|^2.
struct DirConst {
  double w[3];
  double d[3];
  double inv_d[3];
  double hi[3];
  double inv_w2;
  double h;
};

// The clipped set-up of a ray from p0 along the block's direction, the clip in float64 (so that a line in a face of
// the box meets it or misses it as the float64 reference does) and the walk's set-up in float32: the clip divides by
// nothing (the reciprocals are the block's), the exit point is p0 + d.
__device__ __forceinline__ Setup<float> ray_setup_dir(const Box& b, const double p0[3], const DirConst& dc) {
  Setup<float> s;
  double a_lo = 0, a_hi = 1;
  for (int a = 0; a < 3; ++a) {
    const double lo = b.lo[a], hi = dc.hi[a];
    if (dc.d[a] != 0) {
      const double t1 = (lo - p0[a]) * dc.inv_d[a], t2 = (hi - p0[a]) * dc.inv_d[a];
      a_lo = fmax(a_lo, fmin(t1, t2));
      a_hi = fmin(a_hi, fmax(t1, t2));
    } else if (!(p0[a] >= lo && p0[a] <= hi)) {
      a_hi = -1;  // parallel to this slab and outside it
    }
  }
  const float df[3] = {(float)dc.d[0], (float)dc.d[1], (float)dc.d[2]};
  const float len = sqrtf(df[0] * df[0] + df[1] * df[1] + df[2] * df[2]);
  s.hit = a_hi > a_lo && len > 0.f;
  if (!s.hit) {
    s.total = 0.f;
    return s;
  }
  s.total = (float)(a_hi - a_lo) * len;
  for (int a = 0; a < 3; ++a) {
    const float delta = (float)b.delta[a];
    s.v[a] = df[a] / len / delta;
    const float q = (float)(p0[a] + a_lo * dc.d[a] - b.lo[a]) / delta;   // entry, in voxels from the corner
    int i = (int)floorf(q);
    if (i < 0) i = 0;
    if (i > b.n[a] - 1) i = b.n[a] - 1;
    s.idx[a] = i;
    s.f[a] = fminf(fmaxf(q - (float)i, 0.f), 1.f);
    int ie = (int)floorf((float)(p0[a] + a_hi * dc.d[a] - b.lo[a]) / delta);   // exit voxel, clamped alike
    if (ie < 0) ie = 0;
    if (ie > b.n[a] - 1) ie = b.n[a] - 1;
    s.cross[a] = ie > i ? ie - i : i - ie;
  }
  return s;
}

// ---- float-pair set-up of the oblique rays --------------------------------------------------------------------
// float64 runs at a small fraction of the float32 rate on this GPU, so the oblique set-up is carried in float pairs
// (hi + lo, Knuth's two-sum and an fmaf-exact product error: ~2^-44 relative), which place a line's entry point and
// its clip to ~1e-11 cm, far inside the tolerances below. Every discrete decision of the float64 set-up (hit or miss,
// the binding faces, the entry and exit voxels) is taken from the pair values only when they lie clear of the
// decision's boundary by a margin (kFaceTol in cm, kParamTol along the line, kVoxelTol in voxels) that dwarfs both
// set-ups' rounding; a line nearer than that (a line in a face of the box, through an edge, or onto a voxel plane)
// is set up in float64 as before, so its voxels are the float64 set-up's.
constexpr float kFaceTol = 1e-7f;
constexpr float kParamTol = 1e-6f;
constexpr float kVoxelTol = 1e-5f;

struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF ff_norm(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return ff_norm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ FF ff_sub(FF a, FF b) { return ff_add(a, FF{-b.hi, -b.lo}); }
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = fmaf(a.hi, b.hi, -p);
  return ff_norm(p, __fadd_rn(e, __fadd_rn(__fmul_rn(a.hi, b.lo), __fmul_rn(a.lo, b.hi))));
}
__device__ __forceinline__ FF ff_mul(FF a, float b) {
  const float p = __fmul_rn(a.hi, b);
  const float e = fmaf(a.hi, b, -p);
  return ff_norm(p, __fadd_rn(e, __fmul_rn(a.lo, b)));
}
__device__ __forceinline__ float ff_float(FF a) { return __fadd_rn(a.hi, a.lo); }

// A float64 value as a float pair by integer operations on its bits: the top 24 bits of the significand (exact) and
// the low 29 rounded to float (2^-49 relative); magnitudes outside [2^-74, 2^151) are converted directly (zero).
__device__ __forceinline__ FF ff_from(double x) {
  const long long bits = __double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ff);
  if (e < 949 || e > 1173) return {__double2float_rn(x), 0.f};
  const unsigned long long m = ((unsigned long long)bits & 0xfffffffffffffull) | (1ull << 52);
  const float hi = __fmul_rn(__uint2float_rn((unsigned)(m >> 29)), __int_as_float((e - 919) << 23));
  const float lo = __fmul_rn(__uint2float_rn((unsigned)(m & 0x1fffffffull)), __int_as_float((e - 948) << 23));
  return bits < 0 ? FF{-hi, -lo} : FF{hi, lo};
}

// The per-direction constants of the float-pair set-up (formed once per block from the float64 ones).
struct DirPair {
  FF c[3], inv_w2, h, d[3], inv_d[3], lo[3], hi[3];
  float w[3], inv_df[3], delta[3], v[3], len;
};

__device__ __forceinline__ void make_dir_pair(const Box& b, const DirConst& dc, const double c[3], DirPair& dp) {
  dp.inv_w2 = ff_from(dc.inv_w2);
  dp.h = ff_from(dc.h);
  float df[3];
  for (int a = 0; a < 3; ++a) {
    dp.c[a] = ff_from(c[a]);
    dp.d[a] = ff_from(dc.d[a]);
    dp.inv_d[a] = ff_from(dc.inv_d[a]);
    dp.lo[a] = ff_from(b.lo[a]);
    dp.hi[a] = ff_from(dc.hi[a]);
    dp.w[a] = (float)dc.w[a];
    dp.inv_df[a] = (float)dc.inv_d[a];
    dp.delta[a] = (float)b.delta[a];
    df[a] = (float)dc.d[a];
  }
  dp.len = sqrtf(df[0] * df[0] + df[1] * df[1] + df[2] * df[2]);
  for (int a = 0; a < 3; ++a) dp.v[a] = df[a] / dp.len / dp.delta[a];
}

// The entry voxel along one axis from the pair position x (cm from the box's low face), as the float64 set-up forms
// it; false when x lies within kVoxelTol of an interior voxel plane.
__device__ __forceinline__ bool pair_voxel(FF x, float delta, int n, int& i, float& q) {
  q = ff_float(x) / delta;
  const float r = rintf(q);
  if (r >= 1.f && r <= (float)(n - 1) && fabsf(q - r) < kVoxelTol) return false;
  i = (int)floorf(q);
  if (i < 0) i = 0;
  if (i > n - 1) i = n - 1;
  return true;
}

// The clipped set-up of the ray through the pixel centre (px, py, pz) along the block's direction in float pairs:
// the same entry point (ray_tracing.py:588-595), clip and walk set-up as ray_setup_dir. Returns false, with s
// undefined, when a decision lies within its tolerance; the caller then sets the ray up in float64.
__device__ __forceinline__ bool ray_setup_pair(const Box& b, const DirPair& dp, double px, double py, double pz,
                                               Setup<float>& s) {
  const FF p[3] = {ff_from(px), ff_from(py), ff_from(pz)};
  FF dot = ff_mul(ff_sub(dp.c[0], p[0]), dp.w[0]);
  dot = ff_add(dot, ff_mul(ff_sub(dp.c[1], p[1]), dp.w[1]));
  dot = ff_add(dot, ff_mul(ff_sub(dp.c[2], p[2]), dp.w[2]));
  const FF tm = ff_sub(ff_mul(dot, dp.inv_w2), dp.h);
  FF a[3];
  for (int k = 0; k < 3; ++k) a[k] = ff_add(p[k], ff_mul(tm, dp.w[k]));
  // the clip: the largest entry and smallest exit parameter over the slabs (and the segment's own 0 and 1), with the
  // runner-up of each, so that a binding face that another one nearly ties with is left to float64
  float t_lo = 0.f, t_lo2 = -INFINITY, t_hi = 1.f, t_hi2 = INFINITY;
  FF f_lo = {0.f, 0.f}, f_hi = {0.f, 0.f};  // the binding faces' distances (cm), -1 axis: the segment's end
  int ax_lo = -1, ax_hi = -1;
  bool inside = true;
  for (int k = 0; k < 3; ++k) {
    const FF dl = ff_sub(dp.lo[k], a[k]), dh = ff_sub(dp.hi[k], a[k]);
    const float dlf = ff_float(dl), dhf = ff_float(dh);
    if (fabsf(dlf) < kFaceTol || fabsf(dhf) < kFaceTol) return false;
    if (dp.w[k] != 0.f) {
      const float t1 = dlf * dp.inv_df[k], t2 = dhf * dp.inv_df[k];
      const bool first = t1 <= t2;
      const float tn = first ? t1 : t2, tx = first ? t2 : t1;
      if (tn > t_lo) {
        t_lo2 = t_lo;
        t_lo = tn;
        ax_lo = k;
        f_lo = first ? dl : dh;
      } else {
        t_lo2 = fmaxf(t_lo2, tn);
      }
      if (tx < t_hi) {
        t_hi2 = t_hi;
        t_hi = tx;
        ax_hi = k;
        f_hi = first ? dh : dl;
      } else {
        t_hi2 = fminf(t_hi2, tx);
      }
    } else if (!(dlf <= 0.f && dhf >= 0.f)) {
      inside = false;  // parallel to this slab and outside it
    }
  }
  if (t_lo - t_lo2 < kParamTol || t_hi2 - t_hi < kParamTol) return false;
  if (fabsf(t_hi - t_lo) < kParamTol) return false;
  s.hit = inside && t_hi > t_lo && dp.len > 0.f;
  if (!s.hit) {
    s.total = 0.f;
    return true;
  }
  const FF a_lo = ax_lo >= 0 ? ff_mul(f_lo, dp.inv_d[ax_lo]) : FF{0.f, 0.f};
  const FF a_hi = ax_hi >= 0 ? ff_mul(f_hi, dp.inv_d[ax_hi]) : FF{1.f, 0.f};
  s.total = ff_float(ff_sub(a_hi, a_lo)) * dp.len;
  for (int k = 0; k < 3; ++k) {
    const FF rel = ff_sub(a[k], dp.lo[k]);
    int i, ie;
    float q, qe;
    if (!pair_voxel(ff_add(rel, ff_mul(a_lo, dp.d[k])), dp.delta[k], b.n[k], i, q)) return false;
    if (!pair_voxel(ff_add(rel, ff_mul(a_hi, dp.d[k])), dp.delta[k], b.n[k], ie, qe)) return false;
    s.v[k] = dp.v[k];
    s.idx[k] = i;
    s.f[k] = fminf(fmaxf(q - (float)i, 0.f), 1.f);
    s.cross[k] = ie > i ? ie - i : i - ie;
  }
  return true;
}

// Walk one clipped ray and add the integral of the C channels to acc (in cm times the field unit).
template <int kC, bool kCompensated>
__device__ __forceinline__ void ray_walk(const Box& b, const Setup<float>& s, const float* __restrict__ vol, int C,
                                         float* acc) {
  const int nC = kC > 0 ? kC : C;
  float comp_acc[kC > 0 ? kC : kMaxChannels];
  if (kCompensated)
    for (int c = 0; c < nC; ++c) comp_acc[c] = 0.f;
  int ix = s.idx[0], iy = s.idx[1], iz = s.idx[2];
  float fx = s.f[0], fy = s.f[1], fz = s.f[2];
  const float vx = s.v[0], vy = s.v[1], vz = s.v[2];
  const float ivx = vx != 0.f ? 1.f / fabsf(vx) : INFINITY;
  const float ivy = vy != 0.f ? 1.f / fabsf(vy) : INFINITY;
  const float ivz = vz != 0.f ? 1.f / fabsf(vz) : INFINITY;
  const int stx = vx > 0.f ? 1 : -1, sty = vy > 0.f ? 1 : -1, stz = vz > 0.f ? 1 : -1;
  int cx = s.cross[0], cy = s.cross[1], cz = s.cross[2];  // crossings left along each axis
  float t = 0.f, t_comp = 0.f;  // travelled distance, Kahan-compensated
  const int max_steps = b.n[0] + b.n[1] + b.n[2] + 3;
  for (int step = 0; step < max_steps; ++step) {
    const float dx = cx > 0 ? (vx > 0.f ? 1.f - fx : fx) * ivx : INFINITY;
    const float dy = cy > 0 ? (vy > 0.f ? 1.f - fy : fy) * ivy : INFINITY;
    const float dz = cz > 0 ? (vz > 0.f ? 1.f - fz : fz) * ivz : INFINITY;
    int axis = 0;
    float dt = dx;
    if (dy < dt) { dt = dy; axis = 1; }
    if (dz < dt) { dt = dz; axis = 2; }
    const float remaining = (s.total - t) + t_comp;
    const bool last = dt >= remaining;
    if (last) dt = fmaxf(remaining, 0.f);
    const float* vox = vol + ((int64_t)(iy * b.n[0] + ix) * b.n[2] + iz) * nC;
    if (kC == 8 || kC == 4) {
#pragma unroll
      for (int c = 0; c < (kC > 0 ? kC : 1); c += 4) {
        const float4 w = __ldg(reinterpret_cast<const float4*>(vox + c));
        if (kCompensated) {
          const float vals[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float y = dt * vals[q] - comp_acc[c + q];
            const float tt = acc[c + q] + y;
            comp_acc[c + q] = (tt - acc[c + q]) - y;
            acc[c + q] = tt;
          }
        } else {
          acc[c] = fmaf(dt, w.x, acc[c]);
          acc[c + 1] = fmaf(dt, w.y, acc[c + 1]);
          acc[c + 2] = fmaf(dt, w.z, acc[c + 2]);
          acc[c + 3] = fmaf(dt, w.w, acc[c + 3]);
        }
      }
    } else {
      for (int c = 0; c < nC; ++c) {
        const float w = __ldg(vox + c);
        if (kCompensated) {
          const float y = dt * w - comp_acc[c];
          const float tt = acc[c] + y;
          comp_acc[c] = (tt - acc[c]) - y;
          acc[c] = tt;
        } else {
          acc[c] = fmaf(dt, w, acc[c]);
        }
      }
    }
    if (last) break;
    {  // t += dt, compensated
      const float y = dt - t_comp;
      const float tt = t + y;
      t_comp = (tt - t) - y;
      t = tt;
    }
    fx = fminf(fmaxf(fmaf(dt, vx, fx), 0.f), 1.f);
    fy = fminf(fmaxf(fmaf(dt, vy, fy), 0.f), 1.f);
    fz = fminf(fmaxf(fmaf(dt, vz, fz), 0.f), 1.f);
    if (axis == 0) {
      ix += stx;
      --cx;
      fx = stx > 0 ? 0.f : 1.f;
      if (ix < 0 || ix >= b.n[0]) break;
    } else if (axis == 1) {
      iy += sty;
      --cy;
      fy = sty > 0 ? 0.f : 1.f;
      if (iy < 0 || iy >= b.n[1]) break;
    } else {
      iz += stz;
      --cz;
      fz = stz > 0 ? 0.f : 1.f;
      if (iz < 0 || iz >= b.n[2]) break;
    }
  }
}

// ray_walk of one channel without compensation (the oblique projection), four steps at a time: the walk's geometry
// never waits for a load, so the voxels and lengths of four steps are found first, their four gathers issued
// together and the products summed in step order (the same sums as ray_walk).
__device__ __forceinline__ float ray_walk_one_channel(const Box& b, const Setup<float>& s,
                                                      const float* __restrict__ vol) {
  float acc = 0.f;
  int ix = s.idx[0], iy = s.idx[1], iz = s.idx[2];
  float fx = s.f[0], fy = s.f[1], fz = s.f[2];
  const float vx = s.v[0], vy = s.v[1], vz = s.v[2];
  const float ivx = vx != 0.f ? 1.f / fabsf(vx) : INFINITY;
  const float ivy = vy != 0.f ? 1.f / fabsf(vy) : INFINITY;
  const float ivz = vz != 0.f ? 1.f / fabsf(vz) : INFINITY;
  const int stx = vx > 0.f ? 1 : -1, sty = vy > 0.f ? 1 : -1, stz = vz > 0.f ? 1 : -1;
  int cx = s.cross[0], cy = s.cross[1], cz = s.cross[2];  // crossings left along each axis
  float t = 0.f, t_comp = 0.f;  // travelled distance, Kahan-compensated
  const int max_steps = b.n[0] + b.n[1] + b.n[2] + 3;
  int step = 0;
  bool done = false;
  while (!done) {
    int64_t at[4];
    float len[4];
    int n = 0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (done || step >= max_steps) {
        done = true;
        continue;
      }
      ++step;
      const float dx = cx > 0 ? (vx > 0.f ? 1.f - fx : fx) * ivx : INFINITY;
      const float dy = cy > 0 ? (vy > 0.f ? 1.f - fy : fy) * ivy : INFINITY;
      const float dz = cz > 0 ? (vz > 0.f ? 1.f - fz : fz) * ivz : INFINITY;
      int axis = 0;
      float dt = dx;
      if (dy < dt) { dt = dy; axis = 1; }
      if (dz < dt) { dt = dz; axis = 2; }
      const float remaining = (s.total - t) + t_comp;
      const bool last = dt >= remaining;
      if (last) dt = fmaxf(remaining, 0.f);
      at[u] = (int64_t)(iy * b.n[0] + ix) * b.n[2] + iz;
      len[u] = dt;
      n = u + 1;
      if (last) {
        done = true;
        continue;
      }
      {  // t += dt, compensated
        const float y = dt - t_comp;
        const float tt = t + y;
        t_comp = (tt - t) - y;
        t = tt;
      }
      fx = fminf(fmaxf(fmaf(dt, vx, fx), 0.f), 1.f);
      fy = fminf(fmaxf(fmaf(dt, vy, fy), 0.f), 1.f);
      fz = fminf(fmaxf(fmaf(dt, vz, fz), 0.f), 1.f);
      if (axis == 0) {
        ix += stx;
        --cx;
        fx = stx > 0 ? 0.f : 1.f;
        if (ix < 0 || ix >= b.n[0]) done = true;
      } else if (axis == 1) {
        iy += sty;
        --cy;
        fy = sty > 0 ? 0.f : 1.f;
        if (iy < 0 || iy >= b.n[1]) done = true;
      } else {
        iz += stz;
        --cz;
        fz = stz > 0 ? 0.f : 1.f;
        if (iz < 0 || iz >= b.n[2]) done = true;
      }
    }
    float q[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) q[u] = u < n ? __ldg(vol + at[u]) : 0.f;
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (u < n) acc = fmaf(len[u], q[u], acc);
  }
  return acc;
}

template <int kC, bool kCompensated, typename T>
__device__ __forceinline__ void integrate(const Box& b, const T p0[3], const T p1[3], const float* vol, int C,
                                          float* acc) {
  const Setup<T> st = ray_setup<T>(b, p0, p1);
  if (!st.hit) return;
  Setup<float> s;
  s.hit = true;
  s.total = st.total;
  for (int a = 0; a < 3; ++a) {
    s.v[a] = st.v[a];
    s.idx[a] = st.idx[a];
    s.f[a] = st.f[a];
    s.cross[a] = st.cross[a];
  }
  ray_walk<kC, kCompensated>(b, s, vol, C, acc);
}

// ---- generic segments ----------------------------------------------------------------------------------------
template <int kC>
__global__ void __launch_bounds__(kThreads) segments_kernel(Box b, const float* __restrict__ vol, int C,
                                                            const float* __restrict__ starts,
                                                            const float* __restrict__ ends, int64_t R,
                                                            float* __restrict__ out) {
  const int64_t r = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (r >= R) return;
  double p0[3], p1[3];
  for (int a = 0; a < 3; ++a) {
    p0[a] = starts[3 * r + a];
    p1[a] = ends[3 * r + a];
  }
  float acc[kC > 0 ? kC : kMaxChannels];
  const int nC = kC > 0 ? kC : C;
  for (int c = 0; c < nC; ++c) acc[c] = 0.f;
  integrate<kC, true, double>(b, p0, p1, vol, C, acc);
  for (int c = 0; c < nC; ++c) out[(int64_t)c * R + r] = acc[c];
}

// ---- from a source point to points (explicit float64 points, or the centres of a point grid) ----------------
template <int kC>
__global__ void __launch_bounds__(kThreads) from_source_kernel(Box b, const float* __restrict__ vol, int C, double sx,
                                                               double sy, double sz, const double* __restrict__ pts,
                                                               const double* __restrict__ ax_x,
                                                               const double* __restrict__ ax_y,
                                                               const double* __restrict__ ax_z, int gc, int gs,
                                                               int64_t P, float* __restrict__ out) {
  const int64_t r = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (r >= P) return;
  double p1[3];
  if (pts != nullptr) {
    p1[0] = pts[3 * r];
    p1[1] = pts[3 * r + 1];
    p1[2] = pts[3 * r + 2];
  } else {  // flat index (row * cols + col) * slices + slice of the point grid
    const int64_t row = r / ((int64_t)gc * gs);
    const int64_t rem = r - row * (int64_t)gc * gs;
    const int64_t col = rem / gs;
    p1[0] = ax_x[col];
    p1[1] = ax_y[row];
    p1[2] = ax_z[rem - col * gs];
  }
  const double p0[3] = {sx, sy, sz};
  float acc[kC > 0 ? kC : kMaxChannels];
  const int nC = kC > 0 ? kC : C;
  for (int c = 0; c < nC; ++c) acc[c] = 0.f;
  integrate<kC, true, double>(b, p0, p1, vol, C, acc);
  for (int c = 0; c < nC; ++c) out[(int64_t)c * P + r] = acc[c];
}

// ---- downstream: from every voxel centre along each direction to the panel ----------------------------------
// The detector surface the downstream rays stop at, in float (rounded on the host, once).
struct Panel {
  int curved;
  float center[3], normal[3];  // flat panel: a point of the plane and its normal (toward the source)
  float source[3], radius2;    // curved panel: the cylinder about the vertical axis through the source
};

__device__ __forceinline__ float panel_distance(const Panel& p, const float r[3], const float w[3]) {
  if (!p.curved) {
    const float den = w[0] * p.normal[0] + w[1] * p.normal[1] + w[2] * p.normal[2];
    const float num = (p.center[0] - r[0]) * p.normal[0] + (p.center[1] - r[1]) * p.normal[1] +
                      (p.center[2] - r[2]) * p.normal[2];
    return num / den;
  }
  const float dx = r[0] - p.source[0], dy = r[1] - p.source[1];
  const float a = w[0] * w[0] + w[1] * w[1];
  const float bb = dx * w[0] + dy * w[1];
  const float c = dx * dx + dy * dy - p.radius2;
  const float disc = bb * bb - a * c;
  const float root = sqrtf(fmaxf(disc, 0.f));
  const bool pos = bb >= 0.f;
  const float den = pos ? bb + root : (a > 0.f ? a : 1.f);
  const float num = pos ? -c : root - bb;
  if (!(a > 0.f) || !(disc >= 0.f) || den == 0.f) return INFINITY;
  return num / den;
}

template <int kC>
__global__ void __launch_bounds__(kThreads) downstream_kernel(Box b, const float* __restrict__ vol, int C,
                                                              const float* __restrict__ omegas,
                                                              const uint8_t* __restrict__ toward, Panel panel,
                                                              float diagonal, int64_t V, float* __restrict__ out,
                                                              int64_t os_k, int64_t os_c, int64_t os_v) {
  const int64_t v = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const int k = blockIdx.y;
  if (v >= V) return;
  const int nC = kC > 0 ? kC : C;
  float* o = out + (int64_t)k * os_k + v * os_v;
  if (toward != nullptr && toward[k] == 0) {
    for (int c = 0; c < nC; ++c) o[(int64_t)c * os_c] = INFINITY;
    return;
  }
  const int64_t nzx = (int64_t)b.n[0] * b.n[2];
  const int iy = (int)(v / nzx);
  const int64_t rem = v - (int64_t)iy * nzx;
  const int ix = (int)(rem / b.n[2]);
  const int iz = (int)(rem - (int64_t)ix * b.n[2]);
  const float r[3] = {voxel_centre(b, 0, ix), voxel_centre(b, 1, iy), voxel_centre(b, 2, iz)};
  const float w[3] = {omegas[3 * k], omegas[3 * k + 1], omegas[3 * k + 2]};
  float t = panel_distance(panel, r, w);
  t = fminf(fmaxf(t, 0.f), diagonal);
  const float p1[3] = {r[0] + t * w[0], r[1] + t * w[1], r[2] + t * w[2]};
  float acc[kC > 0 ? kC : kMaxChannels];
  for (int c = 0; c < nC; ++c) acc[c] = 0.f;
  integrate<kC, false, float>(b, r, p1, vol, C, acc);
  for (int c = 0; c < nC; ++c) o[(int64_t)c * os_c] = acc[c];
}

// ---- downstream on the lattice: one crossing sequence per direction ------------------------------------------
// Every downstream ray starts at a voxel centre, so along a direction all of them meet the voxel planes at the same
// distances from their start: the m-th crossing of axis a lies at (m + 1/2) delta_a / |omega_a|. The merged sequence
// of these crossings (distance, flat index step) is built once per direction in float64 (crossing_table_kernel), and
// a ray is then a walk down that table from its own voxel, up to the crossing at which it leaves the box or to the
// panel, whichever comes first: one broadcast shared-memory read, one gather and the channel FMAs per segment.
//
// Table of direction k, E = nx + ny + nz words per part: t[E] (float distance of crossing j from the start, +inf past
// the last), dv[E] (flat index step of crossing j), first[E] (entry of the m-th crossing of axis a at
// first[off_a + m], off = 0, nx, nx + ny).
__global__ void crossing_table_kernel(Box b, const float* __restrict__ omegas, int K, int32_t* __restrict__ table) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const int E = b.n[0] + b.n[1] + b.n[2];
  float* t = reinterpret_cast<float*>(table + (int64_t)k * 3 * E);
  int32_t* dv = table + (int64_t)k * 3 * E + E;
  int32_t* first = table + (int64_t)k * 3 * E + 2 * E;
  const int64_t stride[3] = {b.n[2], (int64_t)b.n[0] * b.n[2], 1};  // x: columns, y: rows, z: slices
  const int off[3] = {0, b.n[0], b.n[0] + b.n[1]};
  double step[3], next[3];
  int m[3] = {0, 0, 0};
  int32_t dir[3];
  for (int a = 0; a < 3; ++a) {
    const double w = omegas[3 * k + a];
    step[a] = w != 0.0 ? b.delta[a] / fabs(w) : INFINITY;
    next[a] = 0.5 * step[a];
    dir[a] = (int32_t)(w > 0.0 ? stride[a] : -stride[a]);
    for (int i = 0; i < b.n[a]; ++i) first[off[a] + i] = E;  // never reached along a parallel axis
  }
  for (int j = 0; j < E; ++j) {
    int a = 0;
    if (next[1] < next[a]) a = 1;
    if (next[2] < next[a]) a = 2;
    if (!(next[a] < INFINITY)) {
      t[j] = INFINITY;
      dv[j] = 0;
      continue;
    }
    t[j] = (float)next[a];
    dv[j] = dir[a];
    first[off[a] + m[a]] = j;
    ++m[a];
    next[a] = m[a] < b.n[a] ? (m[a] + 0.5) * step[a] : INFINITY;
  }
}

template <int kC>
__global__ void __launch_bounds__(kThreads) downstream_lattice_kernel(Box b, const float* __restrict__ vol, int C,
                                                                      const float* __restrict__ omegas,
                                                                      const uint8_t* __restrict__ toward, Panel panel,
                                                                      float diagonal, int64_t V,
                                                                      const int32_t* __restrict__ table,
                                                                      float* __restrict__ out, int64_t os_k,
                                                                      int64_t os_c, int64_t os_v) {
  // [4E] words of this direction: the steps (segment length, flat index step) as int2 [E] (E rounded up to even, so
  // that two steps are one 16-byte load), then t [E] and first [E]
  extern __shared__ int4 s_tab4[];
  const int k = blockIdx.y;
  const int E = b.n[0] + b.n[1] + b.n[2];
  const int E2 = (E + 1) & ~1;
  int2* s_step = reinterpret_cast<int2*>(s_tab4);
  int32_t* s_words = reinterpret_cast<int32_t*>(s_tab4) + 2 * E2;
  const int32_t* src = table + (int64_t)k * 3 * E;
  for (int i = threadIdx.x; i < E; i += kThreads) {
    // the length of the segment that ends at crossing i: t[i] - t[i - 1] (t[-1] = 0), as the walk forms it
    const float tj = __int_as_float(src[i]), tp = i > 0 ? __int_as_float(src[i - 1]) : 0.f;
    s_step[i] = make_int2(__float_as_int(tj - tp), src[E + i]);
    s_words[i] = src[i];
    s_words[E + i] = src[2 * E + i];
  }
  if (threadIdx.x == 0 && E2 > E) s_step[E] = make_int2(0, 0);
  __syncthreads();
  const float* t_cross = reinterpret_cast<const float*>(s_words);
  const int32_t* first = s_words + E;
  const int64_t v = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (v >= V) return;
  const int nC = kC > 0 ? kC : C;
  float* o = out + (int64_t)k * os_k + v * os_v;
  if (toward != nullptr && toward[k] == 0) {
    for (int c = 0; c < nC; ++c) o[(int64_t)c * os_c] = INFINITY;
    return;
  }
  const int64_t nzx = (int64_t)b.n[0] * b.n[2];
  const int iy = (int)(v / nzx);
  const int64_t rem = v - (int64_t)iy * nzx;
  const int ix = (int)(rem / b.n[2]);
  const int iz = (int)(rem - (int64_t)ix * b.n[2]);
  const float r[3] = {voxel_centre(b, 0, ix), voxel_centre(b, 1, iy), voxel_centre(b, 2, iz)};
  const float w[3] = {omegas[3 * k], omegas[3 * k + 1], omegas[3 * k + 2]};
  float t_end = fminf(fmaxf(panel_distance(panel, r, w), 0.f), diagonal);
  // the crossing that leaves the box: along axis a after the voxels left between i_a and the face ahead
  const int idx[3] = {ix, iy, iz};
  const int off[3] = {0, b.n[0], b.n[0] + b.n[1]};
  int exit_j = E;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (w[a] == 0.f) continue;
    const int left = w[a] > 0.f ? b.n[a] - 1 - idx[a] : idx[a];
    exit_j = min(exit_j, first[off[a] + left]);
  }
  if (exit_j < E) t_end = fminf(t_end, t_cross[exit_j]);
  // the segments ending at crossings 0 .. J - 1 are whole (t_j <= t_end); the one ending at crossing J, when the ray
  // ends before its exit crossing, is cut at t_end (the first j with t_j > t_end, by bisection of the sorted table)
  int J = min(exit_j + 1, E);
  bool cut = false;
  if (J > 0 && t_cross[J - 1] > t_end) {
    int lo = 0, hi = J - 1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (t_cross[mid] > t_end) hi = mid;
      else lo = mid + 1;
    }
    J = lo;
    cut = true;
  }
  float acc[kC > 0 ? kC : kMaxChannels];
  for (int c = 0; c < nC; ++c) acc[c] = 0.f;
  int cur = (int)v;
  int j = 0;
  if (kC == 2) {
    // four segments at a time: the four gathers are issued before their sums (the crossing table gives every step's
    // voxel in advance)
    for (; j + 4 <= J; j += 4) {
      const int4 e01 = s_tab4[j >> 1], e23 = s_tab4[(j >> 1) + 1];  // steps j .. j + 3 (j even)
      const int c1 = cur + e01.y, c2 = c1 + e01.w, c3 = c2 + e23.y;
      const float2 q0 = __ldg(reinterpret_cast<const float2*>(vol) + cur);
      const float2 q1 = __ldg(reinterpret_cast<const float2*>(vol) + c1);
      const float2 q2 = __ldg(reinterpret_cast<const float2*>(vol) + c2);
      const float2 q3 = __ldg(reinterpret_cast<const float2*>(vol) + c3);
      const float s0 = __int_as_float(e01.x), s1 = __int_as_float(e01.z), s2 = __int_as_float(e23.x),
                  s3 = __int_as_float(e23.z);
      acc[0] = fmaf(s0, q0.x, acc[0]);
      acc[kC > 1 ? 1 : 0] = fmaf(s0, q0.y, acc[kC > 1 ? 1 : 0]);
      acc[0] = fmaf(s1, q1.x, acc[0]);
      acc[kC > 1 ? 1 : 0] = fmaf(s1, q1.y, acc[kC > 1 ? 1 : 0]);
      acc[0] = fmaf(s2, q2.x, acc[0]);
      acc[kC > 1 ? 1 : 0] = fmaf(s2, q2.y, acc[kC > 1 ? 1 : 0]);
      acc[0] = fmaf(s3, q3.x, acc[0]);
      acc[kC > 1 ? 1 : 0] = fmaf(s3, q3.y, acc[kC > 1 ? 1 : 0]);
      cur = c3 + e23.w;
    }
  }
  // the remaining whole segments, then the cut one (step j == J)
  for (; j <= J; ++j) {
    float seg;
    if (j < J) {
      seg = __int_as_float(s_step[j].x);
    } else {
      const float prev = j > 0 ? t_cross[j - 1] : 0.f;
      if (!cut || !(prev < t_end)) break;
      seg = t_end - prev;
    }
    const float* vox = vol + (int64_t)cur * nC;
    if (kC == 8 || kC == 4) {
#pragma unroll
      for (int c = 0; c < (kC > 0 ? kC : 1); c += 4) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(vox + c));
        acc[c] = fmaf(seg, q.x, acc[c]);
        acc[c + 1] = fmaf(seg, q.y, acc[c + 1]);
        acc[c + 2] = fmaf(seg, q.z, acc[c + 2]);
        acc[c + 3] = fmaf(seg, q.w, acc[c + 3]);
      }
    } else if (kC == 2) {
      const float2 q = __ldg(reinterpret_cast<const float2*>(vox));
      acc[0] = fmaf(seg, q.x, acc[0]);
      acc[kC > 1 ? 1 : 0] = fmaf(seg, q.y, acc[kC > 1 ? 1 : 0]);
    } else {
      for (int c = 0; c < nC; ++c) acc[c] = fmaf(seg, __ldg(vox + c), acc[c]);
    }
    if (j < J) cur += s_step[j].y;
  }
  if ((kC == 8 || kC == 4) && os_c == 1 && os_v == nC) {  // voxel-major out: the channels of a ray in float4s
#pragma unroll
    for (int c = 0; c < (kC > 0 ? kC : 1); c += 4)
      *reinterpret_cast<float4*>(o + c) = make_float4(acc[c], acc[c + 1], acc[c + 2], acc[c + 3]);
  } else {
    for (int c = 0; c < nC; ++c) o[(int64_t)c * os_c] = acc[c];
  }
}

// ---- oblique: through every pixel centre along each direction, clipped to the box on both sides --------------
// The set-up starts from the float64 pixel centres, as the reference forms these lines, in float pairs
// (ray_setup_pair), and in float64 for a line within its tolerances of a face, an edge or a voxel plane: a line that
// grazes a face of the box is inside or outside exactly as in float64, where a float32 rounding of the pixel centre
// could move it onto the face and integrate a whole slice.
// The float64 constants of direction k and their float pairs (the divisions and the square root of the set-up).
__device__ __forceinline__ void oblique_direction(const Box& b, const float* __restrict__ omegas, int k, double cx,
                                                  double cy, double cz, double half, DirConst& dc, DirPair& dp) {
  dc.w[0] = omegas[3 * k];
  dc.w[1] = omegas[3 * k + 1];
  dc.w[2] = omegas[3 * k + 2];
  const double sq = add_rn(add_rn(mul_rn(dc.w[0], dc.w[0]), mul_rn(dc.w[1], dc.w[1])), mul_rn(dc.w[2], dc.w[2]));
  dc.h = half / sqrt(sq);
  dc.inv_w2 = 1.0 / sq;
  for (int a = 0; a < 3; ++a) {
    dc.d[a] = mul_rn(2.0 * dc.h, dc.w[a]);
    dc.inv_d[a] = dc.d[a] != 0 ? 1.0 / dc.d[a] : 0.0;
    dc.hi[a] = add_rn(b.lo[a], mul_rn(b.delta[a], (double)b.n[a]));
  }
  const double c[3] = {cx, cy, cz};
  make_dir_pair(b, dc, c, dp);
}

// One thread per direction: the constants every block of that direction reads (float64 on this GPU runs at a small
// fraction of float32, and a block per 128 pixels would otherwise repeat them hundreds of times per direction)
__global__ void oblique_setup_kernel(Box b, const float* __restrict__ omegas, int K, double cx, double cy, double cz,
                                     double half, DirConst* __restrict__ dcs, DirPair* __restrict__ dps) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  DirConst dc;
  DirPair dp;
  oblique_direction(b, omegas, k, cx, cy, cz, half, dc, dp);
  dcs[k] = dc;
  dps[k] = dp;
}

template <int kC>
__global__ void __launch_bounds__(kThreads) oblique_kernel(Box b, const float* __restrict__ vol, int C,
                                                           int64_t field_stride, const float* __restrict__ omegas,
                                                           const double* __restrict__ pixels, int64_t P, double cx,
                                                           double cy, double cz, double half,
                                                           float* __restrict__ out, int64_t os_k, int64_t os_c,
                                                           int64_t os_r, int64_t os_col, int64_t cols,
                                                           const DirConst* __restrict__ dcs,
                                                           const DirPair* __restrict__ dps) {
  const int64_t p = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const int k = blockIdx.y;
  // the direction's constants: from the set-up kernel's table when given, else formed once per block by thread 0
  __shared__ DirConst s_dc;
  __shared__ DirPair s_dp;
  if (dcs != nullptr) {
    constexpr int nc = sizeof(DirConst) / 4, np = sizeof(DirPair) / 4;
    static_assert(sizeof(DirConst) % 4 == 0 && sizeof(DirPair) % 4 == 0, "4-byte words");
    for (int i = threadIdx.x; i < nc + np; i += kThreads) {
      if (i < nc) reinterpret_cast<int*>(&s_dc)[i] = reinterpret_cast<const int*>(dcs + k)[i];
      else reinterpret_cast<int*>(&s_dp)[i - nc] = reinterpret_cast<const int*>(dps + k)[i - nc];
    }
  } else if (threadIdx.x == 0) {
    oblique_direction(b, omegas, k, cx, cy, cz, half, s_dc, s_dp);
  }
  __syncthreads();
  if (p >= P) return;
  const DirConst& dc = s_dc;
  const double px = pixels[3 * p], py = pixels[3 * p + 1], pz = pixels[3 * p + 2];
  const int nC = kC > 0 ? kC : C;
  float acc[kC > 0 ? kC : kMaxChannels];
  for (int c = 0; c < nC; ++c) acc[c] = 0.f;
  Setup<float> st;
  if (!ray_setup_pair(b, s_dp, px, py, pz, st)) {
    // the entry point of ray_tracing.py:588-595 in float64, its exit point the entry plus the direction's segment
    const double dot = add_rn(add_rn(mul_rn(cx - px, dc.w[0]), mul_rn(cy - py, dc.w[1])), mul_rn(cz - pz, dc.w[2]));
    const double tm = mul_rn(dot, dc.inv_w2) - dc.h;
    const double a[3] = {add_rn(px, mul_rn(tm, dc.w[0])), add_rn(py, mul_rn(tm, dc.w[1])),
                         add_rn(pz, mul_rn(tm, dc.w[2]))};
    st = ray_setup_dir(b, a, dc);
  }
  if (st.hit) {
    if (kC == 1) acc[0] = ray_walk_one_channel(b, st, vol + (int64_t)k * field_stride);
    else ray_walk<kC, false>(b, st, vol + (int64_t)k * field_stride, C, acc);
  }
  const int64_t row = p / cols;
  float* o = out + (int64_t)k * os_k + row * os_r + (p - row * cols) * os_col;
  for (int c = 0; c < nC; ++c) o[(int64_t)c * os_c] = acc[c];
}

int check_common(const float* vol, int64_t C, const double* box, const int64_t* dims, const void* out) {
  CITRUS_REQUIRE(vol && box && dims && out, "ray tracing: null pointer argument");
  CITRUS_REQUIRE(C >= 1 && C <= kMaxChannels, "ray tracing: %lld channels outside [1, %d]", (long long)C,
                 kMaxChannels);
  CITRUS_REQUIRE(dims[0] >= 1 && dims[1] >= 1 && dims[2] >= 1 && dims[0] * dims[1] * dims[2] < (1ll << 31),
                 "ray tracing: bad grid dimensions");
  CITRUS_REQUIRE(box[3] > 0 && box[4] > 0 && box[5] > 0, "ray tracing: voxel sizes must be positive");
  if (C % 4 == 0) CITRUS_REQUIRE(((uintptr_t)vol % 16) == 0, "ray tracing: volume must be 16-byte aligned");
  return CITRUS_OK;
}

#define CITRUS_CHANNEL_DISPATCH(C, KERNEL, GRID, STREAM, ...)                            \
  switch (C) {                                                                            \
    case 1: KERNEL<1><<<GRID, kThreads, 0, STREAM>>>(__VA_ARGS__); break;                \
    case 2: KERNEL<2><<<GRID, kThreads, 0, STREAM>>>(__VA_ARGS__); break;                \
    case 4: KERNEL<4><<<GRID, kThreads, 0, STREAM>>>(__VA_ARGS__); break;                \
    case 8: KERNEL<8><<<GRID, kThreads, 0, STREAM>>>(__VA_ARGS__); break;                \
    default: KERNEL<0><<<GRID, kThreads, 0, STREAM>>>(__VA_ARGS__); break;               \
  }                                                                                       \
  note_launches();

}  // namespace
}  // namespace citrus

using namespace citrus;

extern "C" int citrus_line_integrals(const float* volume, int64_t channels, const double* box, const int64_t* dims,
                                     const float* starts, const float* ends, int64_t num_rays, float* out,
                                     void* stream) {
  int status = check_common(volume, channels, box, dims, out);
  if (status) return status;
  CITRUS_REQUIRE(num_rays >= 0 && (num_rays == 0 || (starts && ends)), "citrus_line_integrals: bad rays");
  if (num_rays == 0) return CITRUS_OK;
  const Box b = make_box(box, dims);
  const int C = (int)channels;
  dim3 grid((unsigned)cdiv(num_rays, kThreads));
  CITRUS_CHANNEL_DISPATCH(C, segments_kernel, grid, as_stream(stream), b, volume, C, starts, ends, num_rays, out)
  return launch_status("citrus_line_integrals");
}

extern "C" int citrus_trace_from_source(const float* volume, int64_t channels, const double* box, const int64_t* dims,
                                        const double* source, const double* points, const double* axis_x,
                                        const double* axis_y, const double* axis_z, const int64_t* point_dims,
                                        int64_t num_points, float* out, void* stream) {
  int status = check_common(volume, channels, box, dims, out);
  if (status) return status;
  CITRUS_REQUIRE(source != nullptr, "citrus_trace_from_source: null source");
  CITRUS_REQUIRE(points != nullptr || (axis_x && axis_y && axis_z && point_dims),
                 "citrus_trace_from_source: give explicit points or the axes of a point grid");
  int gc = 1, gs = 1;
  if (points == nullptr) {
    CITRUS_REQUIRE(point_dims[0] * point_dims[1] * point_dims[2] == num_points,
                   "citrus_trace_from_source: point grid dims disagree with num_points");
    gc = (int)point_dims[1];
    gs = (int)point_dims[2];
  }
  if (num_points == 0) return CITRUS_OK;
  const Box b = make_box(box, dims);
  const int C = (int)channels;
  dim3 grid((unsigned)cdiv(num_points, kThreads));
  CITRUS_CHANNEL_DISPATCH(C, from_source_kernel, grid, as_stream(stream), b, volume, C, source[0], source[1],
                          source[2], points, axis_x, axis_y, axis_z, gc, gs, num_points, out)
  return launch_status("citrus_trace_from_source");
}

namespace citrus {
namespace {
int downstream(const float* volume, int64_t channels, const double* box, const int64_t* dims, const float* omegas,
               const uint8_t* toward, int64_t num_directions, const double* panel, double diagonal, float* out,
               int64_t os_k, int64_t os_c, int64_t os_v, int32_t* crossings, int64_t crossings_words, bool build,
               void* stream);
}  // namespace
}  // namespace citrus

extern "C" int citrus_crossing_tables(const double* box, const int64_t* dims, const float* omegas,
                                      int64_t num_directions, int32_t* crossings, int64_t crossings_words,
                                      void* stream) {
  CITRUS_REQUIRE(box && dims && omegas && crossings, "citrus_crossing_tables: null pointer argument");
  CITRUS_REQUIRE(num_directions >= 0 && dims[0] >= 1 && dims[1] >= 1 && dims[2] >= 1,
                 "citrus_crossing_tables: bad sizes");
  const int64_t E = dims[0] + dims[1] + dims[2];
  CITRUS_REQUIRE(crossings_words >= 3 * E * num_directions,
                 "citrus_crossing_tables: the table holds %lld words, needs %lld", (long long)crossings_words,
                 (long long)(3 * E * num_directions));
  if (num_directions == 0) return CITRUS_OK;
  const Box b = make_box(box, dims);
  crossing_table_kernel<<<(unsigned)cdiv(num_directions, 64), 64, 0, as_stream(stream)>>>(
      b, omegas, (int)num_directions, crossings);
  note_launches();
  return launch_status("citrus_crossing_tables");
}

extern "C" int citrus_downstream_cumulative_tables(const float* volume, int64_t channels, const double* box,
                                                   const int64_t* dims, const float* omegas, const uint8_t* toward,
                                                   int64_t num_directions, const double* panel, double diagonal,
                                                   float* out, int64_t os_k, int64_t os_c, int64_t os_v,
                                                   const int32_t* crossings, int64_t crossings_words, void* stream) {
  CITRUS_REQUIRE(crossings != nullptr, "citrus_downstream_cumulative_tables: null crossing tables");
  return downstream(volume, channels, box, dims, omegas, toward, num_directions, panel, diagonal, out, os_k, os_c,
                    os_v, const_cast<int32_t*>(crossings), crossings_words, false, stream);
}

extern "C" int citrus_downstream_cumulative(const float* volume, int64_t channels, const double* box,
                                            const int64_t* dims, const float* omegas, const uint8_t* toward,
                                            int64_t num_directions, const double* panel, double diagonal,
                                            float* out, int64_t os_k, int64_t os_c, int64_t os_v, int32_t* crossings,
                                            int64_t crossings_words, void* stream) {
  return downstream(volume, channels, box, dims, omegas, toward, num_directions, panel, diagonal, out, os_k, os_c,
                    os_v, crossings, crossings_words, true, stream);
}

namespace citrus {
namespace {
int downstream(const float* volume, int64_t channels, const double* box, const int64_t* dims, const float* omegas,
               const uint8_t* toward, int64_t num_directions, const double* panel, double diagonal, float* out,
               int64_t os_k, int64_t os_c, int64_t os_v, int32_t* crossings, int64_t crossings_words, bool build,
               void* stream) {
  int status = check_common(volume, channels, box, dims, out);
  if (status) return status;
  CITRUS_REQUIRE(omegas && panel, "citrus_downstream_cumulative: null directions or panel");
  CITRUS_REQUIRE(num_directions >= 0 && num_directions <= 65535, "citrus_downstream_cumulative: bad direction count");
  if (num_directions == 0) return CITRUS_OK;
  Panel p;
  p.curved = panel[0] != 0.0;
  for (int a = 0; a < 3; ++a) {
    p.center[a] = (float)panel[1 + a];
    p.normal[a] = (float)panel[4 + a];
    p.source[a] = (float)panel[7 + a];
  }
  p.radius2 = (float)(panel[10] * panel[10]);
  const Box b = make_box(box, dims);
  const int64_t V = dims[0] * dims[1] * dims[2];
  const int C = (int)channels;
  dim3 grid((unsigned)cdiv(V, kThreads), (unsigned)num_directions);
  cudaStream_t s = as_stream(stream);
  if (crossings == nullptr) {
    CITRUS_CHANNEL_DISPATCH(C, downstream_kernel, grid, s, b, volume, C, omegas, toward, p, (float)diagonal, V, out,
                            os_k, os_c, os_v)
    return launch_status("citrus_downstream_cumulative");
  }
  const int64_t E = dims[0] + dims[1] + dims[2];
  CITRUS_REQUIRE(crossings_words >= 3 * E * num_directions,
                 "citrus_downstream_cumulative: crossing table holds %lld words, needs %lld",
                 (long long)crossings_words, (long long)(3 * E * num_directions));
  CITRUS_REQUIRE(4 * E * 4 <= 48 * 1024, "citrus_downstream_cumulative: grid too large for the crossing table");
  CITRUS_REQUIRE(V * (int64_t)channels < (1ll << 31), "citrus_downstream_cumulative: volume too large");
  if (C % 2 == 0) CITRUS_REQUIRE(((uintptr_t)volume % 16) == 0, "citrus_downstream_cumulative: unaligned volume");
  if (C % 4 == 0 && os_c == 1 && os_v == C)
    CITRUS_REQUIRE(((uintptr_t)out % 16) == 0 && os_k % 4 == 0, "citrus_downstream_cumulative: unaligned out");
  if (build) {  // else the caller's tables of these directions (citrus_crossing_tables)
    crossing_table_kernel<<<(unsigned)cdiv(num_directions, 64), 64, 0, s>>>(b, omegas, (int)num_directions,
                                                                           crossings);
    note_launches();
  }
  const size_t smem = (size_t)(2 * ((E + 1) & ~1) + 2 * E) * sizeof(int32_t);
#define CITRUS_LATTICE(KC)                                                                                        \
  downstream_lattice_kernel<KC><<<grid, kThreads, smem, s>>>(b, volume, C, omegas, toward, p, (float)diagonal, V, \
                                                            crossings, out, os_k, os_c, os_v)
  switch (C) {
    case 1: CITRUS_LATTICE(1); break;
    case 2: CITRUS_LATTICE(2); break;
    case 4: CITRUS_LATTICE(4); break;
    case 8: CITRUS_LATTICE(8); break;
    default: CITRUS_LATTICE(0); break;
  }
#undef CITRUS_LATTICE
  note_launches();
  return launch_status("citrus_downstream_cumulative");
}
}  // namespace
}  // namespace citrus

extern "C" int64_t citrus_oblique_scratch_bytes(int64_t num_directions) {
  return num_directions <= 0 ? 0 : num_directions * (int64_t)(sizeof(DirConst) + sizeof(DirPair)) + 16;
}

extern "C" int citrus_oblique_project_scratch(const float* field, int64_t channels, int64_t field_stride,
                                              const double* box, const int64_t* dims, const float* omegas,
                                              int64_t num_directions, const double* pixels, int64_t num_rows,
                                              int64_t num_cols, float* out, int64_t os_k, int64_t os_c, int64_t os_r,
                                              int64_t os_col, void* direction_scratch, int64_t scratch_bytes,
                                              void* stream) {
  int status = check_common(field, channels, box, dims, out);
  if (status) return status;
  CITRUS_REQUIRE(omegas && pixels, "citrus_oblique_project: null directions or pixels");
  CITRUS_REQUIRE(num_directions >= 0 && num_directions <= 65535 && num_rows >= 0 && num_cols >= 1,
                 "citrus_oblique_project: bad sizes");
  CITRUS_REQUIRE(direction_scratch == nullptr || scratch_bytes >= citrus_oblique_scratch_bytes(num_directions),
                 "citrus_oblique_project: the direction scratch holds %lld bytes, needs %lld",
                 (long long)scratch_bytes, (long long)citrus_oblique_scratch_bytes(num_directions));
  const int64_t num_pixels = num_rows * num_cols;
  if (num_directions == 0 || num_pixels == 0) return CITRUS_OK;
  const Box b = make_box(box, dims);
  double ext[3], center[3], diag2 = 0;
  for (int a = 0; a < 3; ++a) {
    ext[a] = b.delta[a] * b.n[a];
    center[a] = b.lo[a] + 0.5 * ext[a];
    diag2 += ext[a] * ext[a];
  }
  const double half = 0.5 * sqrt(diag2) * (1 + 1e-6) + 1e-6;
  const int C = (int)channels;
  DirConst* dcs = nullptr;
  DirPair* dps = nullptr;
  if (direction_scratch != nullptr) {  // 16-byte aligned tables: the constants of every direction, then their pairs
    const uintptr_t base = ((uintptr_t)direction_scratch + 15) & ~(uintptr_t)15;
    dcs = reinterpret_cast<DirConst*>(base);
    dps = reinterpret_cast<DirPair*>(base + num_directions * sizeof(DirConst));
    oblique_setup_kernel<<<(unsigned)cdiv(num_directions, 64), 64, 0, as_stream(stream)>>>(
        b, omegas, (int)num_directions, center[0], center[1], center[2], half, dcs, dps);
    note_launches();
  }
  dim3 grid((unsigned)cdiv(num_pixels, kThreads), (unsigned)num_directions);
  CITRUS_CHANNEL_DISPATCH(C, oblique_kernel, grid, as_stream(stream), b, field, C, field_stride, omegas, pixels,
                          num_pixels, center[0], center[1], center[2], half, out, os_k, os_c, os_r, os_col,
                          num_cols, dcs, dps)
  return launch_status("citrus_oblique_project");
}

extern "C" int citrus_oblique_project(const float* field, int64_t channels, int64_t field_stride, const double* box,
                                      const int64_t* dims, const float* omegas, int64_t num_directions,
                                      const double* pixels, int64_t num_rows, int64_t num_cols, float* out,
                                      int64_t os_k, int64_t os_c, int64_t os_r, int64_t os_col, void* stream) {
  return citrus_oblique_project_scratch(field, channels, field_stride, box, dims, omegas, num_directions, pixels,
                                        num_rows, num_cols, out, os_k, os_c, os_r, os_col, nullptr, 0, stream);
}
