// Linear-discontinuous discrete-ordinates sweep: the closed-form cell solve of every (entry, direction, group) of a
// diagonal wavefront plane, in place in the chunk's cell-major store [views, 8, Dc, N, 4G].
//
// The cell equations are those of citrus/scatter_solver/linear_discontinuous_cell.py:14-87 (right-hand sides from the
// source and the three upstream neighbours, then the closed-form 4 x 4 solve), evaluated term by term in float32: the
// coefficients of a lane with IEEE division, the per-view quotients as products with correctly rounded reciprocals.
// Two drivers share the lane body: one launch per plane (the reference's plan, sweep_kernels.py:265-290) and one
// persistent cooperative launch that walks all planes with a bounded grid barrier between them, so a whole chunk is a
// single launch.
#include "common.cuh"
#include <mutex>

namespace citrus {
namespace {

constexpr int kThreads = 256;

template <bool kCoherent>
__device__ __forceinline__ float4 load4(const float4* p) {
  if (kCoherent) return __ldcg(p);  // L2 only: written by other SMs this launch
  return *p;
}

// The view-independent part of one lane (entry e of the plane, direction d of the chunk, group g): the octant signs,
// the direction's c_a, every coefficient of the 4 x 4 solve that depends on c and the cell's attenuation only, and
// the float4 positions within one view's store of the cell and of its three upstream neighbours (upstream neighbours
// lie on the previous plane, already swept; kVacuum marks a vacuum face, which reads zeros). The views of a launch
// share it: a thread computes it once and solves the lane in every view.
constexpr uint32_t kVacuum = 0xffffffffu;

struct LaneCoef {
  float sx, sy, sz, cx, cy, cz;
  float k3x, k3y, k3z;  // 3 s_a c_a
  float rdx, rdy, rdz;  // 1 / d_a, d_a = 3 c_a + sum_{b != a} c_b + m
  float qsx, qsy, qsz;  // s_a c_a / d_a
  float rden;           // 1 / (sum_a c_a + m + 3 sum_a c_a q_a)
  uint32_t at, ax, ay, az;
};

// The lane of entry e, direction d and group g; every float4 position of a view is below 2^31 (checked on the host)
template <int kG>
__device__ __forceinline__ void lane_coef_edg(uint32_t e, uint32_t d, uint32_t g, LaneCoef& k,
                                              const float* __restrict__ mu, const float* __restrict__ c,
                                              const int* __restrict__ octant, const int* __restrict__ cell,
                                              const int* __restrict__ upstream, uint32_t N, int G_runtime,
                                              uint32_t Dc) {
  const uint32_t G = kG > 0 ? kG : G_runtime;
  const int o = __ldg(octant + e);
  const uint32_t n = __ldg(cell + e);
  const uint32_t ux = __ldg(upstream + 3 * e), uy = __ldg(upstream + 3 * e + 1), uz = __ldg(upstream + 3 * e + 2);
  const uint32_t od = (uint32_t)o * Dc + d;
  const float cx = __ldg(c + 3 * od), cy = __ldg(c + 3 * od + 1), cz = __ldg(c + 3 * od + 2);
  const float m = __ldg(mu + (size_t)n * G + g);
  const uint32_t base = od * N;
  k.at = (base + n) * G + g;
  k.ax = ux < N ? (base + ux) * G + g : kVacuum;
  k.ay = uy < N ? (base + uy) * G + g : kVacuum;
  k.az = uz < N ? (base + uz) * G + g : kVacuum;
  // every operation is rounded on its own (no multiply-add contraction), so every kernel computes the same bits
  const float sx = (o & 4) ? -1.f : 1.f, sy = (o & 2) ? -1.f : 1.f, sz = (o & 1) ? -1.f : 1.f;
  k.sx = sx, k.sy = sy, k.sz = sz, k.cx = cx, k.cy = cy, k.cz = cz;
  k.k3x = __fmul_rn(__fmul_rn(3.f, sx), cx);
  k.k3y = __fmul_rn(__fmul_rn(3.f, sy), cy);
  k.k3z = __fmul_rn(__fmul_rn(3.f, sz), cz);
  const float csum = __fadd_rn(__fadd_rn(cx, cy), cz);
  const float dx = __fadd_rn(__fadd_rn(__fmul_rn(3.f, cx), __fsub_rn(csum, cx)), m);
  const float dy = __fadd_rn(__fadd_rn(__fmul_rn(3.f, cy), __fsub_rn(csum, cy)), m);
  const float dz = __fadd_rn(__fadd_rn(__fmul_rn(3.f, cz), __fsub_rn(csum, cz)), m);
  const float qx = __fdiv_rn(cx, dx), qy = __fdiv_rn(cy, dy), qz = __fdiv_rn(cz, dz);
  const float qsum = __fadd_rn(__fadd_rn(__fmul_rn(cx, qx), __fmul_rn(cy, qy)), __fmul_rn(cz, qz));
  k.rden = __frcp_rn(__fadd_rn(__fadd_rn(csum, m), __fmul_rn(3.f, qsum)));
  k.rdx = __frcp_rn(dx);
  k.rdy = __frcp_rn(dy);
  k.rdz = __frcp_rn(dz);
  k.qsx = __fmul_rn(sx, qx);
  k.qsy = __fmul_rn(sy, qy);
  k.qsz = __fmul_rn(sz, qz);
}

// lane = (e - start) Dc G + d G + g of a plane starting at entry start
template <int kG>
__device__ __forceinline__ void lane_coef(uint32_t lane, LaneCoef& k, const float* __restrict__ mu,
                                          const float* __restrict__ c, const int* __restrict__ octant,
                                          const int* __restrict__ cell, const int* __restrict__ upstream,
                                          uint32_t start, uint32_t N, int G_runtime, uint32_t Dc) {
  const uint32_t G = kG > 0 ? kG : G_runtime;
  const uint32_t g = lane % G, t = lane / G;
  lane_coef_edg<kG>(start + t / Dc, t % Dc, g, k, mu, c, octant, cell, upstream, N, G_runtime, Dc);
}

// The store moments a lane reads in one view: the source (s) and (psi0, psi_x, psi_y, psi_z) of the x, y, z upstream
// neighbours
struct LaneIn {
  float4 s, X, Y, Z;
};

template <bool kCoherent>
__device__ __forceinline__ void gather_view(const LaneCoef& k, const float4* view, LaneIn& in) {
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  in.s = load4<kCoherent>(view + k.at);
  in.X = k.ax != kVacuum ? load4<kCoherent>(view + k.ax) : zero;
  in.Y = k.ay != kVacuum ? load4<kCoherent>(view + k.ay) : zero;
  in.Z = k.az != kVacuum ? load4<kCoherent>(view + k.az) : zero;
}

// The closed-form cell solve of the equations of linear_discontinuous_cell.py:14-87 in one view, stored over the
// source.
__device__ __forceinline__ void solve_view(const LaneCoef& k, const LaneIn& in, float4* view) {
  const float4 s = in.s, X = in.X, Y = in.Y, Z = in.Z;
  // face-averaged inflow psibar_a = psi_0[N_a] + s_a psi_a[N_a]
  const float pbx = __fadd_rn(X.x, __fmul_rn(k.sx, X.y));
  const float pby = __fadd_rn(Y.x, __fmul_rn(k.sy, Y.z));
  const float pbz = __fadd_rn(Z.x, __fmul_rn(k.sz, Z.w));
  const float r0 =
      __fadd_rn(s.x, __fadd_rn(__fadd_rn(__fmul_rn(k.cx, pbx), __fmul_rn(k.cy, pby)), __fmul_rn(k.cz, pbz)));
  // R_a = S_a - 3 s_a c_a psibar_a + sum_{b != a} c_b psi_a[N_b]
  const float rx = __fadd_rn(__fsub_rn(s.y, __fmul_rn(k.k3x, pbx)), __fadd_rn(__fmul_rn(k.cy, Y.y), __fmul_rn(k.cz, Z.y)));
  const float ry = __fadd_rn(__fsub_rn(s.z, __fmul_rn(k.k3y, pby)), __fadd_rn(__fmul_rn(k.cx, X.z), __fmul_rn(k.cz, Z.z)));
  const float rz = __fadd_rn(__fsub_rn(s.w, __fmul_rn(k.k3z, pbz)), __fadd_rn(__fmul_rn(k.cx, X.w), __fmul_rn(k.cy, Y.w)));
  const float corr =
      __fadd_rn(__fadd_rn(__fmul_rn(k.qsx, rx), __fmul_rn(k.qsy, ry)), __fmul_rn(k.qsz, rz));
  // the per-view quotients as products with the lane's correctly rounded reciprocals (within 1.5 ulp of the quotient)
  const float p0 = __fmul_rn(__fsub_rn(r0, corr), k.rden);
  float4 out;
  out.x = p0;
  out.y = __fmul_rn(__fadd_rn(rx, __fmul_rn(k.k3x, p0)), k.rdx);
  out.z = __fmul_rn(__fadd_rn(ry, __fmul_rn(k.k3y, p0)), k.rdy);
  out.w = __fmul_rn(__fadd_rn(rz, __fmul_rn(k.k3z, p0)), k.rdz);
  view[k.at] = out;
}

// One plane, one lane (view v, entry, direction, group) per thread: the reference's launch plan.
template <int kG>
__global__ void __launch_bounds__(kThreads) plane_kernel(float4* __restrict__ store, const float* __restrict__ mu,
                                                         const float* __restrict__ c, const int* __restrict__ octant,
                                                         const int* __restrict__ cell, const int* __restrict__ upstream,
                                                         uint32_t start, uint32_t per_view, uint32_t N, int G,
                                                         uint32_t Dc, int64_t views, int64_t view_stride) {
  const int64_t lane = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (lane >= views * per_view) return;
  const int64_t v = lane / per_view;
  LaneCoef k;
  lane_coef<kG>((uint32_t)(lane - v * per_view), k, mu, c, octant, cell, upstream, start, N, G, Dc);
  LaneIn in;
  float4* view = store + v * view_stride;
  gather_view<false>(k, view, in);
  solve_view(k, in, view);
}

// All planes in one cooperative launch, with a bounded grid barrier between planes. A thread takes one lane (entry,
// direction, group) of a plane at a time and solves it in every view, kVB views at a time: the loads of kVB views are
// issued before their solves (which a plain loop cannot do: the stores might alias the next view's loads as far as
// the compiler knows; within a plane they never do).
template <int kG, int kVB, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks) persistent_kernel(
    float4* __restrict__ store, const float* __restrict__ mu, const float* __restrict__ c,
    const int* __restrict__ octant, const int* __restrict__ cell, const int* __restrict__ upstream,
    const int* __restrict__ offsets, int num_planes, uint32_t N, int G, uint32_t Dc, int views, int64_t view_stride,
    unsigned* sync, uint64_t timeout_ns, int skip) {
  const uint32_t stride = gridDim.x * kThreads;
  const uint32_t per_entry = Dc * (kG > 0 ? kG : G);
  for (int p = 0; p < num_planes; ++p) {
    const uint32_t start = __ldg(offsets + p);
    const uint32_t total = (__ldg(offsets + p + 1) - start) * per_entry;
    for (uint32_t lane = blockIdx.x * kThreads + threadIdx.x; lane < total; lane += stride) {
      LaneCoef k;
      lane_coef<kG>(lane, k, mu, c, octant, cell, upstream, start, N, G, Dc);
      float4* view = store;
      for (int v0 = 0; v0 < views; v0 += kVB, view += kVB * view_stride) {
        LaneIn in[kVB];
#pragma unroll
        for (int j = 0; j < kVB; ++j)
          if (v0 + j < views) gather_view<true>(k, view + j * view_stride, in[j]);
#pragma unroll
        for (int j = 0; j < kVB; ++j)
          if (v0 + j < views) solve_view(k, in[j], view + j * view_stride);
      }
    }
    if (p + 1 < num_planes && !grid_barrier(sync, gridDim.x, timeout_ns, skip)) return;
  }
}

// The tiled schedule: in each octant's sweep frame the cells are cut into tiles of T^3; the tiles with the same sum
// of tile coordinates (a tile diagonal) depend only on earlier diagonals, so the grid barrier runs once per tile
// diagonal instead of once per plane. A block takes one task (a tile of one octant and a block of up to dpb
// directions) and walks the tile's 3 T - 2 sub-planes (cells with the same sum of in-tile coordinates) with a block
// barrier between them: the upstream reads of a sub-plane are the block's own writes one sub-plane earlier (L2 hits),
// and only the reads across a tile face come from an earlier diagonal. Every lane is the per-plane kernel's lane with
// the same inputs, so the store comes out bit for bit the same.
//
// Tables (host-built, transport_sweep.build_tiled_plan): entries (octant, cell, upstream) ordered by task and
// sub-plane; sub_offsets [tasks, num_sub + 1] the entry range of each sub-plane of each task; diagonal_offsets
// [num_diagonals + 1] the task range of each diagonal.
template <int kG, int kVB, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks) tiled_kernel(
    float4* __restrict__ store, const float* __restrict__ mu, const float* __restrict__ c,
    const int* __restrict__ octant, const int* __restrict__ cell, const int* __restrict__ upstream,
    const int* __restrict__ diagonal_offsets, const int* __restrict__ sub_offsets, int num_diagonals, int num_sub,
    uint32_t N, int G_runtime, uint32_t Dc, uint32_t dpb, int views, int64_t view_stride, unsigned* sync,
    uint64_t timeout_ns, int skip) {
  const uint32_t G = kG > 0 ? kG : G_runtime;
  const uint32_t dir_blocks = (Dc + dpb - 1) / dpb;
  for (int D = 0; D < num_diagonals; ++D) {
    const uint32_t t0 = __ldg(diagonal_offsets + D);
    const uint32_t work = (__ldg(diagonal_offsets + D + 1) - t0) * dir_blocks;
    for (uint32_t w = blockIdx.x; w < work; w += gridDim.x) {
      const uint32_t task = t0 + w / dir_blocks, d0 = (w % dir_blocks) * dpb;
      const uint32_t nd = min(dpb, Dc - d0);
      const int* so = sub_offsets + (size_t)task * (num_sub + 1);
      for (int sp = 0; sp < num_sub; ++sp) {
        const uint32_t start = __ldg(so + sp), count = __ldg(so + sp + 1) - start;
        if (count == 0) continue;  // the same for every thread of the block
        const uint32_t total = count * nd * G;
        for (uint32_t lane = threadIdx.x; lane < total; lane += kThreads) {
          const uint32_t g = lane % G, t = lane / G;
          LaneCoef k;
          lane_coef_edg<kG>(start + t / nd, d0 + t % nd, g, k, mu, c, octant, cell, upstream, N, G_runtime, Dc);
          float4* view = store;
          for (int v0 = 0; v0 < views; v0 += kVB, view += kVB * view_stride) {
            LaneIn in[kVB];
#pragma unroll
            for (int j = 0; j < kVB; ++j)
              if (v0 + j < views) gather_view<true>(k, view + j * view_stride, in[j]);
#pragma unroll
            for (int j = 0; j < kVB; ++j)
              if (v0 + j < views) solve_view(k, in[j], view + j * view_stride);
          }
        }
        __syncthreads();  // the sub-plane's outputs are written before the next sub-plane reads them
      }
    }
    if (D + 1 < num_diagonals && !grid_barrier(sync, gridDim.x, timeout_ns, skip)) return;
  }
}

template <int kG>
int launch_planes(float* store, const float* mu, const float* c, const int* octant, const int* cell,
                  const int* upstream, const int64_t* offsets, int64_t num_planes, int64_t N, int G, int64_t Dc,
                  int64_t views, cudaStream_t stream) {
  const int64_t view_stride = 8 * Dc * N * (int64_t)G;  // float4 per view
  for (int64_t p = 0; p < num_planes; ++p) {
    const int64_t start = offsets[p], E = offsets[p + 1] - offsets[p];
    const int64_t per_view = E * Dc * G;
    if (per_view <= 0) continue;
    plane_kernel<kG><<<(unsigned)cdiv(views * per_view, kThreads), kThreads, 0, stream>>>(
        reinterpret_cast<float4*>(store), mu, c, octant, cell, upstream, (uint32_t)start, (uint32_t)per_view,
        (uint32_t)N, G, (uint32_t)Dc, views, view_stride);
    note_launches();
  }
  return launch_status("citrus_sweep_planes");
}

template <int kG, int kVB, int kMinBlocks = 1>
int launch_persistent_u(float* store, const float* mu, const float* c, const int* octant, const int* cell,
                        const int* upstream, const int* offsets, int num_planes, int64_t N, int G, int64_t Dc,
                        int64_t views, unsigned* sync, int64_t max_blocks, uint64_t timeout_ns, int skip,
                        cudaStream_t stream) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_kernel<kG, kVB, kMinBlocks>,
                                                                kThreads, 0);
  if (e != cudaSuccess || per_sm < 1) return set_error(CITRUS_ECUDA, "citrus_sweep_persistent: occupancy query failed");
  int64_t blocks = (int64_t)per_sm * num_sms();
  if (max_blocks > 0 && max_blocks < blocks) blocks = max_blocks;
  if (skip >= blocks) skip = (int)blocks - 1;
  float4* store4 = reinterpret_cast<float4*>(store);
  uint32_t n32 = (uint32_t)N, dc32 = (uint32_t)Dc;
  int views32 = (int)views;
  int64_t view_stride = 8 * Dc * N * (int64_t)G;  // float4 per view
  cudaError_t z = cudaMemsetAsync(sync, 0, 4 * sizeof(unsigned), stream);
  if (z != cudaSuccess) return set_error(CITRUS_ECUDA, "citrus_sweep_persistent: %s", cudaGetErrorString(z));
  void* args[] = {&store4, &mu, &c, &octant, &cell, &upstream, &offsets, &num_planes, &n32, &G, &dc32, &views32,
                  &view_stride, &sync, &timeout_ns, &skip};
  e = cudaLaunchCooperativeKernel((const void*)persistent_kernel<kG, kVB, kMinBlocks>, dim3((unsigned)blocks),
                                  dim3(kThreads), args, 0, stream);
  if (e != cudaSuccess) return set_error(CITRUS_ELAUNCH, "citrus_sweep_persistent: %s", cudaGetErrorString(e));
  note_launches();
  return CITRUS_OK;
}

template <int kG, int kVB, int kMinBlocks>
int launch_tiled_u(float* store, const float* mu, const float* c, const int* octant, const int* cell,
                   const int* upstream, const int* diagonal_offsets, const int* sub_offsets, int num_diagonals,
                   int num_sub, int64_t N, int G, int64_t Dc, int64_t dpb, int64_t views, unsigned* sync,
                   int64_t max_blocks, uint64_t timeout_ns, int skip, cudaStream_t stream) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tiled_kernel<kG, kVB, kMinBlocks>, kThreads,
                                                                0);
  if (e != cudaSuccess || per_sm < 1) return set_error(CITRUS_ECUDA, "citrus_sweep_tiled: occupancy query failed");
  int64_t blocks = (int64_t)per_sm * num_sms();
  if (max_blocks > 0 && max_blocks < blocks) blocks = max_blocks;
  if (skip >= blocks) skip = (int)blocks - 1;
  float4* store4 = reinterpret_cast<float4*>(store);
  uint32_t n32 = (uint32_t)N, dc32 = (uint32_t)Dc, dpb32 = (uint32_t)dpb;
  int views32 = (int)views;
  int64_t view_stride = 8 * Dc * N * (int64_t)G;  // float4 per view
  cudaError_t z = cudaMemsetAsync(sync, 0, 4 * sizeof(unsigned), stream);
  if (z != cudaSuccess) return set_error(CITRUS_ECUDA, "citrus_sweep_tiled: %s", cudaGetErrorString(z));
  void* args[] = {&store4, &mu, &c, &octant, &cell, &upstream, &diagonal_offsets, &sub_offsets, &num_diagonals,
                  &num_sub, &n32, &G, &dc32, &dpb32, &views32, &view_stride, &sync, &timeout_ns, &skip};
  e = cudaLaunchCooperativeKernel((const void*)tiled_kernel<kG, kVB, kMinBlocks>, dim3((unsigned)blocks),
                                  dim3(kThreads), args, 0, stream);
  if (e != cudaSuccess) return set_error(CITRUS_ELAUNCH, "citrus_sweep_tiled: %s", cudaGetErrorString(e));
  note_launches();
  return CITRUS_OK;
}

// the thread forms of the tiled launch: one view at a time (four blocks per SM), or the loads of two views issued
// before their solves (three blocks per SM)
template <int kG>
int launch_tiled(float* store, const float* mu, const float* c, const int* octant, const int* cell,
                 const int* upstream, const int* diagonal_offsets, const int* sub_offsets, int num_diagonals,
                 int num_sub, int64_t N, int G, int64_t Dc, int64_t dpb, int64_t views, unsigned* sync,
                 int64_t max_blocks, uint64_t timeout_ns, int skip, cudaStream_t stream, int form) {
  if (form == 2)
    return launch_tiled_u<kG, 2, 3>(store, mu, c, octant, cell, upstream, diagonal_offsets, sub_offsets,
                                    num_diagonals, num_sub, N, G, Dc, dpb, views, sync, max_blocks, timeout_ns, skip,
                                    stream);
  if (form == 1)
    return launch_tiled_u<kG, 1, 4>(store, mu, c, octant, cell, upstream, diagonal_offsets, sub_offsets,
                                    num_diagonals, num_sub, N, G, Dc, dpb, views, sync, max_blocks, timeout_ns, skip,
                                    stream);
  return set_error(CITRUS_EINVAL, "citrus_sweep_tiled: thread form %d (1 or 2)", form);
}

constexpr int kDefaultUnroll = 1;

// the forms of the persistent launch's threads, chosen per grid by the autotuner
template <int kG>
int launch_persistent(float* store, const float* mu, const float* c, const int* octant, const int* cell,
                      const int* upstream, const int* offsets, int num_planes, int64_t N, int G, int64_t Dc,
                      int64_t views, unsigned* sync, int64_t max_blocks, uint64_t timeout_ns, int skip,
                      cudaStream_t stream, int unroll = kDefaultUnroll) {
  switch (unroll) {
    case 1:  // one view at a time, five blocks of 256 threads per SM
      return launch_persistent_u<kG, 1, 5>(store, mu, c, octant, cell, upstream, offsets, num_planes, N, G, Dc,
                                           views, sync, max_blocks, timeout_ns, skip, stream);
    case 3:  // one view at a time, registers capped for six blocks of 256 threads per SM
      return launch_persistent_u<kG, 1, 6>(store, mu, c, octant, cell, upstream, offsets, num_planes, N, G, Dc,
                                           views, sync, max_blocks, timeout_ns, skip, stream);
    case 5:  // one view at a time, four blocks per SM
      return launch_persistent_u<kG, 1, 4>(store, mu, c, octant, cell, upstream, offsets, num_planes, N, G, Dc,
                                           views, sync, max_blocks, timeout_ns, skip, stream);
    case 2:  // the loads of two views before their solves, three blocks per SM
      return launch_persistent_u<kG, 2, 3>(store, mu, c, octant, cell, upstream, offsets, num_planes, N, G, Dc,
                                           views, sync, max_blocks, timeout_ns, skip, stream);
    case 4:  // the loads of four views before their solves, two blocks per SM
      return launch_persistent_u<kG, 4, 2>(store, mu, c, octant, cell, upstream, offsets, num_planes, N, G, Dc,
                                           views, sync, max_blocks, timeout_ns, skip, stream);
    default:
      return set_error(CITRUS_EINVAL, "citrus_sweep_persistent: thread form %d (1, 2, 3, 4 or 5)", unroll);
  }
}

int check_sweep_args(const float* store, const float* mu, const float* c, const int* octant, const int* cell,
                     const int* upstream, int64_t num_planes, int64_t N, int64_t G, int64_t Dc, int64_t views) {
  CITRUS_REQUIRE(store && mu && c && octant && cell && upstream, "sweep: null pointer argument");
  CITRUS_REQUIRE(num_planes >= 1 && N >= 1 && G >= 1 && Dc >= 1 && views >= 1,
                 "sweep: sizes must be positive (planes %lld, cells %lld, groups %lld, dc %lld, views %lld)",
                 (long long)num_planes, (long long)N, (long long)G, (long long)Dc, (long long)views);
  CITRUS_REQUIRE(N < (1ll << 31) / 8, "sweep: %lld cells exceed the int32 entry tables", (long long)N);
  CITRUS_REQUIRE(views < (1ll << 31), "sweep: too many views (%lld)", (long long)views);
  CITRUS_REQUIRE(8 * N * Dc * G < (1ll << 31),
                 "sweep: one view's store of %lld float4 exceeds the 32-bit lane positions; sweep fewer directions "
                 "per chunk", (long long)(8 * N * Dc * G));
  CITRUS_REQUIRE(G <= 4096, "sweep: too many groups (%lld)", (long long)G);
  CITRUS_REQUIRE(((uintptr_t)store % 16) == 0, "sweep: store must be 16-byte aligned");
  return CITRUS_OK;
}

}  // namespace
}  // namespace citrus

using namespace citrus;

extern "C" int citrus_sweep_planes(float* store, const float* mu_cells, const float* c, const int32_t* octant,
                                   const int32_t* cell, const int32_t* upstream, const int64_t* plane_offsets_host,
                                   int64_t num_planes, int64_t num_cells, int64_t num_groups, int64_t dc,
                                   int64_t views, void* stream) {
  int status = check_sweep_args(store, mu_cells, c, octant, cell, upstream, num_planes, num_cells, num_groups, dc,
                                views);
  if (status) return status;
  CITRUS_REQUIRE(plane_offsets_host != nullptr, "citrus_sweep_planes: null plane offsets");
  const int G = (int)num_groups;
  cudaStream_t s = as_stream(stream);
  switch (G) {
    case 1: return launch_planes<1>(store, mu_cells, c, octant, cell, upstream, plane_offsets_host, num_planes,
                                    num_cells, G, dc, views, s);
    case 2: return launch_planes<2>(store, mu_cells, c, octant, cell, upstream, plane_offsets_host, num_planes,
                                    num_cells, G, dc, views, s);
    case 4: return launch_planes<4>(store, mu_cells, c, octant, cell, upstream, plane_offsets_host, num_planes,
                                    num_cells, G, dc, views, s);
    case 8: return launch_planes<8>(store, mu_cells, c, octant, cell, upstream, plane_offsets_host, num_planes,
                                    num_cells, G, dc, views, s);
    case 16: return launch_planes<16>(store, mu_cells, c, octant, cell, upstream, plane_offsets_host, num_planes,
                                      num_cells, G, dc, views, s);
    default: return launch_planes<0>(store, mu_cells, c, octant, cell, upstream, plane_offsets_host, num_planes,
                                     num_cells, G, dc, views, s);
  }
}

extern "C" int citrus_sweep_persistent_config(float* store, const float* mu_cells, const float* c,
                                              const int32_t* octant, const int32_t* cell, const int32_t* upstream,
                                              const int32_t* plane_offsets_dev, int64_t num_planes, int64_t num_cells,
                                              int64_t num_groups, int64_t dc, int64_t views, uint32_t* sync,
                                              int64_t max_blocks, int32_t thread_form, int64_t timeout_ns,
                                              int64_t skip_block, void* stream) {
  int status = check_sweep_args(store, mu_cells, c, octant, cell, upstream, num_planes, num_cells, num_groups, dc,
                                views);
  if (status) return status;
  CITRUS_REQUIRE(plane_offsets_dev != nullptr && sync != nullptr, "citrus_sweep_persistent: null offsets or sync");
  CITRUS_REQUIRE(num_planes < (1ll << 30), "citrus_sweep_persistent: too many planes");
  CITRUS_REQUIRE(timeout_ns > 0, "citrus_sweep_persistent: timeout_ns must be positive");
  const int G = (int)num_groups, P = (int)num_planes, skip = skip_block < 0 ? -1 : (int)skip_block;
  const uint64_t t = (uint64_t)timeout_ns;
  const int u = thread_form <= 0 ? kDefaultUnroll : thread_form;
  unsigned* sy = reinterpret_cast<unsigned*>(sync);
  cudaStream_t s = as_stream(stream);
  switch (G) {
    case 1: return launch_persistent<1>(store, mu_cells, c, octant, cell, upstream, plane_offsets_dev, P, num_cells,
                                        G, dc, views, sy, max_blocks, t, skip, s, u);
    case 2: return launch_persistent<2>(store, mu_cells, c, octant, cell, upstream, plane_offsets_dev, P, num_cells,
                                        G, dc, views, sy, max_blocks, t, skip, s, u);
    case 4: return launch_persistent<4>(store, mu_cells, c, octant, cell, upstream, plane_offsets_dev, P, num_cells,
                                        G, dc, views, sy, max_blocks, t, skip, s, u);
    case 8: return launch_persistent<8>(store, mu_cells, c, octant, cell, upstream, plane_offsets_dev, P, num_cells,
                                        G, dc, views, sy, max_blocks, t, skip, s, u);
    case 16: return launch_persistent<16>(store, mu_cells, c, octant, cell, upstream, plane_offsets_dev, P,
                                          num_cells, G, dc, views, sy, max_blocks, t, skip, s, u);
    default: return launch_persistent<0>(store, mu_cells, c, octant, cell, upstream, plane_offsets_dev, P, num_cells,
                                         G, dc, views, sy, max_blocks, t, skip, s, u);
  }
}

extern "C" int citrus_sweep_persistent(float* store, const float* mu_cells, const float* c, const int32_t* octant,
                                       const int32_t* cell, const int32_t* upstream, const int32_t* plane_offsets_dev,
                                       int64_t num_planes, int64_t num_cells, int64_t num_groups, int64_t dc,
                                       int64_t views, uint32_t* sync, int64_t max_blocks, int64_t timeout_ns,
                                       int64_t skip_block, void* stream) {
  return citrus_sweep_persistent_config(store, mu_cells, c, octant, cell, upstream, plane_offsets_dev, num_planes,
                                        num_cells, num_groups, dc, views, sync, max_blocks, 0, timeout_ns, skip_block,
                                        stream);
}

extern "C" int citrus_sweep_tiled(float* store, const float* mu_cells, const float* c, const int32_t* octant,
                                  const int32_t* cell, const int32_t* upstream, const int32_t* diagonal_offsets,
                                  const int32_t* sub_offsets, int64_t num_diagonals, int64_t num_sub,
                                  int64_t num_cells, int64_t num_groups, int64_t dc, int64_t views,
                                  int64_t dirs_per_block, uint32_t* sync, int64_t max_blocks, int64_t thread_form,
                                  int64_t timeout_ns, int64_t skip_block, void* stream) {
  int status = check_sweep_args(store, mu_cells, c, octant, cell, upstream, num_diagonals, num_cells, num_groups, dc,
                                views);
  if (status) return status;
  CITRUS_REQUIRE(diagonal_offsets && sub_offsets && sync, "citrus_sweep_tiled: null tables or sync words");
  CITRUS_REQUIRE(num_sub >= 1 && num_sub <= 4096 && num_diagonals <= (1 << 20),
                 "citrus_sweep_tiled: bad table sizes (diagonals %lld, sub-planes %lld)", (long long)num_diagonals,
                 (long long)num_sub);
  CITRUS_REQUIRE(dirs_per_block >= 1 && dirs_per_block <= dc, "citrus_sweep_tiled: directions per block %lld outside "
                 "[1, %lld]", (long long)dirs_per_block, (long long)dc);
  CITRUS_REQUIRE(timeout_ns > 0, "citrus_sweep_tiled: timeout_ns must be positive");
  const int G = (int)num_groups, ND = (int)num_diagonals, NS = (int)num_sub, form = (int)thread_form;
  const uint64_t t = (uint64_t)timeout_ns;
  const int skip = (int)skip_block;
  unsigned* sy = reinterpret_cast<unsigned*>(sync);
  cudaStream_t s = as_stream(stream);
#define CITRUS_TILED(KG)                                                                                           \
  launch_tiled<KG>(store, mu_cells, c, octant, cell, upstream, diagonal_offsets, sub_offsets, ND, NS, num_cells, G, \
                   dc, dirs_per_block, views, sy, max_blocks, t, skip, s, form)
  switch (G) {
    case 1: status = CITRUS_TILED(1); break;
    case 2: status = CITRUS_TILED(2); break;
    case 4: status = CITRUS_TILED(4); break;
    case 8: status = CITRUS_TILED(8); break;
    case 16: status = CITRUS_TILED(16); break;
    default: status = CITRUS_TILED(0); break;
  }
#undef CITRUS_TILED
  if (status) return status;
  return launch_status("citrus_sweep_tiled");
}

// ---- allocation-free persistent sweep ----------------------------------------------------------------------------
//
// The same persistent launch with its scratch in a file-scope device array instead of caller-provided device memory:
// the barrier words at [0, 4) and the int32 plane offsets from word 64 (byte 256) on. The call makes no device
// allocation of any kind; it only clears the barrier words and copies the offsets into the array, both on the stream.
namespace citrus {
namespace {

constexpr int64_t kStaticMaxPlanes = 8191;  // R + C + S - 2 <= 8191: every grid up to 2730^3 cells
constexpr int kStaticOffsetsWord = 64;
constexpr int kStaticWords = kStaticOffsetsWord + (int)kStaticMaxPlanes + 1;  // 8256 words, 33 KB per device
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) uint32_t g_static_sweep_scratch[kStaticWords];

std::mutex g_static_mutex;
uint32_t* g_static_address[kStaticMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once per device.
int static_scratch(uint32_t** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(CITRUS_ECUDA, "citrus_sweep_persistent_static: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kStaticMaxDevices)
    return set_error(CITRUS_EINVAL, "citrus_sweep_persistent_static: device %d beyond the %d supported", dev,
                     kStaticMaxDevices);
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (g_static_address[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_sweep_scratch);
    if (e != cudaSuccess || p == nullptr)
      return set_error(CITRUS_ECUDA, "citrus_sweep_persistent_static: scratch address on device %d: %s", dev,
                       cudaGetErrorString(e));
    g_static_address[dev] = static_cast<uint32_t*>(p);
  }
  *out = g_static_address[dev];
  return CITRUS_OK;
}

}  // namespace
}  // namespace citrus

extern "C" int citrus_sweep_persistent_static(float* store, const float* mu_cells, const float* c,
                                              const int32_t* octant, const int32_t* cell, const int32_t* upstream,
                                              const int32_t* plane_offsets_host, int64_t num_planes,
                                              int64_t num_cells, int64_t num_groups, int64_t dc, int64_t views,
                                              uint32_t* timeout_word, int64_t timeout_ns, void* stream) {
  int status = check_sweep_args(store, mu_cells, c, octant, cell, upstream, num_planes, num_cells, num_groups, dc,
                                views);
  if (status) return status;
  CITRUS_REQUIRE(plane_offsets_host != nullptr, "citrus_sweep_persistent_static: null plane offsets");
  CITRUS_REQUIRE(num_planes <= kStaticMaxPlanes,
                 "citrus_sweep_persistent_static: %lld planes exceed the static scratch (at most %lld planes, "
                 "R + C + S - 2 <= %lld); use citrus_sweep_persistent with caller scratch",
                 (long long)num_planes, (long long)kStaticMaxPlanes, (long long)kStaticMaxPlanes);
  CITRUS_REQUIRE(timeout_ns > 0, "citrus_sweep_persistent_static: timeout_ns must be positive");
  uint32_t* scratch = nullptr;
  status = static_scratch(&scratch);
  if (status) return status;
  cudaStream_t s = as_stream(stream);
  int32_t* offsets = reinterpret_cast<int32_t*>(scratch + kStaticOffsetsWord);
  cudaError_t e = cudaMemcpyAsync(offsets, plane_offsets_host, (size_t)(num_planes + 1) * sizeof(int32_t),
                                  cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess)
    return set_error(CITRUS_ECUDA, "citrus_sweep_persistent_static: offsets copy: %s", cudaGetErrorString(e));
  // the barrier words are cleared by the launch below (cudaMemsetAsync on the stream)
  const int G = (int)num_groups, P = (int)num_planes;
  const uint64_t t = (uint64_t)timeout_ns;
  unsigned* sy = reinterpret_cast<unsigned*>(scratch);
  switch (G) {
    case 1: status = launch_persistent<1>(store, mu_cells, c, octant, cell, upstream, offsets, P, num_cells, G, dc,
                                          views, sy, 0, t, -1, s); break;
    case 2: status = launch_persistent<2>(store, mu_cells, c, octant, cell, upstream, offsets, P, num_cells, G, dc,
                                          views, sy, 0, t, -1, s); break;
    case 4: status = launch_persistent<4>(store, mu_cells, c, octant, cell, upstream, offsets, P, num_cells, G, dc,
                                          views, sy, 0, t, -1, s); break;
    case 8: status = launch_persistent<8>(store, mu_cells, c, octant, cell, upstream, offsets, P, num_cells, G, dc,
                                          views, sy, 0, t, -1, s); break;
    case 16: status = launch_persistent<16>(store, mu_cells, c, octant, cell, upstream, offsets, P, num_cells, G, dc,
                                            views, sy, 0, t, -1, s); break;
    default: status = launch_persistent<0>(store, mu_cells, c, octant, cell, upstream, offsets, P, num_cells, G, dc,
                                           views, sy, 0, t, -1, s); break;
  }
  if (status || timeout_word == nullptr) return status;
  e = cudaMemcpyAsync(timeout_word, scratch + 2, sizeof(uint32_t), cudaMemcpyDefault, s);
  if (e != cudaSuccess)
    return set_error(CITRUS_ECUDA, "citrus_sweep_persistent_static: timeout word copy: %s", cudaGetErrorString(e));
  return CITRUS_OK;
}
