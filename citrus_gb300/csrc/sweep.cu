// Linear-discontinuous discrete-ordinates sweep: the closed-form cell solve of every (entry, direction, group) of a
// diagonal wavefront plane, in place in the chunk's cell-major store [views, 8, Dc, N, 4G].
//
// The cell equations are those of citrus/scatter_solver/linear_discontinuous_cell.py:14-87 (right-hand sides from the
// source and the three upstream neighbours, then the closed-form 4 x 4 solve), evaluated term by term in float32 with
// IEEE division. Two drivers share the lane body: one launch per plane (the reference's plan,
// sweep_kernels.py:265-290) and one persistent cooperative launch that walks all planes with a bounded grid barrier
// between them, so a whole chunk is a single launch.
#include "common.cuh"
#include <mutex>

namespace citrus {
namespace {

constexpr int kThreads = 256;

template <bool kCoherent>
__device__ __forceinline__ float4 load4(const float* p) {
  if (kCoherent) return __ldcg(reinterpret_cast<const float4*>(p));  // L2 only: written by other SMs this launch
  return *reinterpret_cast<const float4*>(p);
}

// The inputs of one lane: entry e of the plane, direction d of the chunk, group g, view v. Upstream neighbours lie on
// the previous plane (already swept); an upstream index N is a vacuum face and reads zeros.
struct LaneIn {
  float4 s, X, Y, Z;  // source moments, and (psi0, psi_x, psi_y, psi_z) of the x, y, z upstream neighbours
  float cx, cy, cz, m;
  int o;
  float* dst;
};

template <int kG, bool kCoherent>
__device__ __forceinline__ void gather_lane(int64_t lane, LaneIn& in, float* __restrict__ store,
                                            const float* __restrict__ mu, const float* __restrict__ c,
                                            const int* __restrict__ octant, const int* __restrict__ cell,
                                            const int* __restrict__ upstream, int64_t start, int64_t E, int64_t N,
                                            int G_runtime, int64_t Dc, int64_t view_stride) {
  const int G = kG > 0 ? kG : G_runtime;
  const int g = (int)(lane % G);
  int64_t t = lane / G;
  const int64_t d = t % Dc;
  t /= Dc;
  const int64_t e = start + t % E;
  const int64_t v = t / E;
  const int o = __ldg(octant + e);
  const int64_t n = __ldg(cell + e);
  const int64_t ux = __ldg(upstream + 3 * e), uy = __ldg(upstream + 3 * e + 1), uz = __ldg(upstream + 3 * e + 2);
  const int64_t od = (int64_t)o * Dc + d;
  in.o = o;
  in.cx = __ldg(c + 3 * od);
  in.cy = __ldg(c + 3 * od + 1);
  in.cz = __ldg(c + 3 * od + 2);
  in.m = __ldg(mu + n * G + g);
  const int64_t Q = 4 * (int64_t)G;
  float* base = store + v * view_stride + od * N * Q + 4 * g;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  in.dst = base + n * Q;
  in.s = load4<kCoherent>(in.dst);
  in.X = ux < N ? load4<kCoherent>(base + ux * Q) : zero;
  in.Y = uy < N ? load4<kCoherent>(base + uy * Q) : zero;
  in.Z = uz < N ? load4<kCoherent>(base + uz * Q) : zero;
}

// The closed-form cell solve of one lane and its store over the source. Every operation is rounded on its own (no
// multiply-add contraction), so every kernel that inlines it computes the same bits.
__device__ __forceinline__ void finish_lane(const LaneIn& in) {
  const float sx = (in.o & 4) ? -1.f : 1.f, sy = (in.o & 2) ? -1.f : 1.f, sz = (in.o & 1) ? -1.f : 1.f;
  const float cx = in.cx, cy = in.cy, cz = in.cz, m = in.m;
  const float4 s = in.s, X = in.X, Y = in.Y, Z = in.Z;
  // face-averaged inflow psibar_a = psi_0[N_a] + s_a psi_a[N_a]
  const float pbx = __fadd_rn(X.x, __fmul_rn(sx, X.y));
  const float pby = __fadd_rn(Y.x, __fmul_rn(sy, Y.z));
  const float pbz = __fadd_rn(Z.x, __fmul_rn(sz, Z.w));
  const float r0 = __fadd_rn(s.x, __fadd_rn(__fadd_rn(__fmul_rn(cx, pbx), __fmul_rn(cy, pby)), __fmul_rn(cz, pbz)));
  // R_a = S_a - 3 s_a c_a psibar_a + sum_{b != a} c_b psi_a[N_b]
  const float tx = __fmul_rn(__fmul_rn(__fmul_rn(3.f, sx), cx), pbx);
  const float ty = __fmul_rn(__fmul_rn(__fmul_rn(3.f, sy), cy), pby);
  const float tz = __fmul_rn(__fmul_rn(__fmul_rn(3.f, sz), cz), pbz);
  const float rx = __fadd_rn(__fsub_rn(s.y, tx), __fadd_rn(__fmul_rn(cy, Y.y), __fmul_rn(cz, Z.y)));
  const float ry = __fadd_rn(__fsub_rn(s.z, ty), __fadd_rn(__fmul_rn(cx, X.z), __fmul_rn(cz, Z.z)));
  const float rz = __fadd_rn(__fsub_rn(s.w, tz), __fadd_rn(__fmul_rn(cx, X.w), __fmul_rn(cy, Y.w)));
  const float csum = __fadd_rn(__fadd_rn(cx, cy), cz);
  const float dx = __fadd_rn(__fadd_rn(__fmul_rn(3.f, cx), __fsub_rn(csum, cx)), m);
  const float dy = __fadd_rn(__fadd_rn(__fmul_rn(3.f, cy), __fsub_rn(csum, cy)), m);
  const float dz = __fadd_rn(__fadd_rn(__fmul_rn(3.f, cz), __fsub_rn(csum, cz)), m);
  const float qx = __fdiv_rn(cx, dx), qy = __fdiv_rn(cy, dy), qz = __fdiv_rn(cz, dz);
  const float qsum = __fadd_rn(__fadd_rn(__fmul_rn(cx, qx), __fmul_rn(cy, qy)), __fmul_rn(cz, qz));
  const float denom = __fadd_rn(__fadd_rn(csum, m), __fmul_rn(3.f, qsum));
  const float corr = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(sx, qx), rx), __fmul_rn(__fmul_rn(sy, qy), ry)),
                               __fmul_rn(__fmul_rn(sz, qz), rz));
  const float p0 = __fdiv_rn(__fsub_rn(r0, corr), denom);
  float4 out;
  out.x = p0;
  out.y = __fdiv_rn(__fadd_rn(rx, __fmul_rn(__fmul_rn(__fmul_rn(3.f, sx), cx), p0)), dx);
  out.z = __fdiv_rn(__fadd_rn(ry, __fmul_rn(__fmul_rn(__fmul_rn(3.f, sy), cy), p0)), dy);
  out.w = __fdiv_rn(__fadd_rn(rz, __fmul_rn(__fmul_rn(__fmul_rn(3.f, sz), cz), p0)), dz);
  *reinterpret_cast<float4*>(in.dst) = out;
}

template <int kG, bool kCoherent>
__device__ __forceinline__ void solve_lane(int64_t lane, float* __restrict__ store, const float* __restrict__ mu,
                                           const float* __restrict__ c, const int* __restrict__ octant,
                                           const int* __restrict__ cell, const int* __restrict__ upstream,
                                           int64_t start, int64_t E, int64_t N, int G_runtime, int64_t Dc,
                                           int64_t view_stride) {
  LaneIn in;
  gather_lane<kG, kCoherent>(lane, in, store, mu, c, octant, cell, upstream, start, E, N, G_runtime, Dc,
                             view_stride);
  finish_lane(in);
}

template <int kG>
__global__ void __launch_bounds__(kThreads) plane_kernel(float* __restrict__ store, const float* __restrict__ mu,
                                                         const float* __restrict__ c, const int* __restrict__ octant,
                                                         const int* __restrict__ cell, const int* __restrict__ upstream,
                                                         int64_t start, int64_t E, int64_t N, int G, int64_t Dc,
                                                         int64_t views, int64_t view_stride) {
  const int64_t lane = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const int64_t total = views * E * Dc * (kG > 0 ? kG : G);
  if (lane >= total) return;
  solve_lane<kG, false>(lane, store, mu, c, octant, cell, upstream, start, E, N, G, Dc, view_stride);
}

// All planes in one cooperative launch. A thread takes kU lanes of a plane at a time (stride apart, so every warp
// still reads whole cells): all their loads are issued before the first solve and store, which a plain loop cannot
// do (the stores might alias the next lane's loads as far as the compiler knows; within a plane they never do).
template <int kG, int kU, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks) persistent_kernel(
    float* __restrict__ store, const float* __restrict__ mu, const float* __restrict__ c,
    const int* __restrict__ octant, const int* __restrict__ cell, const int* __restrict__ upstream,
    const int* __restrict__ offsets, int num_planes, int64_t N, int G, int64_t Dc, int64_t views,
    int64_t view_stride, unsigned* sync, uint64_t timeout_ns, int skip) {
  const int64_t stride = (int64_t)gridDim.x * kThreads;
  const int64_t per_entry = Dc * (kG > 0 ? kG : G) * views;
  for (int p = 0; p < num_planes; ++p) {
    const int64_t start = __ldg(offsets + p);
    const int64_t E = __ldg(offsets + p + 1) - start;
    const int64_t total = E * per_entry;
    for (int64_t lane0 = (int64_t)blockIdx.x * kThreads + threadIdx.x; lane0 < total; lane0 += stride * kU) {
      LaneIn in[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u)
        if (lane0 + u * stride < total)
          gather_lane<kG, true>(lane0 + u * stride, in[u], store, mu, c, octant, cell, upstream, start, E, N, G, Dc,
                                view_stride);
#pragma unroll
      for (int u = 0; u < kU; ++u)
        if (lane0 + u * stride < total) finish_lane(in[u]);
    }
    if (p + 1 < num_planes && !grid_barrier(sync, gridDim.x, timeout_ns, skip)) return;
  }
}

template <int kG>
int launch_planes(float* store, const float* mu, const float* c, const int* octant, const int* cell,
                  const int* upstream, const int64_t* offsets, int64_t num_planes, int64_t N, int G, int64_t Dc,
                  int64_t views, cudaStream_t stream) {
  const int64_t view_stride = 8 * Dc * N * 4 * (int64_t)G;
  for (int64_t p = 0; p < num_planes; ++p) {
    const int64_t start = offsets[p], E = offsets[p + 1] - offsets[p];
    const int64_t total = views * E * Dc * G;
    if (total <= 0) continue;
    plane_kernel<kG><<<(unsigned)cdiv(total, kThreads), kThreads, 0, stream>>>(
        store, mu, c, octant, cell, upstream, start, E, N, G, Dc, views, view_stride);
    note_launches();
  }
  return launch_status("citrus_sweep_planes");
}

template <int kG, int kU, int kMinBlocks = 1>
int launch_persistent_u(float* store, const float* mu, const float* c, const int* octant, const int* cell,
                        const int* upstream, const int* offsets, int num_planes, int64_t N, int G, int64_t Dc,
                        int64_t views, unsigned* sync, int64_t max_blocks, uint64_t timeout_ns, int skip,
                        cudaStream_t stream) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_kernel<kG, kU, kMinBlocks>,
                                                                kThreads, 0);
  if (e != cudaSuccess || per_sm < 1) return set_error(CITRUS_ECUDA, "citrus_sweep_persistent: occupancy query failed");
  int64_t blocks = (int64_t)per_sm * num_sms();
  if (max_blocks > 0 && max_blocks < blocks) blocks = max_blocks;
  if (skip >= blocks) skip = (int)blocks - 1;
  int64_t view_stride = 8 * Dc * N * 4 * (int64_t)G;
  cudaError_t z = cudaMemsetAsync(sync, 0, 4 * sizeof(unsigned), stream);
  if (z != cudaSuccess) return set_error(CITRUS_ECUDA, "citrus_sweep_persistent: %s", cudaGetErrorString(z));
  void* args[] = {&store, &mu, &c, &octant, &cell, &upstream, &offsets, &num_planes, &N, &G, &Dc, &views,
                  &view_stride, &sync, &timeout_ns, &skip};
  e = cudaLaunchCooperativeKernel((const void*)persistent_kernel<kG, kU, kMinBlocks>, dim3((unsigned)blocks),
                                  dim3(kThreads), args, 0, stream);
  if (e != cudaSuccess) return set_error(CITRUS_ELAUNCH, "citrus_sweep_persistent: %s", cudaGetErrorString(e));
  note_launches();
  return CITRUS_OK;
}

constexpr int kDefaultUnroll = 1;

template <int kG>
int launch_persistent(float* store, const float* mu, const float* c, const int* octant, const int* cell,
                      const int* upstream, const int* offsets, int num_planes, int64_t N, int G, int64_t Dc,
                      int64_t views, unsigned* sync, int64_t max_blocks, uint64_t timeout_ns, int skip,
                      cudaStream_t stream, int unroll = kDefaultUnroll) {
  switch (unroll) {
    case 1:  // one lane per thread, five blocks of 256 threads per SM
      return launch_persistent_u<kG, 1, 5>(store, mu, c, octant, cell, upstream, offsets, num_planes, N, G, Dc,
                                           views, sync, max_blocks, timeout_ns, skip, stream);
    case 3:  // one lane per thread, registers capped for six blocks of 256 threads per SM
      return launch_persistent_u<kG, 1, 6>(store, mu, c, octant, cell, upstream, offsets, num_planes, N, G, Dc,
                                           views, sync, max_blocks, timeout_ns, skip, stream);
    case 5:  // one lane per thread, eight blocks per SM
      return launch_persistent_u<kG, 1, 8>(store, mu, c, octant, cell, upstream, offsets, num_planes, N, G, Dc,
                                           views, sync, max_blocks, timeout_ns, skip, stream);
    case 2: return launch_persistent_u<kG, 2>(store, mu, c, octant, cell, upstream, offsets, num_planes, N, G, Dc,
                                              views, sync, max_blocks, timeout_ns, skip, stream);
    case 4: return launch_persistent_u<kG, 4>(store, mu, c, octant, cell, upstream, offsets, num_planes, N, G, Dc,
                                              views, sync, max_blocks, timeout_ns, skip, stream);
    default:
      return set_error(CITRUS_EINVAL, "citrus_sweep_persistent: lanes per thread form %d (1, 2, 3, 4 or 5)", unroll);
  }
}

int check_sweep_args(const float* store, const float* mu, const float* c, const int* octant, const int* cell,
                     const int* upstream, int64_t num_planes, int64_t N, int64_t G, int64_t Dc, int64_t views) {
  CITRUS_REQUIRE(store && mu && c && octant && cell && upstream, "sweep: null pointer argument");
  CITRUS_REQUIRE(num_planes >= 1 && N >= 1 && G >= 1 && Dc >= 1 && views >= 1,
                 "sweep: sizes must be positive (planes %lld, cells %lld, groups %lld, dc %lld, views %lld)",
                 (long long)num_planes, (long long)N, (long long)G, (long long)Dc, (long long)views);
  CITRUS_REQUIRE(N < (1ll << 31) / 8, "sweep: %lld cells exceed the int32 entry tables", (long long)N);
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
                                              int64_t max_blocks, int32_t lanes_per_thread, int64_t timeout_ns,
                                              int64_t skip_block, void* stream) {
  int status = check_sweep_args(store, mu_cells, c, octant, cell, upstream, num_planes, num_cells, num_groups, dc,
                                views);
  if (status) return status;
  CITRUS_REQUIRE(plane_offsets_dev != nullptr && sync != nullptr, "citrus_sweep_persistent: null offsets or sync");
  CITRUS_REQUIRE(num_planes < (1ll << 30), "citrus_sweep_persistent: too many planes");
  CITRUS_REQUIRE(timeout_ns > 0, "citrus_sweep_persistent: timeout_ns must be positive");
  const int G = (int)num_groups, P = (int)num_planes, skip = skip_block < 0 ? -1 : (int)skip_block;
  const uint64_t t = (uint64_t)timeout_ns;
  const int u = lanes_per_thread <= 0 ? kDefaultUnroll : lanes_per_thread;
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
