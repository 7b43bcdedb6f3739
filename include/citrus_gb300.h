/*
 * citrus_gb300 C ABI: the GB300 (sm_103a) kernels of the CITRUS scatter step behind plain pointers and sizes.
 *
 * Every entry point takes device pointers, 64-bit sizes and a CUDA stream (as void*), enqueues its kernels on that
 * stream without synchronizing, and returns a status: CITRUS_OK, or a code with a message readable through
 * citrus_last_error_string() (per calling thread). Tensors are caller-owned; nothing here allocates device memory
 * unless an entry point says so. All floating data are float32 unless named otherwise; integer tables are int32.
 *
 * Each declaration names the reference interface it replaces (file:line within cabouman/citrus v0.28.0).
 */
#ifndef CITRUS_GB300_H
#define CITRUS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CITRUS_GB300_ABI_VERSION 1

#define CITRUS_OK 0
#define CITRUS_EINVAL 1   /* bad argument (null pointer, size out of range, unsupported shape) */
#define CITRUS_ELAUNCH 2  /* a kernel launch failed */
#define CITRUS_ETIMEOUT 3 /* a bounded device-side wait ran out (read back from a sync word) */
#define CITRUS_ECUDA 4    /* another CUDA runtime error */

/* ABI version of the loaded library (CITRUS_GB300_ABI_VERSION). */
int citrus_abi_version(void);

/* Message of the last failed call on this host thread ("" if none). */
const char* citrus_last_error_string(void);

/* ------------------------------------------------------------------------------------------------------------------
 * Linear-discontinuous transport sweep.
 * Replaces citrus/scatter_solver/kernels/sweep_kernels.py:265-290 (sweep_planes) and the plane kernel of
 * sweep_kernels.py:172-258.
 *
 * store      [views, 8, Dc, N, 4G] source moments of the chunk, overwritten in place with the angular-fluence moments
 *            (moment order 0, x, y, z per group).
 * mu_cells   [N, G] total attenuation per cell in 1/cm (shared by the views).
 * c          [8, Dc, 3] |Omega_a| / Delta_a of the chunk directions in 1/cm.
 * octant, cell [E] and upstream [E, 3]: the plane-sorted entry tables of the sweep plan (E = 8 N); an upstream index
 *            equal to N marks a vacuum face.
 * plane_offsets_host [num_planes + 1] entry offsets of the planes (host memory).
 * ------------------------------------------------------------------------------------------------------------------ */
int citrus_sweep_planes(float* store, const float* mu_cells, const float* c, const int32_t* octant,
                        const int32_t* cell, const int32_t* upstream, const int64_t* plane_offsets_host,
                        int64_t num_planes, int64_t num_cells, int64_t num_groups, int64_t dc, int64_t views,
                        void* stream);

/* The same sweep as one persistent cooperative launch with a bounded grid barrier between planes.
 * plane_offsets_dev [num_planes + 1] int32 offsets in device memory; sync [4] uint32 device scratch, zeroed on the
 * stream by the call itself; sync[2] is non-zero after the sweep if a barrier wait ran out (the sweep is then
 * invalid and the caller must raise).
 * max_blocks caps the grid (0: as many as fit); timeout_ns bounds every barrier wait; skip_block is -1 (a
 * non-negative value makes that block skip its arrivals, which forces the timeout path for tests). */
int citrus_sweep_persistent(float* store, const float* mu_cells, const float* c, const int32_t* octant,
                            const int32_t* cell, const int32_t* upstream, const int32_t* plane_offsets_dev,
                            int64_t num_planes, int64_t num_cells, int64_t num_groups, int64_t dc, int64_t views,
                            uint32_t* sync, int64_t max_blocks, int64_t timeout_ns, int64_t skip_block, void* stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Small-K matrix products of the sweep and of the image.
 * C[b] (=|+=) A @ B[b] with A [M, K] row-major (lda), B[b] [K, J] row-major (ldb), C[b] [M, J] row-major (ldc),
 * batch b with element strides stride_b, stride_c. Replaces the torch.mm/addmm_ calls of
 * citrus/scatter_solver/transport_sweep.py:524-528 (moment accumulation), source_iteration.py:94-103 (scattering
 * source) and scatter_image.py:1246 (multiple-collision source). Requires J % 4 == 0 and 16-byte aligned rows.
 * ------------------------------------------------------------------------------------------------------------------ */
int citrus_small_k_gemm(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int64_t M,
                        int64_t K, int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c, int32_t accumulate,
                        void* stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Spherical-harmonic moments of the scattering source,
 * T[g, n, k, x] = sum_g' transfer[g', g, l(n), x] phi[g', n, k, x], phi and T through element strides.
 * Replaces citrus/scatter_solver/kernels/scattering_kernels.py:159-252 (scattering_moments).
 * transfer [G_in, G_out, num_legendre, X] contiguous; K = 4 (linear-discontinuous axis) or 1.
 * ------------------------------------------------------------------------------------------------------------------ */
int citrus_scattering_moments(const float* transfer, const float* phi, float* out, int64_t g_in, int64_t g_out,
                              int64_t num_legendre, int64_t num_moments, int64_t k_count, int64_t num_points,
                              int64_t ps_g, int64_t ps_n, int64_t ps_k, int64_t ps_x, int64_t os_g, int64_t os_n,
                              int64_t os_k, int64_t os_x, void* stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Siddon line integrals (exact for voxel-wise constant fields, zero outside the grid box).
 * Replaces the Projectors protocol operations of citrus/scatter_solver/ray_tracing.py:27-115 and their Triton kernels
 * in kernels/ray_tracing_kernels.py:215-1063.
 *
 * volume [V, C] voxel-major (the C channels of a voxel contiguous), V = dims[0] * dims[1] * dims[2] in the flat order
 * (row * cols + col) * slices + slice. box (host) = lower corner (x, y, z) and voxel sizes (dx, dy, dz) in cm; dims
 * (host) = (cols, rows, slices). Outputs are channel-major [C, rays] unless stated.
 * ------------------------------------------------------------------------------------------------------------------ */

/* Generic segments starts[r] -> ends[r] ([R, 3] float32); replaces ray_tracing.line_integrals (ray_tracing.py:205-284). */
int citrus_line_integrals(const float* volume, int64_t channels, const double* box, const int64_t* dims,
                          const float* starts, const float* ends, int64_t num_rays, float* out, void* stream);

/* From the focal spot (host double [3]) to points: explicit float64 points [P, 3] (device), or, with points NULL, the
 * centres of a point grid given by its float64 axes x [cols], y [rows], z [slices] (device) and point_dims (host:
 * rows, cols, slices). Replaces upstream_cumulative / upstream_to_points / primary_project (ray_tracing.py:405-498). */
int citrus_trace_from_source(const float* volume, int64_t channels, const double* box, const int64_t* dims,
                             const double* source, const double* points, const double* axis_x, const double* axis_y,
                             const double* axis_z, const int64_t* point_dims, int64_t num_points, float* out,
                             void* stream);

/* From every voxel centre along each direction omegas[k] ([K, 3]) to the panel, out [K, C, V]; +inf for directions
 * with toward[k] == 0 (uint8 [K], NULL: all toward), 0 beyond the panel. panel (host double [11]) = curved flag,
 * flat-panel centre [3], normal [3], focal spot [3], cylinder radius; diagonal clamps the distance.
 * Replaces downstream_cumulative (ray_tracing.py:501-545, ray_tracing_kernels.py:516-639). */
int citrus_downstream_cumulative(const float* volume, int64_t channels, const double* box, const int64_t* dims,
                                 const float* omegas, const uint8_t* toward, int64_t num_directions,
                                 const double* panel, double diagonal, float* out, void* stream);

/* Line through every pixel centre (pixels [rows, cols, 3]) along each direction, clipped to the box on both sides;
 * field [K or 1, V, C] with field_stride elements between directions (0: shared); out element (k, c, row, col) at
 * k * os_k + c * os_c + row * os_r + col * os_col (any layout, e.g. rows-outer [K, rows, C, cols]).
 * Replaces oblique_project (ray_tracing.py:548-620). */
int citrus_oblique_project(const float* field, int64_t channels, int64_t field_stride, const double* box,
                           const int64_t* dims, const float* omegas, int64_t num_directions, const float* pixels,
                           int64_t num_rows, int64_t num_cols, float* out, int64_t os_k, int64_t os_c, int64_t os_r,
                           int64_t os_col, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CITRUS_GB300_H */
