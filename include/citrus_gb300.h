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

/* Kernels this library has launched in this process (all threads and devices), a counter for measurements; no
 * counterpart in the reference. */
int64_t citrus_launch_count(void);

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

/* citrus_sweep_persistent with the form of its threads chosen by the caller (the autotuner). Every thread solves its
 * lane (entry, direction, group) in all views of the store, with the view-independent part of the cell solve
 * computed once: thread_form 2 or 4 views whose loads a thread issues before their solves, or one view at a
 * time with the registers capped for 5 (1), 6 (3) or 4 (5) blocks of 256 threads per SM (0: 1). */
int citrus_sweep_persistent_config(float* store, const float* mu_cells, const float* c, const int32_t* octant,
                                   const int32_t* cell, const int32_t* upstream, const int32_t* plane_offsets_dev,
                                   int64_t num_planes, int64_t num_cells, int64_t num_groups, int64_t dc,
                                   int64_t views, uint32_t* sync, int64_t max_blocks, int32_t thread_form,
                                   int64_t timeout_ns, int64_t skip_block, void* stream);

/* The accumulator sweep of one chunk in the tiled schedule (no counterpart in the reference, whose sweep_planes,
 * citrus/scatter_solver/kernels/sweep_kernels.py:265-290, launches once per plane): the same lanes and the same store
 * as citrus_sweep_planes, bit for bit, in one cooperative launch whose grid barrier runs once per tile diagonal. The
 * entries (octant, cell, upstream; num_cells for vacuum) are ordered by task (one tile of T^3 cells of one octant) and
 * sub-plane; sub_offsets [tasks, num_sub + 1] (num_sub = 3 T - 2) holds each task's sub-plane entry ranges and
 * diagonal_offsets [num_diagonals + 1] each diagonal's task range (int32 device tables). A block sweeps one task for
 * dirs_per_block directions of the chunk (1..dc) through its sub-planes with block barriers. thread_form: 1 one view
 * at a time, 2 the loads of two views before their solves. sync: 4 device words (sync[2] != 0 after the launch: a
 * barrier wait ran past timeout_ns and the store is invalid); skip_block >= 0 is a test hook (that block never
 * arrives). */
int citrus_sweep_tiled(float* store, const float* mu_cells, const float* c, const int32_t* octant, const int32_t* cell,
                       const int32_t* upstream, const int32_t* diagonal_offsets, const int32_t* sub_offsets,
                       int64_t num_diagonals, int64_t num_sub, int64_t num_cells, int64_t num_groups, int64_t dc,
                       int64_t views, int64_t dirs_per_block, uint32_t* sync, int64_t max_blocks, int64_t thread_form,
                       int64_t timeout_ns, int64_t skip_block, void* stream);

/* The persistent sweep without any allocation: no counterpart in the reference, which always runs the sweep through
 * torch's allocator. The barrier words and the plane offsets live in a static device array of this library (33 KB
 * per device, at most 8191 planes, i.e. R + C + S - 2 <= 8191; more planes return CITRUS_EINVAL). The call clears
 * the barrier words and copies plane_offsets_host [num_planes + 1] (int32, host memory; a pinned buffer must stay
 * unchanged until the stream reaches the copy) into the array on the stream, then launches. The first call on each
 * device looks the array's address up (that device must be current); make it before any stream capture. The address
 * is kept for the life of the process: after cudaDeviceReset (or any teardown of the device's primary context) the
 * entry point must not be called again in that process. A pageable plane_offsets_host has been read by the time the
 * call returns. Calls on one device share the array, so calls that overlap in time (two streams, two host threads)
 * race and must not be made. timeout_word, when not NULL, receives the barrier error word on the stream (non-zero: a wait ran out and
 * the store is invalid); a pageable host word makes the call wait for the sweep. */
int citrus_sweep_persistent_static(float* store, const float* mu_cells, const float* c, const int32_t* octant,
                                   const int32_t* cell, const int32_t* upstream, const int32_t* plane_offsets_host,
                                   int64_t num_planes, int64_t num_cells, int64_t num_groups, int64_t dc,
                                   int64_t views, uint32_t* timeout_word, int64_t timeout_ns, void* stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Small-K matrix products of the sweep and of the image.
 * C[b] (=|+=) A @ B[b] with A [M, K] row-major (lda), B[b] [K, J] row-major (ldb), C[b] [M, J] row-major (ldc),
 * batch b with element strides stride_b, stride_c. Replaces the torch.mm/addmm_ calls of
 * citrus/scatter_solver/transport_sweep.py:524-528 (moment accumulation), source_iteration.py:94-103 (scattering
 * source) and scatter_image.py:1246 (multiple-collision source). Rows that are 16-byte aligned with J % 4 == 0 move
 * as float4; any other shape takes the element-wise path.
 * ------------------------------------------------------------------------------------------------------------------ */
int citrus_small_k_gemm(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc, int64_t M,
                        int64_t K, int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c, int32_t accumulate,
                        void* stream);

/* The same product with its kernel chosen by the caller (the autotuner): variant 0 = the shape rule of
 * citrus_small_k_gemm, 1 = the streaming forms (columns of B in registers for K <= 64, rows of C in registers for
 * M <= 64), 2 = the shared-memory tiled kernel with tile_rows groups of 8 rows per CTA (1-6, 8, 12, 16; 0 = fit M). */
int citrus_small_k_gemm_config(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
                               int64_t M, int64_t K, int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c,
                               int32_t accumulate, int32_t variant, int32_t tile_rows, void* stream);

/* The source of an accumulator sweep in one pass: C[b] = A B[b] + the quadruples (F[b], 0, 0, 0), i.e. the source
 * expansion Y @ T (transport_sweep.py:524, source_iteration.py:94) added to the first-collision LD moments of one
 * point per cell given by their means F[b] [M, J / 4] (ldf floats per row, stride_f floats between batches), without
 * reading C. The float32 column-stationary form of citrus_small_k_gemm: the same products in the same order, so C
 * equals that of citrus_first_collision_moments followed by an accumulating citrus_small_k_gemm. K <= 64, J a multiple
 * of 4, B and C in 8-byte aligned column pairs. */
int citrus_source_expansion_first(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
                                  const float* F, int64_t ldf, int64_t M, int64_t K, int64_t J, int64_t batch,
                                  int64_t stride_b, int64_t stride_c, int64_t stride_f, void* stream);

/* The same product on the tcgen05 tensor cores, M <= 128 and K <= 128: each float32 operand is split into a bfloat16
 * high part and a bfloat16 low part (x - hi), the product accumulated in float32 as A_hi B_hi + A_hi B_lo + A_lo B_hi
 * (relative error ~1e-5 of the largest term). error_word (NULL: none), when given, is set to 1 if a wait for the
 * tensor cores ran out (the result is then invalid). The BF16 hi/lo scattering-source contraction of the mixed-
 * precision configuration; no counterpart in the reference, which contracts in float32 (transport_sweep.py:524-528,
 * source_iteration.py:94-103, scatter_image.py:1246). */
int citrus_small_k_gemm_bf16x3(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
                               int64_t M, int64_t K, int64_t J, int64_t batch, int64_t stride_b, int64_t stride_c,
                               int32_t accumulate, uint32_t* error_word, void* stream);

/* The source of an accumulator sweep (citrus_source_expansion_first: C[b] = A B[b] + the quadruples (F[b], 0, 0, 0),
 * C written without being read) on the tcgen05 tensor cores in the same bfloat16 hi/lo split, M <= 128, K <= 128, J a
 * multiple of 4: the scattering-source expansion Y @ T of transport_sweep.py:524 and source_iteration.py:94-103 in
 * the mixed precision, with the first-collision means added in its epilogue. error_word as above. */
int citrus_source_expansion_first_bf16x3(const float* A, int64_t lda, const float* B, int64_t ldb, float* C,
                                         int64_t ldc, const float* F, int64_t ldf, int64_t M, int64_t K, int64_t J,
                                         int64_t batch, int64_t stride_b, int64_t stride_c, int64_t stride_f,
                                         uint32_t* error_word, void* stream);

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

/* From every voxel centre along each direction omegas[k] ([K, 3]) to the panel, out element (k, c, v) at
 * k * os_k + c * os_c + v * os_v (the reference's [K, C, V]: C V, V, 1; voxel-major [K, V, C]: V C, 1, C); +inf for
 * directions with toward[k] == 0 (uint8 [K], NULL: all toward), 0 beyond the panel. panel (host double [11]) = curved flag,
 * flat-panel centre [3], normal [3], focal spot [3], cylinder radius; diagonal clamps the distance.
 * crossings: device scratch of crossings_words >= 3 (nx + ny + nz) K int32 words for the per-direction crossing
 * tables (every ray starts at a voxel centre, so one merged sequence of plane crossings serves all rays of a
 * direction), or NULL for an independent walk per ray.
 * Replaces downstream_cumulative (ray_tracing.py:501-545, ray_tracing_kernels.py:516-639). */
int citrus_downstream_cumulative(const float* volume, int64_t channels, const double* box, const int64_t* dims,
                                 const float* omegas, const uint8_t* toward, int64_t num_directions,
                                 const double* panel, double diagonal, float* out, int64_t os_k, int64_t os_c,
                                 int64_t os_v, int32_t* crossings, int64_t crossings_words, void* stream);

/* The crossing tables of citrus_downstream_cumulative for num_directions directions at once ([K, 3 (nx + ny + nz)]
 * int32: per direction the distances of the plane crossings from a voxel centre, the flat-index steps and the first
 * crossing of each axis), and the downstream trace reading such prebuilt tables instead of building them: a
 * direction set whose tables are kept (one build per view's direction set) needs no build per chunk. */
int citrus_crossing_tables(const double* box, const int64_t* dims, const float* omegas, int64_t num_directions,
                           int32_t* crossings, int64_t crossings_words, void* stream);
int citrus_downstream_cumulative_tables(const float* volume, int64_t channels, const double* box,
                                        const int64_t* dims, const float* omegas, const uint8_t* toward,
                                        int64_t num_directions, const double* panel, double diagonal, float* out,
                                        int64_t os_k, int64_t os_c, int64_t os_v, const int32_t* crossings,
                                        int64_t crossings_words, void* stream);

/* Line through every pixel centre (float64 pixels [rows, cols, 3]) along each direction, clipped to the box on both
 * sides (float64 set-up);
 * field [K or 1, V, C] with field_stride elements between directions (0: shared); out element (k, c, row, col) at
 * k * os_k + c * os_c + row * os_r + col * os_col (any layout, e.g. rows-outer [K, rows, C, cols]).
 * Replaces oblique_project (ray_tracing.py:548-620). */
int citrus_oblique_project(const float* field, int64_t channels, int64_t field_stride, const double* box,
                           const int64_t* dims, const float* omegas, int64_t num_directions, const double* pixels,
                           int64_t num_rows, int64_t num_cols, float* out, int64_t os_k, int64_t os_c, int64_t os_r,
                           int64_t os_col, void* stream);

/* The same with a caller-owned device scratch of at least citrus_oblique_scratch_bytes(num_directions) bytes: one
 * thread per direction forms the direction's float64 set-up constants there first, and every block of the direction
 * reads them instead of forming them itself (the same values; NULL scratch: formed per block). */
int64_t citrus_oblique_scratch_bytes(int64_t num_directions);
int citrus_oblique_project_scratch(const float* field, int64_t channels, int64_t field_stride, const double* box,
                                   const int64_t* dims, const float* omegas, int64_t num_directions,
                                   const double* pixels, int64_t num_rows, int64_t num_cols, float* out, int64_t os_k,
                                   int64_t os_c, int64_t os_r, int64_t os_col, void* direction_scratch,
                                   int64_t scratch_bytes, void* stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Uncollided fluence and first-collision source.
 * ------------------------------------------------------------------------------------------------------------------ */

/* T[g, p] = factor[p] * sum_{e: fine_group[e] = g} fine_weight[e] exp(-sum_m fine_mu[m, e] path[m, p]
 *           - filter_mu[e] filter_path[p]); path [M', P], fine_mu [M', E]; filter and factor optional (NULL).
 * Replaces cross_sections.group_transmission (cross_sections.py:797-883, transmission_kernels.py:187-275). */
int citrus_group_transmission(const float* path, int64_t num_materials, int64_t num_points, const float* fine_mu,
                              const float* fine_weight, const int32_t* fine_group, int64_t num_fine,
                              int64_t num_groups, const float* filter_path, const float* filter_mu,
                              const float* factor, float* out, void* stream);

/* Focal-spot weight b(Omega) (1 where the ray from the focal spot meets the collimated field), divided by |r - r0|^2
 * when asked, at explicit float64 points [P, 3] or at the centres of a point grid (float64 axes, point_dims host).
 * field (host double [23]) = curved flag, focal spot [3], panel centre [3], u_hat [3], v_hat [3], n_hat [3],
 * source-detector distance, channel and row offsets, panel half widths (u, v), field margins (u, v).
 * Replaces SourceModel.angular_weight (source.py:289-382) and the 1 / |r - r0|^2 of uncollided.py:193-197. */
int citrus_source_weight(const double* field, const double* points, const double* axis_x, const double* axis_y,
                         const double* axis_z, const int64_t* point_dims, int64_t num_points,
                         int32_t divide_by_distance_squared, float* out, void* stream);

/* The same weight with the rest of the source model: b(Omega) is the field weight (1 inside the field, past its edge
 * the off-focal fraction of the distance to the field rectangle, linear between off_focal_nodes [n] with values
 * off_focal_values [n], 0 past the last node; no table: 0) times the emission profile [rows, channels] interpolated
 * bilinearly at the ray's panel point and held at the outermost pixel centres; with a filter thickness
 * [thickness_rows = 1 | rows, channels] in cm, filter_path_out [P] receives filter_density * thickness interpolated
 * the same way (g/cm^2). panel (host double [6]) = rows, channels, row pitch, channel pitch, row offset, channel
 * offset. All tables are float64 device arrays; null profile, thickness and off-focal nodes leave them out.
 * Replaces SourceModel.angular_weight / filter_path (source.py:289-430) with panel_interpolate (source.py:484-510). */
int citrus_source_field(const double* field, const double* panel, const double* profile, const double* thickness,
                        int64_t thickness_rows, double filter_density, const double* off_focal_nodes,
                        const double* off_focal_values, int64_t num_off_focal, const double* points,
                        const double* axis_x, const double* axis_y, const double* axis_z, const int64_t* point_dims,
                        int64_t num_points, int32_t divide_by_distance_squared, float* out, float* filter_path_out,
                        void* stream);

/* Shared arguments of the first-collision kernels: rho [M, V] densities on the point grid, phi [G, V] uncollided
 * fluence, axes = float32 point coordinates x [cols], y [rows], z [slices] back to back, point_dims (host) = rows,
 * cols, slices, focal_spot (host double [3]), table [M, N_eta, G_out, G_in] per-steradian transfer (zero for
 * G_in > G_out) on the uniform cosine nodes eta_lo .. eta_hi, omegas [K, 3].
 *
 * S_FC [K, G, V] at the points (uncollided.py:200-308, uncollided_kernels.py:488-550). */
int citrus_first_collision_source(const float* rho, int64_t num_materials, const float* phi, int64_t num_groups,
                                  const float* axes, const int64_t* point_dims, const double* focal_spot,
                                  const float* table, int64_t num_eta, double eta_lo, double eta_hi,
                                  const float* omegas, int64_t num_directions, float* out, void* stream);

/* LD moments (mean, x, y, z slopes) of the corrected source scale (1 + beta cos) S_FC over the points_per_cell^3
 * points of each transport cell, cell-major into out [K, NC, G, 4] with out_direction_stride floats between
 * directions (the sweep's store). With cache (from citrus_first_collision_correction) S_FC of chunk direction k is
 * read from cache row cache_index[k] (int32 [K]) instead of evaluated from the table again.
 * Replaces first_collision_moments_at_directions (uncollided.py:464-511, uncollided_kernels.py:552-634). */
int citrus_first_collision_moments(const float* rho, int64_t num_materials, const float* phi, int64_t num_groups,
                                   const float* axes, const int64_t* point_dims, int64_t points_per_cell,
                                   const double* focal_spot, const float* table, int64_t num_eta, double eta_lo,
                                   double eta_hi, const float* omegas, int64_t num_directions, const float* scale,
                                   const float* beta, const float* cache, const int32_t* cache_index, float* out,
                                   int64_t out_direction_stride, void* stream);

/* The means of the first-collision LD moments at one point per cell (points_per_cell 1, where the slopes vanish),
 * from the S_FC that citrus_first_collision_correction cached (cache row cache_index[k] for chunk direction k): out
 * [K, NC, G] with out_direction_stride floats between directions, the first components of the quadruples that
 * citrus_first_collision_moments writes; read by citrus_source_expansion_first. Part of
 * first_collision_moments_at_directions (uncollided.py:464-511, uncollided_kernels.py:552-634). */
int citrus_first_collision_means(int64_t num_groups, const float* axes, const int64_t* point_dims,
                                 const double* focal_spot, const float* omegas, int64_t num_directions,
                                 const float* scale, const float* beta, const float* cache, const int32_t* cache_index,
                                 float* out, int64_t out_direction_stride, void* stream);

/* Sampling correction: quadrature sums I0, I1, I2 over the K sweep directions (weights [K]) and exact moments E0, E1
 * from moments [M, 2, G_out, G_in] (Legendre l = 0, 1), optionally stored in sums [5, G, V], and the float64 factors
 * scale, beta [G, V] (uncollided.py:357-461, 538-636, uncollided_kernels.py:636-710). With cache (NULL: none) the
 * source values S_FC are kept, cache [K, G, V], for citrus_first_collision_moments. The quadrature sums run over
 * the directions in the order of their cosine with each block's first point (a rounding-level difference from the
 * reference's direction order). */
int citrus_first_collision_correction(const float* rho, int64_t num_materials, const float* phi, int64_t num_groups,
                                      const float* axes, const int64_t* point_dims, const double* focal_spot,
                                      const float* table, int64_t num_eta, double eta_lo, double eta_hi,
                                      const float* omegas, const float* weights, int64_t num_directions,
                                      const float* moments, float* sums, float* scale, float* beta, float* cache,
                                      void* stream);

/* Attenuated total emission of the collapsed-cone image: (S_FC + multiple[k, cell, g]) exp(-max(0, tau[k, cell, g]
 * - mu[g, cell] omega . (r - r_cell))) written voxel-major out [K, V, G], or with signal_weight [K, G] its weighted
 * group sum [K, V]; height_sums [K, 2] = (sum e, sum e h) with the panel heights h [V] (NULL: 0), summed in a fixed
 * order through partial [K, ceil(V / 32), 2] (device scratch of partial_capacity floats). With tau_mu [TM, G]
 * (NULL: none), tau holds material path lengths [K, NC, TM] (TM = tau_materials, the downstream trace of the cell
 * densities) and the optical depth is tau[k, cell, g] = sum_m tau_mu[m, g] P[k, cell, m].
 * Replaces attenuated_emission (uncollided_kernels.py:712-795, 1138-1205) and supervoxel_subpoint_emission
 * (scatter_image.py:829-874). */
int citrus_attenuated_emission(const float* rho, int64_t num_materials, const float* phi, int64_t num_groups,
                               const float* axes, const int64_t* point_dims, int64_t points_per_cell,
                               const double* point_deltas, const double* focal_spot, const float* table,
                               int64_t num_eta, double eta_lo, double eta_hi, const float* omegas,
                               int64_t num_directions, const float* tau, const float* tau_mu, int64_t tau_materials,
                               const float* mu, const float* multiple, const float* heights,
                               const float* signal_weight, float* out, float* partial, int64_t partial_capacity,
                               float* height_sums, void* stream);

/* The same emission with the multiple-collision source formed in registers, S_MC[k, g, cell] = sum_n
 * harmonics[k, n] moments[n, cell, g] (harmonics [K, num_moments], moments [num_moments, NC, G], num_moments <= 64),
 * instead of read from a [K, NC, G] buffer. Replaces the product torch.mm(harmonics, moments) of
 * scatter_image.py:1246 together with attenuated_emission (uncollided_kernels.py:1138-1205). */
int citrus_attenuated_emission_moments(const float* rho, int64_t num_materials, const float* phi, int64_t num_groups,
                                       const float* axes, const int64_t* point_dims, int64_t points_per_cell,
                                       const double* point_deltas, const double* focal_spot, const float* table,
                                       int64_t num_eta, double eta_lo, double eta_hi, const float* omegas,
                                       int64_t num_directions, const float* tau, const float* tau_mu,
                                       int64_t tau_materials, const float* mu, const float* harmonics,
                                       const float* moments, int64_t num_moments,
                                       const float* heights, const float* signal_weight, float* out, float* partial,
                                       int64_t partial_capacity, float* height_sums, void* stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Finite-cone footprint and accumulation of the collapsed-cone image (scatter_image.py:897-1135, 1234-1323).
 * ------------------------------------------------------------------------------------------------------------------ */

/* Box blur along one axis of length N: out[k, line, c] = sum_j B_k[c, j] in[k, line, j] with the overlap weights of
 * scatter_image.box_matrix (scatter_image.py:952-1007), element strides for directions, lines and pixels. The width
 * in pixels is widths[k], or, with widths NULL, hbar_k cell_width[k, axis] / pitch with the mean height
 * hbar_k = height_sums[k, 1] / height_sums[k, 0] (center_height where the sum vanishes) (scatter_image.py:1079-1135). */
int citrus_box_blur(const float* in, float* out, int64_t num_directions, int64_t lines, int64_t length, int64_t is_k,
                    int64_t is_l, int64_t is_p, int64_t os_k, int64_t os_l, int64_t os_p, const float* widths,
                    const float* height_sums, const float* cell_width, int32_t axis, double pitch,
                    double center_height, void* stream);

/* Dense overlap matrices [K, N, N] of the footprint filter (scatter_image.box_matrix, scatter_image.py:952-1007). */
int citrus_box_matrix(const float* widths, int64_t num_directions, int64_t length, float* out, void* stream);

/* out[k, r, c] = sum_g image[k, r, g, c] weights[k, g, c] of rows-outer images (weight_cols 1: one weight per
 * (k, g)) (the signal weighting of scatter_image.py:1290-1310). */
int citrus_weighted_group_sum(const float* image, const float* weights, int64_t num_directions, int64_t rows,
                              int64_t groups, int64_t cols, int64_t weight_cols, float* out, void* stream);

/* accumulator[g, r, c] (+)= sum_k weights[k, g, r | 0, c | 0] image[k, g, r, c] with image element strides (the
 * accumulation of the full images, DirectionSetContext.accumulate, scatter_image.py:340-371). */
int citrus_weighted_direction_sum(const float* image, int64_t num_directions, int64_t groups, int64_t rows,
                                  int64_t cols, int64_t is_k, int64_t is_g, int64_t is_r, int64_t is_c,
                                  const float* weights, int64_t weight_rows, int64_t weight_cols, float* accumulator,
                                  int32_t accumulate, void* stream);

/* Signal behind an anti-scatter grid that varies over the panel: accumulator[g, r, c] (per_group) or
 * accumulator[r, c] (+)= sum_k W image[k, g, r, c] (image element strides), with
 * W = weights[k, g, c | 0] * row_weights[k, g, r] (null: 1) * prod_s T_s(g, theta1_s, theta2_s) where, for each of
 * num_septa <= 2 sets of septa, theta_i = theta_channels_s[i, k, c] + theta_pixels_s[i, r, c] (float32, [2, K, cols]
 * and [2, rows, cols]) and T_s is tables_s [G, T1, T2] interpolated bilinearly at |theta1|, |theta2| in the nodes
 * theta1_nodes_s [T1], theta2_nodes_s [T2], clamped to the end nodes. The septa arguments are host arrays of
 * num_septa device pointers (and host counts). groups <= 32.
 * Replaces DirectionSetContext.pixel_signal_weight and the signal accumulation with _PixelGrid and signal_row_weight
 * (scatter_image.py:340-389, 437-486, 1290-1313). */
int citrus_grid_signal_sum(const float* image, int64_t num_directions, int64_t groups, int64_t rows, int64_t cols,
                           int64_t is_k, int64_t is_g, int64_t is_r, int64_t is_c, const float* weights,
                           int64_t weight_cols, const float* row_weights, int64_t num_septa,
                           const float* const* theta_channels, const float* const* theta_pixels,
                           const float* const* tables, const float* const* theta1_nodes, const int64_t* num_theta1,
                           const float* const* theta2_nodes, const int64_t* num_theta2, float* accumulator,
                           int32_t per_group, int32_t accumulate, void* stream);

/* accumulator[p] (+)= sum_k image[k * stride_k + p], directions in order (scatter_image.py:1289-1319). */
int citrus_sum_directions(const float* image, int64_t num_directions, int64_t pixels, int64_t stride_k,
                          float* accumulator, int32_t accumulate, void* stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Per-view accumulator storage: the linear-discontinuous cell mean in scaled float16 (citrus/citrus.py:620-720,
 * StateStore.put / get).
 * ------------------------------------------------------------------------------------------------------------------ */

/* data [groups, moments, cells] float16 = mean / scale and scale [groups, moments] = max |mean| / 2^14 (1 where the
 * maximum is 0), from the cell-mean component of an accumulator at g s_g + n s_n + cell s_x. */
int citrus_state_encode(const float* accumulator, int64_t groups, int64_t moments, int64_t cells, int64_t s_g,
                        int64_t s_n, int64_t s_x, uint16_t* data, float* scale, void* stream);

/* The accumulator back, element (g, n, k, cell) at g o_g + n o_n + k o_k + cell o_x: k = 0 the decoded cell mean,
 * k = 1..3 (the slopes) zero. */
int citrus_state_decode(const uint16_t* data, const float* scale, int64_t groups, int64_t moments, int64_t cells,
                        float* accumulator, int64_t o_g, int64_t o_n, int64_t o_k, int64_t o_x, void* stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Density model of the CITRUS loop (citrus/utilities.py:710-799, attenuation_to_density).
 * out [V] = density of the material in bracketing slot `slot` of X [V] (1/cm): mu, mass, nominal [M] float32 are the
 * nominal attenuations, mass attenuations and nominal densities of the materials sorted by nominal attenuation.
 * ------------------------------------------------------------------------------------------------------------------ */
int citrus_attenuation_to_density(const float* X, int64_t num_voxels, const float* mu, const float* mass,
                                  const float* nominal, int64_t num_materials, int64_t slot, float* out, void* stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Learned higher-order proposal: the layers of a 3D U-Net on the transport cells and their gradients. The reference
 * has no counterpart (its cold start is an empty accumulator, citrus/citrus.py:70-87 and :192-247); these entry points
 * train and run the network that proposes the higher collision orders of that accumulator.
 * Volumes are NCDHW float32 [batch, C, depth, height, width]; weights bfloat16 bit patterns [C_out, C_in, k, k, k]
 * (k = 1 or 3, zero padding k / 2); float32 accumulation.
 * ------------------------------------------------------------------------------------------------------------------ */

/* out = act(bias + w * [A, up(B)]): input channels [0, channels_a) from in_a, [channels_a, channels_a + channels_b)
 * from in_b (at half resolution, nearest 2x upsampling, when b_upsampled); act = ReLU when relu != 0. */
int citrus_conv3d_forward(const float* in_a, int64_t channels_a, const float* in_b, int64_t channels_b,
                          int32_t b_upsampled, const uint16_t* weight, const float* bias, float* out,
                          int64_t channels_out, int64_t batch, int64_t depth, int64_t height, int64_t width,
                          int32_t kernel_size, int32_t relu, void* stream);

/* citrus_conv3d_forward with the kernel chosen by the caller (the autotuner): variant 1 = the FP32 SIMT kernel
 * (a 4 x 8 x 8 voxel brick x 16 output channels per CTA), 2 (and 0) = the implicit GEMM on the tcgen05 tensor cores
 * (128 voxels x up to 256 output channels per CTA, every input split into bfloat16 high and low parts against the
 * exact bfloat16 weights, float32 accumulation in tensor memory). error_word (NULL: none) is set to 1 if a wait for
 * the tensor cores ran out (the output is then invalid). */
int citrus_conv3d_forward_config(const float* in_a, int64_t channels_a, const float* in_b, int64_t channels_b,
                                 int32_t b_upsampled, const uint16_t* weight, const float* bias, float* out,
                                 int64_t channels_out, int64_t batch, int64_t depth, int64_t height, int64_t width,
                                 int32_t kernel_size, int32_t relu, int32_t variant, uint32_t* error_word,
                                 void* stream);

/* Input gradient of citrus_conv3d_forward: grad_a (channels_a, times (mask_a > 0) when mask_a is set) and grad_b
 * (channels_b, at full resolution, before the upsampling's backward pass) from grad_out (channels_out). */
int citrus_conv3d_backward_input(const float* grad_out, int64_t channels_out, const uint16_t* weight, float* grad_a,
                                 int64_t channels_a, const float* mask_a, float* grad_b, int64_t channels_b,
                                 int64_t batch, int64_t depth, int64_t height, int64_t width, int32_t kernel_size,
                                 void* stream);

/* citrus_conv3d_backward_input with the kernel chosen by the caller (variants as citrus_conv3d_forward_config). */
int citrus_conv3d_backward_input_config(const float* grad_out, int64_t channels_out, const uint16_t* weight,
                                        float* grad_a, int64_t channels_a, const float* mask_a, float* grad_b,
                                        int64_t channels_b, int64_t batch, int64_t depth, int64_t height,
                                        int64_t width, int32_t kernel_size, int32_t variant, uint32_t* error_word,
                                        void* stream);

/* Partial sums the weight gradient uses for these sizes: it wants partial_capacity >= splits * C_out * C_in * k^3
 * floats (fewer splits, or none, with less). */
int64_t citrus_conv3d_weight_grad_splits(int64_t channels_out, int64_t channels_a, int64_t channels_b, int64_t batch,
                                         int64_t depth, int64_t height, int64_t width, int32_t kernel_size);

/* grad_weight [C_out, C_in, k^3] and grad_bias [C_out] (null: skipped) of citrus_conv3d_forward, reduced over the
 * batch and the voxels in a fixed order. */
int citrus_conv3d_backward_weight(const float* grad_out, int64_t channels_out, const float* in_a, int64_t channels_a,
                                  const float* in_b, int64_t channels_b, int32_t b_upsampled, float* grad_weight,
                                  float* grad_bias, int64_t batch, int64_t depth, int64_t height, int64_t width,
                                  int32_t kernel_size, float* partial, int64_t partial_capacity, void* stream);

/* 2x2x2 average pooling of [batch_channels, depth, height, width] (even sizes) and its backward pass:
 * grad_in = ((accumulate ? grad_in : 0) + grad_out / 8 at the parent) * (mask > 0 when mask is set). */
int citrus_avg_pool2(const float* in, float* out, int64_t batch_channels, int64_t depth, int64_t height,
                     int64_t width, void* stream);
int citrus_avg_pool2_backward(const float* grad_out, float* grad_in, const float* mask, int32_t accumulate,
                              int64_t batch_channels, int64_t depth, int64_t height, int64_t width, void* stream);

/* Backward pass of the nearest 2x upsampling: grad_coarse [batch_channels, depth, height, width] = sum of the eight
 * children in grad_fine, times (mask_coarse > 0) when mask_coarse is set. */
int citrus_upsample2_backward(const float* grad_fine, const float* mask_coarse, float* grad_coarse,
                              int64_t batch_channels, int64_t depth, int64_t height, int64_t width, void* stream);

/* grad = 2 (pred - target) / n and partial[block] = the squared errors of each block of 256 elements. */
int citrus_mse(const float* pred, const float* target, int64_t n, float* grad, float* partial,
               int64_t partial_capacity, void* stream);

/* One Adam step (bias-corrected, step >= 1) of float32 parameters; param_bf16 (optional) receives their bfloat16
 * rounding. */
int citrus_adam(float* param, const float* grad, float* m, float* v, uint16_t* param_bf16, int64_t n, double lr,
                double beta1, double beta2, double eps, int64_t step, void* stream);

/* dst = bfloat16 rounding (to nearest even) of src. */
int citrus_to_bf16(const float* src, uint16_t* dst, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CITRUS_GB300_H */
