/*
 * lyem.h -- C ABI of the GB300 raycasting + frequency-domain propagation library
 * (liblyem_gpu.so, built from lyceanem-python_gb300/csrc).
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and returns
 * an int status (LYEM_OK = 0).  No entry point calls exit() or traps the GPU.
 *
 * Two families:
 *   lyem_*     device-pointer entry points, stream-ordered on the cudaStream_t
 *              passed as `stream` (NULL = legacy default stream).  They never
 *              allocate: scratch space is passed in by the caller, sized by the
 *              matching *_workspace() query.
 *   lyem_em_*  host-buffer mirrors of the four functions of the reference's
 *              pybind11 module `lyceanem.em` (lyceanem/src/frequency_domain_models.cu:314-320):
 *              same arguments in the same order, host arrays in, host array
 *              out, synchronous.  They allocate and free device memory per
 *              call, as the reference does.
 *
 * Layouts: points are [n,3] float32; complex 3-vectors are [n,6] float32
 * interleaved (x.re, x.im, y.re, y.im, z.re, z.im), which is numpy/torch
 * complex64 [n,3]; packed triangles are [n_tris,12] float32 (v0, 0, e1, 0,
 * e2, 0) with e1 = v1 - v0, e2 = v2 - v0.
 */
#ifndef LYEM_H_
#define LYEM_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define LYEM_API __attribute__((visibility("default")))
#else
#define LYEM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

enum {
    LYEM_OK = 0,
    LYEM_ERR_INVALID = 1,  /* bad argument: null pointer, negative or inconsistent size */
    LYEM_ERR_CUDA = 2,     /* a CUDA runtime call failed (see lyem_last_cuda_error) */
    LYEM_ERR_NOMEM = 3,    /* device allocation failed (lyem_em_* only) */
    LYEM_ERR_TIMEOUT = 4,  /* a bounded device-side wait expired */
    LYEM_ERR_OVERFLOW = 5, /* a size exceeds the 32-bit index range of a buffer */
    LYEM_ERR_WORKSPACE = 6 /* workspace smaller than the *_workspace() query */
};

/* Version of this ABI (major*10000 + minor*100 + patch). */
LYEM_API int lyem_version(void);
/* Static description of a status code. */
LYEM_API const char *lyem_status_string(int status);
/* cudaError_t of the last failing CUDA call made by this library (0 if none). */
LYEM_API int lyem_last_cuda_error(void);
/* Number of kernels this library has launched in this process so far (all
 * entry points, all threads); the difference across a region counts its launches. */
LYEM_API uint64_t lyem_kernel_launches(void);
/* Calibration probe with no counterpart in the reference: runs a dependent-FMA
 * loop on every SM (iterations per thread, >= 16) and reports the achieved FP32
 * FMA lane-operations per second, the denominator of the visibility roofline. */
LYEM_API int lyem_fp32_fma_probe(int64_t iterations, double *fma_per_second, void *stream);
/* Synchronises `stream`, then reads and clears the library's device error word
 * (bit 0: a bounded wait expired; bit 1: an index check failed).  Returns
 * LYEM_ERR_TIMEOUT if bit 0 was set. */
LYEM_API int lyem_device_errors(void *stream, uint32_t *flags_out);

/* ---------------------------------------------------------------- geometry */

/* Packs a triangle mesh into [n_tris,12] float32 (v0, e1, e2).
 * Replaces the per-test vertex gather tri_vertex[idx.y] - tri_vertex[idx.x]
 * (lyceanem/src/raycasting_brute_force.cuh:39-43) and convertTriangles
 * (lyceanem/raycasting/rayfunctions.py:531-557).  Index values are checked;
 * an out-of-range index sets device error bit 1 and packs a degenerate triangle. */
LYEM_API int lyem_pack_triangles(const float *d_verts, int64_t n_verts, const int32_t *d_idx, int64_t n_tris,
                                 float *d_tris, void *stream);

/* Axis-aligned bounds of packed triangles: d_bounds6 = (xmin, ymin, zmin, xmax, ymax, zmax).
 * Replaces the host min/max of Tile_acceleration_structure.__init__
 * (lyceanem/models/acceleration_structures.py:55-61). */
LYEM_API int lyem_tris_bounds(const float *d_tris, int64_t n_tris, float *d_bounds6, void *stream);

/* Host helper: grid geometry for packed-triangle bounds.  cell <= 0 picks a
 * cell size giving about two cells per triangle.  The box is the bounds
 * padded by 2*pad (pad = 1e-3*cell). */
LYEM_API int lyem_grid_plan(const float *bounds6, int64_t n_tris, float cell, float *origin3_out,
                            float *cell_out, int32_t *dims3_out);

/* Uniform-grid build, phase 1: per-triangle reference counts over the cells
 * its padded box overlaps, and their exclusive scan (d_tri_offsets has
 * n_tris+1 entries; d_tri_offsets[n_tris] is the total).  d_total_refs (one
 * int64) receives the exact 64-bit total.  Replaces triangle_counter_kernel /
 * count_triangles_in_bin (lyceanem/src/terrain_acceleration_build.cuh:57-134, 287-293)
 * without its device asserts. */
LYEM_API size_t lyem_grid_count_workspace(int64_t n_tris);
LYEM_API int lyem_grid_count(const float *d_tris, int64_t n_tris, const float *origin3, float cell,
                             const int32_t *dims3, int32_t *d_tri_offsets, int64_t *d_total_refs, void *d_ws,
                             size_t ws_bytes, void *stream);

/* Uniform-grid build, phase 2: emits (cell, triangle) keys, radix-sorts them
 * by cell (stable, so triangles are ascending within a cell), writes the cell
 * ranges d_cell_start[ncells+1], the triangles in cell order
 * d_cell_tris[n_refs,12] and the traversal's cell table d_cell_box[ncells,16]
 * (16-byte aligned).  Within a cell the triangles are split by the axis-aligned
 * plane (k/8 of the cell on one axis, k = 1..7) of least surface-area cost
 * into child A (centroid below) then child B, each in ascending triangle order; the record is (loA.xyz, first ref,
 * hiA.xyz, first ref of B, loB.xyz, first ref of B, hiB.xyz, end ref), refs
 * stored as int32 bits, each [lo, hi] the box of the child's triangles (padded
 * as for the binning) within the cell widened by two pads; a segment that
 * misses a child's box skips that child's triangles.  Replaces bin_triangles_kernel_precounted /
 * compute_bin_offsets / insert_triangle_in_bin
 * (lyceanem/src/terrain_acceleration_build.cuh:135-205, 349-368) and the host
 * prefix sum of lyceanem/src/frequency_domain_models.cu:118-123. */
LYEM_API size_t lyem_grid_fill_workspace(int64_t n_refs, int64_t n_cells);
LYEM_API int lyem_grid_fill(const float *d_tris, int64_t n_tris, const float *origin3, float cell,
                            const int32_t *dims3, const int32_t *d_tri_offsets, int64_t n_refs,
                            int32_t *d_cell_start, float *d_cell_tris, float *d_cell_box, void *d_ws, size_t ws_bytes,
                            void *stream);

/* Spatial (Morton / Z-order) order of a point set: d_order[n_points] lists the
 * point indices so that consecutive entries are close in space.  Passed to
 * lyem_pair_stage as d_src_order / d_snk_order it makes the rays of a warp
 * coherent.  No counterpart in the reference (it processes pairs in index order). */
LYEM_API size_t lyem_spatial_order_workspace(int64_t n_points);

/* Direction order of a point set seen from centre3 (host, 3 floats): the
 * sphere of directions is cut into square (elevation, azimuth) tiles of about
 * 16 points (edge 4 * sqrt(2 pi^2 / n_points) radians, at least 0.009), tiles
 * ordered by elevation band then azimuth, so consecutive entries lie in small
 * angular patches.  Passed as d_snk_order for sinks far from the
 * scene (far-field spheres) it gives each warp rays of nearly one direction,
 * hence similar walks; centre3 is typically the centre of the grid box.
 * Workspace: lyem_spatial_order_workspace(n_points) bytes. */
LYEM_API int lyem_direction_order(const float *d_points, int64_t n_points, const float *centre3, int32_t *d_order,
                                  void *d_ws, size_t ws_bytes, void *stream);
LYEM_API int lyem_spatial_order(const float *d_points, int64_t n_points, int32_t *d_order, void *d_ws,
                                size_t ws_bytes, void *stream);

/* ------------------------------------------------------------- pair stage */

/* Visibility + fused field for every (source n, sink m) pair:
 *   sink_out[m, c] (+)= sum_n W[n, c] * S[n, m, c]
 * with S[n, m, :] = vis(n, m) * em_wave(ray n->m) (lyceanem/src/em.cuh:64-120),
 * W = d_src_W or 1.  Visibility is the Moller-Trumbore any-hit test of
 * lyceanem/src/raycasting.cuh:19-68 (cull = 1) or the numba engine's
 * lyceanem/raycasting/rayfunctions.py:37-104 (cull = 0, eps = 1e-7) against all
 * packed triangles (brute force, d_cell_start == NULL) or a grid from
 * lyem_grid_fill (d_cell_start, d_cell_tris and d_cell_box all given); eps, the determinant threshold, must be
 * finite and not negative (LYEM_ERR_INVALID otherwise).  self_to_self = 0 reproduces the reference's skip of the pair
 * whose source index equals its sink index (lyceanem/src/raycasting_brute_force.cuh:27).
 * Replaces raycast_brute_force / raycast_tiles + set_values + points_to_rays
 * (lyceanem/src/raycasting_brute_force.cuh:68-88, raycasting_accelerated.cuh:458-482,
 * raycasting.cuh:80-108) and the host sum over sources
 * (lyceanem/models/frequency_domain.py:847-849).
 * Optional outputs (NULL to skip): d_pair_out [n_src, n_snk, 6] (the
 * reference's scattering network layout, zero for blocked pairs), d_mask_bits
 * [n_src, ceil(n_snk/32)] uint32 (bit m%32 of word m/32 = visible),
 * d_counters uint64[2] incremented by (visible pairs, ray/triangle tests),
 * d_src_visible int32[n_src] / d_snk_visible int32[n_snk] incremented by the
 * visible pairs of each source / sink.
 * d_src_order / d_snk_order (NULL = index order): permutations from
 * lyem_spatial_order that set which sources share a thread block and which
 * sinks share a warp; results are unchanged (sink sums are summed in chunk
 * order, so a different source order can change the last bits of the field).
 * d_src_order may also list a subset: n_src distinct row indices into source
 * arrays (d_src_pos, d_src_E, d_src_W) that hold more rows.  Only the listed
 * sources are traced; every per-source output (d_pair_out, d_mask_bits,
 * d_src_visible) is indexed by the source's row, so it needs as many rows as
 * the source arrays, and the rows left out are not written.  A source keeps
 * its row index, so self_to_self = 0 still skips the pair of equal row and
 * sink index.  Nothing checks the indices: each must be below the row count.
 * src_chunk: sources per thread block (0 = automatic; at most 32 for brute
 * force, 64 for the grid).  traversal (grid only): 1 = all lanes of a warp
 * trace the same source in lockstep; k in 2..33 = each lane moves on to its
 * next source when its ray ends, new rays being started in batches once k-1
 * lanes of the warp are idle; 34, 35, 36 = lockstep with the registers capped
 * so that 10, 12, 16 blocks fit an SM; 100 + k / 200 + k (k in 1..64) = two
 * phases with the registers capped for 16 / 12 blocks per SM: lockstep up to
 * k grid cells along each ray, then the rays still open are queued per warp
 * and walked to their end 32 at a time; 38 = transposed: the lanes of a warp
 * are 32 sources (32 sources per block, whatever src_chunk says: query the
 * workspace with src_chunk = 32) and the warp walks one sink at a time, which
 * pays when the sources are compact (the elements of an array) and no per-pair
 * output is asked for (its d_pair_out writes are strided); 0 = automatic
 * (currently 36).  Every schedule gives the same masks; the transposed one
 * sums each sink's field in another order (same result to FP32 rounding). */
LYEM_API size_t lyem_pair_stage_workspace(int64_t n_src, int64_t n_snk, int64_t n_tris, int32_t use_grid,
                                          int32_t src_chunk);
LYEM_API int lyem_pair_stage(const float *d_src_pos, const float *d_src_E, const float *d_src_W, int64_t n_src,
                             const float *d_snk_pos, const float *d_snk_nrm, int64_t n_snk, const float *d_tris,
                             int64_t n_tris, const int32_t *d_cell_start, const float *d_cell_tris,
                             const float *d_cell_box, const float *grid_origin3, float grid_cell,
                             const int32_t *grid_dims3, double alpha, double beta, int32_t self_to_self, int32_t cull,
                             float eps, float *d_sink_out,
                             int32_t accumulate, float *d_pair_out, uint32_t *d_mask_bits, uint64_t *d_counters,
                             int32_t *d_src_visible, int32_t *d_snk_visible, const int32_t *d_src_order,
                             const int32_t *d_snk_order, int32_t src_chunk, int32_t traversal, void *d_ws,
                             size_t ws_bytes, void *stream);

/* lyem_pair_stage for callers that may not allocate device memory (a host
 * whose own allocator owns all device memory, or code that forbids allocation
 * calls once running), so cannot pass the stage's scratch buffer.  No
 * counterpart in the reference (its bindings allocate and free per call).
 * Same arguments as lyem_pair_stage without d_ws / ws_bytes; the scratch is a
 * fixed array inside the library of lyem_pair_stage_noalloc_scratch_bytes()
 * (32 MiB) on every device that loads it.  Limit: the per-chunk partial sums,
 * ceil(n_src / src_chunk) * n_snk * 24 bytes, must fit in it (src_chunk at most
 * 32 for brute force, 64 for the grid; with src_chunk = 0 the automatic
 * chunk of lyem_pair_stage is used when its partial sums fit, else the
 * smallest larger chunk whose partial sums fit); larger problems return
 * LYEM_ERR_WORKSPACE and launch nothing.  Each call looks up the array's
 * device address in the current device's context (so a device reset between
 * calls is harmless); the first call on a device loads the library's device
 * code there and should come before any stream capture.  All calls share the array (it
 * keeps the last call's contents; nothing in it needs to start at zero), so
 * calls that overlap on the GPU race.  Calls no allocation routine. */
LYEM_API size_t lyem_pair_stage_noalloc_scratch_bytes(void);
LYEM_API int lyem_pair_stage_noalloc(const float *d_src_pos, const float *d_src_E, const float *d_src_W,
                                     int64_t n_src, const float *d_snk_pos, const float *d_snk_nrm, int64_t n_snk,
                                     const float *d_tris, int64_t n_tris, const int32_t *d_cell_start,
                                     const float *d_cell_tris, const float *d_cell_box, const float *grid_origin3,
                                     float grid_cell,
                                     const int32_t *grid_dims3, double alpha, double beta, int32_t self_to_self,
                                     int32_t cull, float eps, float *d_sink_out, int32_t accumulate,
                                     float *d_pair_out, uint32_t *d_mask_bits, uint64_t *d_counters,
                                     int32_t *d_src_visible, int32_t *d_snk_visible, const int32_t *d_src_order,
                                     const int32_t *d_snk_order, int32_t src_chunk, int32_t traversal,
                                     void *stream);

/* Expands a bit mask [n_src, ceil(n_snk/32)] to bytes [n_src, n_snk] (0/1). */
LYEM_API int lyem_mask_to_bytes(const uint32_t *d_mask_bits, int64_t n_src, int64_t n_snk, uint8_t *d_out,
                                void *stream);

/* ------------------------------------------------------------ beam sweep */

/* Sink fields of K excitation vectors for a formed network:
 *   E[m, k, c] = sum_n G[n, m, c] W[k, n]
 * with G the pair-stage network (d_pair_out of lyem_pair_stage for unit
 * excitations, complex64 [n_src, n_snk, 3]) and W complex64 [n_beams, n_src].
 * Replaces re-running the whole model once per excitation
 * (lyceanem/models/frequency_domain.py:858-921, multiE) and the host GEMMs of
 * lyceanem/models/frequency_domain.py:258-260.
 * mode 0: plain complex64 FP32 (cublasCgemm), the comparison path.
 * mode 3: BF16 split on the tensor cores (this library's tcgen05 kernel): each
 *   real operand x = hi + lo, the complex product from three real products
 *   (Gauss: Gr Wr, Gi Wi, (Gr + Gi)(Wr + Wi); 6 M N K flops per component
 *   instead of 8), each accumulated in FP32 as hi*hi + lo*hi + hi*lo.
 * mode 4: the same with FP16 halves; the network (per component) and the
 *   weights are scaled by powers of two that put their largest magnitude at
 *   2^14 (no overflow, few subnormal halves) and the result is unscaled exactly.
 * Modes 1 and 2 (the four-product forms of earlier versions) are refused with
 * LYEM_ERR_INVALID.
 * Step 1 converts G into the GEMM operand (d_network, lyem_sweep_network_bytes;
 * ld >= n_snk, a multiple of 8; modes 3, 4: 256-byte aligned); step 2 converts
 * W (modes 3, 4 only, d_B, lyem_sweep_weights_bytes, 256-byte aligned); step 3
 * runs the three component products into d_out, complex64 [3][n_beams][ldc]
 * (component c, beam k: column-major E[:, k, c]; ldc >= ld; mode 0 writes
 * zeros to rows n_snk..ld-1, modes 3, 4 leave them untouched). */
LYEM_API size_t lyem_sweep_network_bytes(int64_t n_src, int64_t ld, int32_t mode);
LYEM_API size_t lyem_sweep_weights_bytes(int64_t n_src, int64_t n_beams, int32_t mode);
LYEM_API int lyem_sweep_prepare_network(const float *d_pairs, int64_t n_src, int64_t n_snk, int32_t mode, int64_t ld,
                                        void *d_network, void *stream);
LYEM_API int lyem_sweep_prepare_weights(const float *d_W, int64_t n_src, int64_t n_beams, int32_t mode, void *d_B,
                                        void *stream);
LYEM_API int lyem_sweep_run(const void *d_network, int64_t n_src, int64_t n_snk, int64_t ld, const float *d_W,
                            const void *d_B, int64_t n_beams, int32_t mode, float *d_out, int64_t ldc, void *stream);
/* lyem_sweep_run with a workspace argument, kept for callers of earlier
 * versions: no mode needs a workspace now (lyem_sweep_workspace_bytes returns
 * 0) and d_ws / ws_bytes are ignored. */
LYEM_API size_t lyem_sweep_workspace_bytes(int64_t ld, int64_t n_beams, int32_t mode);
LYEM_API int lyem_sweep_run_ws(const void *d_network, int64_t n_src, int64_t n_snk, int64_t ld, const float *d_W,
                               const void *d_B, int64_t n_beams, int32_t mode, float *d_out, int64_t ldc, void *d_ws,
                               size_t ws_bytes, void *stream);
/* Sources per pipeline stage of the tensor-core kernel (process-wide): 32
 * (default; 64-byte swizzled rows, 4 stages) or 64 (128-byte rows, 2 stages).
 * Results are the same; only the speed differs.  No counterpart in the reference. */
LYEM_API int lyem_sweep_set_k_tile(int32_t k_tile);
/* 1: the tensor-core kernel runs in clusters of two CTAs on neighbouring row
 * tiles that share each weight tile, each loading half of it and multicasting
 * it to both (a third fewer operand bytes requested per SM); the single-CTA
 * kernel runs instead when no pair can be co-resident.  0 (default): the
 * single-CTA kernel, measured as fast or faster.  Results are the same.  No
 * counterpart in the reference. */
LYEM_API int lyem_sweep_set_multicast(int32_t on);

/* --------------------------------------------------------------- adjoint */

/* Reverse-mode derivatives of the direct + one-bounce sink field with the
 * visibility masks of the forward pass held fixed.  Element n is excited by
 * a_n e_n (d_src_a complex64 [N], d_src_pol complex64 [N,3]); w_p (complex64
 * [P,3]) is the scatter-point excitation of the forward pass (sum over
 * elements of the source->scatter network); masks are the forward stages' bit
 * masks (d_mask0 sources x sinks, d_mask1 sources x scatter, d_mask2 scatter x
 * sinks).  Given the cotangent d_grad_E = dL/dE* of a real loss (complex64
 * [M,3], torch convention) it writes grad a (complex64 [N]), grad x (float
 * [N,3], element positions) and, if d_grad_y != NULL, grad y (float [M,3],
 * sink positions); d_scat_z (complex64 [P,3]) receives the back-propagated
 * field at the scatter points.  Phases are recomputed (FP64 reduction), the
 * N x M network is not stored.  The forward model is em_wave / ray_launch
 * (lyceanem/src/em.cuh:18-120) composed as lyceanem/models/frequency_domain.py:195-264
 * and summed as :847-849; the reference itself has no derivatives.
 * n_scat = 0 gives the direct path only (scatter pointers may be NULL). */
LYEM_API size_t lyem_adjoint_workspace(int64_t n_src, int64_t n_scat, int64_t n_snk);
LYEM_API int lyem_adjoint(const float *d_src_pos, const float *d_src_pol, const float *d_src_a, int64_t n_src,
                          const float *d_scat_pos, const float *d_scat_nrm, const float *d_scat_w, int64_t n_scat,
                          const float *d_snk_pos, const float *d_snk_nrm, const float *d_grad_E, int64_t n_snk,
                          const uint32_t *d_mask0, const uint32_t *d_mask1, const uint32_t *d_mask2, double alpha,
                          double beta, float *d_grad_a, float *d_grad_x, float *d_grad_y, float *d_scat_z,
                          void *d_ws, size_t ws_bytes, void *stream);

/* ------------------------------------ many scenes x many frequencies */

/* One scene of a batch: the composition of calculate_scattering_cuda
 * (lyceanem/models/frequency_domain.py:195-264) summed over the sources
 * (:847-849), evaluated at every frequency of the batch.  Device pointers.
 * Scatter points are given in processing order (e.g. lyem_spatial_order);
 * scat_id[slot] is the caller's index of a slot, used only by the
 * self_to_self pair-skip rule (NULL: the slot is the index).  The grid is
 * the scene's uniform grid (lyem_grid_plan / lyem_grid_fill). */
typedef struct lyem_batch_scene {
    const float *src_pos;      /* [n_src, 3] */
    const float *src_E;        /* [n_src, 6] complex excitation (re, im) x (x, y, z) */
    const float *scat_pos;     /* [n_scat, 3] */
    const float *scat_nrm;     /* [n_scat, 3] */
    const int32_t *scat_id;    /* [n_scat] or NULL */
    const int32_t *cell_start; /* [cells + 1] */
    const float *cell_tris;    /* [refs, 12], 16-byte aligned */
    const float *cell_box;     /* [cells, 16], 16-byte aligned (lyem_grid_fill) */
    int64_t n_src;
    int64_t n_scat;
    float grid_origin[3];
    float grid_cell;
    int32_t grid_dims[3];
    int32_t reserved;
} lyem_batch_scene;

typedef struct lyem_batch_config {
    int32_t freq_group;    /* frequencies per thread: 1, 2, 4 or 8; above 1 the beta list must be uniform */
    int32_t src_chunk;     /* sources per visibility item: 32 or 64 */
    int32_t blocks_per_sm; /* resident blocks per SM of the persistent launch, 0..8 (0: as many as fit) */
    int32_t cull;          /* back-face culling (the CUDA engine's rule) */
    float eps;             /* determinant threshold of the ray-triangle test (finite, >= 0) */
    int32_t self_to_self;  /* 0: the pair (n, m) with equal indices is not tested (the reference default) */
    double alpha;          /* attenuation */
} lyem_batch_config;

/* No counterpart in the reference, which evaluates one scene at one
 * frequency per call.  All scenes share the sinks (processing order; snk_id
 * maps a slot to the caller's index, which indexes the output) and the
 * frequency list beta[n_freq] (rad/m).  Output field[n_scenes][n_freq][n_snk][6]
 * float (complex64 [S, F, M, 3]):
 *   E_f(m) = sum_n S0_f(n, m) + sum_p e_p(f) (.) S2_f(p, m; e_p(f)),
 *   e_p(f) = sum_n S1_f(n, p).
 * lyem_batch_workspace: bytes of the workspace (0: invalid arguments).
 * lyem_batch_items: work items of the launch (per kind: three visibility
 *   stages, scatter fields, sink fields), or minus a status.
 * lyem_batch_prepare: writes the scene table, the work list and the
 *   frequency tables into the workspace (256-byte aligned); host -> device
 *   copies, synchronous with the stream.  Repeat after any change of scenes,
 *   frequencies or configuration.
 * lyem_batch_launch: two memsets and one kernel on the stream, nothing else
 *   (no allocation, no host synchronisation); counters (optional, [n_scenes][4]
 *   u64: visible pairs of the three stages, ray-triangle tests) are zeroed
 *   first; blocks_out (optional) receives the persistent grid size. */
LYEM_API size_t lyem_batch_workspace(const lyem_batch_scene *scenes, int32_t n_scenes, int64_t n_snk,
                                     int32_t n_freq, const lyem_batch_config *config);
LYEM_API int64_t lyem_batch_items(const lyem_batch_scene *scenes, int32_t n_scenes, int64_t n_snk, int32_t n_freq,
                                  const lyem_batch_config *config, int64_t *per_kind5);
LYEM_API int lyem_batch_prepare(const lyem_batch_scene *scenes, int32_t n_scenes, int64_t n_snk, const double *beta,
                                int32_t n_freq, const lyem_batch_config *config, void *d_ws, size_t ws_bytes,
                                void *stream);
LYEM_API int lyem_batch_launch(const lyem_batch_scene *scenes, int32_t n_scenes, const float *d_snk_pos,
                               const float *d_snk_nrm, const int32_t *d_snk_id, int64_t n_snk, const double *beta,
                               int32_t n_freq, const lyem_batch_config *config, void *d_ws, size_t ws_bytes,
                               float *d_field_out, uint64_t *d_counters, int32_t *blocks_out, void *stream);

/* ------------------------------------------------ numba-engine products */

/* f <- f - (f . n^) n^ for complex 3-vectors d_vec [n,6] and vectors d_normals [n,3]
 * (n^ = n/|n|; a zero n leaves f unchanged): the tangential projection of
 * sourcelaunchtransformGPU (lyceanem/electromagnetics/empropagation.py:179-258). */
LYEM_API int lyem_tangential_project(float *d_vec, const float *d_normals, int64_t n, void *stream);

/* Field of every path row of the numba engine, summed per (source, sink):
 * freqdomainkernal (lyceanem/electromagnetics/empropagation.py:1083-1265) over
 * the index of workchunkingv2 (lyceanem/raycasting/rayfunctions.py:2681-2955).
 * d_paths [n_paths, n_cols] int32, 1-based indices into the point arrays
 * (sources 1..n_src, sinks n_src+1..n_src+n_snk, then scatter points; 0 = none);
 * d_pos, d_nrm [n_pts,3]; d_w [n_pts,6] complex weights (the sources' field,
 * factors at later points); d_magnetic [n_pts] (NULL: all electric) with
 * d_impedance [n_pts] (sqrt(mu/eps)).  Adds to d_out [n_src, n_snk, 3, 2]
 * double (complex128 [n_src, n_snk, 3]; the caller zeroes it).  Rows with an
 * index out of range set device error bit 1 and are skipped. */
LYEM_API int lyem_path_field(const int32_t *d_paths, int64_t n_paths, int32_t n_cols, const float *d_pos,
                             const float *d_nrm, const float *d_w, const uint8_t *d_magnetic,
                             const float *d_impedance, int64_t n_pts, int64_t n_src, int64_t n_snk, double alpha,
                             double beta, double *d_out, void *stream);

/* Time-domain form of the same rows (timedomainkernal,
 * lyceanem/electromagnetics/empropagation.py:1346-1560): per row the real
 * magnitude vector d_amp [n_paths,3] (real parts of the weights, the same
 * projections, |loss| of the segments), the arrival time d_arrival [n_paths]
 * in seconds (path length / c plus the imaginary parts of the x weights of the
 * source and of each later point; for i >= 1 the length adds the distance to
 * the point of index row[i+1] even when it is 0, read as the last point, as
 * the reference does) and d_pair [n_paths,2] (source, sink), or (-1, -1) with
 * device error bit 1 for a row with an index out of range. */
LYEM_API int lyem_path_time(const int32_t *d_paths, int64_t n_paths, int32_t n_cols, const float *d_pos,
                            const float *d_nrm, const float *d_w, const uint8_t *d_magnetic, const float *d_impedance,
                            int64_t n_pts, int64_t n_src, int64_t n_snk, double alpha, double beta, double *d_amp,
                            double *d_arrival, int32_t *d_pair, void *stream);

/* ------------------------------------------ host mirrors of lyceanem.em */

/* bin_counts_to_numpy (lyceanem/src/terrain_acceleration_build.cuh:296-348):
 * triangles binned over the y-z grid of ncells_x (along y) by ncells_y
 * (along z) square cells of width cell_width from (ymin, z_min); cell index
 * iy*ncells_y + iz.  Every cell a triangle's y-z box overlaps receives it
 * (the reference bins vertex cells plus one corner and asserts adjacency). */
LYEM_API int lyem_em_bin_counts(const float *tri_vertex, int64_t n_vertex, const int32_t *tri_index, int64_t n_tris,
                                int32_t ncells_x, int32_t ncells_y, float ymin, float cell_width, float z_min,
                                int32_t *counts_out);

/* bin_triangles_to_numpy (lyceanem/src/terrain_acceleration_build.cuh:370-431):
 * the vertex-index triples of the binned triangles in cell order, triangles
 * ascending within a cell; out has 3*sum_bin_counts entries. */
LYEM_API int lyem_em_bin_triangles(const float *tri_vertex, int64_t n_vertex, const int32_t *tri_index,
                                   int64_t n_tris, int32_t ncells_x, int32_t ncells_y, float ymin, float cell_width,
                                   float z_min, const int32_t *bin_counts, int64_t sum_bin_counts, int32_t *out);

/* calculate_scattering_brute_force (lyceanem/src/frequency_domain_models.cu:190-311),
 * returning the network the reference computes (its binding never copies it
 * back): out[n_source*n_end*6] float32. */
LYEM_API int lyem_em_calculate_scattering_brute_force(
    const float *source, int64_t n_source, const float *end, int64_t n_end, const int32_t *triangles, int64_t n_tris,
    const float *triangle_vertex, int64_t n_vertex, float wave_length, const float *ex_real, const float *ex_imag,
    const float *ey_real, const float *ey_imag, const float *ez_real, const float *ez_imag, const float *normal,
    float alpha, float beta, int32_t not_self_to_self, float *out);

/* calculate_scattering_tiles (lyceanem/src/frequency_domain_models.cu:44-187):
 * the triangle set is the distinct vertex triples of bin_triangles; the
 * traversal uses this library's own uniform grid, so bounds, tile size and
 * bin counts only describe the caller's binning.  out[n_source*n_end*6]. */
LYEM_API int lyem_em_calculate_scattering_tiles(
    const float *source, int64_t n_source, const float *end, int64_t n_end, const float *triangle_vertex,
    int64_t n_vertex, float wave_length, const float *ex_real, const float *ex_imag, const float *ey_real,
    const float *ey_imag, const float *ez_real, const float *ez_imag, const float *normal, float xmin, float xmax,
    float ymin, float ymax, float zmin, float zmax, float tile_size, const int32_t *bin_count,
    const int32_t *bin_triangles, int32_t n_cellsx, int32_t n_cellsy, int32_t binned_tri_num, float alpha,
    float beta, int32_t not_self_to_self, float *out);

#ifdef __cplusplus
}
#endif

#endif /* LYEM_H_ */
