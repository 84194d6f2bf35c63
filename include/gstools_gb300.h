/*
 * gstools_gb300 -- C ABI of the GB300 (sm_103a) randomization-method
 * summation kernels.
 *
 * These entry points replace the native summators that GSTools' generators
 * call through module-level wrappers:
 *
 *   gstools_cython.field.summate          (src/gstools/field/generator.py:22,
 *                                          wrapper _summate :42-48, called at
 *                                          RandMeth.__call__ :266-268)
 *   gstools_cython.field.summate_incompr  (generator.py:24, wrapper
 *                                          _summate_incompr :51-64, called at
 *                                          IncomprRandMeth.__call__ :554-560)
 *   gstools_cython.field.summate_fourier  (generator.py:23, wrapper
 *                                          _summate_fourier :67-75, called at
 *                                          Fourier.__call__ :682-689)
 *
 * Conventions shared by every entry point
 * ---------------------------------------
 * - Arrays are DEVICE pointers (cudaMalloc / torch CUDA memory) of the
 *   current device, C-contiguous, in the reference's layouts:
 *   cov_samples (dim, n_modes) row-major, z_1 / z_2 (n_modes,),
 *   pos (dim, n_pts) row-major, scalar output (n_pts,), vector output
 *   (dim, n_pts).  Inputs are read-only and borrowed.
 * - `stream` is a cudaStream_t (NULL = legacy default stream).  Every call is
 *   asynchronous with respect to the host and ordered on that stream.
 * - Return value: GST_OK (0) or a GST_ERR_* code; no entry point aborts.
 *   gst_status_string() names a code.  The `num_threads` argument of the
 *   reference (CPU thread count) has no counterpart: parallelism is the GPU.
 * - Internal scratch (packed mode tables, split-mode partial sums, per-axis
 *   phase tables) is taken from the stream-ordered allocator
 *   (cudaMallocAsync) and released on the same stream.
 * - Results are the raw mode sums of the reference; the caller applies
 *   sqrt(var / N) and the nugget exactly as generator.py:269-270 and
 *   :561-567 do.  The grid entry points take an optional `scale` that is
 *   fused into the epilogue (pass 1.0 for raw sums).
 */
#ifndef GSTOOLS_GB300_H
#define GSTOOLS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GST_OK 0
#define GST_ERR_INVALID_ARGUMENT 1 /* bad size, NULL pointer, ... */
#define GST_ERR_UNSUPPORTED_DIM 2  /* dim outside the supported range */
#define GST_ERR_CUDA 3             /* a CUDA runtime call failed */
#define GST_ERR_ALIGNMENT 4        /* a pointer violates the stated alignment */
#define GST_ERR_NO_DEVICE 5        /* no usable sm_103 device is current */
#define GST_ERR_DEVICE_TIMEOUT 6   /* a bounded device-side wait gave up */
#define GST_ERR_TOO_LARGE 7        /* a size exceeds a documented maximum */

/* Output element types for the mixed-precision and grid entry points. */
#define GST_OUT_F64 0
#define GST_OUT_F32 1

/* Library version as 10000*major + 100*minor + patch. */
int gst_version(void);

/* Human-readable name of a status code (static storage). */
const char *gst_status_string(int status);

/* cudaError_t value behind the calling thread's last GST_ERR_CUDA. */
int gst_last_cuda_error(void);

/* Reads and clears the device-side error word that bounded waits in the
 * kernels set when they give up (GST_ERR_DEVICE_TIMEOUT bits).  Synchronises
 * `stream`.  *device_error receives the word (0 = none). */
int gst_read_device_error(void *stream, uint32_t *device_error);

/* Host-side gather (no device work): n_arrays row-major float64 arrays of
 * `rows` rows and cols[a] columns each (src[a] their addresses) side by
 * side into the row-major rows x dst_cols array dst (dst_cols = sum of
 * cols), on up to `threads` host threads -- one ensemble's per-realization
 * inputs into its page-locked staging buffer.  No counterpart in the
 * reference. */
int gst_host_gather(int64_t n_arrays, const uint64_t *src, const int64_t *cols,
                    int64_t rows, double *dst, int64_t dst_cols, int threads);

/* ----------------------------------------------------------------------- */
/* Plain FP64 pointwise kernels (parity anchors).                           */
/* ----------------------------------------------------------------------- */

/* summate: out[i] = sum_j z_1[j] cos(<k_j, x_i>) + z_2[j] sin(<k_j, x_i>).
 * Replaces gstools_cython.field.summate (generator.py:22, math :193-199).
 * dim in 1..4.  FP64 throughout. */
int gst_summate_f64(int dim, int64_t n_modes, int64_t n_pts,
                    const double *cov_samples, const double *z_1,
                    const double *z_2, const double *pos, double *out,
                    void *stream);

/* summate_incompr: out[c, i] = sum_j (delta_c0 - k_cj k_0j / |k_j|^2)
 *                    (z_1[j] cos(<k_j, x_i>) + z_2[j] sin(<k_j, x_i>)).
 * Replaces gstools_cython.field.summate_incompr (generator.py:24, math
 * :479-495).  dim in 2..3.  out is (dim, n_pts).  FP64 throughout. */
int gst_summate_incompr_f64(int dim, int64_t n_modes, int64_t n_pts,
                            const double *cov_samples, const double *z_1,
                            const double *z_2, const double *pos, double *out,
                            void *stream);

/* summate_fourier: out[i] = sum_j f[j] (z_1[j] cos(<k_j, x_i>)
 *                                       + z_2[j] sin(<k_j, x_i>)).
 * Replaces gstools_cython.field.summate_fourier (generator.py:23, called at
 * :682-689).  `modes` is (dim, n_modes) like cov_samples.  dim in 1..4. */
int gst_summate_fourier_f64(int dim, int64_t n_modes, int64_t n_pts,
                            const double *spectrum_factor, const double *modes,
                            const double *z_1, const double *z_2,
                            const double *pos, double *out, void *stream);

/* Allocation-free variant of gst_summate_f64 (same arguments and result).
 * No counterpart in the reference: it exists for callers that cannot let a
 * library allocate device memory -- hosts that reserve the GPU's memory for
 * their own pool and forbid other allocations, and latency-critical loops
 * that cannot pay for an allocator call.  Its scratch is a fixed 5 MiB
 * device array inside the library (held on every GPU that loads it until
 * the process exits); it never calls cudaMalloc or cudaFree.
 * Limits: n_modes <= 16384 (GST_ERR_TOO_LARGE beyond); the mode range is
 * split across CTAs only as far as the partial sums fit in 4 MiB, so small
 * point counts may run with less parallelism.  The first call on a device
 * looks up the array's device address (make it before any stream capture:
 * a first call on a capturing stream returns GST_ERR_INVALID_ARGUMENT).
 * All calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller. */
int gst_summate_f64_noalloc(int dim, int64_t n_modes, int64_t n_pts,
                            const double *cov_samples, const double *z_1,
                            const double *z_2, const double *pos, double *out,
                            void *stream);

/* ----------------------------------------------------------------------- */
/* Mixed-precision pointwise kernels (same inputs, FP64 in).                */
/* The phase is reduced to turns exactly (error-free FP32 splitting of the  */
/* FP64 wave vectors and positions), sin/cos run on the SFU in FP32, each   */
/* 256-mode block is summed in FP32 and blocks are accumulated in FP64.     */
/* Domain: |k_d x_d| / (2 pi) < 2^21 turns per axis.                        */
/* ----------------------------------------------------------------------- */

/* Same contract as gst_summate_f64; `out` is double (GST_OUT_F64) or float
 * (GST_OUT_F32).  dim in 1..3.  Sums with at most 16384 modes and at least
 * 1e9 mode-points, or in 2-D / 3-D at least 4e8 mode-points over at least
 * 2e5 points, run the sorted amplitude-phase path of the ensembles (points
 * sorted spatially, modes by |k|_1, one SFU cosine per mode and point);
 * smaller ones the pointwise kernel described above. */
int gst_summate_mixed(int dim, int64_t n_modes, int64_t n_pts,
                      const double *cov_samples, const double *z_1,
                      const double *z_2, const double *pos, void *out,
                      int out_type, void *stream);

/* Same contract as gst_summate_incompr_f64, mixed precision.  dim in 2..3. */
int gst_summate_incompr_mixed(int dim, int64_t n_modes, int64_t n_pts,
                              const double *cov_samples, const double *z_1,
                              const double *z_2, const double *pos, void *out,
                              int out_type, void *stream);

/* ----------------------------------------------------------------------- */
/* Structured grids.                                                        */
/* A structured grid is the meshgrid ("ij" order, last axis fastest) of     */
/* `dim` axis arrays (generate_grid, src/gstools/tools/geometric.py:340-356) */
/* passed concatenated in `axes` (axis_len[0] + ... + axis_len[dim-1]       */
/* values; `axes` is device memory, `axis_len` is HOST memory).             */
/* The reference isometrizes the materialised grid with a linear  */
/* map M (covmodel/base.py:572-582); because <k, M x> = <M^T k, x>, callers */
/* pass cov_samples already multiplied by M^T and the kernels never         */
/* materialise the grid.  Output shape is (axis_len[0], ..., axis_len[d-1]) */
/* (scalar) or (dim, axis_len[0], ...) (vector).                            */
/* ----------------------------------------------------------------------- */

/* Plain FP64 pointwise kernel over structured-grid points. dim in 1..4. */
int gst_summate_grid_f64(int dim, int64_t n_modes, const int64_t *axis_len,
                         const double *axes, const double *cov_samples,
                         const double *z_1, const double *z_2, double *out,
                         void *stream);

/* Mixed-precision pointwise kernel over structured-grid points.  dim 1..3.
 * `scale` multiplies the result (1.0 = raw sums). */
int gst_summate_grid_mixed(int dim, int64_t n_modes, const int64_t *axis_len,
                           const double *axes, const double *cov_samples,
                           const double *z_1, const double *z_2, void *out,
                           int out_type, double scale, void *stream);

/* FP64 incompressible field over structured-grid points. dim in 2..3. */
int gst_summate_incompr_grid_f64(int dim, int64_t n_modes,
                                 const int64_t *axis_len, const double *axes,
                                 const double *cov_samples, const double *z_1,
                                 const double *z_2, double *out, void *stream);

/* Mixed-precision incompressible field over structured-grid points. */
int gst_summate_incompr_grid_mixed(int dim, int64_t n_modes,
                                   const int64_t *axis_len, const double *axes,
                                   const double *cov_samples,
                                   const double *z_1, const double *z_2,
                                   void *out, int out_type, double scale,
                                   void *stream);

/* Separable structured-grid path on the tensor cores (dim 2 or 3).
 * exp(i<k, x>) factorises per axis, so the grid sum is the real part of a
 * complex contraction Re(E_x diag(w) (E_y (.) E_z)^T), w = z_1 - i z_2, run as
 * a 3xTF32 GEMM (tcgen05, FP32 accumulation in tensor memory) over per-axis
 * tables built from an exact turn reduction.  Same arguments and output as
 * gst_summate_grid_mixed.  Field RMS error vs FP64 is ~1e-6 of the field's
 * standard deviation (see the parity tests). */
int gst_summate_grid_tc(int dim, int64_t n_modes, const int64_t *axis_len,
                        const double *axes, const double *cov_samples,
                        const double *z_1, const double *z_2, void *out,
                        int out_type, double scale, void *stream);

/* summate_incompr on a structured grid through the tensor-core path: the
 * projector p_c(k) = delta_c0 - k_c k_0 / |k|^2 is a per-mode real weight on
 * z_1 - i z_2, so the field is dim weighted contractions.  cov_samples are
 * the (possibly M^T-mapped) wave vectors of the phases; proj_cov (dim, N)
 * are the unmapped wave vectors of the projector (NULL: cov_samples).
 * out is (dim, axis_len[0], ...).  dim 2..3.  Replaces
 * gstools_cython.field.summate_incompr on generate_grid + isometrize. */
int gst_summate_incompr_grid_tc(int dim, int64_t n_modes, const int64_t *axis_len,
                                const double *axes, const double *cov_samples,
                                const double *proj_cov, const double *z_1,
                                const double *z_2, void *out, int out_type,
                                double scale, void *stream);

/* summate_fourier on a structured grid through the tensor-core path (the
 * spectrum factor is the per-mode weight).  Replaces
 * gstools_cython.field.summate_fourier (generator.py:23, :682-689) when the
 * Fourier generator evaluates a structured mesh.  dim 2..3. */
int gst_summate_fourier_grid_tc(int dim, int64_t n_modes, const int64_t *axis_len,
                                const double *axes, const double *spectrum_factor,
                                const double *modes, const double *z_1,
                                const double *z_2, void *out, int out_type,
                                double scale, void *stream);

/* The tensor-core grid path in two steps with a caller-owned workspace, so
 * that the per-axis tables can be built once and contracted many times (and
 * each step timed on its own).  The workspace is device memory, 256-byte
 * aligned, of at least the size gst_grid_tc_workspace_size reports (0 when
 * there is nothing to do).  gst_grid_tc_tables fills it from the modes and
 * axes; gst_grid_tc_contract writes the field from it.  Arguments otherwise
 * as gst_summate_grid_tc; both calls must see the same dim, n_modes and
 * axis_len.  No counterpart in the reference (its summation has no
 * precomputation step). */
int gst_grid_tc_workspace_size(int dim, int64_t n_modes,
                               const int64_t *axis_len, size_t *bytes);
/* Width of the z tile (the MMA's N: 128, 192 or 256 points) the grid path
 * uses for a last axis of nz points; -1 for nz < 0.  Informational. */
int gst_grid_tc_tile_cols(int64_t nz);
int gst_grid_tc_tables(int dim, int64_t n_modes, const int64_t *axis_len,
                       const double *axes, const double *cov_samples,
                       const double *z_1, const double *z_2, void *workspace,
                       size_t workspace_bytes, void *stream);
int gst_grid_tc_contract(int dim, int64_t n_modes, const int64_t *axis_len,
                         const void *workspace, size_t workspace_bytes,
                         void *out, int out_type, double scale, void *stream);

/* ----------------------------------------------------------------------- */
/* Adjoint of summate (no counterpart in the reference, which has no        */
/* gradients).  For u = summate(cov_samples, z_1, z_2, pos) and an upstream */
/* gradient grad_out = dL/du (n_pts,):                                      */
/*   gst_summate_vjp_modes_*: grad_z1 (N,), grad_z2 (N,) and grad_cov       */
/*     (dim, N) = dL/dz_1, dL/dz_2, dL/dk; any output may be NULL.          */
/*   gst_summate_vjp_pos_*: v (dim, n_pts) with                             */
/*     v[d, i] = sum_j k_jd (z2_j cos(<k_j, x_i>) - z1_j sin(<k_j, x_i>)),  */
/*     so dL/dx[d, i] = grad_out[i] * v[d, i].                              */
/* sin/cos are recomputed, nothing of the forward pass is stored.  dim 1..3.*/
/* _f64 in FP64, _mixed with the mixed-precision phase reduction.           */
/* ----------------------------------------------------------------------- */
int gst_summate_vjp_modes_f64(int dim, int64_t n_modes, int64_t n_pts,
                              const double *cov_samples, const double *z_1,
                              const double *z_2, const double *pos,
                              const double *grad_out, double *grad_z1,
                              double *grad_z2, double *grad_cov, void *stream);
int gst_summate_vjp_modes_mixed(int dim, int64_t n_modes, int64_t n_pts,
                                const double *cov_samples, const double *z_1,
                                const double *z_2, const double *pos,
                                const double *grad_out, double *grad_z1,
                                double *grad_z2, double *grad_cov, void *stream);
int gst_summate_vjp_pos_f64(int dim, int64_t n_modes, int64_t n_pts,
                            const double *cov_samples, const double *z_1,
                            const double *z_2, const double *pos, double *out,
                            void *stream);
int gst_summate_vjp_pos_mixed(int dim, int64_t n_modes, int64_t n_pts,
                              const double *cov_samples, const double *z_1,
                              const double *z_2, const double *pos, double *out,
                              void *stream);
/* The points of a structured grid (axes concatenated, "ij" order, axis_len
 * with dim entries) followed by n_extra points x_extra (dim, n_extra) that
 * the n_idx indices idx (device int64) select: xs (dim, n_idx) their
 * coordinates and gs (n_idx,) = g[idx] their cotangents -- the inputs of
 * gst_summate_vjp_* for the points of a field with a nonzero cotangent.
 * An index outside [0, grid points + n_extra) gives zeros. */
/* The mode map of a differentiable RandMeth field, on the device (no host
 * round trip): mt (dim x dim, row-major) = M^T len_scale_ref / len_scale
 * with M the reference's isometrize matrix (src/gstools/tools/geometric.py:
 * 184-294: Givens rotations of the planes (0,1), (0,2), (1,2) by
 * (-1)^i (-angles_i), then diag(1, 1/anis)), and jac (dim^2 x n_params,
 * row-major) = d mt / d params, params = [len_scale, anis (dim - 1),
 * angles (dim (dim - 1) / 2)] (device).  The wave vectors are mt @ k_ref. */
int gst_mode_map(int dim, const double *params, double len_scale_ref, double *mt,
                 double *jac, void *stream);
int gst_gather_points(int dim, const int64_t *axis_len, const double *axes,
                      int64_t n_extra, const double *x_extra, int64_t n_idx,
                      const int64_t *idx, const double *g, double *xs,
                      double *gs, void *stream);

/* ----------------------------------------------------------------------- */
/* Batched ensembles: many realizations with their own modes and point sets. */
/* The reference generates an ensemble by looping over seeds, one summate   */
/* call per realization (examples/01_random_field/01_srf_ensemble.py); here */
/* the ensemble is one persistent launch over a queue of (realization,      */
/* point tile) work items, longest first.  Realization r owns modes        */
/* [sum(mode_counts[:r]), +mode_counts[r]) of cov (dim, total_modes), z_1,  */
/* z_2 and points [sum(point_counts[:r]), +point_counts[r]) of pos          */
/* (dim, total_points) and out (total_points,).  mode_counts and            */
/* point_counts are HOST arrays; scales (device, n_items, may be NULL)      */
/* multiplies each realization's result (sqrt(var_r / N_r) for RandMeth).   */
/* Arithmetic: mixed precision in amplitude-phase form (one SFU cosine per  */
/* mode and point); each realization's points are sorted spatially and its  */
/* modes by |k|_1 inside gst_batch_run, so that compact work tiles run the  */
/* phase in plain FP32 where |<k, x - x_warp>| stays small and the exact    */
/* split turn reduction elsewhere.  variant (0 .. gst_batch_variants() - 1) */
/* selects the kernel shape: points per tile, modes per shared-memory stage */
/* and CTAs per SM (0: 512/256/2, 1: 1024/256/2, 2: 512/256/3,             */
/* 3: 512/128/3, 4: 256/256/4, 5: 1024/128/2).  gst_batch_prepare           */
/* (synchronous, once per ensemble shape and variant) writes the work list  */
/* into the caller's workspace; gst_batch_run is asynchronous, allocates    */
/* nothing and may be captured in a CUDA graph; it must see the same counts */
/* and variant as prepare.  gst_batch_variants has no counterpart in the    */
/* reference: the number of compiled kernel shapes.                         */
/* ----------------------------------------------------------------------- */
int gst_batch_variants(void);
int gst_batch_workspace_size(int dim, int64_t n_items, const int64_t *mode_counts,
                             const int64_t *point_counts, int variant,
                             size_t *bytes);
int gst_batch_prepare(int dim, int64_t n_items, const int64_t *mode_counts,
                      const int64_t *point_counts, int variant, void *workspace,
                      size_t workspace_bytes, void *stream);
int gst_batch_run(int dim, int64_t n_items, const int64_t *mode_counts,
                  const int64_t *point_counts, int variant, const double *cov,
                  const double *z_1, const double *z_2, const double *pos,
                  const double *scales, void *out, int out_type,
                  void *workspace, size_t workspace_bytes, void *stream);

/* ----------------------------------------------------------------------- */
/* Device-side spectral sampling for ensembles (replaces the per-realization */
/* host loop of RandMeth.reset_seed, src/gstools/field/generator.py:346-387, */
/* with the RNG of src/gstools/random/rng.py:38-203).  Draws, for every      */
/* realization r of a batch laid out as gst_batch_run expects, its          */
/* mode_counts[r] modes: z_1, z_2 ~ N(0, 1), directions uniform on the unit  */
/* sphere and radii from the model's radial spectral law with length scale  */
/* len_rescaled[r]: Gaussian (normal), Exponential (multivariate t, 1 dof), */
/* Matern nu (multivariate t, 2 nu dof; 0 < nu <= 20).  Mode j of           */
/* realization r is a pure function of (seeds[r], j) through a Philox4x64-10 */
/* stream (key (seeds[r], 0), counter (j, block, 0, 0)), so the draw is      */
/* reproducible and independent of the batch it is part of.  It is not the  */
/* reference's MT19937 stream.  mode_offsets (device, n_items + 1) are the  */
/* prefix sums of the mode counts, seeds (device, uint64) and len_rescaled  */
/* (device) one per realization; cov (dim, total_modes), z_1, z_2 device   */
/* outputs.  Asynchronous, allocates nothing, may be captured in a graph.   */
/* No counterpart in the reference (its sampling is host-side).             */
/* ----------------------------------------------------------------------- */
#define GST_MODEL_GAUSSIAN 0
#define GST_MODEL_EXPONENTIAL 1
#define GST_MODEL_MATERN 2
int gst_batch_sample_modes(int dim, int64_t n_items, int64_t total_modes,
                           const int64_t *mode_offsets, int model, double nu,
                           const uint64_t *seeds, const double *len_rescaled,
                           double *cov, double *z_1, double *z_2, void *stream);
/* The raw Philox4x64-10 stream: out[4 i .. 4 i + 3] = Philox(counter       */
/* (i, counter1, 0, 0), key (key0, key1)) for i < n_blocks (device out).    */
/* For checking the generator against known-answer vectors.                 */
int gst_philox4x64_fill(uint64_t key0, uint64_t key1, int64_t n_blocks,
                        uint64_t counter1, uint64_t *out, void *stream);

/* ----------------------------------------------------------------------- */
/* Kriging field and error variance (CondSRF / Krige hot loop).  Replaces   */
/* gstools_cython.krige.calc_field_krige and                                */
/* calc_field_krige_and_variance (imported src/gstools/krige/base.py:16-19, */
/* called through _calc_field_krige(_and_variance) at :42-60 from           */
/* Krige._summate, :307-320).  For the inverted kriging matrix krig_mat      */
/* (n_cond x n_cond, row-major), the right-hand sides krig_vecs (n_cond x   */
/* n_pts, row-major) and the condition values cond (n_cond):                */
/*   field[k] = sum_i cond[i] (M v_k)_i,  error[k] = sum_i v_ik (M v_k)_i    */
/* error may be NULL for the field only, computed as field = V^T (M^T c):   */
/* n_cond^2 + n_cond n_pts flops instead of n_cond^2 n_pts, same FP64 error */
/* bound, n_cond doubles of stream-ordered scratch.  Variances with         */
/* n_cond <= 4096 and n_cond^2 n_pts >= 4e9 form M V from error-free FP16   */
/* slices on the tensor cores (exact slice products, FP64 folds; FP64-level */
/* accuracy; a non-finite value in M makes every error NaN, one in column k */
/* of V error[k]), with ~34 n_cond n_pts bytes of scratch.                 */
/* Device pointers; FP64; deterministic.                                    */
/* ----------------------------------------------------------------------- */
int gst_calc_field_krige(int64_t n_cond, int64_t n_pts, const double *krig_mat,
                         const double *krig_vecs, const double *cond, double *field,
                         double *error, void *stream);

/* ----------------------------------------------------------------------- */
/* Empirical variograms.  Replace gstools-cython's variogram kernels        */
/* unstructured, directional, structured and ma_structured (imported        */
/* src/gstools/variogram/variogram.py:14-17, called through the wrappers at */
/* :48-124 from vario_estimate / vario_estimate_axis).  estimator 'm'       */
/* (Matheron) or 'c' (Cressie); distance_type 'e' (Euclidean) or 'h'         */
/* (haversine, dim 2: latitude and longitude in degrees, bins in radians).  */
/* f (f_max x n fields; NaN = no data), pos (dim x n), bin_edges (n_bins + */
/* 1, non-decreasing) and directions (n_dirs x dim unit vectors) are device */
/* pointers; vario / counts (n_bins, or n_dirs x n_bins) device outputs,    */
/* counts int64.  Pairs are binned exactly as the reference bins them       */
/* (edge <= distance < next edge); sums are FP64 in another order (equal   */
/* within rounding), counts exact.                                          */
/* ----------------------------------------------------------------------- */
int gst_vario_unstructured(int dim, int64_t n, int64_t f_max, const double *f,
                           int64_t n_bins, const double *bin_edges, const double *pos,
                           int estimator, int distance_type, double *vario,
                           int64_t *counts, void *stream);
int gst_vario_directional(int dim, int64_t n, int64_t f_max, const double *f,
                          int64_t n_bins, const double *bin_edges, const double *pos,
                          int64_t n_dirs, const double *directions, double angles_tol,
                          double bandwidth, int separate_dirs, int estimator,
                          double *vario, int64_t *counts, void *stream);
/* Variogram along axis 0 of f (n0 x rest, row-major), lags 0 .. n0 - 1;   */
/* The directional estimators' angle test, the reference's
 * "acos(|s| / dist) < angles_tol", is decided exactly as
 * "|s| / dist > cos(b)" with b the midpoint of angles_tol and the next double
 * below it (the decision of a correctly rounded acos); this returns cos(b) as
 * a double-double (hi + lo).  Host-only, informational (no device needed). */
int gst_vario_angle_boundary(double angles_tol, double *cos_hi, double *cos_lo);

/* mask (n0 x rest bytes, nonzero = masked) may be NULL.  Deterministic.    */
int gst_vario_structured(int64_t n0, int64_t rest, const double *f,
                         const unsigned char *mask, int estimator, double *vario,
                         void *stream);

/* Operand format of the tensor-core grid path's split GEMM (hi*hi + hi*lo +
 * lo*hi): GST_TC_F16 (default; FP16 products at twice the TF32 rate, the
 * amplitudes normalised by a power of two) or GST_TC_TF32.  Both keep 10
 * explicit mantissa bits per part.  Process-wide; returns the previous kind
 * (or -1 for an unknown kind, leaving it unchanged).  A workspace filled by
 * gst_grid_tc_tables must be contracted under the kind it was filled with.
 * No counterpart in the reference. */
#define GST_TC_TF32 0
#define GST_TC_F16 1
int gst_grid_tc_set_operands(int kind);

/* gst_grid_tc_contract restricted to the output rows x_begin <= x < x_end
 * (first grid axis; both multiples of the 16-row pair block for 3-D grids,
 * 256 for 2-D grids, or x_end = axis_len[0]).  Rows outside are untouched, so
 * a caller can contract slab by slab and copy finished slabs to the host
 * while the next one computes.  No counterpart in the reference. */
int gst_grid_tc_contract_rows(int dim, int64_t n_modes, const int64_t *axis_len,
                              const void *workspace, size_t workspace_bytes,
                              void *out, int out_type, double scale,
                              int64_t x_begin, int64_t x_end, void *stream);

/* Host-buffer forms of gst_summate_grid_tc, gst_summate_incompr_grid_tc and
 * gst_summate_fourier_grid_tc: every array argument (axes, cov_samples /
 * modes, proj_cov, spectrum_factor, z_1, z_2) and `out` are in HOST memory,
 * as the reference's summators take and return them
 * (src/gstools/field/generator.py:266-268, :554-560, :682-689 call them with
 * numpy arrays).  The call copies the inputs to the device, contracts the
 * field in slabs along the first axis and copies each finished slab to
 * `out` on a library-owned copy stream while the next slab computes.  The
 * result is complete when `stream` is (synchronise it before reading
 * `out`).  `out` in page-locked memory (cudaHostAlloc / cudaHostRegister)
 * keeps the copies asynchronous; pageable `out` works but serialises them.
 * The inputs may be pageable. */
int gst_summate_grid_tc_host(int dim, int64_t n_modes, const int64_t *axis_len,
                             const double *axes, const double *cov_samples,
                             const double *z_1, const double *z_2, void *out,
                             int out_type, double scale, void *stream);
int gst_summate_incompr_grid_tc_host(int dim, int64_t n_modes,
                                     const int64_t *axis_len, const double *axes,
                                     const double *cov_samples,
                                     const double *proj_cov, const double *z_1,
                                     const double *z_2, void *out, int out_type,
                                     double scale, void *stream);
int gst_summate_fourier_grid_tc_host(int dim, int64_t n_modes,
                                     const int64_t *axis_len, const double *axes,
                                     const double *spectrum_factor,
                                     const double *modes, const double *z_1,
                                     const double *z_2, void *out, int out_type,
                                     double scale, void *stream);

/* ----------------------------------------------------------------------- */
/* Diagnostics (no reference counterpart).                                  */
/* ----------------------------------------------------------------------- */

/* Launches one throughput probe on `stream`: kind 0 = FP32 FMA, 1 = FP64
 * FMA, 2 = SFU sin.approx.  *ops_per_launch receives the operations the
 * launch executes (an FMA counts 2 flops, a sin 1 op); the caller times the
 * launch.  `sink` is a device buffer of >= 256 floats. */
int gst_peak_probe(int kind, int64_t iters, float *sink,
                   double *ops_per_launch, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GSTOOLS_GB300_H */
