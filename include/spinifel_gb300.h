/*
 * spinifel_gb300 -- C ABI of the GB300 (sm_103a) orientation-matching and
 * 3D NUFFT library (libspinifel_gb300.so).
 *
 * Every entry point takes plain pointers and 64-bit sizes, runs on the CUDA
 * stream it is given (cudaStream_t passed as void*; NULL = legacy default
 * stream), never synchronises unless it says so, and returns an int status:
 *   SPF_OK (0) or a negative SPF_ERR_* code.  spf_last_error() returns a
 * thread-local message for the last failure on the calling thread.
 * Device pointers ("d_") must point to device memory of the current device;
 * host pointers ("h_") to host memory (pinned for asynchronous copies).
 *
 * Functions that replace a reference interface cite it as path:line within
 * the spinifel project.
 */
#ifndef SPINIFEL_GB300_H
#define SPINIFEL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPF_OK 0
#define SPF_ERR_ARG (-1)        /* bad argument (size, pointer, alignment)   */
#define SPF_ERR_OOM (-2)        /* device allocation failed                  */
#define SPF_ERR_TIMEOUT (-3)    /* a bounded device wait gave up             */
#define SPF_ERR_LAUNCH (-4)     /* kernel launch failed                      */
#define SPF_ERR_CUDA (-5)       /* other CUDA runtime / cuFFT error          */
#define SPF_ERR_UNSUPPORTED (-6) /* device or shape not supported            */

typedef struct spf_nufft_plan_s *spf_nufft_plan;
typedef struct spf_nufft64_plan_s *spf_nufft64_plan;
typedef struct spf_merge_s *spf_merge;
typedef struct spf_server_s *spf_server;
typedef struct spf_phaser_s *spf_phaser;

/* ---- library ---------------------------------------------------------- */
const char *spf_version(void);
const char *spf_status_string(int status);
const char *spf_last_error(void);
/* Number of kernels this library has launched in this process (all entry
 * points, all devices).  Used to count launches inside a timed region. */
uint64_t spf_launch_count(void);
/* Device-side error word written by bounded waits (0 = none); reset to 0. */
int spf_device_error(void *stream, int *h_code);
/* Self-test of the bounded-wait path used by the tensor-core kernels: one
 * thread waits on an mbarrier that nothing completes, gives up after
 * timeout_ms (1..5000), records -SPF_ERR_TIMEOUT in the device error word and
 * writes d_result[0] = 0 (gave up) / 1, d_result[1] = milliseconds waited. */
int spf_selftest_bounded_wait(int64_t timeout_ms, int *d_result, void *stream);

/* Runtime tunables, set by the autotuner (spinifel_gb300/autotune.py); 0
 * restores the built-in default.
 *   SPF_TUNE_BF16_GROUP_M : image tiles per rasterisation group of the
 *                           tensor-core kernels (default 16)
 *   SPF_TUNE_FP32_GROUP_M : the same for the plain FP32 kernels (default 8)
 *   SPF_TUNE_BF16_GRID    : persistent CTAs of the tensor-core kernels
 *                           (default: one per SM)
 *   SPF_TUNE_PRIME_DFT    : the merge regulariser on a prime grid size M
 *                           (read by spf_merge_create): 1 = Rader DFT
 *                           (default, when M - 1 is 2,3,5,7-smooth),
 *                           2 = cuFFT D2Z / Z2D
 *   SPF_TUNE_SLICE_SHAPE  : tile shape of spf_slice_t2_det (patch and warp
 *                           block, codes 0..5; 6 and 7 are shapes 0 and 1
 *                           with a per-CTA choice of the shared box's
 *                           strides against bank conflicts; default 0 =
 *                           16 x 16 patches of 4 x 8 warp blocks); every
 *                           shape gives the same bits
 *   SPF_TUNE_SORT_ITEM    : points per work item of the bin-sorted passes
 *                           (read by spf_nufft_sort_orient /
 *                           spf_nufft_sort_points; default 2048,
 *                           256 .. 8192)
 *   SPF_TUNE_STATIC_ABORT_TEST : 1 makes spf_match_bf16_static record a
 *                           given-up GEMM wait (SPF_ERR_TIMEOUT in its
 *                           error word, after the GEMM) so that tests can
 *                           check the void answers and the report through
 *                           spf_device_error without a device hang; 0
 *                           (default) in production */
#define SPF_TUNE_BF16_GROUP_M 1
#define SPF_TUNE_FP32_GROUP_M 2
#define SPF_TUNE_BF16_GRID 3
#define SPF_TUNE_PRIME_DFT 4
#define SPF_TUNE_SLICE_SHAPE 5
#define SPF_TUNE_SORT_ITEM 6
#define SPF_TUNE_STATIC_ABORT_TEST 7
int spf_tune_set(int param, int64_t value);
int spf_tune_get(int param, int64_t *value);

/* ---- NUFFT plan ---------------------------------------------------------
 * Replaces the cufinufft / finufft plans built in
 * spinifel/extern/nufft_ext.py:271-280 (type 2) and :308-319 (type 1).
 * Modes k = -floor(m/2) .. ceil(m/2)-1 on each axis of a C-ordered
 * (m1, m2, m3) array; the first coordinate runs along axis 0 (the reference
 * passes (L, K, H) to the Fortran-ordered library, cufinufft_ext.py:120-122).
 * eps selects the exponential-of-semicircle width (w = ceil(-log10(eps/10))
 * at upsampfac 2); upsampfac <= 0 selects 2.0. */
int spf_nufft_plan_create(int m1, int m2, int m3, double eps, double upsampfac,
                          spf_nufft_plan *out);
int spf_nufft_plan_destroy(spf_nufft_plan plan);
/* n_fine[3], kernel width, beta, padded fine-grid dims[3] */
int spf_nufft_plan_info(spf_nufft_plan plan, int *n_fine, int *width, double *beta,
                        int *n_padded);

/* Type 2 set-up: real modes d_modes (m1*m2*m3 float, C order), optionally
 * multiplied by d_support (same shape, NULL = none), deconvolved, FFT'd to
 * the fine grid; keeps Re (and Im when want_imag) of the fine grid in the
 * plan.  isign = -1 as in spinifel/extern/nufft_ext.py:63. */
int spf_nufft_t2_set_modes(spf_nufft_plan plan, const float *d_modes,
                           const float *d_support, int isign, int want_imag,
                           void *stream);

/* Type 2 at explicit points (radians, |x| < 3 pi): c_j real (and imaginary)
 * parts.  Replaces nufft_3d_t2 (spinifel/autocorrelation.py:59,
 * spinifel/extern/cufinufft_ext.py:384-) for real modes. */
int spf_nufft_t2_interp(spf_nufft_plan plan, const float *d_x, const float *d_y,
                        const float *d_z, int64_t npts, float *d_out_re,
                        float *d_out_im, void *stream);

/* Fused slicing (type 2 with coordinates made in the kernel): for each
 * orientation o (quaternion [w,x,y,z], d_quats[4*o]) and pixel p
 * (d_ppr = pixel_position_reciprocal, 3 x n_pix, float), the point
 * scale * R(q_o)^-1 . ppr[:,p] is evaluated; d_out[o*n_pix + p] = Re c.
 * scale = pi / (oversampling * max |q|).  Replaces NUFFT.forward
 * (spinifel/extern/nufft_ext.py:248-284) together with the host-side
 * HKL precompute it reads (nufft_ext.py:136-144).  When d_out_bf16 is not
 * NULL the same values are also written there rounded to bf16. */
int spf_slice_t2(spf_nufft_plan plan, const float *d_quats, int64_t n_orient,
                 const float *d_ppr, int64_t n_pix, double scale, float *d_out,
                 void *d_out_bf16, void *stream);

/* spf_slice_t2 for a detector of n_panels x nx x ny pixels (d_ppr is
 * 3 x n_panels x nx x ny, C order): 16 x 16 pixel patches are sliced from a
 * shared-memory copy of their grid footprint.  Same values as spf_slice_t2. */
int spf_slice_t2_det(spf_nufft_plan plan, const float *d_quats, int64_t n_orient,
                     const float *d_ppr, int n_panels, int nx, int ny, double scale,
                     float *d_out, void *d_out_bf16, void *stream);

/* Type 1: zero the plan's fine grid, spread real strengths, then FFT and
 * deconvolve onto the (m1, m2, m3) modes.  isign as in the caller
 * (+1 in spinifel/autocorrelation.py:118, -1 in nufft_ext.py:316).
 * d_out_re/d_out_im receive m1*m2*m3 floats (d_out_im may be NULL). */
int spf_nufft_t1_zero(spf_nufft_plan plan, void *stream);
int spf_nufft_t1_spread(spf_nufft_plan plan, const float *d_x, const float *d_y,
                        const float *d_z, const float *d_c, int64_t npts,
                        void *stream);
int spf_nufft_t1_spread_orient(spf_nufft_plan plan, const float *d_quats,
                               int64_t n_orient, const float *d_ppr, int64_t n_pix,
                               double scale, const float *d_c, void *stream);
int spf_nufft_t1_finish(spf_nufft_plan plan, int isign, float *d_out_re,
                        float *d_out_im, void *stream);
/* spf_nufft_t1_spread_orient / spf_nufft_interp_spread_orient for a detector
 * of n_panels x nx x ny pixels: 16 x 16 pixel patches spread into a
 * shared-memory box of their footprints, added to the accumulator once per
 * cell. */
int spf_nufft_t1_spread_det(spf_nufft_plan plan, const float *d_quats, int64_t n_orient,
                            const float *d_ppr, int n_panels, int nx, int ny, double scale,
                            const float *d_c, void *stream);
int spf_nufft_interp_spread_det(spf_nufft_plan plan, const float *d_quats, int64_t n_orient,
                                const float *d_ppr, int n_panels, int nx, int ny,
                                double scale, const float *d_weights, void *stream);

/* Bin-sorted points for repeated type 2 -> type 1 products over a fixed set
 * of orientation points (the direct merge operator): spf_nufft_sort_orient
 * places every point o*n_pix + p in its 8^3-cell bin of the padded fine grid
 * (a counting sort on the device; large bins split into 2048-point work
 * items) and keeps the order in the plan (allocates; synchronises the
 * stream once).  spf_nufft_interp_spread_sorted then does the fused
 * interpolate / weight / spread with each work item's grid box staged in
 * shared memory.  The points' geometry pointers must stay valid. */
int spf_nufft_sort_orient(spf_nufft_plan plan, const float *d_quats, int64_t n_orient,
                          const float *d_ppr, int64_t n_pix, double scale, void *stream);
/* The same bin sort for n explicit points (coordinates in radians, as
 * spf_nufft_t1_spread takes them); the sorted passes then read the points
 * from d_x, d_y, d_z, which must stay valid. */
int spf_nufft_sort_points(spf_nufft_plan plan, const float *d_x, const float *d_y,
                          const float *d_z, int64_t n, void *stream);
int spf_nufft_interp_spread_sorted(spf_nufft_plan plan, const float *d_weights, void *stream);
/* Type-1 spreading of real values (d_values[o*n_pix + p], or 1 for every
 * point when NULL) over the points sorted by spf_nufft_sort_orient, into the
 * plan's type-1 accumulator (spf_nufft_t1_zero before, spf_nufft_t1_finish
 * after), the adjoint's spreading stage (nufft_ext.py:287-327 NUFFT.adjoint;
 * autocorrelation.py:152-166, the type 1 of ones).  Points sharing a
 * footprint cell are summed in registers before the shared-memory adds. */
int spf_nufft_spread_sorted(spf_nufft_plan plan, const float *d_values, void *stream);

/* Fused type 2 -> type 1 at orientation points (the direct A^H D A product):
 * every point interpolates Re of the type-2 fine grid set by
 * spf_nufft_t2_set_modes, multiplies by d_weights[o*n_pix+p] (NULL = 1) and
 * spreads the product into the type-1 accumulator (zero it first with
 * spf_nufft_t1_zero, finish with spf_nufft_t1_finish).  Replaces the
 * forward / adjoint pair the reference's core_problem composes
 * (spinifel/autocorrelation.py:161-172). */
int spf_nufft_interp_spread_orient(spf_nufft_plan plan, const float *d_quats,
                                   int64_t n_orient, const float *d_ppr, int64_t n_pix,
                                   double scale, const float *d_weights, void *stream);

/* Type 1 in one call at explicit points (radians, |x| < 3 pi): zero the
 * accumulator, spread the real strengths d_c, fold, FFT and deconvolve onto
 * the modes (spf_nufft_t1_zero + _spread + _finish).  Replaces nufft_3d_t1 /
 * NUFFT.adjoint before the support multiply and the 1/M^3
 * (spinifel/autocorrelation.py:97-128, spinifel/extern/nufft_ext.py:287-327). */
int spf_spread_t1(spf_nufft_plan plan, const float *d_x, const float *d_y, const float *d_z,
                  const float *d_c, int64_t npts, int isign, float *d_out_re, float *d_out_im,
                  void *stream);

/* The FFT + deconvolution stage of either transform.  type 2: d_modes_in
 * (times d_support when not NULL) is deconvolved, zero-padded and
 * transformed onto the plan's fine grid (Re kept; spf_nufft_t2_set_modes
 * with want_imag 0), d_modes_out_* must be NULL.  type 1: the plan's spread
 * accumulator is folded, transformed and deconvolved into d_modes_out_re
 * (and _im when not NULL) (spf_nufft_t1_finish), d_modes_in and d_support
 * must be NULL.  The reference runs this stage inside cufinufft / finufft
 * (spinifel/extern/nufft_ext.py:271-282, :310-321). */
int spf_fft_deconv(spf_nufft_plan plan, int type, int isign, const float *d_modes_in,
                   const float *d_support, float *d_modes_out_re, float *d_modes_out_im,
                   void *stream);

/* ---- FP64 NUFFT plan (the reference's tolerance) -----------------------
 * The reference runs its NUFFTs at eps = 1e-12 in double
 * (spinifel/extern/nufft_ext.py:62; finufft_ext.py:70-89 for type 2,
 * finufft_ext.py:41-60 for type 1); an FP32 grid cannot reach that, so these
 * entry points repeat the FP32 plan's type 2 and type 1 in FP64 with kernel
 * widths up to 16 (w = 13 at eps 1e-12).  Same mode ordering, axis
 * convention and isign meaning as spf_nufft_plan_create.  eps in [1e-15, 1). */
int spf_nufft64_plan_create(int m1, int m2, int m3, double eps, double upsampfac,
                            spf_nufft64_plan *out);
int spf_nufft64_plan_destroy(spf_nufft64_plan plan);
int spf_nufft64_plan_info(spf_nufft64_plan plan, int *n_fine, int *width, double *beta,
                          int *n_padded);
/* spf_nufft_t2_set_modes in FP64 (d_modes, d_support: m1*m2*m3 doubles). */
int spf_nufft64_t2_set_modes(spf_nufft64_plan plan, const double *d_modes,
                             const double *d_support, int isign, int want_imag, void *stream);
/* spf_nufft_t2_interp in FP64 (NUFFT.forward at explicit points,
 * spinifel/autocorrelation.py:32-61). */
int spf_nufft64_t2_interp(spf_nufft64_plan plan, const double *d_x, const double *d_y,
                          const double *d_z, int64_t npts, double *d_out_re, double *d_out_im,
                          void *stream);
/* spf_slice_t2 in FP64: quaternions (4 per orientation) and pixel positions
 * (3 x n_pix) in double, rotation by R(q)^-1 in double, d_out[o*n_pix + p]
 * = Re c.  Replaces NUFFT.forward at the reference's eps
 * (spinifel/extern/nufft_ext.py:420-446 with the HKL precompute :136-144). */
int spf_slice_t2_f64(spf_nufft64_plan plan, const double *d_quats, int64_t n_orient,
                     const double *d_ppr, int64_t n_pix, double scale, double *d_out,
                     void *stream);
/* Type 1 in FP64: zero (allocates the accumulator on first use), spread real
 * strengths at explicit points, fold + FFT + deconvolve onto the modes
 * (NUFFT.adjoint before the support multiply and 1/M^3,
 * spinifel/extern/nufft_ext.py:450-487). */
int spf_nufft64_t1_zero(spf_nufft64_plan plan, void *stream);
int spf_nufft64_t1_spread(spf_nufft64_plan plan, const double *d_x, const double *d_y,
                          const double *d_z, const double *d_c, int64_t npts, void *stream);
int spf_nufft64_t1_finish(spf_nufft64_plan plan, int isign, double *d_out_re,
                          double *d_out_im, void *stream);

/* ---- orientation matching --------------------------------------------- */

/* pyCudaKNearestNeighbors.cudaEuclideanDistance
 * (spinifel/sequential/orientation_matching_sp.cu:612-680): d_out[d*n_ref+r]
 * = sum over the first 16*floor(n_pix/16) pixels of (data - ref)^2.
 * f32 and f64 variants (the _SP and _DP modules). */
int spf_knn_eudist_f32(const float *d_ref, const float *d_data, int64_t n_ref,
                       int64_t n_data, int64_t n_pix, float *d_out, void *stream);
int spf_knn_eudist_f64(const double *d_ref, const double *d_data, int64_t n_ref,
                       int64_t n_data, int64_t n_pix, double *d_out, void *stream);

/* pyCudaKNearestNeighbors.cudaHeapSort (orientation_matching_sp.cu:682-730):
 * the k smallest entries of each row of d_dist [n_data][n_ref], ascending,
 * indices written to d_idx [n_data][k]; ties go to the lower index.
 * k <= 32. */
int spf_knn_topk_f32(const float *d_dist, int64_t n_data, int64_t n_ref, int k,
                     int32_t *d_idx, void *stream);
int spf_knn_topk_f64(const double *d_dist, int64_t n_data, int64_t n_ref, int k,
                     int32_t *d_idx, void *stream);

/* Frame ingest: uint16 photon counts [n_img][n_pix] -> FP32 copy, and
 * optionally a bf16 copy (row stride ld >= n_pix, padding zeroed), the FP32
 * squared norm and sqrt(sum x^4) of each frame (NULL to skip).  Replaces
 * the host-side cast of the data images in SNM.__init__
 * (spinifel/sequential/orientation_matching.py:70-75). */
int spf_frames_ingest_u16(const uint16_t *d_counts, int64_t n_img, int64_t n_pix,
                          float *d_f32, void *d_bf16, int64_t ld, float *d_sq, float *d_n4,
                          void *stream);

/* Squared norms of rows: d_out[r] = sum_p x[r,p]^2 (FP32 data, FP32 result
 * accumulated in FP64 then rounded). */
int spf_row_sqnorm_f32(const float *d_x, int64_t n_rows, int64_t n_pix,
                       float *d_out, void *stream);

/* Plain FP32 matching, the drop-in for SNM.euclidean_dist + argmin
 * (spinifel/sequential/orientation_matching.py:98-109,179):
 * dist(i, r) = x2[i] + s2[r] - 2 x_i . s_r over all n_ref references
 * (ref_offset is added to the reported index), running minimum kept in
 * d_best (one uint64 per image: order-preserving float bits << 32 | index;
 * initialise with spf_best_init).  Ties go to the lower index. */
int spf_best_init(uint64_t *d_best, int64_t n_img, void *stream);
int spf_dist_argmin_f32(const float *d_img, const float *d_img_sq, int64_t n_img,
                        const float *d_ref, const float *d_ref_sq, int64_t n_ref,
                        int64_t n_pix, int64_t ref_offset, uint64_t *d_best,
                        void *stream);
int spf_best_unpack(const uint64_t *d_best, int64_t n_img, int32_t *d_idx,
                    float *d_dist, void *stream);

/* The whole plain FP32 match in one call (spf_best_init +
 * spf_dist_argmin_f32 + spf_best_unpack): best reference index and its
 * FP32 distance for every image; d_best (n_img uint64) is caller scratch.
 * Replaces SNM.euclidean_dist + argmin over all references
 * (spinifel/sequential/orientation_matching.py:98-109,179). */
int spf_dist_argmin_fp32(const float *d_img, const float *d_img_sq, int64_t n_img,
                         const float *d_ref, const float *d_ref_sq, int64_t n_ref,
                         int64_t n_pix, uint64_t *d_best, int32_t *d_idx, float *d_dist,
                         void *stream);

/* FP64 matching at the reference's double precision (use_single_prec =
 * false: SNM.euclidean_dist in float64, orientation_matching.py:32-36,
 * 98-109, and the sklearn branch of nearest_neighbor.py:134-135).
 * spf_dist_f64: d_out[d*n_ref + r] = sum over ALL n_pix pixels of
 * (data - ref)^2 in FP64.  spf_argmin_rows_f64 folds each row's minimum
 * (index + ref_offset; ties to the lower index; the running best changes only
 * on a strictly smaller distance) into d_best_dist / d_best_idx
 * (initialise with spf_best64_init: +inf, -1). */
int spf_dist_f64(const double *d_ref, const double *d_data, int64_t n_ref, int64_t n_data,
                 int64_t n_pix, double *d_out, void *stream);
int spf_best64_init(double *d_best_dist, int64_t *d_best_idx, int64_t n_img, void *stream);
int spf_argmin_rows_f64(const double *d_dist, int64_t n_img, int64_t n_ref, int64_t ref_offset,
                        double *d_best_dist, int64_t *d_best_idx, void *stream);

/* ---- autocorrelation merge: operator and device-resident CG -----------
 * Replaces Merge.setup_linops / W_matvec / cg
 * (spinifel/sequential/autocorrelation.py:152-225):
 *   W x = S.conv(S.x) + rlambda x + flambda S.reg(S.x)
 * with conv the Toeplitz product with ugrid_conv (type 1 of ones onto the
 * M_ups grid, / M_ups^3, spf_merge_set_kernel) divided by M^3, or (form 1)
 * the direct Re T1(D T2(.)) / (M_ups^3 M^3) through an attached NUFFT plan;
 * reg the size-M circular filter by ifftshift(F_antisupport) (:116-128).
 * d_support and d_antisupport are M^3 floats (C order, centred). */
int spf_merge_create(int M, int M_ups, double rlambda, double flambda,
                     const float *d_support, const float *d_antisupport, spf_merge *out);
int spf_merge_destroy(spf_merge merge);
int spf_merge_info(spf_merge merge, int *fft_size);
int spf_merge_set_kernel(spf_merge merge, const float *d_ugrid_conv, int M_ups,
                         void *stream);
/* The Toeplitz kernel in FP64 (d_ugrid_conv: M_ups^3 doubles): from this call
 * on the form-0 product runs in FP64 (D2Z / Z2D on the L grid) as the
 * reference's double-precision run computes it (use_single_prec false,
 * spinifel/sequential/autocorrelation.py:130-149); spf_merge_set_kernel
 * returns the operator to the FP32 product.  Allocates the FP64 buffers
 * (4 L^3 doubles) on the first call. */
int spf_merge_set_kernel_f64(spf_merge merge, const double *d_ugrid_conv, int M_ups,
                             void *stream);
/* The points are bin-sorted once here (spf_nufft_sort_orient) and every
 * direct-form product uses the sorted kernel; det_panels/det_nx/det_ny
 * describe a multi-panel detector (n_pix = their product, 0 = unordered). */
int spf_merge_set_direct(spf_merge merge, spf_nufft_plan plan, const float *d_quats,
                         int64_t n_orient, const float *d_ppr, int64_t n_pix, int det_panels,
                         int det_nx, int det_ny, double coord_scale, const float *d_weights);
/* d_y = W d_x (M^3 doubles); form 0 = Toeplitz, 1 = direct. */
int spf_merge_apply(spf_merge merge, int form, const double *d_x, double *d_y,
                    void *stream);
/* scipy.sparse.linalg.cg semantics: stop when ||r|| < rtol ||b|| or after
 * maxiter iterations; d_x holds x0 on entry (x0_is_zero skips W x0) and the
 * solution on return; FP64 vectors and dot products.  d_hist (maxiter
 * doubles, may be NULL) gets ||r|| at the start of each iteration and
 * d_iters (device int, may be NULL) the iteration count.  No host
 * synchronisation: the launch sequence can be captured in a CUDA graph. */
int spf_merge_cg(spf_merge merge, int form, const double *d_b, double *d_x, int x0_is_zero,
                 int maxiter, double rtol, double *d_hist, int *d_iters, void *stream);
/* Regularisation sweep (the MPI merge's per-rank lambdas,
 * spinifel/mpi/autocorrelation.py:64-68,160-214) as one batched solve: n_lambda
 * systems W_l x = c conv(x) + rlambda_l x + flambda_l reg(x) = d_adb +
 * rlambda_l x0 (h_rlambda / h_flambda: n_lambda host doubles; the merge's own
 * rlambda / flambda are not used), each CG from x0 (d_x0 M^3 doubles, NULL =
 * 0) with scipy's stopping rule, all systems advanced by the same launches;
 * c = conv_factor (1: the sequential merge's conv; M^3: the MPI merge's,
 * whose kernel transform lacks the 1/M^3, mpi/autocorrelation.py:95-104)
 * (batched cuFFT plans, allocated on the first call for a given n_lambda).
 * d_x: n_lambda x M^3 solutions; d_norms (may be NULL): 2 n_lambda doubles,
 * ||x_l|| and ||W_l x_l - d_l||; d_hist (may be NULL): n_lambda x maxiter
 * residual norms; d_iters (may be NULL): n_lambda ints.  Toeplitz form. */
int spf_merge_cg_sweep(spf_merge merge, int n_lambda, double conv_factor,
                       const double *h_rlambda, const double *h_flambda, const double *d_adb,
                       const double *d_x0,
                       double *d_x, int maxiter, double rtol, double *d_norms, double *d_hist,
                       int *d_iters, void *stream);
/* The same solve under the name of the reference's step: Merge.solve_ac's
 * cg(W, d, maxiter=...) (spinifel/sequential/autocorrelation.py:198-225). */
int spf_cg_solve(spf_merge merge, int form, const double *d_b, double *d_x, int x0_is_zero,
                 int maxiter, double rtol, double *d_hist, int *d_iters, void *stream);

/* ---- BF16 tensor-core matching with exact FP32 re-rank ----------------
 * The precision form of SNM.euclidean_dist + argmin
 * (spinifel/sequential/orientation_matching.py:98-109,179): x.s on tcgen05
 * tensor cores from bf16 copies (FP32 accumulation), the 8 smallest
 * s2 - 2 x.s per image and reference tile (tile t holds references
 * [t * R, (t + 1) * R), R = spf_dist_topk_bf16_tile_refs() = 224) written
 * to the candidate buffers d_cand_d / d_cand_i, each tiles * n_img * 8
 * entries with tiles = spf_dist_topk_bf16_tiles(n_ref) (scratch owned by the
 * caller).  Rows are ld bf16 elements apart (ld >= n_pix, ld % 8 == 0, pad
 * with 0).  Needs sm_103 (GB300). */
int64_t spf_dist_topk_bf16_tiles(int64_t n_ref);
int64_t spf_dist_topk_bf16_tile_refs(void);
int spf_dist_topk_bf16(const void *d_img_bf16, int64_t n_img, const void *d_ref_bf16,
                       int64_t n_ref, int64_t n_pix, int64_t ld, const float *d_ref_sq,
                       float *d_cand_d, int32_t *d_cand_i, void *stream);

/* Merge the candidates of all tiles into the per-frame top-8 (written over
 * tile 0 of the candidate buffers, so each candidate set is re-ranked once),
 * recompute those 8 distances in FP32 with exactly the arithmetic of
 * spf_dist_argmin_f32 (acc = fma(x_p, s_p, acc) in pixel order, then
 * (x2 + s2) - 2 acc: bit-identical values), return the best (d_idx, d_dist;
 * ties to the lower index; index + ref_offset) and, in d_uncertified (may be
 * NULL), 1 where the bf16 error bound cannot exclude a reference outside the
 * 8 (the caller then runs the exact path for that frame).  d_ref_m2 is the
 * per-pixel max over references of s^2 (spf_col_maxsq_f32), ref_sq_max the
 * largest s2; d_work (n_img floats) is scratch that on return holds each
 * frame's search bound for spf_dist_range_bf16.  d_top8 (may be NULL)
 * receives the 8 candidates. */
int spf_rerank_fp32(float *d_cand_d, int32_t *d_cand_i, int64_t n_tiles,
                    const float *d_img, const float *d_img_sq, int64_t n_img,
                    const float *d_ref, const float *d_ref_sq, const float *d_ref_m2,
                    float ref_sq_max, int64_t n_ref, int64_t n_pix, int64_t ref_offset,
                    float *d_work, int32_t *d_idx, float *d_dist, int32_t *d_uncertified,
                    int32_t *d_top8, void *stream);

/* Certified completion for frames the top-8 certificate left open: after
 * spf_rerank_fp32, d_work[i] holds the frame's search bound T_i (re-ranked
 * best minus x2 plus the error band).  spf_dist_range_bf16 runs the same
 * tensor-core GEMM and appends every reference r with s2_r - 2 x.s_r <= T_i
 * to d_list[i*cap ..] (d_count[i] = number found, zeroed by the call; a count
 * above cap means the list overflowed); spf_rerank_list_fp32 computes the
 * listed distances with the plain path's arithmetic and folds the
 * lexicographic minimum into d_best (the spf_best_* format); a frame whose
 * count is above cap is skipped (its list is incomplete). */
int spf_dist_range_bf16(const void *d_img_bf16, int64_t n_img, const void *d_ref_bf16,
                        int64_t n_ref, int64_t n_pix, int64_t ld, const float *d_ref_sq,
                        const float *d_thresh, int32_t *d_list, int32_t *d_count, int cap,
                        void *stream);
int spf_rerank_list_fp32(const int32_t *d_list, const int32_t *d_count, int cap,
                         const float *d_img, const float *d_img_sq, int64_t n_img,
                         const float *d_ref, const float *d_ref_sq, int64_t n_pix,
                         int64_t ref_offset, uint64_t *d_best, void *stream);

/* spf_rerank_fp32 that keeps the candidate buffers intact: the merged top-8
 * of each frame goes to d_merged_d / d_merged_i (n_img x 8 each) instead of
 * over tile 0, so that the per-tile lists remain for spf_complete_open. */
int spf_rerank_fp32_keep(const float *d_cand_d, const int32_t *d_cand_i, int64_t n_tiles,
                         const float *d_img, const float *d_img_sq, int64_t n_img,
                         const float *d_ref, const float *d_ref_sq, const float *d_ref_m2,
                         float ref_sq_max, int64_t n_ref, int64_t n_pix, int64_t ref_offset,
                         float *d_work, int32_t *d_idx, float *d_dist, int32_t *d_uncertified,
                         float *d_merged_d, int32_t *d_merged_i, void *stream);

/* Certified completion from the kept tile lists.  spf_scan_band_bf16: for
 * each open frame d_rows[r] with bound d_thresh[r] (spf_rerank_fp32's d_work
 * value), the references of every tile list whose approximate distance lies
 * within the bound go to d_list[r][..] (d_count[r] of them); a tile whose 8
 * entries all lie within the bound may hold more and sets d_count[r] to
 * cap + 1.  spf_complete_open runs the whole completion for n_rows open
 * frames: the scan, the exact re-rank of the lists (plain-path arithmetic),
 * the range GEMM for frames whose tile lists may hide references, and the
 * plain pass for a range list over its cap; d_idx / d_dist (n_rows each)
 * receive the answers in row order; h_stats (may be NULL) gets {frames sent
 * to the range GEMM, frames sent to the plain pass, 0}.  Allocates
 * stream-ordered scratch and synchronises the stream. */
int spf_scan_band_bf16(const float *d_cand_d, const int32_t *d_cand_i, int64_t n_tiles,
                       int64_t n_img, const int64_t *d_rows, int64_t n_rows,
                       const float *d_thresh, int32_t *d_list, int32_t *d_count, int cap,
                       void *stream);
int spf_complete_open(const float *d_cand_d, const int32_t *d_cand_i, int64_t n_tiles,
                      const void *d_img_bf16, const float *d_img, const float *d_img_sq,
                      const float *d_work, int64_t n_img, const int64_t *d_rows, int64_t n_rows,
                      const void *d_ref_bf16, const float *d_ref, const float *d_ref_sq,
                      int64_t n_ref, int64_t n_pix, int64_t ld, int32_t *d_idx, float *d_dist,
                      int64_t *h_stats, void *stream);

/* Batch matching from host memory in one synchronous call, the form of the
 * reference's slicing_and_match step (host frames in, host indices out;
 * spinifel/sequential/orientation_matching.py:113-186): h_counts [n_img][n_pix]
 * uint16 (pinned memory lets the copies overlap the work) is moved to the
 * device in chunks on an internal copy stream and ingested (FP32, bf16,
 * norms) on an internal ingest stream while the chunk before it is matched on
 * the tensor cores and re-ranked on `stream`; chunk_frames > 0 gives fixed
 * chunks, 0 fixed chunks of 2560 frames and a negative value chunks doubling
 * from -chunk_frames (>= -2^30).  The frames the certificate leaves open are
 * completed from each chunk's kept tile lists at the end.  h_idx / h_dist (n_img each;
 * h_dist may be NULL) receive the plain FP32 path's answer; h_stats (may be
 * NULL, 3 int64) gets {uncertified frames, frames completed by the range
 * GEMM, frames completed by the plain pass}.  Scratch comes from the
 * device's stream-ordered pool. */
int spf_match_bf16_host(const uint16_t *h_counts, int64_t n_img, const void *d_ref_bf16,
                        const float *d_ref, const float *d_ref_sq, const float *d_ref_m2,
                        float ref_sq_max, int64_t n_ref, int64_t n_pix, int64_t ld,
                        int64_t chunk_frames, int32_t *h_idx, float *h_dist, int64_t *h_stats,
                        void *stream);

/* Matching for callers that cannot allocate device memory: online
 * data-acquisition processes that fix their GPU memory when they start and
 * must not allocate while frames stream in, and plug-ins hosted by an
 * application whose own allocator owns the device's memory.
 * No counterpart in the reference.  Same result as spf_dist_topk_bf16 +
 * spf_rerank_fp32 (best index, exact FP32 distance, uncertified flags; the
 * caller completes uncertified frames), but all scratch lives in a static
 * device array of the library: 16 MiB + 16 KiB + 256 B held by every GPU
 * that loads the library until the process exits.  Limits per call: n_img <=
 * SPF_STATIC_MAX_FRAMES and spf_dist_topk_bf16_tiles(n_ref) * n_img <=
 * SPF_STATIC_MAX_TILE_FRAMES; larger calls are rejected with SPF_ERR_ARG.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and sets the kernel's shared-memory limit; make it
 * before any stream capture.  It calls no cudaMalloc or cudaFree.  All calls
 * on a device share the array: calls that overlap on the GPU race, so
 * serialise them.  If a bounded device wait of the tensor-core kernel gives
 * up, every frame of the call comes back void (d_idx -1, d_dist NaN,
 * d_uncertified 1) and spf_device_error reports the code. */
#define SPF_STATIC_MAX_FRAMES 4096
#define SPF_STATIC_MAX_TILE_FRAMES 262144
int spf_match_bf16_static(const void *d_img_bf16, const float *d_img, const float *d_img_sq,
                          int64_t n_img, const void *d_ref_bf16, const float *d_ref,
                          const float *d_ref_sq, const float *d_ref_m2, float ref_sq_max,
                          int64_t n_ref, int64_t n_pix, int64_t ld, int32_t *d_idx,
                          float *d_dist, int32_t *d_uncertified, void *stream);

/* ---- continuous-batching server ----------------------------------------
 * Streaming form of SNM.slicing_and_match's matching step
 * (spinifel/sequential/orientation_matching.py:113-186) against references
 * kept resident: requests of 1..slot_frames uint16 frames are queued, a
 * server thread packs whatever has arrived into a free slot (one CUDA stream
 * each; n_slots in flight) while the in-flight frames stay within
 * hbm_budget bytes (<= 0: slot_frames * n_slots frames' worth), and runs
 * copy-in, ingest, the bf16 tcgen05 top-8 + exact FP32 re-rank (path 0) or
 * the plain FP32 pass (path 1), and the certified completion of open frames.
 * Results equal spf_dist_argmin_fp32's on the same frames.  The reference
 * buffers (as for spf_rerank_fp32; d_ref_bf16/d_ref_m2 may be NULL for
 * path 1) must outlive the server.  spf_serve_create allocates every buffer
 * up front and starts the thread on `device`.
 * spf_serve_submit queues h_counts [n_frames][n_pix] (read when the request
 * is launched; keep it valid until the request completes; pinned memory is
 * copied directly, pageable memory through pinned staging) and returns a
 * ticket; h_idx / h_dist (n_frames each, h_dist may be NULL) receive the
 * answer before the request is marked done.  arrival: the request's arrival
 * time on spf_serve_clock() (< 0 = now), the start of its latency.
 * spf_serve_wait blocks up to timeout_ms (< 0 = until done); *done = 1 once
 * the request completed, and its status is returned (the ticket is then
 * released).  A bounded device wait that gave up fails the slot's requests
 * with SPF_ERR_TIMEOUT while the device error word stays set.
 * spf_serve_stats: h_out[0..8] = requests, frames, launches, uncertified
 * frames, frames whose tile lists could hide references (completed by the
 * range GEMM or the plain pass), summed GPU ms of the matching stage, budget
 * waits, p50 and p99 latency in ms.  spf_serve_destroy completes queued
 * requests, stops the thread and frees the buffers. */
double spf_serve_clock(void);
int spf_serve_create(int device, const void *d_ref_bf16, const float *d_ref,
                     const float *d_ref_sq, const float *d_ref_m2, float ref_sq_max,
                     int64_t n_ref, int64_t n_pix, int64_t ld, int path, int64_t slot_frames,
                     int n_slots, int64_t hbm_budget, spf_server *out);
int spf_serve_submit(spf_server server, const uint16_t *h_counts, int64_t n_frames,
                     int32_t *h_idx, float *h_dist, double arrival, int64_t *ticket);
int spf_serve_wait(spf_server server, int64_t ticket, int64_t timeout_ms, int *done);
int spf_serve_stats(spf_server server, double *h_out, int n_out);
int spf_serve_latencies(spf_server server, double *h_ms, int64_t cap, int64_t *n);
int spf_serve_destroy(spf_server server);

/* ---- phase retrieval ----------------------------------------------------
 * ER / HIO / shrink-wrap of spinifel/sequential/phasing.py in FP64 on the
 * device, for an M^3 grid (M odd in the reference: 4 Mquat + 1).  Arrays
 * with a trailing underscore are ifftshifted, as in the reference.
 * spf_phase_set_ac: ac (M^3 doubles, centred) -> ac_filt_ =
 *   ifftshift(gaussian_filter(max(ac, 0), sigma 1, truncate 2, zero
 *   boundary)) and amplitudes_ = sqrt(|fftn(ac_filt_)|)  (phasing.py:250-257).
 * spf_phase_create_support: support_ = central cube [Mquat, M-Mquat)^3 &
 *   ac_filt_ > 1e-2 max(ac_filt_)  (create_support_, :84-107).
 * spf_phase_set_state / _get_state copy rho_ (M^3 doubles) and support_
 *   (M^3 bytes, 0/1) in or out (either may be NULL).
 * spf_phase_er / _hio: n_loops of ER (:130-147) / HIO (:151-169), the
 *   Fourier projection replacing every amplitude but the (0,0,0) one.
 * spf_phase_shrink_wrap: support_ = gaussian_filter(|rho_|, sigma, periodic)
 *   > threshold, threshold std * weight (method 0) or max|rho_| * cutoff *
 *   weight (method 1)  (:193-221).
 * spf_phase_run: phase()'s schedule (:270-282): n_phase_loops x (ER, HIO,
 *   ER, shrink-wrap sigma 1), then ER.
 * spf_phase_finish: recenter rho_ and support_ on the centre of mass of
 *   |rho_| (rounded half to even; the three shifts go to h_shift when not
 *   NULL; synchronises the stream once), then d_ac_phased (M^3 doubles,
 *   centred) = fftshift(|ifftn(|fftn(rho_)|^2)|)  (:287-309).
 * No host synchronisation except in spf_phase_finish. */
int spf_phase_create(int M, spf_phaser *out);
int spf_phase_destroy(spf_phaser phaser);
int spf_phase_set_ac(spf_phaser phaser, const double *d_ac, void *stream);
int spf_phase_create_support(spf_phaser phaser, int Mquat, void *stream);
int spf_phase_set_state(spf_phaser phaser, const double *d_rho_, const uint8_t *d_support_,
                        void *stream);
int spf_phase_get_state(spf_phaser phaser, double *d_rho_, uint8_t *d_support_, void *stream);
int spf_phase_er(spf_phaser phaser, int n_loops, double rho_max, void *stream);
int spf_phase_hio(spf_phaser phaser, int n_loops, double beta, double rho_max, void *stream);
int spf_phase_shrink_wrap(spf_phaser phaser, double sigma, int method, double weight,
                          double cutoff, void *stream);
int spf_phase_run(spf_phaser phaser, int n_phase_loops, int n_er, int n_hio, double beta,
                  double rho_max, int method, double weight, double cutoff, void *stream);
int spf_phase_finish(spf_phaser phaser, double *d_ac_phased, int *h_shift, void *stream);

/* ---- frame preparation ---------------------------------------------------
 * Clipping and 2^n_bin x 2^n_bin binning of uint16 photon-count frames
 * [n_img][n_panels][sa][sb] in one pass (spinifel/prep.py:37-125,
 * binning_sum / binning_mean): the high-resolution border is clipped by
 * 2^n_clip (four PnCCD panels: panels 0 and 2 keep the last rows and columns,
 * 1 and 3 the last rows and first columns; one panel: the central region),
 * then blocks are summed (mean = 0) or averaged (mean = 1) exactly.
 * d_out: [n_img][n_panels][ca >> n_bin][cb >> n_bin] floats, ca x cb the
 * clipped panel.  Clipping of other panel counts is rejected (the reference
 * prints a message and returns zeros). */
int spf_bin_frames_u16(const uint16_t *d_raw, int64_t n_img, int n_panels, int sa, int sb,
                       int n_clip, int n_bin, int mean, float *d_out, void *stream);

/* ---- reconstruction quality (eval/fsc.py, eval/align.py) ----------------
 * Volumes are M^3 doubles, C order; quaternions [w, x, y, z] doubles.
 * spf_eval_score_rotations: d_cc[q] = Pearson correlation between vol1
 *   rotated by quaternion q (rotate_volume, align.py:36-67: trilinear,
 *   zero outside the grid) and vol2 -- score_deformations (align.py:92-120)
 *   without materialising the rotated copies.
 * spf_eval_rotate_volume: d_out [n_quat][M^3] = the rotated copies.
 * spf_eval_fsc_shells: d_sums [n_shells][3] = per shell i (i*spacing < |q| <
 *   i*spacing + spacing, |q| = |(c_a, c_b, c_c)| * scale on the fftshifted
 *   grid, d_coord = the M mesh coordinates) the sums of Re(F1 conj F2),
 *   |F1|^2 and |F2|^2 of F = fftshift(fftn(vol)) (fsc.py:67-125); the FSC is
 *   sums[0] / sqrt(sums[1] sums[2]).  These evaluation calls allocate
 *   stream-ordered scratch (cudaMallocAsync). */
int spf_eval_score_rotations(const double *d_vol1, const double *d_vol2, int M,
                             const double *d_quats, int64_t n_quat, double *d_cc, void *stream);
int spf_eval_rotate_volume(const double *d_vol, int M, const double *d_quats, int64_t n_quat,
                           double *d_out, void *stream);
int spf_eval_fsc_shells(const double *d_vol1, const double *d_vol2, int M, const double *d_coord,
                        double scale, double spacing, int n_shells, double *d_sums,
                        void *stream);

/* d_out[p] = max over rows r of x[r, p]^2 (n_pix floats). */
int spf_col_maxsq_f32(const float *d_x, int64_t n_rows, int64_t n_pix, float *d_out,
                      void *stream);

/* Row norms: d_sq[r] = sum x^2 and d_n4[r] = sqrt(sum x^4) (either may be
 * NULL), FP64 accumulation. */
int spf_row_norms_f32(const float *d_x, int64_t n_rows, int64_t n_pix, float *d_sq,
                      float *d_n4, void *stream);

/* Row gather: d_dst[i] = d_src[d_rows[i]] for rows of row_bytes bytes
 * (indices are not checked against n_src_rows on the device; the caller
 * guarantees 0 <= d_rows[i] < n_src_rows). */
int spf_gather_rows(const void *d_src, int64_t n_src_rows, int64_t row_bytes,
                    const int64_t *d_rows, int64_t n, void *d_dst, void *stream);

/* Row scatter, the inverse of spf_gather_rows: d_dst[d_rows[i]] = d_src[i]
 * (the caller guarantees 0 <= d_rows[i] < n_dst_rows, no repeats). */
int spf_scatter_rows(const void *d_src, int64_t row_bytes, const int64_t *d_rows, int64_t n,
                     void *d_dst, int64_t n_dst_rows, void *stream);

/* FP32 -> bf16 with a padded row stride: dst[r*ld + p] = bf16(src[r*n_pix+p])
 * for p < n_pix, 0 for n_pix <= p < ld. */
int spf_f32_to_bf16(const float *d_src, int64_t n_rows, int64_t n_pix, void *d_dst,
                    int64_t ld, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SPINIFEL_GB300_H */
