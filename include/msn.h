/*
 * msn.h -- C ABI of libmsn, the GB300 (sm_103a) implementation of the
 * PyMORESANE deconvolution hot path.
 *
 * Conventions
 *   - Every pointer named d_* is a device pointer on the current CUDA device.
 *   - Every entry point is stream-explicit (`stream` is a cudaStream_t passed
 *     as void*; NULL means the legacy default stream) and asynchronous with
 *     respect to the host unless stated otherwise.
 *   - Every entry point returns an int status: MSN_OK (0) or a negative
 *     MSN_ERR_* code; msn_last_error() returns a message for the calling
 *     thread's last failure.
 *   - Images are row-major float32, shape [ny][nx]; coefficient stacks are
 *     [planes][ny][nx] contiguous.
 *   - Scratch memory is supplied by the caller (d_work, work_bytes), sized by
 *     the matching *_workspace_bytes() query; the library itself never
 *     allocates device memory on these paths.
 *
 * The reference (ratt-ru/PyMORESANE) has no C interface: its GPU path is
 * Python calling pyCUDA kernels. Each entry point below names the reference
 * Python function (file:line) whose mode='gpu' behaviour it replaces.
 */
#ifndef MSN_H
#define MSN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSN_OK 0
#define MSN_ERR_INVALID (-1)   /* bad argument (shape, scale count, null pointer) */
#define MSN_ERR_CUDA (-2)      /* a CUDA runtime call or kernel launch failed */
#define MSN_ERR_WORKSPACE (-3) /* the supplied workspace is too small */
#define MSN_ERR_TIMEOUT (-4)   /* a bounded device-side wait gave up */

/* Message describing the calling thread's most recent failure ("" if none). */
const char *msn_last_error(void);

/* ABI version of this library (major * 10000 + minor * 100 + patch). */
int msn_version(void);

/* Number of kernels this library has launched in the process (all threads);
 * reset != 0 returns the count and sets it back to zero. Diagnostics only. */
unsigned long long msn_launch_count(int reset);

/* ---------------------------------------------------------------------------
 * IUWT (a trous, B3 spline [1,4,6,4,1]/16, dilation 2^s, mirror borders)
 * ------------------------------------------------------------------------- */

/* Bytes of scratch needed by msn_iuwt_decompose / msn_iuwt_recompose for an
 * ny x nx image (two planes). */
size_t msn_iuwt_workspace_bytes(int ny, int nx);  /* four planes of scratch */

/* Replaces iuwt_decomposition(in1, scale_count, scale_adjust, mode='gpu',
 * store_smoothed=...) -- pymoresane/iuwt.py:17 -> gpu_iuwt_decomposition
 * pymoresane/iuwt.py:384-499.
 * d_detail: [scale_count - scale_adjust][ny][nx] output.
 * d_smoothed: [ny][nx] output of the smoothest plane, or NULL.
 * Requires nx % 4 == 0, 0 <= scale_adjust <= scale_count and
 * 2^scale_count <= min(ny, nx). */
int msn_iuwt_decompose(const float *d_in, float *d_detail, float *d_smoothed, int ny, int nx,
                       int scale_count, int scale_adjust, void *d_work, size_t work_bytes,
                       void *stream);

/* Decomposition with the source mask applied in the detail pass:
 * d_detail[s] = d_mask[s] * w_s (float32 product), d_mask and d_detail
 * [scale_count - scale_adjust][ny][nx]. Replaces the minor-loop sequence
 * iuwt_decomposition(...) followed by extracted_sources_mask * Ap
 * (pymoresane/main.py:381-383,400-402,414-416) in one set of passes. */
int msn_iuwt_decompose_masked(const float *d_in, const float *d_mask, float *d_detail, int ny, int nx,
                              int scale_count, int scale_adjust, void *d_work, size_t work_bytes, void *stream);

/* msn_iuwt_decompose_masked for a mask with empty rows: d_row_flags
 * [planes][ny] (msn_row_flags of the mask) is 0 where a mask row is all zero,
 * and those detail rows are NOT written -- the caller keeps them zero (the
 * values there would be zeros). No counterpart in the reference: the minor
 * loop's A operator with a sparse extraction mask (main.py:375-384). */
int msn_iuwt_decompose_masked_rows(const float *d_in, const float *d_mask, const unsigned char *d_row_flags,
                                   float *d_detail, int ny, int nx, int scale_count, int scale_adjust, void *d_work,
                                   size_t work_bytes, void *stream);

/* Replaces iuwt_recomposition(in1, scale_adjust, mode='gpu',
 * smoothed_array=...) -- pymoresane/iuwt.py:43 -> gpu_iuwt_recomposition
 * pymoresane/iuwt.py:501-581.
 * d_detail: [planes][ny][nx]; d_smoothed: [ny][nx] or NULL (start from 0);
 * d_out: [ny][nx]. */
int msn_iuwt_recompose(const float *d_detail, int planes, const float *d_smoothed, float *d_out,
                       int ny, int nx, int scale_adjust, void *d_work, size_t work_bytes,
                       void *stream);

/* Row activity of a recomposition started from zero whose detail stack is zero
 * outside the rows flagged in d_row_flags [planes][ny] (msn_row_flags of the
 * extraction mask): d_act [planes + scale_adjust][ny] bytes, level s active
 * where any of its vertical taps at dilation 2^s in level s + 1 is active or
 * its own detail row is flagged. No counterpart in the reference (support of
 * msn_iuwt_recompose_rows for the minor loop's sparse A p). */
int msn_recompose_row_activity(const unsigned char *d_row_flags, int planes, int ny, int scale_adjust,
                               unsigned char *d_act, void *stream);

/* msn_iuwt_recompose (no smoothed plane) computing only the rows d_act marks
 * active and writing zeros elsewhere; equal to msn_iuwt_recompose on a detail
 * stack that is zero outside the flagged rows (up to the sign of zeros). */
int msn_iuwt_recompose_rows(const float *d_detail, int planes, const unsigned char *d_act, float *d_out, int ny,
                            int nx, int scale_adjust, void *d_work, size_t work_bytes, void *stream);

/* msn_iuwt_recompose_rows with almost no zero writes: rows that d_act marks
 * inactive at every level are neither computed nor written, so the caller
 * must keep them at zero in d_out and in planes 2 and 3 of the workspace
 * (clear both once, e.g. with cudaMemsetAsync, before the calls that share one
 * activity map; transforms sharing the workspace only use its planes 0 and 1).
 * Rows that one call's lower levels made non-zero are re-zeroed by the next
 * call's higher levels where those are inactive.
 * No counterpart in the reference (the minor loop's A p, main.py:375-384,
 * applied to a detail stack that is zero outside the mask rows). */
int msn_iuwt_recompose_active_rows(const float *d_detail, int planes, const unsigned char *d_act, float *d_out,
                                   int ny, int nx, int scale_adjust, void *d_work, size_t work_bytes, void *stream);

/* Same result as msn_iuwt_decompose, but the two scratch planes come from a
 * fixed device array inside libmsn.so instead of a caller workspace, so the
 * call allocates nothing. No counterpart in the reference: it exists for
 * callers that cannot allocate device memory themselves (a host pipeline whose
 * own pool allocator owns the GPU, or a loop that must never call cudaMalloc).
 * Limit: ny * nx <= 1,048,576 pixels (e.g. 1024 x 1024); larger images return
 * MSN_ERR_INVALID. The array (8 MiB) is reserved on every GPU
 * that loads the library until the process exits. The first call on each
 * device resolves the array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture. All calls share the one array:
 * calls that can overlap on the GPU (different streams, or different host
 * threads on the same device) race and must be serialised by the caller.
 * The resolved address is kept for the life of the process, so the library
 * must not be used on a device after cudaDeviceReset or any other teardown of
 * its primary context. */
int msn_iuwt_decompose_static(const float *d_in, float *d_detail, float *d_smoothed, int ny, int nx,
                              int scale_count, int scale_adjust, void *stream);

/* ---------------------------------------------------------------------------
 * Real 2-D FFTs and the PSF convolution (square grids, side m = 2^a in
 * [32, 8192] or 3 * 2^a in [24, 6144]; complex data is interleaved float2,
 * i.e. complex64)
 * ------------------------------------------------------------------------- */

/* Scratch bytes for msn_fft_convolve(n, m) and for msn_rfft2 / msn_irfft2 /
 * msn_psf_spectrum at grid side m. */
size_t msn_fft_workspace_bytes(int n, int m);

/* Number of complex64 elements of a packed PSF spectrum for grid side m. */
size_t msn_spectrum_elems(int m);

/* Packed spectrum (library layout, consumed by msn_fft_convolve) of a real
 * rows x cols PSF block placed at (off_r, off_c) in an m x m zero grid, i.e.
 * rfft2 of that grid. Replaces the PSF-spectrum set-up of
 * DataImage.moresane, pymoresane/main.py:135-213 (gpu_r2c_fft of the PSF or
 * of pad_array(PSF)). */
int msn_psf_spectrum(const float *d_psf, int rows, int cols, int m, int off_r, int off_c, void *d_spec,
                     void *d_work, size_t work_bytes, void *stream);

/* Converts a standard-layout rfft2 spectrum [m][m/2+1] into the packed
 * layout used by msn_fft_convolve. */
int msn_spectrum_pack(const void *d_std, int m, void *d_packed, void *stream);

/* Replaces fft_convolve(in1, in2, conv_device='gpu', conv_mode) --
 * pymoresane/iuwt_convolution.py:18-61: x [n][n] convolved with the PSF whose
 * packed spectrum is d_spec; linear != 0: m == 2n, result
 * crop_centre(fftshift(irfft2(rfft2(pad(x)) * H))); linear == 0: m == n,
 * result fftshift(irfft2(rfft2(x) * H)). d_out: [n][n]. */
int msn_fft_convolve(const float *d_x, int n, int m, const void *d_spec, float *d_out, int linear, void *d_work,
                     size_t work_bytes, void *stream);

/* msn_fft_convolve for an input known to be zero outside some rows: d_rows [n]
 * bytes, d_rows[r] != 0 where row r of d_x may be non-zero (rows flagged zero
 * must hold zeros). The result equals msn_fft_convolve's (zeros compare equal);
 * the 2048^2 linear case skips the row transforms of pairs of zero rows. Used
 * by the minor loop, whose vectors live on the rows of the extraction mask's
 * dilated support. No counterpart in the reference. */
int msn_fft_convolve_rows(const float *d_x, int n, int m, const void *d_spec, float *d_out, int linear,
                          const unsigned char *d_rows, void *d_work, size_t work_bytes, void *stream);

/* Reads and clears the status word of the persistent FFT kernels (synchronous):
 * bit 0 is set when a bounded wait for a bulk copy gave up, in which case the
 * convolution's output is not valid. No counterpart in the reference. */
int msn_fft_status(unsigned *out);

/* Grid sizes (persistent CTAs) the four-step 4096-point kernels launch with on the
 * current device under the current tuning values: out[0] forward rows, out[1]
 * columns, out[2] inverse rows. Introspection for the autotuner; no counterpart
 * in the reference. */
int msn_fft_sq_grids(int *out);

/* Replaces gpu_r2c_fft -- pymoresane/iuwt_convolution.py:76-106:
 * d_out [m][m/2+1] = rfft2(d_in [m][m]). */
int msn_rfft2(const float *d_in, int m, void *d_out, void *d_work, size_t work_bytes, void *stream);

/* Replaces gpu_c2r_ifft (+ scale_fft) -- pymoresane/iuwt_convolution.py:108-139:
 * d_out [m][m] = irfft2(d_in [m][m/2+1]) (divided by m^2). */
int msn_irfft2(const void *d_in, int m, float *d_out, void *d_work, size_t work_bytes, void *stream);

/* Replaces fft_shift -- pymoresane/iuwt_convolution.py:161-201: in-place
 * quadrant swap of an even m x m image. */
int msn_fft_shift(float *d_data, int m, void *stream);

/* Replaces contiguous_slice -- pymoresane/iuwt_convolution.py:204-239:
 * d_out [m/2][m/2] = d_in[m/4 : 3m/4, m/4 : 3m/4]. */
int msn_crop_centre(const float *d_in, int m, float *d_out, void *stream);

/* Replaces scale_fft -- pymoresane/iuwt_convolution.py:242-265:
 * d_data[i] /= divisor for i < count. */
int msn_scale(float *d_data, size_t count, float divisor, void *stream);

/* ---------------------------------------------------------------------------
 * Noise estimate, thresholding, labelling, source extraction
 * ------------------------------------------------------------------------- */

/* Scratch bytes for msn_mad_sigma / msn_source_extraction / msn_label on
 * `planes` planes of ny x nx. */
size_t msn_toolbox_workspace_bytes(int planes, int ny, int nx);

/* Replaces estimate_threshold(in1, edge_excl, int_excl) --
 * pymoresane/iuwt_toolbox.py:17-48: d_sigma[p] (float64 holding the float32
 * result, as the reference's float64 output array does) = median(|w_p| over
 * the pixel set) / 0.6745 (exact median; float32 mean of the two middle
 * values for even counts, float32 division). rects[8] = {y0, y1, x0, x1, ey0, ey1, ex0, ex1}: pixels in
 * [y0,y1) x [x0,x1) and not in [ey0,ey1) x [ex0,ex1) (host array). */
int msn_mad_sigma(const float *d_w, int planes, int ny, int nx, const int *rects, double *d_sigma, void *d_work,
                  size_t work_bytes, void *stream);

/* Replaces apply_threshold(in1, threshold, sigma_level) --
 * pymoresane/iuwt_toolbox.py:50-75 -- fused with the edge-suppression
 * product (pymoresane/main.py:292-293; d_supp_rects [planes][4] = {y0, y1,
 * x0, x1} kept region, or NULL) and the per-plane maximum used for the
 * normalised scale maxima (pymoresane/main.py:297-300; d_plane_max or NULL;
 * then d_work needs planes * 4 bytes). d_sigma: float64 [planes] (device);
 * the comparison |w| > sigma_level * sigma is made in float64. */
int msn_apply_threshold(const float *d_w, int planes, int ny, int nx, const double *d_sigma, double sigma_level,
                        const int *d_supp_rects, float *d_out, float *d_plane_max, void *d_work, size_t work_bytes,
                        void *stream);

/* Replaces source_extraction(in1, tolerance, mode='gpu', neg_comp) --
 * pymoresane/iuwt_toolbox.py:77-95 -> gpu_source_extraction :156-290.
 * d_mask (float32 0/1) and d_extracted (= mask * w, may be NULL) are
 * [planes][ny][nx]. */
int msn_source_extraction(const float *d_w, int planes, int ny, int nx, float tolerance, int neg_comp, float *d_mask,
                          float *d_extracted, void *d_work, size_t work_bytes, void *stream);

/* Per-plane maximum (of |w| when use_abs) as float32 [planes]; per_plane % 4
 * == 0; d_work needs planes * 4 bytes (np.max at pymoresane/main.py:267 and
 * iuwt_toolbox.py:127-129,232-234). */
int msn_plane_max(const float *d_w, int planes, size_t per_plane, int use_abs, float *d_out, void *d_work,
                  size_t work_bytes, void *stream);

/* 8-connected labelling of d_img != 0 with scipy.ndimage.label numbering (the
 * labelling used by pymoresane/iuwt_toolbox.py:130,235). d_labels int32
 * [ny][nx]; d_count (device int, may be NULL) receives the label count. */
int msn_label(const float *d_img, int ny, int nx, int *d_labels, int *d_count, void *d_work, size_t work_bytes,
              void *stream);

/* ---------------------------------------------------------------------------
 * CG minor loop / major loop vector work (float64 reductions, deterministic)
 * Scalar block d_scal (float64): [0] r.r  [1] p.Ap  [2] alpha  [3] rn.rn  [4] beta
 * ------------------------------------------------------------------------- */

/* Scratch bytes for every reduction below. Zero the workspace once after
 * allocating it: it holds the completion counter of the single-launch
 * reductions, which every call leaves at zero again. One workspace per stream
 * (calls that overlap on the GPU must not share it). */
size_t msn_reduce_workspace_bytes(void);

/* Accumulation type of every reduction of the library (CG inner products,
 * SNR norms, residual statistics), process-wide:
 *   64 (default): float32 four-element partials accumulated in float64;
 *   48: the same partials accumulated in float-float pairs (about 48
 *       significant bits, float32 pipes only) within each CTA and in float64
 *       across CTAs; faster on GB300, whose float64 rate is low;
 *   32: plain float32 accumulation.
 * The 48 and 32 settings exist for the precision comparison; the reference's
 * GPU path reduces on the host in its arrays' precision
 * (pymoresane/main.py:386-411). Minor-loop graphs are cached per setting.
 * Returns MSN_ERR_INVALID for other values. */
int msn_set_reduction_precision(int bits);
int msn_reduction_precision(void);

/* Tunable launch parameters, chosen per device by the autotuner
 * (pymoresane_gb300/tune.py) and read by every launch. Names and ranges:
 *   fft_four_step    0 or 1: the 2048^2 linear convolution with a 4096^2 PSF
 *                    runs on the four-step kernels (1) or the Stockham ones (0)
 *   fft_sq_fwd_ctas, fft_sq_col_ctas, fft_sq_inv_ctas
 *                    0..8: resident CTAs per SM of the three four-step kernels
 *                    (0: as many as fit)
 *   iuwt_threads     64, 128 or 256: threads per CTA of the a trous passes on
 *                    rows of up to 2048 floats
 *   iuwt_threads_wide  the same for wider rows
 * Results do not depend on them. Changing one invalidates cached minor-loop
 * graphs. No counterpart in the reference (which fixes its launch shapes,
 * 32 x 32 blocks, pymoresane/iuwt.py:452-460). */
int msn_tune_set(const char *name, int value);
int msn_tune_get(const char *name, int *value);
int msn_tune_reset(void);
unsigned msn_tune_epoch(void);

/* d_out2[0] = sum a*b, d_out2[1] = sum c*d (c, d may both be NULL) in float64
 * (np.dot at pymoresane/main.py:386-387,407-408). */
int msn_dot2(const float *d_a, const float *d_b, const float *d_c, const float *d_d, size_t n, double *d_out2,
             void *d_work, size_t work_bytes, void *stream);

/* d_out2[0] = sum a^2, d_out2[1] = sum (a - b)^2 in float64: the norms of
 * snr_ratio, pymoresane/iuwt_toolbox.py:292-306. */
int msn_snr_sums(const float *d_a, const float *d_b, size_t n, double *d_out2, void *d_work, size_t work_bytes,
                 void *stream);

/* The same two sums for float64 inputs, accumulated entirely in float64:
 * snr_ratio of float64 arrays (pymoresane/iuwt_toolbox.py:292-306, whose
 * np.linalg.norm reduces in the arrays' own float64). */
int msn_snr_sums_f64(const double *d_a, const double *d_b, size_t n, double *d_out2, void *d_work,
                     size_t work_bytes, void *stream);

/* Running model sources for the minor-loop SNR (pymoresane/main.py:413-424):
 * ms += alpha * q (float32, alpha = (float)scal[2]) where q = mask * W(H p) is
 * the plane stack formed for Ap; d_out2[0] = sum e^2, d_out2[1] =
 * sum (e - ms)^2 in float64 (e: the extracted sources). By linearity this
 * equals recomputing mask * W(H xn) from xn = x + alpha p. */
int msn_snr_update(const float *d_e, float *d_ms, const float *d_q, const double *d_scal, size_t n, double *d_out2,
                   void *d_work, size_t work_bytes, void *stream);

/* alpha = scal[0] / scal[1] -> scal[2]; xn = x + alpha p; *d_neg_count = #(xn < 0)
 * (pymoresane/main.py:386-390). */
/* Segment activity of a mask: d_flags[s] = 1 when any of the 128 floats
 * [128 s, 128 s + 128) of d_mask [n] is non-zero; msn_segment_flags_bytes(n)
 * bytes. No counterpart in the reference (support of the sparse SNR pass). */
size_t msn_segment_flags_bytes(size_t n);
int msn_segment_flags(const float *d_mask, size_t n, unsigned char *d_flags, void *stream);

/* d_flags[r] = 1 when row r of d_mask [rows][cols] has a non-zero element. */
int msn_row_flags(const float *d_mask, size_t rows, int cols, unsigned char *d_flags, void *stream);

/* msn_snr_update restricted to the segments flagged by msn_segment_flags of the
 * extraction mask (zero elsewhere in all three stacks); bit-identical result. */
int msn_snr_update_masked(const float *d_e, float *d_ms, const float *d_q, const double *d_scal, size_t n,
                          const unsigned char *d_flags, double *d_out2, void *d_work, size_t work_bytes,
                          void *stream);

int msn_cg_alpha_x(const float *d_x, const float *d_p, double *d_scal, float *d_xn, size_t n, int *d_neg_count,
                   void *stream);

/* xn[xn < 0] = 0; p = (xn - x) / alpha (pymoresane/main.py:394-397). */
int msn_cg_positivity(const float *d_x, float *d_xn, float *d_p, const double *d_scal, size_t n, void *stream);

/* rn = r - alpha Ap; scal[3] = rn.rn; scal[4] = beta = scal[3] / scal[0]
 * (pymoresane/main.py:405-409). */
int msn_cg_residual(const float *d_r, const float *d_ap, double *d_scal, float *d_rn, size_t n, void *d_work,
                    size_t work_bytes, void *stream);

/* msn_cg_alpha_x (without the negative count) and msn_cg_residual in one
 * pass, for the minor loop without positivity (main.py:386-390,405-409):
 * xn = x + alpha p, rn = r - alpha Ap, rn.rn and beta; bit-identical to the
 * two calls. */
int msn_cg_step(const float *d_x, const float *d_p, const float *d_r, const float *d_ap, double *d_scal, float *d_xn,
                float *d_rn, size_t n, void *d_work, size_t work_bytes, void *stream);

/* p = rn + beta p (pymoresane/main.py:411). */
int msn_cg_direction(const float *d_rn, float *d_p, const double *d_scal, size_t n, void *stream);

/* model[off_r + i][off_c + j] += sign * gain * x[i][j] in float32
 * (pymoresane/main.py:483,498); model has row pitch `pitch`. */
int msn_model_update(float *d_model, int pitch, const float *d_x, int n_sub, int off_r, int off_c, float gain,
                     int sign, void *stream);

/* out = a - b (float32; pymoresane/main.py:485). */
int msn_sub(const float *d_a, const float *d_b, float *d_out, size_t n, void *stream);

/* out = a + b (float32; the residual added to the restored model, pymoresane/main.py:614). */
int msn_add(const float *d_a, const float *d_b, float *d_out, size_t n, void *stream);

/* out = a * b (float32; mask products, pymoresane/main.py:383,402,416). */
int msn_mul(const float *d_a, const float *d_b, float *d_out, size_t n, void *stream);

/* Mean and standard deviation (float64) of a rows x cols region of an image
 * with row pitch `pitch` (np.std at pymoresane/main.py:490):
 * d_out4 = {sum, sum of squared deviations, mean, std}. */
int msn_region_std(const float *d_img, int pitch, int rows, int cols, int off_r, int off_c, double *d_out4,
                   void *d_work, size_t work_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Native minor loop (CUDA graph with device-side stop rules).
 *
 * Replaces the host-driven conjugate-gradient loop of DataImage.moresane,
 * pymoresane/main.py:365-457 (one host round trip per iteration). One call
 * runs a whole minor loop on the device: x = 0, model sources = 0,
 * r = p = rec, then CG iterations until one of the reference's stop rules
 * fires (main.py:420-455) or minor_loop_miter iterations are done. On
 * return x holds the solution the reference keeps (its xn when the loop
 * converged or hit the iteration cap, the previous x otherwise).
 * --------------------------------------------------------------------------- */
#define MSN_MINOR_RUNNING 0
#define MSN_MINOR_FALSE_DETECTION 1 /* minor == 1 and SNR > 40: xn discarded */
#define MSN_MINOR_CONVERGED 2       /* SNR > 40: xn kept */
#define MSN_MINOR_STALLED 3         /* minor > 2 and SNR <= previous SNR: xn discarded */
#define MSN_MINOR_ITERATION_CAP 4   /* minor == minor_loop_miter: xn kept */

typedef struct msn_minor_args {
    int n;                  /* sub-region side: every vector is n x n, row-major */
    int m;                  /* FFT grid side of spec (2n linear, n circular) */
    int linear;             /* convolution mode of msn_fft_convolve */
    int max_scale;          /* decomposition depth of A */
    int scale_adjust;       /* first kept scale; planes = max_scale - scale_adjust */
    int minor_loop_miter;   /* iteration cap */
    int enforce_positivity; /* clamp xn >= 0 (main.py:392-398) */
    int reserved;
    const void *spec;       /* packed sub-PSF spectrum (msn_psf_spectrum) */
    const float *rec;       /* R(extracted sources): initial r and p */
    float *x, *xn, *r, *rn, *p, *ap, *tmp; /* n*n each */
    float *planes;          /* planes x n x n: mask * W(H p) */
    const float *emask;     /* planes x n x n extraction mask */
    const float *esrc;      /* planes x n x n extracted sources */
    float *ms;              /* planes x n x n running model sources */
    double *scal;           /* 5 doubles: r.r, p.Ap, alpha, rn.rn, beta */
    double *snr2;           /* 2 doubles: |esrc|^2, |esrc - ms|^2 */
    int *neg;               /* 1 int: #(xn < 0) */
    unsigned char *seg_flags; /* msn_segment_flags_bytes(planes * n * n) */
    unsigned char *row_flags; /* planes * n bytes */
    unsigned char *rec_rows;  /* max_scale * n bytes: recomposition row activity */
    void *fft_work;         /* msn_fft_workspace_bytes(n, m) */
    size_t fft_work_bytes;
    void *iuwt_work;        /* msn_iuwt_workspace_bytes(n, n) */
    size_t iuwt_work_bytes;
    void *red_work;         /* msn_reduce_workspace_bytes() */
    size_t red_work_bytes;
} msn_minor_args;

typedef struct msn_minor_result {
    int minor;           /* iterations performed */
    int outcome;         /* MSN_MINOR_* */
    int positivity_runs; /* iterations that clamped xn */
    int reserved;
    double snr_current;  /* SNR of the last iteration */
    double snr_last;     /* SNR of the iteration before it */
} msn_minor_result;

/* An engine owns a small device state block, capture streams and the cache of
 * instantiated graphs (keyed by the whole argument block); it belongs to the
 * device current at creation. One engine serves one caller thread at a time
 * (calls are serialised by a lock); use one engine per concurrent
 * deconvolution. */
int msn_minor_engine_create(void **engine);
int msn_minor_engine_destroy(void *engine);

/* Runs one minor loop on stream and waits for it. snr_history (host, may be
 * NULL) receives the SNR of each iteration, up to history_len entries. */
int msn_minor_loop(void *engine, const msn_minor_args *args, msn_minor_result *result, double *snr_history,
                   int history_len, void *stream);

/* ---------------------------------------------------------------------------
 * Native MORESANE run (major loop on the host side of the library).
 *
 * Replaces the major loop of DataImage.moresane, pymoresane/main.py:266-514,
 * for one PSF set-up: threshold (MAD, main.py:279-296), scale selection
 * (main.py:298-335), source extraction (main.py:337-351), the minor loop
 * (msn_minor_loop), model update, residual and the standard-deviation test
 * with revert (main.py:466-503). The caller prepares the PSF spectra, the
 * PSF scale energies and the buffers (sizes below), as the set-up code of
 * main.py:99-236 does, then one call runs every major iteration with no
 * interpreter involvement; log events and per-major records are returned in
 * caller arrays so that the caller can replay them into its own logger.
 * --------------------------------------------------------------------------- */
#define MSN_EV_MINIMUM_SCALE 1   /* a = min_scale */
#define MSN_EV_MAXIMUM_SCALE 2   /* a = max_scale */
#define MSN_EV_SCALE_EMPTY 3     /* a = scale_adjust */
#define MSN_EV_NO_COEFFICIENTS 4 /* no significant wavelet coefficients */
#define MSN_EV_MINOR_DONE 5      /* a = minor iterations, b = MSN_MINOR_* outcome, v = SNR */
#define MSN_EV_ALL_SCALES_POOR 6
#define MSN_EV_REVERTED 7        /* residual worsened: model change undone */
#define MSN_EV_MAJOR_DONE 8      /* a = major iterations so far */
#define MSN_EV_NO_WORK 9         /* the run did no work: complete */

typedef struct msn_event {
    int code, a, b, reserved;
    double v;
} msn_event;

typedef struct msn_major_record {
    int major, max_scale, scale_adjust, minor, outcome, reverted;
    double snr, std;
} msn_major_record;

typedef struct msn_moresane_args {
    int n;                   /* dirty image side */
    int ns;                  /* subregion side; the subregion starts at off = n/2 - ns/2 */
    int off;
    int scale_count;
    int m_sub, m_data;       /* FFT sides of spec_sub / spec_data */
    int linear;
    int major_loop_miter, minor_loop_miter;
    int enforce_positivity, neg_comp;
    int noise_rects[8];      /* estimate_threshold pixel set (msn_mad_sigma rects) */
    int reserved;
    double sigma_level, tolerance, accuracy, flux_threshold;
    float loop_gain;
    float reserved_f;
    const float *dirty;      /* n x n */
    const float *mask_sub;   /* ns x ns, or NULL */
    const int *supp_rects;   /* device [scale_count][4] (msn_apply_threshold), or NULL */
    const float *energies;   /* HOST [scale_count]: ||w_s|| of the PSF subregion (float32) */
    const void *spec_sub, *spec_data;
    float *model, *residual; /* n x n outputs */
    float *dec, *thr, *emask, *esrc, *planes, *ms; /* scale_count x ns x ns */
    float *x, *xn, *r, *rn, *p, *ap, *tmp, *rec, *masked, *sub; /* ns x ns */
    float *conv_full;        /* n x n */
    double *sigma;           /* scale_count */
    float *pmax;             /* scale_count */
    double *scal;            /* 5 */
    double *snr2;            /* 2 */
    double *std4;            /* 4 */
    int *neg;                /* 1 */
    unsigned char *seg_flags; /* msn_segment_flags_bytes(scale_count * ns * ns) */
    unsigned char *row_flags; /* scale_count * ns bytes */
    unsigned char *rec_rows;  /* scale_count * ns bytes */
    float *fmax;             /* 1 */
    void *small;             /* >= 16 and >= 4 * scale_count bytes */
    size_t small_bytes;
    void *iuwt_work;         /* msn_iuwt_workspace_bytes(ns, ns) */
    size_t iuwt_work_bytes;
    void *fft_work;          /* msn_fft_workspace_bytes(ns, m_sub) */
    size_t fft_work_bytes;
    void *fft_work_full;     /* msn_fft_workspace_bytes(n, m_data) */
    size_t fft_work_full_bytes;
    void *tool_work;         /* msn_toolbox_workspace_bytes(scale_count, ns, ns) */
    size_t tool_work_bytes;
    void *red_work;          /* msn_reduce_workspace_bytes() */
    size_t red_work_bytes;
} msn_moresane_args;

typedef struct msn_moresane_result {
    int major;          /* major iterations performed */
    int complete;       /* the run did no work (main.py:511-514) */
    int have_residual;  /* residual was written (at least one model update) */
    int n_records;      /* entries written to records */
    int n_events;       /* entries written to events */
    int events_dropped; /* events that did not fit */
} msn_moresane_result;

/* Runs one MORESANE deconvolution on stream (waits for it). */
int msn_moresane_run(void *engine, const msn_moresane_args *args, msn_moresane_result *result,
                     msn_major_record *records, int records_len, msn_event *events, int events_len, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MSN_H */
