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

/* ---------------------------------------------------------------------------
 * IUWT (a trous, B3 spline [1,4,6,4,1]/16, dilation 2^s, mirror borders)
 * ------------------------------------------------------------------------- */

/* Bytes of scratch needed by msn_iuwt_decompose / msn_iuwt_recompose for an
 * ny x nx image (two planes). */
size_t msn_iuwt_workspace_bytes(int ny, int nx);

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

/* Replaces iuwt_recomposition(in1, scale_adjust, mode='gpu',
 * smoothed_array=...) -- pymoresane/iuwt.py:43 -> gpu_iuwt_recomposition
 * pymoresane/iuwt.py:501-581.
 * d_detail: [planes][ny][nx]; d_smoothed: [ny][nx] or NULL (start from 0);
 * d_out: [ny][nx]. */
int msn_iuwt_recompose(const float *d_detail, int planes, const float *d_smoothed, float *d_out,
                       int ny, int nx, int scale_adjust, void *d_work, size_t work_bytes,
                       void *stream);

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

#ifdef __cplusplus
}
#endif

#endif /* MSN_H */
