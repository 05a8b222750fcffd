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

#ifdef __cplusplus
}
#endif

#endif /* MSN_H */
