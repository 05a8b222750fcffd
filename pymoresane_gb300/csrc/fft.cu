// Real 2-D FFTs and the fused PSF convolution: C ABI and length dispatch.
//
// The transform kernels are in fft_kernels.cuh, compiled per supported length
// M in fft_inst_*.cu; this file maps a runtime length onto those entry points
// and holds the small elementwise helpers of the reference's GPU path
// (fft_shift, contiguous_slice, scale_fft and the conversion of a standard
// spectrum into the packed layout).
#include "fft_plan.cuh"
#include "msn_common.cuh"

namespace msn {
namespace {

using fftk::CtPlan;
using fftk::ct_plan;

__global__ void fft_shift_kernel(float *__restrict__ d, int m) {
    // In-place quadrant swap of an even m x m image (fftshift == ifftshift).
    const int half = m / 2;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (size_t)half * m;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(idx / m), c = (int)(idx - (size_t)r * m);
        const int r2 = r + half, c2 = (c + half) % m;
        const size_t a = (size_t)r * m + c, b = (size_t)r2 * m + c2;
        const float t = d[a];
        d[a] = d[b];
        d[b] = t;
    }
}

__global__ void crop_centre_kernel(const float *__restrict__ in, int m, float *__restrict__ out) {
    const int n = m / 2, off = m / 4;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (size_t)n * n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(idx / n), c = (int)(idx - (size_t)r * n);
        out[idx] = in[(size_t)(r + off) * m + c + off];
    }
}

__global__ void scale_kernel(float *__restrict__ d, size_t count, float div) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        d[i] = __fdiv_rn(d[i], div);
}

// Standard layout [m][w] -> packed group-major layout [groups][m][C].
template <int C>
__global__ void pack_spectrum_kernel(const float2 *__restrict__ in, int m, int w, float2 *__restrict__ out) {
    const int groups = (w + C - 1) / C;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (size_t)groups * m * C;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int cc = (int)(idx % C);
        const size_t rest = idx / C;
        const int r = (int)(rest % m), g = (int)(rest / m);
        const int col = g * C + cc;
        out[idx] = col < w ? in[(size_t)r * w + col] : make_float2(0.0f, 0.0f);
    }
}


size_t packed_elems(const CtPlan &p, int rows) { return (size_t)p.groups * rows * p.group; }
size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

int get_plan(int m, CtPlan *p, const char *fn) {
    *p = ct_plan(m);
    if (!p->ok)
        return set_error(MSN_ERR_INVALID, "%s: unsupported FFT size %d (need 2^a in [32, 8192] or 3*2^a in [24, 6144])",
                         fn, m);
    return MSN_OK;
}

#define MSN_CASE_CONV(M) \
    case M:              \
        return fftk::conv_run<M>(x, n, spec, out, linear, t1, t2, st, rows);
int dispatch_conv(int m, const float *x, int n, const float2 *spec, float *out, int linear, float2 *t1, float2 *t2,
                  cudaStream_t st, const unsigned char *rows) {
    switch (m) { MSN_FFT_SIZES(MSN_CASE_CONV) }
    return set_error(MSN_ERR_INVALID, "unsupported FFT size %d", m);
}
#define MSN_CASE_SPEC(M) \
    case M:              \
        return fftk::spectrum_run<M>(psf, rows, cols, off_r, off_c, out, t1, st);
int dispatch_spectrum(int m, const float *psf, int rows, int cols, int off_r, int off_c, float2 *out, float2 *t1,
                      cudaStream_t st) {
    switch (m) { MSN_FFT_SIZES(MSN_CASE_SPEC) }
    return set_error(MSN_ERR_INVALID, "unsupported FFT size %d", m);
}
#define MSN_CASE_R2C(M) \
    case M:             \
        return fftk::rfft2_run<M>(in, out, t1, st);
int dispatch_rfft2(int m, const float *in, float2 *out, float2 *t1, cudaStream_t st) {
    switch (m) { MSN_FFT_SIZES(MSN_CASE_R2C) }
    return set_error(MSN_ERR_INVALID, "unsupported FFT size %d", m);
}
#define MSN_CASE_C2R(M) \
    case M:             \
        return fftk::irfft2_run<M>(in, out, t2, st);
int dispatch_irfft2(int m, const float2 *in, float *out, float2 *t2, cudaStream_t st) {
    switch (m) { MSN_FFT_SIZES(MSN_CASE_C2R) }
    return set_error(MSN_ERR_INVALID, "unsupported FFT size %d", m);
}

}  // namespace

size_t conv_workspace_bytes(int n, int m) {
    const CtPlan p = ct_plan(m);
    if (!p.ok || n <= 0) return 0;
    return 2 * align256(packed_elems(p, n) * sizeof(float2));
}

size_t spectrum_elems(int m) {
    const CtPlan p = ct_plan(m);
    return p.ok ? packed_elems(p, m) : 0;
}

}  // namespace msn

using namespace msn;

extern "C" size_t msn_fft_workspace_bytes(int n, int m) {
    // Enough for msn_fft_convolve(n, m) and for msn_rfft2 / msn_irfft2 / msn_psf_spectrum(m).
    const size_t a = conv_workspace_bytes(n, m);
    const size_t b = conv_workspace_bytes(m, m) / 2;
    return a > b ? a : b;
}

extern "C" size_t msn_spectrum_elems(int m) { return spectrum_elems(m); }

extern "C" int msn_psf_spectrum(const float *d_psf, int rows, int cols, int m, int off_r, int off_c, void *d_spec,
                                void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_psf_spectrum";
    CtPlan pl;
    MSN_TRY(get_plan(m, &pl, fn));
    if (!d_psf || !d_spec) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    if (rows <= 0 || cols <= 0 || off_r < 0 || off_c < 0 || off_r + rows > m || off_c + cols > m)
        return set_error(MSN_ERR_INVALID, "%s: %d x %d block at (%d, %d) does not fit the %d grid", fn, rows, cols,
                         off_r, off_c, m);
    const size_t need = align256(packed_elems(pl, rows) * sizeof(float2));
    if (!d_work || work_bytes < need) return set_error(MSN_ERR_WORKSPACE, "%s: workspace %zu < %zu", fn, work_bytes, need);
    return dispatch_spectrum(m, d_psf, rows, cols, off_r, off_c, (float2 *)d_spec, (float2 *)d_work,
                             as_stream(stream));
}

namespace msn {
// msn_fft_convolve with the rows of d_x that may be non-zero (rows[r] != 0, null: all rows).
int fft_convolve_rows(const float *d_x, int n, int m, const void *d_spec, float *d_out, int linear, void *d_work,
                      size_t work_bytes, const unsigned char *rows, cudaStream_t st) {
    static const char *fn = "msn_fft_convolve";
    CtPlan pl;
    MSN_TRY(get_plan(m, &pl, fn));
    if (!d_x || !d_spec || !d_out) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    if (linear && m != 2 * n) return set_error(MSN_ERR_INVALID, "%s: linear mode needs m == 2n (n=%d, m=%d)", fn, n, m);
    if (!linear && m != n) return set_error(MSN_ERR_INVALID, "%s: circular mode needs m == n (n=%d, m=%d)", fn, n, m);
    if (n % 2) return set_error(MSN_ERR_INVALID, "%s: image side %d must be even", fn, n);
    const size_t half = align256(packed_elems(pl, n) * sizeof(float2));
    if (!d_work || work_bytes < 2 * half)
        return set_error(MSN_ERR_WORKSPACE, "%s: workspace %zu < %zu", fn, work_bytes, 2 * half);
    float2 *t1 = (float2 *)d_work;
    float2 *t2 = (float2 *)((char *)d_work + half);
    return dispatch_conv(m, d_x, n, (const float2 *)d_spec, d_out, linear, t1, t2, st, rows);
}
}  // namespace msn

extern "C" int msn_fft_convolve(const float *d_x, int n, int m, const void *d_spec, float *d_out, int linear,
                                void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    return fft_convolve_rows(d_x, n, m, d_spec, d_out, linear, d_work, work_bytes, nullptr, as_stream(stream));
}

extern "C" int msn_fft_convolve_rows(const float *d_x, int n, int m, const void *d_spec, float *d_out, int linear,
                                     const unsigned char *d_rows, void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    if (!d_rows) return set_error(MSN_ERR_INVALID, "msn_fft_convolve_rows: null row flags");
    return fft_convolve_rows(d_x, n, m, d_spec, d_out, linear, d_work, work_bytes, d_rows, as_stream(stream));
}

extern "C" int msn_rfft2(const float *d_in, int m, void *d_out, void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_rfft2";
    CtPlan pl;
    MSN_TRY(get_plan(m, &pl, fn));
    if (!d_in || !d_out) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    const size_t need = align256(packed_elems(pl, m) * sizeof(float2));
    if (!d_work || work_bytes < need) return set_error(MSN_ERR_WORKSPACE, "%s: workspace %zu < %zu", fn, work_bytes, need);
    return dispatch_rfft2(m, d_in, (float2 *)d_out, (float2 *)d_work, as_stream(stream));
}

extern "C" int msn_irfft2(const void *d_in, int m, float *d_out, void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_irfft2";
    CtPlan pl;
    MSN_TRY(get_plan(m, &pl, fn));
    if (!d_in || !d_out) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    const size_t need = align256(packed_elems(pl, m) * sizeof(float2));
    if (!d_work || work_bytes < need) return set_error(MSN_ERR_WORKSPACE, "%s: workspace %zu < %zu", fn, work_bytes, need);
    return dispatch_irfft2(m, (const float2 *)d_in, d_out, (float2 *)d_work, as_stream(stream));
}

extern "C" int msn_spectrum_pack(const void *d_std, int m, void *d_packed, void *stream) {
    clear_error();
    static const char *fn = "msn_spectrum_pack";
    CtPlan pl;
    MSN_TRY(get_plan(m, &pl, fn));
    if (!d_std || !d_packed) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    const size_t total = packed_elems(pl, m);
    int grid = (int)((total + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    if (pl.group == 4)
        pack_spectrum_kernel<4><<<grid, 256, 0, as_stream(stream)>>>((const float2 *)d_std, m, pl.w, (float2 *)d_packed);
    else
        pack_spectrum_kernel<2><<<grid, 256, 0, as_stream(stream)>>>((const float2 *)d_std, m, pl.w, (float2 *)d_packed);
    return check_launch("pack_spectrum");
}

extern "C" int msn_fft_shift(float *d_data, int m, void *stream) {
    clear_error();
    if (!d_data || m <= 0 || m % 2) return set_error(MSN_ERR_INVALID, "msn_fft_shift: need an even side (got %d)", m);
    const size_t total = (size_t)(m / 2) * m;
    int grid = (int)((total + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    fft_shift_kernel<<<grid, 256, 0, as_stream(stream)>>>(d_data, m);
    return check_launch("fft_shift");
}

extern "C" int msn_crop_centre(const float *d_in, int m, float *d_out, void *stream) {
    clear_error();
    if (!d_in || !d_out || m <= 0 || m % 4)
        return set_error(MSN_ERR_INVALID, "msn_crop_centre: need a side divisible by 4 (got %d)", m);
    const size_t total = (size_t)(m / 2) * (m / 2);
    int grid = (int)((total + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    crop_centre_kernel<<<grid, 256, 0, as_stream(stream)>>>(d_in, m, d_out);
    return check_launch("crop_centre");
}

extern "C" int msn_scale(float *d_data, size_t count, float divisor, void *stream) {
    clear_error();
    if (!d_data && count) return set_error(MSN_ERR_INVALID, "msn_scale: null pointer");
    if (!count) return MSN_OK;
    int grid = (int)((count + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    scale_kernel<<<grid, 256, 0, as_stream(stream)>>>(d_data, count, divisor);
    return check_launch("scale");
}
