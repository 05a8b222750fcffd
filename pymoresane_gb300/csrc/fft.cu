// Real 2-D FFTs and the fused PSF convolution for sm_103a.
//
// fft_convolve (pymoresane/iuwt_convolution.py:18-73) becomes three kernels:
//   1. rfft_rows: two real image rows packed into one complex sequence
//      (z = a + i b), zero-padded into the M-point grid, transformed in shared
//      memory and split into the two Hermitian half-spectra (R2C along x).
//   2. conv_cols: per group of C adjacent spectrum columns, the forward column
//      FFT, the product with the cached PSF spectrum and the inverse column FFT
//      in one pass; only the M/2 (linear) or M (circular) rows that survive
//      the fft-shift and the centre crop are written.
//   3. irfft_rows: the Hermitian rows are rebuilt into packed pairs, inverse
//      transformed, divided by M^2 (scale_fft, :242-265) and written with the
//      fft-shift (:161-201) and crop (contiguous_slice, :204-239) folded into
//      the output index map.
// Intermediate spectra use a group-major layout [ceil(W/C)][rows][C] (W =
// M/2 + 1) so that the column pass moves contiguous blocks; the PSF spectrum
// is stored the same way ("packed" spectrum).
#include <mutex>

#include "fft_core.cuh"
#include "msn_common.cuh"

namespace msn {
namespace {

enum ColMode { kConv = 0, kFwd = 1, kInv = 2 };

template <int C>
struct GroupMajor {
    int rows;
    __device__ __forceinline__ size_t at(int r, int col) const {
        return ((size_t)(col / C) * rows + r) * C + (col % C);
    }
    __device__ __forceinline__ bool valid(int col, int) const { return true; }
};

struct RowMajor {
    int pitch;
    __device__ __forceinline__ size_t at(int r, int col) const { return (size_t)r * pitch + col; }
    __device__ __forceinline__ bool valid(int col, int w) const { return col < w; }
};

constexpr int launch_cap(int e) { return e == 16 ? 1024 : 512; }

// --------------------------------------------------------------------------
// 1. Row R2C: rows [2q, 2q+1] of a real nrows x ncols image placed at column
//    offset col_off of an M-point row; writes W = M/2 + 1 bins per row.
// --------------------------------------------------------------------------
template <int E, class OutL>
__global__ void __launch_bounds__(512)
rfft_rows(const float *__restrict__ x, int nrows, int ncols, int col_off, FftPlan plan, float2 *__restrict__ out,
          OutL lay, int w) {
    extern __shared__ float2 sm[];
    const int m = plan.m;
    const int team = m / E;
    const int p = threadIdx.x / team, t = threadIdx.x - p * team;
    const int pairs = blockDim.x / team;
    float2 *buf = sm + p * padded_len(m);
    const int ra = 2 * (blockIdx.x * pairs + p), rb = ra + 1;
    const bool has_a = ra < nrows, has_b = rb < nrows;
    for (int n = t; n < m; n += team) {
        const int c = n - col_off;
        float a = 0.0f, b = 0.0f;
        if (c >= 0 && c < ncols) {
            if (has_a) a = __ldg(x + (size_t)ra * ncols + c);
            if (has_b) b = __ldg(x + (size_t)rb * ncols + c);
        }
        buf[sidx(n)] = make_float2(a, b);
    }
    __syncthreads();
    fft_team<false, E>(buf, plan, t);
    for (int k = t; k < w; k += team) {
        const float2 zk = buf[sidx(k)];
        const float2 zm = buf[sidx(k == 0 ? 0 : m - k)];
        // Xa = (Z[k] + conj Z[M-k]) / 2, Xb = (Z[k] - conj Z[M-k]) / (2i)
        const float2 xa = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
        const float2 xb = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
        if (has_a) out[lay.at(ra, k)] = xa;
        if (has_b) out[lay.at(rb, k)] = xb;
    }
}

// --------------------------------------------------------------------------
// 2. Column pass over C adjacent columns. Input rows [0, in_rows) land at
//    sequence positions in_off + r (zero elsewhere); output row i takes
//    sequence position (i + shift) mod M.
// --------------------------------------------------------------------------
template <int E, int C, int MODE, class InL, class OutL>
__global__ void __launch_bounds__(launch_cap(E))
conv_cols(const float2 *__restrict__ in, InL in_lay, int in_rows, int in_off, const float2 *__restrict__ h,
          float2 *__restrict__ out, OutL out_lay, int out_rows, int shift, FftPlan plan, int w) {
    extern __shared__ float2 sm[];
    const int m = plan.m;
    const int plen = padded_len(m);
    const int team = m / E;
    const int col0 = blockIdx.x * C;
    // Load with the column index fastest: contiguous in the group-major layout.
    for (int idx = threadIdx.x; idx < m * C; idx += blockDim.x) {
        const int n = idx / C, cc = idx - n * C;
        const int r = n - in_off;
        float2 v = make_float2(0.0f, 0.0f);
        if (r >= 0 && r < in_rows && in_lay.valid(col0 + cc, w)) v = in[in_lay.at(r, col0 + cc)];
        sm[cc * plen + sidx(n)] = v;
    }
    __syncthreads();
    const int cc = threadIdx.x / team, t = threadIdx.x - cc * team;
    float2 *buf = sm + cc * plen;
    if (MODE != kInv) fft_team<false, E>(buf, plan, t);
    if (MODE == kConv) {
        const float2 *hg = h + (size_t)blockIdx.x * m * C;
        for (int idx = threadIdx.x; idx < m * C; idx += blockDim.x) {
            const int k = idx / C, c2 = idx - k * C;
            float2 *s = sm + c2 * plen + sidx(k);
            *s = cmul(*s, __ldg(hg + idx));
        }
        __syncthreads();
    }
    if (MODE != kFwd) fft_team<true, E>(buf, plan, t);
    for (int idx = threadIdx.x; idx < out_rows * C; idx += blockDim.x) {
        const int i = idx / C, c2 = idx - i * C;
        int n = i + shift;
        if (n >= m) n -= m;
        if (out_lay.valid(col0 + c2, w)) out[out_lay.at(i, col0 + c2)] = sm[c2 * plen + sidx(n)];
    }
}

// --------------------------------------------------------------------------
// 3. Row C2R of Hermitian half-rows [2q, 2q+1]; output column j takes
//    sample (j + shift) mod M, divided by `div` (M^2).
// --------------------------------------------------------------------------
template <int E, class InL>
__global__ void __launch_bounds__(512)
irfft_rows(const float2 *__restrict__ in, InL lay, int nrows, FftPlan plan, float *__restrict__ out, int out_cols,
           int shift, float div) {
    extern __shared__ float2 sm[];
    const int m = plan.m;
    const int team = m / E;
    const int half = m / 2;
    const int p = threadIdx.x / team, t = threadIdx.x - p * team;
    const int pairs = blockDim.x / team;
    float2 *buf = sm + p * padded_len(m);
    const int ra = 2 * (blockIdx.x * pairs + p), rb = ra + 1;
    const bool has_a = ra < nrows, has_b = rb < nrows;
    for (int k = t; k <= half; k += team) {
        float2 xa = has_a ? in[lay.at(ra, k)] : make_float2(0.0f, 0.0f);
        float2 xb = has_b ? in[lay.at(rb, k)] : make_float2(0.0f, 0.0f);
        if (k == 0 || k == half) {  // c2r uses only the real part of the DC and Nyquist bins
            xa.y = 0.0f;
            xb.y = 0.0f;
        }
        buf[sidx(k)] = make_float2(xa.x - xb.y, xa.y + xb.x);                 // Xa + i Xb
        if (k != 0 && k != half) buf[sidx(m - k)] = make_float2(xa.x + xb.y, xb.x - xa.y);  // conj(Xa) + i conj(Xb)
    }
    __syncthreads();
    fft_team<true, E>(buf, plan, t);
    for (int j = t; j < out_cols; j += team) {
        int n = j + shift;
        if (n >= m) n -= m;
        const float2 z = buf[sidx(n)];
        if (has_a) out[(size_t)ra * out_cols + j] = __fdiv_rn(z.x, div);
        if (has_b) out[(size_t)rb * out_cols + j] = __fdiv_rn(z.y, div);
    }
}

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

template <int C>
__global__ void pack_spectrum_kernel(const float2 *__restrict__ in, int m, int w, float2 *__restrict__ out) {
    const int groups = (w + C - 1) / C;
    const GroupMajor<C> lay{m};
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (size_t)groups * m * C;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int cc = (int)(idx % C);
        const size_t rest = idx / C;
        const int r = (int)(rest % m), g = (int)(rest / m);
        const int col = g * C + cc;
        out[lay.at(r, col)] = col < w ? in[(size_t)r * w + col] : make_float2(0.0f, 0.0f);
    }
}

// --------------------------------------------------------------------------
// Host-side planning.
// --------------------------------------------------------------------------
struct Plan {
    FftPlan p;
    int e;       // elements per thread (16 for 2^a, 24 for 3 * 2^a)
    int group;   // spectrum columns per column-pass CTA
    int w;       // m/2 + 1
    int groups;  // ceil(w / group)
};

bool make_plan(int m, Plan *pl) {
    if (m < 32) return false;
    int rem = m, np = 0;
    if (m % 3 == 0) {
        rem = m / 3;
        if ((rem & (rem - 1)) != 0 || rem < 8 || m > 6144) return false;
        pl->e = 24;
        pl->p.radix[np++] = 3;
        while (rem % 8 == 0 && rem > 1) {
            pl->p.radix[np++] = 8;
            rem /= 8;
        }
        if (rem > 1) pl->p.radix[np++] = rem;  // 2 or 4
    } else {
        if ((m & (m - 1)) != 0 || m > 8192) return false;
        pl->e = 16;
        while (rem % 16 == 0) {
            pl->p.radix[np++] = 16;
            rem /= 16;
        }
        if (rem > 1) pl->p.radix[np++] = rem;  // 2, 4 or 8
    }
    pl->p.m = m;
    pl->p.npass = np;
    pl->group = (m > 4096) ? 2 : 4;
    pl->w = m / 2 + 1;
    pl->groups = (pl->w + pl->group - 1) / pl->group;
    return true;
}

int row_pairs(const Plan &pl) {
    const int team = pl.p.m / pl.e;
    int pairs = 512 / team;
    const int by_smem = (110 * 1024) / (padded_len(pl.p.m) * (int)sizeof(float2));
    if (pairs > by_smem) pairs = by_smem;
    return pairs < 1 ? 1 : pairs;
}

template <class K>
void raise_smem(K kernel) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

template <int E, class OutL>
int launch_rfft_rows(const float *x, int nrows, int ncols, int col_off, const Plan &pl, float2 *out, OutL lay,
                     cudaStream_t st) {
    static std::once_flag once;
    std::call_once(once, [] { raise_smem(rfft_rows<E, OutL>); });
    const int pairs = row_pairs(pl);
    const int team = pl.p.m / E;
    const int npairs = (nrows + 1) / 2;
    const int grid = (npairs + pairs - 1) / pairs;
    const size_t smem = (size_t)pairs * padded_len(pl.p.m) * sizeof(float2);
    rfft_rows<E, OutL><<<grid, pairs * team, smem, st>>>(x, nrows, ncols, col_off, pl.p, out, lay, pl.w);
    return check_launch("rfft_rows");
}

template <int E, class InL>
int launch_irfft_rows(const float2 *in, InL lay, int nrows, const Plan &pl, float *out, int out_cols, int shift,
                      float div, cudaStream_t st) {
    static std::once_flag once;
    std::call_once(once, [] { raise_smem(irfft_rows<E, InL>); });
    const int pairs = row_pairs(pl);
    const int team = pl.p.m / E;
    const int npairs = (nrows + 1) / 2;
    const int grid = (npairs + pairs - 1) / pairs;
    const size_t smem = (size_t)pairs * padded_len(pl.p.m) * sizeof(float2);
    irfft_rows<E, InL><<<grid, pairs * team, smem, st>>>(in, lay, nrows, pl.p, out, out_cols, shift, div);
    return check_launch("irfft_rows");
}

template <int E, int C, int MODE, class InL, class OutL>
int launch_cols(const float2 *in, InL in_lay, int in_rows, int in_off, const float2 *h, float2 *out, OutL out_lay,
                int out_rows, int shift, const Plan &pl, cudaStream_t st) {
    static std::once_flag once;
    std::call_once(once, [] { raise_smem(conv_cols<E, C, MODE, InL, OutL>); });
    const int team = pl.p.m / E;
    const size_t smem = (size_t)C * padded_len(pl.p.m) * sizeof(float2);
    conv_cols<E, C, MODE, InL, OutL><<<pl.groups, C * team, smem, st>>>(in, in_lay, in_rows, in_off, h, out,
                                                                        out_lay, out_rows, shift, pl.p, pl.w);
    return check_launch("conv_cols");
}

// Dispatch helpers over (E, C).
template <class F>
int with_ec(const Plan &pl, F &&f) {
    if (pl.e == 16 && pl.group == 4) return f.template operator()<16, 4>();
    if (pl.e == 16 && pl.group == 2) return f.template operator()<16, 2>();
    if (pl.e == 24 && pl.group == 4) return f.template operator()<24, 4>();
    return f.template operator()<24, 2>();
}

size_t packed_elems(const Plan &pl, int rows) { return (size_t)pl.groups * rows * pl.group; }
size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

int get_plan(int m, Plan *pl, const char *fn) {
    if (!make_plan(m, pl))
        return set_error(MSN_ERR_INVALID, "%s: unsupported FFT size %d (need 2^a in [32, 8192] or 3*2^a in [24, 6144])",
                         fn, m);
    return MSN_OK;
}

}  // namespace

// Packed-spectrum forward transform of a real rows x cols block placed at
// (off_r, off_c) in an m x m zero grid. out: group-major [groups][m][C].
int psf_spectrum_impl(const float *psf, int rows, int cols, int m, int off_r, int off_c, float2 *out, float2 *t1,
                      cudaStream_t st) {
    Plan pl;
    MSN_TRY(get_plan(m, &pl, "msn_psf_spectrum"));
    return with_ec(pl, [&]<int E, int C>() -> int {
        const GroupMajor<C> l1{rows};
        MSN_TRY(launch_rfft_rows<E>(psf, rows, cols, off_c, pl, t1, l1, st));
        return launch_cols<E, C, kFwd>(t1, l1, rows, off_r, (const float2 *)nullptr, out, GroupMajor<C>{m}, m, 0,
                                       pl, st);
    });
}

int fft_convolve_impl(const float *x, int n, int m, const float2 *spec, float *out, int linear, float2 *t1,
                      float2 *t2, cudaStream_t st) {
    Plan pl;
    MSN_TRY(get_plan(m, &pl, "msn_fft_convolve"));
    const int off = linear ? (m - n) / 2 : 0;
    const int shift = (off + m / 2) % m;
    const float div = (float)m * (float)m;
    return with_ec(pl, [&]<int E, int C>() -> int {
        const GroupMajor<C> l1{n};
        MSN_TRY(launch_rfft_rows<E>(x, n, n, off, pl, t1, l1, st));
        MSN_TRY(launch_cols<E, C, kConv>(t1, l1, n, off, spec, t2, l1, n, shift, pl, st));
        return launch_irfft_rows<E>(t2, l1, n, pl, out, n, shift, div, st);
    });
}

size_t conv_workspace_bytes(int n, int m) {
    Plan pl;
    if (!make_plan(m, &pl) || n <= 0) return 0;
    return 2 * align256(packed_elems(pl, n) * sizeof(float2));
}

size_t spectrum_elems(int m) {
    Plan pl;
    if (!make_plan(m, &pl)) return 0;
    return packed_elems(pl, m);
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
    Plan pl;
    MSN_TRY(get_plan(m, &pl, fn));
    if (!d_psf || !d_spec) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    if (rows <= 0 || cols <= 0 || off_r < 0 || off_c < 0 || off_r + rows > m || off_c + cols > m)
        return set_error(MSN_ERR_INVALID, "%s: %d x %d block at (%d, %d) does not fit the %d grid", fn, rows, cols,
                         off_r, off_c, m);
    const size_t need = align256(packed_elems(pl, rows) * sizeof(float2));
    if (!d_work || work_bytes < need) return set_error(MSN_ERR_WORKSPACE, "%s: workspace %zu < %zu", fn, work_bytes, need);
    return psf_spectrum_impl(d_psf, rows, cols, m, off_r, off_c, (float2 *)d_spec, (float2 *)d_work,
                             as_stream(stream));
}

extern "C" int msn_fft_convolve(const float *d_x, int n, int m, const void *d_spec, float *d_out, int linear,
                                void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_fft_convolve";
    Plan pl;
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
    return fft_convolve_impl(d_x, n, m, (const float2 *)d_spec, d_out, linear, t1, t2, as_stream(stream));
}

extern "C" int msn_rfft2(const float *d_in, int m, void *d_out, void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_rfft2";
    Plan pl;
    MSN_TRY(get_plan(m, &pl, fn));
    if (!d_in || !d_out) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    const size_t need = align256(packed_elems(pl, m) * sizeof(float2));
    if (!d_work || work_bytes < need) return set_error(MSN_ERR_WORKSPACE, "%s: workspace %zu < %zu", fn, work_bytes, need);
    cudaStream_t st = as_stream(stream);
    float2 *t1 = (float2 *)d_work;
    return with_ec(pl, [&]<int E, int C>() -> int {
        const GroupMajor<C> l1{m};
        MSN_TRY(launch_rfft_rows<E>(d_in, m, m, 0, pl, t1, l1, st));
        return launch_cols<E, C, kFwd>(t1, l1, m, 0, (const float2 *)nullptr, (float2 *)d_out, RowMajor{pl.w}, m,
                                       0, pl, st);
    });
}

extern "C" int msn_irfft2(const void *d_in, int m, float *d_out, void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_irfft2";
    Plan pl;
    MSN_TRY(get_plan(m, &pl, fn));
    if (!d_in || !d_out) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    const size_t need = align256(packed_elems(pl, m) * sizeof(float2));
    if (!d_work || work_bytes < need) return set_error(MSN_ERR_WORKSPACE, "%s: workspace %zu < %zu", fn, work_bytes, need);
    cudaStream_t st = as_stream(stream);
    float2 *t2 = (float2 *)d_work;
    const float div = (float)m * (float)m;
    return with_ec(pl, [&]<int E, int C>() -> int {
        const GroupMajor<C> l2{m};
        MSN_TRY(launch_cols<E, C, kInv>((const float2 *)d_in, RowMajor{pl.w}, m, 0, (const float2 *)nullptr, t2, l2,
                                        m, 0, pl, st));
        return launch_irfft_rows<E>(t2, l2, m, pl, d_out, m, 0, div, st);
    });
}

extern "C" int msn_spectrum_pack(const void *d_std, int m, void *d_packed, void *stream) {
    clear_error();
    static const char *fn = "msn_spectrum_pack";
    Plan pl;
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
