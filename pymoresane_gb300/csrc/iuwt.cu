// Isotropic undecimated wavelet transform (a trous, B3 spline) for sm_103a.
//
// One kernel launch performs one complete separable smoothing at dilation d:
// a CTA owns a band of full-width rows; the axis-0 (vertical) pass reads the
// five taps straight from global memory with float4 loads (the taps of one
// output row are whole rows r, r +- d, r +- 2d, mirrored at the borders) and
// leaves the band in shared memory; the axis-1 (horizontal) pass then runs
// entirely out of shared memory, so any dilation up to the row length is
// handled without a horizontal halo. The epilogue optionally fuses the
// wavelet detail (w = C_s - smooth(C_{s+1})) or the recomposition add
// (rec = smooth(rec) + w), so no separate elementwise pass is ever launched.
//
// Arithmetic follows the reference's pyCUDA kernels bit for bit: FP32, centre
// product then four fused multiply-adds, axis 0 before axis 1
// (pymoresane/iuwt.py:588-659), detail as a rounded subtraction
// (pymoresane/iuwt.py:403-417) and the recomposition add as a rounded addition
// (pymoresane/iuwt.py:562).
#include <mutex>

#include "msn_common.cuh"

namespace msn {
namespace {

enum Epilogue { kStore = 0, kDetail = 1, kAdd = 2, kDetailMask = 3 };

constexpr int kThreads = 256;
constexpr int kMaxSmem = 200 * 1024;

__device__ __forceinline__ float4 b3_tap4(const float4 &xc, const float4 &a, const float4 &b, const float4 &e,
                                          const float4 &f) {
    float4 v;
    v.x = b3_tap(xc.x, a.x, b.x, e.x, f.x);
    v.y = b3_tap(xc.y, a.y, b.y, e.y, f.y);
    v.z = b3_tap(xc.z, a.z, b.z, e.z, f.z);
    v.w = b3_tap(xc.w, a.w, b.w, e.w, f.w);
    return v;
}

struct Taps4 {
    float4 c, a, b, e, f;
};

__device__ __forceinline__ Taps4 load_vertical(const float4 *__restrict__ in4, int r, int c4, int ny, int nx4, int d) {
    Taps4 t;
    t.c = __ldg(in4 + (size_t)r * nx4 + c4);
    t.a = __ldg(in4 + (size_t)mirror(r - 2 * d, ny) * nx4 + c4);
    t.b = __ldg(in4 + (size_t)mirror(r - d, ny) * nx4 + c4);
    t.e = __ldg(in4 + (size_t)mirror(r + d, ny) * nx4 + c4);
    t.f = __ldg(in4 + (size_t)mirror(r + 2 * d, ny) * nx4 + c4);
    return t;
}

// Horizontal pass for the four outputs at columns c .. c+3 of one shared-memory row.
__device__ __forceinline__ float4 horizontal4(const float *__restrict__ s, int c, int nx, int d) {
    const float4 *s4 = reinterpret_cast<const float4 *>(s);
    if (d <= 2 && c >= 4 && c + 8 <= nx) {
        // Window s[c-4 .. c+8) from three aligned LDS.128 covers every tap for d = 1, 2.
        const float4 w0 = s4[(c >> 2) - 1], w1 = s4[c >> 2], w2 = s4[(c >> 2) + 1];
        float e[12] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y, w2.z, w2.w};
        float4 v;
        float *vp = reinterpret_cast<float *>(&v);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int m = 4 + k;
            vp[k] = (d == 1) ? b3_tap(e[m], e[m - 2], e[m - 1], e[m + 1], e[m + 2])
                             : b3_tap(e[m], e[m - 4], e[m - 2], e[m + 2], e[m + 4]);
        }
        return v;
    }
    if (d >= 4 && c - 2 * d >= 0 && c + 3 + 2 * d < nx) {
        // Every tap offset is a multiple of 4: five aligned LDS.128.
        return b3_tap4(s4[c >> 2], s4[(c - 2 * d) >> 2], s4[(c - d) >> 2], s4[(c + d) >> 2], s4[(c + 2 * d) >> 2]);
    }
    float4 v;
    float *vp = reinterpret_cast<float *>(&v);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int cc = c + k;
        vp[k] = b3_tap(s[cc], s[mirror(cc - 2 * d, nx)], s[mirror(cc - d, nx)], s[mirror(cc + d, nx)],
                       s[mirror(cc + 2 * d, nx)]);
    }
    return v;
}

template <int EPI>
__global__ void __launch_bounds__(kThreads)
atrous_band(const float *__restrict__ in, float *__restrict__ out, const float *__restrict__ aux,
            const float *__restrict__ mask, int ny, int nx, int d, int band_rows,
            const unsigned char *__restrict__ row_flags, int skip_inactive,
            const unsigned char *__restrict__ zero_rows) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ float4 smem4[];
    // masked detail with row flags: rows whose mask row is empty are left as they are (zero)
    if (EPI == kDetailMask && row_flags && band_rows == 1 && !row_flags[blockIdx.x]) return;
    // recomposition with row activity: an inactive output row is exactly zero (all its
    // taps and its detail row are zero), so it is written as zeros without reading anything
    if ((EPI == kAdd || EPI == kStore) && row_flags && band_rows == 1 && !row_flags[blockIdx.x]) {
        // skip mode: only rows in zero_rows need zeros (they may hold a previous call's values);
        // every other inactive row is kept at zero by the caller
        if (skip_inactive && !(zero_rows && zero_rows[blockIdx.x])) return;
        float4 *o4 = reinterpret_cast<float4 *>(out) + (size_t)blockIdx.x * (nx >> 2);
        for (int j = threadIdx.x; j < (nx >> 2); j += blockDim.x) o4[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float *band = reinterpret_cast<const float *>(smem4);
    const int r0 = blockIdx.x * band_rows;
    const int rows = min(band_rows, ny - r0);
    const int nx4 = nx >> 2;
    const int total4 = rows * nx4;
    const float4 *in4 = reinterpret_cast<const float4 *>(in);

    // Axis 0: two float4 columns per thread per iteration keep ten loads in flight.
    const int nt = blockDim.x;
    int i = threadIdx.x;
    for (; i + nt < total4; i += 2 * nt) {
        const int i2 = i + nt;
        const int rr1 = i / nx4, rr2 = i2 / nx4;
        const Taps4 t1 = load_vertical(in4, r0 + rr1, i - rr1 * nx4, ny, nx4, d);
        const Taps4 t2 = load_vertical(in4, r0 + rr2, i2 - rr2 * nx4, ny, nx4, d);
        smem4[i] = b3_tap4(t1.c, t1.a, t1.b, t1.e, t1.f);
        smem4[i2] = b3_tap4(t2.c, t2.a, t2.b, t2.e, t2.f);
    }
    if (i < total4) {
        const int rr = i / nx4;
        const Taps4 t = load_vertical(in4, r0 + rr, i - rr * nx4, ny, nx4, d);
        smem4[i] = b3_tap4(t.c, t.a, t.b, t.e, t.f);
    }
    __syncthreads();

    // Axis 1 out of shared memory (four columns per thread), fused epilogue, float4 stores.
    const float4 *aux4 = reinterpret_cast<const float4 *>(aux);
    float4 *out4 = reinterpret_cast<float4 *>(out);
    for (int j = threadIdx.x; j < total4; j += nt) {
        const int rr = j / nx4;
        const int c4 = j - rr * nx4;
        const size_t g4 = (size_t)(r0 + rr) * nx4 + c4;
        float4 x;
        if (EPI != kStore) x = __ldg(aux4 + g4);
        float4 v = horizontal4(band + rr * nx, c4 * 4, nx, d);
        if (EPI == kDetail || EPI == kDetailMask) {
            v.x = __fsub_rn(x.x, v.x);
            v.y = __fsub_rn(x.y, v.y);
            v.z = __fsub_rn(x.z, v.z);
            v.w = __fsub_rn(x.w, v.w);
        }
        if (EPI == kDetailMask) {  // mask * detail, as the reference's separate product (main.py:383)
            const float4 m = __ldg(reinterpret_cast<const float4 *>(mask) + g4);
            v.x = __fmul_rn(v.x, m.x);
            v.y = __fmul_rn(v.y, m.y);
            v.z = __fmul_rn(v.z, m.z);
            v.w = __fmul_rn(v.w, m.w);
        }
        if (EPI == kAdd) {
            v.x = __fadd_rn(v.x, x.x);
            v.y = __fadd_rn(v.y, x.y);
            v.z = __fadd_rn(v.z, x.z);
            v.w = __fadd_rn(v.w, x.w);
        }
        out4[g4] = v;
    }
}

// Fused decomposition step: one launch reads the smoothed plane C once and
// writes both the detail of scale s, w = (C0 - h_s * C) [* mask], and the next
// smoothing C' = h_{s+1} * C. The vertical taps of the two dilations d and 2d
// share the rows r +- 2d (seven row loads instead of ten); the two vertical
// results stay in shared memory and both horizontal passes and epilogues run
// from there. The arithmetic of each output is that of its own atrous_band
// pass, so the results are bit-identical to the unfused sequence.
// c0 may alias next: each element of c0 is read once, by the thread that
// writes next at the same index, before it writes (no __restrict__, no __ldg).
template <bool MASK>
__global__ void __launch_bounds__(kThreads)
atrous_pair(const float *__restrict__ in, const float *c0, const float *__restrict__ mask, float *__restrict__ w,
            float *next, int ny, int nx, int d, const unsigned char *__restrict__ row_flags) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ float4 smem4[];
    const int r = blockIdx.x;
    // with row flags, a row whose mask row is empty only needs the next smoothing
    const bool detail = !(MASK && row_flags && !row_flags[r]);
    const int nx4 = nx >> 2;
    const int nt = blockDim.x;
    const float4 *in4 = reinterpret_cast<const float4 *>(in);
    const size_t rc = (size_t)r * nx4, rm2 = (size_t)mirror(r - 2 * d, ny) * nx4,
                 rm1 = (size_t)mirror(r - d, ny) * nx4, rp1 = (size_t)mirror(r + d, ny) * nx4,
                 rp2 = (size_t)mirror(r + 2 * d, ny) * nx4, rm4 = (size_t)mirror(r - 4 * d, ny) * nx4,
                 rp4 = (size_t)mirror(r + 4 * d, ny) * nx4;
    for (int c4 = threadIdx.x; c4 < nx4; c4 += nt) {
        const float4 c = __ldg(in4 + rc + c4), a = __ldg(in4 + rm2 + c4), f = __ldg(in4 + rp2 + c4),
                     a2 = __ldg(in4 + rm4 + c4), f2 = __ldg(in4 + rp4 + c4);
        float4 b = make_float4(0.f, 0.f, 0.f, 0.f), e = b;
        if (detail) {
            b = __ldg(in4 + rm1 + c4);
            e = __ldg(in4 + rp1 + c4);
        }
        smem4[nx4 + c4] = b3_tap4(c, a2, a, f, f2);    // dilation 2d: taps r -+ 4d, r -+ 2d
        if (detail) smem4[c4] = b3_tap4(c, a, b, e, f);   // dilation d
    }
    __syncthreads();
    const float *band1 = reinterpret_cast<const float *>(smem4);
    const float *band2 = band1 + nx;
    const float4 *c04 = reinterpret_cast<const float4 *>(c0);
    float4 *w4 = reinterpret_cast<float4 *>(w);
    float4 *next4 = reinterpret_cast<float4 *>(next);
    for (int c4 = threadIdx.x; c4 < nx4; c4 += nt) {
        const size_t g4 = rc + c4;
        if (!detail) {
            next4[g4] = horizontal4(band2, c4 * 4, nx, 2 * d);
            continue;
        }
        const float4 x = c04[g4];
        float4 v = horizontal4(band1, c4 * 4, nx, d);
        v.x = __fsub_rn(x.x, v.x);
        v.y = __fsub_rn(x.y, v.y);
        v.z = __fsub_rn(x.z, v.z);
        v.w = __fsub_rn(x.w, v.w);
        if (MASK) {  // mask * detail, as the reference's separate product (main.py:383)
            const float4 mk = __ldg(reinterpret_cast<const float4 *>(mask) + g4);
            v.x = __fmul_rn(v.x, mk.x);
            v.y = __fmul_rn(v.y, mk.y);
            v.z = __fmul_rn(v.z, mk.z);
            v.w = __fmul_rn(v.w, mk.w);
        }
        w4[g4] = v;
        next4[g4] = horizontal4(band2, c4 * 4, nx, 2 * d);
    }
}

// Row activity of every level of a recomposition started from zero: the top
// level (scale max_scale - 1) is active where its detail rows are (mask row
// flags), each lower level where any of its five vertical taps at dilation 2^s
// is active or its own detail row is; scales below scale_adjust have no detail.
// One CTA, levels in sequence.
__global__ void recompose_activity(const unsigned char *__restrict__ qrows, int planes, int ny, int scale_adjust,
                                   unsigned char *__restrict__ act) {
    const int top = planes + scale_adjust - 1;
    for (int r = threadIdx.x; r < ny; r += blockDim.x) act[(size_t)top * ny + r] = qrows[(size_t)(planes - 1) * ny + r];
    __syncthreads();
    for (int s = top - 1; s >= 0; --s) {
        const unsigned char *up = act + (size_t)(s + 1) * ny;
        const int d = 1 << s;
        for (int r = threadIdx.x; r < ny; r += blockDim.x) {
            unsigned char a = up[r] | up[mirror(r - d, ny)] | up[mirror(r + d, ny)] | up[mirror(r - 2 * d, ny)] |
                              up[mirror(r + 2 * d, ny)];
            if (s >= scale_adjust) a |= qrows[(size_t)(s - scale_adjust) * ny + r];
            act[(size_t)s * ny + r] = a ? 1 : 0;
        }
        __syncthreads();
    }
}

// rec = 0 + w: the first recomposition step when no smoothed plane is given
// (the smoothing of an all-zero plane is exactly +0, and +0 + w maps -0 to +0
// exactly as the reference's addition does).
__global__ void zero_plus(const float4 *__restrict__ w, float4 *__restrict__ out, size_t n4) {
    pdl_wait();
    pdl_trigger();
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        float4 v = __ldg(w + i);
        v.x = __fadd_rn(0.0f, v.x);
        v.y = __fadd_rn(0.0f, v.y);
        v.z = __fadd_rn(0.0f, v.z);
        v.w = __fadd_rn(0.0f, v.w);
        out[i] = v;
    }
}

// rec = 0 + w on the rows act marks active (one row per CTA); inactive rows are
// not touched (the caller keeps them at zero).
__global__ void zero_plus_rows(const float4 *__restrict__ w, float4 *__restrict__ out, int nx4,
                               const unsigned char *__restrict__ act, const unsigned char *__restrict__ zero_rows) {
    pdl_wait();
    pdl_trigger();
    const size_t base = (size_t)blockIdx.x * nx4;
    if (!act[blockIdx.x]) {
        if (zero_rows && zero_rows[blockIdx.x])
            for (int j = threadIdx.x; j < nx4; j += blockDim.x) out[base + j] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    for (int j = threadIdx.x; j < nx4; j += blockDim.x) {
        float4 v = __ldg(w + base + j);
        v.x = __fadd_rn(0.0f, v.x);
        v.y = __fadd_rn(0.0f, v.y);
        v.z = __fadd_rn(0.0f, v.z);
        v.w = __fadd_rn(0.0f, v.w);
        out[base + j] = v;
    }
}

// One row per CTA. Measured on GB300 (one smoothing pass, d = 1 .. 256):
// 2048^2 10.3-14.4 us and 4096^2 33.9-45.1 us with one row, against 12.4-16.4
// and 43.0-63.5 us with three; a plain float4 copy of the same plane takes
// 6.2 and 22.6 us. Rows of the same dilation class that share vertical taps
// are then neighbouring CTAs, which read them from L2 close together in time.
int band_rows_for(int, int) { return 1; }

template <int EPI>
int launch_band(const float *in, float *out, const float *aux, int ny, int nx, int d, cudaStream_t st,
                const float *mask = nullptr, const unsigned char *row_flags = nullptr, int skip_inactive = 0,
                const unsigned char *zero_rows = nullptr) {
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(atrous_band<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    });
    const int band = band_rows_for(ny, nx);
    const size_t smem = (size_t)band * nx * sizeof(float);
    const int grid = (ny + band - 1) / band;
    const int work4 = band * (nx >> 2);
    const int cta = tune_value(nx <= 2048 ? kKnobIuwtThreads : kKnobIuwtThreadsWide);  // 64, 128 or 256
    const int threads = work4 >= cta ? cta : ((work4 + 31) / 32) * 32;
    return launch_k("atrous_band", atrous_band<EPI>, grid, threads, smem, st, in, out, aux, mask, ny, nx, d, band,
                    row_flags, skip_inactive, zero_rows);
}

// The fused step keeps two rows in shared memory.
bool pair_fits(int nx) { return (size_t)2 * nx * sizeof(float) <= (size_t)kMaxSmem; }

template <bool MASK>
int launch_pair(const float *in, const float *c0, const float *mask, float *w, float *next, int ny, int nx, int d,
                cudaStream_t st, const unsigned char *row_flags = nullptr) {
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(atrous_pair<MASK>, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmem);
    });
    const int nx4 = nx >> 2;
    const int cta = tune_value(nx <= 2048 ? kKnobIuwtThreads : kKnobIuwtThreadsWide);  // 64, 128 or 256
    const int threads = nx4 >= cta ? cta : ((nx4 + 31) / 32) * 32;
    return launch_k("atrous_pair", atrous_pair<MASK>, ny, threads, 2 * (size_t)nx * sizeof(float), st, in, c0, mask, w,
                    next, ny, nx, d, row_flags);
}

int launch_zero_plus(const float *w, float *out, size_t n, cudaStream_t st) {
    const size_t n4 = n / 4;
    int grid = (int)((n4 + kThreads - 1) / kThreads);
    if (grid > 152 * 16) grid = 152 * 16;
    return launch_k("zero_plus", zero_plus, grid, kThreads, 0, st, reinterpret_cast<const float4 *>(w),
                    reinterpret_cast<float4 *>(out), n4);
}

size_t plane_stride_bytes(int ny, int nx) { return (((size_t)ny * nx * sizeof(float)) + 255) & ~(size_t)255; }

int validate_image(int ny, int nx, const char *fn) {
    if (ny <= 0 || nx <= 0) return set_error(MSN_ERR_INVALID, "%s: empty image (%d x %d)", fn, ny, nx);
    if (nx % 4 != 0) return set_error(MSN_ERR_INVALID, "%s: nx=%d must be a multiple of 4", fn, nx);
    if ((size_t)nx * 4 > (size_t)kMaxSmem)
        return set_error(MSN_ERR_INVALID, "%s: nx=%d exceeds the supported row length", fn, nx);
    return MSN_OK;
}

int validate_scales(int ny, int nx, int top_scale, const char *fn) {
    // Scales 0 .. top_scale-1 are used; the mirror needs 2^(s+1) <= n.
    if (top_scale < 0 || top_scale > 30) return set_error(MSN_ERR_INVALID, "%s: bad scale count %d", fn, top_scale);
    const long long span = 1LL << top_scale;
    if (top_scale > 0 && (span > ny || span > nx))
        return set_error(MSN_ERR_INVALID, "%s: 2^%d exceeds the image side (%d x %d)", fn, top_scale, ny, nx);
    return MSN_OK;
}

}  // namespace

// Smoothing entry points shared with the other translation units.
int iuwt_smooth(const float *in, float *out, int ny, int nx, int scale, cudaStream_t st) {
    return launch_band<kStore>(in, out, nullptr, ny, nx, 1 << scale, st);
}
int iuwt_smooth_detail(const float *in, const float *c0, float *w, int ny, int nx, int scale, cudaStream_t st) {
    return launch_band<kDetail>(in, w, c0, ny, nx, 1 << scale, st);
}
int iuwt_smooth_add(const float *in, const float *w, float *out, int ny, int nx, int scale, cudaStream_t st,
                    const unsigned char *row_act = nullptr, int skip_inactive = 0,
                    const unsigned char *zero_rows = nullptr) {
    return launch_band<kAdd>(in, out, w, ny, nx, 1 << scale, st, nullptr, row_act, skip_inactive, zero_rows);
}
int iuwt_smooth_detail_mask(const float *in, const float *c0, const float *mask, float *w, int ny, int nx, int scale,
                            cudaStream_t st, const unsigned char *row_flags = nullptr) {
    return launch_band<kDetailMask>(in, w, c0, ny, nx, 1 << scale, st, mask, row_flags);
}

// Decomposition as the reference sequences it: per scale one smoothing and one
// detail pass (used for a single detail plane or rows too long for atrous_pair).
int iuwt_decompose_unfused(const float *d_in, float *d_detail, float *d_smoothed, int ny, int nx, int scale_count,
                           int scale_adjust, float *p0, float *p1, cudaStream_t st, const float *d_mask,
                           const unsigned char *d_row_flags) {
    const size_t plane = (size_t)ny * nx;
    float *bufs[2] = {p0, p1};
    const float *cur = d_in;
    int cur_buf = -1;
    auto next = [&]() { return cur_buf == 0 ? 1 : 0; };
    for (int s = 0; s < scale_adjust; ++s) {
        const int nb = next();
        MSN_TRY(iuwt_smooth(cur, bufs[nb], ny, nx, s, st));
        cur = bufs[nb];
        cur_buf = nb;
    }
    for (int s = scale_adjust; s < scale_count; ++s) {
        const bool last = (s == scale_count - 1);
        const int nb = next();
        float *c = (last && d_smoothed) ? d_smoothed : bufs[nb];
        MSN_TRY(iuwt_smooth(cur, c, ny, nx, s, st));
        float *w = d_detail + (size_t)(s - scale_adjust) * plane;
        if (d_mask)
            MSN_TRY(iuwt_smooth_detail_mask(c, cur, d_mask + (size_t)(s - scale_adjust) * plane, w, ny, nx, s, st,
                                            d_row_flags ? d_row_flags + (size_t)(s - scale_adjust) * ny : nullptr));
        else
            MSN_TRY(iuwt_smooth_detail(c, cur, w, ny, nx, s, st));
        cur = c;
        cur_buf = (c == d_smoothed) ? -1 : nb;
    }
    if (d_smoothed && cur != d_smoothed) {
        MSN_TRY(check_cuda(cudaMemcpyAsync(d_smoothed, cur, plane * sizeof(float), cudaMemcpyDeviceToDevice, st),
                           "copy smoothed plane"));
    }
    return MSN_OK;
}

// Decomposition with the detail pass of scale s fused with the smoothing of
// scale s + 1 (atrous_pair): scale_count - scale_adjust + 1 launches after the
// warm-up smoothings instead of twice that. Scratch: the two planes p0, p1.
// d_row_flags (masked only, may be null): [planes][ny] bytes, 0 where the mask
// row is empty; such detail rows are not written (the caller keeps them zero).
int iuwt_decompose_impl(const float *d_in, float *d_detail, float *d_smoothed, int ny, int nx, int scale_count,
                        int scale_adjust, float *p0, float *p1, cudaStream_t st, const float *d_mask = nullptr,
                        const unsigned char *d_row_flags = nullptr) {
    if (scale_count - scale_adjust < 2 || !pair_fits(nx))
        return iuwt_decompose_unfused(d_in, d_detail, d_smoothed, ny, nx, scale_count, scale_adjust, p0, p1, st,
                                      d_mask, d_row_flags);
    auto flags_of = [&](int s) {
        return d_row_flags ? d_row_flags + (size_t)(s - scale_adjust) * ny : nullptr;
    };
    const size_t plane = (size_t)ny * nx;
    float *bufs[2] = {p0, p1};
    const float *cur = d_in;  // C_{s-1}: the detail epilogue's minuend
    int cur_buf = -1;
    for (int s = 0; s < scale_adjust; ++s) {
        const int nb = cur_buf == 0 ? 1 : 0;
        MSN_TRY(iuwt_smooth(cur, bufs[nb], ny, nx, s, st));
        cur = bufs[nb];
        cur_buf = nb;
    }
    int c_buf = cur_buf == 0 ? 1 : 0;
    float *c = bufs[c_buf];  // C_s = h_s * C_{s-1}
    MSN_TRY(iuwt_smooth(cur, c, ny, nx, scale_adjust, st));
    for (int s = scale_adjust; s < scale_count - 1; ++s) {
        float *w = d_detail + (size_t)(s - scale_adjust) * plane;
        // C_{s+1} overwrites C_{s-1} (or fills the free plane / the caller's smoothed plane)
        float *next = (s == scale_count - 2 && d_smoothed) ? d_smoothed : bufs[1 - c_buf];
        if (d_mask)
            MSN_TRY(launch_pair<true>(c, cur, d_mask + (size_t)(s - scale_adjust) * plane, w, next, ny, nx, 1 << s,
                                      st, flags_of(s)));
        else
            MSN_TRY(launch_pair<false>(c, cur, nullptr, w, next, ny, nx, 1 << s, st));
        cur = c;
        c = next;
        c_buf = (next == d_smoothed) ? -1 : 1 - c_buf;
    }
    const int s = scale_count - 1;
    float *w = d_detail + (size_t)(s - scale_adjust) * plane;
    if (d_mask)
        MSN_TRY(iuwt_smooth_detail_mask(c, cur, d_mask + (size_t)(s - scale_adjust) * plane, w, ny, nx, s, st,
                                        flags_of(s)));
    else
        MSN_TRY(iuwt_smooth_detail(c, cur, w, ny, nx, s, st));
    return MSN_OK;
}

// d_act (may be null): [max_scale][ny] bytes, row r of the level of scale s is
// active when d_act[s * ny + r] != 0 (msn_recompose_row_activity); inactive rows
// are written as zeros without being computed.
// skip_inactive (with d_act, no smoothed plane): inactive rows are not computed.
// The levels alternate between p0 and p1, and activity only grows from the top
// level down, so a row a level leaves inactive can hold a value only if a lower
// level writing the same plane made it active (in an earlier call). Each level
// therefore writes zeros on the rows active at the lowest level of its plane but
// inactive at its own, and touches no other inactive row; the caller guarantees
// that rows never active anywhere hold zeros in p0, p1 and d_out
// (msn_iuwt_recompose_active_rows).
int iuwt_recompose_impl(const float *d_detail, int planes, const float *d_smoothed, float *d_out, int ny, int nx,
                        int scale_adjust, float *p0, float *p1, cudaStream_t st,
                        const unsigned char *d_act = nullptr, int skip_inactive = 0) {
    const size_t plane = (size_t)ny * nx;
    float *bufs[2] = {p0, p1};
    const int max_scale = planes + scale_adjust;
    const int total = planes + scale_adjust;
    const float *cur = d_smoothed;
    int cur_buf = -1, op = 0;
    auto dst_for = [&](int &nb) -> float * {
        nb = (cur_buf == 0) ? 1 : 0;
        return (op == total - 1) ? d_out : bufs[nb];
    };
    // lowest level (scale) written to each plane: ops alternate p0, p1 and the last op writes d_out
    int low_scale[2] = {-1, -1};
    for (int k = 0; k < total - 1; ++k) low_scale[k & 1] = max_scale - 1 - k;
    auto zero_rows_for = [&](float *dst, int nb) -> const unsigned char * {
        if (!skip_inactive || dst == d_out || low_scale[nb] < 0) return nullptr;
        return d_act + (size_t)low_scale[nb] * ny;
    };
    for (int s = max_scale - 1; s >= scale_adjust; --s, ++op) {
        int nb;
        float *dst = dst_for(nb);
        const float *w = d_detail + (size_t)(s - scale_adjust) * plane;
        if (cur == nullptr && skip_inactive) {
            MSN_TRY(launch_k("zero_plus_rows", zero_plus_rows, ny, 128, 0, st, reinterpret_cast<const float4 *>(w),
                             reinterpret_cast<float4 *>(dst), nx / 4, d_act + (size_t)s * ny, zero_rows_for(dst, nb)));
        } else if (cur == nullptr) {
            MSN_TRY(launch_zero_plus(w, dst, plane, st));
        } else {
            MSN_TRY(iuwt_smooth_add(cur, w, dst, ny, nx, s, st, d_act ? d_act + (size_t)s * ny : nullptr,
                                    skip_inactive, zero_rows_for(dst, nb)));
        }
        cur = dst;
        cur_buf = (dst == d_out) ? -1 : nb;
    }
    for (int s = scale_adjust - 1; s >= 0; --s, ++op) {
        int nb;
        float *dst = dst_for(nb);
        if (cur == nullptr) {
            MSN_TRY(check_cuda(cudaMemsetAsync(dst, 0, plane * sizeof(float), st), "zero plane"));
        } else if (d_act) {
            MSN_TRY(launch_band<kStore>(cur, dst, nullptr, ny, nx, 1 << s, st, nullptr, d_act + (size_t)s * ny,
                                        skip_inactive, zero_rows_for(dst, nb)));
        } else {
            MSN_TRY(iuwt_smooth(cur, dst, ny, nx, s, st));
        }
        cur = dst;
        cur_buf = (dst == d_out) ? -1 : nb;
    }
    if (total == 0) {
        if (d_smoothed) {
            MSN_TRY(check_cuda(cudaMemcpyAsync(d_out, d_smoothed, plane * sizeof(float), cudaMemcpyDeviceToDevice, st),
                               "copy smoothed plane"));
        } else {
            MSN_TRY(check_cuda(cudaMemsetAsync(d_out, 0, plane * sizeof(float), st), "zero plane"));
        }
    }
    return MSN_OK;
}

int split_workspace(void *d_work, size_t work_bytes, int ny, int nx, float **p0, float **p1, const char *fn) {
    const size_t need = msn_iuwt_workspace_bytes(ny, nx);
    if (d_work == nullptr || work_bytes < need)
        return set_error(MSN_ERR_WORKSPACE, "%s: workspace of %zu bytes given, %zu needed", fn, work_bytes, need);
    if (!aligned16(d_work)) return set_error(MSN_ERR_INVALID, "%s: workspace not 16-byte aligned", fn);
    *p0 = reinterpret_cast<float *>(d_work);
    *p1 = reinterpret_cast<float *>(reinterpret_cast<char *>(d_work) + plane_stride_bytes(ny, nx));
    return MSN_OK;
}

}  // namespace msn

using namespace msn;

extern "C" size_t msn_iuwt_workspace_bytes(int ny, int nx) {
    if (ny <= 0 || nx <= 0) return 0;
    // planes 0, 1: every transform's scratch; planes 2, 3: the recomposition of
    // msn_iuwt_recompose_active_rows, whose inactive rows the caller keeps at zero
    return 4 * plane_stride_bytes(ny, nx);
}

extern "C" int msn_iuwt_decompose(const float *d_in, float *d_detail, float *d_smoothed, int ny, int nx,
                                  int scale_count, int scale_adjust, void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_iuwt_decompose";
    MSN_TRY(validate_image(ny, nx, fn));
    MSN_TRY(validate_scales(ny, nx, scale_count, fn));
    if (scale_adjust < 0 || scale_adjust > scale_count)
        return set_error(MSN_ERR_INVALID, "%s: scale_adjust=%d outside [0, %d]", fn, scale_adjust, scale_count);
    if (!d_in || (scale_count > scale_adjust && !d_detail))
        return set_error(MSN_ERR_INVALID, "%s: null input or detail pointer", fn);
    if (!aligned16(d_in) || !aligned16(d_detail) || !aligned16(d_smoothed))
        return set_error(MSN_ERR_INVALID, "%s: device pointers must be 16-byte aligned", fn);
    float *p0, *p1;
    MSN_TRY(split_workspace(d_work, work_bytes, ny, nx, &p0, &p1, fn));
    return iuwt_decompose_impl(d_in, d_detail, d_smoothed, ny, nx, scale_count, scale_adjust, p0, p1,
                               as_stream(stream));
}

extern "C" int msn_iuwt_decompose_masked(const float *d_in, const float *d_mask, float *d_detail, int ny, int nx,
                                         int scale_count, int scale_adjust, void *d_work, size_t work_bytes,
                                         void *stream) {
    clear_error();
    static const char *fn = "msn_iuwt_decompose_masked";
    MSN_TRY(validate_image(ny, nx, fn));
    MSN_TRY(validate_scales(ny, nx, scale_count, fn));
    if (scale_adjust < 0 || scale_adjust > scale_count)
        return set_error(MSN_ERR_INVALID, "%s: scale_adjust=%d outside [0, %d]", fn, scale_adjust, scale_count);
    if (!d_in || !d_mask || (scale_count > scale_adjust && !d_detail))
        return set_error(MSN_ERR_INVALID, "%s: null input, mask or detail pointer", fn);
    if (!aligned16(d_in) || !aligned16(d_detail) || !aligned16(d_mask))
        return set_error(MSN_ERR_INVALID, "%s: device pointers must be 16-byte aligned", fn);
    float *p0, *p1;
    MSN_TRY(split_workspace(d_work, work_bytes, ny, nx, &p0, &p1, fn));
    return iuwt_decompose_impl(d_in, d_detail, nullptr, ny, nx, scale_count, scale_adjust, p0, p1, as_stream(stream),
                               d_mask);
}

extern "C" int msn_iuwt_decompose_masked_rows(const float *d_in, const float *d_mask, const unsigned char *d_row_flags,
                                              float *d_detail, int ny, int nx, int scale_count, int scale_adjust,
                                              void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_iuwt_decompose_masked_rows";
    MSN_TRY(validate_image(ny, nx, fn));
    MSN_TRY(validate_scales(ny, nx, scale_count, fn));
    if (scale_adjust < 0 || scale_adjust > scale_count)
        return set_error(MSN_ERR_INVALID, "%s: scale_adjust=%d outside [0, %d]", fn, scale_adjust, scale_count);
    if (!d_in || !d_mask || !d_row_flags || (scale_count > scale_adjust && !d_detail))
        return set_error(MSN_ERR_INVALID, "%s: null input, mask, row flags or detail pointer", fn);
    if (!aligned16(d_in) || !aligned16(d_detail) || !aligned16(d_mask))
        return set_error(MSN_ERR_INVALID, "%s: device pointers must be 16-byte aligned", fn);
    float *p0, *p1;
    MSN_TRY(split_workspace(d_work, work_bytes, ny, nx, &p0, &p1, fn));
    return iuwt_decompose_impl(d_in, d_detail, nullptr, ny, nx, scale_count, scale_adjust, p0, p1, as_stream(stream),
                               d_mask, d_row_flags);
}

extern "C" int msn_recompose_row_activity(const unsigned char *d_row_flags, int planes, int ny, int scale_adjust,
                                          unsigned char *d_act, void *stream) {
    clear_error();
    if (!d_row_flags || !d_act || planes < 1 || ny < 1 || scale_adjust < 0)
        return set_error(MSN_ERR_INVALID, "msn_recompose_row_activity: bad arguments");
    if (2LL << (planes + scale_adjust - 1) > 2LL * ny)
        return set_error(MSN_ERR_INVALID, "msn_recompose_row_activity: 2^%d exceeds the side %d",
                         planes + scale_adjust, ny);
    recompose_activity<<<1, 1024, 0, as_stream(stream)>>>(d_row_flags, planes, ny, scale_adjust, d_act);
    return check_launch("recompose_activity");
}

extern "C" int msn_iuwt_recompose_rows(const float *d_detail, int planes, const unsigned char *d_act, float *d_out,
                                       int ny, int nx, int scale_adjust, void *d_work, size_t work_bytes,
                                       void *stream) {
    clear_error();
    static const char *fn = "msn_iuwt_recompose_rows";
    MSN_TRY(validate_image(ny, nx, fn));
    if (planes < 1 || scale_adjust < 0) return set_error(MSN_ERR_INVALID, "%s: bad plane count / adjust", fn);
    MSN_TRY(validate_scales(ny, nx, planes + scale_adjust, fn));
    if (!d_out || !d_detail || !d_act) return set_error(MSN_ERR_INVALID, "%s: null detail, activity or output", fn);
    if (!aligned16(d_detail) || !aligned16(d_out))
        return set_error(MSN_ERR_INVALID, "%s: device pointers must be 16-byte aligned", fn);
    float *p0, *p1;
    MSN_TRY(split_workspace(d_work, work_bytes, ny, nx, &p0, &p1, fn));
    return iuwt_recompose_impl(d_detail, planes, nullptr, d_out, ny, nx, scale_adjust, p0, p1, as_stream(stream),
                               d_act);
}

extern "C" int msn_iuwt_recompose_active_rows(const float *d_detail, int planes, const unsigned char *d_act,
                                              float *d_out, int ny, int nx, int scale_adjust, void *d_work,
                                              size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_iuwt_recompose_active_rows";
    MSN_TRY(validate_image(ny, nx, fn));
    if (planes < 1 || scale_adjust < 0) return set_error(MSN_ERR_INVALID, "%s: planes=%d scale_adjust=%d", fn, planes,
                                                         scale_adjust);
    MSN_TRY(validate_scales(ny, nx, planes + scale_adjust, fn));
    if (!d_detail || !d_act || !d_out) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    if (!aligned16(d_detail) || !aligned16(d_out)) return set_error(MSN_ERR_INVALID, "%s: pointers not 16-byte aligned", fn);
    float *p0, *p1;
    MSN_TRY(split_workspace(d_work, work_bytes, ny, nx, &p0, &p1, fn));
    const size_t stride = plane_stride_bytes(ny, nx);
    float *q0 = reinterpret_cast<float *>(reinterpret_cast<char *>(d_work) + 2 * stride);
    float *q1 = reinterpret_cast<float *>(reinterpret_cast<char *>(d_work) + 3 * stride);
    return iuwt_recompose_impl(d_detail, planes, nullptr, d_out, ny, nx, scale_adjust, q0, q1, as_stream(stream), d_act,
                               1);
}

extern "C" int msn_iuwt_recompose(const float *d_detail, int planes, const float *d_smoothed, float *d_out, int ny,
                                  int nx, int scale_adjust, void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_iuwt_recompose";
    MSN_TRY(validate_image(ny, nx, fn));
    if (planes < 0 || scale_adjust < 0) return set_error(MSN_ERR_INVALID, "%s: negative plane count / adjust", fn);
    MSN_TRY(validate_scales(ny, nx, planes + scale_adjust, fn));
    if (!d_out || (planes > 0 && !d_detail)) return set_error(MSN_ERR_INVALID, "%s: null detail or output", fn);
    if (!aligned16(d_detail) || !aligned16(d_smoothed) || !aligned16(d_out))
        return set_error(MSN_ERR_INVALID, "%s: device pointers must be 16-byte aligned", fn);
    float *p0, *p1;
    MSN_TRY(split_workspace(d_work, work_bytes, ny, nx, &p0, &p1, fn));
    return iuwt_recompose_impl(d_detail, planes, d_smoothed, d_out, ny, nx, scale_adjust, p0, p1,
                               as_stream(stream));
}

// ---------------------------------------------------------------------------
// Decomposition with library-owned scratch, for callers that cannot allocate.
//
// Some hosts cannot hand this library any device scratch: a C or Fortran
// imaging pipeline whose own pool allocator owns all device memory, or a
// latency-critical loop that must never call cudaMalloc (it can block, fail
// under memory pressure, or implicitly synchronise the device). For them the
// decomposition's two intermediate planes live in a fixed device array that
// is part of the library image itself: it is reserved on every GPU that loads
// libmsn.so and stays there until the process exits, so the entry point below
// performs no allocation of any kind (no cudaMalloc, cudaFree or allocating
// library call). The caller still owns and passes the input and the outputs.
// ---------------------------------------------------------------------------
namespace msn {
namespace {

constexpr size_t kStaticScratchPixels = (size_t)1 << 20;  // 1,048,576 pixels, e.g. 1024 x 1024
constexpr size_t kStaticPlaneFloats = kStaticScratchPixels;

// Two planes of up to kStaticScratchPixels floats each: 8 MiB per device.
static __device__ __align__(256) float g_static_scratch[2 * kStaticPlaneFloats];

// Device address of g_static_scratch, resolved once per device. In host code
// the symbol is only a host-side stand-in and must never reach a kernel.
std::mutex g_static_mu;
float *g_static_addr[64] = {};

int static_scratch(float **out) {
    int device = 0;
    MSN_TRY(check_cuda(cudaGetDevice(&device), "cudaGetDevice"));
    if (device < 0 || device >= 64) return set_error(MSN_ERR_INVALID, "device index %d out of range", device);
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (g_static_addr[device] == nullptr) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        MSN_TRY(check_cuda(e, "cudaGetSymbolAddress(g_static_scratch)"));
        g_static_addr[device] = reinterpret_cast<float *>(p);
    }
    *out = g_static_addr[device];
    return MSN_OK;
}

}  // namespace
}  // namespace msn

extern "C" int msn_iuwt_decompose_static(const float *d_in, float *d_detail, float *d_smoothed, int ny, int nx,
                                         int scale_count, int scale_adjust, void *stream) {
    using namespace msn;
    clear_error();
    static const char *fn = "msn_iuwt_decompose_static";
    MSN_TRY(validate_image(ny, nx, fn));
    if ((size_t)ny * (size_t)nx > kStaticScratchPixels)
        return set_error(MSN_ERR_INVALID,
                         "%s: %d x %d = %zu pixels exceeds the static scratch limit of %zu pixels "
                         "(use msn_iuwt_decompose with a caller-supplied workspace)",
                         fn, ny, nx, (size_t)ny * nx, kStaticScratchPixels);
    MSN_TRY(validate_scales(ny, nx, scale_count, fn));
    if (scale_adjust < 0 || scale_adjust > scale_count)
        return set_error(MSN_ERR_INVALID, "%s: scale_adjust=%d outside [0, %d]", fn, scale_adjust, scale_count);
    if (!d_in || (scale_count > scale_adjust && !d_detail))
        return set_error(MSN_ERR_INVALID, "%s: null input or detail pointer", fn);
    if (!aligned16(d_in) || !aligned16(d_detail) || !aligned16(d_smoothed))
        return set_error(MSN_ERR_INVALID, "%s: device pointers must be 16-byte aligned", fn);
    float *scratch = nullptr;
    MSN_TRY(static_scratch(&scratch));
    // Both planes are written before they are read, so nothing needs clearing.
    return iuwt_decompose_impl(d_in, d_detail, d_smoothed, ny, nx, scale_count, scale_adjust, scratch,
                               scratch + kStaticPlaneFloats, as_stream(stream));
}
