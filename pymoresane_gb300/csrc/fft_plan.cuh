// FFT plans (compile-time and host) and the per-length entry points of the
// FFT kernels. Supported lengths: M = 2^a (32 <= M <= 8192) and M = 3 * 2^a
// (24 <= M <= 6144); each is compiled as its own set of kernels with every
// stride, Ns and twiddle offset a compile-time constant.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace msn {
namespace fftk {

enum ColMode { kConv = 0, kFwd = 1, kInv = 2 };

// Radix sequence of one length. The main radix (16, or 8 next to the single
// radix 3) is placed first and last when it occurs at least twice, so that the
// PSF product can be fused between the last forward and the first inverse
// pass; the per-pass twiddle tables follow one another (twbase).
struct CtPlan {
    int e;          // elements per thread: 16 for 2^a, 24 for 3 * 2^a
    int np;         // passes
    int radix[8];
    int ns[8];      // Ns before each pass (product of the earlier radices)
    int twbase[8];  // offset of pass q's twiddles exp(-2 pi i r k / (Ns R)), k < Ns, 1 <= r < R
    int twlen;      // total twiddle entries (M - radix[0])
    int group;      // spectrum columns per column-pass work item
    int w;          // M / 2 + 1
    int groups;     // ceil(w / group)
    bool fusable;   // radix[0] == radix[np-1] and the fused pass fits 512 threads
    bool ok;
};

__host__ __device__ constexpr CtPlan ct_plan(int m) {
    CtPlan p{};
    p.ok = false;
    if (m < 24) return p;
    int main_r = 16, rem = m, others[4] = {0, 0, 0, 0}, no = 0, nmain = 0;
    if (m % 3 == 0) {
        rem = m / 3;
        if ((rem & (rem - 1)) != 0 || rem < 8 || m > 6144) return p;
        p.e = 24;
        main_r = 8;
        others[no++] = 3;
        while (rem % 8 == 0) {
            ++nmain;
            rem /= 8;
        }
    } else {
        if ((m & (m - 1)) != 0 || m < 32 || m > 8192) return p;
        p.e = 16;
        while (rem % 16 == 0) {
            ++nmain;
            rem /= 16;
        }
    }
    if (rem > 1) others[no++] = rem;
    int np = 0;
    if (nmain >= 2) {
        p.radix[np++] = main_r;
        for (int i = 0; i < no; ++i) p.radix[np++] = others[i];
        for (int i = 1; i < nmain; ++i) p.radix[np++] = main_r;
    } else {
        for (int i = 0; i < no; ++i) p.radix[np++] = others[i];
        for (int i = 0; i < nmain; ++i) p.radix[np++] = main_r;
    }
    p.np = np;
    int ns = 1, base = 0;
    for (int q = 0; q < np; ++q) {
        p.ns[q] = ns;
        p.twbase[q] = base;
        if (q > 0) base += ns * (p.radix[q] - 1);
        ns *= p.radix[q];
    }
    p.twlen = base;
    p.group = (m >= 4096) ? 2 : 4;
    p.w = m / 2 + 1;
    p.groups = (p.w + p.group - 1) / p.group;
    p.fusable = np >= 2 && p.radix[0] == p.radix[np - 1] && p.group * (m / p.e) <= 512 &&
                (m / p.radix[0]) % 16 == 0 && 16 % p.radix[0] == 0;
    p.ok = true;
    return p;
}

// Whether the plan of length m runs the global-fed / global-stored ("direct")
// kernels: a first pass with Ns = 1 and a radix dividing 16, and a last pass
// with Ns = M / R on 16-element blocks (every plan with at least two passes).
__host__ __device__ constexpr bool direct_ok(const CtPlan &p, int m) {
    return p.ok && p.np >= 2 && p.ns[0] == 1 && 16 % p.radix[0] == 0 && (m / p.radix[p.np - 1]) % 16 == 0;
}

// Per-length entry points (defined in fft_kernels.cuh, instantiated in fft_inst_*.cu).
// rows (may be null): the rows of x that may be non-zero (rows[r] != 0); the
// four-step kernels skip the transforms of row pairs that are both zero.
template <int M>
int conv_run(const float *x, int n, const float2 *spec, float *out, int linear, float2 *t1, float2 *t2,
             cudaStream_t st, const unsigned char *rows);
template <int M>
int spectrum_run(const float *psf, int rows, int cols, int off_r, int off_c, float2 *out, float2 *t1, cudaStream_t st);
template <int M>
int rfft2_run(const float *in, float2 *out, float2 *t1, cudaStream_t st);
template <int M>
int irfft2_run(const float2 *in, float *out, float2 *t2, cudaStream_t st);

namespace sq {
// Linear convolution of a 2048^2 image with a 4096^2 PSF spectrum (packed,
// group-major with 2 columns per group) by the four-step kernels of
// fft_sq.cuh; lo / hi: two workspaces of kPlaneElems float2 each.
constexpr int kLength = 4096;
int conv_run(const float *x, const float2 *spec, float *out, float2 *lo, float2 *hi, cudaStream_t st,
             const unsigned char *rows);
}  // namespace sq

#define MSN_FFT_SIZES(X) \
    X(24) X(48) X(96) X(192) X(384) X(768) X(1536) X(3072) X(6144) \
    X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096) X(8192)

#define MSN_FFT_EXTERN(M)                                                                                      \
    extern template int conv_run<M>(const float *, int, const float2 *, float *, int, float2 *, float2 *,     \
                                    cudaStream_t, const unsigned char *);                                      \
    extern template int spectrum_run<M>(const float *, int, int, int, int, float2 *, float2 *, cudaStream_t); \
    extern template int rfft2_run<M>(const float *, float2 *, float2 *, cudaStream_t);                       \
    extern template int irfft2_run<M>(const float2 *, float *, float2 *, cudaStream_t);
MSN_FFT_SIZES(MSN_FFT_EXTERN)
#undef MSN_FFT_EXTERN

}  // namespace fftk
}  // namespace msn
