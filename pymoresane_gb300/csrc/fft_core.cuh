// Shared-memory Stockham FFT core (mixed radix 2, 3, 4, 8, 16) for sm_103a.
//
// A "team" of M/E threads transforms one complex sequence of length M held in
// shared memory; every thread keeps E elements (16 for M = 2^a, 24 for
// M = 3 * 2^a) in registers per pass, i.e. E/R independent radix-R butterflies.
// Each pass of radix R performs the Stockham autosort step (Govindaraju et
// al., "High performance discrete Fourier transforms on graphics processors",
// SC 2008): butterfly j reads x[j + r M/R], applies the twiddles
// w^(r (j mod Ns)) with w = exp(-+2 pi i / (Ns R)), transforms the R values in
// registers and writes them to (j div Ns) Ns R + (j mod Ns) + r Ns. Any order
// of the radices gives the natural-order transform (the passes themselves are
// in fft_kernels.cuh). Shared-memory indices are padded by one element every
// 16 (sidx) to keep strided passes free of bank conflicts.
//
// Twiddles: kTwiddle is exp(-2 pi i k / kTwN) rounded from float64 to float32
// at build time (msn_twiddles.inc, generated by build.py); kTwN = 2^13 * 3
// covers every supported length.
#pragma once

#include <cuda_runtime.h>

namespace msn {

constexpr int kTwN = 24576;

__device__ __forceinline__ int sidx(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded_len(int m) { return m + (m >> 4) + 4; }

// Asynchronous global -> shared copies (cp.async); with valid == false the
// destination is zero-filled and nothing is read.
__device__ __forceinline__ void cp_async8(void *smem_dst, const void *gmem_src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(gmem_src), "r"(valid ? 8 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem_dst, const void *gmem_src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(gmem_src), "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// Multiply by -i (forward) or +i (inverse).
template <bool INV>
__host__ __device__ __forceinline__ float2 rot90(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <bool INV>
__host__ __device__ __forceinline__ void dft2(float2 *v) {
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <bool INV>
__host__ __device__ __forceinline__ void dft3(float2 *v) {
    const float s = INV ? 0.86602540378443864676f : -0.86602540378443864676f;
    const float2 a = v[0], b = v[1], c = v[2];
    const float2 t1 = cadd(b, c);
    const float2 t2 = make_float2(a.x - 0.5f * t1.x, a.y - 0.5f * t1.y);
    const float2 d = csub(b, c);
    const float2 t3 = make_float2(-s * d.y, s * d.x);  // i * s * (b - c)
    v[0] = cadd(a, t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
}

// 4-point DFT of v[o], v[o+s], v[o+2s], v[o+3s] in place, natural order.
template <bool INV, int O, int S>
__host__ __device__ __forceinline__ void dft4s(float2 *v) {
    const float2 x0 = v[O], x1 = v[O + S], x2 = v[O + 2 * S], x3 = v[O + 3 * S];
    const float2 a0 = cadd(x0, x2), a1 = csub(x0, x2), a2 = cadd(x1, x3), a3 = rot90<INV>(csub(x1, x3));
    v[O] = cadd(a0, a2);
    v[O + S] = cadd(a1, a3);
    v[O + 2 * S] = csub(a0, a2);
    v[O + 3 * S] = csub(a1, a3);
}

template <bool INV>
__host__ __device__ __forceinline__ void dft4(float2 *v) {
    dft4s<INV, 0, 1>(v);
}

template <bool INV>
__host__ __device__ __forceinline__ void dft8(float2 *v) {
    // X[k] = E[k] + w8^k O[k], X[k+4] = E[k] - w8^k O[k].
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    dft4<INV>(e);
    dft4<INV>(o);
    const float h = 0.70710678118654752440f;
    const float2 o1 = INV ? make_float2(h * (o[1].x - o[1].y), h * (o[1].x + o[1].y))
                          : make_float2(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x));
    const float2 o2 = rot90<INV>(o[2]);
    const float2 o3 = INV ? make_float2(-h * (o[3].x + o[3].y), h * (o[3].x - o[3].y))
                          : make_float2(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
}

template <bool INV>
__host__ __device__ __forceinline__ void dft16(float2 *v) {
    // 4 x 4: n = 4 n1 + n2, k = k1 + 4 k2.
    dft4s<INV, 0, 4>(v);
    dft4s<INV, 1, 4>(v);
    dft4s<INV, 2, 4>(v);
    dft4s<INV, 3, 4>(v);
    // slot n2 + 4 k1 holds Y[n2][k1]; twiddle by w16^(n2 k1).
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f, h = 0.70710678118654752440f;
    const float sg = INV ? 1.0f : -1.0f;
    const float2 w1 = make_float2(c1, sg * s1), w2 = make_float2(h, sg * h), w3 = make_float2(s1, sg * c1);
    const float2 w6 = make_float2(-h, sg * h), w9 = make_float2(-c1, -sg * s1);
    v[5] = cmul(v[5], w1);
    v[6] = cmul(v[6], w2);
    v[7] = cmul(v[7], w3);
    v[9] = cmul(v[9], w2);
    v[10] = rot90<INV>(v[10]);
    v[11] = cmul(v[11], w6);
    v[13] = cmul(v[13], w3);
    v[14] = cmul(v[14], w6);
    v[15] = cmul(v[15], w9);
    dft4s<INV, 0, 1>(v);
    dft4s<INV, 4, 1>(v);
    dft4s<INV, 8, 1>(v);
    dft4s<INV, 12, 1>(v);
    // slot 4 k1 + k2 now holds X[k1 + 4 k2]; out_slot<16> maps output index to slot.
}

// Register slot holding output X[r] after dft<INV, R>: natural order except for
// radix 16, whose 4 x 4 decomposition leaves X[k1 + 4 k2] in slot 4 k1 + k2.
template <int R>
__host__ __device__ constexpr int out_slot(int r) {
    return R == 16 ? 4 * (r & 3) + (r >> 2) : r;
}

template <bool INV, int R>
__host__ __device__ __forceinline__ void dft(float2 *v) {
    if constexpr (R == 2) dft2<INV>(v);
    if constexpr (R == 3) dft3<INV>(v);
    if constexpr (R == 4) dft4<INV>(v);
    if constexpr (R == 8) dft8<INV>(v);
    if constexpr (R == 16) dft16<INV>(v);
}

#ifndef MSN_HOST_ONLY  // host-only test programs compile the arithmetic without the device table
static __device__ const float2 kTwiddle[kTwN] = {
#include "msn_twiddles.inc"
};
#endif

}  // namespace msn
