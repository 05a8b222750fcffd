// Shared-memory Stockham FFT core (mixed radix 2, 3, 4, 8, 16) for sm_103a.
//
// A "team" of M/E threads transforms one complex sequence of length M held in
// shared memory; every thread keeps E elements in registers per pass. Each
// pass of radix R performs the Stockham autosort step (Govindaraju et al.,
// "High performance discrete Fourier transforms on graphics processors",
// SC 2008): butterfly j reads x[j + r M/R], applies the twiddles
// w^(r (j mod Ns)) with w = exp(-+2 pi i / (Ns R)), transforms the R values
// in registers and writes them to (j div Ns) Ns R + (j mod Ns) + r Ns.
// Output is in natural order. Shared-memory indices are padded by one
// element every 16 (sidx) to keep the strided first pass conflict-free.
//
// Twiddles come from kTwiddle, a table of exp(-2 pi i k / kTwN) rounded from
// float64 to float32 at build time (msn_twiddles.inc, generated by build.py);
// kTwN = 2^13 * 3 covers every supported length M = 2^a or 3 * 2^a.
#pragma once

#include <cuda_runtime.h>

namespace msn {

constexpr int kTwN = 24576;

__device__ __forceinline__ int sidx(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded_len(int m) { return m + (m >> 4) + 4; }

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// Multiply by -i (forward) or +i (inverse).
template <bool INV>
__device__ __forceinline__ float2 rot90(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <bool INV>
__device__ __forceinline__ void dft2(float2 *v) {
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <bool INV>
__device__ __forceinline__ void dft3(float2 *v) {
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
__device__ __forceinline__ void dft4s(float2 *v) {
    const float2 x0 = v[O], x1 = v[O + S], x2 = v[O + 2 * S], x3 = v[O + 3 * S];
    const float2 a0 = cadd(x0, x2), a1 = csub(x0, x2), a2 = cadd(x1, x3), a3 = rot90<INV>(csub(x1, x3));
    v[O] = cadd(a0, a2);
    v[O + S] = cadd(a1, a3);
    v[O + 2 * S] = csub(a0, a2);
    v[O + 3 * S] = csub(a1, a3);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2 *v) {
    dft4s<INV, 0, 1>(v);
}

template <bool INV>
__device__ __forceinline__ void dft8(float2 *v) {
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
__device__ __forceinline__ void dft16(float2 *v) {
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
    // slot 4 k1 + k2 holds X[k1 + 4 k2]: transpose to natural order.
    float2 t[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) t[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = t[i];
}

template <bool INV, int R>
__device__ __forceinline__ void dft(float2 *v) {
    if constexpr (R == 2) dft2<INV>(v);
    if constexpr (R == 3) dft3<INV>(v);
    if constexpr (R == 4) dft4<INV>(v);
    if constexpr (R == 8) dft8<INV>(v);
    if constexpr (R == 16) dft16<INV>(v);
}

struct FftPlan {
    int m;          // transform length
    int npass;
    int radix[8];
};

static __device__ const float2 kTwiddle[kTwN] = {
#include "msn_twiddles.inc"
};

template <bool INV>
__device__ __forceinline__ float2 twiddle(int idx) {
    const float2 w = __ldg(&kTwiddle[idx]);
    return INV ? cconj(w) : w;
}

// One Stockham pass of radix R over a team's sequence (all CTA threads call it).
template <bool INV, int E, int R>
__device__ __forceinline__ void fft_pass(float2 *buf, int m, int ns, int t) {
    if constexpr (E % R == 0) {
        constexpr int NB = E / R;
        const int team = m / E;
        const int stride = m / R;
        float2 v[E];
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            const int j = t + b * team;
#pragma unroll
            for (int r = 0; r < R; ++r) v[b * R + r] = buf[sidx(j + r * stride)];
        }
        __syncthreads();
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            const int j = t + b * team;
            const int k = j % ns;
            if (ns > 1) {
                const int step = kTwN / (ns * R);
#pragma unroll
                for (int r = 1; r < R; ++r) v[b * R + r] = cmul(v[b * R + r], twiddle<INV>(r * k * step));
            }
            dft<INV, R>(v + b * R);
            const int base = (j - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) buf[sidx(base + r * ns)] = v[b * R + r];
        }
        __syncthreads();
    }
}

// Full transform of one team's sequence (unnormalised; INV uses exp(+2 pi i/M)).
template <bool INV, int E>
__device__ __forceinline__ void fft_team(float2 *buf, const FftPlan &p, int t) {
    int ns = 1;
    for (int q = 0; q < p.npass; ++q) {
        const int r = p.radix[q];
        if (r == 16) fft_pass<INV, E, 16>(buf, p.m, ns, t);
        else if (r == 8) fft_pass<INV, E, 8>(buf, p.m, ns, t);
        else if (r == 4) fft_pass<INV, E, 4>(buf, p.m, ns, t);
        else if (r == 3) fft_pass<INV, E, 3>(buf, p.m, ns, t);
        else fft_pass<INV, E, 2>(buf, p.m, ns, t);
        ns *= r;
    }
}

}  // namespace msn
