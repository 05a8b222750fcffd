// Conjugate-gradient minor loop and major-loop vector work
// (pymoresane/main.py:365-503) for sm_103a.
//
// Every inner product, the step sizes alpha / beta and the residual
// statistics are accumulated in float64 (four-element float32 partials, see
// dot4). Reductions are deterministic: a
// fixed grid writes one float64 partial per CTA and a single CTA sums the
// partials in a fixed order, so results are bit-identical run to run and do
// not depend on what else shares the GPU. The CG scalars live in a small
// device array (layout MSN_S_* in msn.h) so that the vector updates read
// alpha and beta on the device and the host only needs the stop decisions.
#include <atomic>

#include "minor_state.cuh"
#include "msn_common.cuh"

namespace msn {
namespace {

constexpr int kRedGrid = 4 * 152;
constexpr int kRedThreads = 256;

enum { S_RR = 0, S_PAP = 1, S_ALPHA = 2, S_RNRN = 3, S_BETA = 4 };

// A float-float number: the unevaluated sum hi + lo of two floats, |lo| <= ulp(hi)/2.
// Additions keep their rounding error with Knuth's TwoSum (every operation a
// separately rounded float32 add, no contraction), so a running sum carries about
// 48 significant bits while using only the float32 pipes. GB300's float64 rate is
// a small fraction of its float32 rate, and float64 per-thread accumulation made
// each reduction over a 2048^2 vector about 9 us slower than float32.
struct FF {
    float hi, lo;
    FF() = default;  // trivial, so FF can live in __shared__ arrays; FF() value-initialises to zero
    __device__ __forceinline__ explicit FF(float v) : hi(v), lo(0.0f) {}
    __device__ __forceinline__ explicit FF(int v) : hi((float)v), lo(0.0f) {}
    __device__ __forceinline__ explicit FF(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
    __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
    __device__ __forceinline__ FF &operator+=(const FF &b) {
        // TwoSum of the high parts, then the low parts, then a fast renormalisation
        const float s = __fadd_rn(hi, b.hi);
        const float bb = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
        const float t = __fadd_rn(e, __fadd_rn(lo, b.lo));
        hi = __fadd_rn(s, t);
        lo = __fsub_rn(t, __fsub_rn(hi, s));
        return *this;
    }
};

__device__ __forceinline__ float shfl_xor(float v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ double shfl_xor(double v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ FF shfl_xor(FF v, int off) {
    FF r;
    r.hi = __shfl_xor_sync(0xffffffffu, v.hi, off);
    r.lo = __shfl_xor_sync(0xffffffffu, v.lo, off);
    return r;
}

// Accumulation type of the reductions within a CTA: double (the default,
// msn_set_reduction_precision(64)), FF (float-float, 48) or float (the plain
// float32 variant, 32); the sum across CTAs is float64 except in the float32 variant.
template <class T>
__device__ __forceinline__ T block_sum(T v) {
    __shared__ T sh[32];
    for (int off = 16; off > 0; off >>= 1) v += shfl_xor(v, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    v = threadIdx.x < nw ? sh[threadIdx.x] : T(0);
    if (threadIdx.x < 32)
        for (int off = 16; off > 0; off >>= 1) v += shfl_xor(v, off);
    __syncthreads();
    return v;  // valid in thread 0
}

// Type of the sum across CTAs: float for the plain float32 variant, double otherwise.
template <class T> struct CrossSum { using type = double; };
template <> struct CrossSum<float> { using type = float; };

// Two-stage deterministic reduction in one launch: every CTA writes its
// partial pair, and the last CTA to finish (completion counter after the
// partials, reset to zero by that CTA) sums the kRedGrid pairs in a fixed
// order -- thread t adds pairs t, t + 256, t + 512, then warp-shuffle trees --
// so the totals do not depend on which CTA finishes last.
// cta_has_work == 0 (uniform across the CTA): every thread's sums are the +0 they
// started from, so the block sums (+0) are written without being formed.
// second == 0 (uniform): the second sum is identically +0 (a single dot product or
// the residual norm), so its block and cross-CTA sums are skipped and +0 written.
template <class T>
__device__ __forceinline__ bool finish_pairs(T s0, T s1, double *__restrict__ partials, double *out,
                                             double *beta_scal, int cta_has_work = 1, int second = 1) {
    using X = typename CrossSum<T>::type;
    __shared__ bool last;
    __shared__ X ws[2][kRedThreads / 32];
    if (cta_has_work) {
        s0 = block_sum(s0);
        s1 = second ? block_sum(s1) : T(0);
    } else {
        s0 = T(0);
        s1 = T(0);
    }
    unsigned *counter = reinterpret_cast<unsigned *>(partials + 2 * kRedGrid);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = (double)s0;
        partials[2 * blockIdx.x + 1] = (double)s1;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    const int t = threadIdx.x;
    X a = X(0), b = X(0);
    for (int k = t; k < (int)gridDim.x; k += kRedThreads) {
        a += (X)__ldcg(partials + 2 * k);
        if (second) b += (X)__ldcg(partials + 2 * k + 1);
    }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        if (second) b += __shfl_xor_sync(0xffffffffu, b, off);
    }
    if ((t & 31) == 0) {
        ws[0][t >> 5] = a;
        ws[1][t >> 5] = b;
    }
    __syncthreads();
    if (t < 32) {
        a = t < kRedThreads / 32 ? ws[0][t] : X(0);
        b = t < kRedThreads / 32 ? ws[1][t] : X(0);
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, off);
            if (second) b += __shfl_xor_sync(0xffffffffu, b, off);
        }
        if (t == 0) {
            out[0] = (double)a;
            if (beta_scal) {
                beta_scal[4] = (double)a / beta_scal[0];  // beta = rn.rn / r.r (main.py:407-409)
            } else {
                out[1] = (double)b;
            }
            *counter = 0u;
        }
    }
    return true;
}

// Float64 accumulation at a low float64 instruction count (the FP64 rate of
// GB300 is a small fraction of its FP32 rate): every thread forms the products
// of four consecutive elements with a float32 fused multiply-add chain, then
// adds that four-element partial to its float64 accumulator (one conversion
// and one float64 add per four elements). The relative error of each
// four-element partial is a few float32 ulps; all longer sums are float64.
__device__ __forceinline__ float dot4(const float4 &a, const float4 &b) {
    return __fmaf_rn(a.w, b.w, __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x))));
}
__device__ __forceinline__ float sqdiff4(const float4 &a, const float4 &b) {
    const float x = __fsub_rn(a.x, b.x), y = __fsub_rn(a.y, b.y), z = __fsub_rn(a.z, b.z), w = __fsub_rn(a.w, b.w);
    return __fmaf_rn(w, w, __fmaf_rn(z, z, __fmaf_rn(y, y, __fmul_rn(x, x))));
}

// partials[2*b + 0] = sum a*b, partials[2*b + 1] = sum c*d (or sum (a - c)^2 when DIFF).
// n4 float4 groups (callers guarantee n % 4 == 0 and 16-byte alignment).
// With a row support, elements outside it are skipped (their terms are zero).
template <bool DIFF, class T>
__global__ void __launch_bounds__(kRedThreads)
dual_partials(const float4 *__restrict__ a, const float4 *__restrict__ b, const float4 *__restrict__ c,
              const float4 *__restrict__ d, size_t n4, double *__restrict__ partials, double *__restrict__ out,
              RowSupport sup) {
    pdl_wait();
    pdl_trigger();
    T s0 = T(0), s1 = T(0);
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    // Four grid-stride steps per round with all their loads issued first (memory-level
    // parallelism); the terms are added in the same order as one step at a time.
    for (; i + 3 * stride < n4; i += 4 * stride) {
        bool on[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) on[u] = sup.active(i + u * stride);
        float4 va[4], vb[4], vc[4], vd[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (!on[u]) continue;
            va[u] = __ldg(a + i + u * stride);
            vb[u] = __ldg(b + i + u * stride);
            if (DIFF || c) vc[u] = __ldg(c + i + u * stride);
            if (!DIFF && c) vd[u] = __ldg(d + i + u * stride);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (!on[u]) continue;
            s0 += (T)dot4(va[u], vb[u]);
            if (DIFF) {
                s1 += (T)sqdiff4(va[u], vc[u]);
            } else if (c) {
                s1 += (T)dot4(vc[u], vd[u]);
            }
        }
    }
    for (; i < n4; i += stride) {
        if (!sup.active(i)) continue;
        const float4 va = __ldg(a + i);
        s0 += (T)dot4(va, __ldg(b + i));
        if (DIFF) {
            s1 += (T)sqdiff4(va, __ldg(c + i));
        } else if (c) {
            s1 += (T)dot4(__ldg(c + i), __ldg(d + i));
        }
    }
    finish_pairs<T>(s0, s1, partials, out, nullptr, 1, DIFF || c != nullptr);
}

// Float64 inputs: partials of sum a^2 and sum (a - b)^2 with every product and
// difference in float64 (np.linalg.norm of float64 arrays, iuwt_toolbox.py:304).
__global__ void __launch_bounds__(kRedThreads)
snr_partials_f64(const double *__restrict__ a, const double *__restrict__ b, size_t n,
                 double *__restrict__ partials, double *__restrict__ out) {
    double s0 = 0.0, s1 = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double va = __ldg(a + i);
        const double d = __dsub_rn(va, __ldg(b + i));
        s0 = __fma_rn(va, va, s0);
        s1 = __fma_rn(d, d, s1);
    }
    finish_pairs<double>(s0, s1, partials, out, nullptr);
}

// Sums the kRedGrid partial pairs in a fixed order into out[0], out[1]: one
// warp-shuffle tree per warp, then one over the warp sums.
constexpr int kFinalizeThreads = ((kRedGrid + 31) / 32) * 32;

template <class T0>
__global__ void __launch_bounds__(kFinalizeThreads)
finalize_pairs(const double *__restrict__ partials, double *__restrict__ out) {
    using T = typename CrossSum<T0>::type;
    __shared__ T ws[2][kFinalizeThreads / 32];
    const int t = threadIdx.x;
    T a = t < kRedGrid ? (T)partials[2 * t] : T(0);
    T b = t < kRedGrid ? (T)partials[2 * t + 1] : T(0);
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
    }
    if ((t & 31) == 0) {
        ws[0][t >> 5] = a;
        ws[1][t >> 5] = b;
    }
    __syncthreads();
    if (t < 32) {
        a = t < kFinalizeThreads / 32 ? ws[0][t] : T(0);
        b = t < kFinalizeThreads / 32 ? ws[1][t] : T(0);
        for (int off = 16; off > 0; off >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, off);
            b += __shfl_xor_sync(0xffffffffu, b, off);
        }
        if (t == 0) {
            out[0] = (double)a;
            out[1] = (double)b;
        }
    }
}

// model_sources += alpha * Q with the partials of sum E^2 and sum (E - model_sources)^2.
// By linearity mask * W(H (x + alpha p)) = mask * W(H x) + alpha * mask * W(H p), and
// mask * W(H p) is the plane stack Q already formed for Ap, so the model sources of
// pymoresane/main.py:413-416 and the norms of snr_ratio (iuwt_toolbox.py:304) come
// from one pass instead of a convolution plus a decomposition.
// With seg_flags, 32-float4 segments whose flag is 0 are skipped: there e, q
// and ms are all zero (the extraction mask is zero), so each skipped term would
// add exactly +0 to the same per-thread partial, and the sums are bit-identical
// to the dense pass. A warp's 32 consecutive indices form one segment, so the
// test is warp-uniform.
template <class T>
__global__ void __launch_bounds__(kRedThreads)
snr_update(const float4 *__restrict__ e, float4 *__restrict__ ms, const float4 *__restrict__ q,
           const double *__restrict__ scal, size_t n4, double *__restrict__ partials,
           const unsigned char *__restrict__ seg_flags, double *__restrict__ out) {
    const float a = (float)scal[S_ALPHA];
    T s0 = T(0), s1 = T(0);
    int worked = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    // The segment flags of eight grid-stride steps are loaded together: one flag load
    // per step would make every step wait for the previous one (the pass is almost all
    // skipped segments). Elements are still visited, and summed, in the same order.
    constexpr int kAhead = 8;
    for (size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n4; i0 += kAhead * stride) {
        unsigned char f[kAhead];
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
            const size_t i = i0 + u * stride;
            f[u] = i < n4 ? (seg_flags ? __ldg(seg_flags + (i >> 5)) : (unsigned char)1) : (unsigned char)0;
        }
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
            if (!f[u]) continue;
            const size_t i = i0 + u * stride;
            worked = 1;
            const float4 ev = __ldg(e + i), qv = __ldg(q + i);
            float4 mv = ms[i];
            mv.x = __fadd_rn(mv.x, __fmul_rn(a, qv.x));
            mv.y = __fadd_rn(mv.y, __fmul_rn(a, qv.y));
            mv.z = __fadd_rn(mv.z, __fmul_rn(a, qv.z));
            mv.w = __fadd_rn(mv.w, __fmul_rn(a, qv.w));
            ms[i] = mv;
            s0 += (T)dot4(ev, ev);
            s1 += (T)sqdiff4(ev, mv);
        }
    }
    // most CTAs of the masked pass see no non-empty segment: skip their block sums
    finish_pairs<T>(s0, s1, partials, out, nullptr, __syncthreads_or(worked));
}

// The vector updates evaluate the reference's float32 expressions
// (pymoresane/main.py:390,397,405,411 on float32 arrays in GPU mode) with
// alpha and beta computed in float64 from the float64 inner products and then
// rounded to float32: xn = x + a*p, p = (xn - x)/a, rn = r - a*Ap,
// p = rn + b*p, each product and sum rounded separately (no contraction).

// xn = x + alpha p with alpha = rr / pAp (main.py:386-390); counts xn < 0.
__global__ void cg_alpha_x(const float4 *__restrict__ x, const float4 *__restrict__ p, double *__restrict__ scal,
                           float4 *__restrict__ xn, size_t n4, int *__restrict__ neg) {
    const double alpha = scal[S_RR] / scal[S_PAP];
    if (blockIdx.x == 0 && threadIdx.x == 0) scal[S_ALPHA] = alpha;
    const float a = (float)alpha;
    int local = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        const float4 xv = __ldg(x + i), pv = __ldg(p + i);
        float4 v;
        v.x = __fadd_rn(xv.x, __fmul_rn(a, pv.x));
        v.y = __fadd_rn(xv.y, __fmul_rn(a, pv.y));
        v.z = __fadd_rn(xv.z, __fmul_rn(a, pv.z));
        v.w = __fadd_rn(xv.w, __fmul_rn(a, pv.w));
        xn[i] = v;
        local += (v.x < 0.0f) + (v.y < 0.0f) + (v.z < 0.0f) + (v.w < 0.0f);
    }
    local = __reduce_add_sync(0xffffffffu, local);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(neg, local);
}

// Positivity (main.py:394-397): xn[xn < 0] = 0; p = (xn - x) / alpha.
__global__ void cg_positivity(const float *__restrict__ x, float *__restrict__ xn, float *__restrict__ p,
                              const double *__restrict__ scal, size_t n) {
    const float a = (float)scal[S_ALPHA];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float v = xn[i];
        if (v < 0.0f) v = 0.0f;
        xn[i] = v;
        p[i] = __fdiv_rn(__fsub_rn(v, x[i]), a);
    }
}

// rn = r - alpha Ap with the per-CTA float64 partial of rn . rn (main.py:405-408).
template <class T>
__global__ void __launch_bounds__(kRedThreads)
cg_residual(const float4 *__restrict__ r, const float4 *__restrict__ ap, double *__restrict__ scal,
            float4 *__restrict__ rn, size_t n4, double *__restrict__ partials) {
    const float a = (float)scal[S_ALPHA];
    T s = T(0);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        const float4 rv = __ldg(r + i), av = __ldg(ap + i);
        float4 v;
        v.x = __fsub_rn(rv.x, __fmul_rn(a, av.x));
        v.y = __fsub_rn(rv.y, __fmul_rn(a, av.y));
        v.z = __fsub_rn(rv.z, __fmul_rn(a, av.z));
        v.w = __fsub_rn(rv.w, __fmul_rn(a, av.w));
        rn[i] = v;
        s += (T)dot4(v, v);
    }
    // scal[S_RNRN] = rn.rn, scal[S_BETA] = rn.rn / r.r
    finish_pairs<T>(s, T(0), partials, scal + S_RNRN, scal, 1, 0);
}

// One pass of the step without positivity: xn = x + alpha p and rn = r - alpha Ap
// with the float64 partials of rn . rn (then rn.rn and beta), the arithmetic of
// cg_alpha_x followed by cg_residual. The reduction uses cg_residual's grid and
// order, so rn.rn and beta are bit-identical to the two-kernel sequence.
template <class T>
__global__ void __launch_bounds__(kRedThreads)
cg_step(const float4 *__restrict__ x, const float4 *__restrict__ p, const float4 *__restrict__ r,
        const float4 *__restrict__ ap, double *__restrict__ scal, float4 *__restrict__ xn, float4 *__restrict__ rn,
        size_t n4, double *__restrict__ partials, RowSupport sup) {
    const double alpha = scal[S_RR] / scal[S_PAP];
    if (blockIdx.x == 0 && threadIdx.x == 0) scal[S_ALPHA] = alpha;
    const float a = (float)alpha;
    T s = T(0);
    // with a row support, xn and rn outside it are left as they are (the caller keeps them zero)
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        if (!sup.active(i)) continue;
        const float4 xv = __ldg(x + i), pv = __ldg(p + i), rv = __ldg(r + i), av = __ldg(ap + i);
        float4 v, u;
        v.x = __fadd_rn(xv.x, __fmul_rn(a, pv.x));
        v.y = __fadd_rn(xv.y, __fmul_rn(a, pv.y));
        v.z = __fadd_rn(xv.z, __fmul_rn(a, pv.z));
        v.w = __fadd_rn(xv.w, __fmul_rn(a, pv.w));
        xn[i] = v;
        u.x = __fsub_rn(rv.x, __fmul_rn(a, av.x));
        u.y = __fsub_rn(rv.y, __fmul_rn(a, av.y));
        u.z = __fsub_rn(rv.z, __fmul_rn(a, av.z));
        u.w = __fsub_rn(rv.w, __fmul_rn(a, av.w));
        rn[i] = u;
        s += (T)dot4(u, u);
    }
    finish_pairs<T>(s, T(0), partials, scal + S_RNRN, scal, 1, 0);
}

// The graph minor loop's pass after p.Ap without positivity, in one launch: cg_step
// on the row support (xn, rn, rn.rn, beta), then snr_update's model-source update
// and SNR sums (same alpha: the same float64 quotient rounded to float32), then, in
// the CTA that completes the SNR sums, the stop rules (minor_control_apply). Each
// sum keeps its kernel's grid, per-thread order and cross-CTA order, in its own
// set of partials, so every result is bit-identical to the three launches.
template <class T>
__global__ void __launch_bounds__(kRedThreads)
cg_step_snr(const float4 *__restrict__ x, const float4 *__restrict__ p, const float4 *__restrict__ r,
            const float4 *__restrict__ ap, double *__restrict__ scal, float4 *__restrict__ xn,
            float4 *__restrict__ rn, size_t n4, RowSupport sup, const float4 *__restrict__ e,
            float4 *__restrict__ ms, const float4 *__restrict__ q, size_t nq4,
            const unsigned char *__restrict__ seg_flags, double *__restrict__ partials_rn,
            double *__restrict__ partials_snr, double *__restrict__ snr2, MinorState *state, double *hist,
            int hist_len, cudaGraphConditionalHandle h) {
    pdl_wait();
    pdl_trigger();
    const double alpha = scal[S_RR] / scal[S_PAP];
    if (blockIdx.x == 0 && threadIdx.x == 0) scal[S_ALPHA] = alpha;
    const float a = (float)alpha;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    // the CG step (cg_step)
    T s = T(0);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
        if (!sup.active(i)) continue;
        const float4 xv = __ldg(x + i), pv = __ldg(p + i), rv = __ldg(r + i), av = __ldg(ap + i);
        float4 v, u;
        v.x = __fadd_rn(xv.x, __fmul_rn(a, pv.x));
        v.y = __fadd_rn(xv.y, __fmul_rn(a, pv.y));
        v.z = __fadd_rn(xv.z, __fmul_rn(a, pv.z));
        v.w = __fadd_rn(xv.w, __fmul_rn(a, pv.w));
        xn[i] = v;
        u.x = __fsub_rn(rv.x, __fmul_rn(a, av.x));
        u.y = __fsub_rn(rv.y, __fmul_rn(a, av.y));
        u.z = __fsub_rn(rv.z, __fmul_rn(a, av.z));
        u.w = __fsub_rn(rv.w, __fmul_rn(a, av.w));
        rn[i] = u;
        s += (T)dot4(u, u);
    }
    // the model sources and SNR sums (snr_update)
    T s0 = T(0), s1 = T(0);
    int worked = 0;
    constexpr int kAhead = 8;
    for (size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < nq4; i0 += kAhead * stride) {
        unsigned char f[kAhead];
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
            const size_t i = i0 + u * stride;
            f[u] = i < nq4 ? __ldg(seg_flags + (i >> 5)) : (unsigned char)0;
        }
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
            if (!f[u]) continue;
            const size_t i = i0 + u * stride;
            worked = 1;
            const float4 ev = __ldg(e + i), qv = __ldg(q + i);
            float4 mv = ms[i];
            mv.x = __fadd_rn(mv.x, __fmul_rn(a, qv.x));
            mv.y = __fadd_rn(mv.y, __fmul_rn(a, qv.y));
            mv.z = __fadd_rn(mv.z, __fmul_rn(a, qv.z));
            mv.w = __fadd_rn(mv.w, __fmul_rn(a, qv.w));
            ms[i] = mv;
            s0 += (T)dot4(ev, ev);
            s1 += (T)sqdiff4(ev, mv);
        }
    }
    // scal[S_RNRN] = rn.rn, scal[S_BETA] = rn.rn / r.r
    finish_pairs<T>(s, T(0), partials_rn, scal + S_RNRN, scal, 1, 0);
    __syncthreads();  // finish_pairs' shared state is reused below
    const int any = __syncthreads_or(worked);
    if (finish_pairs<T>(s0, s1, partials_snr, snr2, nullptr, any) && threadIdx.x == 0) {
        __threadfence();
        minor_control_apply(state, snr2, hist, hist_len, h);
    }
}

// flags[s] = 1 when any element of float4 segment s (32 float4) of m is non-zero.
__global__ void segment_flags(const float4 *__restrict__ m, size_t n4, unsigned char *__restrict__ flags) {
    const size_t nseg = (n4 + 31) / 32;
    const int lane = threadIdx.x & 31;
    const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t seg = warp; seg < nseg; seg += nwarps) {
        const size_t i = seg * 32 + lane;
        bool nz = false;
        if (i < n4) {
            const float4 v = __ldg(m + i);
            nz = v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f;
        }
        const unsigned any = __any_sync(0xffffffffu, nz);
        if (lane == 0) flags[seg] = any ? 1 : 0;
    }
}

// flags[r] = 1 when row r (cols floats, cols % 4 == 0) of m has a non-zero element.
__global__ void row_flags(const float4 *__restrict__ m, size_t rows, int cols4, unsigned char *__restrict__ flags) {
    const int lane = threadIdx.x & 31;
    const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t r = warp; r < rows; r += nwarps) {
        bool nz = false;
        for (int c = lane; c < cols4; c += 32) {
            const float4 v = __ldg(m + r * cols4 + c);
            nz = nz || v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f;
        }
        const unsigned any = __any_sync(0xffffffffu, nz);
        if (lane == 0) flags[r] = any ? 1 : 0;
    }
}

// p = rn + beta p (main.py:411).
__global__ void cg_direction(const float4 *__restrict__ rn, float4 *__restrict__ p, const double *__restrict__ scal,
                             size_t n4) {
    const float b = (float)scal[S_BETA];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        const float4 rv = __ldg(rn + i);
        float4 pv = p[i];
        pv.x = __fadd_rn(rv.x, __fmul_rn(b, pv.x));
        pv.y = __fadd_rn(rv.y, __fmul_rn(b, pv.y));
        pv.z = __fadd_rn(rv.z, __fmul_rn(b, pv.z));
        pv.w = __fadd_rn(rv.w, __fmul_rn(b, pv.w));
        p[i] = pv;
    }
}

// model[sub] += sign * gain * x, in float32 as the reference does (main.py:483, 498).
__global__ void model_update(float *__restrict__ model, int pitch, const float *__restrict__ x, int n_sub, int off_r,
                             int off_c, float gain, float sign) {
    const size_t total = (size_t)n_sub * n_sub;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / n_sub), c = (int)(i - (size_t)r * n_sub);
        float *m = model + (size_t)(r + off_r) * pitch + (c + off_c);
        const float step = __fmul_rn(gain, x[i]);
        *m = sign > 0.0f ? __fadd_rn(*m, step) : __fsub_rn(*m, step);
    }
}

__global__ void sub_kernel(const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __fsub_rn(a[i], b[i]);
}

__global__ void add_kernel(const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __fadd_rn(a[i], b[i]);
}

__global__ void mul_kernel(const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __fmul_rn(a[i], b[i]);
}

// Region sums for the standard deviation: pass 0 sums x, pass 1 sums (x - mean)^2.
template <class T>
__global__ void __launch_bounds__(kRedThreads)
region_partials(const float *__restrict__ img, int pitch, int rows, int cols, int off_r, int off_c,
                const double *__restrict__ mean_in, double *__restrict__ partials) {
    const double mean = mean_in ? mean_in[0] / ((double)rows * cols) : 0.0;
    const float mean_f = (float)mean;
    const size_t total = (size_t)rows * cols;
    T s = T(0);
    // float32 partials over runs of up to four elements per thread, float64 across runs
    float part = 0.0f;
    int run = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(i / cols), c = (int)(i - (size_t)r * cols);
        const float v = img[(size_t)(r + off_r) * pitch + c + off_c];
        if (mean_in) {
            const float dv = __fsub_rn(v, mean_f);
            part = __fmaf_rn(dv, dv, part);
        } else {
            part = __fadd_rn(part, v);
        }
        if (++run == 4) {
            s += (T)part;
            part = 0.0f;
            run = 0;
        }
    }
    s += (T)part;
    s = block_sum<T>(s);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = (double)s;
        partials[2 * blockIdx.x + 1] = 0.0;
    }
}

__global__ void std_finish(double *__restrict__ out2, long long count) {
    // out2[0] = sum x, out2[1] = sum (x - mean)^2 -> out2[2] = mean, out2[3] = std
    out2[2] = out2[0] / (double)count;
    out2[3] = sqrt(out2[1] / (double)count);
}

}  // namespace

// Accumulation type of the reductions, process-wide: 64 (float64, the default)
// or 32 (plain float32 accumulation, for the error comparison).
std::atomic<int> g_reduce_bits{64};
bool reduce_fp32() { return g_reduce_bits.load(std::memory_order_relaxed) == 32; }

namespace {

// Launches kernel template K<..., T> with T = FF, double or float as selected.
#define MSN_RED_LAUNCH(KERNEL, GRID, BLOCK, ST, ...)                       \
    do {                                                                   \
        const int bits_ = g_reduce_bits.load(std::memory_order_relaxed);   \
        if (bits_ == 32)                                                   \
            KERNEL<float><<<GRID, BLOCK, 0, ST>>>(__VA_ARGS__);            \
        else if (bits_ == 64)                                              \
            KERNEL<double><<<GRID, BLOCK, 0, ST>>>(__VA_ARGS__);           \
        else                                                               \
            KERNEL<FF><<<GRID, BLOCK, 0, ST>>>(__VA_ARGS__);               \
    } while (0)

int ew_grid(size_t n) {
    size_t g = (n + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    return g < 1 ? 1 : (int)g;
}

// kRedGrid partial pairs and the completion counter of finish_pairs (zero
// between calls: the workspace is zeroed once when it is allocated).
// One set of partials: kRedGrid pairs and the completion counter. The workspace holds two
// sets (the fused CG / SNR pass runs two reductions at once).
constexpr size_t kPartialSetBytes = 2 * kRedGrid * sizeof(double) + 16;
constexpr size_t kPartialBytes = 2 * kPartialSetBytes;

}  // namespace

int dual_reduce(const float *a, const float *b, const float *c, const float *d, size_t n, bool diff, double *out,
                double *partials, cudaStream_t st, RowSupport sup = {nullptr, 1u}) {
    if (n % 4 || !aligned16(a) || !aligned16(b) || !aligned16(c) || !aligned16(d))
        return set_error(MSN_ERR_INVALID, "reduction: length must be a multiple of 4 and pointers 16-byte aligned");
    const float4 *a4 = (const float4 *)a, *b4 = (const float4 *)b, *c4 = (const float4 *)c, *d4 = (const float4 *)d;
    const int bits = g_reduce_bits.load(std::memory_order_relaxed);
    auto go = [&](auto kernel) {
        return launch_k("dual_partials", kernel, kRedGrid, kRedThreads, 0, st, a4, b4, c4, d4, n / 4, partials, out, sup);
    };
    if (diff && bits == 32) return go(dual_partials<true, float>);
    if (diff && bits == 64) return go(dual_partials<true, double>);
    if (diff) return go(dual_partials<true, FF>);
    if (bits == 32) return go(dual_partials<false, float>);
    if (bits == 64) return go(dual_partials<false, double>);
    return go(dual_partials<false, FF>);

}

int dot_rows(const float *a, const float *b, size_t n, RowSupport sup, double *out, void *work, size_t work_bytes,
             cudaStream_t st) {
    if (!a || !b || !out || !work || work_bytes < kPartialBytes || sup.cols4 == 0)
        return set_error(MSN_ERR_INVALID, "dot_rows: bad arguments");
    return dual_reduce(a, b, nullptr, nullptr, n, false, out, (double *)work, st, sup);
}

int cg_step_snr_rows(const float *x, const float *p, const float *r, const float *ap, double *scal, float *xn,
                     float *rn, size_t n, RowSupport sup, const float *e, float *ms, const float *q, size_t nq,
                     const unsigned char *seg_flags, double *snr2, MinorState *state, double *hist, int hist_len,
                     cudaGraphConditionalHandle h, void *work, size_t work_bytes, cudaStream_t st) {
    if (!x || !p || !r || !ap || !scal || !xn || !rn || !e || !ms || !q || !seg_flags || !snr2 || !state || !hist ||
        !work || work_bytes < kPartialBytes || sup.cols4 == 0)
        return set_error(MSN_ERR_INVALID, "cg_step_snr_rows: bad arguments");
    if (n % 4 || nq % 4 || !aligned16(x) || !aligned16(p) || !aligned16(r) || !aligned16(ap) || !aligned16(xn) ||
        !aligned16(rn) || !aligned16(e) || !aligned16(ms) || !aligned16(q))
        return set_error(MSN_ERR_INVALID, "cg_step_snr_rows: lengths must be multiples of 4, pointers 16-byte aligned");
    double *set0 = (double *)work;
    double *set1 = (double *)((char *)work + kPartialSetBytes);
    auto go = [&](auto kernel) {
        return launch_k("cg_step_snr", kernel, kRedGrid, kRedThreads, 0, st, (const float4 *)x, (const float4 *)p,
                        (const float4 *)r, (const float4 *)ap, scal, (float4 *)xn, (float4 *)rn, n / 4, sup,
                        (const float4 *)e, (float4 *)ms, (const float4 *)q, nq / 4, seg_flags, set0, set1, snr2, state,
                        hist, hist_len, h);
    };
    const int bits = g_reduce_bits.load(std::memory_order_relaxed);
    if (bits == 32) return go(cg_step_snr<float>);
    if (bits == 64) return go(cg_step_snr<double>);
    return go(cg_step_snr<FF>);
}

}  // namespace msn

using namespace msn;

extern "C" size_t msn_reduce_workspace_bytes(void) { return kPartialBytes; }

static int check_red_ws(void *w, size_t b, const char *fn) {
    if (!w || b < kPartialBytes) return set_error(MSN_ERR_WORKSPACE, "%s: workspace of %zu bytes needed", fn, kPartialBytes);
    return MSN_OK;
}

extern "C" int msn_dot2(const float *d_a, const float *d_b, const float *d_c, const float *d_d, size_t n,
                        double *d_out2, void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    if (!d_a || !d_b || !d_out2 || ((d_c == nullptr) != (d_d == nullptr)))
        return set_error(MSN_ERR_INVALID, "msn_dot2: null pointer");
    MSN_TRY(check_red_ws(d_work, work_bytes, "msn_dot2"));
    return dual_reduce(d_a, d_b, d_c, d_d, n, false, d_out2, (double *)d_work, as_stream(stream));
}

extern "C" int msn_snr_sums(const float *d_a, const float *d_b, size_t n, double *d_out2, void *d_work,
                            size_t work_bytes, void *stream) {
    clear_error();
    if (!d_a || !d_b || !d_out2) return set_error(MSN_ERR_INVALID, "msn_snr_sums: null pointer");
    MSN_TRY(check_red_ws(d_work, work_bytes, "msn_snr_sums"));
    // out[0] = sum a^2, out[1] = sum (a - b)^2
    return dual_reduce(d_a, d_a, d_b, nullptr, n, true, d_out2, (double *)d_work, as_stream(stream));
}

extern "C" int msn_snr_sums_f64(const double *d_a, const double *d_b, size_t n, double *d_out2, void *d_work,
                                size_t work_bytes, void *stream) {
    clear_error();
    if (!d_a || !d_b || !d_out2) return set_error(MSN_ERR_INVALID, "msn_snr_sums_f64: null pointer");
    MSN_TRY(check_red_ws(d_work, work_bytes, "msn_snr_sums_f64"));
    snr_partials_f64<<<kRedGrid, kRedThreads, 0, as_stream(stream)>>>(d_a, d_b, n, (double *)d_work, d_out2);
    return check_launch("snr_partials_f64");
}

extern "C" int msn_snr_update(const float *d_e, float *d_ms, const float *d_q, const double *d_scal, size_t n,
                              double *d_out2, void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    if (!d_e || !d_ms || !d_q || !d_scal || !d_out2) return set_error(MSN_ERR_INVALID, "msn_snr_update: null pointer");
    if (n % 4 || !aligned16(d_e) || !aligned16(d_ms) || !aligned16(d_q))
        return set_error(MSN_ERR_INVALID, "msn_snr_update: length must be a multiple of 4, pointers 16-byte aligned");
    MSN_TRY(check_red_ws(d_work, work_bytes, "msn_snr_update"));
    cudaStream_t st = as_stream(stream);
    double *partials = (double *)d_work;
    MSN_RED_LAUNCH(snr_update, kRedGrid, kRedThreads, st, (const float4 *)d_e, (float4 *)d_ms, (const float4 *)d_q, d_scal, n / 4,
                                                  partials, nullptr, d_out2);
    return check_launch("snr_update");
}

extern "C" size_t msn_segment_flags_bytes(size_t n) { return (n / 4 + 31) / 32; }

extern "C" int msn_segment_flags(const float *d_mask, size_t n, unsigned char *d_flags, void *stream) {
    clear_error();
    if (!d_mask || !d_flags) return set_error(MSN_ERR_INVALID, "msn_segment_flags: null pointer");
    if (n % 4 || !aligned16(d_mask))
        return set_error(MSN_ERR_INVALID, "msn_segment_flags: length must be a multiple of 4, pointer 16-byte aligned");
    const size_t nseg = (n / 4 + 31) / 32;
    size_t g = (nseg * 32 + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    segment_flags<<<(int)(g < 1 ? 1 : g), 256, 0, as_stream(stream)>>>((const float4 *)d_mask, n / 4, d_flags);
    return check_launch("segment_flags");
}

extern "C" int msn_row_flags(const float *d_mask, size_t rows, int cols, unsigned char *d_flags, void *stream) {
    clear_error();
    if (!d_mask || !d_flags) return set_error(MSN_ERR_INVALID, "msn_row_flags: null pointer");
    if (cols <= 0 || cols % 4 || !aligned16(d_mask))
        return set_error(MSN_ERR_INVALID, "msn_row_flags: cols must be a positive multiple of 4, pointer 16-byte aligned");
    size_t g = (rows * 32 + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    row_flags<<<(int)(g < 1 ? 1 : g), 256, 0, as_stream(stream)>>>((const float4 *)d_mask, rows, cols / 4, d_flags);
    return check_launch("row_flags");
}

extern "C" int msn_snr_update_masked(const float *d_e, float *d_ms, const float *d_q, const double *d_scal, size_t n,
                                     const unsigned char *d_flags, double *d_out2, void *d_work, size_t work_bytes,
                                     void *stream) {
    clear_error();
    if (!d_e || !d_ms || !d_q || !d_scal || !d_out2 || !d_flags)
        return set_error(MSN_ERR_INVALID, "msn_snr_update_masked: null pointer");
    if (n % 4 || !aligned16(d_e) || !aligned16(d_ms) || !aligned16(d_q))
        return set_error(MSN_ERR_INVALID,
                         "msn_snr_update_masked: length must be a multiple of 4, pointers 16-byte aligned");
    MSN_TRY(check_red_ws(d_work, work_bytes, "msn_snr_update_masked"));
    cudaStream_t st = as_stream(stream);
    double *partials = (double *)d_work;
    MSN_RED_LAUNCH(snr_update, kRedGrid, kRedThreads, st, (const float4 *)d_e, (float4 *)d_ms, (const float4 *)d_q, d_scal, n / 4,
                                                  partials, d_flags, d_out2);
    return check_launch("snr_update");
}

extern "C" int msn_cg_alpha_x(const float *d_x, const float *d_p, double *d_scal, float *d_xn, size_t n,
                              int *d_neg_count, void *stream) {
    clear_error();
    if (!d_x || !d_p || !d_scal || !d_xn || !d_neg_count) return set_error(MSN_ERR_INVALID, "msn_cg_alpha_x: null pointer");
    if (n % 4 || !aligned16(d_x) || !aligned16(d_p) || !aligned16(d_xn))
        return set_error(MSN_ERR_INVALID, "msn_cg_alpha_x: length must be a multiple of 4, pointers 16-byte aligned");
    MSN_TRY(check_cuda(cudaMemsetAsync(d_neg_count, 0, sizeof(int), as_stream(stream)), "reset count"));
    cg_alpha_x<<<ew_grid(n / 4), 256, 0, as_stream(stream)>>>((const float4 *)d_x, (const float4 *)d_p, d_scal,
                                                             (float4 *)d_xn, n / 4, d_neg_count);
    return check_launch("cg_alpha_x");
}

extern "C" int msn_cg_positivity(const float *d_x, float *d_xn, float *d_p, const double *d_scal, size_t n,
                                 void *stream) {
    clear_error();
    if (!d_x || !d_xn || !d_p || !d_scal) return set_error(MSN_ERR_INVALID, "msn_cg_positivity: null pointer");
    cg_positivity<<<ew_grid(n), 256, 0, as_stream(stream)>>>(d_x, d_xn, d_p, d_scal, n);
    return check_launch("cg_positivity");
}

extern "C" int msn_cg_residual(const float *d_r, const float *d_ap, double *d_scal, float *d_rn, size_t n,
                               void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    if (!d_r || !d_ap || !d_scal || !d_rn) return set_error(MSN_ERR_INVALID, "msn_cg_residual: null pointer");
    MSN_TRY(check_red_ws(d_work, work_bytes, "msn_cg_residual"));
    if (n % 4 || !aligned16(d_r) || !aligned16(d_ap) || !aligned16(d_rn))
        return set_error(MSN_ERR_INVALID, "msn_cg_residual: length must be a multiple of 4, pointers 16-byte aligned");
    cudaStream_t st = as_stream(stream);
    double *partials = (double *)d_work;
    MSN_RED_LAUNCH(cg_residual, kRedGrid, kRedThreads, st, (const float4 *)d_r, (const float4 *)d_ap, d_scal, (float4 *)d_rn,
                                                  n / 4, partials);
    return check_launch("cg_residual");
}

extern "C" int msn_cg_step(const float *d_x, const float *d_p, const float *d_r, const float *d_ap, double *d_scal,
                           float *d_xn, float *d_rn, size_t n, void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    if (!d_x || !d_p || !d_r || !d_ap || !d_scal || !d_xn || !d_rn) return set_error(MSN_ERR_INVALID, "msn_cg_step: null pointer");
    if (n % 4 || !aligned16(d_x) || !aligned16(d_p) || !aligned16(d_r) || !aligned16(d_ap) || !aligned16(d_xn) ||
        !aligned16(d_rn))
        return set_error(MSN_ERR_INVALID, "msn_cg_step: length must be a multiple of 4, pointers 16-byte aligned");
    MSN_TRY(check_red_ws(d_work, work_bytes, "msn_cg_step"));
    cudaStream_t st = as_stream(stream);
    MSN_RED_LAUNCH(cg_step, kRedGrid, kRedThreads, st, (const float4 *)d_x, (const float4 *)d_p, (const float4 *)d_r,
                   (const float4 *)d_ap, d_scal, (float4 *)d_xn, (float4 *)d_rn, n / 4, (double *)d_work,
                   RowSupport{nullptr, 1u});
    return check_launch("cg_step");
}

extern "C" int msn_cg_direction(const float *d_rn, float *d_p, const double *d_scal, size_t n, void *stream) {
    clear_error();
    if (!d_rn || !d_p || !d_scal) return set_error(MSN_ERR_INVALID, "msn_cg_direction: null pointer");
    if (n % 4 || !aligned16(d_rn) || !aligned16(d_p))
        return set_error(MSN_ERR_INVALID, "msn_cg_direction: length must be a multiple of 4, pointers 16-byte aligned");
    cg_direction<<<ew_grid(n / 4), 256, 0, as_stream(stream)>>>((const float4 *)d_rn, (float4 *)d_p, d_scal, n / 4);
    return check_launch("cg_direction");
}

extern "C" int msn_model_update(float *d_model, int pitch, const float *d_x, int n_sub, int off_r, int off_c,
                                float gain, int sign, void *stream) {
    clear_error();
    if (!d_model || !d_x || n_sub <= 0 || off_r < 0 || off_c < 0 || off_c + n_sub > pitch)
        return set_error(MSN_ERR_INVALID, "msn_model_update: bad arguments");
    model_update<<<ew_grid((size_t)n_sub * n_sub), 256, 0, as_stream(stream)>>>(d_model, pitch, d_x, n_sub, off_r,
                                                                                off_c, gain, sign >= 0 ? 1.0f : -1.0f);
    return check_launch("model_update");
}

extern "C" int msn_sub(const float *d_a, const float *d_b, float *d_out, size_t n, void *stream) {
    clear_error();
    if (!d_a || !d_b || !d_out) return set_error(MSN_ERR_INVALID, "msn_sub: null pointer");
    sub_kernel<<<ew_grid(n), 256, 0, as_stream(stream)>>>(d_a, d_b, d_out, n);
    return check_launch("sub");
}

extern "C" int msn_add(const float *d_a, const float *d_b, float *d_out, size_t n, void *stream) {
    clear_error();
    if (!d_a || !d_b || !d_out) return set_error(MSN_ERR_INVALID, "msn_add: null pointer");
    add_kernel<<<ew_grid(n), 256, 0, as_stream(stream)>>>(d_a, d_b, d_out, n);
    return check_launch("add");
}

extern "C" int msn_mul(const float *d_a, const float *d_b, float *d_out, size_t n, void *stream) {
    clear_error();
    if (!d_a || !d_b || !d_out) return set_error(MSN_ERR_INVALID, "msn_mul: null pointer");
    mul_kernel<<<ew_grid(n), 256, 0, as_stream(stream)>>>(d_a, d_b, d_out, n);
    return check_launch("mul");
}

extern "C" int msn_region_std(const float *d_img, int pitch, int rows, int cols, int off_r, int off_c, double *d_out4,
                              void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    if (!d_img || !d_out4 || rows <= 0 || cols <= 0 || off_r < 0 || off_c < 0 || off_c + cols > pitch)
        return set_error(MSN_ERR_INVALID, "msn_region_std: bad arguments");
    MSN_TRY(check_red_ws(d_work, work_bytes, "msn_region_std"));
    cudaStream_t st = as_stream(stream);
    double *partials = (double *)d_work;
    MSN_RED_LAUNCH(region_partials, kRedGrid, kRedThreads, st, d_img, pitch, rows, cols, off_r, off_c, nullptr, partials);
    MSN_TRY(check_launch("region_partials"));
    MSN_RED_LAUNCH(finalize_pairs, 1, kFinalizeThreads, st, partials, d_out4);
    MSN_TRY(check_launch("finalize_pairs"));
    MSN_RED_LAUNCH(region_partials, kRedGrid, kRedThreads, st, d_img, pitch, rows, cols, off_r, off_c, d_out4, partials);
    MSN_TRY(check_launch("region_partials"));
    // keep the first sum: write the second pair to out[1] via a temporary slot
    MSN_RED_LAUNCH(finalize_pairs, 1, kFinalizeThreads, st, partials, d_out4 + 1);
    MSN_TRY(check_launch("finalize_pairs"));
    std_finish<<<1, 1, 0, st>>>(d_out4, (long long)rows * cols);
    return check_launch("std_finish");
}

extern "C" int msn_set_reduction_precision(int bits) {
    clear_error();
    if (bits != 32 && bits != 48 && bits != 64)
        return set_error(MSN_ERR_INVALID, "msn_set_reduction_precision: bits must be 32, 48 or 64, got %d", bits);
    g_reduce_bits.store(bits);
    return MSN_OK;
}

extern "C" int msn_reduction_precision(void) { return g_reduce_bits.load(); }
