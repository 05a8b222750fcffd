// Noise estimate, thresholding, connected-component labelling and source
// extraction (pymoresane/iuwt_toolbox.py) for sm_103a.
//
// * MAD: exact median of |w| per plane by a three-pass radix select on the
//   float bit patterns (|w| >= 0 orders like its uint32 bits): digits of
//   12, 12 and 8 bits, each pass a shared-memory histogram restricted to the
//   prefix selected so far, followed by a one-CTA bin search. Both middle order
//   statistics are tracked, so even counts average them exactly as numpy's
//   median does (float32 mean, then division by 0.6745 in float32).
// * Threshold: w * (|w| > k sigma) with the comparison in float64 (the
//   reference compares float32 coefficients with a float64 threshold), the
//   optional edge-suppression rectangle and the per-plane signed maximum fused.
// * Labelling: 8-connected union-find on w != 0 with atomicMin hooking of the
//   larger root under the smaller one, so every component's root is its
//   first pixel in raster order; a final pass compresses every pixel onto its
//   root. Ranking the roots in raster order reproduces scipy.ndimage.label's
//   numbering exactly.
// * Extraction: top-down over scales, an island is kept when one of its pixels
//   passes w >= tol * max (|w| with neg_comp; the product rounded to float32 as
//   in gpu_source_extraction) and, below the top scale, lies inside the kept
//   mask of the scale above.
#include <cfloat>

#include "msn_common.cuh"

namespace msn {
namespace {

constexpr int kHistBins = 4096;

struct Rects {
    int y0, y1, x0, x1;      // included rectangle [y0, y1) x [x0, x1)
    int ey0, ey1, ex0, ex1;  // excluded rectangle (empty when ey0 >= ey1)
};

struct SelectState {
    unsigned prefix[2];
    unsigned long long k[2];
};

__device__ __forceinline__ bool in_rects(const Rects &r, int y, int x) {
    const bool inc = (y >= r.y0) & (y < r.y1) & (x >= r.x0) & (x < r.x1);
    const bool exc = (y >= r.ey0) & (y < r.ey1) & (x >= r.ex0) & (x < r.ex1);
    return inc & !exc;
}

__device__ __forceinline__ int enc_ord(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float dec_ord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

// ---------------------------------------------------------------------------
// MAD radix select
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(512)
mad_hist(const float *__restrict__ w, int ny, int nx, Rects rects, const SelectState *__restrict__ state,
         unsigned *__restrict__ hist, int shift, int bits) {
    __shared__ unsigned sh[2][kHistBins];
    const int plane = blockIdx.y;
    const SelectState st = state[plane];
    const bool two = st.prefix[0] != st.prefix[1];
    const int nbins = 1 << bits;
    for (int i = threadIdx.x; i < 2 * kHistBins; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    const int hi = shift + bits;
    const unsigned dmask = (unsigned)nbins - 1u;
    const float4 *w4 = reinterpret_cast<const float4 *>(w + (size_t)plane * ny * nx);
    const int nx4 = nx >> 2;
    const int total4 = ny * nx4;
    const bool all_in = rects.y0 <= 0 && rects.y1 >= ny && rects.x0 <= 0 && rects.x1 >= nx && rects.ey0 >= rects.ey1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total4; i += gridDim.x * blockDim.x) {
        const float4 v = __ldg(w4 + i);
        int y = 0, x = 0;
        if (!all_in) {
            y = i / nx4;
            x = (i - y * nx4) * 4;
        }
        const float vals[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (!all_in && !in_rects(rects, y, x + k)) continue;
            const unsigned key = __float_as_uint(vals[k]) & 0x7FFFFFFFu;
            const unsigned pre = hi >= 32 ? 0u : (key >> hi);
            const unsigned dig = (key >> shift) & dmask;
            if (pre == st.prefix[0]) atomicAdd(&sh[0][dig], 1u);
            if (two && pre == st.prefix[1]) atomicAdd(&sh[1][dig], 1u);
        }
    }
    __syncthreads();
    unsigned *gh = hist + (size_t)plane * 2 * kHistBins;
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
        if (sh[0][b]) atomicAdd(gh + b, sh[0][b]);
        if (two && sh[1][b]) atomicAdd(gh + kHistBins + b, sh[1][b]);
    }
}

// One CTA per plane: locate the bin holding rank k for both targets, extend
// the prefixes, reduce the ranks, clear the histograms for the next pass.
__global__ void __launch_bounds__(1024)
mad_pick(SelectState *__restrict__ state, unsigned *__restrict__ hist, int bits) {
    __shared__ unsigned long long csum[1024];
    __shared__ int found_bin[2];
    __shared__ unsigned long long found_below[2];
    const int plane = blockIdx.x;
    SelectState st = state[plane];
    const bool two = st.prefix[0] != st.prefix[1];
    const int nbins = 1 << bits;
    const int per = (nbins + 1023) / 1024;
    unsigned *gh = hist + (size_t)plane * 2 * kHistBins;
    if (threadIdx.x == 0) {
        found_bin[0] = found_bin[1] = 0;
        found_below[0] = found_below[1] = 0;
    }
    __syncthreads();
    for (int t = 0; t < 2; ++t) {
        const unsigned *h = gh + (two ? t : 0) * kHistBins;
        unsigned long long local = 0;
        const int b0 = threadIdx.x * per;
        for (int b = b0; b < b0 + per && b < nbins; ++b) local += h[b];
        csum[threadIdx.x] = local;
        __syncthreads();
        // inclusive scan (Hillis-Steele) over 1024 partial sums
        for (int off = 1; off < 1024; off <<= 1) {
            const unsigned long long v = threadIdx.x >= off ? csum[threadIdx.x - off] : 0ull;
            __syncthreads();
            csum[threadIdx.x] += v;
            __syncthreads();
        }
        const unsigned long long before = threadIdx.x ? csum[threadIdx.x - 1] : 0ull;
        const unsigned long long k = st.k[t];
        if (k >= before && k < csum[threadIdx.x]) {
            unsigned long long acc = before;
            for (int b = b0; b < b0 + per && b < nbins; ++b) {
                if (k < acc + h[b]) {
                    found_bin[t] = b;
                    found_below[t] = acc;
                    break;
                }
                acc += h[b];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int t = 0; t < 2; ++t) {
            st.prefix[t] = (st.prefix[t] << bits) | (unsigned)found_bin[t];
            st.k[t] -= found_below[t];
        }
        state[plane] = st;
    }
    for (int b = threadIdx.x; b < 2 * kHistBins; b += blockDim.x) gh[b] = 0;
}

__global__ void mad_init(SelectState *state, unsigned long long n, int planes) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= planes) return;
    SelectState st;
    st.prefix[0] = st.prefix[1] = 0;
    st.k[0] = (n - 1) / 2;  // lower middle
    st.k[1] = n / 2;        // upper middle
    state[p] = st;
}

__global__ void mad_finish(const SelectState *__restrict__ state, double *__restrict__ sigma, int planes,
                           unsigned long long n) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= planes) return;
    if (n == 0) {
        sigma[p] = __longlong_as_double(0x7FF8000000000000LL);
        return;
    }
    const float a = __uint_as_float(state[p].prefix[0]);
    const float b = __uint_as_float(state[p].prefix[1]);
    const float med = (n & 1ull) ? b : __fdiv_rn(__fadd_rn(a, b), 2.0f);
    sigma[p] = (double)__fdiv_rn(med, 0.6745f);
}

// ---------------------------------------------------------------------------
// Threshold (+ edge suppression + per-plane maximum)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
threshold_kernel(const float *__restrict__ w, int ny, int nx, const double *__restrict__ sigma, double sigma_level,
                 const int *__restrict__ supp, float *__restrict__ out, int *__restrict__ plane_max) {
    const int plane = blockIdx.y;
    const double thr = sigma_level * sigma[plane];
    int r0 = 0, r1 = ny, c0 = 0, c1 = nx;
    if (supp) {
        r0 = supp[4 * plane + 0];
        r1 = supp[4 * plane + 1];
        c0 = supp[4 * plane + 2];
        c1 = supp[4 * plane + 3];
    }
    const size_t base = (size_t)plane * ny * nx;
    const float4 *w4 = reinterpret_cast<const float4 *>(w + base);
    float4 *o4 = reinterpret_cast<float4 *>(out + base);
    const int nx4 = nx >> 2;
    const int total4 = ny * nx4;
    // For a float a, (double)a > thr exactly when a > thr rounded down to float
    // (NaN and infinities included), so the reference's float64 comparison
    // (iuwt_toolbox.py:70) needs no float64 arithmetic per element.
    const float thr_f = __double2float_rd(thr);
    float mx = -FLT_MAX;
    bool any = false;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total4; i += gridDim.x * blockDim.x) {
        const float4 v = __ldg(w4 + i);
        float vals[4] = {v.x, v.y, v.z, v.w};
        int y = 0, x = 0;
        if (supp) {
            y = i / nx4;
            x = (i - y * nx4) * 4;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float keep = (fabsf(vals[k]) > thr_f) ? 1.0f : 0.0f;
            float o = __fmul_rn(keep, vals[k]);
            if (supp) {
                const bool inside = (y >= r0) & (y < r1) & (x + k >= c0) & (x + k < c1);
                o = __fmul_rn(o, inside ? 1.0f : 0.0f);
            }
            vals[k] = o;
            mx = fmaxf(mx, o);
            any = true;
        }
        o4[i] = make_float4(vals[0], vals[1], vals[2], vals[3]);
    }
    if (plane_max) {
        for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        any = __any_sync(0xffffffffu, any);
        if ((threadIdx.x & 31) == 0 && any) atomicMax(plane_max + plane, enc_ord(mx));
    }
}

__global__ void init_max(int *m, int planes) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < planes) m[p] = enc_ord(-INFINITY);
}

__global__ void decode_max(const int *__restrict__ m, float *__restrict__ out, int planes) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < planes) out[p] = dec_ord(m[p]);
}

// seg (may be null): per plane, one byte per 128-float segment (32 float4, the
// float4 indices of one warp), 1 when the segment holds a non-zero value.
__global__ void __launch_bounds__(256)
plane_max_kernel(const float *__restrict__ w, size_t per_plane4, int use_abs, int *__restrict__ plane_max,
                 unsigned char *__restrict__ seg) {
    const int plane = blockIdx.y;
    const float4 *w4 = reinterpret_cast<const float4 *>(w) + (size_t)plane * per_plane4;
    unsigned char *seg_p = seg ? seg + (size_t)plane * ((per_plane4 + 31) / 32) : nullptr;
    float mx = -FLT_MAX;
    const int lane = threadIdx.x & 31;
    // warp-aligned bases: the 32 lanes of a warp read one segment
    for (size_t base = (size_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < per_plane4;
         base += (size_t)gridDim.x * blockDim.x) {
        const size_t i = base + lane;
        bool nz = false;
        if (i < per_plane4) {
            float4 v = __ldg(w4 + i);
            nz = v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f;
            if (use_abs) {
                v.x = fabsf(v.x);
                v.y = fabsf(v.y);
                v.z = fabsf(v.z);
                v.w = fabsf(v.w);
            }
            mx = fmaxf(mx, fmaxf(fmaxf(v.x, v.y), fmaxf(v.z, v.w)));
        }
        if (seg_p) {
            const unsigned any = __any_sync(0xffffffffu, nz);
            if (lane == 0) seg_p[base >> 5] = any ? 1 : 0;
        }
    }
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    if ((threadIdx.x & 31) == 0) atomicMax(plane_max + plane, enc_ord(mx));
}

// ---------------------------------------------------------------------------
// Union-find labelling (8-connectivity), roots = first pixel in raster order
// ---------------------------------------------------------------------------
__device__ __forceinline__ int uf_find(const int *P, int x) {
    int p = __ldcg(P + x);
    while (p != x) {
        x = p;
        p = __ldcg(P + x);
    }
    return x;
}

// Find with path halving: every visited node is re-pointed at its grandparent.
// Parents always have smaller indices than their children (links are made with
// atomicMin towards the smaller root), so the grandparent is an ancestor and
// the store only shortens the path; a store that races a concurrent hook of
// the same node at worst undoes a link that the hooking thread's retry (it
// saw a non-root) makes again.
__device__ __forceinline__ int uf_find_halve(int *P, int x) {
    while (true) {
        const int p = __ldcg(P + x);
        if (p == x) return x;
        const int gp = __ldcg(P + p);
        if (gp == p) return p;
        __stcg(P + x, gp);
        x = gp;
    }
}

__device__ __forceinline__ void uf_union(int *P, int a, int b) {
    // Lock-free: every failed hook means another thread lowered P[a]; indices
    // only decrease, so the loop terminates.
    while (true) {
        a = uf_find_halve(P, a);
        b = uf_find_halve(P, b);
        if (a == b) return;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicMin(P + a, b);
        if (old == a) return;
        a = old;
    }
}

// With segment flags (seg: per plane, one byte per 128 pixels, 0 when every pixel
// of the segment is zero), P of an empty segment is neither written nor read by any
// labelling or extraction kernel: those pixels are background.
__device__ __forceinline__ bool seg_live(const unsigned char *seg, size_t local) {
    return !seg || __ldg(seg + (local >> 7)) != 0;
}

// One plane per blockIdx.y, four pixels per step (float4 of w, int4 of P); a warp's
// 32 steps are one segment.
__global__ void uf_init(const float *__restrict__ w, int *__restrict__ P, int per4,
                        const unsigned char *__restrict__ seg_all) {
    const size_t plane = blockIdx.y;
    const float4 *w4 = reinterpret_cast<const float4 *>(w) + plane * per4;
    int4 *P4 = reinterpret_cast<int4 *>(P) + plane * per4;
    const unsigned char *seg = seg_all ? seg_all + plane * ((per4 + 31) / 32) : nullptr;
    for (int i4 = blockIdx.x * blockDim.x + threadIdx.x; i4 < per4; i4 += gridDim.x * blockDim.x) {
        if (seg && !__ldg(seg + (i4 >> 5))) continue;
        const float4 v = __ldg(w4 + i4);
        const int b = 4 * i4;
        P4[i4] = make_int4(v.x != 0.0f ? b : -1, v.y != 0.0f ? b + 1 : -1, v.z != 0.0f ? b + 2 : -1,
                           v.w != 0.0f ? b + 3 : -1);
    }
}

// Scalar forms for any plane size and alignment (msn_label): one pixel per step.
__global__ void uf_init_scalar(const float *__restrict__ w, int *__restrict__ P, int per) {
    const size_t plane = blockIdx.y;
    const float *wp = w + plane * per;
    int *Pp = P + plane * per;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < per; i += gridDim.x * blockDim.x)
        Pp[i] = (wp[i] != 0.0f) ? i : -1;
}

__global__ void uf_compress_scalar(int *__restrict__ P, int per) {
    int *Pp = P + (size_t)blockIdx.y * per;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < per; i += gridDim.x * blockDim.x)
        if (Pp[i] >= 0) Pp[i] = uf_find(Pp, i);
}

// Unions of each foreground pixel e with its earlier 8-neighbours a = (y-1, x-1),
// b = (y-1, x), c = (y-1, x+1), d = (y, x-1), by the decision tree of Wu, Otoo and
// Suzuki ("Optimizing two-pass connected-component labeling algorithms", 2009):
// when b is foreground, a, c and d are already joined to it through other pixels'
// unions, so e joins b alone; otherwise e joins c and, since c is not adjacent to
// a or d, also a or else d; with neither b nor c, e joins a or else d. The
// transitive closure is 8-connectivity, as with all four unions, and the roots
// (smallest index of each component, by the atomicMin hooking) are unchanged.
__global__ void uf_merge(int *__restrict__ Pall, int ny, int nx, const unsigned char *__restrict__ seg_all) {
    const int plane = blockIdx.y;
    int *P = Pall + (size_t)plane * ny * nx;
    const int total = ny * nx;
    const unsigned char *seg = seg_all ? seg_all + (size_t)plane * ((total + 127) / 128) : nullptr;
    // a foreground pixel: in a live segment and labelled
    auto fg = [&](int j) { return seg_live(seg, (size_t)j) && __ldcg(P + j) >= 0; };
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        if (!fg(i)) continue;
        const int y = i / nx, x = i - y * nx;
        const int up = i - nx;
        const bool b = y > 0 && fg(up);
        if (b) {
            uf_union(P, i, up);
            continue;
        }
        const bool c = y > 0 && x + 1 < nx && fg(up + 1);
        const bool a = y > 0 && x > 0 && fg(up - 1);
        const bool d = x > 0 && fg(i - 1);
        if (c) uf_union(P, i, up + 1);
        if (a)
            uf_union(P, i, up - 1);
        else if (d)
            uf_union(P, i, i - 1);
    }
}

__global__ void uf_compress(int *__restrict__ P, int per4, const unsigned char *__restrict__ seg_all) {
    const size_t plane = blockIdx.y;
    int *Pp = P + plane * per4 * 4;
    const unsigned char *seg = seg_all ? seg_all + plane * ((per4 + 31) / 32) : nullptr;
    for (int i4 = blockIdx.x * blockDim.x + threadIdx.x; i4 < per4; i4 += gridDim.x * blockDim.x) {
        if (seg && !__ldg(seg + (i4 >> 5))) continue;
        int4 v = reinterpret_cast<const int4 *>(Pp)[i4];
        if ((v.x & v.y & v.z & v.w) < 0) continue;  // all four background
        if (v.x >= 0) v.x = uf_find(Pp, v.x);
        if (v.y >= 0) v.y = uf_find(Pp, v.y);
        if (v.z >= 0) v.z = uf_find(Pp, v.z);
        if (v.w >= 0) v.w = uf_find(Pp, v.w);
        reinterpret_cast<int4 *>(Pp)[i4] = v;
    }
}

// ---------------------------------------------------------------------------
// Extraction: mark kept islands at one scale, then write that scale's mask.
// ---------------------------------------------------------------------------
__global__ void extract_mark(const float *__restrict__ w, const int *__restrict__ P, const float *__restrict__ mask_above,
                             const int *__restrict__ maxima_enc, int plane, float tolerance, int neg_comp,
                             unsigned char *__restrict__ keep, int n, const unsigned char *__restrict__ seg) {
    const float thr = __fmul_rn(tolerance, dec_ord(maxima_enc[plane]));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!seg_live(seg, (size_t)i)) continue;
        const int root = P[i];
        if (root < 0) continue;
        const float v = neg_comp ? fabsf(w[i]) : w[i];
        if (!(v >= thr)) continue;
        if (mask_above && mask_above[i] == 0.0f) continue;
        keep[root] = 1;
    }
}

// A pixel of an empty segment is background (mask 0) without reading its label;
// extracted is still the product 0 * w, which keeps the sign of a zero w.
__global__ void extract_apply(const float *__restrict__ w, const int *__restrict__ P,
                              const unsigned char *__restrict__ keep, float *__restrict__ mask,
                              float *__restrict__ extracted, int n, const unsigned char *__restrict__ seg) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!seg_live(seg, (size_t)i)) {
            mask[i] = 0.0f;
            if (extracted) extracted[i] = __fmul_rn(0.0f, w[i]);
            continue;
        }
        const int root = P[i];
        const float m = (root >= 0 && keep[root]) ? 1.0f : 0.0f;
        mask[i] = m;
        if (extracted) extracted[i] = __fmul_rn(m, w[i]);
    }
}

// ---------------------------------------------------------------------------
// scipy-compatible label numbering: rank of each root in raster order.
// ---------------------------------------------------------------------------
constexpr int kScanBlock = 1024;

__global__ void root_block_counts(const int *__restrict__ P, int n, int *__restrict__ block_sums) {
    __shared__ int s[32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int is_root = (i < n && P[i] == i) ? 1 : 0;
    int v = __reduce_add_sync(0xffffffffu, is_root);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = __reduce_add_sync(0xffffffffu, s[threadIdx.x]);
        if (threadIdx.x == 0) block_sums[blockIdx.x] = v;
    }
}

__global__ void scan_block_sums(int *__restrict__ block_sums, int nblocks, int *__restrict__ count) {
    // Single CTA exclusive scan of the per-block root counts (in place).
    __shared__ int carry;
    __shared__ int s[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += kScanBlock) {
        const int i = base + threadIdx.x;
        const int v = i < nblocks ? block_sums[i] : 0;
        // warp inclusive scan
        int x = v;
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, off);
            if ((threadIdx.x & 31) >= off) x += y;
        }
        if ((threadIdx.x & 31) == 31) s[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            int t = s[threadIdx.x];
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, t, off);
                if (threadIdx.x >= off) t += y;
            }
            s[threadIdx.x] = t;
        }
        __syncthreads();
        const int warp_prefix = (threadIdx.x >= 32) ? s[(threadIdx.x >> 5) - 1] : 0;
        const int incl = x + warp_prefix;
        if (i < nblocks) block_sums[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = carry;
}

__global__ void write_labels(const int *__restrict__ P, int n, const int *__restrict__ block_offsets,
                             int *__restrict__ rank, int *__restrict__ labels) {
    // rank[i] = number of roots before i (for roots); labels use the root's rank.
    __shared__ int s[32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int is_root = (i < n && P[i] == i) ? 1 : 0;
    const unsigned ball = __ballot_sync(0xffffffffu, is_root);
    const int lane = threadIdx.x & 31;
    const int in_warp = __popc(ball & ((1u << lane) - 1u));
    if (lane == 0) s[threadIdx.x >> 5] = __popc(ball);
    __syncthreads();
    if (threadIdx.x < 32) {
        int t = s[threadIdx.x];
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, off);
            if (threadIdx.x >= off) t += y;
        }
        s[threadIdx.x] = t;
    }
    __syncthreads();
    const int warp_prefix = (threadIdx.x >= 32) ? s[(threadIdx.x >> 5) - 1] : 0;
    if (is_root) rank[i] = block_offsets[blockIdx.x] + warp_prefix + in_warp;
}

__global__ void gather_labels(const int *__restrict__ P, const int *__restrict__ rank, int n, int *__restrict__ labels) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int r = P[i];
        labels[i] = r >= 0 ? rank[r] + 1 : 0;
    }
}

// One step down the scales: extract_apply of plane hi, then extract_mark of plane
// lo = hi - 1 against the mask just formed at the same pixel (what extract_mark
// would read back from mask_hi), so each plane pair takes one pass.
__global__ void extract_step(const float *__restrict__ w_hi, const int *__restrict__ P_hi,
                             const unsigned char *__restrict__ keep_hi, float *__restrict__ mask_hi,
                             float *__restrict__ ext_hi, const unsigned char *__restrict__ seg_hi,
                             const float *__restrict__ w_lo, const int *__restrict__ P_lo,
                             const unsigned char *__restrict__ seg_lo, const int *__restrict__ maxima_enc, int lo_plane,
                             float tolerance, int neg_comp, unsigned char *__restrict__ keep_lo, int n) {
    const float thr = __fmul_rn(tolerance, dec_ord(maxima_enc[lo_plane]));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float m = 0.0f;
        if (seg_live(seg_hi, (size_t)i)) {
            const int root = P_hi[i];
            m = (root >= 0 && keep_hi[root]) ? 1.0f : 0.0f;
        }
        mask_hi[i] = m;
        if (ext_hi) ext_hi[i] = __fmul_rn(m, w_hi[i]);
        if (m == 0.0f || !seg_live(seg_lo, (size_t)i)) continue;
        const int root = P_lo[i];
        if (root < 0) continue;
        const float v = neg_comp ? fabsf(w_lo[i]) : w_lo[i];
        if (!(v >= thr)) continue;
        keep_lo[root] = 1;
    }
}

int grid_for(size_t n, int threads, int cap = 152 * 16) {
    size_t g = (n + threads - 1) / threads;
    if (g > (size_t)cap) g = cap;
    return g < 1 ? 1 : (int)g;
}

size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

// seg (may be null): segment flags of every plane (plane_max_kernel).
int launch_labelling(const float *w, int planes, int ny, int nx, int *P, cudaStream_t st,
                     const unsigned char *seg = nullptr) {
    const size_t per = (size_t)ny * nx;
    // four pixels per step where the planes allow it (the segment flags need it)
    const bool vec = per % 4 == 0 && aligned16(w) && aligned16(P);
    if (seg && !vec) return set_error(MSN_ERR_INVALID, "labelling: segment flags need 16-byte aligned planes");
    const int per4 = (int)(per / 4);
    const int gx = grid_for(vec ? (size_t)per4 : per, 256, 8 * 152 / planes + 8);
    if (vec)
        uf_init<<<dim3(gx, planes), 256, 0, st>>>(w, P, per4, seg);
    else
        uf_init_scalar<<<dim3(gx, planes), 256, 0, st>>>(w, P, (int)per);
    MSN_TRY(check_launch("uf_init"));
    dim3 g(grid_for(per, 256, 152 * 8), planes);
    uf_merge<<<g, 256, 0, st>>>(P, ny, nx, seg);
    MSN_TRY(check_launch("uf_merge"));
    if (vec)
        uf_compress<<<dim3(gx, planes), 256, 0, st>>>(P, per4, seg);
    else
        uf_compress_scalar<<<dim3(gx, planes), 256, 0, st>>>(P, (int)per);
    return check_launch("uf_compress");
}

}  // namespace

// Workspace layouts -------------------------------------------------------------
size_t mad_workspace(int planes) {
    return a256((size_t)planes * 2 * kHistBins * sizeof(unsigned)) + a256((size_t)planes * sizeof(SelectState));
}
size_t seg_bytes(int ny, int nx) { return ((size_t)ny * nx + 127) / 128; }
size_t extract_workspace(int planes, int ny, int nx) {
    const size_t per = (size_t)ny * nx;
    return a256(per * planes * sizeof(int)) + a256(per * planes) + a256((size_t)planes * sizeof(int)) +
           a256(seg_bytes(ny, nx) * planes);
}
size_t label_workspace(int ny, int nx) {
    const size_t per = (size_t)ny * nx;
    const size_t nblocks = (per + kScanBlock - 1) / kScanBlock;
    return a256(per * sizeof(int)) + a256(per * sizeof(int)) + a256(nblocks * sizeof(int)) + a256(sizeof(int));
}

int mad_sigma_impl(const float *w, int planes, int ny, int nx, const Rects &rects, unsigned long long n, double *sigma,
                   void *work, cudaStream_t st) {
    unsigned *hist = (unsigned *)work;
    SelectState *state = (SelectState *)((char *)work + a256((size_t)planes * 2 * kHistBins * sizeof(unsigned)));
    MSN_TRY(check_cuda(cudaMemsetAsync(hist, 0, (size_t)planes * 2 * kHistBins * sizeof(unsigned), st), "mad memset"));
    mad_init<<<(planes + 127) / 128, 128, 0, st>>>(state, n, planes);
    MSN_TRY(check_launch("mad_init"));
    if (n > 0) {
        const int shifts[3] = {20, 8, 0}, bits[3] = {12, 12, 8};
        const size_t per4 = (size_t)ny * nx / 4;
        const int bx = grid_for(per4, 512, 2 * 152 / (planes < 1 ? 1 : planes) + 8);
        for (int p = 0; p < 3; ++p) {
            mad_hist<<<dim3(bx, planes), 512, 0, st>>>(w, ny, nx, rects, state, hist, shifts[p], bits[p]);
            MSN_TRY(check_launch("mad_hist"));
            mad_pick<<<planes, 1024, 0, st>>>(state, hist, bits[p]);
            MSN_TRY(check_launch("mad_pick"));
        }
    }
    mad_finish<<<(planes + 127) / 128, 128, 0, st>>>(state, sigma, planes, n);
    return check_launch("mad_finish");
}

int threshold_impl(const float *w, int planes, int ny, int nx, const double *sigma, double sigma_level, const int *supp,
                   float *out, float *plane_max, int *max_scratch, cudaStream_t st) {
    if (plane_max) {
        init_max<<<(planes + 127) / 128, 128, 0, st>>>(max_scratch, planes);
        MSN_TRY(check_launch("init_max"));
    }
    const size_t per4 = (size_t)ny * nx / 4;
    const int bx = grid_for(per4, 256, 4 * 152 / (planes < 1 ? 1 : planes) + 8);
    threshold_kernel<<<dim3(bx, planes), 256, 0, st>>>(w, ny, nx, sigma, sigma_level, supp, out,
                                                       plane_max ? max_scratch : nullptr);
    MSN_TRY(check_launch("threshold"));
    if (plane_max) {
        decode_max<<<(planes + 127) / 128, 128, 0, st>>>(max_scratch, plane_max, planes);
        MSN_TRY(check_launch("decode_max"));
    }
    return MSN_OK;
}

int extraction_impl(const float *w, int planes, int ny, int nx, float tolerance, int neg_comp, float *mask,
                    float *extracted, void *work, cudaStream_t st) {
    const size_t per = (size_t)ny * nx;
    int *P = (int *)work;
    unsigned char *keep = (unsigned char *)work + a256(per * planes * sizeof(int));
    int *maxima = (int *)((char *)keep + a256(per * planes));
    // per plane, one flag per 128 pixels: labelling and extraction skip empty segments
    unsigned char *seg = (unsigned char *)maxima + a256((size_t)planes * sizeof(int));
    const size_t nseg = seg_bytes(ny, nx);
    init_max<<<(planes + 127) / 128, 128, 0, st>>>(maxima, planes);
    MSN_TRY(check_launch("init_max"));
    plane_max_kernel<<<dim3(grid_for(per / 4, 256, 4 * 152 / planes + 8), planes), 256, 0, st>>>(w, per / 4, neg_comp,
                                                                                                 maxima, seg);
    MSN_TRY(check_launch("plane_max"));
    MSN_TRY(launch_labelling(w, planes, ny, nx, P, st, seg));
    MSN_TRY(check_cuda(cudaMemsetAsync(keep, 0, per * planes, st), "keep memset"));
    // top-down over the scales: mark the top plane, then per step apply plane i + 1 and mark
    // plane i, then apply plane 0
    const int top = planes - 1;
    const size_t ot = (size_t)top * per;
    extract_mark<<<grid_for(per, 256), 256, 0, st>>>(w + ot, P + ot, nullptr, maxima, top, tolerance, neg_comp,
                                                     keep + ot, (int)per, seg + (size_t)top * nseg);
    MSN_TRY(check_launch("extract_mark"));
    for (int i = top - 1; i >= 0; --i) {
        const size_t hi = (size_t)(i + 1) * per, lo = (size_t)i * per;
        extract_step<<<grid_for(per, 256), 256, 0, st>>>(w + hi, P + hi, keep + hi, mask + hi,
                                                         extracted ? extracted + hi : nullptr, seg + (size_t)(i + 1) * nseg,
                                                         w + lo, P + lo, seg + (size_t)i * nseg, maxima, i, tolerance,
                                                         neg_comp, keep + lo, (int)per);
        MSN_TRY(check_launch("extract_step"));
    }
    extract_apply<<<grid_for(per, 256), 256, 0, st>>>(w, P, keep, mask, extracted, (int)per, seg);
    return check_launch("extract_apply");
}

int label_impl(const float *img, int ny, int nx, int *labels, int *count, void *work, cudaStream_t st) {
    const size_t per = (size_t)ny * nx;
    const int nblocks = (int)((per + kScanBlock - 1) / kScanBlock);
    int *P = (int *)work;
    int *rank = (int *)((char *)work + a256(per * sizeof(int)));
    int *bsum = (int *)((char *)rank + a256(per * sizeof(int)));
    int *cnt = count ? count : (int *)((char *)bsum + a256((size_t)nblocks * sizeof(int)));
    MSN_TRY(launch_labelling(img, 1, ny, nx, P, st));
    root_block_counts<<<nblocks, kScanBlock, 0, st>>>(P, (int)per, bsum);
    MSN_TRY(check_launch("root_block_counts"));
    scan_block_sums<<<1, kScanBlock, 0, st>>>(bsum, nblocks, cnt);
    MSN_TRY(check_launch("scan_block_sums"));
    write_labels<<<nblocks, kScanBlock, 0, st>>>(P, (int)per, bsum, rank, labels);
    MSN_TRY(check_launch("write_labels"));
    gather_labels<<<grid_for(per, 256), 256, 0, st>>>(P, rank, (int)per, labels);
    return check_launch("gather_labels");
}

int validate_planes(int planes, int ny, int nx, const char *fn) {
    if (planes <= 0 || ny <= 0 || nx <= 0) return set_error(MSN_ERR_INVALID, "%s: empty input", fn);
    if (nx % 4) return set_error(MSN_ERR_INVALID, "%s: nx=%d must be a multiple of 4", fn, nx);
    if ((size_t)ny * nx >= (size_t)1 << 31) return set_error(MSN_ERR_INVALID, "%s: plane too large", fn);
    return MSN_OK;
}

}  // namespace msn

using namespace msn;

extern "C" size_t msn_toolbox_workspace_bytes(int planes, int ny, int nx) {
    if (planes <= 0 || ny <= 0 || nx <= 0) return 0;
    size_t a = mad_workspace(planes), b = extract_workspace(planes, ny, nx), c = label_workspace(ny, nx);
    size_t m = a > b ? a : b;
    return m > c ? m : c;
}

extern "C" int msn_mad_sigma(const float *d_w, int planes, int ny, int nx, const int *rects, double *d_sigma,
                             void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_mad_sigma";
    MSN_TRY(validate_planes(planes, ny, nx, fn));
    if (!d_w || !d_sigma || !rects) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    if (!d_work || work_bytes < mad_workspace(planes)) return set_error(MSN_ERR_WORKSPACE, "%s: workspace too small", fn);
    Rects r{rects[0], rects[1], rects[2], rects[3], rects[4], rects[5], rects[6], rects[7]};
    // Count the pixels of include \ exclude.
    auto clampi = [](int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); };
    r.y0 = clampi(r.y0, 0, ny), r.y1 = clampi(r.y1, 0, ny), r.x0 = clampi(r.x0, 0, nx), r.x1 = clampi(r.x1, 0, nx);
    r.ey0 = clampi(r.ey0, 0, ny), r.ey1 = clampi(r.ey1, 0, ny), r.ex0 = clampi(r.ex0, 0, nx), r.ex1 = clampi(r.ex1, 0, nx);
    auto area = [](long long a0, long long a1, long long b0, long long b1) {
        return (a1 > a0 && b1 > b0) ? (a1 - a0) * (b1 - b0) : 0LL;
    };
    const long long inc = area(r.y0, r.y1, r.x0, r.x1);
    const long long both = area(r.y0 > r.ey0 ? r.y0 : r.ey0, r.y1 < r.ey1 ? r.y1 : r.ey1, r.x0 > r.ex0 ? r.x0 : r.ex0,
                                r.x1 < r.ex1 ? r.x1 : r.ex1);
    return mad_sigma_impl(d_w, planes, ny, nx, r, (unsigned long long)(inc - both), d_sigma, d_work,
                          as_stream(stream));
}

extern "C" int msn_apply_threshold(const float *d_w, int planes, int ny, int nx, const double *d_sigma,
                                   double sigma_level, const int *d_supp_rects, float *d_out, float *d_plane_max,
                                   void *d_work, size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_apply_threshold";
    MSN_TRY(validate_planes(planes, ny, nx, fn));
    if (!d_w || !d_sigma || !d_out) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    if (d_plane_max && (!d_work || work_bytes < (size_t)planes * sizeof(int)))
        return set_error(MSN_ERR_WORKSPACE, "%s: workspace too small", fn);
    return threshold_impl(d_w, planes, ny, nx, d_sigma, sigma_level, d_supp_rects, d_out, d_plane_max, (int *)d_work,
                          as_stream(stream));
}

extern "C" int msn_source_extraction(const float *d_w, int planes, int ny, int nx, float tolerance, int neg_comp,
                                     float *d_mask, float *d_extracted, void *d_work, size_t work_bytes,
                                     void *stream) {
    clear_error();
    static const char *fn = "msn_source_extraction";
    MSN_TRY(validate_planes(planes, ny, nx, fn));
    if (!d_w || !d_mask) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    if (!aligned16(d_w) || !aligned16(d_work))
        return set_error(MSN_ERR_INVALID, "%s: planes and workspace must be 16-byte aligned", fn);
    if (!d_work || work_bytes < extract_workspace(planes, ny, nx))
        return set_error(MSN_ERR_WORKSPACE, "%s: workspace too small", fn);
    return extraction_impl(d_w, planes, ny, nx, tolerance, neg_comp, d_mask, d_extracted, d_work, as_stream(stream));
}

extern "C" int msn_plane_max(const float *d_w, int planes, size_t per_plane, int use_abs, float *d_out, void *d_work,
                             size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_plane_max";
    if (!d_w || !d_out || planes <= 0 || per_plane == 0 || per_plane % 4 || !aligned16(d_w))
        return set_error(MSN_ERR_INVALID,
                         "%s: bad arguments (plane size a positive multiple of 4, planes 16-byte aligned)", fn);
    if (!d_work || work_bytes < (size_t)planes * sizeof(int)) return set_error(MSN_ERR_WORKSPACE, "%s: workspace", fn);
    cudaStream_t st = as_stream(stream);
    int *enc = (int *)d_work;
    init_max<<<(planes + 127) / 128, 128, 0, st>>>(enc, planes);
    MSN_TRY(check_launch("init_max"));
    plane_max_kernel<<<dim3(grid_for(per_plane / 4, 256, 4 * 152 / planes + 8), planes), 256, 0, st>>>(
        d_w, per_plane / 4, use_abs, enc, nullptr);
    MSN_TRY(check_launch("plane_max"));
    decode_max<<<(planes + 127) / 128, 128, 0, st>>>(enc, d_out, planes);
    return check_launch("decode_max");
}

extern "C" int msn_label(const float *d_img, int ny, int nx, int *d_labels, int *d_count, void *d_work,
                         size_t work_bytes, void *stream) {
    clear_error();
    static const char *fn = "msn_label";
    if (ny <= 0 || nx <= 0 || (size_t)ny * nx >= ((size_t)1 << 31))
        return set_error(MSN_ERR_INVALID, "%s: bad shape %d x %d", fn, ny, nx);
    if (!d_img || !d_labels) return set_error(MSN_ERR_INVALID, "%s: null pointer", fn);
    if (!d_work || work_bytes < label_workspace(ny, nx))
        return set_error(MSN_ERR_WORKSPACE, "%s: workspace too small", fn);
    return label_impl(d_img, ny, nx, d_labels, d_count, d_work, as_stream(stream));
}
