// FFT kernels specialised per transform length M (every stride, Ns and twiddle
// offset is a compile-time constant, so shared-memory addressing in a pass is
// one index computation plus immediate offsets).
//
// fft_convolve (pymoresane/iuwt_convolution.py:18-73) is three kernels:
//   1. rfft_rows: two real image rows packed into one complex sequence
//      (z = a + i b), zero-padded into the M-point grid, transformed in shared
//      memory and split into the two Hermitian half-spectra (R2C along x).
//   2. conv_cols: per group of C adjacent spectrum columns, the forward column
//      FFT, the product with the cached PSF spectrum (fused between the last
//      forward and first inverse pass when the plan allows) and the inverse
//      column FFT; only the rows that survive the fft-shift and centre crop
//      are written.
//   3. irfft_rows: the Hermitian half-rows are staged, rebuilt into packed
//      pairs, inverse transformed, divided by M^2 (scale_fft, :242-265) and
//      written with the fft-shift (:161-201) and crop (contiguous_slice,
//      :204-239) folded into the output index map.
// Every kernel is persistent: CTAs walk rounds of work items and, when two
// buffers fit in shared memory, prefetch the next item with cp.async while the
// current one is transformed. Spectra use a group-major layout
// [ceil(W/C)][rows][C] (W = M/2 + 1), so a column group is one contiguous
// block; the PSF spectrum is stored the same way ("packed" spectrum).
#pragma once

#include <utility>

#include "fft_core.cuh"
#include "fft_plan.cuh"
#include "msn_common.cuh"

namespace msn {
namespace fftk {

template <int C>
struct GroupMajor {
    int rows;
    __device__ __forceinline__ size_t at(int r, int col) const {
        return ((size_t)(col / C) * rows + r) * C + (col % C);
    }
    __device__ __forceinline__ bool valid(int, int) const { return true; }
};

struct RowMajor {
    int pitch;
    __device__ __forceinline__ size_t at(int r, int col) const { return (size_t)r * pitch + col; }
    __device__ __forceinline__ bool valid(int col, int w) const { return col < w; }
};

template <int M>
struct P {
    static constexpr CtPlan plan = ct_plan(M);
    static constexpr int E = plan.e;
    static constexpr int TEAM = M / E;
    static constexpr int NP = plan.np;
    static constexpr int C = plan.group;
    static constexpr int TW_WORDS = (plan.twlen + 1) & ~1;  // even: keeps the buffers 16-byte aligned
    static constexpr int PLEN = padded_len(M);
};

template <int N, class F>
__device__ __forceinline__ void static_for(F &&f) {
    [&]<int... I>(std::integer_sequence<int, I...>) { (f(std::integral_constant<int, I>{}), ...); }
    (std::make_integer_sequence<int, N>{});
}

// Direct per-pass twiddle tables: entry twbase[q] + k (R - 1) + (r - 1) holds
// exp(-2 pi i r k / (Ns R)) for pass q (Ns = ns[q], R = radix[q]).
template <int M>
__device__ __forceinline__ void build_twiddles(float2 *tw) {
    static_for<P<M>::NP>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        if constexpr (q > 0) {
            constexpr int R = P<M>::plan.radix[q], NS = P<M>::plan.ns[q];
            constexpr int count = NS * (R - 1), step = kTwN / (NS * R);
            float2 *dst = tw + P<M>::plan.twbase[q];
            for (int i = threadIdx.x; i < count; i += blockDim.x) {
                const int k = i / (R - 1), r = i - k * (R - 1) + 1;
                dst[i] = __ldg(&kTwiddle[r * k * step]);
            }
        }
    });
}

// Offset of sidx(base + off) from sidx(base) when it does not depend on base:
// off a multiple of 16, or base aligned so that [base, base + off] stays in
// one 16-element block.
__host__ __device__ constexpr int pad_off(int off) { return off + off / 16; }

// One Stockham pass (pass Q of length M) over a team's sequence.
template <bool INV, int M, int Q>
__device__ __forceinline__ void pass(float2 *__restrict__ buf, const float2 *__restrict__ tw, int t) {
    constexpr int E = P<M>::E, R = P<M>::plan.radix[Q], NS = P<M>::plan.ns[Q];
    constexpr int NB = E / R, TEAM = P<M>::TEAM, STRIDE = M / R;
    static_assert(E % R == 0, "radix must divide the per-thread element count");
    constexpr bool RD_LIN = STRIDE % 16 == 0;
    constexpr bool WR_LIN = NS % 16 == 0 || 16 % (NS * R) == 0;
    float2 v[E];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * TEAM;
        if constexpr (RD_LIN) {
            const float2 *s = buf + sidx(j);
#pragma unroll
            for (int r = 0; r < R; ++r) v[b * R + r] = s[pad_off(r * STRIDE)];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) v[b * R + r] = buf[sidx(j + r * STRIDE)];
        }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * TEAM;
        const int k = j % NS;
        if constexpr (NS > 1) {
            const float2 *w = tw + P<M>::plan.twbase[Q] + k * (R - 1) - 1;
#pragma unroll
            for (int r = 1; r < R; ++r) v[b * R + r] = cmul(v[b * R + r], INV ? cconj(w[r]) : w[r]);
        }
        dft<INV, R>(v + b * R);
        const int base = (j - k) * R + k;
        if constexpr (WR_LIN) {
            float2 *s = buf + sidx(base);
#pragma unroll
            for (int r = 0; r < R; ++r) s[NS % 16 == 0 ? pad_off(r * NS) : r * NS] = v[b * R + out_slot<R>(r)];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) buf[sidx(base + r * NS)] = v[b * R + out_slot<R>(r)];
        }
    }
    __syncthreads();
}

// Passes [Q0, Q1) of a team's transform (unnormalised; INV uses exp(+2 pi i/M)).
template <bool INV, int M, int Q0, int Q1>
__device__ __forceinline__ void passes(float2 *buf, const float2 *tw, int t) {
    static_for<Q1 - Q0>([&](auto qc) { pass<INV, M, Q0 + decltype(qc)::value>(buf, tw, t); });
}

// Last forward pass (radix R, Ns = M / R), product with the PSF spectrum and
// first inverse pass (radix R, Ns = 1) in registers: the forward pass leaves
// X[j + r M/R] with butterfly j, exactly the values the inverse pass's
// butterfly j reads. h: the column group's spectrum block [M][C]; cc: column.
template <int M>
__device__ __forceinline__ void fused_product(float2 *__restrict__ buf, const float2 *__restrict__ tw,
                                              const float2 *__restrict__ h, int cc, int t) {
    constexpr int QL = P<M>::NP - 1;
    constexpr int E = P<M>::E, R = P<M>::plan.radix[QL], C = P<M>::C;
    constexpr int NB = E / R, TEAM = P<M>::TEAM, STRIDE = M / R;
    static_assert(P<M>::plan.radix[0] == R && STRIDE % 16 == 0 && 16 % R == 0, "plan not fusable");
    float2 v[E], hv[E];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * TEAM;
        const float2 *s = buf + sidx(j);
        const float2 *hs = h + (size_t)j * C + cc;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            v[b * R + r] = s[pad_off(r * STRIDE)];
            hv[b * R + r] = __ldg(hs + r * STRIDE * C);
        }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * TEAM;  // k = j mod (M / R) = j
        const float2 *w = tw + P<M>::plan.twbase[QL] + j * (R - 1) - 1;
#pragma unroll
        for (int r = 1; r < R; ++r) v[b * R + r] = cmul(v[b * R + r], w[r]);
        dft<false, R>(v + b * R);
        float2 u[R];
#pragma unroll
        for (int r = 0; r < R; ++r) u[r] = cmul(v[b * R + out_slot<R>(r)], hv[b * R + r]);
        dft<true, R>(u);
        float2 *s = buf + sidx(j * R);
#pragma unroll
        for (int r = 0; r < R; ++r) s[r] = u[out_slot<R>(r)];
    }
    __syncthreads();
}

// First pass (Ns = 1, no twiddles) fed from registers: load(n) returns
// sequence element n (global loads, zero padding, Hermitian extension ...).
// Writes the pass output to the team's shared-memory sequence.
template <bool INV, int M, class Load>
__device__ __forceinline__ void first_pass_load(float2 *__restrict__ buf, Load load, int t) {
    constexpr int E = P<M>::E, R = P<M>::plan.radix[0];
    constexpr int NB = E / R, TEAM = P<M>::TEAM, STRIDE = M / R;
    static_assert(P<M>::plan.ns[0] == 1 && 16 % R == 0, "first pass must be Ns = 1 with R dividing 16");
    float2 v[E];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * TEAM;
#pragma unroll
        for (int r = 0; r < R; ++r) v[b * R + r] = load(j + r * STRIDE);
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * TEAM;
        dft<INV, R>(v + b * R);
        float2 *s = buf + sidx(j * R);
#pragma unroll
        for (int r = 0; r < R; ++r) s[r] = v[b * R + out_slot<R>(r)];
    }
    __syncthreads();
}

// Last pass (Ns = M / R) from the team's shared-memory sequence to
// store(n, X[n]) for every output element n (no shared-memory write back).
template <bool INV, int M, class Store>
__device__ __forceinline__ void last_pass_store(const float2 *__restrict__ buf, const float2 *__restrict__ tw,
                                                Store store, int t) {
    constexpr int Q = P<M>::NP - 1;
    constexpr int E = P<M>::E, R = P<M>::plan.radix[Q], NS = P<M>::plan.ns[Q];
    constexpr int NB = E / R, TEAM = P<M>::TEAM, STRIDE = M / R;
    static_assert(NS == STRIDE && STRIDE % 16 == 0, "last pass must have Ns = M / R");
    float2 v[E];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * TEAM;
        const float2 *s = buf + sidx(j);
#pragma unroll
        for (int r = 0; r < R; ++r) v[b * R + r] = s[pad_off(r * STRIDE)];
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const int j = t + b * TEAM;  // k = j mod Ns = j
        const float2 *w = tw + P<M>::plan.twbase[Q] + j * (R - 1) - 1;
#pragma unroll
        for (int r = 1; r < R; ++r) v[b * R + r] = cmul(v[b * R + r], INV ? cconj(w[r]) : w[r]);
        dft<INV, R>(v + b * R);
#pragma unroll
        for (int r = 0; r < R; ++r) store(j + r * NS, v[b * R + out_slot<R>(r)]);
    }
}

// Plans whose first pass has Ns = 1 with a radix dividing 16 and whose last pass
// has Ns = M / R on 16-element blocks (every plan with at least two passes).
template <int M>
constexpr bool direct_ok() {
    return direct_ok(P<M>::plan, M);
}

// --------------------------------------------------------------------------
// 1. Row R2C: rows [2q, 2q+1] of a real nrows x ncols image placed at column
//    offset col_off of the M-point row; writes W = M/2 + 1 bins per row.
// --------------------------------------------------------------------------
template <int M, class OutL, bool DB>
__global__ void __launch_bounds__(512)
rfft_rows(const float *__restrict__ x, int nrows, int ncols, int col_off, float2 *__restrict__ out, OutL lay) {
    extern __shared__ float2 smem[];
    constexpr int TEAM = P<M>::TEAM, PLEN = P<M>::PLEN, W = M / 2 + 1;
    const int p = threadIdx.x / TEAM, t = threadIdx.x - p * TEAM, teams = blockDim.x / TEAM;
    float2 *tw = smem;
    build_twiddles<M>(tw);
    float2 *buf0 = smem + P<M>::TW_WORDS + p * (DB ? 2 : 1) * PLEN;
    float2 *buf1 = DB ? buf0 + PLEN : buf0;
    const int npairs = (nrows + 1) / 2;
    const int per_round = gridDim.x * teams;
    const int rounds = (npairs + per_round - 1) / per_round;
    auto issue = [&](int round, float2 *buf) {
        const int ra = 2 * (round * per_round + blockIdx.x * teams + p), rb = ra + 1;
        const bool ha = ra < nrows, hb = rb < nrows;
        for (int n = t; n < M; n += TEAM) {
            const int c = n - col_off;
            const bool in_row = c >= 0 && c < ncols;
            float *slot = reinterpret_cast<float *>(buf + sidx(n));
            cp_async4(slot, ha && in_row ? x + (size_t)ra * ncols + c : x, ha && in_row);
            cp_async4(slot + 1, hb && in_row ? x + (size_t)rb * ncols + c : x, hb && in_row);
        }
        cp_async_commit();
    };
    if (DB && rounds > 0) issue(0, buf0);
    for (int round = 0; round < rounds; ++round) {
        float2 *cur = (round & 1) ? buf1 : buf0;
        if (DB) {
            if (round + 1 < rounds) {
                issue(round + 1, (round & 1) ? buf0 : buf1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
        } else {
            issue(round, cur);
            cp_async_wait<0>();
        }
        __syncthreads();
        passes<false, M, 0, P<M>::NP>(cur, tw, t);
        const int ra = 2 * (round * per_round + blockIdx.x * teams + p), rb = ra + 1;
        const bool ha = ra < nrows, hb = rb < nrows;
        for (int k = t; k < W; k += TEAM) {
            const float2 zk = cur[sidx(k)];
            const float2 zm = cur[sidx(k == 0 ? 0 : M - k)];
            // Xa = (Z[k] + conj Z[M-k]) / 2, Xb = (Z[k] - conj Z[M-k]) / (2i)
            if (ha) out[lay.at(ra, k)] = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
            if (hb) out[lay.at(rb, k)] = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
        }
        __syncthreads();
    }
}

// --------------------------------------------------------------------------
// 2. Column pass over groups of C adjacent columns. Input rows [0, in_rows)
//    land at sequence positions in_off + r (zero elsewhere); output row i takes
//    sequence position (i + shift) mod M.
// --------------------------------------------------------------------------
template <int M, int MODE, class InL, class OutL, bool DB, bool FUSED>
__global__ void __launch_bounds__(P<M>::C * P<M>::TEAM)
conv_cols(const float2 *__restrict__ in, InL in_lay, int in_rows, int in_off, const float2 *__restrict__ h,
          float2 *__restrict__ out, OutL out_lay, int out_rows, int shift) {
    extern __shared__ float2 smem[];
    constexpr int TEAM = P<M>::TEAM, PLEN = P<M>::PLEN, C = P<M>::C, W = M / 2 + 1, GROUPS = P<M>::plan.groups;
    const int cc = threadIdx.x / TEAM, t = threadIdx.x - cc * TEAM;
    float2 *tw = smem;
    build_twiddles<M>(tw);
    float2 *set0 = smem + P<M>::TW_WORDS;
    float2 *set1 = DB ? set0 + C * PLEN : set0;
    const int rounds = (GROUPS + gridDim.x - 1) / gridDim.x;
    auto issue = [&](int round, float2 *set) {
        const int g = round * gridDim.x + blockIdx.x;
        const bool gv = g < GROUPS;
#pragma unroll
        for (int c2 = 0; c2 < C; ++c2) {
            const int col = g * C + c2;
            const bool cv = gv && in_lay.valid(col, W);
            for (int n = threadIdx.x; n < M; n += blockDim.x) {
                const int r = n - in_off;
                const bool valid = cv && r >= 0 && r < in_rows;
                cp_async8(set + c2 * PLEN + sidx(n), valid ? in + in_lay.at(r, col) : in, valid);
            }
        }
        cp_async_commit();
    };
    if (DB && rounds > 0) issue(0, set0);
    for (int round = 0; round < rounds; ++round) {
        float2 *cur = (round & 1) ? set1 : set0;
        if (DB) {
            if (round + 1 < rounds) {
                issue(round + 1, (round & 1) ? set0 : set1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
        } else {
            issue(round, cur);
            cp_async_wait<0>();
        }
        __syncthreads();
        const int g = round * gridDim.x + blockIdx.x;
        const float2 *hg = h + (size_t)(g < GROUPS ? g : GROUPS - 1) * M * C;
        float2 *buf = cur + cc * PLEN;
        if constexpr (MODE == kConv && FUSED) {
            passes<false, M, 0, P<M>::NP - 1>(buf, tw, t);
            fused_product<M>(buf, tw, hg, cc, t);
            passes<true, M, 1, P<M>::NP>(buf, tw, t);
        } else {
            if constexpr (MODE != kInv) passes<false, M, 0, P<M>::NP>(buf, tw, t);
            if constexpr (MODE == kConv) {
#pragma unroll
                for (int c2 = 0; c2 < C; ++c2) {
                    for (int k = threadIdx.x; k < M; k += blockDim.x) {
                        float2 *s = cur + c2 * PLEN + sidx(k);
                        *s = cmul(*s, __ldg(hg + (size_t)k * C + c2));
                    }
                }
                __syncthreads();
            }
            if constexpr (MODE != kFwd) passes<true, M, 0, P<M>::NP>(buf, tw, t);
        }
        if (g < GROUPS) {
#pragma unroll
            for (int c2 = 0; c2 < C; ++c2) {
                const int col = g * C + c2;
                if (!out_lay.valid(col, W)) continue;
                for (int i = threadIdx.x; i < out_rows; i += blockDim.x) {
                    int n = i + shift;
                    if (n >= M) n -= M;
                    out[out_lay.at(i, col)] = cur[c2 * PLEN + sidx(n)];
                }
            }
        }
        __syncthreads();
    }
}

// Column convolution with global-fed first pass and global-written last pass:
// one shared-memory sequence per column (no staging copies, no double buffer),
// so two or more CTAs fit on an SM. Requires a fusable plan.
template <int M, class InL, class OutL>
__global__ void __launch_bounds__(P<M>::C * P<M>::TEAM)
conv_cols_direct(const float2 *__restrict__ in, InL in_lay, int in_rows, int in_off, const float2 *__restrict__ h,
                 float2 *__restrict__ out, OutL out_lay, int out_rows, int shift) {
    extern __shared__ float2 smem[];
    constexpr int TEAM = P<M>::TEAM, PLEN = P<M>::PLEN, C = P<M>::C, W = M / 2 + 1, GROUPS = P<M>::plan.groups;
    constexpr int NP = P<M>::NP;
    static_assert(P<M>::plan.fusable && NP >= 2, "conv_cols_direct needs a fusable plan");
    const int cc = threadIdx.x / TEAM, t = threadIdx.x - cc * TEAM;
    float2 *tw = smem;
    build_twiddles<M>(tw);
    float2 *buf = smem + P<M>::TW_WORDS + cc * PLEN;
    __syncthreads();
    for (int g = blockIdx.x; g < GROUPS; g += gridDim.x) {
        const int col = g * C + cc;
        const bool in_valid = in_lay.valid(col, W), out_valid = out_lay.valid(col, W);
        // sequence position n is input row n - in_off when that row exists, zero otherwise
        first_pass_load<false, M>(buf, [&](int n) {
            const int row = n - in_off;
            return (in_valid && row >= 0 && row < in_rows) ? __ldg(in + in_lay.at(row, col)) : make_float2(0.f, 0.f);
        }, t);
        passes<false, M, 1, NP - 1>(buf, tw, t);
        fused_product<M>(buf, tw, h + (size_t)g * M * C, cc, t);
        passes<true, M, 1, NP - 1>(buf, tw, t);
        // output row i takes sequence position (i + shift) mod M
        last_pass_store<true, M>(buf, tw, [&](int n, float2 v) {
            int i = n - shift;
            if (i < 0) i += M;
            if (out_valid && i < out_rows) out[out_lay.at(i, col)] = v;
        }, t);
        __syncthreads();
    }
}

// Row R2C with the first pass fed from the image rows (two real rows packed as
// one complex sequence, zero outside [col_off, col_off + ncols)); one
// shared-memory sequence per team. The loop over row pairs is uniform across
// the CTA (teams past the last pair compute zeros and store nothing).
template <int M, class OutL>
__global__ void __launch_bounds__(512)
rfft_rows_direct(const float *__restrict__ x, int nrows, int ncols, int col_off, float2 *__restrict__ out, OutL lay) {
    extern __shared__ float2 smem[];
    constexpr int TEAM = P<M>::TEAM, PLEN = P<M>::PLEN, W = M / 2 + 1, NP = P<M>::NP;
    const int p = threadIdx.x / TEAM, t = threadIdx.x - p * TEAM, teams = blockDim.x / TEAM;
    float2 *tw = smem;
    build_twiddles<M>(tw);
    float2 *buf = smem + P<M>::TW_WORDS + p * PLEN;
    __syncthreads();
    const int npairs = (nrows + 1) / 2;
    for (int pair0 = blockIdx.x * teams; pair0 < npairs; pair0 += gridDim.x * teams) {
        const int ra = 2 * (pair0 + p), rb = ra + 1;
        const bool ha = ra < nrows, hb = rb < nrows;
        first_pass_load<false, M>(buf, [&](int n) {
            const int c = n - col_off;
            const bool in_row = c >= 0 && c < ncols;
            return make_float2(ha && in_row ? __ldg(x + (size_t)ra * ncols + c) : 0.f,
                               hb && in_row ? __ldg(x + (size_t)rb * ncols + c) : 0.f);
        }, t);
        passes<false, M, 1, NP>(buf, tw, t);
        for (int k = t; k < W; k += TEAM) {
            const float2 zk = buf[sidx(k)];
            const float2 zm = buf[sidx(k == 0 ? 0 : M - k)];
            // Xa = (Z[k] + conj Z[M-k]) / 2, Xb = (Z[k] - conj Z[M-k]) / (2i)
            if (ha) out[lay.at(ra, k)] = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
            if (hb) out[lay.at(rb, k)] = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
        }
        __syncthreads();
    }
}

// Row C2R of Hermitian half-rows [2q, 2q+1] with the first inverse pass fed from
// the half spectra (Z = Xa + i Xb extended by Hermitian symmetry) and the last
// pass writing the shifted, cropped, scaled real rows; one shared-memory
// sequence per team.
// Measured on GB300 at M = 4096: left free to use 128 registers (one 512-thread
// CTA per SM, all 32 first-pass loads in flight) it beats both a 64-register
// bound (two CTAs per SM, loads serialised) and the staged cp.async version.
template <int M, class InL>
__global__ void __launch_bounds__(512)
irfft_rows_direct(const float2 *__restrict__ in, InL lay, int nrows, float *__restrict__ out, int out_cols,
                  int shift, float div) {
    extern __shared__ float2 smem[];
    constexpr int TEAM = P<M>::TEAM, PLEN = P<M>::PLEN, HALF = M / 2, NP = P<M>::NP;
    const int p = threadIdx.x / TEAM, t = threadIdx.x - p * TEAM, teams = blockDim.x / TEAM;
    float2 *tw = smem;
    build_twiddles<M>(tw);
    float2 *buf = smem + P<M>::TW_WORDS + p * PLEN;
    __syncthreads();
    const int npairs = (nrows + 1) / 2;
    for (int pair0 = blockIdx.x * teams; pair0 < npairs; pair0 += gridDim.x * teams) {
        const int ra = 2 * (pair0 + p), rb = ra + 1;
        const bool ha = ra < nrows, hb = rb < nrows;
        first_pass_load<true, M>(buf, [&](int n) {
            const int k = n <= HALF ? n : M - n;
            float2 a = ha ? __ldg(in + lay.at(ra, k)) : make_float2(0.f, 0.f);
            float2 b = hb ? __ldg(in + lay.at(rb, k)) : make_float2(0.f, 0.f);
            if (k == 0 || k == HALF) {  // c2r uses only the real part of the DC and Nyquist bins
                a.y = 0.0f;
                b.y = 0.0f;
            }
            return n <= HALF ? make_float2(a.x - b.y, a.y + b.x)   // Xa + i Xb
                             : make_float2(a.x + b.y, b.x - a.y);  // conj(Xa) + i conj(Xb)
        }, t);
        passes<true, M, 1, NP - 1>(buf, tw, t);
        last_pass_store<true, M>(buf, tw, [&](int n, float2 z) {
            int j = n - shift;
            if (j < 0) j += M;
            if (j < out_cols) {
                if (ha) out[(size_t)ra * out_cols + j] = __fdiv_rn(z.x, div);
                if (hb) out[(size_t)rb * out_cols + j] = __fdiv_rn(z.y, div);
            }
        }, t);
        __syncthreads();
    }
}

// --------------------------------------------------------------------------
// 3. Row C2R of Hermitian half-rows [2q, 2q+1]; output column j takes sample
//    (j + shift) mod M, divided by `div` (M^2).
// --------------------------------------------------------------------------
template <int M, class InL, bool DB>
__global__ void __launch_bounds__(512)
irfft_rows(const float2 *__restrict__ in, InL lay, int nrows, float *__restrict__ out, int out_cols, int shift,
           float div) {
    extern __shared__ float2 smem[];
    constexpr int TEAM = P<M>::TEAM, PLEN = P<M>::PLEN, HALF = M / 2, WLEN = HALF + 1;
    constexpr int SLEN = (2 * WLEN + 1) & ~1;
    const int p = threadIdx.x / TEAM, t = threadIdx.x - p * TEAM, teams = blockDim.x / TEAM;
    float2 *tw = smem;
    build_twiddles<M>(tw);
    float2 *buf = smem + P<M>::TW_WORDS + p * (PLEN + (DB ? 2 : 1) * SLEN);
    float2 *st0 = buf + PLEN, *st1 = DB ? st0 + SLEN : st0;
    const int npairs = (nrows + 1) / 2;
    const int per_round = gridDim.x * teams;
    const int rounds = (npairs + per_round - 1) / per_round;
    auto issue = [&](int round, float2 *stage) {
        const int ra = 2 * (round * per_round + blockIdx.x * teams + p), rb = ra + 1;
        const bool ha = ra < nrows, hb = rb < nrows;
        for (int k = t; k < WLEN; k += TEAM) {
            cp_async8(stage + k, ha ? in + lay.at(ra, k) : in, ha);
            cp_async8(stage + WLEN + k, hb ? in + lay.at(rb, k) : in, hb);
        }
        cp_async_commit();
    };
    if (DB && rounds > 0) issue(0, st0);
    for (int round = 0; round < rounds; ++round) {
        float2 *stage = (round & 1) ? st1 : st0;
        if (DB) {
            if (round + 1 < rounds) {
                issue(round + 1, (round & 1) ? st0 : st1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
        } else {
            issue(round, stage);
            cp_async_wait<0>();
        }
        __syncthreads();
        for (int k = t; k <= HALF; k += TEAM) {
            float2 a = stage[k], b = stage[WLEN + k];
            if (k == 0 || k == HALF) {  // c2r uses only the real part of the DC and Nyquist bins
                a.y = 0.0f;
                b.y = 0.0f;
            }
            buf[sidx(k)] = make_float2(a.x - b.y, a.y + b.x);                                  // Xa + i Xb
            if (k != 0 && k != HALF) buf[sidx(M - k)] = make_float2(a.x + b.y, b.x - a.y);  // conj(Xa) + i conj(Xb)
        }
        __syncthreads();
        passes<true, M, 0, P<M>::NP>(buf, tw, t);
        const int ra = 2 * (round * per_round + blockIdx.x * teams + p), rb = ra + 1;
        const bool ha = ra < nrows, hb = rb < nrows;
        for (int j = t; j < out_cols; j += TEAM) {
            int n = j + shift;
            if (n >= M) n -= M;
            const float2 z = buf[sidx(n)];
            if (ha) out[(size_t)ra * out_cols + j] = __fdiv_rn(z.x, div);
            if (hb) out[(size_t)rb * out_cols + j] = __fdiv_rn(z.y, div);
        }
        __syncthreads();
    }
}

// --------------------------------------------------------------------------
// Host-side launchers.
// --------------------------------------------------------------------------
constexpr size_t kMaxSmem = 227 * 1024;

inline int num_sms() {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    return sms;
}

template <class K>
int persistent_grid(K kernel, int threads, size_t smem, int items) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (per_sm < 1) per_sm = 1;
    const int grid = per_sm * num_sms();
    return grid < items ? grid : (items < 1 ? 1 : items);
}

// Teams (row pairs in flight) per row-kernel CTA: 512 threads when they fit in
// about half the shared memory, so that two CTAs share an SM.
template <int M>
int row_teams(size_t per_team, size_t fixed) {
    int teams = 512 / P<M>::TEAM;
    const int by_smem = (int)((112 * 1024 - fixed) / per_team);
    if (teams > by_smem) teams = by_smem;
    return teams < 1 ? 1 : teams;
}

template <int M, class OutL>
int launch_rfft_rows(const float *x, int nrows, int ncols, int col_off, float2 *out, OutL lay, cudaStream_t st) {
    const size_t tw = P<M>::TW_WORDS * sizeof(float2), seq = P<M>::PLEN * sizeof(float2);
    if constexpr (direct_ok<M>()) {
        const int teams = row_teams<M>(seq, tw);
        const size_t smem = tw + (size_t)teams * seq;
        const int threads = teams * P<M>::TEAM;
        const int items = ((nrows + 1) / 2 + teams - 1) / teams;
        const int grid = persistent_grid(rfft_rows_direct<M, OutL>, threads, smem, items);
        rfft_rows_direct<M, OutL><<<grid, threads, smem, st>>>(x, nrows, ncols, col_off, out, lay);
        return check_launch("rfft_rows");
    }
    const bool db = tw + 2 * seq <= kMaxSmem;
    const int teams = row_teams<M>((db ? 2 : 1) * seq, tw);
    const size_t smem = tw + (size_t)teams * (db ? 2 : 1) * seq;
    const int threads = teams * P<M>::TEAM;
    const int items = ((nrows + 1) / 2 + teams - 1) / teams;
    if (db) {
        const int grid = persistent_grid(rfft_rows<M, OutL, true>, threads, smem, items);
        rfft_rows<M, OutL, true><<<grid, threads, smem, st>>>(x, nrows, ncols, col_off, out, lay);
    } else {
        const int grid = persistent_grid(rfft_rows<M, OutL, false>, threads, smem, items);
        rfft_rows<M, OutL, false><<<grid, threads, smem, st>>>(x, nrows, ncols, col_off, out, lay);
    }
    return check_launch("rfft_rows");
}

template <int M, class InL>
int launch_irfft_rows(const float2 *in, InL lay, int nrows, float *out, int out_cols, int shift, float div,
                      cudaStream_t st) {
    const size_t tw = P<M>::TW_WORDS * sizeof(float2), seq = P<M>::PLEN * sizeof(float2);
    if constexpr (direct_ok<M>()) {
        const int teams = row_teams<M>(seq, tw);
        const size_t smem = tw + (size_t)teams * seq;
        const int threads = teams * P<M>::TEAM;
        const int items = ((nrows + 1) / 2 + teams - 1) / teams;
        const int grid = persistent_grid(irfft_rows_direct<M, InL>, threads, smem, items);
        irfft_rows_direct<M, InL><<<grid, threads, smem, st>>>(in, lay, nrows, out, out_cols, shift, div);
        return check_launch("irfft_rows");
    }
    const size_t stage = (size_t)((2 * (M / 2 + 1) + 1) & ~1) * sizeof(float2);
    const bool db = tw + seq + 2 * stage <= 112 * 1024;
    const size_t per_team = seq + (db ? 2 : 1) * stage;
    const int teams = row_teams<M>(per_team, tw);
    const size_t smem = tw + (size_t)teams * per_team;
    const int threads = teams * P<M>::TEAM;
    const int items = ((nrows + 1) / 2 + teams - 1) / teams;
    if (db) {
        const int grid = persistent_grid(irfft_rows<M, InL, true>, threads, smem, items);
        irfft_rows<M, InL, true><<<grid, threads, smem, st>>>(in, lay, nrows, out, out_cols, shift, div);
    } else {
        const int grid = persistent_grid(irfft_rows<M, InL, false>, threads, smem, items);
        irfft_rows<M, InL, false><<<grid, threads, smem, st>>>(in, lay, nrows, out, out_cols, shift, div);
    }
    return check_launch("irfft_rows");
}

template <int M, int MODE, class InL, class OutL>
int launch_cols(const float2 *in, InL in_lay, int in_rows, int in_off, const float2 *h, float2 *out, OutL out_lay,
                int out_rows, int shift, cudaStream_t st) {
    constexpr int C = P<M>::C;
    constexpr bool FUSED = MODE == kConv && P<M>::plan.fusable;
    const size_t tw = P<M>::TW_WORDS * sizeof(float2), set = (size_t)C * P<M>::PLEN * sizeof(float2);
    const int threads = C * P<M>::TEAM;
    if constexpr (FUSED && direct_ok<M>()) {
        const size_t smem = tw + set;
        const int grid = persistent_grid(conv_cols_direct<M, InL, OutL>, threads, smem, P<M>::plan.groups);
        conv_cols_direct<M, InL, OutL><<<grid, threads, smem, st>>>(in, in_lay, in_rows, in_off, h, out, out_lay,
                                                                     out_rows, shift);
        return check_launch("conv_cols");
    }
    const bool db = tw + 2 * set <= kMaxSmem;
    const size_t smem = tw + (db ? 2 : 1) * set;
    if (db) {
        const int grid = persistent_grid(conv_cols<M, MODE, InL, OutL, true, FUSED>, threads, smem,
                                         P<M>::plan.groups);
        conv_cols<M, MODE, InL, OutL, true, FUSED><<<grid, threads, smem, st>>>(in, in_lay, in_rows, in_off, h, out,
                                                                               out_lay, out_rows, shift);
    } else {
        const int grid = persistent_grid(conv_cols<M, MODE, InL, OutL, false, FUSED>, threads, smem,
                                         P<M>::plan.groups);
        conv_cols<M, MODE, InL, OutL, false, FUSED><<<grid, threads, smem, st>>>(in, in_lay, in_rows, in_off, h, out,
                                                                                out_lay, out_rows, shift);
    }
    return check_launch("conv_cols");
}

// --------------------------------------------------------------------------
// Per-length operations.
// --------------------------------------------------------------------------
template <int M>
int conv_run(const float *x, int n, const float2 *spec, float *out, int linear, float2 *t1, float2 *t2,
             cudaStream_t st, const unsigned char *rows) {
    if constexpr (M == sq::kLength) {
        // the 2048^2 linear convolution with a 4096^2 PSF: four-step kernels. Their bulk and
        // tensor copies need 16-byte aligned image, spectrum, output and workspace addresses;
        // other pointers take the Stockham kernels below (same results within rounding).
        const bool aligned = aligned16(x) && aligned16(spec) && aligned16(out) && aligned16(t1) && aligned16(t2);
        if (linear && n == M / 2 && aligned && tune_value(kKnobFourStep))
            return sq::conv_run(x, spec, out, t1, t2, st, rows);
    }
    const int off = linear ? (M - n) / 2 : 0;
    const int shift = (off + M / 2) % M;
    const float div = (float)M * (float)M;
    const GroupMajor<P<M>::C> l1{n};
    MSN_TRY(launch_rfft_rows<M>(x, n, n, off, t1, l1, st));
    MSN_TRY(launch_cols<M, kConv>(t1, l1, n, off, spec, t2, l1, n, shift, st));
    return launch_irfft_rows<M>(t2, l1, n, out, n, shift, div, st);
}

template <int M>
int spectrum_run(const float *psf, int rows, int cols, int off_r, int off_c, float2 *out, float2 *t1,
                 cudaStream_t st) {
    const GroupMajor<P<M>::C> l1{rows};
    MSN_TRY(launch_rfft_rows<M>(psf, rows, cols, off_c, t1, l1, st));
    return launch_cols<M, kFwd>(t1, l1, rows, off_r, (const float2 *)nullptr, out, GroupMajor<P<M>::C>{M}, M, 0, st);
}

template <int M>
int rfft2_run(const float *in, float2 *out, float2 *t1, cudaStream_t st) {
    const GroupMajor<P<M>::C> l1{M};
    MSN_TRY(launch_rfft_rows<M>(in, M, M, 0, t1, l1, st));
    return launch_cols<M, kFwd>(t1, l1, M, 0, (const float2 *)nullptr, out, RowMajor{M / 2 + 1}, M, 0, st);
}

template <int M>
int irfft2_run(const float2 *in, float *out, float2 *t2, cudaStream_t st) {
    const GroupMajor<P<M>::C> l2{M};
    MSN_TRY(launch_cols<M, kInv>(in, RowMajor{M / 2 + 1}, M, 0, (const float2 *)nullptr, t2, l2, M, 0, st));
    return launch_irfft_rows<M>(t2, l2, M, out, M, 0, (float)M * (float)M, st);
}

#define MSN_FFT_INSTANTIATE(M)                                                                                 \
    template int conv_run<M>(const float *, int, const float2 *, float *, int, float2 *, float2 *,            \
                             cudaStream_t, const unsigned char *);                                             \
    template int spectrum_run<M>(const float *, int, int, int, int, float2 *, float2 *, cudaStream_t);        \
    template int rfft2_run<M>(const float *, float2 *, float2 *, cudaStream_t);                               \
    template int irfft2_run<M>(const float2 *, float *, float2 *, cudaStream_t);

}  // namespace fftk
}  // namespace msn
