// Four-step ("square") FFT convolution for M = 64 x 64 = 4096-point grids:
// the linear convolution of an M/2 x M/2 image with an M x M PSF
// (pymoresane/iuwt_convolution.py:18-73, linear branch, double-size PSF).
//
// Each 4096-point transform is one team of 64 threads. Thread t holds the 64
// elements x[t + 64 j] in registers, and a transform is two register passes
// with one shared-memory exchange between them (the four-step / "six-step"
// factorisation of Bailey, "FFTs in external or hierarchical memory", 1990):
//
//   X[k1 + 64 k2] = sum_n1 w64^(n1 k2) * ( w4096^(n1 k1) * sum_n2 x[n1 + 64 n2] w64^(n2 k1) )
//
//   pass A: thread n1 = t forms the inner 64-point DFT over n2 and applies the
//           twiddle w4096^(t k1); the values go to shared memory as [k1][n1];
//   pass B: thread k1 = t reads its row and forms the outer DFT over n1, so
//           it ends up holding X[t + 64 k2] -- the same distribution as the
//           input. An inverse transform of that spectrum therefore starts with
//           its own pass A without any exchange.
//
// A 64-point DFT in registers is an 8 x 8 Cooley-Tukey split with constant
// internal twiddles. With natural input order (slot n) it leaves X[k] in slot
// 8 (k mod 8) + k div 8; with that transposed input order it leaves natural
// output order. Both are free register renamings.
//
// Compared with the three-pass Stockham kernels this halves the shared-memory
// traffic (one exchange per transform instead of two), needs no twiddle table
// in shared memory (the 4096-point twiddles are formed from 14 loads of the
// float64-accurate table per pass), and synchronises only the two warps of a
// team (named barriers).
//
// The three kernels of one convolution (n = M/2, linear):
//   1. sq_rows_fwd: two real image rows packed as z = a + i b, zero-padded to
//      M (the image occupies sequence positions [M/4, 3M/4)), transformed; the
//      spectrum Z[k] is stored as two planes: lo[k] = Z[k] (k <= M/2) and
//      hi[k] = Z[(M - k) mod M] (k <= M/2), so that column k finds both
//      Hermitian partners in the same place.
//   2. sq_cols_conv: per spectrum column k <= M/2 the real rows' spectra are
//      split off (Xa = (Z[k] + conj Z[M-k]) / 2, Xb = (Z[k] - conj Z[M-k]) / 2i),
//      transformed along the column, multiplied by the PSF spectrum, inverse
//      transformed, and only the rows that survive the fft-shift and centre
//      crop are kept, re-packed in pairs as the Hermitian-extended rows of the
//      inverse real transform (written in place over lo / hi).
//   3. sq_rows_inv: each packed row pair is inverse transformed; the real and
//      imaginary parts are the two output rows, divided by M^2 (scale_fft,
//      :242-265) and written through the shift and crop (:161-239).
// Planes lo / hi are group-major [ceil(W/2)][n/2][2] (W = M/2 + 1): the two
// columns of a group are the two teams of one column-kernel CTA, so every
// 32-byte sector a CTA reads or writes is used in full by that CTA.
#pragma once

#include <utility>

#include <cuda.h>

#include "fft_core.cuh"
#include "msn_common.cuh"

namespace msn {
namespace fftk {
namespace sq {

constexpr int R = 64;              // points per register pass (= threads per team)
constexpr int M = R * R;           // transform length
constexpr int HALF = M / 2;        // image side and Nyquist index
constexpr int W = HALF + 1;        // spectrum columns
constexpr int PADR = R + 1;        // padded row of the exchange buffer (conflict-free both ways)
constexpr int SEQ = R * PADR;      // float2 per team exchange buffer
constexpr int TEAMS = 2;           // teams per CTA (= columns per group)
constexpr int J0 = R / 4, J1 = 3 * R / 4;  // register index range of the image within the padded row
constexpr int PAIRS = HALF / 2;    // row pairs of the n = M/2 image
constexpr int ZCOL = 2 * PAIRS;    // float2 between spectrum columns k and k + 2 in a plane

// sin(2 pi m / 64) for m = 0..16, float32-rounded from float64.
__host__ __device__ constexpr float sin64q(int m) {
    constexpr float s[17] = {0.0f,         0.0980171412f, 0.195090324f, 0.290284663f, 0.382683426f, 0.471396744f,
                             0.555570245f, 0.634393275f,  0.707106769f, 0.773010433f, 0.831469595f, 0.881921291f,
                             0.923879504f, 0.956940353f,  0.980785251f, 0.99518472f,  1.0f};
    return s[m];
}
// (cos, sin)(2 pi e / 64)
__host__ __device__ constexpr float2 cs64(int e) {
    e &= 63;
    const int q = e / 16, r = e % 16;
    const float c = sin64q(16 - r), s = sin64q(r);
    return q == 0 ? float2{c, s} : q == 1 ? float2{-s, c} : q == 2 ? float2{-c, -s} : float2{s, -c};
}

// a * w64^(+-E): forward uses exp(-2 pi i E / 64), inverse its conjugate.
template <bool INV, int E>
__host__ __device__ __forceinline__ float2 mul_w64(float2 a) {
    constexpr int e = E & 63;
    if constexpr (e == 0) {
        return a;
    } else if constexpr (e == 16) {
        return rot90<INV>(a);
    } else if constexpr (e == 32) {
        return make_float2(-a.x, -a.y);
    } else if constexpr (e == 48) {
        return rot90<!INV>(a);
    } else {
        constexpr float2 w = cs64(e);
        // forward: (a.x + i a.y)(c - i s); inverse: (a.x + i a.y)(c + i s)
        return INV ? make_float2(a.x * w.x - a.y * w.y, a.y * w.x + a.x * w.y)
                   : make_float2(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
    }
}

// 8-point DFT of v[O + S i], i = 0..7, natural order in and out.
template <bool INV, int O, int S>
__host__ __device__ __forceinline__ void dft8s(float2 *v) {
    float2 t[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) t[i] = v[O + S * i];
    dft8<INV>(t);
#pragma unroll
    for (int i = 0; i < 8; ++i) v[O + S * i] = t[i];
}

template <int N, class F>
__host__ __device__ __forceinline__ void unroll(F &&f) {
    [&]<int... I>(std::integer_sequence<int, I...>) { (f(std::integral_constant<int, I>{}), ...); }
    (std::make_integer_sequence<int, N>{});
}

// Register slot of element k of a 64-sequence in transposed order.
__host__ __device__ constexpr int tslot(int k) { return 8 * (k & 7) + (k >> 3); }

// 64-point DFT in registers (unnormalised). TIN = false: input v[n] in slot n,
// output X[k] in slot tslot(k). TIN = true: input in slot tslot(n), output in
// slot k.
template <bool INV, bool TIN>
__host__ __device__ __forceinline__ void dft64(float2 *v) {
    if constexpr (!TIN) {
        // n = a + 8 b: DFT over b for each a, twiddle w64^(a k_lo), DFT over a for each k_lo
        unroll<8>([&](auto a) { dft8s<INV, decltype(a)::value, 8>(v); });
        unroll<8>([&](auto a) {
            unroll<8>([&](auto b) {
                constexpr int A = decltype(a)::value, B = decltype(b)::value;
                v[A + 8 * B] = mul_w64<INV, A * B>(v[A + 8 * B]);
            });
        });
        unroll<8>([&](auto b) { dft8s<INV, 8 * decltype(b)::value, 1>(v); });
    } else {
        // n = a + 8 b sits in slot 8 a + b
        unroll<8>([&](auto a) { dft8s<INV, 8 * decltype(a)::value, 1>(v); });
        unroll<8>([&](auto a) {
            unroll<8>([&](auto b) {
                constexpr int A = decltype(a)::value, B = decltype(b)::value;
                v[8 * A + B] = mul_w64<INV, A * B>(v[8 * A + B]);
            });
        });
        unroll<8>([&](auto b) { dft8s<INV, decltype(b)::value, 8>(v); });
    }
}

#ifndef MSN_HOST_ONLY
// w4096^(m) from the float64-rounded table of fft_core.cuh.
__device__ __forceinline__ float2 w4096(int m) { return __ldg(&kTwiddle[(m & (M - 1)) * (kTwN / M)]); }
#endif

// Multiplies element k1 (k1 = a + 8 b) of a thread's 64-sequence by
// w4096^(+-t k1); TSLOT: the sequence is in transposed slot order. The twiddle
// is w^(t a) * w^(8 t b), both factors correctly rounded table entries
// (wtab(m) returns w4096^m).
template <bool INV, bool TSLOT, class WA, class WB>
__host__ __device__ __forceinline__ void twiddle_ab(float2 *v, WA wa_of, WB wb_of) {
    float2 wa[8];
#pragma unroll
    for (int i = 1; i < 8; ++i) wa[i] = wa_of(i);
    unroll<8>([&](auto bc) {
        constexpr int B = decltype(bc)::value;
        const float2 wb = B == 0 ? make_float2(1.0f, 0.0f) : wb_of(B);
        unroll<8>([&](auto ac) {
            constexpr int A = decltype(ac)::value;
            if constexpr (A != 0 || B != 0) {
                float2 w = A == 0 ? wb : (B == 0 ? wa[A] : cmul(wa[A], wb));
                if (INV) w = cconj(w);
                constexpr int slot = TSLOT ? 8 * A + B : A + 8 * B;
                v[slot] = cmul(v[slot], w);
            }
        });
    });
}

// twiddle_ab with the factors read from a table: wtab(m) returns w4096^m.
template <bool INV, bool TSLOT, class Wtab>
__host__ __device__ __forceinline__ void twiddle_t(float2 *v, int t, Wtab wtab) {
    twiddle_ab<INV, TSLOT>(v, [&](int i) { return wtab(t * i); }, [&](int i) { return wtab(8 * t * i); });
}

// Per-thread twiddle factors in shared memory: tab[(i - 1) * 64 + t] = w^(t i) and
// tab[(6 + i) * 64 + t] = w^(8 t i), i = 1..7 (7 KB, read conflict-free).
constexpr int kTabElems = 14 * R;

template <bool INV, bool TSLOT>
__host__ __device__ __forceinline__ void twiddle_tab(float2 *v, const float2 *tab, int t) {
    twiddle_ab<INV, TSLOT>(v, [&](int i) { return tab[(i - 1) * R + t]; },
                           [&](int i) { return tab[(6 + i) * R + t]; });
}

#ifdef MSN_SQ_KERNELS  // the kernels are compiled in fft_sq.cu only
struct W4096 {
    __device__ __forceinline__ float2 operator()(int m) const { return w4096(m); }
};

// Fills the per-thread twiddle table (threads t < 64 of the CTA; caller synchronises).
__device__ __forceinline__ void fill_tab(float2 *tab) {
    const int t = threadIdx.x;
    if (t < R) {
#pragma unroll
        for (int i = 1; i < 8; ++i) {
            tab[(i - 1) * R + t] = w4096(t * i);
            tab[(6 + i) * R + t] = w4096(8 * t * i);
        }
    }
}

__device__ __forceinline__ void team_sync(int team) {
    asm volatile("bar.sync %0, %1;\n" ::"r"(team + 1), "r"(R) : "memory");
}

// Pass A twiddle + exchange + pass B of a transform whose pass-A DFT has run:
// TSLOT tells the slot order pass A left (transposed for natural input).
// On return thread t holds X[t + 64 k2] in slot tslot(k2).
template <bool INV, bool TSLOT>
__device__ __forceinline__ void exchange_and_pass_b(float2 *v, float2 *buf, int t, int team) {
    twiddle_t<INV, TSLOT>(v, t, W4096{});
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) buf[k1 * PADR + t] = v[TSLOT ? tslot(k1) : k1];
    team_sync(team);
#pragma unroll
    for (int n1 = 0; n1 < R; ++n1) v[n1] = buf[t * PADR + n1];
    team_sync(team);  // the buffer is free for the team's next exchange
    dft64<INV, false>(v);
}

// ---------------------------------------------------------------------------
// Bulk asynchronous copies (the TMA engine's 1-D form) and mbarriers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Global -> shared bulk copy completing on an mbarrier (16-byte aligned, size a multiple of 16).
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// Shared -> global bulk copy (bulk-group completion).
__device__ __forceinline__ void bulk_store(void *dst, const void *src, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst), "r"(smem_addr(src)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(src), "r"(bytes) : "memory");
}
// Orders this thread's generic-proxy shared-memory accesses with later async-proxy (bulk copy) ones.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// Tiled 3-D tensor copies (TMA) through a CUtensorMap kernel parameter.
__device__ __forceinline__ void tensor_load3(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void tensor_store3(const CUtensorMap *map, int x, int y, int z, const void *src) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];\n" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(z), "r"(smem_addr(src))
                 : "memory");
}

// Set when a bounded wait in these kernels gives up (read with msn_fft_status).
__device__ unsigned g_sq_status;
constexpr unsigned kSqWaitTimeout = 1u;
constexpr long kSqSpinLimit = 1L << 24;   // polls of about 0.1-1 us each: well over a second

// Waits for the phase `parity` of an mbarrier to complete; false (and the status
// word set) if it has not completed after kSqSpinLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    for (long i = 0; i < kSqSpinLimit; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if (i > 64) __nanosleep(64);
    }
    atomicOr(&g_sq_status, kSqWaitTimeout);
    return false;
}

// Index of spectrum column k, row pair p in a group-major plane [ceil(W/2)][PAIRS][2].
__device__ __forceinline__ int zidx(int k, int p) { return ((k >> 1) * PAIRS + p) * 2 + (k & 1); }

// Row pair p of a plane as TMA boxes: the plane is the 3-D tensor
// {4 floats (columns 2g, 2g+1 of pair p), PAIRS, G} and one box is
// {4, 1, kBoxG} = 16 B x kBoxG groups; kBoxes boxes cover the G = 1025 groups.
// In shared memory a pair's row of a plane is kBoxes box slots of kBoxSlot bytes.
constexpr int kBoxG = 205;
constexpr int kBoxes = 5;
constexpr unsigned kBoxBytes = kBoxG * 16;                 // 3280
constexpr unsigned kBoxSlot = (kBoxBytes + 127) / 128 * 128;  // 3328: 128-byte aligned slots
constexpr unsigned kRowSlots = kBoxes * kBoxSlot;          // 16,640 bytes per plane row
static_assert(kBoxG * kBoxes == (W + 1) / 2, "boxes must tile the groups exactly");
static_assert(2 * kRowSlots <= SEQ * sizeof(float2), "a pair's lo and hi rows fit in one exchange buffer");

// Byte offset of spectrum column k of a pair's row within its box slots.
__device__ __forceinline__ unsigned slot_off(int k) {
    const int g = k >> 1;
    return (unsigned)(g / kBoxG) * kBoxSlot + (unsigned)(g % kBoxG) * 16u + (unsigned)(k & 1) * 8u;
}

constexpr unsigned kRowInBytes = 2 * HALF * sizeof(float);  // two image rows, 16 KB
constexpr size_t kTeamArea = SEQ * sizeof(float2);          // 33,280
constexpr size_t kRowFwdSmem = kTeamArea + kRowInBytes + 16;

// 1. Forward row transforms of image rows 2p, 2p + 1 (n = M/2 columns placed at
// [M/4, 3M/4) of the padded row). Persistent one-team CTAs; the next pair's two
// rows are bulk-copied into IN while the current pair is transformed, and the
// spectrum rows leave through TMA tensor stores from box slots in the exchange
// buffer (lo[k] = Z[k] for k <= M/2, hi[c] = Z[(M - c) mod M] for c <= M/2).
//
// rows (may be null) flags the image rows that may be non-zero. A pair of zero
// rows has a zero spectrum: its lo / hi rows are stored as zeros without a
// transform (the transform of zeros gives zeros, up to the sign of zero). The
// pairs are then taken from a work list with the pairs that need a transform
// first, so that those spread evenly over the CTAs.
constexpr int kPairsPerThread = PAIRS / R;
static_assert(kPairsPerThread * R == PAIRS && kPairsPerThread <= 32, "work-list scan: whole pairs per thread");

__global__ void __launch_bounds__(R, 4)
sq_rows_fwd(const float *__restrict__ x, const __grid_constant__ CUtensorMap lo_map,
            const __grid_constant__ CUtensorMap hi_map, const unsigned char *__restrict__ rows) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ __align__(128) float2 smem[];
    const int t = threadIdx.x;
    const bool leader = t == 0;
    float2 *buf = smem;
    char *out_lo = reinterpret_cast<char *>(smem), *out_hi = out_lo + kRowSlots;
    const float *in_a = reinterpret_cast<const float *>(reinterpret_cast<char *>(smem) + kTeamArea);
    const float *in_b = in_a + HALF;
    uint64_t *bar = reinterpret_cast<uint64_t *>(reinterpret_cast<char *>(smem) + kTeamArea + kRowInBytes);
    __shared__ int ok;
    __shared__ unsigned short order[PAIRS];
    __shared__ int warp_total[R / 32];
    if (leader) {
        mbar_init(bar, 1);
        mbar_init_fence();
    }
    // work list: item i is pair order[i]; items [0, n_work) need a transform
    int n_work = PAIRS;
    if (rows) {
        unsigned m = 0;
#pragma unroll
        for (int k = 0; k < kPairsPerThread; ++k) {
            const int pp = kPairsPerThread * t + k;
            if (__ldg(rows + 2 * pp) | __ldg(rows + 2 * pp + 1)) m |= 1u << k;
        }
        const int c = __popc(m);
        int inc = c;  // inclusive scan over the warp
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, off);
            if ((t & 31) >= off) inc += y;
        }
        if ((t & 31) == 31) warp_total[t >> 5] = inc;
        __syncthreads();
        int before = inc - c;
        n_work = 0;
#pragma unroll
        for (int w = 0; w < R / 32; ++w) {
            if (w < (t >> 5)) before += warp_total[w];
            n_work += warp_total[w];
        }
        int a = before, z = n_work + (kPairsPerThread * t - before);
#pragma unroll
        for (int k = 0; k < kPairsPerThread; ++k) {
            const int pp = kPairsPerThread * t + k;
            if ((m >> k) & 1u)
                order[a++] = (unsigned short)pp;
            else
                order[z++] = (unsigned short)pp;
        }
    }
    __syncthreads();
    auto pair_of = [&](int item) { return rows ? (int)order[item] : item; };
    int item = blockIdx.x;
    if (leader && item < n_work) {
        mbar_expect_tx(bar, kRowInBytes);
        bulk_load((void *)in_a, x + (size_t)(2 * pair_of(item)) * HALF, kRowInBytes, bar);
    }
    unsigned parity = 0;
    for (; item < PAIRS; item += gridDim.x) {
        const int p = pair_of(item);
        if (item >= n_work) {
            // a pair of zero rows: zero spectrum rows (the items of a CTA that need a
            // transform all come before its zero items, so no input copy is pending)
            if (leader) bulk_wait_read_all();  // the previous pair's spectrum rows have left the area
            __syncthreads();
            float4 *z4 = reinterpret_cast<float4 *>(smem);
            for (int k = t; k < (int)(2 * kRowSlots / 16); k += R) z4[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            if (leader) ok = mbar_wait(bar, parity);
            __syncthreads();
            if (!ok) {
                if (leader) mbar_wait(bar, parity);
                break;
            }
            if (!leader) mbar_wait(bar, parity);
            parity ^= 1u;
            float2 v[R];
#pragma unroll
            for (int j = 0; j < R; ++j)
                v[j] = (j >= J0 && j < J1) ? make_float2(in_a[t + R * (j - J0)], in_b[t + R * (j - J0)])
                                           : make_float2(0.0f, 0.0f);
            if (leader) bulk_wait_read_all();  // the previous pair's spectrum rows have left the area
            __syncthreads();                   // IN consumed
            const int in_next = item + gridDim.x;
            if (leader && in_next < n_work) {
                fence_proxy_async();
                mbar_expect_tx(bar, kRowInBytes);
                bulk_load((void *)in_a, x + (size_t)(2 * pair_of(in_next)) * HALF, kRowInBytes, bar);
            }
            dft64<false, false>(v);
            twiddle_t<false, true>(v, t, W4096{});
#pragma unroll
            for (int k1 = 0; k1 < R; ++k1) buf[k1 * PADR + t] = v[tslot(k1)];
            __syncthreads();
#pragma unroll
            for (int n1 = 0; n1 < R; ++n1) v[n1] = buf[t * PADR + n1];
            __syncthreads();
            dft64<false, false>(v);  // Z[t + 64 k2] in slot tslot(k2)
#pragma unroll
            for (int k2 = 0; k2 < R; ++k2) {
                const int k = t + R * k2;
                const float2 z = v[tslot(k2)];
                if (k <= HALF) *reinterpret_cast<float2 *>(out_lo + slot_off(k)) = z;
                if (k >= HALF) *reinterpret_cast<float2 *>(out_hi + slot_off(M - k)) = z;
                if (k == 0) *reinterpret_cast<float2 *>(out_hi) = z;
            }
        }
        fence_proxy_async();
        __syncthreads();
        if (leader) {
#pragma unroll
            for (int b = 0; b < kBoxes; ++b) {
                tensor_store3(&lo_map, 0, p, b * kBoxG, out_lo + b * kBoxSlot);
                tensor_store3(&hi_map, 0, p, b * kBoxG, out_hi + b * kBoxSlot);
            }
            bulk_commit();
        }
    }
    if (leader) bulk_wait_all();
}

// 2. Column group g (spectrum columns 2g, 2g + 1; one team each): forward column
// transforms, product with the PSF spectrum h (packed group-major
// [ceil(W/2)][M][2]), inverse column transforms; the kept rows are written back
// over the group's lo / hi blocks as packed pairs.
//
// Persistent CTAs walk the groups g = blockIdx.x, + gridDim.x, ... A group's
// lo and hi blocks are contiguous 16 KB blocks ([PAIRS][2] float2), so they move
// as bulk copies: the next group's blocks are copied into shared memory while
// the current group's inverse transforms and output run, and the output blocks
// leave from shared memory as bulk stores. The group's 64 KB PSF-spectrum block
// is prefetched into L2 one group ahead and read with ordinary loads.
// Shared memory: AREA = the two teams' exchange buffers; IN = AREA[0, 32 KB)
// (lo block, hi block) and OUT = AREA[32 KB, 64 KB) are disjoint.
constexpr unsigned kBlockBytes = PAIRS * 2 * sizeof(float2);   // 16 KB
constexpr size_t kAreaBytes = (size_t)TEAMS * SEQ * sizeof(float2);
static_assert(4 * kBlockBytes <= kAreaBytes, "IN and OUT must fit in the exchange area");

__global__ void __launch_bounds__(R * TEAMS, 3)
sq_cols_conv(float2 *lo, float2 *hi, const float2 *__restrict__ h) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ __align__(128) float2 smem[];
    constexpr int G = (W + 1) / 2;
    constexpr unsigned kHBytes = M * 2 * sizeof(float2);  // a group's PSF-spectrum block, 64 KB
    static_assert(kHBytes <= kAreaBytes, "the PSF block must fit in the exchange area");
    const int team = threadIdx.x / R, t = threadIdx.x % R;
    const bool leader = threadIdx.x == 0;
    float2 *buf = smem + team * SEQ;
    float2 *in_lo = smem, *in_hi = smem + PAIRS * 2;
    float2 *out_lo = smem + 2 * PAIRS * 2, *out_hi = smem + 3 * PAIRS * 2;
    const float2 *h_s = smem;
    uint64_t *bar_in = reinterpret_cast<uint64_t *>(reinterpret_cast<char *>(smem) + kAreaBytes);
    uint64_t *bar_h = bar_in + 1;
    float2 *tab = reinterpret_cast<float2 *>(bar_in + 2);
    __shared__ int ok;
    if (leader) {
        mbar_init(bar_in, 1);
        mbar_init(bar_h, 1);
        mbar_init_fence();
    }
    fill_tab(tab);
    __syncthreads();
    int g = blockIdx.x;
    if (leader && g < G) {
        mbar_expect_tx(bar_in, 2 * kBlockBytes);
        bulk_load(in_lo, lo + (size_t)g * PAIRS * 2, kBlockBytes, bar_in);
        bulk_load(in_hi, hi + (size_t)g * PAIRS * 2, kBlockBytes, bar_in);
        bulk_prefetch_l2(h + (size_t)g * M * 2, kHBytes);
    }
    // Every thread observes a completed phase after one bounded wait by the leader.
    auto wait_all = [&](uint64_t *bar, unsigned parity) -> bool {
        if (leader) ok = mbar_wait(bar, parity);
        __syncthreads();
        if (!ok) {
            if (leader) mbar_wait(bar, parity);  // a last bounded wait for the copies in flight
            return false;
        }
        if (!leader) mbar_wait(bar, parity);
        return true;
    };
    const bool odd = t & 1;
    const int c = team;
    unsigned parity = 0;
    for (; g < G; g += gridDim.x) {
        const int k = 2 * g + c;
        const int gn = g + gridDim.x;
        if (!wait_all(bar_in, parity)) break;
        float2 v[R];
        // sequence position t + 64 j is image row r = t + 64 (j - J0): pair r / 2,
        // Xa (even rows) or Xb (odd rows) from the two Hermitian partners
#pragma unroll
        for (int j = 0; j < R; ++j) {
            if (j >= J0 && j < J1) {
                const int at = ((t >> 1) + (R / 2) * (j - J0)) * 2 + c;
                const float2 a = in_lo[at], b = in_hi[at];
                v[j] = odd ? make_float2(0.5f * (a.y + b.y), -0.5f * (a.x - b.x))
                           : make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
            } else {
                v[j] = make_float2(0.0f, 0.0f);
            }
        }
        if (leader) {
            if (gn < G) bulk_prefetch_l2(h + (size_t)gn * M * 2, kHBytes);
            bulk_wait_read_all();  // the previous group's output has left OUT
        }
        __syncthreads();  // IN consumed, OUT free: the area becomes the exchange buffers
        // Two runs of one forward transform body (natural order in and out): the forward
        // column transform, then -- on the conjugated product -- the inverse one, since
        // IDFT(y) = conj(DFT(conj(y))).
        bool fail = false;
#pragma unroll 1
        for (int it = 0; it < 2; ++it) {
            dft64<false, false>(v);
            twiddle_tab<false, true>(v, tab, t);
#pragma unroll
            for (int k1 = 0; k1 < R; ++k1) buf[k1 * PADR + t] = v[tslot(k1)];
            team_sync(team);
#pragma unroll
            for (int n1 = 0; n1 < R; ++n1) v[n1] = buf[t * PADR + n1];
            __syncthreads();  // both teams have read their exchange
            if (leader) {
                fence_proxy_async();
                if (it == 0) {
                    mbar_expect_tx(bar_h, kHBytes);
                    bulk_load(smem, h + (size_t)g * M * 2, kHBytes, bar_h);
                } else if (gn < G) {
                    mbar_expect_tx(bar_in, 2 * kBlockBytes);
                    bulk_load(in_lo, lo + (size_t)gn * PAIRS * 2, kBlockBytes, bar_in);
                    bulk_load(in_hi, hi + (size_t)gn * PAIRS * 2, kBlockBytes, bar_in);
                }
            }
            dft64<false, false>(v);  // thread t now holds X[t + 64 k2] in slot tslot(k2)
            if (it == 0) {
                if (!wait_all(bar_h, parity)) {
                    fail = true;
                    break;
                }
                // conj(X * H), with H for row m = t + 64 k2 of this column, written in natural
                // order (slot k2): the inverse pass A takes its input in natural order, so one
                // transform body serves all four passes
                float2 u[R];
#pragma unroll
                for (int k2 = 0; k2 < R; ++k2) {
                    const float2 hv = h_s[(t + R * k2) * 2 + c];
                    const float2 x = v[tslot(k2)];
                    u[k2] = make_float2(x.x * hv.x - x.y * hv.y, -(x.x * hv.y + x.y * hv.x));
                }
#pragma unroll
                for (int k2 = 0; k2 < R; ++k2) v[k2] = u[k2];
                __syncthreads();  // the PSF block is consumed: the area is the exchange again
            }
        }
        if (fail) break;
        parity ^= 1u;
        // v holds conj(y) in slot tslot(k2) for y the inverse column transform; position n = t + 64 k2 is
        // output row i = (n - 3M/4) mod M; rows i < M/2 are kept:
        // i = t + 64 (k2 - 48) for k2 >= 48 and t + 64 k2 + M/4 for k2 < 16, pair i / 2
        const bool edge = k == 0 || k == HALF;  // c2r uses only the real part of these bins
#pragma unroll
        for (int k2 = 0; k2 < R; ++k2) {
            if (k2 >= J0 && k2 < J1) continue;
            const int at = ((t >> 1) + (R / 2) * (k2 >= J1 ? k2 - J1 : k2 + J0)) * 2 + c;
            float2 own = make_float2(v[tslot(k2)].x, -v[tslot(k2)].y);
            float2 other;
            other.x = __shfl_xor_sync(0xffffffffu, own.x, 1);
            other.y = __shfl_xor_sync(0xffffffffu, own.y, 1);
            if (edge) {
                own.y = 0.0f;
                other.y = 0.0f;
            }
            const float2 a = odd ? other : own, b = odd ? own : other;  // rows 2p', 2p' + 1
            if (odd) {
                out_hi[at] = make_float2(a.x + b.y, b.x - a.y);  // conj(a) + i conj(b): column M - k
            } else {
                out_lo[at] = make_float2(a.x - b.y, a.y + b.x);  // a + i b
            }
        }
        fence_proxy_async();
        __syncthreads();
        if (leader) {
            bulk_store(lo + (size_t)g * PAIRS * 2, out_lo, kBlockBytes);
            bulk_store(hi + (size_t)g * PAIRS * 2, out_hi, kBlockBytes);
            bulk_commit();
        }
    }
    if (leader) bulk_wait_all();
}

// 3. Inverse row transforms of the packed pairs; writes rows 2p, 2p + 1 of the
// n x n output (columns through the shift and crop), scaled by 1 / M^2.
// Persistent one-team CTAs. A pair's lo and hi rows arrive by TMA tensor loads
// into the exchange buffer; once the exchange has been read, the next pair's rows
// are loaded there while the current pair's second pass runs. The two output rows
// (16 KB, contiguous) leave as one bulk store from a buffer of their own.
constexpr unsigned kRowOutBytes = 2 * HALF * sizeof(float);
constexpr size_t kRowInvSmem = kTeamArea + kRowOutBytes + 16 + kTabElems * sizeof(float2);
static_assert(2 * kRowSlots <= kTeamArea, "a pair's lo and hi rows fit in the exchange buffer");

__global__ void __launch_bounds__(R, 4)
sq_rows_inv(const __grid_constant__ CUtensorMap lo_map, const __grid_constant__ CUtensorMap hi_map,
            float *__restrict__ out) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ __align__(128) float2 smem[];
    const int t = threadIdx.x;
    const bool leader = t == 0;
    float2 *buf = smem;
    char *in_lo = reinterpret_cast<char *>(smem), *in_hi = in_lo + kRowSlots;
    float *out_s = reinterpret_cast<float *>(reinterpret_cast<char *>(smem) + kTeamArea);
    uint64_t *bar = reinterpret_cast<uint64_t *>(reinterpret_cast<char *>(smem) + kTeamArea + kRowOutBytes);
    float2 *tab = reinterpret_cast<float2 *>(bar + 2);
    __shared__ int ok;
    if (leader) {
        mbar_init(bar, 1);
        mbar_init_fence();
    }
    fill_tab(tab);
    __syncthreads();
    auto issue = [&](int pp) {
        mbar_expect_tx(bar, 2 * kBoxes * kBoxBytes);
#pragma unroll
        for (int b = 0; b < kBoxes; ++b) {
            tensor_load3(in_lo + b * kBoxSlot, &lo_map, 0, pp, b * kBoxG, bar);
            tensor_load3(in_hi + b * kBoxSlot, &hi_map, 0, pp, b * kBoxG, bar);
        }
    };
    int p = blockIdx.x;
    if (leader && p < PAIRS) issue(p);
    unsigned parity = 0;
    for (; p < PAIRS; p += gridDim.x) {
        if (leader) ok = mbar_wait(bar, parity);
        __syncthreads();
        if (!ok) {
            if (leader) mbar_wait(bar, parity);
            break;
        }
        if (!leader) mbar_wait(bar, parity);
        parity ^= 1u;
        float2 v[R];
        // n = t + 64 j: lo[n] for n < M/2, hi[M - n] otherwise
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const int n = t + R * j;
            v[j] = j < R / 2 ? *reinterpret_cast<const float2 *>(in_lo + slot_off(n))
                             : *reinterpret_cast<const float2 *>(in_hi + slot_off(M - n));
        }
        if (leader) bulk_wait_read_all();  // the previous pair's output rows have left OUT
        __syncthreads();                   // IN consumed: the buffer becomes the exchange
        dft64<true, false>(v);
        twiddle_tab<true, true>(v, tab, t);
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) buf[k1 * PADR + t] = v[tslot(k1)];
        __syncthreads();
#pragma unroll
        for (int n1 = 0; n1 < R; ++n1) v[n1] = buf[t * PADR + n1];
        __syncthreads();                   // the exchange is read: the next pair's rows may land
        const int pn = p + gridDim.x;
        if (leader && pn < PAIRS) {
            fence_proxy_async();
            issue(pn);
        }
        dft64<true, false>(v);  // z[t + 64 k2] in slot tslot(k2)
        constexpr float scale = 1.0f / ((float)M * (float)M);  // a power of two: exact
#pragma unroll
        for (int k2 = 0; k2 < R; ++k2) {
            if (k2 >= J0 && k2 < J1) continue;
            const int c = t + R * (k2 >= J1 ? k2 - J1 : k2 + J0);
            out_s[c] = v[tslot(k2)].x * scale;
            out_s[HALF + c] = v[tslot(k2)].y * scale;
        }
        fence_proxy_async();
        __syncthreads();
        if (leader) {
            bulk_store(out + (size_t)(2 * p) * HALF, out_s, kRowOutBytes);
            bulk_commit();
        }
    }
    if (leader) bulk_wait_all();
}

constexpr size_t kColSmem = kAreaBytes + 16 + kTabElems * sizeof(float2);  // + two mbarriers + twiddles
constexpr size_t kPlaneElems = (size_t)((W + 1) / 2) * PAIRS * 2;

// Encodes the 3-D tensor map of a lo / hi plane: {4 floats, PAIRS, G} with
// strides 16 B and PAIRS * 16 B, boxes {4, 1, kBoxG} (fft_sq.cu).
int plane_map(CUtensorMap *map, void *base);

struct SqLaunch {
    int fwd_grid = 0, col_grid = 0, inv_grid = 0;
};

// Persistent grids: resident CTAs per SM (the occupancy limit, or fewer when a
// tuned value asks for it) x SMs; resolved once per device and tuning epoch.
inline int launch_config(SqLaunch *cfg) {
    static SqLaunch cached[64];
    static unsigned cached_epoch[64];
    int dev = 0;
    MSN_TRY(check_cuda(cudaGetDevice(&dev), "cudaGetDevice"));
    const unsigned epoch = tune_epoch();
    if (dev >= 0 && dev < 64 && cached[dev].col_grid > 0 && cached_epoch[dev] == epoch) {
        *cfg = cached[dev];
        return MSN_OK;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
    auto grid_of = [&](const void *fn, int threads, size_t smem, int items, Knob knob) {
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
        if (per_sm < 1) per_sm = 1;
        const int want = tune_value(knob);
        if (want > 0 && want < per_sm) per_sm = want;
        const int g = per_sm * sms;
        return g < items ? g : items;
    };
    SqLaunch c;
    c.fwd_grid = grid_of((const void *)sq_rows_fwd, R, kRowFwdSmem, PAIRS, kKnobSqFwdCtas);
    c.col_grid = grid_of((const void *)sq_cols_conv, R * TEAMS, kColSmem, (W + 1) / 2, kKnobSqColCtas);
    c.inv_grid = grid_of((const void *)sq_rows_inv, R, kRowInvSmem, PAIRS, kKnobSqInvCtas);
    if (dev >= 0 && dev < 64) {
        cached[dev] = c;
        cached_epoch[dev] = epoch;
    }
    *cfg = c;
    return MSN_OK;
}

int conv_run(const float *x, const float2 *spec, float *out, float2 *lo, float2 *hi, cudaStream_t st,
             const unsigned char *rows) {
    SqLaunch cfg;
    MSN_TRY(launch_config(&cfg));
    CUtensorMap lo_map, hi_map;
    MSN_TRY(plane_map(&lo_map, lo));
    MSN_TRY(plane_map(&hi_map, hi));
    MSN_TRY(launch_k("sq_rows_fwd", sq_rows_fwd, cfg.fwd_grid, R, kRowFwdSmem, st, x, lo_map, hi_map, rows));
    MSN_TRY(launch_k("sq_cols_conv", sq_cols_conv, cfg.col_grid, R * TEAMS, kColSmem, st, lo, hi, spec));
    return launch_k("sq_rows_inv", sq_rows_inv, cfg.inv_grid, R, kRowInvSmem, st, lo_map, hi_map, out);
}

#endif  // MSN_SQ_KERNELS

}  // namespace sq
}  // namespace fftk
}  // namespace msn
