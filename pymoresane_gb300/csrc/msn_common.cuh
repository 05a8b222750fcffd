// Shared helpers for libmsn: status handling and small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "msn.h"

namespace msn {

// Records a formatted message as the calling thread's last error and returns
// `code`.
int set_error(int code, const char *fmt, ...);
void clear_error();

// Checks the result of a CUDA runtime call / kernel launch.
int check_cuda(cudaError_t e, const char *what);

// Counts every kernel launch of the library (read with msn_launch_count).
void count_launch();

inline int check_launch(const char *what) {
    count_launch();
    return check_cuda(cudaGetLastError(), what);
}

// Programmatic dependent launch (off by default: tuning value graph_pdl; measured
// slower on GB300). While the graph minor loop captures its body with it enabled,
// pdl_flag() is set and the kernels launched with launch_k carry the
// programmatic-serialization attribute: each may be launched while its
// predecessor finishes. Every kernel launched through launch_k starts with
// pdl_wait(), which returns once the predecessor grid has completed and its
// writes are visible (at once for a kernel launched without the attribute),
// then pdl_trigger(), which lets its own successor be launched.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
bool &pdl_flag();  // per host thread (api.cu)

struct PdlScope {
    bool old;
    explicit PdlScope(bool on) : old(pdl_flag()) { pdl_flag() = on; }
    ~PdlScope() { pdl_flag() = old; }
};

template <class... KArgs, class... Args>
int launch_k(const char *what, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
             Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    if (pdl_flag()) {
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    count_launch();
    return check_cuda(cudaLaunchKernelEx(&cfg, kernel, static_cast<Args &&>(args)...), what);
}

// Tunable launch parameters (tune.cu): the current value of a knob, and an
// epoch that changes whenever any knob does.
enum Knob {
    kKnobFourStep = 0,
    kKnobSqFwdCtas,
    kKnobSqColCtas,
    kKnobSqInvCtas,
    kKnobIuwtThreads,      // a trous CTA size for rows of up to 2048 floats
    kKnobIuwtThreadsWide,  // ... for wider rows
    kKnobGraphPdl,         // programmatic dependent launch inside the minor-loop graph
    kKnobCount
};
int tune_value(Knob k);
unsigned tune_epoch();

// The rows of a row-major vector [rows][cols] that may hold non-zero values:
// rows[r] != 0 (null: every row). A pass over the vector skips the float4
// elements of the other rows, where every operand is zero, so each result it
// writes or sums is the dense pass's (a skipped term would add an exact zero).
// cols4 = cols / 4.
struct RowSupport {
    const unsigned char *rows;
    unsigned cols4;
    __device__ __forceinline__ bool active(size_t i4) const {
        return !rows || __ldg(rows + (unsigned)i4 / cols4) != 0;
    }
};

// msn_fft_convolve with the rows of d_x that may be non-zero (rows[r] != 0, null: every row);
// the four-step kernels skip the row transforms of pairs of zero rows (fft.cu).
int fft_convolve_rows(const float *d_x, int n, int m, const void *d_spec, float *d_out, int linear, void *d_work,
                      size_t work_bytes, const unsigned char *rows, cudaStream_t st);

// cg.cu: out[0] = a . b over the rows of a row support (the graph minor loop's p.Ap).
int dot_rows(const float *a, const float *b, size_t n, RowSupport sup, double *out, void *work, size_t work_bytes,
             cudaStream_t st);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// B3 spline taps [1, 4, 6, 4, 1] / 16 (all exact in float32).
constexpr float kB3Outer = 0.0625f;
constexpr float kB3Inner = 0.25f;
constexpr float kB3Centre = 0.375f;

// Half-sample-symmetric mirror of index i into [0, n): x[-k] = x[k-1],
// x[n-1+k] = x[n-k]. Valid for -n <= i < 2n.
__device__ __forceinline__ int mirror(int i, int n) {
    i = (i < 0) ? (-i - 1) : i;
    i = (i >= n) ? (2 * n - i - 1) : i;
    return i;
}

// One 5-tap B3 smoothing sample in the reference kernels' rounding order:
// centre product, then fused multiply-adds for the taps at -2d, -d, +d, +2d.
__device__ __forceinline__ float b3_tap(float xc, float xm2, float xm1, float xp1, float xp2) {
    float acc = __fmul_rn(kB3Centre, xc);
    acc = __fmaf_rn(kB3Outer, xm2, acc);
    acc = __fmaf_rn(kB3Inner, xm1, acc);
    acc = __fmaf_rn(kB3Inner, xp1, acc);
    acc = __fmaf_rn(kB3Outer, xp2, acc);
    return acc;
}

}  // namespace msn

#define MSN_TRY(...)                  \
    do {                              \
        int _msn_rc = (__VA_ARGS__);  \
        if (_msn_rc != MSN_OK) return _msn_rc; \
    } while (0)
