// State block and stop rules of the graph minor loop (pymoresane/main.py:413-455),
// shared by the loop's control kernel (minor_loop.cu) and the fused CG / SNR pass
// that applies the stop rules in its last CTA (cg.cu).
#pragma once

#include <cmath>

#include "msn_common.cuh"

namespace msn {

struct MinorState {
    int minor;            // iterations performed
    int outcome;          // MSN_MINOR_*
    int commit;           // 1: the iteration's xn becomes x
    int miter;            // minor_loop_miter
    int positivity_runs;  // iterations that took the positivity branch
    int pad;
    double snr_current;
    double snr_last;
};

// SNR and the stop rules of main.py:413-455, in the reference's order:
//   minor == 1 and SNR > 40  -> false detection (xn discarded)
//   SNR > 40                 -> converged (xn kept)
//   minor > 2, SNR <= last   -> stalled (xn discarded)
//   minor == minor_loop_miter -> iteration cap (xn kept, loop condition ends)
// One thread; sets the loop's WHILE condition.
__device__ __forceinline__ void minor_control_apply(MinorState *s, const double *snr2, double *hist, int hist_len,
                                                    cudaGraphConditionalHandle h) {
    const double last = s->snr_current;
    const double cur = 20.0 * log10(sqrt(snr2[0]) / sqrt(snr2[1]));
    const int minor = s->minor + 1;
    int outcome = MSN_MINOR_RUNNING, commit = 1;
    if (minor == 1 && cur > 40.0) {
        outcome = MSN_MINOR_FALSE_DETECTION;
        commit = 0;
    } else if (cur > 40.0) {
        outcome = MSN_MINOR_CONVERGED;
    } else if (minor > 2 && cur <= last) {
        outcome = MSN_MINOR_STALLED;
        commit = 0;
    } else if (minor >= s->miter) {
        outcome = MSN_MINOR_ITERATION_CAP;
    }
    s->snr_last = last;
    s->snr_current = cur;
    s->minor = minor;
    s->outcome = outcome;
    s->commit = commit;
    if (minor - 1 < hist_len) hist[minor - 1] = cur;
    cudaGraphSetConditional(h, outcome == MSN_MINOR_RUNNING ? 1u : 0u);
}

// cg.cu: the graph minor loop's pass after p.Ap without positivity -- the CG step on the
// row support (msn_cg_step), the model-source update with the SNR sums
// (msn_snr_update_masked) and, once both are complete, the stop rules above.
int cg_step_snr_rows(const float *x, const float *p, const float *r, const float *ap, double *scal, float *xn,
                     float *rn, size_t n, RowSupport sup, const float *e, float *ms, const float *q, size_t nq,
                     const unsigned char *seg_flags, double *snr2, MinorState *state, double *hist, int hist_len,
                     cudaGraphConditionalHandle h, void *work, size_t work_bytes, cudaStream_t st);

}  // namespace msn
