// Tunable launch parameters of the library's kernels. The values are chosen
// per device by the project's autotuner (pymoresane_gb300/tune.py, which
// times the alternatives and caches the winners) and set through
// msn_tune_set; every launch reads the current value. Changing a value bumps
// an epoch that invalidates the minor-loop graphs captured with the old one.
#include <atomic>
#include <cstring>

#include "msn_common.cuh"

namespace msn {

namespace {

struct KnobSpec {
    const char *name;
    int def;
    int lo, hi;   // allowed range
    int pow2;     // value must be a power of two
};

// Order follows the Knob enum in msn_common.cuh.
constexpr KnobSpec kSpecs[kKnobCount] = {
    {"fft_four_step", 1, 0, 1, 0},     // 4096-point linear convolution: four-step (1) or Stockham (0) kernels
    {"fft_sq_fwd_ctas", 0, 0, 8, 0},   // resident CTAs per SM of the four-step row kernels (0: as many as fit)
    {"fft_sq_col_ctas", 0, 0, 8, 0},   // ... of the four-step column kernel
    {"fft_sq_inv_ctas", 0, 0, 8, 0},   // ... of the four-step inverse row kernel
    {"iuwt_threads", 256, 64, 256, 1},      // threads per CTA of the a trous passes, rows of <= 2048 floats
    {"iuwt_threads_wide", 256, 64, 256, 1}, // ... rows of more than 2048 floats
    {"graph_pdl", 0, 0, 1, 0},         // programmatic dependent launch between the minor-loop graph's kernels
                                       // (measured slower on GB300: 600 against 516 ms per 2048^2 deconvolution)
};

std::atomic<int> g_values[kKnobCount] = {{1}, {0}, {0}, {0}, {256}, {256}, {0}};
std::atomic<unsigned> g_epoch{0};

int find(const char *name) {
    if (!name) return -1;
    for (int k = 0; k < kKnobCount; ++k)
        if (std::strcmp(kSpecs[k].name, name) == 0) return k;
    return -1;
}

}  // namespace

int tune_value(Knob k) { return g_values[k].load(std::memory_order_relaxed); }
unsigned tune_epoch() { return g_epoch.load(std::memory_order_relaxed); }

}  // namespace msn

using namespace msn;

extern "C" int msn_tune_set(const char *name, int value) {
    clear_error();
    const int k = find(name);
    if (k < 0) return set_error(MSN_ERR_INVALID, "msn_tune_set: unknown parameter '%s'", name ? name : "(null)");
    const KnobSpec &s = kSpecs[k];
    if (value < s.lo || value > s.hi || (s.pow2 && (value & (value - 1)) != 0))
        return set_error(MSN_ERR_INVALID, "msn_tune_set: %s=%d outside [%d, %d]%s", s.name, value, s.lo, s.hi,
                         s.pow2 ? " or not a power of two" : "");
    if (g_values[k].exchange(value) != value) g_epoch.fetch_add(1);
    return MSN_OK;
}

extern "C" int msn_tune_get(const char *name, int *value) {
    clear_error();
    const int k = find(name);
    if (k < 0 || !value) return set_error(MSN_ERR_INVALID, "msn_tune_get: unknown parameter or null pointer");
    *value = g_values[k].load();
    return MSN_OK;
}

extern "C" int msn_tune_reset(void) {
    clear_error();
    for (int k = 0; k < kKnobCount; ++k) g_values[k].store(kSpecs[k].def);
    g_epoch.fetch_add(1);
    return MSN_OK;
}

extern "C" unsigned msn_tune_epoch(void) { return tune_epoch(); }
