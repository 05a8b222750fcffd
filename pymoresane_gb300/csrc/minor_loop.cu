// Native conjugate-gradient minor loop (pymoresane/main.py:365-457) as one
// CUDA graph per configuration, for sm_103a.
//
// The reference drives every minor iteration from the host and decides after
// each one whether to stop (SNR tests, main.py:420-455). Here the whole loop is
// a graph: a prologue (x = 0, model sources = 0, r = p = R(extracted sources))
// followed by a WHILE conditional node whose body is one CG iteration
//
//   A p  (FFT convolution, masked decomposition, recomposition)
//   r.r, p.Ap                          -> alpha           (float64)
//   xn = x + alpha p, #(xn < 0)
//   IF (positivity and #(xn < 0) > 0):  xn = max(xn, 0); p = (xn - x) / alpha; A p
//   ms += alpha mask W(H p); |e|^2, |e - ms|^2             (float64)
//   control: SNR, the reference's four stop rules, WHILE condition
//   rn = r - alpha A p; rn.rn; beta                        (float64)
//   p = rn + beta p; r = rn; x = xn unless the stop rule discards xn
//
// so the host launches one graph per minor loop and reads one small state
// block back. The stop rules run on the device (minor_control) and set the
// WHILE condition with cudaGraphSetConditional; the positivity branch is an IF
// node set the same way. Each body operation is the library's own C-ABI entry
// point, captured on a private stream, so the arithmetic is identical to the
// step-by-step path. Instantiated graphs are cached per engine and keyed by the
// full argument block (buffers, sizes, scales), so a deconvolution that keeps
// its buffers re-uses them across minor loops.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "msn_common.cuh"

namespace msn {

unsigned long long thread_launches();
void adjust_launches(long long delta);

namespace {

enum { S_RR = 0, S_PAP = 1, S_ALPHA = 2, S_RNRN = 3, S_BETA = 4 };

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

__global__ void minor_init(MinorState *s, int miter) {
    s->minor = 0;
    s->outcome = MSN_MINOR_RUNNING;
    s->commit = 0;
    s->miter = miter;
    s->positivity_runs = 0;
    s->pad = 0;
    s->snr_current = 0.0;
    s->snr_last = 0.0;
}

// IF condition of the positivity branch (main.py:392-398): any xn < 0.
__global__ void positivity_gate(const int *neg, MinorState *s, cudaGraphConditionalHandle h) {
    const bool run = *neg > 0;
    if (run) s->positivity_runs += 1;
    cudaGraphSetConditional(h, run ? 1u : 0u);
}

// SNR and the stop rules of main.py:413-455, in the reference's order:
//   minor == 1 and SNR > 40  -> false detection (xn discarded)
//   SNR > 40                 -> converged (xn kept)
//   minor > 2, SNR <= last   -> stalled (xn discarded)
//   minor == minor_loop_miter -> iteration cap (xn kept, loop condition ends)
__global__ void minor_control(MinorState *s, const double *snr2, double *hist, int hist_len,
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

// p = rn + beta p (main.py:411, the arithmetic of msn_cg_direction), r = rn,
// and x = xn when the control kernel kept this iteration's xn.
__global__ void direction_commit(const float4 *__restrict__ rn, float4 *__restrict__ p, float4 *__restrict__ r,
                                 const float4 *__restrict__ xn, float4 *__restrict__ x,
                                 const double *__restrict__ scal, const MinorState *__restrict__ s, size_t n4) {
    const float b = (float)scal[S_BETA];
    const bool commit = s->commit != 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        const float4 rv = __ldg(rn + i);
        float4 pv = p[i];
        pv.x = __fadd_rn(rv.x, __fmul_rn(b, pv.x));
        pv.y = __fadd_rn(rv.y, __fmul_rn(b, pv.y));
        pv.z = __fadd_rn(rv.z, __fmul_rn(b, pv.z));
        pv.w = __fadd_rn(rv.w, __fmul_rn(b, pv.w));
        p[i] = pv;
        r[i] = rv;
        if (commit) x[i] = __ldg(xn + i);
    }
}

int ew_grid4(size_t n4) {
    size_t g = (n4 + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    return g < 1 ? 1 : (int)g;
}

constexpr int kHistory = 4096;   // SNR history entries kept per minor loop
constexpr size_t kMaxGraphs = 64;  // instantiated graphs cached per engine

struct CacheEntry {
    msn_minor_args key;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long last_use = 0;
    long long prologue_kernels = 0, body_kernels = 0, branch_kernels = 0;
};

struct Engine {
    int device = -1;
    MinorState *d_state = nullptr;
    double *d_hist = nullptr;
    MinorState *h_state = nullptr;  // pinned
    cudaStream_t cs[3] = {nullptr, nullptr, nullptr};  // capture streams: top graph, loop body, branch body
    std::vector<CacheEntry> cache;
    unsigned long long tick = 0;
    std::mutex mu;
};

// Field-by-field copy into a zeroed block, so that padding never enters the key.
msn_minor_args make_key(const msn_minor_args *a) {
    msn_minor_args k;
    std::memset(&k, 0, sizeof(k));
    k.n = a->n;
    k.m = a->m;
    k.linear = a->linear;
    k.max_scale = a->max_scale;
    k.scale_adjust = a->scale_adjust;
    k.minor_loop_miter = a->minor_loop_miter;
    k.enforce_positivity = a->enforce_positivity != 0;
    k.spec = a->spec;
    k.rec = a->rec;
    k.x = a->x;
    k.xn = a->xn;
    k.r = a->r;
    k.rn = a->rn;
    k.p = a->p;
    k.ap = a->ap;
    k.tmp = a->tmp;
    k.planes = a->planes;
    k.emask = a->emask;
    k.esrc = a->esrc;
    k.ms = a->ms;
    k.scal = a->scal;
    k.snr2 = a->snr2;
    k.neg = a->neg;
    k.fft_work = a->fft_work;
    k.fft_work_bytes = a->fft_work_bytes;
    k.iuwt_work = a->iuwt_work;
    k.iuwt_work_bytes = a->iuwt_work_bytes;
    k.red_work = a->red_work;
    k.red_work_bytes = a->red_work_bytes;
    return k;
}

// A p: FFT convolution with the sub-PSF, mask * W(.) into a->planes, R(planes)
// (main.py:375-384).
int apply_a(const msn_minor_args *a, const float *in, float *out, cudaStream_t st) {
    const int planes = a->max_scale - a->scale_adjust;
    MSN_TRY(msn_fft_convolve(in, a->n, a->m, a->spec, a->tmp, a->linear, a->fft_work, a->fft_work_bytes, st));
    MSN_TRY(msn_iuwt_decompose_masked(a->tmp, a->emask, a->planes, a->n, a->n, a->max_scale, a->scale_adjust,
                                      a->iuwt_work, a->iuwt_work_bytes, st));
    return msn_iuwt_recompose(a->planes, planes, nullptr, out, a->n, a->n, a->scale_adjust, a->iuwt_work,
                              a->iuwt_work_bytes, st);
}

// Adds a conditional node after the current capture dependencies of st and
// makes it the new dependency; returns its body graph.
int add_conditional(cudaStream_t st, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                    cudaGraph_t *body) {
    cudaStreamCaptureStatus status;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t ndeps = 0;
    MSN_TRY(check_cuda(cudaStreamGetCaptureInfo(st, &status, nullptr, &g, &deps, &edges, &ndeps), "capture info"));
    if (status != cudaStreamCaptureStatusActive) return set_error(MSN_ERR_CUDA, "stream capture is not active");
    cudaGraphNodeParams prm = {};
    prm.type = cudaGraphNodeTypeConditional;
    prm.conditional.handle = h;
    prm.conditional.type = type;
    prm.conditional.size = 1;
    cudaGraphNode_t node;
    MSN_TRY(check_cuda(cudaGraphAddNode(&node, g, deps, edges, ndeps, &prm), "add conditional node"));
    *body = prm.conditional.phGraph_out[0];
    return check_cuda(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies),
                      "update capture dependencies");
}

// Captures ops(st) into graph g (already created); the capture always ends.
template <class F>
int capture_into(cudaStream_t st, cudaGraph_t g, long long *kernels, F ops) {
    MSN_TRY(check_cuda(cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
                       "begin capture"));
    const unsigned long long t0 = thread_launches();
    const int rc = ops(st);
    *kernels = (long long)(thread_launches() - t0);
    cudaGraph_t out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &out);
    if (rc != MSN_OK) return rc;
    return check_cuda(e, "end capture");
}

int build_graph(Engine *e, const msn_minor_args *a, CacheEntry *ce) {
    const size_t nvec = (size_t)a->n * a->n;
    const int planes = a->max_scale - a->scale_adjust;
    MinorState *state = e->d_state;
    double *hist = e->d_hist;
    cudaGraph_t top = nullptr;
    MSN_TRY(check_cuda(cudaGraphCreate(&top, 0), "graph create"));
    ce->graph = top;
    cudaGraphConditionalHandle while_h;
    MSN_TRY(check_cuda(cudaGraphConditionalHandleCreate(&while_h, top, a->minor_loop_miter > 0 ? 1u : 0u,
                                                        cudaGraphCondAssignDefault),
                       "while handle"));
    cudaGraph_t body = nullptr;
    MSN_TRY(capture_into(e->cs[0], top, &ce->prologue_kernels, [&](cudaStream_t st) -> int {
        MSN_TRY(check_cuda(cudaMemsetAsync(a->x, 0, nvec * sizeof(float), st), "zero x"));
        MSN_TRY(check_cuda(cudaMemsetAsync(a->ms, 0, (size_t)planes * nvec * sizeof(float), st), "zero sources"));
        MSN_TRY(check_cuda(cudaMemcpyAsync(a->r, a->rec, nvec * sizeof(float), cudaMemcpyDeviceToDevice, st), "r"));
        MSN_TRY(check_cuda(cudaMemcpyAsync(a->p, a->rec, nvec * sizeof(float), cudaMemcpyDeviceToDevice, st), "p"));
        minor_init<<<1, 1, 0, st>>>(state, a->minor_loop_miter);
        MSN_TRY(check_launch("minor_init"));
        return add_conditional(st, while_h, cudaGraphCondTypeWhile, &body);
    }));

    cudaGraphConditionalHandle if_h = 0;
    if (a->enforce_positivity)
        MSN_TRY(check_cuda(cudaGraphConditionalHandleCreate(&if_h, body, 0u, 0u), "positivity handle"));
    long long branch_kernels = 0;
    MSN_TRY(capture_into(e->cs[1], body, &ce->body_kernels, [&](cudaStream_t st) -> int {
        MSN_TRY(apply_a(a, a->p, a->ap, st));
        MSN_TRY(msn_dot2(a->r, a->r, a->p, a->ap, nvec, a->scal, a->red_work, a->red_work_bytes, st));
        MSN_TRY(msn_cg_alpha_x(a->x, a->p, a->scal, a->xn, nvec, a->neg, st));
        if (a->enforce_positivity) {
            positivity_gate<<<1, 1, 0, st>>>(a->neg, state, if_h);
            MSN_TRY(check_launch("positivity_gate"));
            cudaGraph_t branch = nullptr;
            MSN_TRY(add_conditional(st, if_h, cudaGraphCondTypeIf, &branch));
            MSN_TRY(capture_into(e->cs[2], branch, &branch_kernels, [&](cudaStream_t bst) -> int {
                MSN_TRY(msn_cg_positivity(a->x, a->xn, a->p, a->scal, nvec, bst));
                return apply_a(a, a->p, a->ap, bst);
            }));
        }
        MSN_TRY(msn_snr_update(a->esrc, a->ms, a->planes, a->scal, (size_t)planes * nvec, a->snr2, a->red_work,
                               a->red_work_bytes, st));
        minor_control<<<1, 1, 0, st>>>(state, a->snr2, hist, kHistory, while_h);
        MSN_TRY(check_launch("minor_control"));
        MSN_TRY(msn_cg_residual(a->r, a->ap, a->scal, a->rn, nvec, a->red_work, a->red_work_bytes, st));
        direction_commit<<<ew_grid4(nvec / 4), 256, 0, st>>>(
            (const float4 *)a->rn, (float4 *)a->p, (float4 *)a->r, (const float4 *)a->xn, (float4 *)a->x, a->scal,
            state, nvec / 4);
        return check_launch("direction_commit");
    }));
    // branch kernels were counted inside the body capture as well
    ce->body_kernels -= branch_kernels;
    ce->branch_kernels = branch_kernels;
    // captured launches are not executions: take them back out of the launch count
    adjust_launches(-(ce->prologue_kernels + ce->body_kernels + ce->branch_kernels));
    return check_cuda(cudaGraphInstantiate(&ce->exec, top, 0), "graph instantiate");
}

void destroy_entry(CacheEntry &c) {
    if (c.exec) cudaGraphExecDestroy(c.exec);
    if (c.graph) cudaGraphDestroy(c.graph);
    c.exec = nullptr;
    c.graph = nullptr;
}

int validate_args(const msn_minor_args *a) {
    static const char *fn = "msn_minor_loop";
    if (a->n <= 0 || a->n % 4 != 0) return set_error(MSN_ERR_INVALID, "%s: n=%d must be a positive multiple of 4", fn, a->n);
    if (a->max_scale < 1 || a->scale_adjust < 0 || a->scale_adjust >= a->max_scale || a->max_scale > 30)
        return set_error(MSN_ERR_INVALID, "%s: bad scales max_scale=%d scale_adjust=%d", fn, a->max_scale,
                         a->scale_adjust);
    if ((1LL << a->max_scale) > a->n)
        return set_error(MSN_ERR_INVALID, "%s: 2^%d exceeds the side %d", fn, a->max_scale, a->n);
    if (a->minor_loop_miter < 0) return set_error(MSN_ERR_INVALID, "%s: negative minor_loop_miter", fn);
    const void *ptrs[] = {a->spec, a->rec, a->x,     a->xn,   a->r,    a->rn,  a->p,        a->ap,
                          a->tmp,  a->planes, a->emask, a->esrc, a->ms, a->scal, a->snr2, a->neg,
                          a->fft_work, a->iuwt_work, a->red_work};
    for (const void *p : ptrs)
        if (p == nullptr) return set_error(MSN_ERR_INVALID, "%s: null buffer in the argument block", fn);
    const void *vecs[] = {a->rec, a->x, a->xn, a->r, a->rn, a->p, a->ap, a->tmp, a->planes, a->emask, a->esrc, a->ms};
    for (const void *p : vecs)
        if (!aligned16(p)) return set_error(MSN_ERR_INVALID, "%s: buffers must be 16-byte aligned", fn);
    return MSN_OK;
}

}  // namespace
}  // namespace msn

using namespace msn;

extern "C" int msn_minor_engine_create(void **engine) {
    clear_error();
    if (!engine) return set_error(MSN_ERR_INVALID, "msn_minor_engine_create: null output pointer");
    *engine = nullptr;
    Engine *e = new Engine();
    int rc = check_cuda(cudaGetDevice(&e->device), "cudaGetDevice");
    if (rc == MSN_OK) rc = check_cuda(cudaMalloc(&e->d_state, sizeof(MinorState)), "state");
    if (rc == MSN_OK) rc = check_cuda(cudaMalloc(&e->d_hist, kHistory * sizeof(double)), "history");
    if (rc == MSN_OK) rc = check_cuda(cudaMallocHost(&e->h_state, sizeof(MinorState)), "host state");
    for (int i = 0; i < 3 && rc == MSN_OK; ++i)
        rc = check_cuda(cudaStreamCreateWithFlags(&e->cs[i], cudaStreamNonBlocking), "capture stream");
    if (rc != MSN_OK) {
        msn_minor_engine_destroy(e);
        return rc;
    }
    *engine = e;
    return MSN_OK;
}

extern "C" int msn_minor_engine_destroy(void *engine) {
    clear_error();
    Engine *e = static_cast<Engine *>(engine);
    if (!e) return MSN_OK;
    for (auto &c : e->cache) destroy_entry(c);
    for (auto &s : e->cs)
        if (s) cudaStreamDestroy(s);
    if (e->d_state) cudaFree(e->d_state);
    if (e->d_hist) cudaFree(e->d_hist);
    if (e->h_state) cudaFreeHost(e->h_state);
    delete e;
    return MSN_OK;
}

extern "C" int msn_minor_loop(void *engine, const msn_minor_args *args, msn_minor_result *result,
                              double *snr_history, int history_len, void *stream) {
    clear_error();
    Engine *e = static_cast<Engine *>(engine);
    if (!e || !args || !result) return set_error(MSN_ERR_INVALID, "msn_minor_loop: null engine, arguments or result");
    MSN_TRY(validate_args(args));
    int device = -1;
    MSN_TRY(check_cuda(cudaGetDevice(&device), "cudaGetDevice"));
    if (device != e->device)
        return set_error(MSN_ERR_INVALID, "msn_minor_loop: engine belongs to device %d, current device is %d",
                         e->device, device);
    std::lock_guard<std::mutex> lock(e->mu);
    const msn_minor_args key = make_key(args);
    CacheEntry *ce = nullptr;
    for (auto &c : e->cache)
        if (std::memcmp(&c.key, &key, sizeof(key)) == 0) ce = &c;
    if (!ce) {
        if (e->cache.size() >= kMaxGraphs) {
            size_t lru = 0;
            for (size_t i = 1; i < e->cache.size(); ++i)
                if (e->cache[i].last_use < e->cache[lru].last_use) lru = i;
            destroy_entry(e->cache[lru]);
            e->cache.erase(e->cache.begin() + lru);
        }
        e->cache.emplace_back();
        ce = &e->cache.back();
        ce->key = key;
        const int rc = build_graph(e, &key, ce);
        if (rc != MSN_OK) {
            destroy_entry(*ce);
            e->cache.pop_back();
            return rc;
        }
    }
    ce->last_use = ++e->tick;
    cudaStream_t st = as_stream(stream);
    MSN_TRY(check_cuda(cudaGraphLaunch(ce->exec, st), "graph launch"));
    MSN_TRY(check_cuda(cudaMemcpyAsync(e->h_state, e->d_state, sizeof(MinorState), cudaMemcpyDeviceToHost, st),
                       "read state"));
    MSN_TRY(check_cuda(cudaStreamSynchronize(st), "minor loop"));
    const MinorState s = *e->h_state;
    adjust_launches(ce->prologue_kernels + (long long)s.minor * ce->body_kernels +
                    (long long)s.positivity_runs * ce->branch_kernels);
    result->minor = s.minor;
    result->outcome = s.outcome;
    result->positivity_runs = s.positivity_runs;
    result->snr_current = s.snr_current;
    result->snr_last = s.snr_last;
    if (snr_history && history_len > 0) {
        int cnt = s.minor < history_len ? s.minor : history_len;
        if (cnt > kHistory) cnt = kHistory;
        if (cnt > 0)
            MSN_TRY(check_cuda(cudaMemcpy(snr_history, e->d_hist, cnt * sizeof(double), cudaMemcpyDeviceToHost),
                               "read SNR history"));
    }
    return MSN_OK;
}
