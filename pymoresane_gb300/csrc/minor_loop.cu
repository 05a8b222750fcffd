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
// block back. The stop rules run on the device (minor_control_apply) and set the
// WHILE condition with cudaGraphSetConditional; the positivity branch is an IF
// node set the same way. Without positivity, the lines from xn = x + alpha p
// to rn.rn and beta are one launch (cg_step_snr, whose last CTA applies the stop
// rules), and every vector pass skips the rows outside the recomposition's
// support, where all vectors are zero. The body's operations have the arithmetic
// of the library's step entry points (the host-driven loop gives the same model
// bit for bit). Instantiated graphs are cached per engine and keyed by the
// full argument block (buffers, sizes, scales), so a deconvolution that keeps
// its buffers re-uses them across minor loops.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "minor_state.cuh"
#include "msn_common.cuh"

namespace msn {

unsigned long long thread_launches();
void adjust_launches(long long delta);

namespace {

enum { S_RR = 0, S_PAP = 1, S_ALPHA = 2, S_RNRN = 3, S_BETA = 4 };

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

// SNR and the stop rules (minor_control_apply, minor_state.cuh).
__global__ void minor_control(MinorState *s, const double *snr2, double *hist, int hist_len,
                              cudaGraphConditionalHandle h) {
    minor_control_apply(s, snr2, hist, hist_len, h);
}

// p = rn + beta p (main.py:411, the arithmetic of msn_cg_direction), r = rn,
// and x = xn when the control kernel kept this iteration's xn.
// r.r of the next iteration is this iteration's rn.rn (r = rn; same values, same
// reduction order), so it is carried in the scalar block instead of recomputed.
// Rows outside the support hold zeros in every vector and are not touched.
__global__ void direction_commit(const float4 *__restrict__ rn, float4 *__restrict__ p, float4 *__restrict__ r,
                                 const float4 *__restrict__ xn, float4 *__restrict__ x,
                                 double *__restrict__ scal, const MinorState *__restrict__ s, size_t n4,
                                 RowSupport sup) {
    pdl_wait();
    pdl_trigger();
    const float b = (float)scal[S_BETA];
    const bool commit = s->commit != 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) scal[S_RR] = scal[S_RNRN];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        if (!sup.active(i)) continue;
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
constexpr int kScratch = 512;      // pinned doubles for host reads (plane maxima of up to 30 scales etc.)

struct CacheEntry {
    msn_minor_args key;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long last_use = 0;
    long long prologue_kernels = 0, body_kernels = 0, branch_kernels = 0;
    int red_bits = 64;    // reduction accumulation type the graph was captured with
    unsigned epoch = 0;   // tuning epoch of its launch configurations
};

struct Engine {
    int device = -1;
    MinorState *d_state = nullptr;
    double *d_hist = nullptr;
    MinorState *h_state = nullptr;  // pinned
    double *h_scratch = nullptr;    // pinned, kScratch doubles: scalars read back by the major loop
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
    k.seg_flags = a->seg_flags;
    k.row_flags = a->row_flags;
    k.rec_rows = a->rec_rows;
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
    // in (p) is zero outside the level-0 support of the recomposition: the convolution skips
    // the row transforms of pairs of zero rows
    MSN_TRY(fft_convolve_rows(in, a->n, a->m, a->spec, a->tmp, a->linear, a->fft_work, a->fft_work_bytes,
                              a->rec_rows, st));
    // rows whose mask row is empty stay zero (cleared in the prologue)
    MSN_TRY(msn_iuwt_decompose_masked_rows(a->tmp, a->emask, a->row_flags, a->planes, a->n, a->n, a->max_scale,
                                           a->scale_adjust, a->iuwt_work, a->iuwt_work_bytes, st));
    // rows outside the recomposition's support (fixed for the minor loop) are never touched: the
    // prologue cleared them in A p and in the recomposition planes of the workspace
    return msn_iuwt_recompose_active_rows(a->planes, planes, a->rec_rows, out, a->n, a->n, a->scale_adjust,
                                          a->iuwt_work, a->iuwt_work_bytes, st);
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
        // r.r of the first iteration (later ones are carried from rn.rn)
        MSN_TRY(msn_dot2(a->r, a->r, nullptr, nullptr, nvec, a->scal + S_RR, a->red_work, a->red_work_bytes, st));
        // the extraction mask is fixed for the whole minor loop: flag its non-empty segments and
        // rows once, and clear Q, whose rows outside the mask are then never written again
        MSN_TRY(msn_segment_flags(a->emask, (size_t)planes * nvec, a->seg_flags, st));
        MSN_TRY(msn_row_flags(a->emask, (size_t)planes * a->n, a->n, a->row_flags, st));
        MSN_TRY(msn_recompose_row_activity(a->row_flags, planes, a->n, a->scale_adjust, a->rec_rows, st));
        MSN_TRY(check_cuda(cudaMemsetAsync(a->planes, 0, (size_t)planes * nvec * sizeof(float), st), "zero Q"));
        // A p and the recomposition planes: rows outside the recomposition's support stay zero
        MSN_TRY(check_cuda(cudaMemsetAsync(a->ap, 0, nvec * sizeof(float), st), "zero Ap"));
        MSN_TRY(check_cuda(cudaMemsetAsync(a->iuwt_work, 0, a->iuwt_work_bytes, st), "zero IUWT workspace"));
        // x, r, p, A p (and xn, rn) are zero outside the level-0 support of the recomposition
        // (rec_rows[0 .. n)); the vector passes of the loop body skip those rows, so xn and rn
        // start at zero there
        MSN_TRY(check_cuda(cudaMemsetAsync(a->xn, 0, nvec * sizeof(float), st), "zero xn"));
        MSN_TRY(check_cuda(cudaMemsetAsync(a->rn, 0, nvec * sizeof(float), st), "zero rn"));
        minor_init<<<1, 1, 0, st>>>(state, a->minor_loop_miter);
        MSN_TRY(check_launch("minor_init"));
        return add_conditional(st, while_h, cudaGraphCondTypeWhile, &body);
    }));

    cudaGraphConditionalHandle if_h = 0;
    if (a->enforce_positivity)
        MSN_TRY(check_cuda(cudaGraphConditionalHandleCreate(&if_h, body, 0u, 0u), "positivity handle"));
    long long branch_kernels = 0;
    // float4 elements never straddle rows when n is a multiple of 4 (the IUWT requires it);
    // otherwise the vector passes stay dense
    const RowSupport sup = (a->n % 4 == 0 && a->n >= 4) ? RowSupport{a->rec_rows, (unsigned)(a->n / 4)}
                                                        : RowSupport{nullptr, 1u};
    MSN_TRY(capture_into(e->cs[1], body, &ce->body_kernels, [&](cudaStream_t st) -> int {
        // the body's kernels may each launch while their predecessor finishes (launch_k)
        const PdlScope pdl(tune_value(kKnobGraphPdl) != 0);
        MSN_TRY(apply_a(a, a->p, a->ap, st));
        // p.Ap into scal[S_PAP] (the second output, scal[S_ALPHA], is rewritten right after);
        // r.r is carried from the previous iteration (direction_commit) or the prologue
        MSN_TRY(dot_rows(a->p, a->ap, nvec, sup, a->scal + S_PAP, a->red_work, a->red_work_bytes, st));
        if (a->enforce_positivity) {
            MSN_TRY(msn_cg_alpha_x(a->x, a->p, a->scal, a->xn, nvec, a->neg, st));
            positivity_gate<<<1, 1, 0, st>>>(a->neg, state, if_h);
            MSN_TRY(check_launch("positivity_gate"));
            cudaGraph_t branch = nullptr;
            MSN_TRY(add_conditional(st, if_h, cudaGraphCondTypeIf, &branch));
            MSN_TRY(capture_into(e->cs[2], branch, &branch_kernels, [&](cudaStream_t bst) -> int {
                MSN_TRY(msn_cg_positivity(a->x, a->xn, a->p, a->scal, nvec, bst));
                return apply_a(a, a->p, a->ap, bst);
            }));
            MSN_TRY(msn_snr_update_masked(a->esrc, a->ms, a->planes, a->scal, (size_t)planes * nvec, a->seg_flags,
                                          a->snr2, a->red_work, a->red_work_bytes, st));
            minor_control<<<1, 1, 0, st>>>(state, a->snr2, hist, kHistory, while_h);
            MSN_TRY(check_launch("minor_control"));
            MSN_TRY(msn_cg_residual(a->r, a->ap, a->scal, a->rn, nvec, a->red_work, a->red_work_bytes, st));
        } else {
            // xn = x + alpha p and rn = r - alpha Ap (with rn.rn, beta), MS += alpha Q with the SNR
            // sums, and the stop rules: one launch
            MSN_TRY(cg_step_snr_rows(a->x, a->p, a->r, a->ap, a->scal, a->xn, a->rn, nvec, sup, a->esrc, a->ms,
                                     a->planes, (size_t)planes * nvec, a->seg_flags, a->snr2, state, hist, kHistory,
                                     while_h, a->red_work, a->red_work_bytes, st));
        }
        return launch_k("direction_commit", direction_commit, ew_grid4(nvec / 4), 256, 0, st, (const float4 *)a->rn,
                        (float4 *)a->p, (float4 *)a->r, (const float4 *)a->xn, (float4 *)a->x, a->scal, state,
                        nvec / 4, sup);
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
                          a->seg_flags, a->row_flags, a->rec_rows, a->fft_work, a->iuwt_work, a->red_work};
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
    if (rc == MSN_OK) rc = check_cuda(cudaMallocHost(&e->h_scratch, kScratch * sizeof(double)), "host scratch");
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
    if (e->h_scratch) cudaFreeHost(e->h_scratch);
    delete e;
    return MSN_OK;
}

namespace msn {
namespace {

// One minor loop on stream st; the caller holds e->mu.
int run_minor(Engine *e, const msn_minor_args *args, msn_minor_result *result, double *snr_history,
              int history_len, cudaStream_t st) {
    MSN_TRY(validate_args(args));
    const msn_minor_args key = make_key(args);
    CacheEntry *ce = nullptr;
    const int red_bits = msn_reduction_precision();
    for (auto &c : e->cache)
        if (std::memcmp(&c.key, &key, sizeof(key)) == 0 && c.red_bits == red_bits && c.epoch == tune_epoch()) ce = &c;
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
        ce->red_bits = red_bits;
        ce->epoch = tune_epoch();
        const int rc = build_graph(e, &key, ce);
        if (rc != MSN_OK) {
            destroy_entry(*ce);
            e->cache.pop_back();
            return rc;
        }
    }
    ce->last_use = ++e->tick;
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
    result->reserved = 0;
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

int check_engine_device(Engine *e) {
    int device = -1;
    MSN_TRY(check_cuda(cudaGetDevice(&device), "cudaGetDevice"));
    if (device != e->device)
        return set_error(MSN_ERR_INVALID, "engine belongs to device %d, current device is %d", e->device, device);
    return MSN_OK;
}

}  // namespace
}  // namespace msn

extern "C" int msn_minor_loop(void *engine, const msn_minor_args *args, msn_minor_result *result,
                              double *snr_history, int history_len, void *stream) {
    clear_error();
    Engine *e = static_cast<Engine *>(engine);
    if (!e || !args || !result) return set_error(MSN_ERR_INVALID, "msn_minor_loop: null engine, arguments or result");
    MSN_TRY(check_engine_device(e));
    std::lock_guard<std::mutex> lock(e->mu);
    return run_minor(e, args, result, snr_history, history_len, as_stream(stream));
}

// ---------------------------------------------------------------------------
// Major loop (pymoresane/main.py:266-514)
// ---------------------------------------------------------------------------
namespace msn {
namespace {

struct EventLog {
    msn_event *ev;
    int cap, n = 0, dropped = 0;
    void add(int code, int a = 0, int b = 0, double v = 0.0) {
        if (ev && n < cap) {
            ev[n].code = code;
            ev[n].a = a;
            ev[n].b = b;
            ev[n].reserved = 0;
            ev[n].v = v;
            ++n;
        } else {
            ++dropped;
        }
    }
};

// numpy.argmax of x[from:]: the first maximum, a NaN counting as the maximum.
int first_argmax(const std::vector<float> &x, int from) {
    int best = from;
    for (int i = from; i < (int)x.size(); ++i) {
        if (std::isnan(x[i])) return i;
        if (x[i] > x[best]) best = i;
    }
    return best;
}

int validate_run(const msn_moresane_args *a) {
    static const char *fn = "msn_moresane_run";
    if (a->n <= 0 || a->n % 4 || a->ns <= 0 || a->ns % 4 || a->ns > a->n || a->off < 0 || a->off + a->ns > a->n)
        return set_error(MSN_ERR_INVALID, "%s: bad sides n=%d ns=%d off=%d", fn, a->n, a->ns, a->off);
    if (a->scale_count < 1 || a->scale_count > 30 || (1LL << a->scale_count) > a->ns)
        return set_error(MSN_ERR_INVALID, "%s: bad scale_count %d for side %d", fn, a->scale_count, a->ns);
    if (a->scale_count > kScratch / 2) return set_error(MSN_ERR_INVALID, "%s: too many scales", fn);
    const void *ptrs[] = {a->dirty, a->energies, a->spec_sub, a->spec_data, a->model, a->residual, a->dec, a->thr,
                          a->emask, a->esrc, a->planes, a->ms, a->x, a->xn, a->r, a->rn, a->p, a->ap, a->tmp,
                          a->rec, a->masked, a->sub, a->conv_full, a->sigma, a->pmax, a->scal, a->snr2, a->std4,
                          a->neg, a->seg_flags, a->row_flags, a->rec_rows, a->fmax, a->small, a->iuwt_work, a->fft_work, a->fft_work_full, a->tool_work,
                          a->red_work};
    for (const void *p : ptrs)
        if (!p) return set_error(MSN_ERR_INVALID, "%s: null buffer in the argument block", fn);
    return MSN_OK;
}

int read_back(Engine *e, const void *d_src, size_t bytes, cudaStream_t st) {
    MSN_TRY(check_cuda(cudaMemcpyAsync(e->h_scratch, d_src, bytes, cudaMemcpyDeviceToHost, st), "read back"));
    return check_cuda(cudaStreamSynchronize(st), "major loop");
}

int run_moresane(Engine *e, const msn_moresane_args *a, msn_moresane_result *res, msn_major_record *records,
                 int records_len, EventLog &ev, cudaStream_t st) {
    const int n = a->n, ns = a->ns, o = a->off, S = a->scale_count;
    const size_t nvec = (size_t)ns * ns, nfull = (size_t)n * n;
    const float *dirty_sub = a->sub;
    // dirty_sub = dirty[o:o+ns, o:o+ns] (main.py:249-253); the whole image when ns == n
    auto sub_view = [&](const float *img) -> int {
        if (ns == n) {
            dirty_sub = img;
            return MSN_OK;
        }
        dirty_sub = a->sub;
        return check_cuda(cudaMemcpy2DAsync(a->sub, ns * sizeof(float), img + (size_t)o * n + o, n * sizeof(float),
                                            ns * sizeof(float), ns, cudaMemcpyDeviceToDevice, st),
                          "subregion copy");
    };
    // residual = dirty - H * model over the whole image with the data PSF (main.py:483-486)
    auto residual_of = [&]() -> int {
        MSN_TRY(msn_fft_convolve(a->model, n, a->m_data, a->spec_data, a->conv_full, a->linear, a->fft_work_full,
                                 a->fft_work_full_bytes, st));
        return msn_sub(a->dirty, a->conv_full, a->residual, nfull, st);
    };
    auto dirty_peak = [&](float *out) -> int {
        MSN_TRY(msn_plane_max(dirty_sub, 1, nvec, 0, a->fmax, a->small, a->small_bytes, st));
        MSN_TRY(read_back(e, a->fmax, sizeof(float), st));
        *out = *reinterpret_cast<const float *>(e->h_scratch);
        return MSN_OK;
    };

    MSN_TRY(check_cuda(cudaMemsetAsync(a->model, 0, nfull * sizeof(float), st), "zero model"));
    MSN_TRY(sub_view(a->dirty));
    int major = 0, min_scale = 0, n_rec = 0;
    float max_coeff = 1.0f;
    double std_current = 1000.0, std_ratio = 1.0;
    bool have_x = false, have_residual = false;
    std::vector<float> normalised(S, 0.0f);
    res->complete = 0;

    msn_minor_args m;
    std::memset(&m, 0, sizeof(m));
    m.n = ns;
    m.m = a->m_sub;
    m.linear = a->linear;
    m.minor_loop_miter = a->minor_loop_miter;
    m.enforce_positivity = a->enforce_positivity;
    m.spec = a->spec_sub;
    m.rec = a->rec;
    m.x = a->x;
    m.xn = a->xn;
    m.r = a->r;
    m.rn = a->rn;
    m.p = a->p;
    m.ap = a->ap;
    m.tmp = a->tmp;
    m.planes = a->planes;
    m.emask = a->emask;
    m.esrc = a->esrc;
    m.ms = a->ms;
    m.scal = a->scal;
    m.snr2 = a->snr2;
    m.neg = a->neg;
    m.seg_flags = a->seg_flags;
    m.row_flags = a->row_flags;
    m.rec_rows = a->rec_rows;
    m.fft_work = a->fft_work;
    m.fft_work_bytes = a->fft_work_bytes;
    m.iuwt_work = a->iuwt_work;
    m.iuwt_work_bytes = a->iuwt_work_bytes;
    m.red_work = a->red_work;
    m.red_work_bytes = a->red_work_bytes;

    while (true) {
        if (!(major < a->major_loop_miter && max_coeff > 0 && std_ratio > a->accuracy)) break;
        float peak = 0.0f;
        MSN_TRY(dirty_peak(&peak));
        if (!(peak > a->flux_threshold)) break;
        msn_major_record rec;
        std::memset(&rec, 0, sizeof(rec));
        rec.major = major;
        while (min_scale < S) {
            if (min_scale == 0) {
                // threshold at sigma_level MAD sigmas of the (unmasked) decomposition (main.py:279-296)
                MSN_TRY(msn_iuwt_decompose(dirty_sub, a->dec, nullptr, ns, ns, S, 0, a->iuwt_work, a->iuwt_work_bytes,
                                           st));
                MSN_TRY(msn_mad_sigma(a->dec, S, ns, ns, a->noise_rects, a->sigma, a->tool_work, a->tool_work_bytes,
                                      st));
                if (a->mask_sub) {
                    MSN_TRY(msn_mul(dirty_sub, a->mask_sub, a->masked, nvec, st));
                    MSN_TRY(msn_iuwt_decompose(a->masked, a->dec, nullptr, ns, ns, S, 0, a->iuwt_work,
                                               a->iuwt_work_bytes, st));
                }
                MSN_TRY(msn_apply_threshold(a->dec, S, ns, ns, a->sigma, a->sigma_level, a->supp_rects, a->thr,
                                            a->pmax, a->small, a->small_bytes, st));
                MSN_TRY(read_back(e, a->pmax, S * sizeof(float), st));
                const float *pm = reinterpret_cast<const float *>(e->h_scratch);
                for (int i = 0; i < S; ++i) normalised[i] = pm[i] / a->energies[i];
            }
            const int max_index = first_argmax(normalised, min_scale);
            const int max_scale = max_index + 1;
            max_coeff = normalised[max_index];
            if (max_coeff == 0.0f) {
                ev.add(MSN_EV_NO_COEFFICIENTS);
                break;
            }
            ev.add(MSN_EV_MINIMUM_SCALE, min_scale);
            ev.add(MSN_EV_MAXIMUM_SCALE, max_scale);
            int scale_adjust = 0;
            for (int i = max_index - 1; i >= 0; --i) {
                if (normalised[i] == 0.0f) {
                    scale_adjust = i + 1;
                    ev.add(MSN_EV_SCALE_EMPTY, scale_adjust);
                    break;
                }
            }
            const int planes = max_scale - scale_adjust;
            MSN_TRY(msn_source_extraction(a->thr + (size_t)scale_adjust * nvec, planes, ns, ns, (float)a->tolerance,
                                          a->neg_comp, a->emask, a->esrc, a->tool_work, a->tool_work_bytes, st));
            MSN_TRY(msn_iuwt_recompose(a->esrc, planes, nullptr, a->rec, ns, ns, scale_adjust, a->iuwt_work,
                                       a->iuwt_work_bytes, st));
            m.max_scale = max_scale;
            m.scale_adjust = scale_adjust;
            msn_minor_result mr;
            MSN_TRY(run_minor(e, &m, &mr, nullptr, 0, st));
            if (mr.outcome == MSN_MINOR_FALSE_DETECTION) {
                min_scale += 1;
            } else if (mr.outcome == MSN_MINOR_CONVERGED) {
                min_scale = 0;
            } else if (mr.outcome == MSN_MINOR_STALLED) {
                min_scale = mr.snr_current > 10.5 ? 0 : min_scale + 1;
            }
            ev.add(MSN_EV_MINOR_DONE, mr.minor, mr.outcome, mr.snr_current);
            have_x = true;
            rec.max_scale = max_scale;
            rec.scale_adjust = scale_adjust;
            rec.minor = mr.minor;
            rec.outcome = mr.outcome;
            rec.snr = mr.snr_current;
            if (mr.minor == a->minor_loop_miter && mr.snr_current > 10.5) {
                min_scale = 0;
                break;
            }
            if (min_scale == 0) break;
        }
        if (min_scale == S) {
            ev.add(MSN_EV_ALL_SCALES_POOR);
            break;
        }
        if (max_coeff > 0 && have_x) {
            // model += gain x; residual; revert when the residual's deviation grew (main.py:466-503)
            MSN_TRY(msn_model_update(a->model, n, a->x, ns, o, o, a->loop_gain, 1, st));
            MSN_TRY(residual_of());
            have_residual = true;
            const double std_last = std_current;
            MSN_TRY(msn_region_std(a->residual, n, ns, ns, o, o, a->std4, a->red_work, a->red_work_bytes, st));
            MSN_TRY(read_back(e, a->std4 + 3, sizeof(double), st));
            std_current = e->h_scratch[0];
            std_ratio = (std_last - std_current) / std_last;
            rec.std = std_current;
            rec.reverted = std_ratio < 0;
            if (std_ratio < 0) {
                ev.add(MSN_EV_REVERTED);
                MSN_TRY(msn_model_update(a->model, n, a->x, ns, o, o, a->loop_gain, -1, st));
                MSN_TRY(residual_of());
            }
            MSN_TRY(sub_view(a->residual));
            major += 1;
            if (records && n_rec < records_len) records[n_rec++] = rec;
            ev.add(MSN_EV_MAJOR_DONE, major);
        }
        if (major == 0) {
            ev.add(MSN_EV_NO_WORK);
            res->complete = 1;
            break;
        }
    }
    MSN_TRY(check_cuda(cudaStreamSynchronize(st), "major loop"));
    res->major = major;
    res->have_residual = have_residual;
    res->n_records = n_rec;
    return MSN_OK;
}

}  // namespace
}  // namespace msn

extern "C" int msn_moresane_run(void *engine, const msn_moresane_args *args, msn_moresane_result *result,
                                msn_major_record *records, int records_len, msn_event *events, int events_len,
                                void *stream) {
    clear_error();
    Engine *e = static_cast<Engine *>(engine);
    if (!e || !args || !result) return set_error(MSN_ERR_INVALID, "msn_moresane_run: null engine, arguments or result");
    std::memset(result, 0, sizeof(*result));
    MSN_TRY(validate_run(args));
    MSN_TRY(check_engine_device(e));
    std::lock_guard<std::mutex> lock(e->mu);
    EventLog ev{events, events ? events_len : 0};
    const int rc = run_moresane(e, args, result, records, records ? records_len : 0, ev, as_stream(stream));
    result->n_events = ev.n;
    result->events_dropped = ev.dropped;
    return rc;
}
