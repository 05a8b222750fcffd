// libmsn: error reporting and version query.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "msn_common.cuh"

namespace msn {

static thread_local char g_last_error[512] = "";

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

void clear_error() { g_last_error[0] = '\0'; }

int check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return MSN_OK;
    return set_error(MSN_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

static std::atomic<unsigned long long> g_launches{0};

static thread_local unsigned long long t_launches = 0;

void count_launch() {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ++t_launches;
}

bool &pdl_flag() {
    static thread_local bool flag = false;
    return flag;
}

// Launches issued by the calling thread (graph capture measures its own).
unsigned long long thread_launches() { return t_launches; }

// Graph executions: captured launches are taken out, executed ones added.
void adjust_launches(long long delta) {
    g_launches.fetch_add((unsigned long long)delta, std::memory_order_relaxed);
}

}  // namespace msn

extern "C" unsigned long long msn_launch_count(int reset) {
    return reset ? msn::g_launches.exchange(0) : msn::g_launches.load();
}

extern "C" const char *msn_last_error(void) { return msn::g_last_error; }

extern "C" int msn_version(void) { return 100; }
