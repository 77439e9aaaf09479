// Status strings, error detail and launch counting of the flub_gb300 C ABI.
#include <cstdarg>
#include <cstdio>

#include "common.cuh"

namespace flub {

static thread_local char g_last_error[1024] = "";
static std::atomic<int64_t> g_launches{0};

void set_last_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

void count_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace flub

extern "C" {

const char *flub_status_string(int status) {
    switch (status) {
    case FLUB_OK: return "ok";
    case FLUB_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FLUB_ERR_CUDA: return "CUDA error";
    case FLUB_ERR_UNSUPPORTED: return "unsupported option";
    case FLUB_ERR_OUT_OF_MEMORY: return "out of device memory";
    case FLUB_ERR_BREAKDOWN: return "CG breakdown (non-finite scalar)";
    case FLUB_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
    }
}

const char *flub_last_error(void) { return flub::g_last_error; }

int flub_version(void) { return 100; }

int64_t flub_launch_count(void) { return flub::g_launches.load(std::memory_order_relaxed); }

void flub_reset_launch_count(void) { flub::g_launches.store(0, std::memory_order_relaxed); }

}  // extern "C"
