// Library-wide C-ABI helpers: version, error reporting, device queries.

#include <atomic>
#include <cstdarg>
#include <map>
#include <mutex>
#include <utility>
#include <cstdio>
#include <cstring>

#include "gb_common.cuh"
#include "gb_internal.h"

namespace {
thread_local char g_err[1024] = {0};
std::atomic<long long> g_launches{0};
thread_local int g_capturing = 0;
thread_local long long g_captured = 0;
}

namespace gb {
void note_launch() {
    if (g_capturing) g_captured++;
    else g_launches.fetch_add(1, std::memory_order_relaxed);
}
void note_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
void capture_begin() { g_capturing = 1; g_captured = 0; }
long long capture_end() { g_capturing = 0; return g_captured; }

// The dynamic shared-memory limit is an attribute of the kernel, shared by every
// host thread: raise it, never lower it, so that a launch on one thread cannot find
// the limit lowered by another thread's smaller launch.
cudaError_t ensure_dynamic_smem(const void* func, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> set;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    size_t& cur = set[{dev, func}];
    if (bytes <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}
}   // namespace gb

int gb_set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int gb_set_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
    const char* base = strrchr(file, '/');
    snprintf(g_err, sizeof(g_err), "CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e), what,
             base ? base + 1 : file, line);
    return GB_CUDA_ERROR;
}

extern "C" {

int gb_version(void) { return 10000; }   // 1.0.0

size_t gb_last_error(char* buf, size_t cap) {
    size_t n = strlen(g_err);
    if (buf && cap) {
        size_t c = n < cap - 1 ? n : cap - 1;
        memcpy(buf, g_err, c);
        buf[c] = 0;
    }
    return n;
}

int gb_device_sm_count(void) { return gb::sm_count(); }

long long gb_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

}   // extern "C"
