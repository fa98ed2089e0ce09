// Status codes and CUDA error bookkeeping of the C ABI.
#include <stdio.h>

#include <atomic>

#include "common.cuh"

namespace gstex {

static thread_local char g_last_error[256] = "";
static std::atomic<unsigned long long> g_launches{0};

void set_cuda_error(cudaError_t e, const char* what) {
    snprintf(g_last_error, sizeof(g_last_error), "%s: %s", what, cudaGetErrorString(e));
}

int check_launch(const char* what, int launches) {
    g_launches.fetch_add((unsigned long long)launches, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_cuda_error(e, what);
        return GSTEX_ERR_CUDA;
    }
    return GSTEX_OK;
}

}  // namespace gstex

extern "C" const char* gstex_status_string(int status) {
    switch (status) {
        case GSTEX_OK: return "ok";
        case GSTEX_ERR_INVALID_ARGUMENT: return "invalid argument";
        case GSTEX_ERR_CAPACITY: return "buffer too small";
        case GSTEX_ERR_UNSUPPORTED: return "unsupported configuration";
        case GSTEX_ERR_CUDA: return "CUDA error";
        default: return "unknown status";
    }
}

extern "C" const char* gstex_last_cuda_error(void) { return gstex::g_last_error; }

extern "C" const char* gstex_version(void) { return "0.1.0"; }

extern "C" unsigned long long gstex_launch_count(void) { return gstex::g_launches.load(std::memory_order_relaxed); }
