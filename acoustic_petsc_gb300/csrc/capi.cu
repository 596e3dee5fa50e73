// capi.cu -- library-wide C entry points: error strings, launch accounting, version.
#include <atomic>
#include <stdio.h>

#include "hype_common.cuh"

namespace hype {
static thread_local char g_last_error[512] = "";
static std::atomic<long long> g_launches{0};

void set_last_error(const char* where, cudaError_t e) {
    snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s)", where, cudaGetErrorName(e), cudaGetErrorString(e));
}
void count_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}  // namespace hype

extern "C" const char* hype_strerror(int code) {
    switch (code) {
        case HYPE_OK: return "ok";
        case HYPE_ERR_ARG: return "invalid argument";
        case HYPE_ERR_STATE: return "inadmissible state (density or pressure below floor)";
        case HYPE_ERR_CUDA: return "CUDA error";
        case HYPE_ERR_NOMEM: return "device allocation failed";
        case HYPE_ERR_UNSUPPORTED: return "unsupported option";
        default: return "unknown status";
    }
}
extern "C" const char* hype_last_error(void) { return hype::g_last_error; }
extern "C" long long hype_launch_count(void) { return hype::g_launches.load(); }
extern "C" const char* hype_version(void) { return "hype-gb300 0.1 (sm_103a)"; }

extern "C" int hype_set_device(int device) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        hype::set_last_error("cudaSetDevice", e);
        return HYPE_ERR_CUDA;
    }
    return HYPE_OK;
}

extern "C" int hype_device_count(int* n) {
    if (!n) return HYPE_ERR_ARG;
    cudaError_t e = cudaGetDeviceCount(n);
    if (e != cudaSuccess) {
        *n = 0;
        hype::set_last_error("cudaGetDeviceCount", e);
        return HYPE_ERR_CUDA;
    }
    return HYPE_OK;
}
