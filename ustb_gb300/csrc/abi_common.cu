// Error state of the C-ABI and small shared entry points.
#include "common.cuh"

namespace ustb {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    set_error("CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e), cudaGetErrorString(e), what,
              file, line);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();  // clear the sticky-free allocation error
        return USTB_E_OOM;
    }
    return USTB_E_CUDA;
}

}  // namespace ustb

extern "C" const char* ustb_last_error(void) { return ustb::g_last_error.c_str(); }

extern "C" int ustb_abi_version(void) { return 10300; }
