// Error reporting and version of the commkit-gb300 C ABI.
#include <stdarg.h>
#include <stdio.h>

#include "ck_common.cuh"

namespace ck {

namespace {
thread_local char g_message[512] = "";
}

int fail(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_message, sizeof(g_message), fmt, ap);
    va_end(ap);
    return status;
}

void clear_error() { g_message[0] = '\0'; }

int cuda_check(cudaError_t err, const char* what) {
    if (err == cudaSuccess) return CK_OK;
    // Clear the sticky-free error so later calls on this thread start clean.
    (void)cudaGetLastError();
    const int status =
        err == cudaErrorMemoryAllocation ? CK_ERR_OUT_OF_MEMORY : CK_ERR_CUDA;
    return fail(status, "%s: %s (%s)", what, cudaGetErrorString(err), cudaGetErrorName(err));
}

}  // namespace ck

extern "C" const char* ck_last_error(void) { return ck::g_message; }

extern "C" const char* ck_status_string(int status) {
    switch (status) {
        case CK_OK: return "ok";
        case CK_ERR_INVALID_ARGUMENT: return "invalid argument";
        case CK_ERR_UNSUPPORTED: return "unsupported";
        case CK_ERR_CUDA: return "CUDA error";
        case CK_ERR_OUT_OF_MEMORY: return "out of device memory";
        case CK_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
        default: return "unknown status";
    }
}

extern "C" const char* ck_version(void) { return "0.1.0"; }
