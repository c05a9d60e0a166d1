// Internal helpers shared by the commkit-gb300 CUDA sources: error
// reporting on the host, and (from ck_device.cuh) fast division by a
// run-time constant and the inline-PTX wrappers the kernels use.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ck_device.cuh"
#include "commkit_gb300.h"

namespace ck {

// Records a message for ck_last_error() on this host thread and returns `status`.
int fail(int status, const char* fmt, ...);
// CK_OK, or CK_ERR_CUDA / CK_ERR_OUT_OF_MEMORY with the CUDA error text.
int cuda_check(cudaError_t err, const char* what);
// Clears the last-error message of this host thread.
void clear_error();

#define CK_TRY(expr)                     \
    do {                                 \
        const int ck_status__ = (expr);  \
        if (ck_status__ != CK_OK) return ck_status__; \
    } while (0)

#define CK_CUDA(expr) CK_TRY(::ck::cuda_check((expr), #expr))

}  // namespace ck
