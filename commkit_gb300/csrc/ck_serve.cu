// Batch assembly for the request server: one kernel copies every segment
// of a batch (each request's symbols, its frames' noise scales) from
// pinned host memory into the batch slot's device buffers.
//
// On GB300 the Grace host memory is reachable from the GPU over the
// coherent NVLink-C2C link, and pinned allocations have the same address
// on both sides, so the kernel reads the payloads (and the segment table
// itself) in place: a batch of hundreds of requests costs one launch
// instead of one copy call per request.
#include <stdint.h>

#include <atomic>

#include "ck_common.cuh"

namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) gather_kernel(const ck_segment* __restrict__ segs, int32_t n) {
    for (int32_t s = blockIdx.x; s < n; s += gridDim.x) {
        const ck_segment g = segs[s];
        const uintptr_t src = reinterpret_cast<uintptr_t>(g.src), dst = reinterpret_cast<uintptr_t>(g.dst);
        const int64_t bytes = g.bytes;
        if (((src | dst | static_cast<uintptr_t>(bytes)) & 15u) == 0) {
            const int4* a = reinterpret_cast<const int4*>(g.src);
            int4* b = reinterpret_cast<int4*>(g.dst);
            for (int64_t i = threadIdx.x; i < bytes / 16; i += blockDim.x) b[i] = a[i];
        } else if (((src | dst | static_cast<uintptr_t>(bytes)) & 3u) == 0) {
            const int32_t* a = reinterpret_cast<const int32_t*>(g.src);
            int32_t* b = reinterpret_cast<int32_t*>(g.dst);
            for (int64_t i = threadIdx.x; i < bytes / 4; i += blockDim.x) b[i] = a[i];
        } else {
            const uint8_t* a = static_cast<const uint8_t*>(g.src);
            uint8_t* b = static_cast<uint8_t*>(g.dst);
            for (int64_t i = threadIdx.x; i < bytes; i += blockDim.x) b[i] = a[i];
        }
    }
}

}  // namespace

extern "C" int ck_gather(const ck_segment* segments, int32_t n, void* stream) {
    ck::clear_error();
    if (n < 0) return ck::fail(CK_ERR_INVALID_ARGUMENT, "n must be >= 0");
    if (n == 0) return CK_OK;
    if (!segments) return ck::fail(CK_ERR_INVALID_ARGUMENT, "segments is NULL");
    const int grid = n < 152 * 8 ? n : 152 * 8;
    gather_kernel<<<grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(segments, n);
    return ck::cuda_check(cudaGetLastError(), "gather launch");
}

// An acquire fence on the calling host thread: after it has read a flag the
// device published (a frame's iteration count in mapped memory, written
// after a system-scope fence), the reads that follow see the data written
// before the flag.  Host CPUs such as Grace order loads weakly.
extern "C" void ck_host_acquire(void) { std::atomic_thread_fence(std::memory_order_acquire); }
