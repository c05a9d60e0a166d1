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

extern "C" void ck_host_publish(uint32_t* counter, uint32_t value);

extern "C" int ck_ldpc_feed_publish(ck_ldpc_feed_frame* ring, uint32_t capacity, int32_t* iters_ring,
                                    uint32_t* published, uint32_t first, int32_t frames, const void* symbols,
                                    int64_t symbol_bytes, float* llr_out, int32_t n_in, int8_t* bits,
                                    int32_t k_bits, uint8_t* valid, float inv_s2, uint32_t seq0) {
    ck::clear_error();
    if (!ring || !iters_ring || !published || !symbols || !llr_out || !valid)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "ring, iters_ring, published, symbols, llr_out and valid are required");
    if (capacity < 1 || (capacity & (capacity - 1)))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "capacity %u is not a power of two", capacity);
    if (frames < 0 || static_cast<uint32_t>(frames) > capacity)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "frames must be in [0, capacity], got %d", frames);
    if (n_in < 1 || k_bits < 0 || symbol_bytes < 0)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "bad n_in, k_bits or symbol_bytes");
    const uint32_t mask = capacity - 1u;
    const char* sym = static_cast<const char*>(symbols);
    for (int32_t f = 0; f < frames; ++f) {
        const uint32_t slot = (first + static_cast<uint32_t>(f)) & mask;
        iters_ring[slot] = -2;
        ck_ldpc_feed_frame& d = ring[slot];
        d.symbols = sym + static_cast<int64_t>(f) * symbol_bytes;
        d.llr_out = llr_out + static_cast<int64_t>(f) * n_in;
        d.bits = bits ? bits + static_cast<int64_t>(f) * k_bits : nullptr;
        d.iters = iters_ring + slot;
        d.valid = valid + f;
        d.inv_s2 = inv_s2;
        d.seq = seq0 + static_cast<uint32_t>(f);
    }
    ck_host_publish(published, first + static_cast<uint32_t>(frames));
    return CK_OK;
}

// A release store on the calling host thread: every store it made before
// (a feed ring's descriptors) is visible to a reader that loads `value`
// with acquire semantics (the feed decoder's ld.acquire.sys).
extern "C" void ck_host_publish(uint32_t* counter, uint32_t value) {
    std::atomic_thread_fence(std::memory_order_release);
    __atomic_store_n(counter, value, __ATOMIC_RELEASE);
}
