// Allocation-free LDPC decoding: ck_ldpc_decode_static.
//
// Some callers of the decoder cannot allocate device memory while they
// decode: a receiver that runs a fixed real-time loop cannot afford the
// implicit synchronisation and unbounded latency of cudaMalloc/cudaFree in
// the middle of a burst; a host application that hands this library a
// fixed memory budget at start-up cannot have it reach for more later; and
// code embedded in another runtime that owns the device's memory has no
// allocator it may call at all.  For them this entry point decodes with its
// scratch (the frame-queue counter, the status word and the device-memory
// check-message state) taken from the array below, which the CUDA module
// reserves when it loads, so the call itself allocates nothing.
//
// Facts a caller must know:
//  * The array holds CK_LDPC_STATIC_SCRATCH_BYTES (64 MiB) on every GPU
//    where this module gets loaded, until the process exits.
//  * Its device address is looked up with cudaGetSymbolAddress on the first
//    call on each device, with that device current.  That first call should
//    come before any stream capture begins.
//  * Every call on a device shares the same array and the array keeps the
//    last call's contents: each call clears the counter and status word it
//    needs at the start (a memset queued on the call's stream), and the
//    kernel initialises the message state of every frame it decodes.  Calls
//    whose work overlaps on the GPU (two streams, or two host threads on
//    different streams) race on the array; serialise them on one stream.
//  * The decoder's grid is cut to the frame slots that fit in the array; a
//    code whose single block of frames needs more than the array holds is
//    rejected with CK_ERR_UNSUPPORTED.  Codes whose message state lives in
//    shared memory use only the 256-byte header.
//  * Plans (ck_ldpc_plan_create) allocate their tables when they are
//    created, so create them before the allocation-free phase.
//  * It never compiles a code-specialised kernel (NVRTC and the module load
//    allocate): a plan whose specialised kernel an earlier ck_ldpc_decode
//    compiled runs it, any other runs the table-driven kernel, with the
//    same results.
//  * A frame whose bulk LLR copy timed out comes back with iters = -1 and
//    valid = 0, the only timeout signal here (the status word sits in the
//    shared array and the next call clears it).
//  * The address is cached per device ordinal for the life of the process:
//    after cudaDeviceReset the module is reloaded elsewhere, so the entry
//    point must not be used again in that process.
#include <mutex>

#include "ck_ldpc_internal.h"

namespace {

static __device__ __align__(256) unsigned char g_decode_scratch[CK_LDPC_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once).
int scratch_address(int device, void** out) {
    if (device < 0 || device >= kMaxDevices)
        return ck::fail(CK_ERR_UNSUPPORTED, "device %d is beyond the %d this entry point tracks",
                        device, kMaxDevices);
    std::lock_guard<std::mutex> guard(g_lock);
    if (g_scratch_addr[device] == nullptr) {
        void* p = nullptr;
        CK_CUDA(cudaGetSymbolAddress(&p, g_decode_scratch));
        g_scratch_addr[device] = p;
    }
    *out = g_scratch_addr[device];
    return CK_OK;
}

}  // namespace

extern "C" int ck_ldpc_decode_static(const ck_ldpc_plan* plan, const float* llr_in,
                                     float* llr_out, int64_t B, int32_t n_in, int32_t rule,
                                     float scale, float offset, int32_t max_iterations,
                                     int32_t early_stop, int32_t* iters, uint8_t* valid,
                                     int8_t* bits, int32_t k_bits, void* stream) {
    ck::clear_error();
    if (!plan) return ck::fail(CK_ERR_INVALID_ARGUMENT, "plan is NULL");
    int device = -1;
    CK_CUDA(cudaGetDevice(&device));
    if (device != plan->device)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "plan is for device %d, current device is %d",
                        plan->device, device);
    void* scratch = nullptr;
    CK_TRY(scratch_address(device, &scratch));
    return ck::ldpc_decode_in_scratch(plan, llr_in, llr_out, B, n_in, rule, scale, offset,
                                      max_iterations, early_stop, iters, valid, bits, k_bits,
                                      scratch, CK_LDPC_STATIC_SCRATCH_BYTES,
                                      static_cast<cudaStream_t>(stream));
}
