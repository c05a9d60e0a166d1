// M-point LLR kernels for 9-16 bits per symbol (see ck_llr_points.cuh).
#include "ck_llr_points.cuh"

namespace ck {
namespace llr {
namespace points {

template <int K>
int launch_points(const float2* x, uint32_t n, const Table& t, const NoiseScale& noise, bool exact,
                  float* out, cudaStream_t stream) {
    using Kernel = void (*)(const float2*, uint32_t, Table, NoiseScale, float*, bool);
    constexpr bool kSmem = (1 << K) <= kMaxSmemPoints;
    Kernel kernel;
    if constexpr (kSmem)
        kernel = exact ? llr_points_kernel<K, true, true> : llr_points_kernel<K, false, true>;
    else
        kernel = exact ? llr_points_kernel<K, true, false> : llr_points_kernel<K, false, false>;
    const int bytes = kSmem ? static_cast<int>(smem_bytes(K, exact)) : 0;
    // Shared-memory opt-in and occupancy, once per device and method (the
    // writes are idempotent, so concurrent first calls are harmless).
    static int per_sm_cache[2][kMaxDevices] = {};
    int dev = 0;
    CK_CUDA(cudaGetDevice(&dev));
    int per_sm = dev < kMaxDevices ? per_sm_cache[exact][dev] : 0;
    if (per_sm == 0) {
        if (bytes > 48 * 1024)
            CK_CUDA(cudaFuncSetAttribute(reinterpret_cast<const void*>(kernel),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        CK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(kernel),
                                                              kThreads, bytes));
        if (per_sm < 1) return ck::fail(CK_ERR_UNSUPPORTED, "M-point LLR block does not fit an SM");
        if (dev < kMaxDevices) per_sm_cache[exact][dev] = per_sm;
    }
    // Staged tables run two symbols per thread and step for the exact method.
    const uint32_t units = kSmem && exact ? n / 2 + (n & 1u) : n;
    const uint32_t want = (units + kThreads - 1) / kThreads;
    const uint32_t cap = static_cast<uint32_t>(num_sms()) * static_cast<uint32_t>(per_sm);
    const uint32_t blocks = want < cap ? (want > 0 ? want : 1) : cap;
    const bool vec = reinterpret_cast<uintptr_t>(out) % 16 == 0;
    kernel<<<blocks, kThreads, bytes, stream>>>(x, n, t, noise, out, vec);
    return ck::cuda_check(cudaGetLastError(), "M-point LLR kernel launch");
}

template int launch_points<9>(const float2*, uint32_t, const Table&, const NoiseScale&, bool, float*, cudaStream_t);
template int launch_points<10>(const float2*, uint32_t, const Table&, const NoiseScale&, bool, float*, cudaStream_t);
template int launch_points<11>(const float2*, uint32_t, const Table&, const NoiseScale&, bool, float*, cudaStream_t);
template int launch_points<12>(const float2*, uint32_t, const Table&, const NoiseScale&, bool, float*, cudaStream_t);
template int launch_points<13>(const float2*, uint32_t, const Table&, const NoiseScale&, bool, float*, cudaStream_t);
template int launch_points<14>(const float2*, uint32_t, const Table&, const NoiseScale&, bool, float*, cudaStream_t);
template int launch_points<15>(const float2*, uint32_t, const Table&, const NoiseScale&, bool, float*, cudaStream_t);
template int launch_points<16>(const float2*, uint32_t, const Table&, const NoiseScale&, bool, float*, cudaStream_t);

}  // namespace points
}  // namespace llr
}  // namespace ck
