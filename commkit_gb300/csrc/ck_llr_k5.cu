// LLR kernels for 5 bits per axis (1024-QAM).
#include "ck_llr_kernels.cuh"

namespace ck {
namespace llr {
template int launch_ka<5, 0, ck_axis_maxlog>(const void*, uint32_t, const ck_axis_maxlog&,
                                                const ck_axis_maxlog&, const NoiseScale&, float*,
                                                cudaStream_t);
template int launch_ka<5, 1, ck_axis_levels>(const void*, uint32_t, const ck_axis_levels&,
                                                const ck_axis_levels&, const NoiseScale&, float*,
                                                cudaStream_t);
template int launch_ka<5, 2, ck_axis_levels>(const void*, uint32_t, const ck_axis_levels&,
                                                const ck_axis_levels&, const NoiseScale&, float*,
                                                cudaStream_t);
}  // namespace llr
}  // namespace ck
