// LLR kernels for 2 bits per axis (16-QAM).
#include "ck_llr_kernels.cuh"

namespace ck {
namespace llr {
template int launch_ka<2, 0, ck_axis_maxlog>(const void*, uint32_t, const ck_axis_maxlog&,
                                                const ck_axis_maxlog&, const NoiseScale&, float*,
                                                cudaStream_t);
template int launch_ka<2, 1, ck_axis_levels>(const void*, uint32_t, const ck_axis_levels&,
                                                const ck_axis_levels&, const NoiseScale&, float*,
                                                cudaStream_t);
template int launch_ka<2, 2, ck_axis_levels>(const void*, uint32_t, const ck_axis_levels&,
                                                const ck_axis_levels&, const NoiseScale&, float*,
                                                cudaStream_t);
}  // namespace llr
}  // namespace ck
