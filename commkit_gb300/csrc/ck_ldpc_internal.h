// The LDPC decoding plan shared by the host-side plan code and the decoder.
#pragma once

#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "ck_common.cuh"

namespace ck {

// Circulant tables held in shared memory.
constexpr int32_t kMaxBaseRows = 1024;
constexpr int32_t kMaxBlocks = 2048;

}  // namespace ck

struct ck_ldpc_plan;

namespace ck {

// Decode with all device scratch taken from `scratch` (capacity
// `scratch_bytes`, 256-byte aligned); defined in ck_ldpc.cu, used by the
// allocation-free entry point.
int ldpc_decode_in_scratch(const ck_ldpc_plan* plan, const float* llr_in, float* llr_out,
                           int64_t B, int32_t n_in, int32_t rule, float scale, float offset,
                           int32_t max_iterations, int32_t early_stop, int32_t* iters,
                           uint8_t* valid, int8_t* bits, int32_t k_bits, void* scratch,
                           size_t scratch_bytes, cudaStream_t stream);

}  // namespace ck

struct ck_ldpc_plan {
    int device = 0;
    int32_t m = 0, N = 0, E = 0, L = 0;
    int32_t max_deg = 0;
    int32_t max_layer_rows = 0;
    // Quasi-cyclic form: layer l holds base rows [h_layer[l], h_layer[l+1]),
    // base row b has the circulants h_blk[2 i] (j Z + shift), h_blk[2 i + 1]
    // ((j + 1) Z) for i in [h_eptr[b], h_eptr[b+1]); schedule row b Z + r is
    // its row r, with column r + h_blk[2 i] wrapped by Z at h_blk[2 i + 1].
    // CSR form: h_layer is layer_ptr, d_eptr row_ptr, d_cols cols.
    bool qc = false;
    int32_t Z = 0, mb = 0, nb = 0, nnzb = 0;
    std::vector<int32_t> h_layer, h_eptr, h_blk;
    int32_t* d_layer = nullptr;
    int32_t* d_eptr = nullptr;
    int32_t* d_blk = nullptr;
    int32_t* d_cols = nullptr;
    ck::FastDiv divZ{1, 1, 0};
    ck_ldpc_launch launch{0, 0, 0};
    // The decoder's launch shape per check rule for the current launch
    // setting (everything but the grid, which depends on the frame count),
    // resolved on first use: later calls skip the occupancy queries.
    struct ShapeCache {
        bool valid = false;
        ck_ldpc_launch launch{0, 0, 0};
        int32_t jit_mode = 0;
        int per_sm = 0, sms = 0;
        alignas(16) unsigned char resolved[192];
    };
    mutable ShapeCache shape_cache[2];
    mutable std::mutex shape_mu;
    // Code-specialised min-sum kernels (ck_ldpc_jit.cu), compiled on first
    // use: one per message-state placement.
    struct Jit {
        bool tried = false;
        int dmax = 0;
        cudaLibrary_t lib = nullptr;
        const void* kernel[3] = {nullptr, nullptr, nullptr};  // by placement: device, records, edges
        std::string why;  // why there are none
    };
    uint64_t id = 0;  // unique in the process, never reused
    int32_t jit_mode = CK_LDPC_SPECIALISE_AUTO;
    mutable Jit jit;
    mutable std::mutex jit_mu;
};

namespace ck {
// Raises a kernel's dynamic shared-memory limit to the device's opt-in
// maximum (less its static shared memory), once per kernel and device (a
// limit set per call would let plans sharing the kernel lower it under one
// another).
int allow_max_smem(const void* kernel, int device, int optin);
// Drops a kernel from allow_max_smem's record before its module is unloaded
// (a kernel loaded later may get the same handle).
void forget_kernel(const void* kernel);
namespace ldpc {
// Message-state placements of the specialised kernels (kernel index).
constexpr int kPlaceDevice = 0;  // packed records in device memory
constexpr int kPlaceRecords = 1;  // packed records in shared memory
constexpr int kPlaceEdges = 2;  // one message per edge in shared memory
// The plan's code-specialised min-sum kernel for a row-degree bound and a
// message-state placement (compiled on first use), or nullptr in *out when
// the plan has none (specialisation off, NVRTC missing or the compilation
// failed); an error only when the plan requires specialisation.
int specialised_kernel(const ck_ldpc_plan* plan, int dmax, int place, const void** out);
// The same kernel only if an earlier call already compiled it (nullptr in
// *out otherwise): never compiles or loads code, for the allocation-free
// entry point.  An error only when the plan requires specialisation and has
// no compiled kernel.
int specialised_kernel_ready(const ck_ldpc_plan* plan, int place, const void** out);
// The NVRTC source of a circulant plan's specialised kernels.
std::string specialised_source(const ck_ldpc_plan& plan, int dmax);
// The NVRTC source of the specialised mixed kernel of n plans, batch c with
// parts[c] threads per row slot (0: the table loop) and edges[c] its
// per-edge state.
std::string mixed_source(const ck_ldpc_plan* const* plans, const int* parts, const int* edges, int n, int dmax);
// The code-specialised mixed kernel for these plans with threads per frame
// T[c] (batches with T[c] == Zp or 2 Zp, Zp = Z rounded up to whole warps,
// run their code's program, the others the table loop) and edges[c] (a
// batch run by its program with one thread per row slot keeps one message
// per edge in shared memory), compiled on first use; nullptr in *out when
// there is none.
int mixed_specialised_kernel(const ck_ldpc_plan* const* plans, const int32_t* T, const int* edges, int n,
                             int dmax, const void** out);
// Unloads the specialised kernels that use `plan` (before it is freed).
void forget_plan_kernels(const ck_ldpc_plan* plan);
}  // namespace ldpc
}  // namespace ck
