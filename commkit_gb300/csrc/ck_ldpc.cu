// Layered min-sum LDPC decoding on sm_103a.
//
// The GB300-first replacement of the reference's `ldpc_layered<false>`
// kernel (commkit/_cuda/src/ldpc.cu:107-159) behind its launcher
// (commkit/_cuda/coding.py:27-67).  Same recursion, same layer order, the
// same float32 operations in the same rounding (explicit _rn intrinsics, no
// FMA), so a-posteriori LLRs, hard decisions, iteration counts and the
// syndrome flag are bit-identical; what changes is where the data lives and
// how the work is spread:
//
//  * Persistent frame groups.  The grid is sized to fill the GPU once
//    (SMs x resident blocks); each block holds G frame groups of T threads
//    and each group pulls frame after frame from a device queue (one atomic
//    per frame).  Frames that converge early free their group for the next
//    frame, so uneven iteration counts do not leave SMs idle, and scratch
//    memory is bounded by the grid, not by the batch.
//  * The frame's posterior LLRs live in shared memory for the whole decode,
//    staged in by one bulk (TMA) copy; a layer's updates are shared-memory
//    gathers and scatters, conflict-free for circulants (lanes handle
//    consecutive rows of a circulant, so they touch consecutive columns).
//  * Check-to-variable messages are stored losslessly compressed: a min-sum
//    message of row i edge e is sign_e * (e == argmin ? min2' : min1'), so
//    a row keeps (min1', min2', one word of 27 sign bits + a 5-bit argmin),
//    12 bytes instead of 4 per edge.  The state sits in shared memory beside
//    the LLRs when both fit, else in device memory, where the working set of
//    the resident frames stays in L2.
//  * Quasi-cyclic codes use circulant tables (block column, shift) in shared
//    memory, so a row's columns are computed, not loaded; other codes read
//    the CSR schedule.
//  * The syndrome test runs over chunks of rows with a barrier-OR per chunk
//    and stops at the first unsatisfied chunk, so a failing iteration pays
//    for one chunk, not for the whole matrix.
//
// Within a row the min1/min2/argmin/sign-parity reduction is a multiset
// computation (min2 is the second smallest magnitude counting repeats, the
// argmin the first edge holding min1), so splitting it differently does not
// change a bit; rows of one layer share no variable, and layers run in the
// schedule's order, as in the reference.
#include <math_constants.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <utility>

#include "ck_ldpc_cluster.cuh"
#include "ck_ldpc_kernel.cuh"
#include "ck_ldpc_minsum.cuh"
#include "ck_ldpc_mixed.cuh"


using namespace ck::ldpc;

static_assert(kMaxMixed == CK_LDPC_MAX_MIXED, "mixed-launch code count");


namespace ck {
namespace ldpc {

// The packed state for row-degree bounds up to 27, the wide one for any
// degree (DMAX = 0).
template <int DMAX, template <bool> class State>
struct MinSumPickOf {
    template <bool QC, bool ONE_ROW>
    static KernelFn get(bool app_smem, bool r_smem) {
        if (app_smem && r_smem) return decode_kernel<State, QC, DMAX, true, true, ONE_ROW>;
        if (app_smem) return decode_kernel<State, QC, DMAX, true, false, ONE_ROW>;
        if constexpr (!QC) return decode_kernel<State, QC, DMAX, false, false, false>;
        return nullptr;
    }
};
struct MinSumPick {
    template <bool QC, int DMAX, bool ONE_ROW>
    static KernelFn get(bool app_smem, bool r_smem) {
        if constexpr (DMAX == 0)
            return MinSumPickOf<0, WideMinSumState>::template get<QC, ONE_ROW>(app_smem, r_smem);
        else
            return MinSumPickOf<DMAX, MinSumState>::template get<QC, ONE_ROW>(app_smem, r_smem);
    }
};

KernelFn min_sum_kernel(bool qc, int max_deg, bool app_smem, bool r_smem, bool one_row) {
    return pick_shape<MinSumPick>(qc, max_deg, app_smem, r_smem, one_row);
}

KernelFn min_sum_cluster_kernel(int max_deg) {
    switch (kernel_dmax(false, max_deg)) {
        case 8: return decode_cluster_kernel<MinSumState, 8>;
        case 16: return decode_cluster_kernel<MinSumState, 16>;
        case 27: return decode_cluster_kernel<MinSumState, 27>;
        default: return decode_cluster_kernel<WideMinSumState, 0>;
    }
}

}  // namespace ldpc
}  // namespace ck

namespace {


uint32_t align_up(uint32_t v, uint32_t a) { return (v + a - 1) / a * a; }

struct Resolved {
    const void* kernel;  // a __global__ function, or a code-specialised kernel handle
    int32_t T, G;
    bool app_smem, r_smem;
    uint32_t tables_bytes, group_bytes, gblk_off, app_off, r_off, r_stride, smem;
    int32_t app_stride;
    int grid;
    size_t r_slot_bytes;  // message state of one frame slot in device memory (0 in shared)
    size_t ws_bytes, r_ws_off, app_ws_off;
    // CSR codes with the posterior in device memory: the cluster kernel, and
    // the cluster size a decode uses (1: the plain kernel).
    KernelFn cluster_kernel;
    int cluster_per_sm;
    int cluster;
    int plain_grid;  // the plain kernel's grid for the same frames
    int32_t sign_words;  // wide min-sum state: sign words per row (0: packed or sum-product)
    bool edges;  // min-sum with one message per edge in shared memory (CK_LDPC_PLACE_EDGES)
};

constexpr int kMaxCluster = 8;  // the portable cluster size

constexpr size_t kHeaderBytes = 256;
static_assert(4 * kMaxMixed <= kHeaderBytes, "the mixed launch's queue counters sit in the header");

int device_limits(int dev, int* sms, int* smem_optin) {
    CK_CUDA(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev));
    CK_CUDA(cudaDeviceGetAttribute(smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    return CK_OK;
}

// Launch shape, shared-memory layout, grid and workspace of a decode of B
// frames by `rule`; a pure function of the plan, its launch setting, the
// rule and B.  may_compile false: a code-specialised kernel only if one is
// compiled already (no NVRTC, no module load), and nothing cached.
int resolve_shape(const ck_ldpc_plan* plan, int32_t rule, Resolved* r, int* per_sm_out, int* sms_out,
                  bool may_compile);

int resolve(const ck_ldpc_plan* plan, int32_t rule, int64_t B, Resolved* r, bool may_compile = true) {
    if (rule != CK_LDPC_MIN_SUM && rule != CK_LDPC_SUM_PRODUCT)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "unknown check rule %d", rule);
    static_assert(sizeof(Resolved) <= sizeof(plan->shape_cache[0].resolved), "shape cache too small");
    int per_sm = 0, sms = 0;
    {
        std::lock_guard<std::mutex> lock(plan->shape_mu);
        auto& c = plan->shape_cache[rule];
        if (c.valid && memcmp(&c.launch, &plan->launch, sizeof(ck_ldpc_launch)) == 0 &&
            c.jit_mode == plan->jit_mode) {
            memcpy(static_cast<void*>(r), c.resolved, sizeof(Resolved));
            per_sm = c.per_sm;
            sms = c.sms;
        } else if (!may_compile) {
            CK_TRY(resolve_shape(plan, rule, r, &per_sm, &sms, false));
        } else {
            CK_TRY(resolve_shape(plan, rule, r, &per_sm, &sms, true));
            memcpy(c.resolved, static_cast<const void*>(r), sizeof(Resolved));
            c.launch = plan->launch;
            c.jit_mode = plan->jit_mode;
            c.per_sm = per_sm;
            c.sms = sms;
            c.valid = true;
        }
    }
    int32_t G = r->G;
    r->cluster = 1;
    size_t slots;
    if (r->cluster_kernel && B * 2 <= int64_t(sms) * r->cluster_per_sm) {
        // Fewer frames than the GPU holds: a cluster of C CTAs per frame, the
        // largest C whose clusters can all be resident at once.
        for (int c = kMaxCluster; c >= 2; c /= 2) {
            if (B * c > int64_t(sms) * r->cluster_per_sm) continue;
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute attr;
            attr.id = cudaLaunchAttributeClusterDimension;
            attr.val.clusterDim.x = c;
            attr.val.clusterDim.y = 1;
            attr.val.clusterDim.z = 1;
            cfg.gridDim = dim3(static_cast<unsigned>(B * c));
            cfg.blockDim = dim3(static_cast<unsigned>(r->T));
            cfg.attrs = &attr;
            cfg.numAttrs = 1;
            int clusters = 0;
            if (cudaOccupancyMaxActiveClusters(&clusters, reinterpret_cast<const void*>(r->cluster_kernel), &cfg) !=
                cudaSuccess) {
                (void)cudaGetLastError();
                continue;
            }
            if (clusters >= B) {
                r->cluster = c;
                break;
            }
        }
    }
    if (r->cluster <= 1 && B > 0 && B < int64_t(sms) * per_sm * G) {
        // Less than one resident wave: spread the frames over every resident
        // block (fewer frame groups per block, the same kernel) instead of
        // filling the first blocks and leaving SMs idle.  Any shape gives the
        // same bits.
        const int64_t blocks = int64_t(sms) * per_sm;
        const int32_t g2 = static_cast<int32_t>((B + blocks - 1) / blocks);
        if (g2 >= 1 && g2 < G) {
            G = g2;
            r->G = g2;
            r->smem = r->tables_bytes + static_cast<uint32_t>(g2) * r->group_bytes;
        }
    }
    const int64_t need = (B + G - 1) / G;
    r->plain_grid = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(need, int64_t(sms) * per_sm)));
    if (r->cluster > 1) {
        r->grid = static_cast<int>(B * r->cluster);
        slots = static_cast<size_t>(B);  // one frame slot per cluster
    } else {
        r->grid = r->plain_grid;
        slots = static_cast<size_t>(r->grid) * G;
    }
    r->r_ws_off = kHeaderBytes;
    const size_t r_ws = slots * r->r_slot_bytes;
    r->app_ws_off = kHeaderBytes + ((r_ws + 255) / 256) * 256;
    const size_t app_ws = r->app_smem ? 0 : slots * static_cast<size_t>(r->app_stride) * 4;
    r->ws_bytes = r->app_ws_off + app_ws;
    return CK_OK;
}

// Everything of a decode's launch that does not depend on the frame count.
int resolve_shape(const ck_ldpc_plan* plan, int32_t rule, Resolved* r, int* per_sm_out, int* sms_out,
                  bool may_compile) {
    const bool sp = rule == CK_LDPC_SUM_PRODUCT;
    int sms = 0, optin = 0;
    CK_TRY(device_limits(plan->device, &sms, &optin));
    const uint32_t tables =
        plan->qc ? align_up(align_up(static_cast<uint32_t>(plan->L + 1 + plan->mb + 1) * 4, 8) +
                                static_cast<uint32_t>(plan->nnzb) * 8,
                            128)
                 : align_up(static_cast<uint32_t>(plan->L + 1) * 4, 128);
    const uint32_t ctrl = 128;
    const uint32_t app_bytes = align_up(static_cast<uint32_t>(plan->N) * 4, 128);
    // Message state per frame: min-sum keeps a 16-byte record per row in
    // shared memory (12 bytes in device memory), or for rows above 27 edges
    // the wide state's 3 + sign_words words per row in either; sum-product
    // one float per edge in either.
    const int32_t sign_words = (!sp && plan->max_deg > kPackedDegree) ? (plan->max_deg + 31) / 32 : 0;
    const uint32_t r_stride = align_up(static_cast<uint32_t>(sp ? plan->E : plan->m), 32);
    const uint32_t r_bytes = r_stride * (sp ? 4 : (sign_words ? 4 * (3 + sign_words) : 16));  // in shared memory
    const uint32_t r_bytes_dev = r_stride * (sp ? 4 : (sign_words ? 4 * (3 + sign_words) : 12));  // in device memory
    // Per group: its copy of the circulant table with shared addresses.
    const uint32_t gblk_bytes = plan->qc ? align_up(static_cast<uint32_t>(plan->nnzb) * 8, 128) : 0;
    const uint32_t budget = static_cast<uint32_t>(optin) > tables ? optin - tables : 0;

    bool app_smem = ctrl + gblk_bytes + app_bytes <= budget;
    if (plan->qc && !app_smem)
        return ck::fail(CK_ERR_UNSUPPORTED,
                        "quasi-cyclic code of N = %d: its posterior (%u bytes) does not fit in shared "
                        "memory",
                        plan->N, app_bytes);
    int32_t T = plan->launch.threads_per_frame;
    const int32_t Zp = plan->qc ? (plan->Z + 31) / 32 * 32 : 0;
    if (T == 0) {
        if (plan->qc) {
            // One base row's rows per round: the padded lifting, halved while
            // above 512 threads and still a multiple of 32.
            T = Zp;
            while (T > 512 && T % 64 == 0) T /= 2;
        } else {
            const int32_t avg = std::max(1, plan->m / plan->L);
            T = 32;
            while (T < 512 && T < avg / 2) T *= 2;
        }
    }
    if (plan->qc && T % Zp != 0 && Zp % T != 0)
        return ck::fail(CK_ERR_INVALID_ARGUMENT,
                        "threads_per_frame %d must divide or be a multiple of %d (the lifting %d "
                        "rounded up to whole warps)",
                        T, Zp, plan->Z);
    const int32_t max_threads = max_block_threads(plan->qc, kernel_dmax(plan->qc, plan->max_deg));
    if (T > max_threads)
        return ck::fail(CK_ERR_INVALID_ARGUMENT,
                        "threads_per_frame %d above %d for row degree %d", T, max_threads,
                        plan->max_deg);

    bool r_smem;
    uint32_t r_used = r_bytes, r_stride_used = r_stride;
    // A plan's frames per block and placement are min-sum shapes (tuned or
    // set); sum-product, whose per-edge state is several times larger,
    // always picks its own.
    const int32_t place = sp ? CK_LDPC_PLACE_AUTO : plan->launch.placement;
    // One message per edge in shared memory: the code-specialised kernel of a
    // circulant code with rows up to 27 edges and one thread per row slot,
    // when a frame fits (EDGES) or two frames fit per block budget (AUTO:
    // measured faster than the records on codes A and B); otherwise (or when
    // its kernel is unavailable) the records as SHARED (AUTO as before).
    const void* edge_kernel = nullptr;
    if ((place == CK_LDPC_PLACE_EDGES || place == CK_LDPC_PLACE_AUTO) && !sp && plan->qc && app_smem && T == Zp &&
        plan->max_deg <= kPackedDegree) {
        const uint32_t e_stride = align_up(static_cast<uint32_t>(plan->E), 32);
        const uint32_t frames = place == CK_LDPC_PLACE_AUTO ? 2 : 1;
        if (frames * (ctrl + gblk_bytes + app_bytes + e_stride * 4) <= budget) {
            if (may_compile)
                CK_TRY(specialised_kernel(plan, kernel_dmax(true, plan->max_deg), kPlaceEdges, &edge_kernel));
            else
                CK_TRY(specialised_kernel_ready(plan, kPlaceEdges, &edge_kernel));
            if (edge_kernel) {
                r_used = e_stride * 4;
                r_stride_used = e_stride;
            }
        }
    }
    if (edge_kernel) {
        r_smem = true;
    } else if (!app_smem || place == CK_LDPC_PLACE_GLOBAL) {
        r_smem = false;
    } else if (place == CK_LDPC_PLACE_SHARED || place == CK_LDPC_PLACE_EDGES) {
        r_smem = ctrl + gblk_bytes + app_bytes + r_bytes <= budget;
    } else {
        // Auto: beside the LLRs when two frames still fit per block budget.
        r_smem = 2 * (ctrl + gblk_bytes + app_bytes + r_bytes) <= budget;
    }
    uint32_t group = ctrl + gblk_bytes + (app_smem ? app_bytes : 0) + (r_smem ? r_used : 0);
    int32_t G = sp ? 0 : plan->launch.frames_per_block;
    const int32_t gmax_threads = max_threads / T;
    const int32_t gmax_smem = static_cast<int32_t>(budget / group);
    const int32_t gmax_bar = T > 32 ? ck::kMaxNamedGroups : 32;
    const int32_t gmax = std::min(gmax_threads, std::min(gmax_smem, gmax_bar));
    if (gmax < 1)
        return ck::fail(CK_ERR_UNSUPPORTED, "a frame needs %u bytes of shared memory, %u available",
                        group, budget);
    const bool one_row = plan->qc && T >= Zp;
    const KernelFn table = sp ? sum_product_kernel(plan->qc, plan->max_deg, app_smem, r_smem, one_row)
                              : min_sum_kernel(plan->qc, plan->max_deg, app_smem, r_smem, one_row);
    if (!table) return ck::fail(CK_ERR_UNSUPPORTED, "no decoder kernel for this code shape");
    const void* kernel = reinterpret_cast<const void*>(table);
    if (edge_kernel) {
        kernel = edge_kernel;
    } else if (!sp && plan->qc && T == Zp && app_smem && plan->max_deg <= kPackedDegree) {
        // The code-specialised kernel, where the plan has one (codes with
        // rows above 27 edges have none: they run the any-degree kernels).
        const void* special = nullptr;
        const int kind = r_smem ? kPlaceRecords : kPlaceDevice;
        if (may_compile)
            CK_TRY(specialised_kernel(plan, kernel_dmax(true, plan->max_deg), kind, &special));
        else
            CK_TRY(specialised_kernel_ready(plan, kind, &special));
        if (special) kernel = special;
    }
    CK_TRY(ck::allow_max_smem(kernel, plan->device, optin));
    if (G == 0) {
        // The most resident frames per SM (registers, shared memory, threads),
        // the smaller block on a tie.
        int best = 0;
        for (int32_t g = 1; g <= gmax; ++g) {
            int per_sm = 0;
            CK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, T * g, tables + g * group));
            if (per_sm * g > best) {
                best = per_sm * g;
                G = g;
            }
        }
        if (G == 0) G = 1;
    }
    if (G > gmax)
        return ck::fail(CK_ERR_INVALID_ARGUMENT,
                        "frames_per_block %d above the %d that fit (threads, shared memory, "
                        "barriers)",
                        G, gmax);

    r->kernel = kernel;
    r->T = T;
    r->G = G;
    r->app_smem = app_smem;
    r->r_smem = r_smem;
    r->tables_bytes = tables;
    r->group_bytes = group;
    r->gblk_off = ctrl;
    r->app_off = ctrl + gblk_bytes;
    r->r_off = ctrl + gblk_bytes + (app_smem ? app_bytes : 0);
    r->r_stride = r_stride_used;
    r->edges = edge_kernel != nullptr;
    r->smem = tables + static_cast<uint32_t>(G) * group;
    r->app_stride = static_cast<int32_t>(app_bytes / 4);
    r->sign_words = sign_words;

    int per_sm = 0;
    CK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, r->kernel, T * G, r->smem));
    if (per_sm < 1)
        return ck::fail(CK_ERR_UNSUPPORTED,
                        "decoder block of %d threads and %u bytes of shared memory does not fit "
                        "an SM",
                        T * G, r->smem);
    r->r_slot_bytes = r_smem ? 0 : r_bytes_dev;
    r->cluster_kernel = nullptr;
    r->cluster_per_sm = 0;
    r->cluster = 1;
    if (!plan->qc && !app_smem && !r_smem) {
        KernelFn ck = sp ? sum_product_cluster_kernel(plan->max_deg) : min_sum_cluster_kernel(plan->max_deg);
        int cps = 0;
        CK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cps, reinterpret_cast<const void*>(ck), T, 0));
        if (cps >= 1) {
            r->cluster_kernel = ck;
            r->cluster_per_sm = cps;
        }
    }
    *per_sm_out = per_sm;
    *sms_out = sms;
    return CK_OK;
}

// Launches a resolved decode: the plain kernel, or the cluster kernel with
// its cluster size.
int launch_decode(const Resolved& r, const Params& p, cudaStream_t s) {
    if (r.cluster <= 1) {
        void* args[] = {const_cast<Params*>(&p)};
        return ck::cuda_check(cudaLaunchKernel(r.kernel, dim3(static_cast<unsigned>(r.grid)),
                                               dim3(static_cast<unsigned>(r.T * r.G)), args, r.smem, s),
                              "decoder launch");
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = static_cast<unsigned>(r.cluster);
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.gridDim = dim3(static_cast<unsigned>(r.grid));
    cfg.blockDim = dim3(static_cast<unsigned>(r.T));
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return ck::cuda_check(cudaLaunchKernelEx(&cfg, r.cluster_kernel, p), "cluster decoder launch");
}

int check_device(const ck_ldpc_plan* plan) {
    int dev = -1;
    CK_CUDA(cudaGetDevice(&dev));
    if (dev != plan->device)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "plan is for device %d, current device is %d",
                        plan->device, dev);
    return CK_OK;
}

// Argument checks shared by the decode entry points (the reference's
// wrapper checks, commkit/_cuda/coding.py:27-67, plus this ABI's own).
// The min-sum parameters the reference's MinSum accepts
// (commkit/coding/ldpc.py:345-347): scale finite in (0, 1], offset finite
// and >= 0.  A C caller gets the same refusal as a Python one, before any
// launch.
int check_min_sum_params(float scale, float offset) {
    if (!(scale > 0.0f && scale <= 1.0f))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "scale must be in (0, 1], got %g", static_cast<double>(scale));
    if (!(offset >= 0.0f && offset <= 3.4028234663852886e38f))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "offset must be finite and >= 0, got %g",
                        static_cast<double>(offset));
    return CK_OK;
}

int check_decode_args(const ck_ldpc_plan* plan, const float* llr_in, const float* llr_out,
                      int64_t B, int32_t n_in, int32_t rule, float scale, float offset,
                      int32_t max_iterations, const int32_t* iters, const uint8_t* valid,
                      const int8_t* bits, int32_t k_bits) {
    if (!plan) return ck::fail(CK_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (rule != CK_LDPC_MIN_SUM && rule != CK_LDPC_SUM_PRODUCT)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "unknown check rule %d", rule);
    if (rule == CK_LDPC_MIN_SUM) CK_TRY(check_min_sum_params(scale, offset));
    if (B < 0 || B >= (int64_t(1) << 31))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "B must be in [0, 2**31), got %lld",
                        static_cast<long long>(B));
    if (n_in < 1 || n_in > plan->N)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "n_in must be in [1, N=%d], got %d", plan->N,
                        n_in);
    if (max_iterations < 0)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "max_iterations must be >= 0");
    if (bits && (k_bits < 0 || k_bits > n_in))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "k_bits must be in [0, n_in]");
    if (B == 0) return CK_OK;
    if (!llr_in || !llr_out || !iters || !valid)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "llr_in, llr_out, iters and valid are required");
    if (reinterpret_cast<uintptr_t>(llr_in) % 4 || reinterpret_cast<uintptr_t>(llr_out) % 4)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "LLR buffers must be 4-byte aligned");
    return CK_OK;
}

// Kernel parameters of a resolved decode over the workspace `wsb`.
Params make_params(const ck_ldpc_plan* plan, const Resolved& r, const float* llr_in, float* llr_out,
                   int64_t B, int32_t n_in, float scale, float offset, int32_t max_iterations,
                   int32_t early_stop, int32_t* iters, uint8_t* valid, int8_t* bits,
                   int32_t k_bits, unsigned char* wsb) {
    Params p;
    p.llr_in = llr_in;
    p.llr_out = llr_out;
    p.B = static_cast<uint32_t>(B);
    p.n_in = n_in;
    p.iters = iters;
    p.valid = valid;
    p.bits = k_bits > 0 ? bits : nullptr;
    p.k_bits = k_bits;
    p.N = plan->N;
    p.m = plan->m;
    p.L = plan->L;
    p.E = plan->E;
    p.Z = plan->qc ? plan->Z : 1;
    p.mb = plan->qc ? plan->mb : 0;
    p.nnzb = plan->qc ? plan->nnzb : 0;
    p.divZ = plan->divZ;
    p.Zp = plan->qc ? (plan->Z + 31) / 32 * 32 : 32;
    p.q_bstep = (plan->qc && r.T >= p.Zp) ? r.T / p.Zp : 1;
    p.layer = plan->d_layer;
    p.eptr = plan->d_eptr;
    p.blk = reinterpret_cast<const int2*>(plan->d_blk);
    p.cols = plan->d_cols;
    p.scale = scale;
    p.offset = offset;
    p.max_iterations = max_iterations;
    p.early_stop = early_stop ? 1 : 0;
    p.T = r.T;
    p.G = r.G;
    p.tables_bytes = r.tables_bytes;
    p.group_bytes = r.group_bytes;
    p.gblk_off = r.gblk_off;
    p.app_off = r.app_off;
    p.r_off = r.r_off;
    p.r_stride = r.r_stride;
    p.bulk_load = (r.app_smem && (static_cast<uint32_t>(n_in) * 4u) % 16u == 0 &&
                   reinterpret_cast<uintptr_t>(llr_in) % 16 == 0)
                      ? 1
                      : 0;
    p.counter = reinterpret_cast<uint32_t*>(wsb);
    p.status = reinterpret_cast<uint32_t*>(wsb + 4);
    p.g_r = reinterpret_cast<uint32_t*>(wsb + r.r_ws_off);
    p.g_app = reinterpret_cast<float*>(wsb + r.app_ws_off);
    p.app_stride = r.app_stride;
    p.sign_words = r.sign_words;
    return p;
}

}  // namespace

extern "C" int ck_ldpc_workspace_size(const ck_ldpc_plan* plan, int64_t B, int32_t rule,
                                      size_t* bytes) {
    ck::clear_error();
    if (!plan || !bytes) return ck::fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
    if (B < 0) return ck::fail(CK_ERR_INVALID_ARGUMENT, "B must be >= 0");
    CK_TRY(check_device(plan));
    Resolved r;
    CK_TRY(resolve(plan, rule, std::max<int64_t>(B, 1), &r));
    *bytes = r.ws_bytes;
    return CK_OK;
}

extern "C" int ck_ldpc_decode(const ck_ldpc_plan* plan, const float* llr_in, float* llr_out,
                              int64_t B, int32_t n_in, int32_t rule, float scale, float offset,
                              int32_t max_iterations, int32_t early_stop, int32_t* iters,
                              uint8_t* valid, int8_t* bits, int32_t k_bits, void* workspace,
                              size_t workspace_bytes, void* stream) {
    ck::clear_error();
    CK_TRY(check_decode_args(plan, llr_in, llr_out, B, n_in, rule, scale, offset, max_iterations,
                             iters, valid, bits, k_bits));
    if (B == 0) return CK_OK;
    CK_TRY(check_device(plan));
    Resolved r;
    CK_TRY(resolve(plan, rule, B, &r));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void* ws = workspace;
    bool owned = false;
    if (ws == nullptr) {
        CK_CUDA(cudaMallocAsync(&ws, r.ws_bytes, s));
        owned = true;
    } else {
        if (workspace_bytes < r.ws_bytes)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "workspace of %zu bytes, %zu needed",
                            workspace_bytes, r.ws_bytes);
        if (reinterpret_cast<uintptr_t>(ws) % 256)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    }
    unsigned char* wsb = static_cast<unsigned char*>(ws);
    int status = ck::cuda_check(cudaMemsetAsync(wsb, 0, kHeaderBytes, s), "cudaMemsetAsync");
    const Params p = make_params(plan, r, llr_in, llr_out, B, n_in, scale, offset, max_iterations,
                                 early_stop, iters, valid, bits, k_bits, wsb);
    if (status == CK_OK) status = launch_decode(r, p, s);
    if (owned) {
        const int st = ck::cuda_check(cudaFreeAsync(ws, s), "cudaFreeAsync");
        if (status == CK_OK) status = st;
    }
    return status;
}

extern "C" int ck_ldpc_workspace_status(const void* workspace, void* stream) {
    ck::clear_error();
    if (!workspace) return ck::fail(CK_ERR_INVALID_ARGUMENT, "workspace is NULL");
    uint32_t status = 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    CK_CUDA(cudaMemcpyAsync(&status, static_cast<const unsigned char*>(workspace) + 4,
                            sizeof(status), cudaMemcpyDeviceToHost, s));
    CK_CUDA(cudaStreamSynchronize(s));
    if (status & ck::kStatusTimeout)
        return ck::fail(CK_ERR_DEVICE_TIMEOUT, "a bulk copy of the decoder did not complete");
    return CK_OK;
}

// Decode into caller-provided scratch of a fixed capacity (the allocation-free
// entry point of ck_ldpc_static.cu): the same kernels and launch shape as
// ck_ldpc_decode, with the persistent grid cut down to the frame slots whose
// device-memory state fits in `scratch_bytes`.  Frames beyond the slots wait
// in the device queue, so any B fits; a code whose one slot does not fit is
// rejected.  It never compiles a code-specialised kernel (that loads a module,
// which allocates): it uses one only when an earlier ck_ldpc_decode of the
// plan compiled it, else the table-driven kernel, with the same results.
int ck::ldpc_decode_in_scratch(const ck_ldpc_plan* plan, const float* llr_in, float* llr_out,
                               int64_t B, int32_t n_in, int32_t rule, float scale, float offset,
                               int32_t max_iterations, int32_t early_stop, int32_t* iters,
                               uint8_t* valid, int8_t* bits, int32_t k_bits, void* scratch,
                               size_t scratch_bytes, cudaStream_t s) {
    CK_TRY(check_decode_args(plan, llr_in, llr_out, B, n_in, rule, scale, offset, max_iterations,
                             iters, valid, bits, k_bits));
    if (B == 0) return CK_OK;
    if (reinterpret_cast<uintptr_t>(scratch) % 256)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "scratch must be 256-byte aligned");
    CK_TRY(check_device(plan));
    Resolved r;
    CK_TRY(resolve(plan, rule, B, &r, false));
    // The static scratch serves the plain kernel's frame slots.
    r.cluster = 1;
    r.grid = r.plain_grid;
    // Bytes of device-memory state per frame slot (the header is shared).
    const size_t app_bytes = r.app_smem ? 0 : static_cast<size_t>(r.app_stride) * 4;
    const size_t per_slot = r.r_slot_bytes + app_bytes;
    if (per_slot > 0) {
        const size_t usable = scratch_bytes > kHeaderBytes + 256 ? scratch_bytes - kHeaderBytes - 256 : 0;
        const size_t max_slots = usable / per_slot;
        if (max_slots < static_cast<size_t>(r.G))
            return ck::fail(CK_ERR_UNSUPPORTED,
                            "one block of %d frames needs %zu bytes of scratch, the static "
                            "scratch holds %zu",
                            r.G, kHeaderBytes + 256 + per_slot * r.G, scratch_bytes);
        const int grid_cap = static_cast<int>(max_slots / r.G);
        if (r.grid > grid_cap) r.grid = grid_cap;
    }
    const size_t slots = static_cast<size_t>(r.grid) * r.G;
    r.r_ws_off = kHeaderBytes;
    r.app_ws_off = kHeaderBytes + ((slots * r.r_slot_bytes + 255) / 256) * 256;
    r.ws_bytes = r.app_ws_off + slots * app_bytes;
    if (r.ws_bytes > scratch_bytes)
        return ck::fail(CK_ERR_UNSUPPORTED, "decode needs %zu bytes of scratch, %zu available",
                        r.ws_bytes, scratch_bytes);
    unsigned char* wsb = static_cast<unsigned char*>(scratch);
    // The queue counter and status word must start at zero on every call.
    CK_CUDA(cudaMemsetAsync(wsb, 0, kHeaderBytes, s));
    const Params p = make_params(plan, r, llr_in, llr_out, B, n_in, scale, offset, max_iterations,
                                 early_stop, iters, valid, bits, k_bits, wsb);
    return launch_decode(r, p, s);
}

// ---------------------------------------------------------------------------
// Mixed-code launch
// ---------------------------------------------------------------------------

namespace {

struct MixedResolved {
    MixedParams p;
    const void* kernel;  // the table-driven kernel or a code-specialised one
    int block_threads;
    uint32_t smem;
    int grid;
    size_t ws_bytes;
    uint32_t block_words;  // device-memory message state per block, shared by the codes
    bool wide;  // some code has rows above degree 16
    bool any_degree;  // some code has rows above degree 27: the any-degree kernel, wide state for all
    bool edges;  // some code keeps one message per edge (r_smem == 2; its specialised program only)
};

// Occupancy per (kernel, device, block shape), remembered: the request
// server launches a mixed batch per admission.  forget_kernel drops a
// kernel's entries.
std::mutex g_occ_mu;
std::map<std::tuple<const void*, int, int, uint32_t>, int> g_occ;

int mixed_occupancy(const void* kernel, int dev, int threads, uint32_t smem, int* per_sm) {
    const auto key = std::make_tuple(kernel, dev, threads, smem);
    std::lock_guard<std::mutex> lock(g_occ_mu);
    auto it = g_occ.find(key);
    if (it != g_occ.end()) {
        *per_sm = it->second;
        return CK_OK;
    }
    CK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, kernel, threads, smem));
    g_occ[key] = *per_sm;
    return CK_OK;
}

// feed: the queues of a continuous feed (ck_ldpc_feed_launch): every queue
// may run (its frames come later), the grid is every resident block, and
// the per-frame arrays come from the rings instead.  allow_edges: codes set
// to CK_LDPC_PLACE_EDGES may keep one message per edge.
int resolve_mixed_shape(const ck_ldpc_batch* batches, int32_t n, MixedResolved* R, bool feed, bool allow_edges) {
    if (!batches || n < 1 || n > kMaxMixed)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "1 to %d batches per mixed launch, got %d", kMaxMixed, n);
    int dev = -1;
    CK_CUDA(cudaGetDevice(&dev));
    int sms = 0, optin = 0;
    CK_TRY(device_limits(dev, &sms, &optin));
    memset(&R->p, 0, sizeof(R->p));
    R->p.num_codes = n;
    R->block_threads = 32;
    R->smem = 0;
    R->wide = false;
    R->any_degree = false;
    R->edges = false;
    for (int c = 0; c < n; ++c)
        if (batches[c].plan && batches[c].plan->max_deg > kPackedDegree) R->any_degree = true;
    for (int c = 0; c < n; ++c) {
        const ck_ldpc_batch& b = batches[c];
        const ck_ldpc_plan* plan = b.plan;
        if (!plan) return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d has no plan", c);
        if (plan->device != dev)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: plan is for device %d, current is %d", c,
                            plan->device, dev);
        if (!plan->qc) return ck::fail(CK_ERR_UNSUPPORTED, "batch %d: mixed launches take quasi-cyclic codes", c);
        if (b.rule != CK_LDPC_MIN_SUM) return ck::fail(CK_ERR_UNSUPPORTED, "only the min-sum rule is implemented");
        CK_TRY(check_min_sum_params(b.scale, b.offset));
        if (b.B < 0 || b.B >= (int64_t(1) << 31)) return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: bad B", c);
        if (b.n_in < 1 || b.n_in > plan->N) return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: bad n_in", c);
        if (b.max_iterations < 0) return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: bad max_iterations", c);
        if (b.frames_per_block < 0) return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: bad frames_per_block", c);
        if (b.bits && (b.k_bits < 0 || b.k_bits > b.n_in))
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: bad k_bits", c);
        if (!feed && b.B > 0 && ((!b.llr_in && !b.symbols) || !b.llr_out || !b.iters || !b.valid))
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: missing arrays", c);
        if (feed && !b.symbols)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "queue %d: a feed demaps in the decoder (symbols must be set)",
                            c);
        int32_t ka = 0;
        if (b.symbols) {
            // Fused demapping: closed-form max-log tables of a square
            // separable constellation, 1 to 4 bits per axis.
            if ((!feed && !b.inv_s2) || !b.axis_re || !b.axis_im)
                return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: symbols need inv_s2 and both axes", c);
            ka = b.axis_re->k;
            if (ka < 1 || ka > 4 || b.axis_im->k != ka || b.axis_re->L != (1 << ka) || b.axis_im->L != (1 << ka))
                return ck::fail(CK_ERR_UNSUPPORTED, "batch %d: fused demapping takes 1 to 4 bits on each of two "
                                "equal axes", c);
            if (b.n_in % (2 * ka))
                return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: n_in %d is not a multiple of %d bits per "
                                "symbol", c, b.n_in, 2 * ka);
            if (!feed && reinterpret_cast<uintptr_t>(b.symbols) % 8)
                return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: symbols must be 8-byte aligned", c);
            const ck_axis_maxlog* ax[2] = {b.axis_re, b.axis_im};
            for (int a = 0; a < 2; ++a)
                if (!ax[a]->levels || !ax[a]->labels || !ax[a]->lo || !ax[a]->hi || !ax[a]->pos)
                    return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: an axis table is NULL", c);
        }
        if (plan->max_deg > 16) R->wide = true;
        const int32_t Zp = (plan->Z + 31) / 32 * 32;
        int32_t T = b.threads_per_frame > 0 ? b.threads_per_frame : plan->launch.threads_per_frame;
        if (b.threads_per_frame < 0)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: bad threads_per_frame", c);
        if (T == 0) {
            T = Zp;
            while (T > 512 && T % 64 == 0) T /= 2;
        }
        if (T % Zp != 0 && Zp % T != 0)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "batch %d: threads_per_frame %d vs lifting", c, T);
        const uint32_t code_tables = align_up(static_cast<uint32_t>(plan->L + 1 + plan->mb + 1) * 4, 8) +
                                     static_cast<uint32_t>(plan->nnzb) * 8;
        const uint32_t axes_off = align_up(code_tables, 16);
        // Then one word of the block's frame bookkeeping (busy_off).
        const uint32_t busy_off =
            align_up(ka ? axes_off + static_cast<uint32_t>(sizeof(ck::ldpc::MixedAxes<4>)) : code_tables, 4);
        const uint32_t tables = align_up(busy_off + 4, 128);
        const uint32_t ctrl = 128;
        const uint32_t gblk = align_up(static_cast<uint32_t>(plan->nnzb) * 8, 128);
        const uint32_t app = align_up(static_cast<uint32_t>(plan->N) * 4, 128);
        const uint32_t r_stride = align_up(static_cast<uint32_t>(plan->m), 32);
        // Message state words per row: the packed record (16 bytes in shared
        // memory, 3 words in device memory), or in an any-degree launch every
        // code's wide state, 3 + sign_words words in either.
        const int32_t sign_words = R->any_degree ? std::max(1, (plan->max_deg + 31) / 32) : 0;
        const uint32_t rsm = r_stride * (sign_words ? 4u * static_cast<uint32_t>(3 + sign_words) : 16u);
        // 1 KB stays free for the kernel's static shared variable.
        const uint32_t budget = static_cast<uint32_t>(optin) > tables + 1024 ? optin - tables - 1024 : 0;
        const int32_t max_threads = R->wide ? 512 : kMixedThreads;
        int32_t gmax = std::min(max_threads / T, T > 32 ? ck::kMaxNamedGroups : 32);
        // Message state in shared memory when two frames still fit with it:
        // one message per edge (CK_LDPC_PLACE_EDGES, a code run by its
        // program with one thread per row slot), else the records.
        const uint32_t e_stride = align_up(static_cast<uint32_t>(plan->E), 32);
        const bool edges = allow_edges &&
                           (plan->launch.placement == CK_LDPC_PLACE_EDGES ||
                            plan->launch.placement == CK_LDPC_PLACE_AUTO) &&
                           !R->any_degree && T == Zp && 2 * (ctrl + gblk + app + 4 * e_stride) <= budget;
        const bool r_smem = edges || (plan->launch.placement != CK_LDPC_PLACE_GLOBAL &&
                                      2 * (ctrl + gblk + app + rsm) <= budget);
        const uint32_t group = ctrl + gblk + app + (edges ? 4 * e_stride : (r_smem ? rsm : 0));
        gmax = std::min<int32_t>(gmax, static_cast<int32_t>(budget / group));
        // As many groups as the block's threads and shared memory hold: a
        // plain launch's tuned frames per block (one block of G groups among
        // several per SM) says nothing about a mixed block, which is alone
        // on its SM.
        const int32_t G = b.frames_per_block > 0 ? std::min(gmax, b.frames_per_block) : gmax;
        if (G < 1) return ck::fail(CK_ERR_UNSUPPORTED, "batch %d: a frame does not fit a block", c);
        MixedCode& K = R->p.code[c];
        K.layer = plan->d_layer;
        K.eptr = plan->d_eptr;
        K.blk = reinterpret_cast<const int2*>(plan->d_blk);
        K.N = plan->N;
        K.m = plan->m;
        K.L = plan->L;
        K.Z = plan->Z;
        K.Zp = Zp;
        K.mb = plan->mb;
        K.nnzb = plan->nnzb;
        K.llr_in = b.llr_in;
        K.llr_out = b.llr_out;
        K.order = b.order;
        K.B = static_cast<uint32_t>(b.B);
        K.n_in = b.n_in;
        K.iters = b.iters;
        K.valid = b.valid;
        K.bits = b.k_bits > 0 ? b.bits : nullptr;
        K.k_bits = b.k_bits;
        K.scale = b.scale;
        K.offset = b.offset;
        K.max_iterations = b.max_iterations;
        K.early_stop = b.early_stop ? 1 : 0;
        K.T = T;
        K.G = G;
        K.q_bstep = T >= Zp ? T / Zp : 1;
        K.r_smem = edges ? 2 : (r_smem ? 1 : 0);
        R->edges |= edges;
        K.tables_bytes = tables;
        K.group_bytes = group;
        K.gblk_off = ctrl;
        K.app_off = ctrl + gblk;
        K.r_off = ctrl + gblk + app;
        K.r_stride = edges ? e_stride : r_stride;
        K.weight = static_cast<float>(plan->E);
        K.sign_words = sign_words;
        K.ka = ka;
        K.axes_off = axes_off;
        K.busy_off = busy_off;
        if (ka) {
            K.sym = static_cast<const float2*>(b.symbols);
            K.inv_s2 = b.inv_s2;
            const ck_axis_maxlog* ax[2] = {b.axis_re, b.axis_im};
            for (int a = 0; a < 2; ++a) {
                K.ax_levels[a] = ax[a]->levels;
                K.ax_labels[a] = ax[a]->labels;
                K.ax_lo[a] = ax[a]->lo;
                K.ax_hi[a] = ax[a]->hi;
                K.ax_pos[a] = ax[a]->pos;
            }
        }
        R->block_threads = std::max(R->block_threads, T * G);
        R->smem = std::max(R->smem, tables + static_cast<uint32_t>(G) * group);
    }
    if (R->wide && R->block_threads > 512)
        return ck::fail(CK_ERR_UNSUPPORTED, "mixed launch of %d threads with rows above degree 16",
                        R->block_threads);
    const void* kernel = reinterpret_cast<const void*>(
        R->any_degree ? ldpc_mixed_kernel<0> : (R->wide ? ldpc_mixed_kernel<27> : ldpc_mixed_kernel<16>));
    if (!R->any_degree) {
        // The code-specialised mixed kernel, where the plans have one.
        const ck_ldpc_plan* plans[kMaxMixed];
        int32_t threads[kMaxMixed];
        int edges[kMaxMixed];
        for (int c = 0; c < n; ++c) {
            plans[c] = batches[c].plan;
            threads[c] = R->p.code[c].T;
            edges[c] = R->p.code[c].r_smem == 2 ? 1 : 0;
        }
        const void* special = nullptr;
        CK_TRY(ck::ldpc::mixed_specialised_kernel(plans, threads, edges, n, R->wide ? 27 : 16, &special));
        if (special) kernel = special;
    }
    // The per-edge state runs in the specialised programs only: without
    // them the codes keep the records (the caller sizes the launch again).
    R->kernel = kernel;
    if (R->edges && kernel == reinterpret_cast<const void*>(R->wide ? ldpc_mixed_kernel<27> : ldpc_mixed_kernel<16>))
        return CK_OK;
    CK_TRY(ck::allow_max_smem(kernel, dev, optin));
    int per_sm = 0;
    CK_TRY(mixed_occupancy(kernel, dev, R->block_threads, R->smem, &per_sm));
    if (per_sm < 1) return ck::fail(CK_ERR_UNSUPPORTED, "mixed block does not fit an SM");
    int64_t need = 0;
    for (int c = 0; c < n; ++c)
        need += (R->p.code[c].B + R->p.code[c].G - 1) / R->p.code[c].G;
    R->grid = feed ? sms * per_sm
                   : static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(need, int64_t(sms) * per_sm)));
    // Starting split, longest frames first (mixed_pick's order): the codes
    // by edges per frame times iteration budget, heaviest first (stable), each
    // taking as many blocks as it has frame groups to fill, until the grid is
    // used up.  Codes without frames, or beyond the grid, start no block.
    int rank_code[kMaxMixed];
    for (int c = 0; c < n; ++c) rank_code[c] = c;
    const auto budget = [&](int c) {
        return static_cast<double>(R->p.code[c].weight) * std::max(1, R->p.code[c].max_iterations);
    };
    std::stable_sort(rank_code, rank_code + n, [&](int a, int b) { return budget(a) > budget(b); });
    int start = 0;
    for (int r = 0; r < n; ++r) {
        const MixedCode& K = R->p.code[rank_code[r]];
        R->p.start_code[r] = rank_code[r];
        R->p.start_block[r] = start;
        const int64_t blocks = (static_cast<int64_t>(K.B) + K.G - 1) / K.G;
        start = static_cast<int>(std::min<int64_t>(R->grid, start + blocks));
    }
    R->p.start_block[n] = R->grid;
    // Workspace: counters, then the device-memory message slots.  A block
    // runs one code at a time, so the codes share each block's region,
    // sized for the largest (G groups x 3 r_stride words), in 256-byte units.
    uint32_t block_words = 0;
    for (int c = 0; c < n; ++c)
        if (!R->p.code[c].r_smem && (feed || R->p.code[c].B > 0))  // a code without frames never runs
            block_words = std::max<uint32_t>(block_words, static_cast<uint32_t>(R->p.code[c].G) *
                                                              static_cast<uint32_t>(3 + R->p.code[c].sign_words) *
                                                              R->p.code[c].r_stride);
    R->block_words = (block_words + 63u) / 64u * 64u;
    for (int c = 0; c < n; ++c) R->p.code[c].block_words = R->block_words;
    R->ws_bytes = kHeaderBytes + static_cast<size_t>(R->grid) * R->block_words * 4u;
    return CK_OK;
}

int resolve_mixed(const ck_ldpc_batch* batches, int32_t n, MixedResolved* R, bool feed = false) {
    CK_TRY(resolve_mixed_shape(batches, n, R, feed, true));
    const void* table = reinterpret_cast<const void*>(R->wide ? ldpc_mixed_kernel<27> : ldpc_mixed_kernel<16>);
    if (R->edges && R->kernel == table) CK_TRY(resolve_mixed_shape(batches, n, R, feed, false));
    return CK_OK;
}

}  // namespace

extern "C" int ck_ldpc_plan_resolved_launch(const ck_ldpc_plan* plan, int32_t rule, ck_ldpc_launch* out) {
    ck::clear_error();
    if (!plan || !out) return ck::fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
    int device = -1;
    CK_CUDA(cudaGetDevice(&device));
    if (device != plan->device)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "plan is for device %d, current device is %d", plan->device,
                        device);
    Resolved r;
    CK_TRY(resolve(plan, rule, int64_t(1) << 40, &r));  // a full batch: the shape before any spreading of a short one
    out->threads_per_frame = r.T;
    out->frames_per_block = r.G;
    out->placement = !r.r_smem ? CK_LDPC_PLACE_GLOBAL : (r.edges ? CK_LDPC_PLACE_EDGES : CK_LDPC_PLACE_SHARED);
    return CK_OK;
}

extern "C" int ck_ldpc_mixed_workspace_size(const ck_ldpc_batch* batches, int32_t num_batches,
                                            size_t* bytes) {
    ck::clear_error();
    if (!bytes) return ck::fail(CK_ERR_INVALID_ARGUMENT, "bytes is NULL");
    MixedResolved R;
    CK_TRY(resolve_mixed(batches, num_batches, &R));
    *bytes = R.ws_bytes;
    return CK_OK;
}

extern "C" int ck_ldpc_decode_mixed(const ck_ldpc_batch* batches, int32_t num_batches,
                                    void* workspace, size_t workspace_bytes, void* stream) {
    ck::clear_error();
    MixedResolved R;
    CK_TRY(resolve_mixed(batches, num_batches, &R));
    int64_t total = 0;
    for (int c = 0; c < num_batches; ++c) total += batches[c].B;
    if (total == 0) return CK_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void* ws = workspace;
    bool owned = false;
    if (ws == nullptr) {
        CK_CUDA(cudaMallocAsync(&ws, R.ws_bytes, s));
        owned = true;
    } else {
        if (workspace_bytes < R.ws_bytes)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "workspace of %zu bytes, %zu needed", workspace_bytes,
                            R.ws_bytes);
        if (reinterpret_cast<uintptr_t>(ws) % 256)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    }
    unsigned char* wsb = static_cast<unsigned char*>(ws);
    for (int c = 0; c < num_batches; ++c) {
        R.p.code[c].counter = reinterpret_cast<uint32_t*>(wsb + 4 * c);
        R.p.code[c].g_r = reinterpret_cast<uint32_t*>(wsb + kHeaderBytes);
    }
    int status = ck::cuda_check(cudaMemsetAsync(wsb, 0, kHeaderBytes, s), "cudaMemsetAsync");
    if (status == CK_OK) {
        void* args[] = {&R.p};
        status = ck::cuda_check(cudaLaunchKernel(R.kernel, dim3(static_cast<unsigned>(R.grid)),
                                                 dim3(static_cast<unsigned>(R.block_threads)), args, R.smem, s),
                                "mixed decoder launch");
    }
    if (owned) {
        const int st = ck::cuda_check(cudaFreeAsync(ws, s), "cudaFreeAsync");
        if (status == CK_OK) status = st;
    }
    return status;
}

static_assert(sizeof(ck_ldpc_feed_frame) == sizeof(ck::ldpc::FeedFrame), "feed frame layout");
static_assert(offsetof(ck_ldpc_feed_frame, inv_s2) == offsetof(ck::ldpc::FeedFrame, inv_s2), "feed frame layout");
static_assert(offsetof(ck_ldpc_feed_frame, seq) == offsetof(ck::ldpc::FeedFrame, seq), "feed frame layout");

extern "C" int ck_ldpc_feed_workspace_size(const ck_ldpc_batch* queues, int32_t num_queues, size_t* bytes) {
    ck::clear_error();
    if (!bytes) return ck::fail(CK_ERR_INVALID_ARGUMENT, "bytes is NULL");
    MixedResolved R;
    CK_TRY(resolve_mixed(queues, num_queues, &R, true));
    *bytes = R.ws_bytes;
    return CK_OK;
}

extern "C" int ck_ldpc_feed_reset(void* workspace, void* stream) {
    ck::clear_error();
    if (!workspace) return ck::fail(CK_ERR_INVALID_ARGUMENT, "workspace is NULL");
    return ck::cuda_check(cudaMemsetAsync(workspace, 0, kHeaderBytes, static_cast<cudaStream_t>(stream)),
                          "cudaMemsetAsync");
}

extern "C" int ck_ldpc_feed_launch(const ck_ldpc_batch* queues, const ck_ldpc_feed_ring* rings,
                                   int32_t num_queues, const uint32_t* stop, uint32_t idle_us, int32_t policy,
                                   void* workspace, size_t workspace_bytes, void* stream) {
    ck::clear_error();
    if (!rings) return ck::fail(CK_ERR_INVALID_ARGUMENT, "rings is NULL");
    if (policy != CK_LDPC_FEED_OLDEST && policy != CK_LDPC_FEED_SHORT_FIRST)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "unknown feed policy %d", policy);
    if (idle_us < 1 || idle_us > 1000000)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "idle_us must be in [1, 1000000], got %u", idle_us);
    MixedResolved R;
    CK_TRY(resolve_mixed(queues, num_queues, &R, true));
    for (int c = 0; c < num_queues; ++c) {
        const ck_ldpc_feed_ring& q = rings[c];
        if (!q.frames || !q.published)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "queue %d: ring frames and published count are required", c);
        if (q.capacity < 1 || q.capacity > (1u << 30) || (q.capacity & (q.capacity - 1)))
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "queue %d: ring capacity %u is not a power of two in [1, 2^30]",
                            c, q.capacity);
    }
    if (!workspace) return ck::fail(CK_ERR_INVALID_ARGUMENT, "a feed needs its workspace (its counts persist)");
    if (workspace_bytes < R.ws_bytes)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "workspace of %zu bytes, %zu needed", workspace_bytes, R.ws_bytes);
    if (reinterpret_cast<uintptr_t>(workspace) % 256)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    unsigned char* wsb = static_cast<unsigned char*>(workspace);
    for (int c = 0; c < num_queues; ++c) {
        MixedCode& K = R.p.code[c];
        K.counter = reinterpret_cast<uint32_t*>(wsb + 4 * c);
        K.g_r = reinterpret_cast<uint32_t*>(wsb + kHeaderBytes);
        K.ring = reinterpret_cast<const ck::ldpc::FeedFrame*>(rings[c].frames);
        K.published = rings[c].published;
        K.ring_mask = rings[c].capacity - 1u;
        K.B = 0;
        K.order = nullptr;
    }
    R.p.feed = 1;
    R.p.feed_policy = policy;
    R.p.stop = stop;
    R.p.idle_ns = static_cast<uint64_t>(idle_us) * 1000ull;
    R.p.idle_polls = idle_us;  // each poll sleeps up to 2 us: a second bound on the wait
    void* args[] = {&R.p};
    return ck::cuda_check(cudaLaunchKernel(R.kernel, dim3(static_cast<unsigned>(R.grid)),
                                           dim3(static_cast<unsigned>(R.block_threads)), args, R.smem,
                                           static_cast<cudaStream_t>(stream)),
                          "feed decoder launch");
}

namespace {
std::mutex g_smem_mu;
std::set<std::pair<const void*, int>> g_smem_done;  // (kernel, device) pairs already raised
}  // namespace

void ck::forget_kernel(const void* kernel) {
    {
        std::lock_guard<std::mutex> lock(g_smem_mu);
        for (auto it = g_smem_done.begin(); it != g_smem_done.end();)
            it = it->first == kernel ? g_smem_done.erase(it) : std::next(it);
    }
    std::lock_guard<std::mutex> lock(g_occ_mu);
    for (auto it = g_occ.begin(); it != g_occ.end();)
        it = std::get<0>(it->first) == kernel ? g_occ.erase(it) : std::next(it);
}

int ck::allow_max_smem(const void* kernel, int device, int optin) {
    std::lock_guard<std::mutex> lock(g_smem_mu);
    auto& done = g_smem_done;
    if (done.count({kernel, device})) return CK_OK;
    // The limit covers dynamic shared memory only: the opt-in maximum less
    // the kernel's static shared variables.
    cudaFuncAttributes attr;
    CK_CUDA(cudaFuncGetAttributes(&attr, kernel));
    const int dynamic = optin - static_cast<int>(attr.sharedSizeBytes);
    CK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dynamic));
    done.insert({kernel, device});
    return CK_OK;
}
