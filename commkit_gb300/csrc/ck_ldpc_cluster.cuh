// The thread-block-cluster decoder for CSR codes (ck_ldpc_kernel.cuh has
// the plain frame loop and Params).
#pragma once

#include <cooperative_groups.h>

#include "ck_ldpc_kernel.cuh"

namespace ck {
namespace ldpc {

// Frames of CSR codes whose posterior lives in device memory, when there
// are fewer of them than the GPU has room for (the reference's DVB-S2
// benchmark: 64 frames of N = 64800 on 152 SMs): a thread-block cluster of
// C CTAs, on C SMs, decodes one frame.  The rows of each layer are spread
// over the cluster's C x T threads, and a cluster barrier (release /
// acquire at cluster scope, so one CTA's posterior writes are visible to
// the others) separates the layers.  The syndrome test ORs the CTAs'
// results through rank 0's shared memory.  Every branch that decides a
// barrier depends only on values all CTAs of the cluster read after the
// same barrier, so they all take it.  Same rows, same order, same bits as
// decode_kernel.
template <template <bool> class State, int DMAX>
__global__ void __launch_bounds__(max_block_threads(false, DMAX))
    decode_cluster_kernel(const __grid_constant__ Params p) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int C = static_cast<int>(cluster.num_blocks());
    const int rank = static_cast<int>(cluster.block_rank());
    const uint32_t cid = blockIdx.x / static_cast<uint32_t>(C);
    __shared__ uint32_t s_frame;
    __shared__ int s_flag[16];
    const int tid = threadIdx.x;
    const int first = rank * p.T + tid, stride = C * p.T;
    float* a = p.g_app + static_cast<size_t>(cid) * p.app_stride;
    const State<false> st(p, nullptr, cid);
    const uint32_t* frame0 = cluster.map_shared_rank(&s_frame, 0);
    int* flags0 = cluster.map_shared_rank(s_flag, 0);

    // True in every thread of the cluster when every check is satisfied;
    // rows in chunks of C x T, stopping at the first unsatisfied chunk.
    auto satisfied = [&]() -> bool {
        for (int32_t base = 0; base < p.m; base += stride) {
            const int32_t row = base + first;
            uint32_t parity = 0;
            if (row < p.m) {
                int deg;
                int32_t e0;
                const auto col_of = RowOf<false>::get(p, nullptr, nullptr, static_cast<uint32_t>(row), deg, e0);
                for (int e = 0; e < deg; ++e) parity ^= a[col_of(e)] < 0.0f ? 1u : 0u;
            }
            const int bad = __syncthreads_or(static_cast<int>(parity));
            if (tid == 0) flags0[rank] = bad;
            cluster.sync();
            int any = 0;
            for (int c = 0; c < C; ++c) any |= flags0[c];
            cluster.sync();  // all have read the flags before they are written again
            if (any) return false;
        }
        return true;
    };

    for (;;) {
        if (rank == 0 && tid == 0) s_frame = atomicAdd(p.counter, 1u);
        cluster.sync();
        const uint32_t f = *frame0;
        cluster.sync();  // all have read rank 0's frame before it may exit or move on
        if (f >= p.B) break;
        const float* src = p.llr_in + static_cast<size_t>(f) * p.n_in;
        for (int i = first; i < p.n_in; i += stride) a[i] = __fadd_rn(__ldcs(src + i), 0.0f);
        for (int i = p.n_in + first; i < p.N; i += stride) a[i] = 0.0f;
        st.zero(p, first, stride);
        cluster.sync();

        int32_t it = 0;
        bool ok = p.early_stop && satisfied();
        while (!ok && it < p.max_iterations) {
            for (int32_t l = 0; l < p.L; ++l) {
                const uint32_t row1 = static_cast<uint32_t>(__ldg(p.layer + l + 1));
                for (uint32_t row = static_cast<uint32_t>(__ldg(p.layer + l) + first); row < row1; row += stride) {
                    int deg;
                    int32_t e0;
                    const auto col_of = RowOf<false>::get(p, nullptr, nullptr, row, deg, e0);
                    st.template csr_row<DMAX>(p, a, row, deg, e0, col_of);
                }
                cluster.sync();
            }
            ++it;
            if (p.early_stop) ok = satisfied();
        }
        if (!p.early_stop) ok = satisfied();

        float* dst = p.llr_out + static_cast<size_t>(f) * p.n_in;
        for (int i = first; i < p.n_in; i += stride) __stcs(dst + i, a[i]);
        if (p.bits) {
            int8_t* bdst = p.bits + static_cast<size_t>(f) * p.k_bits;
            for (int i = first; i < p.k_bits; i += stride) bdst[i] = a[i] < 0.0f ? 1 : 0;
        }
        if (rank == 0 && tid == 0) {
            p.iters[f] = it;
            p.valid[f] = ok ? 1 : 0;
        }
        cluster.sync();  // everyone is done with `a` before the next frame
    }
}

}  // namespace ldpc
}  // namespace ck
