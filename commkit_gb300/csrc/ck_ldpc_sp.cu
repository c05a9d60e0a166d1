// Layered sum-product LDPC decoding on sm_103a: the check rule of the
// reference's `ldpc_layered<true>` (commkit/_cuda/src/ldpc.cu:74-91; CPU twin
// commkit/coding/_numba_loops.py:71-94) run by the persistent frame loop the
// min-sum rule uses (ck_ldpc_kernel.cuh): same layers, same order, same
// early stop.
//
// The check-to-variable message of edge e is
//     sign_e * phi(sum_e' phi(|Q_e'|) - phi(|Q_e|)),   phi(x) = -log tanh(x / 2)
// on x clipped to [1e-7, 30], with sign_e the parity of the row's Q signs
// times Q_e's own.  Unlike min-sum a row's messages do not compress, so the
// state is one float per edge: in shared memory beside the posterior when it
// fits (codes of a few thousand edges), else in the frame slot's device
// memory.  Circulant c of a quasi-cyclic code keeps the message of its row r
// at c Z + r, so a warp's lanes (consecutive r) touch consecutive words; a
// CSR code keeps the message of edge e at e, as the reference does.
//
// Arithmetic: Q = APP - R, the running total of phi values (edge by edge, in
// column order), total - phi(|Q_e|) and APP = Q + R_new are explicit
// round-to-nearest float32 operations in the reference's order; phi calls
// logf and tanhf as the reference's kernel does.  Results therefore match
// the CPU decoder up to the rounding of those two functions (the reference
// tests its own GPU path against the CPU at 1e-3).
#include "ck_ldpc_cluster.cuh"
#include "ck_ldpc_kernel.cuh"

namespace ck {
namespace ldpc {
namespace sp {

__device__ __forceinline__ float phi(float x) {
    x = fminf(fmaxf(x, 1e-7f), 30.0f);
    return -logf(tanhf(__fmul_rn(0.5f, x)));
}

template <bool R_SMEM>
struct SumProductState {
    float* r;  // this slot's messages

    __device__ __forceinline__ SumProductState(const Params& p, unsigned char* gbase, uint32_t slot)
        : r(R_SMEM ? reinterpret_cast<float*>(gbase + p.r_off)
                   : reinterpret_cast<float*>(p.g_r) + static_cast<size_t>(slot) * p.r_stride) {}

    __device__ __forceinline__ void zero(const Params& p, int first, int stride) const {
        for (int i = first; i < p.E; i += stride) r[i] = 0.0f;
    }
    __device__ __forceinline__ float ld(uint32_t i) const { return R_SMEM ? r[i] : __ldcg(r + i); }
    __device__ __forceinline__ void st(uint32_t i, float v) const {
        if (R_SMEM)
            r[i] = v;
        else
            __stcg(r + i, v);
    }

    // One row of any degree (the any-degree kernels, DMAX = 0): the
    // reference's kernel loop as it stands (commkit/_cuda/src/ldpc.cu:74-91),
    // Q and phi(|Q|) recomputed in the second pass; edge e's message at
    // msg(e).
    template <class Post, class Msg>
    __device__ __forceinline__ void any_row(const Post& post, const int deg, const Msg& msg) const {
        float total = 0.0f;
        bool neg = false;
        for (int e = 0; e < deg; ++e) {
            const float qe = __fsub_rn(post.ld(post.col(static_cast<uint32_t>(e))), ld(msg(e)));
            neg ^= qe < 0.0f;
            total = __fadd_rn(total, phi(fabsf(qe)));
        }
        for (int e = 0; e < deg; ++e) {
            const uint32_t c = post.col(static_cast<uint32_t>(e));
            const float qe = __fsub_rn(post.ld(c), ld(msg(e)));
            const float mag = phi(__fsub_rn(total, phi(fabsf(qe))));
            const float rn = (neg != (qe < 0.0f)) ? -mag : mag;
            post.st(c, __fadd_rn(qe, rn));
            st(msg(e), rn);
        }
    }
    // Message addresses: circulant c of a base row keeps row r's message at
    // c Z + r; a CSR edge at its index.
    struct QcMsg {
        uint32_t base, Z;
        __device__ __forceinline__ uint32_t operator()(int e) const { return base + static_cast<uint32_t>(e) * Z; }
    };
    struct CsrMsg {
        int32_t e0;
        __device__ __forceinline__ uint32_t operator()(int e) const { return static_cast<uint32_t>(e0 + e); }
    };

    // Row r of base row b: circulants e0 .. e0 + deg of the table, their
    // columns from the group's shared-address copy `gblk`.
    template <int DMAX>
    __device__ __forceinline__ void qc_row(const Params& p, const int2* __restrict__ gblk,
                                           const int deg, uint32_t, const int32_t e0,
                                           const int32_t rr, const uint32_t r4,
                                           const uint32_t Z4) const {
        const uint32_t Z = static_cast<uint32_t>(p.Z);
        const uint32_t base = static_cast<uint32_t>(e0) * Z + static_cast<uint32_t>(rr);
        if constexpr (DMAX == 0) {
            any_row(QcSmemPost{gblk, r4, Z4}, deg, QcMsg{base, Z});
        } else {
            qc_row_fixed<DMAX>(gblk, deg, base, Z, r4, Z4);
        }
    }

    template <int DMAX>
    __device__ __forceinline__ void qc_row_fixed(const int2* __restrict__ gblk, const int deg,
                                                 const uint32_t base, const uint32_t Z,
                                                 const uint32_t r4, const uint32_t Z4) const {
        float q[DMAX], ph[DMAX];
        float total = 0.0f;
        bool neg = false;
#pragma unroll
        for (int e = 0; e < DMAX; ++e) {
            if (e < deg) {
                const int2 b = gblk[e];
                uint32_t ce = r4 + static_cast<uint32_t>(b.x);
                ce = ce >= static_cast<uint32_t>(b.y) ? ce - Z4 : ce;
                const float qe = __fsub_rn(ld_shared_f32(ce), ld(base + e * Z));
                q[e] = qe;
                neg ^= qe < 0.0f;
                ph[e] = phi(fabsf(qe));
                total = __fadd_rn(total, ph[e]);
            }
        }
#pragma unroll
        for (int e = 0; e < DMAX; ++e) {
            if (e < deg) {
                const int2 b = gblk[e];
                uint32_t ce = r4 + static_cast<uint32_t>(b.x);
                ce = ce >= static_cast<uint32_t>(b.y) ? ce - Z4 : ce;
                const float mag = phi(__fsub_rn(total, ph[e]));
                const float rn = (neg != (q[e] < 0.0f)) ? -mag : mag;
                st_shared_f32(ce, __fadd_rn(q[e], rn));
                st(base + e * Z, rn);
            }
        }
    }

    template <int DMAX, class ColOf>
    __device__ __forceinline__ void csr_row(const Params&, float* __restrict__ a, uint32_t,
                                            const int deg, const int32_t e0,
                                            const ColOf& col_of) const {
        if constexpr (DMAX == 0) {
            any_row(CsrPost<ColOf>{a, col_of}, deg, CsrMsg{e0});
        } else {
            csr_row_fixed<DMAX>(a, deg, e0, col_of);
        }
    }

    template <int DMAX, class ColOf>
    __device__ __forceinline__ void csr_row_fixed(float* __restrict__ a, const int deg, const int32_t e0,
                                                  const ColOf& col_of) const {
        float q[DMAX], ph[DMAX];
        int col[DMAX];  // loaded once, all before the first posterior load
        float total = 0.0f;
        bool neg = false;
#pragma unroll
        for (int e = 0; e < DMAX; ++e)
            if (e < deg) col[e] = col_of(e);
#pragma unroll
        for (int e = 0; e < DMAX; ++e) {
            if (e < deg) {
                const float qe = __fsub_rn(a[col[e]], ld(static_cast<uint32_t>(e0 + e)));
                q[e] = qe;
                neg ^= qe < 0.0f;
                ph[e] = phi(fabsf(qe));
                total = __fadd_rn(total, ph[e]);
            }
        }
#pragma unroll
        for (int e = 0; e < DMAX; ++e) {
            if (e < deg) {
                const float mag = phi(__fsub_rn(total, ph[e]));
                const float rn = (neg != (q[e] < 0.0f)) ? -mag : mag;
                a[col[e]] = __fadd_rn(q[e], rn);
                st(static_cast<uint32_t>(e0 + e), rn);
            }
        }
    }
};

struct SumProductPick {
    template <bool QC, int DMAX, bool ONE_ROW>
    static KernelFn get(bool app_smem, bool r_smem) {
        if (app_smem && r_smem) return decode_kernel<SumProductState, QC, DMAX, true, true, ONE_ROW>;
        if (app_smem) return decode_kernel<SumProductState, QC, DMAX, true, false, ONE_ROW>;
        if constexpr (!QC) return decode_kernel<SumProductState, QC, DMAX, false, false, false>;
        return nullptr;
    }
};

}  // namespace sp

KernelFn sum_product_kernel(bool qc, int max_deg, bool app_smem, bool r_smem, bool one_row) {
    return pick_shape<sp::SumProductPick>(qc, max_deg, app_smem, r_smem, one_row);
}

KernelFn sum_product_cluster_kernel(int max_deg) {
    switch (kernel_dmax(false, max_deg)) {
        case 8: return decode_cluster_kernel<sp::SumProductState, 8>;
        case 16: return decode_cluster_kernel<sp::SumProductState, 16>;
        case 27: return decode_cluster_kernel<sp::SumProductState, 27>;
        default: return decode_cluster_kernel<sp::SumProductState, 0>;
    }
}

}  // namespace ldpc
}  // namespace ck
