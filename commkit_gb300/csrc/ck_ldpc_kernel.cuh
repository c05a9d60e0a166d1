// The persistent frame loop of the layered decoder, shared by its check
// rules: min-sum (ck_ldpc.cu) and sum-product (ck_ldpc_sp.cu).
//
// A rule supplies the check-message state of one frame slot as a class
// template State<R_SMEM> (R_SMEM: the state lives in the group's shared
// memory, else in the slot's device-memory workspace) with
//   State(const Params&, unsigned char* group_smem, uint32_t slot)
//   void zero(const Params&, int first, int stride) const
//       fresh state of a frame (entries first, first + stride, ...)
//   template <int DMAX> void qc_row(p, gblk, deg, row, e0, r, r4, Z4) const
//       one circulant row: base row b = row / Z, its circulants gblk[0..deg)
//       (table index e0..e0+deg), row r of them (r4 = 4 r, Z4 = 4 Z)
//   template <int DMAX, class ColOf> void csr_row(p, a, row, deg, e0, col_of) const
//       one CSR row: edges e0..e0+deg, columns col_of(e)
// and the kernel runs frames, layers and the syndrome test around it, so
// both rules decode in the reference's layer order with the same early stop.
//
// The layer loop of a circulant code can also come from a code-specialised
// program (decode_body's Prog, generated and compiled at run time by
// ck_ldpc_jit.cu), which this header and ck_ldpc_minsum.cuh serve as
// NVRTC sources.
#pragma once

#include "ck_device.cuh"
#ifndef __CUDACC_RTC__
#include "ck_ldpc_internal.h"
#endif

namespace ck {
namespace ldpc {

struct Params {
    // frames
    const float* llr_in;
    float* llr_out;
    uint32_t B;
    int32_t n_in;
    int32_t* iters;
    uint8_t* valid;
    int8_t* bits;
    int32_t k_bits;
    // code
    int32_t N, m, L, E;
    int32_t Z, mb, nnzb;
    ck::FastDiv divZ;
    int32_t Zp;       // QC: row slots per base row, Z rounded up to a multiple of 32
    int32_t q_bstep;  // QC: base-row stride of a thread (T / Zp when T >= Zp, else 1)
    const int32_t* layer;  // QC: base rows per layer; CSR: rows per layer (L + 1)
    const int32_t* eptr;   // QC: circulants per base row (mb + 1); CSR: row_ptr (m + 1)
    const int2* blk;       // QC: (j Z, shift) per circulant
    const int32_t* cols;   // CSR: column per edge
    // method
    float scale, offset;
    int32_t max_iterations;
    int32_t early_stop;
    // launch
    int32_t T;  // threads per frame group
    int32_t G;  // frame groups per block
    uint32_t tables_bytes, group_bytes, app_off, r_off, r_stride, gblk_off;
    int32_t bulk_load;  // 1: stage the LLRs with one bulk copy
    // workspace
    uint32_t* counter;
    uint32_t* status;
    uint32_t* g_r;  // check-message state slots in device memory (rule's layout)
    float* g_app;  // posterior slots in device memory (N per slot)
    int32_t app_stride;
    // Min-sum codes with rows above kPackedDegree edges: sign words per row
    // of the wide message state (0 otherwise).
    int32_t sign_words;
};

__device__ __forceinline__ float flip_sign(float v, uint32_t bit) {
    return __uint_as_float(__float_as_uint(v) ^ (bit << 31));
}

// Minimum of three floats, a NaN input counting as absent (min.f32 with
// three inputs, sm_100 and later).
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Maximum that returns NaN when either input is NaN.  In the min1/min2
// updates it keeps an edge whose |Q| is NaN out of min2 as well as min1, as
// the reference's `mag < min1` / `mag < min2` tests do.
__device__ __forceinline__ float fmax_nan(float a, float b) {
    float d;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}

// Shared-memory load and store at a 32-bit shared address (volatile: their
// order against each other and the barriers stays as written).
__device__ __forceinline__ float ld_shared_f32(uint32_t addr) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}
__device__ __forceinline__ void st_shared_f32(uint32_t addr, float v) {
    asm volatile("st.shared.f32 [%0], %1;" ::"r"(addr), "f"(v));
}

// Columns of row r of a circulant base row: j Z + (r + shift) mod Z, from
// the table entry (j Z + shift, (j + 1) Z).
struct QcCols {
    const int2* blk;
    int32_t r, Z;
    __device__ __forceinline__ int operator()(int e) const {
        const int2 b = blk[e];
        const int c = r + b.x;
        return c >= b.y ? c - Z : c;
    }
};

struct CsrCols {
    const int32_t* cols;
    __device__ __forceinline__ int operator()(int e) const { return __ldg(cols + e); }
};

// Row `row` (schedule order) of the code: its degree and column functor.
template <bool QC>
struct RowOf;
template <>
struct RowOf<true> {
    __device__ __forceinline__ static QcCols get(const Params& p, const int32_t* s_eptr,
                                                 const int2* s_blk, uint32_t row, int& deg,
                                                 int32_t& e0) {
        const uint32_t b = p.divZ.div(row);
        const int32_t r = static_cast<int32_t>(row - b * static_cast<uint32_t>(p.Z));
        e0 = s_eptr[b];
        deg = s_eptr[b + 1] - e0;
        return QcCols{s_blk + e0, r, p.Z};
    }
};
template <>
struct RowOf<false> {
    __device__ __forceinline__ static CsrCols get(const Params& p, const int32_t*, const int2*,
                                                  uint32_t row, int& deg, int32_t& e0) {
        e0 = __ldg(p.eptr + row);
        deg = __ldg(p.eptr + row + 1) - e0;
        return CsrCols{p.cols + e0};
    }
};

// True in every thread of the group when every check is satisfied by the
// hard decisions of `a` (commkit/_cuda/src/ldpc.cu:94-105).  Rows go in
// chunks of T; the first chunk with an unsatisfied row ends the test.
template <bool QC>
__device__ __forceinline__ bool syndrome_ok(const Params& p, const float* a, const int32_t* s_eptr,
                                            const int2* s_blk, int tid, int bar, int32_t qr0,
                                            int32_t qb0) {
    if (QC) {
        // Rounds of T row slots, each covering whole warps of one base row
        // (the thread's rows as in the layer loop); an OR per round.
        const int32_t rounds = (p.mb + p.q_bstep - 1) / p.q_bstep;
        for (int32_t k = 0; k < rounds; ++k) {
            const int32_t b = k * p.q_bstep + qb0;
            for (int32_t r = qr0; r - qr0 < p.Zp; r += p.T) {
                uint32_t parity = 0;
                if (b < p.mb && r < p.Z) {
                    const int32_t e0 = s_eptr[b];
                    const int deg = s_eptr[b + 1] - e0;
                    const QcCols col_of{s_blk + e0, r, p.Z};
                    for (int e = 0; e < deg; ++e) parity ^= a[col_of(e)] < 0.0f ? 1u : 0u;
                }
                if (ck::group_any(static_cast<int>(parity), bar, p.T)) return false;
            }
        }
        return true;
    }
    for (int32_t base = 0; base < p.m; base += p.T) {
        const int32_t row = base + tid;
        uint32_t parity = 0;
        if (row < p.m) {
            int deg;
            int32_t e0;
            const auto col_of = RowOf<QC>::get(p, s_eptr, s_blk, static_cast<uint32_t>(row), deg, e0);
            for (int e = 0; e < deg; ++e) parity ^= a[col_of(e)] < 0.0f ? 1u : 0u;
        }
        if (ck::group_any(static_cast<int>(parity), bar, p.T)) return false;
    }
    return true;
}

// Threads per block the kernels are built for (registers scale inversely;
// the any-degree kernels keep no per-edge registers).
__host__ __device__ constexpr int max_block_threads(bool qc, int dmax) {
    return dmax > 16 ? 512 : (qc ? 768 : 1024);
}

// Posterior access of the any-degree row loops: col(e) gives edge e's
// handle, ld/st read and write the posterior there.  Circulant rows address
// the group's shared-memory posterior through its shared-address table
// (gblk, r4 = 4 r, Z4 = 4 Z, as qc_row_fixed); CSR rows index `a`.
struct QcSmemPost {
    const int2* gblk;
    uint32_t r4, Z4;
    __device__ __forceinline__ uint32_t col(uint32_t e) const {
        const int2 b = gblk[e];
        const uint32_t c = r4 + static_cast<uint32_t>(b.x);
        return c >= static_cast<uint32_t>(b.y) ? c - Z4 : c;
    }
    __device__ __forceinline__ float ld(uint32_t c) const { return ld_shared_f32(c); }
    __device__ __forceinline__ void st(uint32_t c, float v) const { st_shared_f32(c, v); }
};
template <class ColOf>
struct CsrPost {
    float* a;
    const ColOf& col_of;
    __device__ __forceinline__ uint32_t col(uint32_t e) const { return static_cast<uint32_t>(col_of(static_cast<int>(e))); }
    __device__ __forceinline__ float ld(uint32_t c) const { return a[c]; }
    __device__ __forceinline__ void st(uint32_t c, float v) const { a[c] = v; }
};

// The layer loop of the table-driven kernels.
struct TableProgram {
    static constexpr bool kSpecialised = false;
};

// The kernel body.  ONE_ROW (circulant codes only): T >= Zp, so a thread
// owns one row of each base row it visits (row qr0 of base rows qb0, qb0 +
// q_bstep, ...) and the layer loop has no inner row loop (on code C 20 %
// faster than the general loop).  Prog: TableProgram, or a program
// specialised to one circulant code (T == Zp) whose
//   template <class St> static void iteration(const St& st, uint32_t base4,
//       uint32_t qr0, float scale, float offset, int bar, int T)
// runs one iteration (every layer, each followed by the group barrier) with
// the code's layers, degrees, block columns and shifts as constants, and
//   static bool syndrome(uint32_t base4, uint32_t qr0, int bar, int T)
// the early-stop test over the same rows (true in every thread of the group
// when every check holds); base4 is the shared address of the posterior
// plus 4 qr0.
template <template <bool> class State, bool QC, int DMAX, bool APP_SMEM, bool R_SMEM, bool ONE_ROW,
          class Prog>
__device__ __forceinline__ void decode_body(const Params& p) {
    extern __shared__ __align__(128) unsigned char smem[];
    using ck::group_any;
    using ck::group_sync;

    // Tables: layer pointers, then (QC) circulants per base row and the
    // circulants themselves.
    int32_t* s_layer = reinterpret_cast<int32_t*>(smem);
    int32_t* s_eptr = s_layer + (p.L + 1);
    int2* s_blk = reinterpret_cast<int2*>(smem + ((static_cast<uint32_t>(p.L + 1 + p.mb + 1) * 4 + 7) & ~7u));
    for (int i = threadIdx.x; i <= p.L; i += blockDim.x) s_layer[i] = p.layer[i];
    if (QC) {
        for (int i = threadIdx.x; i <= p.mb; i += blockDim.x) s_eptr[i] = p.eptr[i];
        for (int i = threadIdx.x; i < p.nnzb; i += blockDim.x) s_blk[i] = p.blk[i];
    }

    const int g = threadIdx.x / p.T;
    const int tid = threadIdx.x - g * p.T;
    const int bar = g + 1;
    // Circulant rows of this thread: row qr0 (+ T, + 2T, ... when T < Zp) of
    // base rows qb0, qb0 + q_bstep, ...  Zp and T are multiples of 32 and one
    // divides the other, so a warp's lanes always share their base row.
    const int32_t qr0 = QC ? (p.T >= p.Zp ? tid % p.Zp : tid) : 0;
    const int32_t qb0 = QC ? (p.T >= p.Zp ? tid / p.Zp : 0) : 0;
    const uint32_t slot = blockIdx.x * static_cast<uint32_t>(p.G) + static_cast<uint32_t>(g);
    unsigned char* gbase = smem + p.tables_bytes + static_cast<uint32_t>(g) * p.group_bytes;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(gbase);
    volatile uint32_t* s_frame = reinterpret_cast<volatile uint32_t*>(gbase + 8);
    float* a = APP_SMEM ? reinterpret_cast<float*>(gbase + p.app_off)
                        : p.g_app + static_cast<size_t>(slot) * p.app_stride;
    // The rule's check-message state of this group's frame slot.
    const State<R_SMEM> st(p, gbase, slot);
    // This group's copy of the circulant table as shared addresses into `a`.
    int2* gblk = reinterpret_cast<int2*>(gbase + p.gblk_off);

    if (tid == 0) {
        ck::mbar_init(mbar, 1);
        ck::fence_mbar_init();
    }
    __syncthreads();
    if (QC) {
        const uint32_t a_addr = ck::smem_addr(a);
        for (int i = tid; i < p.nnzb; i += p.T)
            gblk[i] = make_int2(static_cast<int>(a_addr + 4u * static_cast<uint32_t>(s_blk[i].x)),
                                static_cast<int>(a_addr + 4u * static_cast<uint32_t>(s_blk[i].y)));
    }
    const uint32_t r4 = 4u * static_cast<uint32_t>(qr0);
    const uint32_t Z4 = 4u * static_cast<uint32_t>(p.Z);

    uint32_t phase = 0;
    for (;;) {
        if (tid == 0) *s_frame = atomicAdd(p.counter, 1u);
        group_sync(bar, p.T);
        const uint32_t f = *s_frame;
        if (f >= p.B) break;
        const float* src = p.llr_in + static_cast<size_t>(f) * p.n_in;

        // Stage the frame's channel LLRs; punctured variables start at 0.
        bool loaded = true;
        if (APP_SMEM && p.bulk_load) {
            if (tid == 0) {
                ck::fence_proxy_async_smem();
                ck::mbar_arrive_expect_tx(mbar, static_cast<uint32_t>(p.n_in) * 4u);
                ck::bulk_g2s(a, src, static_cast<uint32_t>(p.n_in) * 4u, mbar);
            }
            for (int i = p.n_in + tid; i < p.N; i += p.T) a[i] = 0.0f;
            loaded = ck::mbar_wait(mbar, phase);
            phase ^= 1u;
            // x + 0 turns -0 into +0 and keeps every other value: the decoder
            // then never meets -0 (see qc_row_fixed).
            if (loaded)
                for (int i = tid; i < p.n_in; i += p.T) a[i] = __fadd_rn(a[i], 0.0f);
        } else {
            for (int i = tid; i < p.n_in; i += p.T) a[i] = __fadd_rn(__ldcs(src + i), 0.0f);
            for (int i = p.n_in + tid; i < p.N; i += p.T) a[i] = 0.0f;
        }
        if (group_any(loaded ? 0 : 1, bar, p.T)) {
            // A bulk copy did not complete in time: report and stop this
            // group after a last bounded wait for the copy in flight.
            if (tid == 0) {
                atomicOr(p.status, ck::kStatusTimeout);
                p.iters[f] = -1;
                p.valid[f] = 0;
            }
            (void)ck::mbar_wait(mbar, phase ^ 1u);
            return;
        }
        st.zero(p, tid, p.T);
        group_sync(bar, p.T);

        int32_t it = 0;
        // The syndrome test: the code's generated one, or the table-driven one.
        auto satisfied = [&]() -> bool {
            if constexpr (Prog::kSpecialised)
                return Prog::syndrome(ck::smem_addr(a) + 4u * static_cast<uint32_t>(qr0),
                                      static_cast<uint32_t>(qr0), bar, p.T, static_cast<uint32_t>(qb0));
            return syndrome_ok<QC>(p, a, s_eptr, s_blk, tid, bar, qr0, qb0);
        };
        // One call site of the test (it is long when generated): before the
        // first iteration and after each one with early stop, after the last
        // one without.
        bool ok = false;
        for (;;) {
            if (p.early_stop || it == p.max_iterations) ok = satisfied();
            if (ok || it >= p.max_iterations) break;
            if constexpr (Prog::kSpecialised) {
                Prog::iteration(st, ck::smem_addr(a) + 4u * static_cast<uint32_t>(qr0),
                                static_cast<uint32_t>(qr0), p.scale, p.offset, bar, p.T, static_cast<uint32_t>(qb0));
            }
            for (int32_t l = 0; l < p.L && QC && ONE_ROW && !Prog::kSpecialised; ++l) {
                if (qr0 < p.Z) {  // lanes past Z (Z % 32 != 0) only meet the barriers
                    const int32_t b1 = s_layer[l + 1];
                    for (int32_t b = s_layer[l] + qb0; b < b1; b += p.q_bstep) {
                        const int32_t e0 = s_eptr[b];
                        const int deg = s_eptr[b + 1] - e0;
                        const uint32_t row = static_cast<uint32_t>(b) * static_cast<uint32_t>(p.Z) +
                                             static_cast<uint32_t>(qr0);
                        st.template qc_row<DMAX>(p, gblk + e0, deg, row, e0, qr0, r4, Z4);
                    }
                }
                group_sync(bar, p.T);
            }
            for (int32_t l = 0; l < p.L && QC && !ONE_ROW && !Prog::kSpecialised; ++l) {
                const int32_t b1 = s_layer[l + 1];
                for (int32_t b = s_layer[l] + qb0; b < b1; b += p.q_bstep) {
                    const int32_t e0 = s_eptr[b];
                    const int deg = s_eptr[b + 1] - e0;
                    for (int32_t r = qr0; r - qr0 < p.Zp; r += p.T) {
                        if (r >= p.Z) continue;  // padding lanes when Z % 32 != 0
                        const uint32_t row = static_cast<uint32_t>(b) * static_cast<uint32_t>(p.Z) +
                                             static_cast<uint32_t>(r);
                        st.template qc_row<DMAX>(p, gblk + e0, deg, row, e0, r,
                                                 r4 + 4u * static_cast<uint32_t>(r - qr0), Z4);
                    }
                }
                group_sync(bar, p.T);
            }
            for (int32_t l = 0; l < p.L && !QC; ++l) {
                const uint32_t row0 = s_layer[l];
                const uint32_t row1 = s_layer[l + 1];
                for (uint32_t row = row0 + tid; row < row1; row += p.T) {
                    int deg;
                    int32_t e0;
                    const auto col_of = RowOf<QC>::get(p, s_eptr, s_blk, row, deg, e0);
                    st.template csr_row<DMAX>(p, a, row, deg, e0, col_of);
                }
                group_sync(bar, p.T);
            }
            ++it;
        }

        float* dst = p.llr_out + static_cast<size_t>(f) * p.n_in;
        for (int i = tid; i < p.n_in; i += p.T) __stcs(dst + i, a[i]);
        if (p.bits) {
            int8_t* bdst = p.bits + static_cast<size_t>(f) * p.k_bits;
            for (int i = tid; i < p.k_bits; i += p.T) bdst[i] = a[i] < 0.0f ? 1 : 0;
        }
        if (tid == 0) {
            p.iters[f] = it;
            p.valid[f] = ok ? 1 : 0;
        }
        // Everyone has read `a` before the next frame overwrites it.
        group_sync(bar, p.T);
    }
}

template <template <bool> class State, bool QC, int DMAX, bool APP_SMEM, bool R_SMEM, bool ONE_ROW>
__global__ void __launch_bounds__(max_block_threads(QC, DMAX))
    decode_kernel(const __grid_constant__ Params p) {
    decode_body<State, QC, DMAX, APP_SMEM, R_SMEM, ONE_ROW, TableProgram>(p);
}

#ifndef __CUDACC_RTC__
using KernelFn = void (*)(Params);

// The decoder kernel of a rule for a code shape (quasi-cyclic or CSR, its
// longest row, where the posterior and the message state live); nullptr
// when no such kernel exists.
KernelFn min_sum_kernel(bool qc, int max_deg, bool app_smem, bool r_smem, bool one_row);
KernelFn sum_product_kernel(bool qc, int max_deg, bool app_smem, bool r_smem, bool one_row);
// The cluster kernel of a rule for CSR codes (posterior and messages in
// device memory) whose longest row has max_deg edges.
KernelFn min_sum_cluster_kernel(int max_deg);
KernelFn sum_product_cluster_kernel(int max_deg);

// Kernels are built for these row-degree bounds: 16, 27 and any (0), CSR
// codes also 8 (kernel_dmax).
template <class Pick>
KernelFn pick_shape(bool qc, int max_deg, bool app_smem, bool r_smem, bool one_row) {
    if (!app_smem && (qc || r_smem)) return nullptr;  // circulant rows address shared memory
    const int d = kernel_dmax(qc, max_deg);
    if (!qc) {
        if (d == 8) return Pick::template get<false, 8, false>(app_smem, r_smem);
        if (d == 16) return Pick::template get<false, 16, false>(app_smem, r_smem);
        if (d == 27) return Pick::template get<false, 27, false>(app_smem, r_smem);
        return Pick::template get<false, 0, false>(app_smem, r_smem);
    }
    if (one_row) {
        if (d == 16) return Pick::template get<true, 16, true>(app_smem, r_smem);
        if (d == 27) return Pick::template get<true, 27, true>(app_smem, r_smem);
        return Pick::template get<true, 0, true>(app_smem, r_smem);
    }
    if (d == 16) return Pick::template get<true, 16, false>(app_smem, r_smem);
    if (d == 27) return Pick::template get<true, 27, false>(app_smem, r_smem);
    return Pick::template get<true, 0, false>(app_smem, r_smem);
}

#endif  // __CUDACC_RTC__

}  // namespace ldpc
}  // namespace ck
