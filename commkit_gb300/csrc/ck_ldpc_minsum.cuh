// The min-sum check rule of the layered decoder: the row updates (CSR and
// circulant) and the compressed check-message state, for decode_kernel
// (ck_ldpc_kernel.cuh), the mixed-code kernel and the code-specialised
// kernels compiled at run time (ck_ldpc_jit.cu).  Compiles under NVRTC.
#pragma once

#include "ck_ldpc_kernel.cuh"

namespace ck {
namespace ldpc {


// One check row, min-sum: reads the row's compressed state (m1, m2, w),
// updates the posterior `a` of its deg variables (columns from col_of) and
// writes the new state back.  Two passes as the reference's min_sum_row
// (commkit/_cuda/src/ldpc.cu:45-72), with Q and the columns kept in
// registers between them.
template <int DMAX, class ColOf>
__device__ __forceinline__ void min_sum_row(float* __restrict__ a, const int deg,
                                            const ColOf& col_of, float& m1, float& m2,
                                            uint32_t& w, const float scale,
                                            const float offset) {
    const uint32_t oidx = w >> 27;
    const uint32_t osign = w;
    const float om1 = m1, om2 = m2;
    float q[DMAX];
    int col[DMAX];  // loaded once, all before the first posterior load
    float min1 = ck::inf_f(), min2 = ck::inf_f();
    uint32_t idx = 31u;  // no edge; matches the reference's -1 when every |Q| is inf
    uint32_t negs = 0u;
#pragma unroll
    for (int e = 0; e < DMAX; ++e)
        if (e < deg) col[e] = col_of(e);
#pragma unroll
    for (int e = 0; e < DMAX; ++e) {
        if (e < deg) {
            const float r_old =
                flip_sign(static_cast<uint32_t>(e) == oidx ? om2 : om1, (osign >> e) & 1u);
            const float qe = __fsub_rn(a[col[e]], r_old);
            q[e] = qe;
            negs |= (qe < 0.0f ? 1u : 0u) << e;
            const float mag = fabsf(qe);
            if (mag < min1) idx = static_cast<uint32_t>(e);
            min2 = fminf(min2, fmax_nan(min1, mag));
            min1 = fminf(min1, mag);
        }
    }
    const float n1 = fmaxf(__fsub_rn(__fmul_rn(scale, min1), offset), 0.0f);
    const float n2 = fmaxf(__fsub_rn(__fmul_rn(scale, min2), offset), 0.0f);
    // Sign of edge e's new message: the parity of all signs times its own.
    const uint32_t signs = negs ^ ((__popc(negs) & 1u) ? 0xffffffffu : 0u);
#pragma unroll
    for (int e = 0; e < DMAX; ++e) {
        if (e < deg) {
            const float rn = flip_sign(static_cast<uint32_t>(e) == idx ? n2 : n1, (signs >> e) & 1u);
            a[col[e]] = __fadd_rn(q[e], rn);
        }
    }
    m1 = n1;
    m2 = n2;
    w = (signs & 0x07ffffffu) | (idx << 27);
}

// The same update for a circulant row of exactly D edges, shaped for the
// ALU pipe, which bounds this kernel: fully unrolled, columns computed once
// and kept in registers,
//  * min1/min2 taken over pairs of edges: with lo/hi the pair's smaller and
//    larger magnitude, min2 = min(min2, hi, max(min1, lo)) and min1 =
//    min(min1, lo), five operations per pair instead of six (three-input
//    min), and half as long a dependency chain; a NaN magnitude (only from
//    infinite input LLRs) drops out of both, as in the reference,
//  * the sign bits of Q taken from the float sign (no -0 ever reaches the
//    posterior: frames are loaded as x + 0, and from such values Q = APP - R
//    and APP = Q + R_new cannot produce -0 either, so "sign bit set" is
//    "Q < 0"), one funnel shift per edge;
//  * the new signs applied with one multiply by the parity sign (exact) and
//    one bitwise or;
//  * no running argmin: an edge takes min2' when |Q| equals min1 (a tie
//    means min2 == min1, so every tied edge gets the same value), and the
//    stored argmin is the first such edge, found in the second pass.
// The compressed state keeps the sign of edge e at bit D - 1 - e here.
// The row's columns come as shared-memory addresses c[0..D).
template <int D>
__device__ __forceinline__ void qc_row_cols(const uint32_t (&c)[D], float& m1, float& m2, uint32_t& w,
                                            const float scale, const float offset) {
    const uint32_t oidx = w >> 27;
    const uint32_t osign = w;
    const float om1 = m1, om2 = m2;
    float q[D];
    float min1 = ck::inf_f(), min2 = ck::inf_f();
    uint32_t negs = 0u;
#pragma unroll
    for (int e = 0; e < D; ++e) {
        const uint32_t ce = c[e];
        const float mag_old = static_cast<uint32_t>(e) == oidx ? om2 : om1;
        const float r_old = __uint_as_float(__float_as_uint(mag_old) ^
                                            ((osign << (32 - D + e)) & 0x80000000u));
        const float qe = __fsub_rn(ld_shared_f32(ce), r_old);
        q[e] = qe;
        negs = __funnelshift_l(__float_as_uint(qe), negs, 1);
        if (e & 1) {
            const float x = fabsf(q[e - 1]), y = fabsf(qe);
            const float hi = fmax_nan(x, y);
            if (e == 1) {
                min1 = fmin3(x, y, ck::inf_f());
                min2 = fminf(hi, ck::inf_f());
            } else {
                const float lo = fminf(x, y);
                min2 = fmin3(min2, hi, fmax_nan(min1, lo));
                min1 = fminf(min1, lo);
            }
        } else if (e == D - 1) {
            const float mag = fabsf(qe);
            min2 = fminf(min2, fmax_nan(min1, mag));
            min1 = fminf(min1, mag);
        }
    }
    const float n1 = fmaxf(__fsub_rn(__fmul_rn(scale, min1), offset), 0.0f);
    const float n2 = fmaxf(__fsub_rn(__fmul_rn(scale, min2), offset), 0.0f);
    const bool odd = __popc(negs) & 1u;
    const float psign = odd ? -1.0f : 1.0f;
    uint32_t idx = 31u;
#pragma unroll
    for (int e = D - 1; e >= 0; --e) {
        const bool at_min = fabsf(q[e]) == min1;
        if (at_min) idx = static_cast<uint32_t>(e);
        const float mag = at_min ? n2 : n1;
        const float t = __fmul_rn(q[e], psign);
        const float rn = __uint_as_float(__float_as_uint(mag) | (__float_as_uint(t) & 0x80000000u));
        st_shared_f32(c[e], __fadd_rn(q[e], rn));
    }
    const uint32_t signs = negs ^ (odd ? ((1u << D) - 1u) : 0u);
    m1 = n1;
    m2 = n2;
    w = (signs & 0x07ffffffu) | (idx << 27);
}

// Row-qr0 column base of a circulant with shift s in the code-specialised
// programs, on the FMA pipe (the kernel is bound by the ALU pipe): the wrap
// (qr0 + s >= Z) is the high word of qr0 * M + s * M with M = ceil(2^32 / Z)
// (exact: qr0 + s < 2 Z and (qr0 + s) Z < 2^32), and the base is
// base4 - wrap * 4 Z; the caller adds the column's constant part.
__device__ __forceinline__ uint32_t wrapped_base(uint32_t base4, uint32_t qr0, uint32_t M, uint64_t sM,
                                                 uint32_t neg_z4) {
    uint32_t hi, c;
    asm("{\n\t.reg .u64 t;\n\t.reg .u32 lo;\n\tmad.wide.u32 t, %1, %2, %3;\n\tmov.b64 {lo, %0}, t;\n\t}"
        : "=r"(hi)
        : "r"(qr0), "r"(M), "l"(sM));
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(c) : "r"(hi), "r"(neg_z4), "r"(base4));
    return c;
}

// Row r of a circulant base row: gblk[e] = (shared address of circulant
// e's row-0 column, address of its block's end), r4 = 4 r, Z4 = 4 Z; row
// r's column is r4 + gblk[e].x, wrapped back by Z4 once it reaches the end.
template <int D>
__device__ __forceinline__ void qc_row_fixed(const int2* __restrict__ gblk, const uint32_t r4,
                                             const uint32_t Z4, float& m1, float& m2, uint32_t& w,
                                             const float scale, const float offset) {
    uint32_t c[D];
#pragma unroll
    for (int e = 0; e < D; ++e) {
        const int2 b = gblk[e];
        const uint32_t ce = r4 + static_cast<uint32_t>(b.x);
        c[e] = ce >= static_cast<uint32_t>(b.y) ? ce - Z4 : ce;
    }
    qc_row_cols<D>(c, m1, m2, w, scale, offset);
}

// Degree dispatch of a circulant row (warp-uniform): D = 2..DMAX unrolled,
// with no case above DMAX (a switch over 2..16 rather than 2..27 for the
// DMAX = 16 kernels).
#define CK_ROW_CASE(D) \
    case D:            \
        qc_row_fixed<D>(gblk, r4, Z4, m1, m2, w, scale, offset); \
        break;
template <int DMAX>
__device__ __forceinline__ void qc_row(const int2* __restrict__ gblk, const int deg,
                                       const uint32_t r4, const uint32_t Z4, float& m1, float& m2,
                                       uint32_t& w, const float scale, const float offset) {
    if constexpr (DMAX <= 16) {
        switch (deg) {
            CK_ROW_CASE(2) CK_ROW_CASE(3) CK_ROW_CASE(4) CK_ROW_CASE(5) CK_ROW_CASE(6)
            CK_ROW_CASE(7) CK_ROW_CASE(8) CK_ROW_CASE(9) CK_ROW_CASE(10) CK_ROW_CASE(11)
            CK_ROW_CASE(12) CK_ROW_CASE(13) CK_ROW_CASE(14) CK_ROW_CASE(15) CK_ROW_CASE(16)
            default:
                break;
        }
    } else {
        switch (deg) {
            CK_ROW_CASE(2) CK_ROW_CASE(3) CK_ROW_CASE(4) CK_ROW_CASE(5) CK_ROW_CASE(6)
            CK_ROW_CASE(7) CK_ROW_CASE(8) CK_ROW_CASE(9) CK_ROW_CASE(10) CK_ROW_CASE(11)
            CK_ROW_CASE(12) CK_ROW_CASE(13) CK_ROW_CASE(14) CK_ROW_CASE(15) CK_ROW_CASE(16)
            CK_ROW_CASE(17) CK_ROW_CASE(18) CK_ROW_CASE(19) CK_ROW_CASE(20) CK_ROW_CASE(21)
            CK_ROW_CASE(22) CK_ROW_CASE(23) CK_ROW_CASE(24) CK_ROW_CASE(25) CK_ROW_CASE(26)
            CK_ROW_CASE(27)
            default:
                break;
        }
    }
}
#undef CK_ROW_CASE

// Min-sum check-message state of a frame slot: per row (min1', min2', one
// word of signs and argmin).  In shared memory one 16-byte record per row
// (one vector access); in device memory 12 bytes, an array of (min1',
// min2') pairs and one of words (two accesses), so the resident frames'
// state (code C: 304 frames x 17664 rows x 12 B = 64 MB) stays in L2.  (A
// 16-byte record there measured 17 % slower on code C: 86 MB of state
// leaves too little of L2 to the rest.)
template <bool R_SMEM>
struct MinSumState {
    uint4* rs;
    uint2* g12;
    uint32_t* g3;
    // Device-memory records written with the L2 priority "evict last"
    // (policy `keep`): the plain kernels.  Measured: code C's DRAM writes
    // per 304-frame launch fell from 806 MB (the records written back
    // between iterations) to 14 MB at the same speed; in the mixed kernel
    // the same stores made the config-4 step 1.4 % slower on one box, so it
    // writes them as before (and its launch wrote 25 MB per 2048 frames).
    bool hint;
    uint64_t keep;

    __device__ __forceinline__ MinSumState(const Params& p, unsigned char* gbase, uint32_t slot)
        : MinSumState(reinterpret_cast<uint4*>(gbase + p.r_off), p.g_r, slot, p.r_stride, !R_SMEM) {}
    // rs: the group's records in shared memory; g_r: the device-memory
    // state slots (3 r_stride words each), slot: this group's.
    __device__ __forceinline__ MinSumState(uint4* rs_, uint32_t* g_r, uint32_t slot, uint32_t r_stride,
                                           bool hint_ = false)
        : rs(rs_),
          g12(reinterpret_cast<uint2*>(g_r + static_cast<size_t>(slot) * 3 * r_stride)),
          g3(g_r + static_cast<size_t>(slot) * 3 * r_stride + 2 * r_stride),
          hint(hint_),
          keep(hint_ ? ck::l2_keep_policy() : 0ull) {}
    // The mixed kernel's form (the same state, no L2 hint; sign_words is unused).
    __device__ __forceinline__ MinSumState(unsigned char* rsm, uint32_t* g_r, uint32_t slot, uint32_t r_stride,
                                           int32_t)
        : MinSumState(reinterpret_cast<uint4*>(rsm), g_r, slot, r_stride, false) {}

    __device__ __forceinline__ void zero(const Params& p, int first, int stride) const {
        zero_rows(p.m, first, stride);
    }
    __device__ __forceinline__ void zero_rows(int32_t m, int first, int stride) const {
        for (int i = first; i < m; i += stride) {
            if (R_SMEM) {
                rs[i] = make_uint4(0u, 0u, 0u, 0u);
            } else if (hint) {
                ck::st_l2keep(g12 + i, make_uint2(0u, 0u), keep);
                ck::st_l2keep(g3 + i, 0u, keep);
            } else {
                g12[i] = make_uint2(0u, 0u);
                g3[i] = 0u;
            }
        }
    }
    // In device memory the records are re-read every iteration; the plain
    // kernels write them with the L2 priority "evict last" (ck::st_l2keep),
    // which keeps them there while frames stream through.  The loads stay
    // plain L2 loads the compiler may schedule freely.
    __device__ __forceinline__ uint4 load(uint32_t row) const {
        if (R_SMEM) return rs[row];
        const uint2 m = __ldcg(g12 + row);
        return make_uint4(m.x, m.y, __ldcg(g3 + row), 0u);
    }
    __device__ __forceinline__ void store(uint32_t row, float m1, float m2, uint32_t w) const {
        if (R_SMEM) {
            rs[row] = make_uint4(__float_as_uint(m1), __float_as_uint(m2), w, 0u);
        } else if (hint) {
            ck::st_l2keep(g12 + row, make_uint2(__float_as_uint(m1), __float_as_uint(m2)), keep);
            ck::st_l2keep(g3 + row, w, keep);
        } else {
            __stcg(g12 + row, make_uint2(__float_as_uint(m1), __float_as_uint(m2)));
            __stcg(g3 + row, w);
        }
    }
    template <int DMAX>
    __device__ __forceinline__ void qc_row(const Params& p, const int2* gblk, int deg, uint32_t row,
                                           int32_t e0, int32_t, uint32_t r4, uint32_t Z4) const {
        qc_row_k<DMAX>(gblk, deg, row, e0, r4, Z4, p.scale, p.offset);
    }
    template <int DMAX>
    __device__ __forceinline__ void qc_row_k(const int2* gblk, int deg, uint32_t row, int32_t, uint32_t r4,
                                             uint32_t Z4, float scale, float offset) const {
        const uint4 s = load(row);
        float m1 = __uint_as_float(s.x), m2 = __uint_as_float(s.y);
        uint32_t w = s.z;
        ck::ldpc::qc_row<DMAX>(gblk, deg, r4, Z4, m1, m2, w, scale, offset);
        store(row, m1, m2, w);
    }
    // Load-ahead for the code-specialised programs: pre(row) starts loading
    // a row's state one row early when it lives in device memory (L2
    // latency); take(pre, row) gives the row's state (the early load, or a
    // shared-memory load now).
    __device__ __forceinline__ uint4 pre(uint32_t row) const {
        return R_SMEM ? make_uint4(0u, 0u, 0u, 0u) : load(row);
    }
    __device__ __forceinline__ uint4 take(const uint4 early, uint32_t row) const {
        return R_SMEM ? load(row) : early;
    }
    // One circulant row with its columns computed by the caller (the
    // code-specialised programs), its state `s` from take(); the edge-state
    // form's message offset and lifting are unused here.
    template <int D, uint32_t Z4>
    __device__ __forceinline__ void row_cols(const uint32_t (&c)[D], const uint4 s, uint32_t row, uint32_t,
                                             float scale, float offset) const {
        float m1 = __uint_as_float(s.x), m2 = __uint_as_float(s.y);
        uint32_t w = s.z;
        qc_row_cols<D>(c, m1, m2, w, scale, offset);
        store(row, m1, m2, w);
    }
    template <int DMAX, class ColOf>
    __device__ __forceinline__ void csr_row(const Params& p, float* a, uint32_t row, int deg, int32_t,
                                            const ColOf& col_of) const {
        const uint4 s = load(row);
        float m1 = __uint_as_float(s.x), m2 = __uint_as_float(s.y);
        uint32_t w = s.z;
        min_sum_row<DMAX>(a, deg, col_of, m1, m2, w, p.scale, p.offset);
        store(row, m1, m2, w);
    }
};



// Min-sum check-message state of codes with rows above kPackedDegree edges
// (the any-degree kernels, row-degree bound 0).  Per row: (min1', min2') as
// a pair, the argmin as a whole word, and the row's sign bits in
// sign_words words (bit j of word w is edge 32 w + j).  Each of these is an
// array of r_stride entries, so rows on consecutive lanes touch consecutive
// words: (3 + sign_words) r_stride words per frame slot, in the group's
// shared memory or in the slot's device memory.  Still lossless: the
// message of row i edge e is sign_e * (e == argmin ? min2' : min1').
template <bool R_SMEM>
struct WideMinSumState {
    uint32_t* w;  // the slot's words
    uint32_t r_stride;
    int32_t nw;

    __device__ __forceinline__ WideMinSumState(const Params& p, unsigned char* gbase, uint32_t slot)
        : WideMinSumState(gbase + p.r_off, p.g_r, slot, p.r_stride, p.sign_words) {}
    __device__ __forceinline__ WideMinSumState(unsigned char* rsm, uint32_t* g_r, uint32_t slot,
                                               uint32_t r_stride_, int32_t sign_words)
        : w(R_SMEM ? reinterpret_cast<uint32_t*>(rsm)
                   : g_r + static_cast<size_t>(slot) * static_cast<uint32_t>(3 + sign_words) * r_stride_),
          r_stride(r_stride_),
          nw(sign_words) {}

    __device__ __forceinline__ uint32_t ld(uint32_t i) const { return R_SMEM ? w[i] : __ldcg(w + i); }
    __device__ __forceinline__ void st(uint32_t i, uint32_t v) const {
        if (R_SMEM)
            w[i] = v;
        else
            __stcg(w + i, v);
    }
    __device__ __forceinline__ uint2 ld2(uint32_t row) const {
        const uint2* m = reinterpret_cast<const uint2*>(w);
        return R_SMEM ? m[row] : __ldcg(m + row);
    }
    __device__ __forceinline__ void st2(uint32_t row, float m1, float m2) const {
        uint2* m = reinterpret_cast<uint2*>(w);
        const uint2 v = make_uint2(__float_as_uint(m1), __float_as_uint(m2));
        if (R_SMEM)
            m[row] = v;
        else
            __stcg(m + row, v);
    }

    __device__ __forceinline__ void zero(const Params& p, int first, int stride) const {
        zero_rows(p.m, first, stride);
    }
    __device__ __forceinline__ void zero_rows(int32_t m, int first, int stride) const {
        for (int i = first; i < m; i += stride) {
            st2(static_cast<uint32_t>(i), 0.0f, 0.0f);
            for (int32_t k = 0; k <= nw; ++k) st((2u + static_cast<uint32_t>(k)) * r_stride + i, 0u);
        }
    }

    // One row of any degree: the reference's two passes
    // (commkit/_cuda/src/ldpc.cu:45-72) edge by edge, with Q recomputed in
    // the second pass from the unchanged posterior and the old state (the
    // same float operations, so the same Q), and the new sign bits written
    // a word at a time after that word's old bits have been read.
    template <class Post>
    __device__ __forceinline__ void any_row(const Post& post, const int deg, const uint32_t row, const float scale,
                                            const float offset) const {
        const uint2 om = ld2(row);
        const float om1 = __uint_as_float(om.x), om2 = __uint_as_float(om.y);
        const uint32_t oidx = ld(2u * r_stride + row);
        float min1 = ck::inf_f(), min2 = ck::inf_f();
        uint32_t idx = 0xffffffffu;  // no edge, the reference's -1
        uint32_t par = 0u;
        for (int w0 = 0; w0 < deg; w0 += 32) {
            const uint32_t os = ld((3u + static_cast<uint32_t>(w0 >> 5)) * r_stride + row);
            const int n = min(32, deg - w0);
            for (int j = 0; j < n; ++j) {
                const uint32_t e = static_cast<uint32_t>(w0 + j);
                const float r_old = flip_sign(e == oidx ? om2 : om1, (os >> j) & 1u);
                const float q = __fsub_rn(post.ld(post.col(e)), r_old);
                par ^= q < 0.0f ? 1u : 0u;
                const float mag = fabsf(q);
                if (mag < min1) {
                    min2 = min1;
                    min1 = mag;
                    idx = e;
                } else if (mag < min2) {
                    min2 = mag;
                }
            }
        }
        const float n1 = fmaxf(__fsub_rn(__fmul_rn(scale, min1), offset), 0.0f);
        const float n2 = fmaxf(__fsub_rn(__fmul_rn(scale, min2), offset), 0.0f);
        for (int w0 = 0; w0 < deg; w0 += 32) {
            const uint32_t wi = (3u + static_cast<uint32_t>(w0 >> 5)) * r_stride + row;
            const uint32_t os = ld(wi);
            uint32_t ns = 0u;
            const int n = min(32, deg - w0);
            for (int j = 0; j < n; ++j) {
                const uint32_t e = static_cast<uint32_t>(w0 + j);
                const uint32_t c = post.col(e);
                const float r_old = flip_sign(e == oidx ? om2 : om1, (os >> j) & 1u);
                const float q = __fsub_rn(post.ld(c), r_old);
                const uint32_t sgn = par ^ (q < 0.0f ? 1u : 0u);
                const float rn = flip_sign(e == idx ? n2 : n1, sgn);
                post.st(c, __fadd_rn(q, rn));
                ns |= sgn << j;
            }
            st(wi, ns);
        }
        st2(row, n1, n2);
        st(2u * r_stride + row, idx);
    }

    template <int DMAX>
    __device__ __forceinline__ void qc_row(const Params& p, const int2* gblk, int deg, uint32_t row,
                                           int32_t, int32_t, uint32_t r4, uint32_t Z4) const {
        any_row(QcSmemPost{gblk, r4, Z4}, deg, row, p.scale, p.offset);
    }
    template <int DMAX>
    __device__ __forceinline__ void qc_row_k(const int2* gblk, int deg, uint32_t row, int32_t, uint32_t r4,
                                             uint32_t Z4, float scale, float offset) const {
        any_row(QcSmemPost{gblk, r4, Z4}, deg, row, scale, offset);
    }
    template <int DMAX, class ColOf>
    __device__ __forceinline__ void csr_row(const Params& p, float* a, uint32_t row, int deg, int32_t,
                                            const ColOf& col_of) const {
        any_row(CsrPost<ColOf>{a, col_of}, deg, row, p.scale, p.offset);
    }
};

// One circulant row of exactly D edges with one message per edge (the
// edge state below): c[e] the shared addresses of its posteriors, mo[e] of
// its messages.  The reference's two passes (commkit/_cuda/src/ldpc.cu:45-72)
// with the record form's reductions (qc_row_cols: min1/min2 over pairs of
// edges, min2' for every edge whose |Q| equals min1), so the same floats:
//  * Q = APP - R_old, the old message a plain load;
//  * the row's sign parity is bit 31 of the XOR of its Q words (no -0
//    reaches Q and its NaNs are positive, so the sign bit is "Q < 0");
//  * the parity goes onto min1' and min2' once per row, and each edge's new
//    message is the chosen magnitude with its own Q sign XORed in.
template <int D>
__device__ __forceinline__ void qc_row_edges(const uint32_t (&c)[D], const uint32_t (&mo)[D], const float scale,
                                             const float offset) {
    float q[D];
    float min1 = ck::inf_f(), min2 = ck::inf_f();
    uint32_t par = 0u;
#pragma unroll
    for (int e = 0; e < D; ++e) {
        const float qe = __fsub_rn(ld_shared_f32(c[e]), ld_shared_f32(mo[e]));
        q[e] = qe;
        par ^= __float_as_uint(qe);
        if (e & 1) {
            const float x = fabsf(q[e - 1]), y = fabsf(qe);
            const float hi = fmax_nan(x, y);
            if (e == 1) {
                min1 = fmin3(x, y, ck::inf_f());
                min2 = fminf(hi, ck::inf_f());
            } else {
                const float lo = fminf(x, y);
                min2 = fmin3(min2, hi, fmax_nan(min1, lo));
                min1 = fminf(min1, lo);
            }
        } else if (e == D - 1) {
            const float mag = fabsf(qe);
            min2 = fminf(min2, fmax_nan(min1, mag));
            min1 = fminf(min1, mag);
        }
    }
    const float n1 = fmaxf(__fsub_rn(__fmul_rn(scale, min1), offset), 0.0f);
    const float n2 = fmaxf(__fsub_rn(__fmul_rn(scale, min2), offset), 0.0f);
    const uint32_t ps = par & 0x80000000u;
    const uint32_t p1 = __float_as_uint(n1) ^ ps, p2 = __float_as_uint(n2) ^ ps;
#pragma unroll
    for (int e = 0; e < D; ++e) {
        const uint32_t pm = fabsf(q[e]) == min1 ? p2 : p1;
        const float rn = __uint_as_float(pm ^ (__float_as_uint(q[e]) & 0x80000000u));
        st_shared_f32(mo[e], rn);
        st_shared_f32(c[e], __fadd_rn(q[e], rn));
    }
}

// The table-driven form: row r of a circulant base row, gblk[e] and r4/Z4
// as in qc_row_fixed, m_r the shared address of circulant 0's message of
// row r (circulant e's is Z4 bytes further per e).
template <int D>
__device__ __forceinline__ void qc_row_edges_fixed(const int2* __restrict__ gblk, const uint32_t r4,
                                                   const uint32_t Z4, const uint32_t m_r, const float scale,
                                                   const float offset) {
    uint32_t c[D], mo[D];
#pragma unroll
    for (int e = 0; e < D; ++e) {
        const int2 b = gblk[e];
        const uint32_t ce = r4 + static_cast<uint32_t>(b.x);
        c[e] = ce >= static_cast<uint32_t>(b.y) ? ce - Z4 : ce;
        mo[e] = m_r + static_cast<uint32_t>(e) * Z4;
    }
    qc_row_edges<D>(c, mo, scale, offset);
}

// Min-sum check-message state of one message per edge, in the group's
// shared memory (R_SMEM only): circulant i of a circulant code keeps row
// r's message at i Z + r, as sum-product does, so a warp's lanes
// (consecutive r) touch consecutive words; r_stride messages (E rounded up
// to 32) per frame.  Uncompressed, it is the reference's own message array:
// the old message is a load rather than a select and a sign flip out of a
// packed record, and no signs or argmin are packed back, which leaves about
// half the ALU work per edge of the record form.  It takes E words against
// the record's four per row, so it serves codes of a few thousand edges
// (the plan offers it as CK_LDPC_PLACE_EDGES, for code-specialised
// circulant decoders of rows up to 27 edges); the results are the same bits
// as every other placement's.
template <bool R_SMEM>
struct EdgeMinSumState {
    static_assert(R_SMEM, "the per-edge min-sum state lives in shared memory");
    uint32_t m0;     // shared address of the frame slot's first message
    uint32_t count;  // messages per frame slot

    __device__ __forceinline__ EdgeMinSumState(const Params& p, unsigned char* gbase, uint32_t)
        : m0(ck::smem_addr(gbase + p.r_off)), count(static_cast<uint32_t>(p.r_stride)) {}
    // The mixed kernel's form: rsm the group's state region, r_stride its
    // message count.
    __device__ __forceinline__ EdgeMinSumState(unsigned char* rsm, uint32_t*, uint32_t, uint32_t r_stride,
                                               int32_t)
        : m0(ck::smem_addr(rsm)), count(r_stride) {}

    __device__ __forceinline__ void zero(const Params&, int first, int stride) const {
        zero_rows(0, first, stride);
    }
    __device__ __forceinline__ void zero_rows(int32_t, int first, int stride) const {
        for (uint32_t i = static_cast<uint32_t>(first); i < count; i += static_cast<uint32_t>(stride))
            st_shared_f32(m0 + 4u * i, 0.0f);
    }
    // Row r of the base row whose circulants are e0 .. e0 + deg of the table.
    template <int DMAX>
    __device__ __forceinline__ void qc_row(const Params& p, const int2* gblk, int deg, uint32_t row,
                                           int32_t e0, int32_t, uint32_t r4, uint32_t Z4) const {
        qc_row_k<DMAX>(gblk, deg, row, e0, r4, Z4, p.scale, p.offset);
    }
    template <int DMAX>
    __device__ __forceinline__ void qc_row_k(const int2* gblk, int deg, uint32_t, int32_t e0, uint32_t r4,
                                             uint32_t Z4, float scale, float offset) const {
        static_assert(DMAX == 16 || DMAX == 27, "per-edge messages serve rows of up to 27 edges");
        const uint32_t m_r = m0 + r4 + static_cast<uint32_t>(e0) * Z4;
#define CK_EDGE_CASE(D) \
    case D:             \
        qc_row_edges_fixed<D>(gblk, r4, Z4, m_r, scale, offset); \
        break;
        switch (deg) {
            CK_EDGE_CASE(2) CK_EDGE_CASE(3) CK_EDGE_CASE(4) CK_EDGE_CASE(5) CK_EDGE_CASE(6)
            CK_EDGE_CASE(7) CK_EDGE_CASE(8) CK_EDGE_CASE(9) CK_EDGE_CASE(10) CK_EDGE_CASE(11)
            CK_EDGE_CASE(12) CK_EDGE_CASE(13) CK_EDGE_CASE(14) CK_EDGE_CASE(15) CK_EDGE_CASE(16)
            default:
                break;
        }
        if constexpr (DMAX > 16) {
            switch (deg) {
                CK_EDGE_CASE(17) CK_EDGE_CASE(18) CK_EDGE_CASE(19) CK_EDGE_CASE(20) CK_EDGE_CASE(21)
                CK_EDGE_CASE(22) CK_EDGE_CASE(23) CK_EDGE_CASE(24) CK_EDGE_CASE(25) CK_EDGE_CASE(26)
                CK_EDGE_CASE(27)
                default:
                    break;
            }
        }
#undef CK_EDGE_CASE
    }
    // The code-specialised programs' form: nothing to load ahead per row.
    __device__ __forceinline__ uint4 pre(uint32_t) const { return make_uint4(0u, 0u, 0u, 0u); }
    __device__ __forceinline__ uint4 take(const uint4, uint32_t) const { return make_uint4(0u, 0u, 0u, 0u); }
    // One circulant row with its columns computed by the caller: mo4 = 4 (e0
    // Z + r) for its first circulant e0 and row r, Z4 = 4 Z a constant.
    template <int D, uint32_t Z4>
    __device__ __forceinline__ void row_cols(const uint32_t (&c)[D], const uint4, uint32_t, uint32_t mo4,
                                             float scale, float offset) const {
        uint32_t mo[D];
#pragma unroll
        for (int e = 0; e < D; ++e) mo[e] = m0 + mo4 + static_cast<uint32_t>(e) * Z4;
        qc_row_edges<D>(c, mo, scale, offset);
    }
    // Circulant codes only: the frame loop's CSR branch is compiled for every
    // state but never runs with this one.
    template <int DMAX, class ColOf>
    __device__ __forceinline__ void csr_row(const Params&, float*, uint32_t, int, int32_t, const ColOf&) const {}
};

// The min-sum state of the kernels with row-degree bound DMAX: the packed
// record, or the wide one for any degree (DMAX = 0).
template <int DMAX, bool R_SMEM>
struct MinSumFor {
    using type = MinSumState<R_SMEM>;
};
template <bool R_SMEM>
struct MinSumFor<0, R_SMEM> {
    using type = WideMinSumState<R_SMEM>;
};
// The same, or the per-edge state (EDGES).
template <int DMAX, bool R_SMEM, bool EDGES>
struct MinSumStateOf {
    using type = typename MinSumFor<DMAX, R_SMEM>::type;
};
template <int DMAX, bool R_SMEM>
struct MinSumStateOf<DMAX, R_SMEM, true> {
    using type = EdgeMinSumState<true>;
};


}  // namespace ldpc
}  // namespace ck
