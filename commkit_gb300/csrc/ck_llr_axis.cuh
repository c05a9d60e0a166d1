// Closed-form max-log LLRs of one axis of a separable constellation
// (commkit/_cuda/src/llr.cu:262-302, commkit/mapping/_numba_llr.py:179-210):
// the per-axis tables and the per-coordinate arithmetic, shared by the
// demapper kernels (ck_llr_kernels.cuh) and the mixed decoder's fused frame
// load (ck_ldpc_mixed.cuh).  Compiles under NVRTC.
//
// Every operation is an explicit _rn intrinsic or an exact one (rint,
// min, max, abs), so the LLRs are the same bits in every kernel and under
// every compiler: bit-identical to the IEEE evaluation of the reference's
// float32 formula.
#pragma once

#include "ck_device.cuh"

namespace ck {
namespace llr {

// -(d*d)*inv_s2 with two roundings and no contraction.
__device__ __forceinline__ float neg_sq_scaled(float d, float inv_s2) {
    return __fmul_rn(-__fmul_rn(d, d), inv_s2);
}

// One axis's tables, one record per level so that a snapped level costs a
// few vector loads: record s holds, as 32-bit words, the level's value,
// then per bit b the nearest level below (lo) and above (hi) whose bit b
// differs, as level VALUES with +inf where there is none (the reference's
// index -1), and the sign mask of bit b's LLR (0x80000000 where the level's
// bit b is 1, else 0); records padded to 16 bytes.
template <int KA>
struct MaxlogAxis {
    static constexpr int L = 1 << KA;
    static constexpr int W = (1 + 3 * KA + 3) / 4 * 4;  // words per level record
    float step, rstep;  // lev[1] - lev[0] and its rounded reciprocal
    float lev0;
    int32_t pos[KA];
    alignas(16) uint32_t rec[L * W];
    __device__ __forceinline__ float lev(int s) const { return __uint_as_float(rec[s * W]); }
};

// LLRs of one axis's KA bits (axis bit order) of the coordinate `x`: the
// reference's closed form, bit for bit.
//
// Snap: s = rint((x - lev0) / step), clamped to [0, L - 1] (round half to
// even, as np.rint), then the reference's neighbour fix (keep the nearer of
// s and its neighbour towards x).  The quotient comes from a multiply by
// the rounded reciprocal, within 3 units in the last place (2^-17 for the
// quotients below 64 that a clamp does not decide) of the IEEE quotient.
// When it lies at most 1/2 - 2^-10 from its nearest integer rq, that is the
// IEEE quotient's nearest integer too, and x is nearer level rq than its
// neighbour by 2^-9 level steps, far beyond the float rounding of the
// distances and of the levels' spacing, so the neighbour fix keeps it: the
// common case is one rint and a clamp.  Otherwise (within 2^-10 of a
// midpoint, or NaN and infinite x) the slow path runs the reference's steps
// as they stand: the IEEE division, the clamp (NaN to 0, +-inf to the ends,
// as the reference's integer conversion) and the neighbour fix.
//
// Per bit the reference takes m_other = max(-3e38, f(x - lo), f(x - hi))
// over the opposite levels that exist, with f(d) = -(d*d)*inv_s2 rounded
// twice.  f falls as |d| grows and rounding is monotone, so that maximum is
// f of the smaller |d| (equal magnitudes give equal values): one metric per
// bit instead of two.  A missing level is +inf, whose |x - inf| never wins
// against a finite distance; the cases where every candidate is infinite or
// NaN end at -3e38 on both routes, as do NaN inputs.  The LLR is m_own -
// m_other, or m_other - m_own where the level's bit is 1: IEEE subtraction
// rounds both to the same magnitude, so that is the sign flip of the first
// (by the level's sign mask), plus 0 to turn the one difference, an exact
// zero (+0 both ways round in the reference), back into +0.
template <int KA>
__device__ __forceinline__ void axis_maxlog(float x, const MaxlogAxis<KA>& t, float inv_s2,
                                            float* o) {
    constexpr int L = 1 << KA, W = MaxlogAxis<KA>::W;
    const float a = __fsub_rn(x, t.lev0);
    const float qp = __fmul_rn(a, t.rstep);
    const float rq = rintf(qp);
    int s;
    if (fabsf(__fsub_rn(qp, rq)) <= 0.5f - 0x1p-10f) {
        s = static_cast<int>(fminf(fmaxf(rq, 0.0f), static_cast<float>(L - 1)));
    } else {
        s = static_cast<int>(fminf(fmaxf(rintf(__fdiv_rn(a, t.step)), 0.0f), static_cast<float>(L - 1)));
        const float d = __fsub_rn(x, t.lev(s));
        const int s2 = d > 0.0f ? s + 1 : s - 1;
        if (s2 >= 0 && s2 < L) {
            const float d2 = __fsub_rn(x, t.lev(s2));
            if (__fmul_rn(d2, d2) < __fmul_rn(d, d)) s = s2;
        }
    }
    uint32_t r[W];
    const uint4* rv = reinterpret_cast<const uint4*>(t.rec + s * W);
#pragma unroll
    for (int q = 0; q < W / 4; ++q) {
        const uint4 v = rv[q];
        r[4 * q] = v.x;
        r[4 * q + 1] = v.y;
        r[4 * q + 2] = v.z;
        r[4 * q + 3] = v.w;
    }
    const float m_own = neg_sq_scaled(__fsub_rn(x, __uint_as_float(r[0])), inv_s2);
#pragma unroll
    for (int b = 0; b < KA; ++b) {
        const float dn = fminf(fabsf(__fsub_rn(x, __uint_as_float(r[1 + 3 * b]))),
                               fabsf(__fsub_rn(x, __uint_as_float(r[2 + 3 * b]))));
        const float m_other = fmaxf(-3.0e38f, neg_sq_scaled(dn, inv_s2));
        const float v = __fsub_rn(m_own, m_other);
        o[b] = __fadd_rn(__uint_as_float(__float_as_uint(v) ^ r[3 + 3 * b]), 0.0f);
    }
}

// Fills `t` from the device arrays of one axis (the C ABI's ck_axis_maxlog:
// levels (L,), labels (L,) MSB first, lo/hi (KA, L) level indices or -1,
// pos (KA,)), threads `first`, `first + stride`, ... sharing the work.  The
// caller synchronizes before `t` is read.
template <int KA>
__device__ __forceinline__ void load_maxlog_axis(MaxlogAxis<KA>& t, const float* levels, const int32_t* labels,
                                                 const int32_t* lo, const int32_t* hi, const int32_t* pos,
                                                 int first, int stride) {
    constexpr int L = 1 << KA, W = MaxlogAxis<KA>::W;
    for (int i = first; i < L * W; i += stride) {
        const int s = i / W, w = i - s * W;
        uint32_t v = 0u;
        if (w == 0) {
            v = __float_as_uint(levels[s]);
        } else if (w <= 3 * KA) {
            const int b = (w - 1) / 3, kind = (w - 1) - 3 * b;
            if (kind == 2) {
                v = ((labels[s] >> (KA - 1 - b)) & 1) ? 0x80000000u : 0u;
            } else {
                const int32_t j = kind == 0 ? lo[b * L + s] : hi[b * L + s];
                v = __float_as_uint(j >= 0 ? levels[j] : ck::inf_f());
            }
        }
        t.rec[i] = v;
    }
    for (int i = first; i < KA; i += stride) t.pos[i] = pos[i];
    if (first == 0) {
        t.lev0 = levels[0];
        t.step = __fsub_rn(levels[1], levels[0]);
        t.rstep = __frcp_rn(t.step);
    }
}

}  // namespace llr
}  // namespace ck
