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

template <int KA>
struct MaxlogAxis {
    static constexpr int L = 1 << KA;
    float step, rstep;  // lev[1] - lev[0] and its rounded reciprocal
    float lev[L];
    int32_t lab[L];
    // For bit b and snapped level s: the nearest level below (lo) and above
    // (hi) whose bit b differs, as level VALUES, +inf where there is none
    // (the reference's index -1).
    float lo[KA * L];
    float hi[KA * L];
    int32_t pos[KA];
};

// LLRs of one axis's KA bits (axis bit order) of the coordinate `x`.
//
// Per bit the reference takes m_other = max(-3e38, f(x - lo), f(x - hi))
// over the opposite levels that exist, with f(d) = -(d*d)*inv_s2 rounded
// twice.  f falls as |d| grows and rounding is monotone, so that maximum
// is f of the smaller |d| (equal magnitudes give equal values): one metric
// per bit instead of two.  A missing level is +inf, whose |x - inf| never
// wins against a finite distance; the cases where every candidate is
// infinite or NaN end at -3e38 on both routes, as do NaN inputs.
template <int KA>
__device__ __forceinline__ void axis_maxlog(float x, const MaxlogAxis<KA>& t, float inv_s2,
                                            float* o) {
    constexpr int L = 1 << KA;
    // s = rint((x - lev0) / step), clamped to [0, L - 1] (round half to
    // even, as np.rint).  The quotient comes from a multiply by the rounded
    // reciprocal, within 3 units in the last place of the IEEE quotient
    // (two roundings of 2^-24 plus the reciprocal's), so it rounds to the
    // same integer unless it lies within that distance of a half-integer;
    // there (rarely) the IEEE division decides.  qp - rint(qp) is exact.
    // NaN and infinite x clamp as the integer conversion of the reference
    // does (NaN to 0, +-inf to the ends).
    const float a = __fsub_rn(x, t.lev[0]);
    const float qp = __fmul_rn(a, t.rstep);
    float rq = rintf(qp);
    if (fabsf(fabsf(__fsub_rn(qp, rq)) - 0.5f) <= __fmul_rn(fabsf(qp), 0x1p-20f))
        rq = rintf(__fdiv_rn(a, t.step));
    int s = static_cast<int>(fminf(fmaxf(rq, 0.0f), static_cast<float>(L - 1)));
    float d = __fsub_rn(x, t.lev[s]);
    // Near a midpoint the rounded quotient can land one level off: keep the
    // nearer of s and its neighbour towards x.
    const int s2 = d > 0.0f ? s + 1 : s - 1;
    if (s2 >= 0 && s2 < L) {
        const float d2 = __fsub_rn(x, t.lev[s2]);
        if (__fmul_rn(d2, d2) < __fmul_rn(d, d)) {
            s = s2;
            d = d2;
        }
    }
    const float m_own = neg_sq_scaled(d, inv_s2);
    const int32_t label = t.lab[s];
#pragma unroll
    for (int b = 0; b < KA; ++b) {
        const float dn = fminf(fabsf(__fsub_rn(x, t.lo[b * L + s])), fabsf(__fsub_rn(x, t.hi[b * L + s])));
        const float m_other = fmaxf(-3.0e38f, neg_sq_scaled(dn, inv_s2));
        const bool one = (label >> (KA - 1 - b)) & 1;
        o[b] = one ? __fsub_rn(m_other, m_own) : __fsub_rn(m_own, m_other);
    }
}

// Fills `t` from the device arrays of one axis (the C ABI's ck_axis_maxlog:
// levels (L,), labels (L,), lo/hi (KA, L) level indices or -1, pos (KA,)),
// threads `first`, `first + stride`, ... sharing the work.  The caller
// synchronizes before `t` is read.
template <int KA>
__device__ __forceinline__ void load_maxlog_axis(MaxlogAxis<KA>& t, const float* levels, const int32_t* labels,
                                                 const int32_t* lo, const int32_t* hi, const int32_t* pos,
                                                 int first, int stride) {
    constexpr int L = 1 << KA;
    for (int i = first; i < L; i += stride) {
        t.lev[i] = levels[i];
        t.lab[i] = labels[i];
    }
    for (int i = first; i < KA * L; i += stride) {
        const int32_t l = lo[i], h = hi[i];
        t.lo[i] = l >= 0 ? levels[l] : ck::inf_f();
        t.hi[i] = h >= 0 ? levels[h] : ck::inf_f();
    }
    for (int i = first; i < KA; i += stride) t.pos[i] = pos[i];
    if (first == 0) {
        t.step = __fsub_rn(levels[1], levels[0]);
        t.rstep = __frcp_rn(t.step);
    }
}

}  // namespace llr
}  // namespace ck
