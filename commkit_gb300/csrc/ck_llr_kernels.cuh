// Soft LLR demapping of separable (Gray square) QAM on sm_103a: the kernels.
// Each ck_llr_k<KA>.cu instantiates them for one number of bits per axis,
// so the build compiles the orders in parallel.
//
// The GB300-first replacement of the reference's `llr_separable_maxlog`
// and `llr_separable` kernels (commkit/_cuda/src/llr.cu:225-337) behind the
// launchers of commkit/_cuda/llr.py:87-206.  The work is a pure HBM
// stream: 8 bytes of complex64 in and 4k bytes of float32 out per symbol,
// a few dozen flops in between.  So the kernels are shaped for bandwidth:
//
//  * each thread loads two symbols with one 16-byte streaming load and
//    writes their 2k LLRs with 16-byte streaming stores: a warp moves
//    512 B in and 32*2k*4 B out per step, contiguous, no shared-memory
//    staging (the reference stages every tile through shared memory to
//    coalesce k-strided stores);
//  * two symbol pairs are in flight per thread per step, and the grid is
//    the SM count times the blocks resident per SM (occupancy query), so
//    the memory system sees enough requests and no block runs in a second
//    wave;
//  * the per-axis tables (levels, labels, opposite levels, bit positions)
//    live in shared memory, indexed by the data-dependent snapped level;
//  * the bits-per-axis count is a template parameter, so every per-bit
//    loop unrolls into registers.
//
// Arithmetic: float32 with explicit _rn intrinsics (and -fmad=false), so
// every operation rounds once, in the reference's order: the closed-form
// max-log and the level-metric max-log are bit-identical to the IEEE
// evaluation of the reference's formulas (commkit/mapping/_numba_llr.py:
// 179-235 and :84-92).  The exact method follows the CPU reference's
// log-sum-exp (_numba_llr.py:35-81: one exponential per level relative to
// the symbol's peak metric, the half-sums in ascending level order, a
// half below 1e-26 redone relative to its own maximum) with expf/logf;
// it agrees with the reference within float32 rounding of exp/log.
#pragma once

#include <stdint.h>

#include "ck_common.cuh"
#include "ck_llr_axis.cuh"

namespace ck {
namespace llr {

int num_sms();


constexpr int kThreads = 256;
constexpr int kOccupancyDevices = 64;  // launch shapes cached per device
constexpr float kExactFloor = 1e-26f;

__device__ __forceinline__ float4 ld_stream(const float4* p) { return __ldcs(p); }
__device__ __forceinline__ float2 ld_stream(const float2* p) { return __ldcs(p); }
__device__ __forceinline__ void st_stream(float4* p, float4 v) { __stcs(p, v); }

// The closed-form max-log pieces (MaxlogAxis, axis_maxlog) are in
// ck_llr_axis.cuh, shared with the mixed decoder's fused frame load.

template <int KA>
__device__ __forceinline__ void load_maxlog_axis(MaxlogAxis<KA>& t, const ck_axis_maxlog& a) {
    load_maxlog_axis<KA>(t, a.levels, a.labels, a.lo, a.hi, a.pos, threadIdx.x, blockDim.x);
}

// ---------------------------------------------------------------------------
// Level metrics, max-log or exact (commkit/mapping/_numba_llr.py:35-92)
// ---------------------------------------------------------------------------

template <int KA>
struct LevelAxis {
    static constexpr int L = 1 << KA;
    float lev[L];
    float logp[L];
    int32_t lab[L];
    int32_t pos[KA];
    // Per-level records of the exact method: level, log prior, then the
    // half weights, 1 in slot 2 + b where level j's bit b is 0 and in slot
    // 2 + KA + b where it is 1, else 0; padded to 16 bytes.
    static constexpr int R = (2 + 2 * KA + 3) / 4 * 4;
    alignas(16) float rec[L][R];
    uint32_t half1[KA];  // per bit: bit j set where level j's bit is 1
    // (level, log prior) pairs, and whether the labels are the binary
    // reflected Gray code of the level index (label j = j ^ (j >> 1), as
    // the axes of the reference's square QAM and of its shaped forms have):
    // then the halves of every bit are known at compile time.
    alignas(16) float2 lp[L];
    int32_t gray;
    alignas(8) float nz[2];  // (-0, -0): the addend of the two-lane products (mul2z)
};

__device__ __forceinline__ float2 lds2(uint32_t addr) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}

// A 16-byte shared-memory load that the compiler may neither hoist out of a
// loop nor merge with another (volatile), so table records are read where
// they are used instead of being held in registers across the symbol loop.
__device__ __forceinline__ float4 lds4(uint32_t addr) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr));
    return v;
}

template <int KA>
__device__ __forceinline__ float level_metric(const LevelAxis<KA>& t, int j, float x,
                                              float inv_s2) {
    return __fadd_rn(neg_sq_scaled(__fsub_rn(x, t.lev[j]), inv_s2), t.logp[j]);
}

// Level loops unroll fully up to 16 levels (256-QAM), by 4 beyond.
template <int KA>
struct Unroll {
    static constexpr int value = KA <= 4 ? (1 << KA) : 4;
};

template <int KA, bool EXACT>
__device__ __forceinline__ void axis_levels(float x, const LevelAxis<KA>& t, float inv_s2,
                                            float* o) {
    constexpr int L = 1 << KA;
    // Pass 1: the peak metric and each bit's maximum over its two halves,
    // each started at the half's first level (the reference's max order).
    float peak = 0.0f;
    float p0[KA], p1[KA];
    bool seen0[KA], seen1[KA];
#pragma unroll
    for (int b = 0; b < KA; ++b) {
        seen0[b] = seen1[b] = false;
        p0[b] = p1[b] = 0.0f;
    }
#pragma unroll Unroll<KA>::value
    for (int j = 0; j < L; ++j) {
        const float mj = level_metric(t, j, x, inv_s2);
        if (j == 0 || mj > peak) peak = mj;
        const int32_t lab = t.lab[j];
#pragma unroll
        for (int b = 0; b < KA; ++b) {
            if ((lab >> (KA - 1 - b)) & 1) {
                if (!seen1[b] || mj > p1[b]) p1[b] = mj;
                seen1[b] = true;
            } else {
                if (!seen0[b] || mj > p0[b]) p0[b] = mj;
                seen0[b] = true;
            }
        }
    }
    if (!EXACT) {
#pragma unroll
        for (int b = 0; b < KA; ++b) o[b] = __fsub_rn(p0[b], p1[b]);
        return;
    }
    // (The exact method of axes up to 16 levels runs axis_exact below.)
    // Pass 2: the half-sums of e_j = exp(m_j - peak), ascending j.
    float s0[KA], s1[KA];
#pragma unroll
    for (int b = 0; b < KA; ++b) s0[b] = s1[b] = 0.0f;
#pragma unroll Unroll<KA>::value
    for (int j = 0; j < L; ++j) {
        const float e = expf(__fsub_rn(level_metric(t, j, x, inv_s2), peak));
        const int32_t lab = t.lab[j];
#pragma unroll
        for (int b = 0; b < KA; ++b) {
            if ((lab >> (KA - 1 - b)) & 1)
                s1[b] = __fadd_rn(s1[b], e);
            else
                s0[b] = __fadd_rn(s0[b], e);
        }
    }
#pragma unroll
    for (int b = 0; b < KA; ++b) {
        float l[2];
#pragma unroll
        for (int v = 0; v < 2; ++v) {
            const float s = v ? s1[b] : s0[b];
            if (s >= kExactFloor) {
                l[v] = logf(s);
                continue;
            }
            // Underflowed half: redo relative to its own maximum (rare).
            const float p = v ? p1[b] : p0[b];
            float r = 0.0f;
            for (int j = 0; j < L; ++j) {
                if (((t.lab[j] >> (KA - 1 - b)) & 1) != v) continue;
                r = __fadd_rn(r, expf(__fsub_rn(level_metric(t, j, x, inv_s2), p)));
            }
            l[v] = __fadd_rn(logf(r), __fsub_rn(p, peak));
        }
        o[b] = __fsub_rn(l[0], l[1]);
    }
}

// e^x for x <= 0 (also -inf and NaN), accurate to a few units in the last
// place: 2^(x log2 e) with the product x log2 e carried beyond float
// precision (the argument split of Cody and Waite, "Software Manual for the
// Elementary Functions", 1980: a float head y = rn(x L2E), its exact residual
// from a fused multiply-add, plus x times the tail of log2 e), then 2^y from
// the hardware's ex2 and the factor 2^r = 1 + r ln 2 (|r| is below an ulp of
// y, so the next term is far below float precision).  The argument is first
// held at -200 or above, NaN kept (e^-200 is 0 in float), so -inf gives 0.
__device__ __forceinline__ float exp_split(float x) {
    constexpr float kL2E = 1.44269502162933349609375f;  // log2(e) rounded to float
    constexpr float kL2ELo = 1.925963033500011e-8f;      // log2(e) - kL2E
    constexpr float kLn2 = 0.693147180559945309f;
    float xc;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(xc) : "f"(x), "f"(-200.0f));
    const float y = __fmul_rn(xc, kL2E);
    const float r = __fmaf_rn(xc, kL2ELo, __fmaf_rn(xc, kL2E, -y));
    float p;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(p) : "f"(y));
    return __fmaf_rn(p, __fmul_rn(r, kLn2), p);
}

// The exact method (the reference's log-sum-exp, commkit/mapping/
// _numba_llr.py:35-81) for axes of up to 16 levels, shaped for issue rate:
// the level metrics stay in registers; the half-sums run in the reference's
// order (ascending level) as fused multiply-adds with a 0/1 weight per level
// and half, each exact (e * 1 + s rounds once as e + s does, e * 0 + s is
// s), so no per-level branch on the label; exp is exp_split and log the
// hardware's lg2 times ln 2 (__logf), within the 1e-5 relative / 1e-6
// absolute tolerance against the reference.  A half-sum below 1e-26 is
// redone relative to that half's own largest metric, as the reference does,
// over the half's levels only (a level of the other half may lie far above
// that maximum).  The peak is the largest metric: the reference's "first,
// then any strictly greater" equals fmaxf here, since the metrics are either
// all NaN (a NaN symbol) or none.
template <int KA>
__device__ __forceinline__ void axis_exact(float x, const LevelAxis<KA>& t, float inv_s2, float* o) {
    constexpr int L = 1 << KA, R = LevelAxis<KA>::R;
    const uint32_t base = ck::smem_addr(&t.rec[0][0]);
    // Level j's record, R words from its shared address.
    auto record = [&](int j, float (&r)[R]) {
#pragma unroll
        for (int q = 0; q < R / 4; ++q) {
            const float4 v = lds4(base + static_cast<uint32_t>((j * R + 4 * q) * 4));
            r[4 * q] = v.x;
            r[4 * q + 1] = v.y;
            r[4 * q + 2] = v.z;
            r[4 * q + 3] = v.w;
        }
    };
    float m[L];
    float peak = 0.0f;
#pragma unroll
    for (int j = 0; j < L; ++j) {
        float r[R];
        record(j, r);
        m[j] = __fadd_rn(neg_sq_scaled(__fsub_rn(x, r[0]), inv_s2), r[1]);
        peak = j == 0 ? m[j] : fmaxf(peak, m[j]);
    }
    float s0[KA], s1[KA];
#pragma unroll
    for (int b = 0; b < KA; ++b) s0[b] = s1[b] = 0.0f;
#pragma unroll
    for (int j = 0; j < L; ++j) {
        float r[R];
        record(j, r);
        const float e = exp_split(__fsub_rn(m[j], peak));
#pragma unroll
        for (int b = 0; b < KA; ++b) {
            s0[b] = __fmaf_rn(e, r[2 + b], s0[b]);
            s1[b] = __fmaf_rn(e, r[2 + KA + b], s1[b]);
        }
    }
#pragma unroll
    for (int b = 0; b < KA; ++b) {
        float l[2];
#pragma unroll
        for (int v = 0; v < 2; ++v) {
            const float sv = v ? s1[b] : s0[b];
            if (sv >= kExactFloor) {
                l[v] = __logf(sv);
                continue;
            }
            // Underflowed half (rare): its largest metric p, then the sum
            // relative to p over its own levels, ascending.
            const uint32_t mask = v ? t.half1[b] : ~t.half1[b];
            float p = -ck::inf_f();
#pragma unroll
            for (int j = 0; j < L; ++j)
                if ((mask >> j) & 1u) p = fmaxf(p, m[j]);
            float acc = 0.0f;
#pragma unroll
            for (int j = 0; j < L; ++j)
                if ((mask >> j) & 1u) acc = __fadd_rn(acc, exp_split(__fsub_rn(m[j], p)));
            l[v] = __fadd_rn(__logf(acc), __fsub_rn(p, peak));
        }
        o[b] = __fsub_rn(l[0], l[1]);
    }
}

// Packed pairs of floats for the FMA pipe's two-lane forms (add, sub, mul,
// fma .rn.f32x2, sm_100 and later): each lane rounds as the scalar _rn
// operation does, at half the instruction count.  One catch, measured on
// GB300: a two-lane product that feeds a two-lane addition is contracted
// into one fused multiply-add by the assembler (mul.rn.f32x2 then
// add.rn.f32x2 differed from the scalar _rn chain in 27 % of random cases,
// every operation alone matched), and an fma with a constant -0 addend is
// treated the same way.  mul2z is the product that stays rounded: an fma
// whose -0 addend comes from memory (nz, loaded from shared memory), which
// the assembler cannot fold away; use it wherever a product is added to.
__device__ __forceinline__ uint64_t pk2(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(uint64_t v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// a * b rounded once, as mul.rn would give it, for a product that is then
// added to: nz is the pair (-0, -0) loaded from memory (see above).
__device__ __forceinline__ uint64_t mul2z(uint64_t a, uint64_t b, uint64_t nz) { return fma2(a, b, nz); }
// The pair (-0, -0) at a shared address, loaded so that the compiler does
// not know its value.
__device__ __forceinline__ uint64_t lds_nz(uint32_t addr) {
    uint64_t v;
    asm volatile("ld.shared.b64 %0, [%1];" : "=l"(v) : "r"(addr));
    return v;
}

// exp_split of two arguments, its multiply-adds in the two-lane forms: the
// same operations, so the same bits.
__device__ __forceinline__ void exp_split2(float x0, float x1, float& e0, float& e1) {
    constexpr float kL2E = 1.44269502162933349609375f;
    constexpr float kL2ELo = 1.925963033500011e-8f;
    constexpr float kLn2 = 0.693147180559945309f;
    float c0, c1;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(c0) : "f"(x0), "f"(-200.0f));
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(c1) : "f"(x1), "f"(-200.0f));
    const uint64_t xc = pk2(c0, c1);
    const uint64_t y = mul2(xc, pk2(kL2E, kL2E));
    float y0, y1;
    upk2(y, y0, y1);
    const uint64_t r = fma2(xc, pk2(kL2ELo, kL2ELo), fma2(xc, pk2(kL2E, kL2E), pk2(-y0, -y1)));
    float p0, p1;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(p0) : "f"(y0));
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(p1) : "f"(y1));
    const uint64_t p = pk2(p0, p1);
    upk2(fma2(p, mul2(r, pk2(kLn2, kLn2)), p), e0, e1);
}

// Bit b (axis order, MSB first) of level j's Gray label.
template <int KA>
__host__ __device__ constexpr int gray_bit(int j, int b) {
    return ((j ^ (j >> 1)) >> (KA - 1 - b)) & 1;
}

// axis_exact for Gray-labelled axes: the same operations in the same order,
// with each bit's halves known at compile time, so the half-sums are plain
// additions over their own levels (ascending, each starting from its first
// term, as 0 + e is e), the underflow redo likewise, and no weights.
template <int KA>
__device__ __forceinline__ void axis_exact_gray(float x, const LevelAxis<KA>& t, float inv_s2, float* o) {
    constexpr int L = 1 << KA;  // even: L >= 2
    const uint32_t base = ck::smem_addr(&t.lp[0]);
    // Metrics two levels at a time: -(d*d)*s2 + logp with d = x - level,
    // rounded as the scalar steps (-(d*d) times s2 is d*d times -s2).
    float m[L];
    const uint64_t x2 = pk2(x, x), ns2 = pk2(-inv_s2, -inv_s2);
    const uint64_t nz = lds_nz(ck::smem_addr(&t.nz[0]));
#pragma unroll
    for (int j = 0; j < L; j += 2) {
        const float4 v = lds4(base + 8u * static_cast<uint32_t>(j));  // (lev j, logp j, lev j+1, logp j+1)
        const uint64_t d = sub2(x2, pk2(v.x, v.z));
        upk2(add2(mul2z(mul2(d, d), ns2, nz), pk2(v.y, v.w)), m[j], m[j + 1]);
    }
    float peak = m[0];
#pragma unroll
    for (int j = 1; j < L; ++j) peak = fmaxf(peak, m[j]);
    float e[L];
#pragma unroll
    for (int j = 0; j < L; j += 2) {
        float a, b;
        upk2(sub2(pk2(m[j], m[j + 1]), pk2(peak, peak)), a, b);
        exp_split2(a, b, e[j], e[j + 1]);
    }
#pragma unroll
    for (int b = 0; b < KA; ++b) {
        float sum[2] = {0.0f, 0.0f};
        bool seen[2] = {false, false};
#pragma unroll
        for (int j = 0; j < L; ++j) {
            const int v = gray_bit<KA>(j, b);
            sum[v] = seen[v] ? __fadd_rn(sum[v], e[j]) : e[j];
            seen[v] = true;
        }
        float l[2];
#pragma unroll
        for (int v = 0; v < 2; ++v) {
            if (sum[v] >= kExactFloor) {
                l[v] = __logf(sum[v]);
                continue;
            }
            // Underflowed half (rare): relative to its own largest metric.
            float p = 0.0f;
            bool first = true;
#pragma unroll
            for (int j = 0; j < L; ++j) {
                if (gray_bit<KA>(j, b) != v) continue;
                p = first ? m[j] : fmaxf(p, m[j]);
                first = false;
            }
            float acc = 0.0f;
            first = true;
#pragma unroll
            for (int j = 0; j < L; ++j) {
                if (gray_bit<KA>(j, b) != v) continue;
                const float ej = exp_split(__fsub_rn(m[j], p));
                acc = first ? ej : __fadd_rn(acc, ej);
                first = false;
            }
            l[v] = __fadd_rn(__logf(acc), __fsub_rn(p, peak));
        }
        o[b] = __fsub_rn(l[0], l[1]);
    }
}

template <int KA>
__device__ __forceinline__ void load_level_axis(LevelAxis<KA>& t, const ck_axis_levels& a) {
    constexpr int L = 1 << KA;
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        t.lev[i] = a.levels[i];
        t.logp[i] = a.logp[i];
        t.lab[i] = a.labels[i];
        constexpr int R = LevelAxis<KA>::R;
        t.lp[i] = make_float2(a.levels[i], a.logp[i]);
        t.rec[i][0] = a.levels[i];
        t.rec[i][1] = a.logp[i];
#pragma unroll
        for (int b = 0; b < KA; ++b) {
            const bool one = (a.labels[i] >> (KA - 1 - b)) & 1;
            t.rec[i][2 + b] = one ? 0.0f : 1.0f;
            t.rec[i][2 + KA + b] = one ? 1.0f : 0.0f;
        }
#pragma unroll
        for (int w = 2 + 2 * KA; w < R; ++w) t.rec[i][w] = 0.0f;
    }
    if (threadIdx.x == 0) {
        int32_t g = 1;
        for (int j = 0; j < L; ++j) g &= a.labels[j] == (j ^ (j >> 1)) ? 1 : 0;
        t.gray = g;
        t.nz[0] = t.nz[1] = -0.0f;
    }
    for (int i = threadIdx.x; i < KA; i += blockDim.x) {
        t.pos[i] = a.pos[i];
        uint32_t h = 0u;
        for (int j = 0; j < L && j < 32; ++j) h |= static_cast<uint32_t>((a.labels[j] >> (KA - 1 - i)) & 1) << j;
        t.half1[i] = h;
    }
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// Noise scaling of symbol i: one value per call, or one per frame.
struct NoiseScale {
    const float* frames;  // nullptr: use `value`
    float value;
    ck::FastDiv frame_len;

    __device__ __forceinline__ float at(uint32_t i) const {
        return frames ? __ldg(frames + frame_len.div(i)) : value;
    }
    // Symbols i and i + 1 (i even): one division; with frames of even
    // length both are in one frame, else the second is in the next frame
    // when i + 1 starts it.
    __device__ __forceinline__ void pair(uint32_t i, float& a, float& b) const {
        if (!frames) {
            a = b = value;
            return;
        }
        const uint32_t f = frame_len.div(i);
        a = __ldg(frames + f);
        if (frame_len.d & 1u)
            b = i + 1 == (f + 1) * frame_len.d ? __ldg(frames + f + 1) : a;
        else
            b = a;
    }
};

// Both axes' tables of one method, in shared memory.
template <int KA, int METHOD>
struct Tables;
template <int KA>
struct Tables<KA, 0> {  // closed-form max-log
    MaxlogAxis<KA> re, im;
    __device__ __forceinline__ void load(const ck_axis_maxlog& r, const ck_axis_maxlog& i) {
        load_maxlog_axis(re, r);
        load_maxlog_axis(im, i);
    }
    __device__ __forceinline__ void symbol(float2 x, float s2, float* o) const {
        axis_maxlog<KA>(x.x, re, s2, o);
        axis_maxlog<KA>(x.y, im, s2, o + KA);
    }
};
template <int KA>
struct Tables<KA, 1> {  // level metrics, max-log
    LevelAxis<KA> re, im;
    __device__ __forceinline__ void load(const ck_axis_levels& r, const ck_axis_levels& i) {
        load_level_axis(re, r);
        load_level_axis(im, i);
    }
    __device__ __forceinline__ void symbol(float2 x, float s2, float* o) const {
        axis_levels<KA, false>(x.x, re, s2, o);
        axis_levels<KA, false>(x.y, im, s2, o + KA);
    }
};
template <int KA>
struct Tables<KA, 2> : Tables<KA, 1> {  // level metrics, exact
    __device__ __forceinline__ void symbol(float2 x, float s2, float* o) const {
        if constexpr (KA <= 4) {
            if (this->re.gray & this->im.gray) {  // block-uniform
                axis_exact_gray<KA>(x.x, this->re, s2, o);
                axis_exact_gray<KA>(x.y, this->im, s2, o + KA);
            } else {
                axis_exact<KA>(x.x, this->re, s2, o);
                axis_exact<KA>(x.y, this->im, s2, o + KA);
            }
        } else {
            axis_levels<KA, true>(x.x, this->re, s2, o);
            axis_levels<KA, true>(x.y, this->im, s2, o + KA);
        }
    }
};

template <int METHOD>
struct AxisArg {
    using type = ck_axis_levels;
};
template <>
struct AxisArg<0> {
    using type = ck_axis_maxlog;
};

// Writes the K = 2 KA LLRs `o` (axis bit order) of symbol i to their
// label positions when those are not the standard ones.
template <int KA, class T>
__device__ __forceinline__ void store_scattered(const T& tab, float* out, uint32_t i,
                                                const float* o) {
    constexpr int K = 2 * KA;
    float* row = out + static_cast<uint64_t>(i) * K;
#pragma unroll
    for (int b = 0; b < KA; ++b) {
        row[tab.re.pos[b]] = o[b];
        row[tab.im.pos[b]] = o[KA + b];
    }
}

// Main kernel: two symbols per 16-byte load, two loads in flight per thread.
// PAIRS = false is the fallback for buffers that are not 16-byte aligned:
// one symbol per thread and scalar stores.  The closed form is held to 64
// registers (4 blocks of 256 per SM): measured at 2^22 symbols against 8,
// 6 and 4 blocks per SM, with and without the next pairs loaded ahead of
// the arithmetic, this was fastest (16-QAM 24.8 -> 22.0 us, 64-QAM 33.1 ->
// 28.5 us against 8 blocks; the load-ahead gained nothing).  The exact
// form is held to 4 blocks up to 64-QAM as well (64 registers, no spills:
// 64-QAM 67.9 -> 63.9 us against 3 blocks at 77 registers), to 2 for
// 256-QAM.
template <int KA, int METHOD, bool PAIRS>
__global__ void __launch_bounds__(kThreads, METHOD == 0 || (METHOD == 2 && KA <= 3) ? 4 : (METHOD == 2 && KA == 4 ? 2 : 1)) llr_kernel(const float2* __restrict__ x, uint32_t n,
                                                       const typename AxisArg<METHOD>::type re,
                                                       const typename AxisArg<METHOD>::type im,
                                                       const NoiseScale noise,
                                                       float* __restrict__ out) {
    constexpr int K = 2 * KA;
    __shared__ Tables<KA, METHOD> tab;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t npairs = n >> 1;
    const float4* x4 = reinterpret_cast<const float4*>(x);
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    // The closed form's first two symbol pairs are requested before the
    // tables are staged, so the two latencies overlap.
    float4 va = zero4, vb = zero4;
    if (PAIRS && METHOD == 0) {
        if (t0 < npairs) va = ld_stream(x4 + t0);
        if (t0 + stride < npairs) vb = ld_stream(x4 + t0 + stride);
    }
    tab.load(re, im);
    __syncthreads();
    bool standard = true;
#pragma unroll
    for (int b = 0; b < KA; ++b)
        standard = standard && tab.re.pos[b] == b && tab.im.pos[b] == KA + b;

    if (PAIRS && METHOD != 0) {
        // The level-metric methods are long (exp/log per level, the rare
        // underflow redo): one symbol at a time through a single copy of the
        // code, so the loop stays in the instruction cache and the registers
        // hold one symbol's state (unrolled over two pairs, the 64-QAM exact
        // kernel took 160 registers and stalled on instruction fetch).
        for (uint32_t p = t0; p < npairs; p += stride) {
            const float4 v = ld_stream(x4 + p);
            float sa, sb;
            noise.pair(2 * p, sa, sb);
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {
                float o[K];
                tab.symbol(h ? make_float2(v.z, v.w) : make_float2(v.x, v.y), h ? sb : sa, o);
                const uint32_t i = 2 * p + h;
                if (standard) {
                    float2* dst = reinterpret_cast<float2*>(out + static_cast<uint64_t>(i) * K);
#pragma unroll
                    for (int q = 0; q < K / 2; ++q) __stcs(dst + q, make_float2(o[2 * q], o[2 * q + 1]));
                } else {
                    store_scattered<KA>(tab, out, i, o);
                }
            }
        }
        if ((n & 1u) && t0 == 0) {
            const uint32_t i = n - 1;
            float o[K];
            tab.symbol(x[i], noise.at(i), o);
            store_scattered<KA>(tab, out, i, o);
        }
    } else if (PAIRS) {
        for (uint32_t p = t0; p < npairs; p += 2 * stride) {
            const uint32_t pb = p + stride;
            const bool two = pb < npairs;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (h == 1 && !two) break;
                const uint32_t pp = h ? pb : p;
                const float4 v = h ? vb : va;
                float o[2 * K];
                float sa, sb;
                noise.pair(2 * pp, sa, sb);
                tab.symbol(make_float2(v.x, v.y), sa, o);
                tab.symbol(make_float2(v.z, v.w), sb, o + K);
                if (standard) {
                    float4* dst = reinterpret_cast<float4*>(out + static_cast<uint64_t>(pp) * 2 * K);
#pragma unroll
                    for (int q = 0; q < K / 2; ++q)
                        st_stream(dst + q, make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2],
                                                       o[4 * q + 3]));
                } else {
                    store_scattered<KA>(tab, out, 2 * pp, o);
                    store_scattered<KA>(tab, out, 2 * pp + 1, o + K);
                }
            }
            const uint32_t q = p + 2 * stride;
            va = q < npairs ? ld_stream(x4 + q) : zero4;
            vb = q + stride < npairs ? ld_stream(x4 + q + stride) : zero4;
        }
        // Odd count: the last symbol.
        if ((n & 1u) && t0 == 0) {
            const uint32_t i = n - 1;
            float o[K];
            tab.symbol(x[i], noise.at(i), o);
            store_scattered<KA>(tab, out, i, o);
        }
    } else {
        for (uint32_t i = t0; i < n; i += stride) {
            float o[K];
            tab.symbol(ld_stream(x + i), noise.at(i), o);
            store_scattered<KA>(tab, out, i, o);
        }
    }
}

template <int KA, int METHOD, class AX>
int launch_ka(const void* x, uint32_t n, const AX& re, const AX& im, const NoiseScale& noise,
              float* out, cudaStream_t stream) {
    const bool aligned = (reinterpret_cast<uintptr_t>(x) % 16 == 0) &&
                         (reinterpret_cast<uintptr_t>(out) % 16 == 0);
    const uint32_t work = aligned ? (n / 2 + 1) : n;
    const uint32_t want = (work + kThreads - 1) / kThreads;
    using Kernel = void (*)(const float2*, uint32_t, const typename AxisArg<METHOD>::type,
                            const typename AxisArg<METHOD>::type, const NoiseScale, float*);
    const Kernel kernel = aligned ? llr_kernel<KA, METHOD, true> : llr_kernel<KA, METHOD, false>;
    // The grid-stride loop gives every block the same share, so the grid is
    // the blocks that are resident at once (registers decide: 38-40
    // registers leave 6 blocks of 256 per SM, and a grid of 8 per SM ran its
    // last quarter as a second, thin wave).  Cached per device and form.
    static int per_sm_cache[2][kOccupancyDevices] = {};
    int dev = 0;
    CK_CUDA(cudaGetDevice(&dev));
    int per_sm = dev < kOccupancyDevices ? per_sm_cache[aligned][dev] : 0;
    if (per_sm == 0) {
        CK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(kernel),
                                                              kThreads, 0));
        if (per_sm < 1) return ck::fail(CK_ERR_UNSUPPORTED, "LLR block does not fit an SM");
        if (dev < kOccupancyDevices) per_sm_cache[aligned][dev] = per_sm;
    }
    const uint32_t cap = static_cast<uint32_t>(num_sms()) * static_cast<uint32_t>(per_sm);
    const uint32_t blocks = want < cap ? (want > 0 ? want : 1) : cap;
    const float2* xs = static_cast<const float2*>(x);
    kernel<<<blocks, kThreads, 0, stream>>>(xs, n, re, im, noise, out);
    return ck::cuda_check(cudaGetLastError(), "LLR kernel launch");
}

}  // namespace llr
}  // namespace ck
