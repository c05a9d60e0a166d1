// Soft LLR demapping against every point of a constellation on sm_103a:
// the kernel templates.  ck_llr_points_lo.cu / _hi.cu instantiate them for
// 1-8 and 9-16 bits per symbol.
//
// The GB300-first replacement of the reference's `llr` kernel
// (commkit/_cuda/src/llr.cu:200-223, with llrs_of :102-185) behind its
// launcher (commkit/_cuda/llr.py:37-84): the path of constellations without
// per-axis factors (PSK, 8-QAM, cross QAM, PAM, arbitrary points and
// labels, any prior).  Per symbol and point the metric is
//     m(s) = -|x - s|^2 / sigma^2 + log P(s),
// and bit b's LLR is the max of m over the points whose bit b is 0 minus
// the max over those whose bit is 1 (max-log), or the difference of the
// log-sums of exp(m) of the two halves (exact).
//
// Unlike the separable demapper this is compute bound (M metrics per
// symbol against 8 + 4k bytes of traffic), so the kernel is shaped for the
// arithmetic:
//  * Each block stages the table in shared memory sorted by label (for the
//    exact method each value twice, (re, re, im, im) and (log P, log P),
//    for its two-lane steps), after checking that the labels are a
//    permutation of 0 .. 2^k - 1 (one bit per label in a shared bitmap);
//    all lanes read the same entry, a broadcast.
//  * Max-log maxima run over chunks of 32 consecutive labels, whose low
//    five bits are then known at compile time: a register max-tree gives
//    the maxima of both halves of those five bits in 83 max operations per
//    chunk (2.6 per point instead of 5 predicated ones per point and bit),
//    and the chunk's maximum goes to the halves of the higher bits.  Max
//    is exact and order-free, so this is bit-identical to the reference's
//    per-point loop.  (Two symbols per thread with two-lane metrics ran no
//    faster here: 221 against 188 us for 128-cross-QAM.)
//  * The exact method from a staged table whose labels are the points' own
//    order (every factory-built constellation) takes each symbol's peak
//    metric, then adds exp(m - peak) to each bit's half point by point, in
//    the reference's order, with each addition's half known at compile time
//    and in the two-lane forms (exact_sorted2; commkit/mapping/
//    _numba_llr.py:35-67: a half below 1e-26 redone relative to its own
//    maximum); other tables sum in the reference's point order with
//    expf/logf, one symbol at a time.
//  * Tables of more than 4096 points, or labels that are not a permutation,
//    take the generic loop: point order, tables read through the cache.
//
// Arithmetic: float32 with explicit _rn intrinsics in the reference's
// order, -(dr*dr + di*di) * inv_s2 + log P, so max-log LLRs are
// bit-identical to the IEEE evaluation of the reference's formula; exact
// ones agree within the 1e-5 relative / 1e-6 absolute tolerance.
#pragma once

#include <math_constants.h>
#include <stdint.h>

#include "ck_llr_kernels.cuh"

namespace ck {
namespace llr {
namespace points {

constexpr int kThreads = 256;
constexpr int kMaxSmemPoints = 4096;  // tables staged in shared memory up to 12 bits
constexpr int kMaxDevices = 64;       // launch settings cached per device

struct Table {
    const float2* pts;      // (M,) complex64
    const float* logp;      // (M,) log prior
    const int32_t* labels;  // (M,) label of each point, MSB first
    int32_t M;
};

// Shared bytes of a staged table of 2^k labels.  Max-log: a float4 (re,
// im, log P, -) per label.  Exact: by label (re, re, im, im) and (log P,
// log P), each value twice so that both lanes of a two-symbol step read it
// as a pair, and the pair (-0, -0) of mul2z.  Then the labels by point and
// one bit per label for the permutation check.
__host__ __device__ constexpr uint32_t table_bytes(int k, bool exact) {
    return exact ? 24u * (1u << k) + 16u : 16u * (1u << k);
}
__host__ __device__ constexpr uint32_t smem_bytes(int k, bool exact) {
    return table_bytes(k, exact) + 4u * (1u << k) + 4u * (((1u << k) + 31u) / 32u);
}

__device__ __forceinline__ float metric(float xr, float xi, float pr, float pi, float lp, float s2) {
    const float dr = __fsub_rn(xr, pr);
    const float di = __fsub_rn(xi, pi);
    const float d2 = __fadd_rn(__fmul_rn(dr, dr), __fmul_rn(di, di));
    return __fadd_rn(__fmul_rn(-d2, s2), lp);
}

// Output bit b of a K-bit label (MSB first).
template <int K>
__device__ __forceinline__ bool label_bit(int32_t lab, int b) {
    return (lab >> (K - 1 - b)) & 1;
}

// One level of the chunk max-tree: a[0 .. 2h) holds the maxima over the
// chunk's labels whose low bits equal the index; split on bit r (h = 2^r),
// record both halves' maxima for that bit, fold it away, recurse on r - 1.
template <int K, int r>
__device__ __forceinline__ void tree_level(float* a, float* p0, float* p1) {
    if constexpr (r >= 0) {
        constexpr int h = 1 << r;
        float lo = a[0], hi = a[h];
#pragma unroll
        for (int j = 1; j < h; ++j) {
            lo = fmaxf(lo, a[j]);
            hi = fmaxf(hi, a[h + j]);
        }
        p0[K - 1 - r] = fmaxf(p0[K - 1 - r], lo);
        p1[K - 1 - r] = fmaxf(p1[K - 1 - r], hi);
#pragma unroll
        for (int j = 0; j < h; ++j) a[j] = fmaxf(a[j], a[j + h]);
        tree_level<K, r - 1>(a, p0, p1);
    }
}

// Max-log maxima of both halves of every bit from a table sorted by label
// (a float4 (re, im, log P, -) per label).
template <int K>
__device__ __forceinline__ void maxima_tree(const float4* __restrict__ tab, float xr, float xi,
                                            float s2, float* p0, float* p1) {
    constexpr int R = K < 5 ? K : 5;  // label bits resolved inside a chunk
    constexpr int C = 1 << R;
    constexpr int L = 1 << K;
#pragma unroll 1
    for (int l0 = 0; l0 < L; l0 += C) {
        float a[C];
#pragma unroll
        for (int j = 0; j < C; ++j) {
            const float4 q = tab[l0 + j];
            a[j] = metric(xr, xi, q.x, q.y, q.z, s2);
        }
        tree_level<K, R - 1>(a, p0, p1);
        // a[0] is the chunk's maximum; its labels share bits R and above.
#pragma unroll
        for (int q = R; q < K; ++q) {
            if ((l0 >> q) & 1)
                p1[K - 1 - q] = fmaxf(p1[K - 1 - q], a[0]);
            else
                p0[K - 1 - q] = fmaxf(p0[K - 1 - q], a[0]);
        }
    }
}

// The same maxima in point order from the table in device memory.
template <int K>
__device__ __forceinline__ void maxima_generic(const Table& t, float xr, float xi, float s2,
                                               float* p0, float* p1) {
#pragma unroll 4
    for (int m = 0; m < t.M; ++m) {
        const float2 p = __ldg(t.pts + m);
        const float v = metric(xr, xi, p.x, p.y, __ldg(t.logp + m), s2);
        const int32_t lab = __ldg(t.labels + m);
#pragma unroll
        for (int b = 0; b < K; ++b) {
            if (label_bit<K>(lab, b))
                p1[b] = fmaxf(p1[b], v);
            else
                p0[b] = fmaxf(p0[b], v);
        }
    }
}

// Point m of the table in device memory (point order).
struct PointOf {
    const Table* t;
    __device__ __forceinline__ void operator()(int m, float& pr, float& pi, float& lp,
                                               int32_t& lab) const {
        const float2 p = __ldg(t->pts + m);
        pr = p.x;
        pi = p.y;
        lp = __ldg(t->logp + m);
        lab = __ldg(t->labels + m);
    }
};

// Exact LLRs from the maxima (commkit/mapping/_numba_llr.py:35-81), point
// by point in the reference's order (tables that are not staged).
template <int K>
__device__ __forceinline__ void exact_llrs(const PointOf& point, int M, float xr, float xi,
                                           float s2, const float* p0, const float* p1, float* o) {
    // Every point lies in one half of bit 0: its two maxima give the peak.
    const float peak = fmaxf(p0[0], p1[0]);
    float s0[K], s1[K];
#pragma unroll
    for (int b = 0; b < K; ++b) s0[b] = s1[b] = 0.0f;
#pragma unroll 2
    for (int m = 0; m < M; ++m) {
        float pr, pi, lp;
        int32_t lab;
        point(m, pr, pi, lp, lab);
        const float e = expf(__fsub_rn(metric(xr, xi, pr, pi, lp, s2), peak));
#pragma unroll
        for (int b = 0; b < K; ++b) {
            if (label_bit<K>(lab, b))
                s1[b] = __fadd_rn(s1[b], e);
            else
                s0[b] = __fadd_rn(s0[b], e);
        }
    }
#pragma unroll
    for (int b = 0; b < K; ++b) {
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
            for (int m = 0; m < M; ++m) {
                float pr, pi, lp;
                int32_t lab;
                point(m, pr, pi, lp, lab);
                if (label_bit<K>(lab, b) != (v == 1)) continue;
                r = __fadd_rn(r, expf(__fsub_rn(metric(xr, xi, pr, pi, lp, s2), p)));
            }
            l[v] = __fadd_rn(logf(r), __fsub_rn(p, peak));
        }
        o[b] = __fsub_rn(l[0], l[1]);
    }
}

// The metrics of one point for two symbols at once, in the FMA pipe's
// two-lane forms: (x - p)^2 terms, their sum, times -1/sigma^2 (each
// lane's own) plus log P; each lane rounds as metric() does (-(d2) s2 is
// d2 (-s2); the products are mul2z, so none is contracted into the
// addition that follows), so the same bits.  X, Y: the symbols' real and
// imaginary parts as pairs; NZ the pair (-0, -0) from shared memory; q =
// (re, re, im, im) and l = (log P, log P) of the point.
__device__ __forceinline__ uint64_t metric2(uint64_t X, uint64_t Y, uint64_t NS2, uint64_t NZ, float4 q,
                                            float2 l) {
    const uint64_t dr = sub2(X, pk2(q.x, q.y));
    const uint64_t di = sub2(Y, pk2(q.z, q.w));
    return add2(mul2z(add2(mul2z(dr, dr, NZ), mul2z(di, di, NZ)), NS2, NZ), pk2(l.x, l.y));
}

// log of the sum of exp(m - peak) over the labels whose bit b (MSB first)
// is v, for a half whose sum underflowed: relative to the half's own
// largest metric p, then shifted back by p - peak (the reference's
// fallback, commkit/mapping/_numba_llr.py:48-67).  One symbol; rare.
template <int K>
__device__ __noinline__ float half_log_sum(const float4* __restrict__ ri, const float2* __restrict__ lp, int b,
                                           int v, float2 x, float s2, float peak) {
    constexpr int L = 1 << K;
    float p = -CUDART_INF_F;
    for (int l = 0; l < L; ++l) {
        if (label_bit<K>(l, b) != (v == 1)) continue;
        const float4 q = ri[l];
        p = fmaxf(p, metric(x.x, x.y, q.x, q.z, lp[l].x, s2));
    }
    float r = 0.0f;
    for (int l = 0; l < L; ++l) {
        if (label_bit<K>(l, b) != (v == 1)) continue;
        const float4 q = ri[l];
        r = __fadd_rn(r, exp_split(__fsub_rn(metric(x.x, x.y, q.x, q.z, lp[l].x, s2), p)));
    }
    return __fadd_rn(logf(r), __fsub_rn(p, peak));
}

// Exact LLRs of two symbols from a table staged by label whose labels are
// the points' own order (label m is point m, as in every constellation the
// reference's factories build), so label order is the reference's point
// order (commkit/mapping/_numba_llr.py:35-81): each symbol's peak metric
// first, then each half-sum adds e = exp(m - peak) point by point in that
// order, as the reference does.  Within a chunk (all labels up to 16, else 8
// at a time, which holds fewer registers) the labels' low bits are
// compile-time, so each addition goes straight to its half (no test of the
// label's bits); the higher bits are one branch per chunk.
// The metrics, the exponent arguments, the exponential's multiply-adds and
// the additions run in the FMA pipe's two-lane forms, each lane rounding as
// the scalar operation.  e is exp_split (a few ulp, as in the separable
// exact path), log is logf; a half-sum below 1e-26 is redone relative to
// that half's own largest metric.  The results stay within the 1e-5
// relative / 1e-6 absolute tolerance against the reference.  (With
// hundreds of points a half-sum reaches the hundreds, where one ulp of its
// log is 5e-7: another summation order, or the hardware's lg2, moves an LLR
// near 0 by more than 1e-6.)
template <int K>
__device__ __forceinline__ void exact_sorted2(const float4* __restrict__ ri, const float2* __restrict__ lp, uint64_t NZ,
                                              float2 xa, float2 xb, float sa, float sb, float* oa, float* ob) {
    constexpr int R = K <= 4 ? K : 3;  // one chunk up to 16 labels, else chunks of 8 (fewer registers)
    constexpr int C = 1 << R;
    constexpr int L = 1 << K;
    const uint64_t X = pk2(xa.x, xb.x), Y = pk2(xa.y, xb.y), NS2 = pk2(-sa, -sb);
    // The peaks: fmaxf over the metrics equals the reference's "first, then
    // any strictly greater", since the metrics are all NaN (a NaN symbol)
    // or none.
    float pa = -CUDART_INF_F, pb = -CUDART_INF_F;
#pragma unroll 1
    for (int l0 = 0; l0 < L; l0 += C) {
#pragma unroll
        for (int j = 0; j < C; ++j) {
            float ma, mb;
            upk2(metric2(X, Y, NS2, NZ, ri[l0 + j], lp[l0 + j]), ma, mb);
            pa = fmaxf(pa, ma);
            pb = fmaxf(pb, mb);
        }
    }
    const uint64_t P = pk2(pa, pb);
    uint64_t s0[K], s1[K];
#pragma unroll
    for (int b = 0; b < K; ++b) s0[b] = s1[b] = 0ull;  // the pair (+0, +0)
#pragma unroll 1
    for (int l0 = 0; l0 < L; l0 += C) {
        uint64_t e[C];
#pragma unroll
        for (int j = 0; j < C; ++j) {
            float da, db, ea, eb;
            upk2(sub2(metric2(X, Y, NS2, NZ, ri[l0 + j], lp[l0 + j]), P), da, db);
            exp_split2(da, db, ea, eb);
            e[j] = pk2(ea, eb);
        }
        // Bits below R: compile-time per label of the chunk.
#pragma unroll
        for (int j = 0; j < C; ++j) {
#pragma unroll
            for (int b = K - R; b < K; ++b) {
                if (label_bit<K>(j, b))
                    s1[b] = add2(s1[b], e[j]);
                else
                    s0[b] = add2(s0[b], e[j]);
            }
        }
        // Bits R and above: the same for the whole chunk.
#pragma unroll
        for (int b = 0; b < K - R; ++b) {
            if (label_bit<K>(l0, b)) {
#pragma unroll
                for (int j = 0; j < C; ++j) s1[b] = add2(s1[b], e[j]);
            } else {
#pragma unroll
                for (int j = 0; j < C; ++j) s0[b] = add2(s0[b], e[j]);
            }
        }
    }
#pragma unroll
    for (int b = 0; b < K; ++b) {
        float s0a, s0b, s1a, s1b;
        upk2(s0[b], s0a, s0b);
        upk2(s1[b], s1a, s1b);
        const float la0 = s0a >= kExactFloor ? logf(s0a) : half_log_sum<K>(ri, lp, b, 0, xa, sa, pa);
        const float la1 = s1a >= kExactFloor ? logf(s1a) : half_log_sum<K>(ri, lp, b, 1, xa, sa, pa);
        const float lb0 = s0b >= kExactFloor ? logf(s0b) : half_log_sum<K>(ri, lp, b, 0, xb, sb, pb);
        const float lb1 = s1b >= kExactFloor ? logf(s1b) : half_log_sum<K>(ri, lp, b, 1, xb, sb, pb);
        oa[b] = __fsub_rn(la0, la1);
        ob[b] = __fsub_rn(lb0, lb1);
    }
}

template <int K>
__device__ __forceinline__ void store_row(float* row, const float* o, bool vec) {
    if constexpr (K % 4 == 0) {
        if (vec) {
#pragma unroll
            for (int j = 0; j < K; j += 4)
                __stcs(reinterpret_cast<float4*>(row + j), make_float4(o[j], o[j + 1], o[j + 2], o[j + 3]));
            return;
        }
    } else if constexpr (K % 2 == 0) {
        if (vec) {
#pragma unroll
            for (int j = 0; j < K; j += 2) __stcs(reinterpret_cast<float2*>(row + j), make_float2(o[j], o[j + 1]));
            return;
        }
    }
#pragma unroll
    for (int j = 0; j < K; ++j) __stcs(row + j, o[j]);
}

// SMEM: the table may be staged (at most kMaxSmemPoints labels, dynamic
// shared memory of smem_bytes(K, EXACT)); then max-log runs the label-order
// max-tree one symbol per grid-stride step, and exact (labels in point
// order) two adjacent symbols per step (exact_sorted2); otherwise one
// symbol in point order.  `vec`: rows of K floats may be stored as float4 /
// float2 (out 16-byte aligned).
template <int K, bool EXACT, bool SMEM>
__global__ void __launch_bounds__(kThreads) llr_points_kernel(const float2* __restrict__ x, uint32_t n,
                                                              const Table t, const NoiseScale noise,
                                                              float* __restrict__ out, bool vec) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int L = 1 << K;
    __shared__ int s_bad, s_ident;
    const uint32_t stride = gridDim.x * blockDim.x;
    if constexpr (SMEM) {
        float4* tab = reinterpret_cast<float4*>(smem);  // max-log: (re, im, log P, -) by label
        float4* ri = reinterpret_cast<float4*>(smem);   // exact: (re, re, im, im) by label
        float2* lp = reinterpret_cast<float2*>(smem + 16u * L);  // exact: (log P, log P) by label
        float* nz = reinterpret_cast<float*>(smem + 24u * L);    // exact: (-0, -0)
        int32_t* lab_s = reinterpret_cast<int32_t*>(smem + table_bytes(K, EXACT));
        uint32_t* seen = reinterpret_cast<uint32_t*>(smem + table_bytes(K, EXACT) + 4u * L);
        if (threadIdx.x == 0) {
            s_bad = t.M != L ? 1 : 0;
            s_ident = 1;
            if (EXACT) nz[0] = nz[1] = -0.0f;
        }
        for (int i = threadIdx.x; i < (L + 31) / 32; i += blockDim.x) seen[i] = 0u;
        __syncthreads();
        if (!s_bad) {
            for (int m = threadIdx.x; m < L; m += blockDim.x) {
                const int32_t lab = t.labels[m];
                lab_s[m] = lab;
                if (lab != m) s_ident = 0;
                if (lab < 0 || lab >= L) {
                    s_bad = 1;
                    continue;
                }
                const uint32_t bit = 1u << (lab & 31);
                if (atomicOr(seen + (lab >> 5), bit) & bit) {
                    s_bad = 1;  // a label twice: not a permutation
                    continue;
                }
                const float2 p = t.pts[m];
                const float l = t.logp[m];
                if (EXACT) {
                    ri[lab] = make_float4(p.x, p.x, p.y, p.y);
                    lp[lab] = make_float2(l, l);
                } else {
                    tab[lab] = make_float4(p.x, p.y, l, 0.0f);
                }
            }
        }
        __syncthreads();
        if constexpr (EXACT) {
            // Exact only where label order is point order, the order of the
            // reference's sums: two symbols per thread and step.
            if (s_bad == 0 && s_ident) {
                const uint64_t NZ = lds_nz(ck::smem_addr(nz));
                const uint32_t pairs = n / 2 + (n & 1u);
                for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < pairs; q += stride) {
                    const uint32_t i0 = 2u * q;
                    const bool two = i0 + 1u < n;
                    const uint32_t i1 = two ? i0 + 1u : i0;  // an odd tail computes its symbol twice
                    const float2 xa = __ldcs(x + i0), xb = __ldcs(x + i1);
                    const float sa = noise.at(i0), sb = noise.at(i1);
                    float oa[K], ob[K];
                    exact_sorted2<K>(ri, lp, NZ, xa, xb, sa, sb, oa, ob);
                    store_row<K>(out + static_cast<uint64_t>(i0) * K, oa, vec);
                    if (two) store_row<K>(out + static_cast<uint64_t>(i1) * K, ob, vec);
                }
                return;
            }
        } else {
            // Max-log from any staged table (order-free), one symbol per step.
            if (s_bad == 0) {
                for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
                    const float2 xv = __ldcs(x + i);
                    const float s2 = noise.at(i);
                    float p0[K], p1[K];
#pragma unroll
                    for (int b = 0; b < K; ++b) p0[b] = p1[b] = -CUDART_INF_F;
                    maxima_tree<K>(tab, xv.x, xv.y, s2, p0, p1);
                    float o[K];
#pragma unroll
                    for (int b = 0; b < K; ++b) o[b] = __fsub_rn(p0[b], p1[b]);
                    store_row<K>(out + static_cast<uint64_t>(i) * K, o, vec);
                }
                return;
            }
        }
    }
    const PointOf point{&t};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float2 xv = __ldcs(x + i);
        const float s2 = noise.at(i);
        float p0[K], p1[K];
#pragma unroll
        for (int b = 0; b < K; ++b) p0[b] = p1[b] = -CUDART_INF_F;
        maxima_generic<K>(t, xv.x, xv.y, s2, p0, p1);
        float o[K];
        if (EXACT) {
            exact_llrs<K>(point, t.M, xv.x, xv.y, s2, p0, p1, o);
        } else {
#pragma unroll
            for (int b = 0; b < K; ++b) o[b] = __fsub_rn(p0[b], p1[b]);
        }
        store_row<K>(out + static_cast<uint64_t>(i) * K, o, vec);
    }
}

// Launch for K bits per symbol (defined in ck_llr_points_lo.cu / _hi.cu).
template <int K>
int launch_points(const float2* x, uint32_t n, const Table& t, const NoiseScale& noise, bool exact,
                  float* out, cudaStream_t stream);

}  // namespace points
}  // namespace llr
}  // namespace ck
