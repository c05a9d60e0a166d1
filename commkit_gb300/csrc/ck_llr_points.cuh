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
//  * Each block stages the table in shared memory sorted by label (a
//    float4 (re, im, log P, -) per label) after checking that the labels
//    are a permutation of 0 .. 2^k - 1 (one bit per label in a shared
//    bitmap); all lanes read the same entry, a broadcast.
//  * Max-log maxima run over chunks of 32 consecutive labels, whose low
//    five bits are then known at compile time: a register max-tree gives
//    the maxima of both halves of those five bits in 83 max operations per
//    chunk (2.6 per point instead of 5 predicated ones per point and bit),
//    and the chunk's maximum goes to the halves of the higher bits.  Max
//    is exact and order-free, so this is bit-identical to the reference's
//    per-point loop.
//  * The exact method takes the maxima the same way, then sums
//    exp(m - peak) in the reference's point order (commkit/mapping/
//    _numba_llr.py:35-67: the peak metric of the symbol, the half-sums in
//    ascending point order, a half below 1e-26 redone relative to its own
//    maximum) with expf/logf.
//  * Tables of more than 4096 points, or labels that are not a permutation,
//    take the generic loop: point order, tables read through the cache.
//
// Arithmetic: float32 with explicit _rn intrinsics in the reference's
// order, -(dr*dr + di*di) * inv_s2 + log P, so max-log LLRs are
// bit-identical to the IEEE evaluation of the reference's formula; exact
// ones agree within the rounding of expf/logf.
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

// Shared bytes of a staged table of 2^k labels: entries by label, labels by
// point, one bit per label.
__host__ __device__ constexpr uint32_t smem_bytes(int k) {
    return 16u * (1u << k) + 4u * (1u << k) + 4u * (((1u << k) + 31u) / 32u);
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

// Max-log maxima of both halves of every bit from a table sorted by label.
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

// Point m of the table: staged (by label, with the labels by point) or not.
struct PointOf {
    const float4* tab;
    const int32_t* lab_s;
    const Table* t;
    bool staged;
    __device__ __forceinline__ void operator()(int m, float& pr, float& pi, float& lp,
                                               int32_t& lab) const {
        if (staged) {
            lab = lab_s[m];
            const float4 q = tab[lab];
            pr = q.x;
            pi = q.y;
            lp = q.z;
        } else {
            const float2 p = __ldg(t->pts + m);
            pr = p.x;
            pi = p.y;
            lp = __ldg(t->logp + m);
            lab = __ldg(t->labels + m);
        }
    }
};

// Exact LLRs from the maxima (commkit/mapping/_numba_llr.py:35-81).
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

// One thread per symbol, grid-stride.  SMEM: the table may be staged (at
// most kMaxSmemPoints labels, dynamic shared memory of smem_bytes(K)).
// `vec`: rows of K floats may be stored as float4 / float2 (out 16-byte
// aligned).
template <int K, bool EXACT, bool SMEM>
__global__ void __launch_bounds__(kThreads) llr_points_kernel(const float2* __restrict__ x, uint32_t n,
                                                              const Table t, const NoiseScale noise,
                                                              float* __restrict__ out, bool vec) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int L = 1 << K;
    __shared__ int s_bad;
    float4* tab = reinterpret_cast<float4*>(smem);
    int32_t* lab_s = reinterpret_cast<int32_t*>(smem + 16u * L);
    uint32_t* seen = reinterpret_cast<uint32_t*>(smem + 20u * L);
    bool staged = false;
    if (SMEM) {
        if (threadIdx.x == 0) s_bad = t.M != L ? 1 : 0;
        for (int i = threadIdx.x; i < (L + 31) / 32; i += blockDim.x) seen[i] = 0u;
        __syncthreads();
        if (!s_bad) {
            for (int m = threadIdx.x; m < L; m += blockDim.x) {
                const int32_t lab = t.labels[m];
                lab_s[m] = lab;
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
                tab[lab] = make_float4(p.x, p.y, t.logp[m], 0.0f);
            }
        }
        __syncthreads();
        staged = s_bad == 0;
    }
    const PointOf point{tab, lab_s, &t, staged};
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float2 xv = __ldcs(x + i);
        const float s2 = noise.at(i);
        float p0[K], p1[K];
#pragma unroll
        for (int b = 0; b < K; ++b) p0[b] = p1[b] = -CUDART_INF_F;
        if (staged)
            maxima_tree<K>(tab, xv.x, xv.y, s2, p0, p1);
        else
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
