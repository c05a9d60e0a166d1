// Coded-link simulation on the device: the steps around the demapper and
// the decoder in the reference's Monte-Carlo error-rate loop
// (commkit/coding/performance.py:172-338) and its encoder
// (commkit/coding/ldpc.py:440-536), so a batch never leaves HBM:
//
//   random information bits -> LDPC encode -> map onto the constellation
//   + AWGN -> (demapper) -> (decoder) -> error counts
//
// and the generalized mutual information of LLRs
// (commkit/metrics/information.py:40-120).
//
// Random numbers come from Philox-4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011): counter-based,
// so element i of a stream is a pure function of (seed, stream, i), the
// same in every launch shape and on the host (tests restate it in NumPy).
// Gaussian noise is Box-Muller on two uniforms in (0, 1).
//
// Every kernel is a plain grid over its outputs with bounds checks; the
// encoder's long accumulator chains use one block-wide XOR scan per chain.
#include <stdint.h>

#include "ck_common.cuh"

namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// Philox-4x32-10
// ---------------------------------------------------------------------------

struct U4 {
    uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    const uint64_t p = static_cast<uint64_t>(a) * b;
    hi = static_cast<uint32_t>(p >> 32);
    lo = static_cast<uint32_t>(p);
}

__host__ __device__ __forceinline__ U4 philox(uint64_t counter, uint64_t stream, uint64_t seed) {
    U4 c{static_cast<uint32_t>(counter), static_cast<uint32_t>(counter >> 32),
         static_cast<uint32_t>(stream), static_cast<uint32_t>(stream >> 32)};
    uint32_t k0 = static_cast<uint32_t>(seed), k1 = static_cast<uint32_t>(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo(0xD2511F53u, c.x, hi0, lo0);
        mulhilo(0xCD9E8D57u, c.z, hi1, lo1);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Uniform in (0, 1): (x + 0.5) 2^-32 rounded to float, never 0 or 1 for
// the log of Box-Muller (x >> 8 keeps 24 bits, exactly representable).
__device__ __forceinline__ float uniform01(uint32_t x) {
    return (static_cast<float>(x >> 8) + 0.5f) * 5.9604644775390625e-08f;  // 2^-24
}

// ---------------------------------------------------------------------------
// Random bits: element i of stream `stream` is bit (i % 32) of word (i / 32)
// of the Philox output for counter i / 128 (words x, y, z, w in order).
// ---------------------------------------------------------------------------

__global__ void random_bits_kernel(int8_t* __restrict__ out, uint64_t count, uint64_t seed,
                                   uint64_t stream) {
    const uint64_t blocks = (count + 127) / 128;
    for (uint64_t b = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; b < blocks;
         b += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const U4 r = philox(b, stream, seed);
        const uint32_t w[4] = {r.x, r.y, r.z, r.w};
        const uint64_t base = b * 128;
        for (int j = 0; j < 128; ++j) {
            const uint64_t i = base + j;
            if (i >= count) break;
            out[i] = static_cast<int8_t>((w[j >> 5] >> (j & 31)) & 1u);
        }
    }
}

// ---------------------------------------------------------------------------
// Encoder: s = H_info u, then the parity part
// ---------------------------------------------------------------------------

// s[f, j] = XOR of u[f, c] over the information columns c of check j.
__global__ void syndrome_kernel(const int8_t* __restrict__ info, int64_t B, int32_t k, int32_t m,
                                const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ cols,
                                int8_t* __restrict__ s) {
    const uint64_t total = static_cast<uint64_t>(B) * m;
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t f = t / m;
        const int32_t j = static_cast<int32_t>(t - f * m);
        const int8_t* u = info + f * k;
        int v = 0;
        for (int32_t e = row_ptr[j]; e < row_ptr[j + 1]; ++e) v ^= u[cols[e]];
        s[t] = static_cast<int8_t>(v & 1);
    }
}

// Accumulator of stride g, one thread per chain (frame, residue r < g):
// p[j] = s[j] ^ p[j - g], written into the codeword at k + j.
__global__ void accumulate_seq_kernel(const int8_t* __restrict__ s, int64_t B, int32_t m, int32_t g,
                                      int32_t k, int32_t n, int8_t* __restrict__ words) {
    const uint64_t chains = static_cast<uint64_t>(B) * g;
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < chains;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t f = t / g;
        const int32_t r = static_cast<int32_t>(t - f * g);
        const int8_t* sf = s + f * m;
        int8_t* wf = words + f * n;
        int8_t p = 0;
        for (int32_t j = r; j < m; j += g) {
            p ^= sf[j];
            if (k + j < n) wf[k + j] = p;
        }
    }
}

// The same for long chains: one block of kThreads per chain; thread t
// takes a contiguous segment of the chain, then the segments' parities are
// XOR-scanned across the block.
__global__ void __launch_bounds__(kThreads) accumulate_scan_kernel(const int8_t* __restrict__ s, int64_t B,
                                                                    int32_t m, int32_t g, int32_t k,
                                                                    int32_t n, int8_t* __restrict__ words) {
    __shared__ uint32_t warp_par[kThreads / 32];
    const uint64_t chain = blockIdx.x;
    if (chain >= static_cast<uint64_t>(B) * g) return;
    const uint64_t f = chain / g;
    const int32_t r = static_cast<int32_t>(chain - f * g);
    const int32_t len = (m - r + g - 1) / g;  // elements j = r, r + g, ...
    const int32_t seg = (len + kThreads - 1) / kThreads;
    const int32_t a = threadIdx.x * seg, b = min(len, a + seg);
    const int8_t* sf = s + f * m;
    int8_t* wf = words + f * n;
    uint32_t par = 0;
    for (int32_t q = a; q < b; ++q) par ^= static_cast<uint32_t>(sf[r + q * g]);
    // Exclusive XOR scan of the segment parities over the block.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = par;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc ^= o;
    }
    if (lane == 31) warp_par[warp] = inc;
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; ++w) before ^= warp_par[w];
    uint32_t p = before ^ inc ^ par;  // parity of everything before this segment
    for (int32_t q = a; q < b; ++q) {
        const int32_t j = r + q * g;
        p ^= static_cast<uint32_t>(sf[j]);
        if (k + j < n) wf[k + j] = static_cast<int8_t>(p);
    }
}

// Packs s (B, m) into words of 32 bits, bit j % 32 of word j / 32.
__global__ void pack_kernel(const int8_t* __restrict__ s, int64_t B, int32_t m, int32_t words_per,
                            uint32_t* __restrict__ packed) {
    const uint64_t total = static_cast<uint64_t>(B) * words_per;
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t f = t / words_per;
        const int32_t w = static_cast<int32_t>(t - f * words_per);
        uint32_t v = 0;
        for (int i = 0; i < 32; ++i) {
            const int32_t j = w * 32 + i;
            if (j < m) v |= static_cast<uint32_t>(s[f * m + j] & 1) << i;
        }
        packed[t] = v;
    }
}

// p[f, i] = parity(row i of H_p^-1 AND s[f]) over GF(2), rows packed as s.
__global__ void inverse_kernel(const uint32_t* __restrict__ packed_s, const uint32_t* __restrict__ inv,
                               int64_t B, int32_t m, int32_t words_per, int32_t k, int32_t n,
                               int8_t* __restrict__ words) {
    const uint64_t total = static_cast<uint64_t>(B) * m;
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t f = t / m;
        const int32_t i = static_cast<int32_t>(t - f * m);
        const uint32_t* row = inv + static_cast<uint64_t>(i) * words_per;
        const uint32_t* sv = packed_s + f * words_per;
        uint32_t par = 0;
        for (int32_t w = 0; w < words_per; ++w) par ^= __popc(row[w] & sv[w]);
        if (k + i < n) words[f * n + k + i] = static_cast<int8_t>(par & 1u);
    }
}

__global__ void copy_info_kernel(const int8_t* __restrict__ info, int64_t B, int32_t k, int32_t n,
                                 int8_t* __restrict__ words) {
    const uint64_t total = static_cast<uint64_t>(B) * k;
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t f = t / k;
        words[f * n + (t - f * k)] = info[t];
    }
}

// Systematic generator encoding: information bit j of a frame goes to
// column cols[j], and bit i of the parity (a GF(2) product of generator row
// i with the packed information bits) to column pivots[i].  Columns at or
// beyond n (punctured) are not written.
__global__ void scatter_info_kernel(const int8_t* __restrict__ info, int64_t B, int32_t k, int32_t n,
                                    const int32_t* __restrict__ cols, int8_t* __restrict__ words) {
    const uint64_t total = static_cast<uint64_t>(B) * k;
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t f = t / k;
        const int32_t c = cols[t - f * k];
        if (c < n) words[f * n + c] = info[t];
    }
}

__global__ void generator_kernel(const uint32_t* __restrict__ packed_u, const uint32_t* __restrict__ gen,
                                 int64_t B, int32_t rank, int32_t words_per, int32_t n,
                                 const int32_t* __restrict__ pivots, int8_t* __restrict__ words) {
    const uint64_t total = static_cast<uint64_t>(B) * rank;
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t f = t / rank;
        const int32_t i = static_cast<int32_t>(t - f * rank);
        const int32_t c = pivots[i];
        if (c >= n) continue;
        const uint32_t* row = gen + static_cast<uint64_t>(i) * words_per;
        const uint32_t* u = packed_u + f * words_per;
        uint32_t par = 0;
        for (int32_t w = 0; w < words_per; ++w) par ^= __popc(row[w] & u[w]);
        words[f * n + c] = static_cast<int8_t>(par & 1u);
    }
}

// Hard decisions at chosen columns: bits[f, j] = (llrs[f, cols[j]] < 0).
__global__ void column_signs_kernel(const float* __restrict__ llrs, int64_t B, int32_t n,
                                    const int32_t* __restrict__ cols, int32_t k, int8_t* __restrict__ bits) {
    const uint64_t total = static_cast<uint64_t>(B) * k;
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const uint64_t f = t / k;
        bits[t] = static_cast<int8_t>(llrs[f * n + cols[t - f * k]] < 0.0f);
    }
}

// ---------------------------------------------------------------------------
// Map + AWGN: symbol i takes bits [i kb, (i + 1) kb) of the record (MSB
// first) as the label of a point; noise from Philox counter i of `stream`.
// ---------------------------------------------------------------------------

__global__ void map_awgn_kernel(const int8_t* __restrict__ bits, uint64_t n_sym, int32_t kb,
                                const float2* __restrict__ points_by_label, float std_re, float std_im,
                                uint64_t seed, uint64_t stream, float2* __restrict__ out) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n_sym;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint32_t label = 0;
        const int8_t* b = bits + i * kb;
        for (int j = 0; j < kb; ++j) label = (label << 1) | static_cast<uint32_t>(b[j] & 1);
        const float2 p = points_by_label[label];
        float2 v = p;
        if (std_re > 0.0f || std_im > 0.0f) {
            const U4 r = philox(i, stream, seed);
            // Box-Muller: radius from the first uniform, angle from the second.
            const float rad = sqrtf(-2.0f * logf(uniform01(r.x)));
            float sn, cs;
            sincospif(2.0f * uniform01(r.y), &sn, &cs);
            v.x = __fadd_rn(p.x, __fmul_rn(std_re, __fmul_rn(rad, cs)));
            v.y = __fadd_rn(p.y, __fmul_rn(std_im, __fmul_rn(rad, sn)));
        }
        out[i] = v;
    }
}

// ---------------------------------------------------------------------------
// Error counts of a decoded batch, accumulated into counts[7] (int64):
// blocks, info bit errors, block errors, pre-FEC bit errors (channel LLR
// sign against the sent bit), detected failures (valid false), undetected
// errors (a block in error reported valid), iterations.  One block per frame.
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long block_sum(unsigned long long v, unsigned long long* sh) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    unsigned long long total = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (blockDim.x + 31) / 32; ++w) total += sh[w];
    return total;
}

__global__ void __launch_bounds__(kThreads) count_kernel(const int8_t* __restrict__ info,
                                                          const int8_t* __restrict__ decoded,
                                                          const float* __restrict__ llr,
                                                          const int8_t* __restrict__ sent, int64_t B,
                                                          int32_t k, int32_t n, const uint8_t* __restrict__ valid,
                                                          const int32_t* __restrict__ iters,
                                                          unsigned long long* __restrict__ counts) {
    __shared__ unsigned long long sh[kThreads / 32];
    for (uint64_t f = blockIdx.x; f < static_cast<uint64_t>(B); f += gridDim.x) {
        unsigned long long bit_err = 0, pre = 0;
        for (int32_t i = threadIdx.x; i < k; i += blockDim.x)
            bit_err += (decoded[f * k + i] != info[f * k + i]) ? 1u : 0u;
        for (int32_t i = threadIdx.x; i < n; i += blockDim.x)
            pre += ((llr[f * n + i] < 0.0f) != (sent[f * n + i] != 0)) ? 1u : 0u;
        const unsigned long long be = block_sum(bit_err, sh);
        const unsigned long long pe = block_sum(pre, sh);
        if (threadIdx.x == 0) {
            const bool wrong = be > 0, ok = valid[f] != 0;
            atomicAdd(counts + 0, 1ull);
            atomicAdd(counts + 1, be);
            atomicAdd(counts + 2, wrong ? 1ull : 0ull);
            atomicAdd(counts + 3, pe);
            atomicAdd(counts + 4, ok ? 0ull : 1ull);
            atomicAdd(counts + 5, (wrong && ok) ? 1ull : 0ull);
            atomicAdd(counts + 6, static_cast<unsigned long long>(max(iters[f], 0)));
        }
    }
}

// ---------------------------------------------------------------------------
// GMI loss: log2(1 + exp(-(1 - 2c) L)) per LLR in float32 (the reference's
// precision), summed in float64 per chunk of CK_GMI_CHUNK LLRs of a row:
// partial[row * chunks + c].  The caller adds the partials in a fixed order,
// so the result does not depend on the launch.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kThreads) gmi_kernel(const float* __restrict__ llr,
                                                        const int8_t* __restrict__ bits, int64_t rows,
                                                        int64_t len, double* __restrict__ partial) {
    __shared__ double sh[kThreads / 32];
    const int64_t chunks = (len + CK_GMI_CHUNK - 1) / CK_GMI_CHUNK;
    for (int64_t t = blockIdx.x; t < rows * chunks; t += gridDim.x) {
        const int64_t row = t / chunks, c0 = (t - row * chunks) * CK_GMI_CHUNK;
        const int64_t c1 = min(len, c0 + static_cast<int64_t>(CK_GMI_CHUNK));
        double acc = 0.0;
        for (int64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
            const float L = llr[row * len + i];
            // -(1 - 2c) L: negative when the LLR favours the sent bit.
            const float x = bits[row * len + i] ? L : -L;
            const float sp = __fdiv_rn(__fadd_rn(log1pf(expf(-fabsf(x))), fmaxf(0.0f, x)), 0.6931471805599453f);
            acc += static_cast<double>(sp);
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, d);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        __syncthreads();
        if (lane == 0) sh[warp] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double total = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) total += sh[w];
            partial[t] = total;
        }
    }
}

int grid_for(uint64_t work) {
    const uint64_t want = (work + kThreads - 1) / kThreads;
    const uint64_t cap = 152ull * 16ull;
    return static_cast<int>(want < 1 ? 1 : (want < cap ? want : cap));
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" int ck_random_bits(int8_t* out, int64_t count, uint64_t seed, uint64_t stream, void* s) {
    ck::clear_error();
    if (count < 0) return ck::fail(CK_ERR_INVALID_ARGUMENT, "count must be >= 0");
    if (count == 0) return CK_OK;
    if (!out) return ck::fail(CK_ERR_INVALID_ARGUMENT, "out is NULL");
    random_bits_kernel<<<grid_for((count + 127) / 128), kThreads, 0, static_cast<cudaStream_t>(s)>>>(
        out, static_cast<uint64_t>(count), seed, stream);
    return ck::cuda_check(cudaGetLastError(), "random bits launch");
}

extern "C" int ck_ldpc_encode(const int8_t* info, int64_t B, int32_t k, int32_t m, int32_t n,
                              const int32_t* info_row_ptr, const int32_t* info_cols, int32_t stride,
                              const uint32_t* inverse, int8_t* scratch, size_t scratch_bytes,
                              int8_t* words, void* stream) {
    ck::clear_error();
    if (B < 0 || k < 1 || m < 1 || n < k || n > k + m)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "bad sizes (B=%lld k=%d m=%d n=%d)",
                        static_cast<long long>(B), k, m, n);
    if (B == 0) return CK_OK;
    if (!info || !words || !info_row_ptr || !info_cols || !scratch)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "an array is NULL");
    if ((stride < 1) == (inverse == nullptr))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "give an accumulator stride >= 1 or an inverse, not both");
    const int32_t words_per = (m + 31) / 32;
    const size_t need = static_cast<size_t>(B) * m + (inverse ? static_cast<size_t>(B) * words_per * 4 + 4 : 0);
    if (scratch_bytes < need)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "scratch of %zu bytes, %zu needed", scratch_bytes, need);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    copy_info_kernel<<<grid_for(static_cast<uint64_t>(B) * k), kThreads, 0, st>>>(info, B, k, n, words);
    syndrome_kernel<<<grid_for(static_cast<uint64_t>(B) * m), kThreads, 0, st>>>(info, B, k, m, info_row_ptr,
                                                                                  info_cols, scratch);
    if (inverse) {
        uint32_t* packed = reinterpret_cast<uint32_t*>(
            scratch + ((static_cast<size_t>(B) * m + 3) / 4) * 4);
        pack_kernel<<<grid_for(static_cast<uint64_t>(B) * words_per), kThreads, 0, st>>>(scratch, B, m,
                                                                                          words_per, packed);
        inverse_kernel<<<grid_for(static_cast<uint64_t>(B) * m), kThreads, 0, st>>>(packed, inverse, B, m,
                                                                                     words_per, k, n, words);
    } else if ((m + stride - 1) / stride <= 256) {
        accumulate_seq_kernel<<<grid_for(static_cast<uint64_t>(B) * stride), kThreads, 0, st>>>(scratch, B, m,
                                                                                                  stride, k, n,
                                                                                                  words);
    } else {
        const uint64_t chains = static_cast<uint64_t>(B) * stride;
        if (chains >= (1ull << 31)) return ck::fail(CK_ERR_UNSUPPORTED, "too many accumulator chains");
        accumulate_scan_kernel<<<static_cast<unsigned>(chains), kThreads, 0, st>>>(scratch, B, m, stride, k, n,
                                                                                   words);
    }
    return ck::cuda_check(cudaGetLastError(), "encoder launch");
}

extern "C" int ck_ldpc_encode_generator(const int8_t* info, int64_t B, int32_t k, int32_t rank, int32_t n,
                                        const int32_t* info_cols, const int32_t* pivot_cols,
                                        const uint32_t* gen, int8_t* scratch, size_t scratch_bytes,
                                        int8_t* words, void* stream) {
    ck::clear_error();
    if (B < 0 || k < 1 || rank < 1 || n < 1 || n > k + rank)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "bad sizes (B=%lld k=%d rank=%d n=%d)",
                        static_cast<long long>(B), k, rank, n);
    if (B == 0) return CK_OK;
    if (!info || !words || !info_cols || !pivot_cols || !gen || !scratch)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "an array is NULL");
    const int32_t words_per = (k + 31) / 32;
    const size_t need = static_cast<size_t>(B) * words_per * 4;
    if (scratch_bytes < need)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "scratch of %zu bytes, %zu needed", scratch_bytes, need);
    if (reinterpret_cast<uintptr_t>(scratch) % 4)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "scratch must be 4-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t* packed = reinterpret_cast<uint32_t*>(scratch);
    scatter_info_kernel<<<grid_for(static_cast<uint64_t>(B) * k), kThreads, 0, st>>>(info, B, k, n, info_cols,
                                                                                     words);
    pack_kernel<<<grid_for(static_cast<uint64_t>(B) * words_per), kThreads, 0, st>>>(info, B, k, words_per,
                                                                                     packed);
    generator_kernel<<<grid_for(static_cast<uint64_t>(B) * rank), kThreads, 0, st>>>(packed, gen, B, rank,
                                                                                     words_per, n, pivot_cols,
                                                                                     words);
    return ck::cuda_check(cudaGetLastError(), "generator encoder launch");
}

extern "C" int ck_ldpc_column_signs(const float* llrs, int64_t B, int32_t n, const int32_t* cols, int32_t k,
                                    int8_t* bits, void* stream) {
    ck::clear_error();
    if (B < 0 || n < 1 || k < 0) return ck::fail(CK_ERR_INVALID_ARGUMENT, "bad sizes");
    if (B == 0 || k == 0) return CK_OK;
    if (!llrs || !cols || !bits) return ck::fail(CK_ERR_INVALID_ARGUMENT, "an array is NULL");
    column_signs_kernel<<<grid_for(static_cast<uint64_t>(B) * k), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        llrs, B, n, cols, k, bits);
    return ck::cuda_check(cudaGetLastError(), "column signs launch");
}

extern "C" int ck_map_awgn(const int8_t* bits, int64_t n_sym, int32_t bits_per_symbol,
                           const void* points_by_label, float std_re, float std_im, uint64_t seed,
                           uint64_t stream_id, void* out, void* stream) {
    ck::clear_error();
    if (n_sym < 0 || bits_per_symbol < 1 || bits_per_symbol > 16)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "bad sizes");
    if (!(std_re >= 0.0f) || !(std_im >= 0.0f))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "noise standard deviations must be >= 0");
    if (n_sym == 0) return CK_OK;
    if (!bits || !points_by_label || !out) return ck::fail(CK_ERR_INVALID_ARGUMENT, "an array is NULL");
    map_awgn_kernel<<<grid_for(static_cast<uint64_t>(n_sym)), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        bits, static_cast<uint64_t>(n_sym), bits_per_symbol, static_cast<const float2*>(points_by_label), std_re,
        std_im, seed, stream_id, static_cast<float2*>(out));
    return ck::cuda_check(cudaGetLastError(), "map/AWGN launch");
}

extern "C" int ck_count_errors(const int8_t* info, const int8_t* decoded, const float* llr, const int8_t* sent,
                               int64_t B, int32_t k, int32_t n, const uint8_t* valid, const int32_t* iters,
                               int64_t* counts, void* stream) {
    ck::clear_error();
    if (B < 0 || k < 1 || n < 1) return ck::fail(CK_ERR_INVALID_ARGUMENT, "bad sizes");
    if (B == 0) return CK_OK;
    if (!info || !decoded || !llr || !sent || !valid || !iters || !counts)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "an array is NULL");
    const int grid = static_cast<int>(B < 152 * 8 ? B : 152 * 8);
    count_kernel<<<grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        info, decoded, llr, sent, B, k, n, valid, iters, reinterpret_cast<unsigned long long*>(counts));
    return ck::cuda_check(cudaGetLastError(), "count launch");
}

extern "C" int ck_gmi_loss(const float* llr, const int8_t* bits, int64_t rows, int64_t len, double* partial,
                           void* stream) {
    ck::clear_error();
    if (rows < 0 || len < 0) return ck::fail(CK_ERR_INVALID_ARGUMENT, "bad sizes");
    if (rows == 0 || len == 0) return CK_OK;
    if (!llr || !bits || !partial) return ck::fail(CK_ERR_INVALID_ARGUMENT, "an array is NULL");
    const int64_t work = rows * ((len + CK_GMI_CHUNK - 1) / CK_GMI_CHUNK);
    const int grid = static_cast<int>(work < 152 * 16 ? work : 152 * 16);
    gmi_kernel<<<grid, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(llr, bits, rows, len, partial);
    return ck::cuda_check(cudaGetLastError(), "GMI launch");
}
