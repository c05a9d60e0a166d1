// Device-side helpers of the commkit-gb300 kernels: fast division by a
// run-time constant and the inline-PTX wrappers (named barriers,
// mbarriers, bulk copies).  This header, and the kernel headers built on
// it, also compile under NVRTC (the code-specialised decoders are compiled
// at run time), so it includes no host header there.
#pragma once

#ifdef __CUDACC_RTC__
typedef signed char int8_t;
typedef unsigned char uint8_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
#else
#include <stdint.h>
#endif

namespace ck {

namespace ldpc {
// Largest row degree of the decoder's packed min-sum record (27 sign bits
// and a 5-bit argmin in one word).  Codes with longer rows run the
// any-degree kernels (row-degree bound 0): a generic row loop and, for
// min-sum, the wide message state.
constexpr int kPackedDegree = 27;

// The row-degree bound of the decoder kernels for a code whose longest row
// has max_deg edges: 8 (CSR codes only), 16, 27, or 0 for any degree.
__host__ __device__ constexpr int kernel_dmax(bool qc, int max_deg) {
    return max_deg > kPackedDegree ? 0 : (max_deg > 16 ? 27 : ((!qc && max_deg <= 8) ? 8 : 16));
}
}  // namespace ldpc

// q = n / d for 0 <= n < 2^31 and a run-time divisor 1 <= d < 2^31, by a
// multiply-high and a shift (the round-up method of Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994).
struct FastDiv {
    uint32_t d;
    uint32_t mul;
    uint32_t shift;

#ifndef __CUDACC_RTC__
    static FastDiv make(uint32_t d) {
        FastDiv f{d, 0u, 0u};
        uint32_t l = 0;
        while ((1ull << l) < d) ++l;
        f.shift = l;
        // mul = floor(2^32 (2^l - d) / d) + 1
        f.mul = static_cast<uint32_t>(((1ull << 32) * ((1ull << l) - d)) / d + 1ull);
        return f;
    }
#endif

    __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
        const uint32_t hi = __umulhi(n, mul);
#else
        const uint32_t hi = static_cast<uint32_t>((static_cast<uint64_t>(n) * mul) >> 32);
#endif
        // hi <= n < 2^31, so the sum does not overflow.
        return (hi + n) >> shift;
    }
};

// Frame groups of more than one warp synchronize on named barriers 1..15.
constexpr int32_t kMaxNamedGroups = 15;

// Iterations a bounded device-side wait spins before it gives up (each
// try_wait itself suspends for a while, so this is seconds).
constexpr uint32_t kWaitLimit = 1u << 24;

// Status bits a kernel leaves in its workspace header.
constexpr uint32_t kStatusTimeout = 1u;

#ifdef __CUDACC__

__device__ __forceinline__ float inf_f() { return __int_as_float(0x7f800000); }

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Barrier over the `count` threads of one frame group: a named barrier
// (ids 1..15; 0 is __syncthreads), or the warp when the group is one warp.
__device__ __forceinline__ void group_sync(int id, int count) {
    if (count == 32) {
        __syncwarp();
    } else {
        asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
    }
}

// OR of `pred` over the group, in every thread of the group.
__device__ __forceinline__ int group_any(int pred, int id, int count) {
    if (count == 32) return __any_sync(0xffffffffu, pred);
    int out;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.s32 p, %1, 0;\n\t"
        "bar.red.or.pred p, %2, %3, p;\n\t"
        "selp.s32 %0, 1, 0, p;\n\t}"
        : "=r"(out)
        : "r"(pred), "r"(id), "r"(count)
        : "memory");
    return out;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile(
        "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
            smem_addr(bar)),
        "r"(bytes)
        : "memory");
}

// Waits (bounded) for the phase with parity `phase` of `bar` to complete.
// Returns false if it gave up after kWaitLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
    const uint32_t addr = smem_addr(bar);
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Bulk copy (TMA, non-tensor) of `bytes` from global to this CTA's shared
// memory, completing on `bar`.  Both addresses 16-byte aligned; bytes a
// multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
        "[%3];" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Loads of words that another agent (the host, over NVLink-C2C, or another
// block) writes while the kernel runs: acquire at system scope (later loads
// see what the writer stored before its release), and relaxed at system
// scope (no caching of a stale value, no ordering).
__device__ __forceinline__ uint32_t ld_acquire_sys(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_relaxed_sys(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_relaxed_sys_u64(const void* p) {
    uint64_t v;
    asm volatile("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// The global nanosecond timer (for waits bounded in wall time).
// Stores of data a kernel keeps re-reading from L2 (the decoder's
// device-memory message state: written and read back once per iteration)
// with the L2 eviction priority "evict last", so that streams passing
// through L2 (frames loaded, posteriors written) are evicted before it and
// it is not written back to DRAM between iterations.  L1 is bypassed (.cg),
// as with __stcg.  Volatile and clobbering memory: kept in order with the
// barriers and with the other accesses.
__device__ __forceinline__ uint64_t l2_keep_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ void st_l2keep(uint2* p, uint2 v, uint64_t pol) {
    asm volatile("st.global.cg.L2::cache_hint.v2.u32 [%0], {%1, %2}, %3;" ::"l"(p), "r"(v.x), "r"(v.y), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void st_l2keep(uint32_t* p, uint32_t v, uint64_t pol) {
    asm volatile("st.global.cg.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

#endif  // __CUDACC__

}  // namespace ck
