// The mixed-code persistent decoder (min-sum, circulant codes): frames of
// several codes in one launch.  Also an NVRTC source: code-specialised
// mixed kernels (ck_ldpc_jit.cu) instantiate mixed_body with a dispatch to
// each code's generated program.
#pragma once

#include "ck_ldpc_minsum.cuh"
#include "ck_llr_axis.cuh"

namespace ck {
namespace ldpc {

// ---------------------------------------------------------------------------
// Mixed-code persistent kernel: frames of several quasi-cyclic codes in one
// launch.  Every block can host any code's frame groups (its shared memory
// and threads are sized for the largest).  Codes go longest first (edges
// per frame times the iteration budget): blocks start on the heaviest code,
// as many as it has frames for, then on the next; a block whose code's
// queue is empty switches to the heaviest code with frames left.  The
// launch then ends on short frames instead of on long frames taken last
// (measured on the mixed batch: 1.8 % faster than a start in proportion to
// each code's work).  The frame loop is the plain kernel's: same rows, same
// order, same bits.
// ---------------------------------------------------------------------------

constexpr int kMaxMixed = 12;  // CK_LDPC_MAX_MIXED
constexpr int kMixedThreads = 768;

// One frame of a continuous feed (the C ABI's ck_ldpc_feed_frame): where
// its symbols are, where its results go, and its place in the order of
// publication across queues.
struct FeedFrame {
    const float2* sym;
    float* llr_out;
    int8_t* bits;
    int32_t* iters;
    uint8_t* valid;
    float inv_s2;
    uint32_t seq;
};
constexpr uint32_t kFeedNone = 0xffffffffu;

struct MixedCode {
    const int32_t* layer;
    const int32_t* eptr;
    const int2* blk;
    int32_t N, m, L, Z, Zp, mb, nnzb;
    const float* llr_in;
    float* llr_out;
    uint32_t B;
    int32_t n_in;
    int32_t* iters;
    uint8_t* valid;
    int8_t* bits;
    int32_t k_bits;
    const int32_t* order;  // queue position -> frame, or null
    float scale, offset;
    int32_t max_iterations, early_stop;
    // r_smem: where the message state lives: 0 device memory, 1 packed
    // records in shared memory, 2 one message per edge in shared memory
    // (set only for a code that runs its specialised program here).
    int32_t T, G, q_bstep, r_smem;
    uint32_t tables_bytes, group_bytes, gblk_off, app_off, r_off, r_stride;
    // Device-memory message state: block b's groups use the words
    // [b * block_words, (b + 1) * block_words) of g_r, 3 r_stride per group.
    // A block runs one code at a time, so every code shares the region.
    uint32_t* g_r;
    uint32_t block_words;
    uint32_t* counter;
    float weight;  // edges per frame
    // Any-degree launches (row-degree bound 0): sign words per row of the
    // code's wide message state, 3 + sign_words words per row; 0 otherwise
    // (the packed record, 3 words per row in device memory).
    int32_t sign_words;
    // Fused demapping (sym != null): frame f's channel LLRs are the
    // closed-form max-log LLRs of its n_in / (2 ka) symbols at
    // sym + f * n_in / (2 ka), with 1/sigma^2 = inv_s2[f]; llr_in is unused.
    // The two axes' tables (ck_axis_maxlog arrays, [0] = in-phase) are
    // loaded into the block's table region at axes_off on a code switch.
    const float2* sym;
    const float* inv_s2;
    const float* ax_levels[2];
    const int32_t* ax_labels[2];
    const int32_t* ax_lo[2];
    const int32_t* ax_hi[2];
    const int32_t* ax_pos[2];
    int32_t ka;
    uint32_t axes_off;
    // Continuous feed (ring != null; fused demapping only): the frames come
    // from a ring of ring_mask + 1 descriptors that the host fills while the
    // kernel runs.  Positions [0, *published) are valid (the host publishes
    // with a release store), position q at ring[q & ring_mask]; counter
    // counts the positions taken, across launches.
    const FeedFrame* ring;
    const uint32_t* published;
    uint32_t ring_mask;
    // A word in the block's table region: how many of the block's groups
    // hold a frame of this code (a feed's groups keep looking for frames of
    // their queue while others of the block still work).
    uint32_t busy_off;
};

// The fused demapper's two axis tables, as laid out at MixedCode::axes_off.
template <int KA>
struct MixedAxes {
    ck::llr::MaxlogAxis<KA> ax[2];
};

// Loads code K's axis tables into the block's shared table region (all
// threads of the block; the caller synchronizes).
template <int KA>
__device__ __forceinline__ void mixed_load_axes(const MixedCode& K, unsigned char* smem) {
    MixedAxes<KA>* t = reinterpret_cast<MixedAxes<KA>*>(smem + K.axes_off);
    for (int a = 0; a < 2; ++a)
        ck::llr::load_maxlog_axis<KA>(t->ax[a], K.ax_levels[a], K.ax_labels[a], K.ax_lo[a], K.ax_hi[a],
                                      K.ax_pos[a], threadIdx.x, blockDim.x);
}

// Frame f's channel LLRs into `a` (n_in values, then the caller zeroes the
// punctured tail): symbol i's 2 KA LLRs go to a[2 KA i + pos[b]], each as
// x + 0 like the loaded LLRs of the unfused path.  The same arithmetic as
// the demapper kernels, so the same bits.
template <int KA>
__device__ __forceinline__ void mixed_demap_frame(const MixedCode& K, const unsigned char* smem, float* a,
                                                  const float2* x, float s2, int tid) {
    constexpr int KB = 2 * KA;
    constexpr int kAhead = 4;  // symbol loads in flight per thread
    const MixedAxes<KA>* t = reinterpret_cast<const MixedAxes<KA>*>(smem + K.axes_off);
    const uint32_t S = static_cast<uint32_t>(K.n_in) / KB;
    const uint32_t T = static_cast<uint32_t>(K.T);
    // The thread's symbols tid, tid + T, ... come through a ring of kAhead
    // registers: the loads of the next ones are in flight while one is
    // demapped (the symbols may sit in host memory, microseconds away).
    float2 ring[kAhead];
#pragma unroll
    for (int r = 0; r < kAhead; ++r) {
        const uint32_t i = tid + r * T;
        ring[r] = i < S ? __ldcs(x + i) : make_float2(0.0f, 0.0f);
    }
    for (uint32_t i = tid; i < S; i += T) {
        const float2 v = ring[0];
#pragma unroll
        for (int r = 0; r + 1 < kAhead; ++r) ring[r] = ring[r + 1];
        const uint32_t next = i + kAhead * T;
        ring[kAhead - 1] = next < S ? __ldcs(x + next) : make_float2(0.0f, 0.0f);
        float o[KB];
        ck::llr::axis_maxlog<KA>(v.x, t->ax[0], s2, o);
        ck::llr::axis_maxlog<KA>(v.y, t->ax[1], s2, o + KA);
        float* dst = a + KB * i;
#pragma unroll
        for (int b = 0; b < KA; ++b) {
            dst[t->ax[0].pos[b]] = __fadd_rn(o[b], 0.0f);
            dst[t->ax[1].pos[b]] = __fadd_rn(o[KA + b], 0.0f);
        }
    }
}

struct MixedParams {
    MixedCode code[kMaxMixed];
    int32_t num_codes;
    // Blocks [start_block[r], start_block[r + 1]) begin on code start_code[r].
    int32_t start_block[kMaxMixed + 1];
    int32_t start_code[kMaxMixed];
    // Continuous feed (feed != 0): a block with no published frame to take
    // polls for one, and returns once none has appeared for idle_ns (or
    // after idle_polls polls, whichever comes first) or once *stop (host
    // memory) is non-zero.
    int32_t feed;
    uint32_t idle_polls;
    uint64_t idle_ns;
    const uint32_t* stop;
    // Which queue a feed block takes next: 0 the one whose oldest untaken
    // frame was published first; 1 the same among the short codes' queues
    // (under a quarter of the longest code's edges per frame) while any has
    // a frame, else among the others.
    int32_t feed_policy;
};

// Takes the next published position of feed queue K for one frame group,
// or returns kFeedNone when every published position is taken (a bounded
// number of tries against other groups taking the same position).
__device__ __forceinline__ uint32_t feed_claim(const MixedCode& K) {
    // One read of the published count (host memory, a round trip over the
    // link); a count that has grown since only makes this group look again
    // later.  A failed compare-and-swap returns the count that won.
    const uint32_t avail = ck::ld_acquire_sys(K.published);
    uint32_t taken = *reinterpret_cast<volatile uint32_t*>(K.counter);
    for (int tries = 0; tries < 64; ++tries) {
        if (static_cast<int32_t>(avail - taken) <= 0) return kFeedNone;
        const uint32_t won = atomicCAS(K.counter, taken, taken + 1u);
        if (won == taken) return taken;
        taken = won;
    }
    return kFeedNone;
}

// The feed queue whose oldest untaken frame was published first, or -1
// when no queue has one.  Every queue's counts are read before any is
// compared, so the host-memory loads overlap (two round trips in all).
__device__ inline int feed_pick(const MixedParams& p) {
    uint32_t taken[kMaxMixed], avail[kMaxMixed], seq[kMaxMixed];
#pragma unroll
    for (int c = 0; c < kMaxMixed; ++c) {
        if (c < p.num_codes) {
            taken[c] = *reinterpret_cast<volatile uint32_t*>(p.code[c].counter);
            avail[c] = ck::ld_acquire_sys(p.code[c].published);
        }
    }
#pragma unroll
    for (int c = 0; c < kMaxMixed; ++c) {
        seq[c] = 0u;
        if (c < p.num_codes && static_cast<int32_t>(avail[c] - taken[c]) > 0)
            seq[c] = ck::ld_relaxed_sys(&p.code[c].ring[taken[c] & p.code[c].ring_mask].seq);
    }
    float heaviest = 0.0f;
    for (int c = 0; c < p.num_codes; ++c) heaviest = fmaxf(heaviest, p.code[c].weight);
    int best = -1;
    uint32_t first = 0;
    bool best_short = false;
#pragma unroll
    for (int c = 0; c < kMaxMixed; ++c) {
        if (c >= p.num_codes || static_cast<int32_t>(avail[c] - taken[c]) <= 0) continue;
        const bool is_short = p.feed_policy == 1 && 4.0f * p.code[c].weight < heaviest;
        const bool older = static_cast<int32_t>(seq[c] - first) < 0;
        if (best < 0 || (is_short && !best_short) || (is_short == best_short && older)) {
            best = c;
            first = seq[c];
            best_short = is_short;
        }
    }
    return best;
}

// feed_pick, polling while nothing is published (sleeping 1 us between
// polls at first, doubling up to 32 us, so idle blocks do not flood the
// link): -1 once the idle time or poll budget is spent, or the host has
// set *stop.
__device__ inline int feed_wait_pick(const MixedParams& p) {
    const uint64_t t0 = ck::globaltimer_ns();
    uint32_t nap = 1000;
    for (uint32_t poll = 0;; ++poll) {
        const int c = feed_pick(p);
        if (c >= 0) return c;
        if (p.stop && ck::ld_relaxed_sys(p.stop) != 0u) return -1;
        if (poll >= p.idle_polls || ck::globaltimer_ns() - t0 >= p.idle_ns) return -1;
        __nanosleep(nap);
        nap = nap < 32000 ? 2 * nap : nap;
    }
}

// The code this block should work on next: `prefer` while its queue has
// frames, else the heaviest (edges per frame times iteration budget) with
// frames left, the lowest index among equals; -1 when all are drained.
__device__ inline int mixed_pick(const MixedParams& p, int prefer) {
    if (prefer >= 0) {
        const uint32_t taken = *reinterpret_cast<volatile uint32_t*>(p.code[prefer].counter);
        if (taken < p.code[prefer].B) return prefer;
    }
    int best = -1;
    float most = 0.0f;
    for (int c = 0; c < p.num_codes; ++c) {
        const uint32_t taken = *reinterpret_cast<volatile uint32_t*>(p.code[c].counter);
        if (taken >= p.code[c].B) continue;
        const float budget = p.code[c].weight * static_cast<float>(p.code[c].max_iterations);
        if (best < 0 || budget > most) {
            best = c;
            most = budget;
        }
    }
    return best;
}

// Decodes frames of code K with group g until K's queue is empty (ONE_ROW:
// K.T >= K.Zp, one row per visited base row, as in decode_body; Prog: the
// table-driven layer loop or the code's specialised program; EDGES: one
// message per edge in shared memory, K.r_smem == 2).
template <int DMAX, bool R_SMEM, bool ONE_ROW, class Prog, bool EDGES = false>
__device__ __forceinline__ void mixed_frames(const MixedCode& K, unsigned char* smem, const int32_t* s_layer,
                             const int32_t* s_eptr, const int2* s_blk, const int g,
                             const int tid) {
    using ck::group_any;
    using ck::group_sync;
    const int bar = g + 1;
    unsigned char* gbase = smem + K.tables_bytes + static_cast<uint32_t>(g) * K.group_bytes;
    volatile uint32_t* s_frame = reinterpret_cast<volatile uint32_t*>(gbase + 8);
    float* a = reinterpret_cast<float*>(gbase + K.app_off);
    using State = typename MinSumStateOf<DMAX, R_SMEM, EDGES>::type;
    const State st(gbase + K.r_off, K.g_r + static_cast<size_t>(blockIdx.x) * K.block_words,
                   static_cast<uint32_t>(g), K.r_stride, K.sign_words);
    int2* gblk = reinterpret_cast<int2*>(gbase + K.gblk_off);
    const uint32_t a_addr = ck::smem_addr(a);
    for (int i = tid; i < K.nnzb; i += K.T)
        gblk[i] = make_int2(static_cast<int>(a_addr + 4u * static_cast<uint32_t>(s_blk[i].x)),
                            static_cast<int>(a_addr + 4u * static_cast<uint32_t>(s_blk[i].y)));
    const int32_t qr0 = K.T >= K.Zp ? tid % K.Zp : tid;
    const int32_t qb0 = K.T >= K.Zp ? tid / K.Zp : 0;
    const uint32_t r4 = 4u * static_cast<uint32_t>(qr0);
    const uint32_t Z4 = 4u * static_cast<uint32_t>(K.Z);

    auto syndrome_table = [&]() -> bool {
        const int32_t rounds = (K.mb + K.q_bstep - 1) / K.q_bstep;
        for (int32_t k = 0; k < rounds; ++k) {
            const int32_t b = k * K.q_bstep + qb0;
            for (int32_t r = qr0; r - qr0 < K.Zp; r += K.T) {
                uint32_t parity = 0;
                if (b < K.mb && r < K.Z) {
                    const int32_t e0 = s_eptr[b];
                    const int deg = s_eptr[b + 1] - e0;
                    const QcCols col_of{s_blk + e0, r, K.Z};
                    for (int e = 0; e < deg; ++e) parity ^= a[col_of(e)] < 0.0f ? 1u : 0u;
                }
                if (group_any(static_cast<int>(parity), bar, K.T)) return false;
            }
        }
        return true;
    };

    auto syndrome_ok = [&]() -> bool {
        if constexpr (Prog::kSpecialised)
            return Prog::syndrome(a_addr + r4, static_cast<uint32_t>(qr0), bar, K.T, static_cast<uint32_t>(qb0));
        return syndrome_table();
    };

    // With a feed, thread 0 copies the descriptor of the group's frame into
    // the group's control block, where the other threads read it.
    FeedFrame* s_io = reinterpret_cast<FeedFrame*>(gbase + 16);
    for (;;) {
        if (tid == 0) {
            uint32_t pos;
            if (K.ring) {
                pos = feed_claim(K);
                // While other groups of the block still decode (the block
                // changes queue only once all its groups are free), keep
                // looking for this queue's frames instead of idling; bounded
                // by their frames' decoding and by the wait limit.
                volatile int32_t* busy = reinterpret_cast<volatile int32_t*>(smem + K.busy_off);
                uint32_t nap = 1000;
                for (uint32_t poll = 0; pos == kFeedNone && *busy > 0 && poll < ck::kWaitLimit; ++poll) {
                    __nanosleep(nap);
                    nap = nap < 8000 ? 2 * nap : nap;
                    pos = feed_claim(K);
                }
                if (pos != kFeedNone) {
                    atomicAdd(const_cast<int32_t*>(busy), 1);
                    // Written by the host before it published the position
                    // (feed_claim's acquire orders these loads after it).
                    const FeedFrame* d = K.ring + (pos & K.ring_mask);
                    s_io->sym = reinterpret_cast<const float2*>(ck::ld_relaxed_sys_u64(&d->sym));
                    s_io->llr_out = reinterpret_cast<float*>(ck::ld_relaxed_sys_u64(&d->llr_out));
                    s_io->bits = reinterpret_cast<int8_t*>(ck::ld_relaxed_sys_u64(&d->bits));
                    s_io->iters = reinterpret_cast<int32_t*>(ck::ld_relaxed_sys_u64(&d->iters));
                    s_io->valid = reinterpret_cast<uint8_t*>(ck::ld_relaxed_sys_u64(&d->valid));
                    s_io->inv_s2 = __uint_as_float(ck::ld_relaxed_sys(reinterpret_cast<const uint32_t*>(&d->inv_s2)));
                }
            } else {
                pos = atomicAdd(K.counter, 1u);
            }
            *s_frame = pos;
        }
        group_sync(bar, K.T);
        const uint32_t pos = *s_frame;
        if (K.ring ? pos == kFeedNone : pos >= K.B) break;
        // This frame's symbols, noise scale and result locations.
        const float2* f_sym;
        float f_s2;
        float* f_llr;
        int8_t* f_bits;
        int32_t* f_iters;
        uint8_t* f_valid;
        uint32_t f = 0;
        if (K.ring) {
            f_sym = s_io->sym;
            f_s2 = s_io->inv_s2;
            f_llr = s_io->llr_out;
            f_bits = K.k_bits > 0 ? s_io->bits : nullptr;
            f_iters = s_io->iters;
            f_valid = s_io->valid;
        } else {
            f = K.order ? static_cast<uint32_t>(__ldg(K.order + pos)) : pos;
            f_sym = K.sym ? K.sym + static_cast<size_t>(f) * static_cast<uint32_t>(K.n_in / (2 * K.ka)) : nullptr;
            f_s2 = K.sym ? K.inv_s2[f] : 0.0f;
            f_llr = K.llr_out + static_cast<size_t>(f) * K.n_in;
            f_bits = K.bits ? K.bits + static_cast<size_t>(f) * K.k_bits : nullptr;
            f_iters = K.iters + f;
            f_valid = K.valid + f;
        }
        if (K.sym) {
            switch (K.ka) {
                case 1: mixed_demap_frame<1>(K, smem, a, f_sym, f_s2, tid); break;
                case 2: mixed_demap_frame<2>(K, smem, a, f_sym, f_s2, tid); break;
                case 3: mixed_demap_frame<3>(K, smem, a, f_sym, f_s2, tid); break;
                default: mixed_demap_frame<4>(K, smem, a, f_sym, f_s2, tid); break;
            }
        } else {
            const float* src = K.llr_in + static_cast<size_t>(f) * K.n_in;
            for (int i = tid; i < K.n_in; i += K.T) a[i] = __fadd_rn(__ldcs(src + i), 0.0f);
        }
        for (int i = K.n_in + tid; i < K.N; i += K.T) a[i] = 0.0f;
        st.zero_rows(K.m, tid, K.T);
        group_sync(bar, K.T);
        int32_t it = 0;
        bool ok = false;  // one call site of the test, as in decode_body
        for (;;) {
            if (K.early_stop || it == K.max_iterations) ok = syndrome_ok();
            if (ok || it >= K.max_iterations) break;
            // One check row: row r of base row b (circulants e0 .. e0 + deg).
            auto do_row = [&](int32_t b, int32_t e0, int deg, int32_t r) {
                const uint32_t row = static_cast<uint32_t>(b) * static_cast<uint32_t>(K.Z) +
                                     static_cast<uint32_t>(r);
                st.template qc_row_k<DMAX>(gblk + e0, deg, row, e0, r4 + 4u * static_cast<uint32_t>(r - qr0), Z4,
                                           K.scale, K.offset);
            };
            if constexpr (Prog::kSpecialised)
                Prog::iteration(st, a_addr + r4, static_cast<uint32_t>(qr0), K.scale, K.offset, bar, K.T,
                                static_cast<uint32_t>(qb0));
            for (int32_t l = 0; l < K.L && !Prog::kSpecialised; ++l) {
                const int32_t b1 = s_layer[l + 1];
                if (!ONE_ROW || qr0 < K.Z) {
                    for (int32_t b = s_layer[l] + qb0; b < b1; b += K.q_bstep) {
                        const int32_t e0 = s_eptr[b];
                        const int deg = s_eptr[b + 1] - e0;
                        if (ONE_ROW) {
                            do_row(b, e0, deg, qr0);
                        } else {
                            for (int32_t r = qr0; r - qr0 < K.Zp; r += K.T)
                                if (r < K.Z) do_row(b, e0, deg, r);
                        }
                    }
                }
                group_sync(bar, K.T);
            }
            ++it;
        }
        for (int i = tid; i < K.n_in; i += K.T) __stcs(f_llr + i, a[i]);
        if (f_bits)
            for (int i = tid; i < K.k_bits; i += K.T) f_bits[i] = a[i] < 0.0f ? 1 : 0;
        // The iteration count is written last, after a system-scope fence
        // that follows the group's writes: a host that reads it from mapped
        // memory (the request server polls frames as they finish) then also
        // sees the frame's LLRs, bits and flag.
        group_sync(bar, K.T);
        if (tid == 0) {
            *f_valid = ok ? 1 : 0;
            __threadfence_system();
            *reinterpret_cast<volatile int32_t*>(f_iters) = it;
            if (K.ring) atomicSub(reinterpret_cast<int32_t*>(smem + K.busy_off), 1);
        }
        group_sync(bar, K.T);
    }
}

// The table-driven frame loops of every code.
struct TableDispatch {
    template <int DMAX>
    __device__ __forceinline__ static void run(int, const MixedCode& K, unsigned char* smem,
                                               const int32_t* s_layer, const int32_t* s_eptr,
                                               const int2* s_blk, int g, int tid) {
        const bool one_row = K.T >= K.Zp;
        if (K.r_smem && one_row)
            mixed_frames<DMAX, true, true, TableProgram>(K, smem, s_layer, s_eptr, s_blk, g, tid);
        else if (K.r_smem)
            mixed_frames<DMAX, true, false, TableProgram>(K, smem, s_layer, s_eptr, s_blk, g, tid);
        else if (one_row)
            mixed_frames<DMAX, false, true, TableProgram>(K, smem, s_layer, s_eptr, s_blk, g, tid);
        else
            mixed_frames<DMAX, false, false, TableProgram>(K, smem, s_layer, s_eptr, s_blk, g, tid);
    }
};

// The kernel body: blocks take codes as mixed_pick says; Dispatch::run<DMAX>
// (code index, code, ...) runs a group's frames of that code (TableDispatch,
// or a generated dispatch to each code's specialised program).
template <int DMAX, class Dispatch>
__device__ __forceinline__ void mixed_body(const MixedParams& p) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int s_code;
    if (threadIdx.x == 0) {
        if (p.feed) {
            s_code = feed_wait_pick(p);
        } else {
            int r = 0;
            while (r + 1 < p.num_codes && static_cast<int32_t>(blockIdx.x) >= p.start_block[r + 1]) ++r;
            s_code = mixed_pick(p, p.start_code[r]);
        }
    }
    __syncthreads();
    for (;;) {
        const int c = s_code;
        if (c < 0) break;
        const MixedCode& K = p.code[c];
        int32_t* s_layer = reinterpret_cast<int32_t*>(smem);
        int32_t* s_eptr = s_layer + (K.L + 1);
        int2* s_blk = reinterpret_cast<int2*>(
            smem + ((static_cast<uint32_t>(K.L + 1 + K.mb + 1) * 4 + 7) & ~7u));
        for (int i = threadIdx.x; i <= K.L; i += blockDim.x) s_layer[i] = K.layer[i];
        for (int i = threadIdx.x; i <= K.mb; i += blockDim.x) s_eptr[i] = K.eptr[i];
        for (int i = threadIdx.x; i < K.nnzb; i += blockDim.x) s_blk[i] = K.blk[i];
        if (threadIdx.x == 0) *reinterpret_cast<int32_t*>(smem + K.busy_off) = 0;
        if (K.sym) {
            switch (K.ka) {
                case 1: mixed_load_axes<1>(K, smem); break;
                case 2: mixed_load_axes<2>(K, smem); break;
                case 3: mixed_load_axes<3>(K, smem); break;
                default: mixed_load_axes<4>(K, smem); break;
            }
        }
        __syncthreads();
        const int g = threadIdx.x / K.T;
        if (g < K.G) {
            const int tid = threadIdx.x - g * K.T;
            Dispatch::template run<DMAX>(c, K, smem, s_layer, s_eptr, s_blk, g, tid);
        }
        __syncthreads();
        if (threadIdx.x == 0) s_code = p.feed ? feed_wait_pick(p) : mixed_pick(p, -1);
        __syncthreads();
    }
}

template <int DMAX>
__global__ void __launch_bounds__(kMixedThreads) ldpc_mixed_kernel(const __grid_constant__ MixedParams p) {
    mixed_body<DMAX, TableDispatch>(p);
}

}  // namespace ldpc
}  // namespace ck
