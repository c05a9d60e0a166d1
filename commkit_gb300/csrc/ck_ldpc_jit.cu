// Code-specialised min-sum decoders for circulant codes, generated from a
// plan and compiled at run time with NVRTC.
//
// The table-driven kernel reads, for every check row, its base row's
// degree (a switch over the unrolled row bodies), its circulants' block
// columns and shifts (shared-memory loads) and its row index.  A
// specialised kernel has all of them as constants: every layer of one
// iteration is straight-line code, each row's columns are an add and a
// conditional subtract of constants, its message state an access at a
// constant offset.  The frame loop around it (queue, staging, syndrome
// test, outputs) and the row arithmetic are the same code as the table
// kernel's (decode_body and qc_row_cols, compiled from the same headers),
// so results are bit-identical; on code C (46 x 68 base, Z = 384) the
// specialised iteration ran 1.22x faster in a side-by-side timing.
//
// Applies to min-sum decodes of circulant codes launched with one frame
// group thread per row slot (threads per frame == Z rounded up to whole
// warps).  NVRTC is loaded with dlopen; where it is missing, or a
// compilation fails, decodes keep the table-driven kernel unless the plan
// requires specialisation.
#include <dlfcn.h>
#include <stdlib.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ck_ldpc_internal.h"
#include "ck_ldpc_kernel.cuh"
#include "ck_ldpc_mixed.cuh"

// The NVRTC sources of the kernel headers (written by the build).
extern const int ck_jit_header_count;
extern const char* const ck_jit_header_names[];
extern const char* const ck_jit_header_sources[];

namespace ck {
namespace ldpc {
namespace {

struct Nvrtc {
    using Create = int (*)(void**, const char*, const char*, int, const char* const*, const char* const*);
    using Compile = int (*)(void*, int, const char* const*);
    using Size = int (*)(void*, size_t*);
    using Get = int (*)(void*, char*);
    using Destroy = int (*)(void**);
    Create create = nullptr;
    Compile compile = nullptr;
    Size log_size = nullptr, cubin_size = nullptr;
    Get log = nullptr, cubin = nullptr;
    Destroy destroy = nullptr;
    std::string why;  // why it is unavailable
};

const Nvrtc& nvrtc() {
    static const Nvrtc n = [] {
        Nvrtc r;
        void* h = nullptr;
        std::string tried;
        std::string paths[] = {"libnvrtc.so.13", "libnvrtc.so", "", "/usr/local/cuda/lib64/libnvrtc.so.13"};
        if (const char* home = getenv("CUDA_HOME")) paths[2] = std::string(home) + "/lib64/libnvrtc.so.13";
        if (const char* only = getenv("COMMKIT_GB300_NVRTC")) {  // an explicit library, and nothing else
            paths[0] = only;
            paths[1] = paths[2] = paths[3] = "";
        }
        for (const std::string& p : paths) {
            if (p.empty()) continue;
            h = dlopen(p.c_str(), RTLD_NOW | RTLD_LOCAL);
            if (h) break;
            tried += (tried.empty() ? "" : ", ") + p;
        }
        if (!h) {
            r.why = "NVRTC not found (tried " + tried + ")";
            return r;
        }
        r.create = reinterpret_cast<Nvrtc::Create>(dlsym(h, "nvrtcCreateProgram"));
        r.compile = reinterpret_cast<Nvrtc::Compile>(dlsym(h, "nvrtcCompileProgram"));
        r.log_size = reinterpret_cast<Nvrtc::Size>(dlsym(h, "nvrtcGetProgramLogSize"));
        r.log = reinterpret_cast<Nvrtc::Get>(dlsym(h, "nvrtcGetProgramLog"));
        r.cubin_size = reinterpret_cast<Nvrtc::Size>(dlsym(h, "nvrtcGetCUBINSize"));
        r.cubin = reinterpret_cast<Nvrtc::Get>(dlsym(h, "nvrtcGetCUBIN"));
        r.destroy = reinterpret_cast<Nvrtc::Destroy>(dlsym(h, "nvrtcDestroyProgram"));
        if (!r.create || !r.compile || !r.log_size || !r.log || !r.cubin_size || !r.cubin || !r.destroy) {
            r.why = "NVRTC lacks an entry point";
            r.create = nullptr;
        }
        return r;
    }();
    return n;
}

void add(std::string& s, const char* fmt, long long a = 0, long long b = 0, long long c = 0) {
    char buf[256];
    snprintf(buf, sizeof(buf), fmt, a, b, c);
    s += buf;
}

// The base rows of layer l that part h of H runs (H threads per row slot,
// part = thread / Zp): balanced by edges, the heaviest row to the lighter
// part first, then in base-row order.  The rows of a layer share no
// variable, so any split gives the same bits.
std::vector<int32_t> layer_part(const ck_ldpc_plan& plan, int32_t l, int H, int h) {
    std::vector<int32_t> rows;
    for (int32_t b = plan.h_layer[l]; b < plan.h_layer[l + 1]; ++b) rows.push_back(b);
    if (H == 1) return rows;
    std::vector<int32_t> order = rows;
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        return plan.h_eptr[x + 1] - plan.h_eptr[x] > plan.h_eptr[y + 1] - plan.h_eptr[y];
    });
    std::vector<long long> load(H, 0);
    std::vector<int32_t> mine;
    for (int32_t b : order) {
        int best = 0;
        for (int q = 1; q < H; ++q)
            if (load[q] < load[best]) best = q;
        load[best] += plan.h_eptr[b + 1] - plan.h_eptr[b];
        if (best == h) mine.push_back(b);
    }
    std::sort(mine.begin(), mine.end());
    return mine;
}

// The program of one circulant code, as struct `name`: every layer's base
// rows, each as its columns (row qr0 of circulant (j, shift) is column j Z +
// (qr0 + shift) mod Z) and its state row b Z + qr0, then the group barrier.
// With H parts (threads per frame = H Zp), part h runs its share of each
// layer's base rows (layer_part), warp-uniformly, so a frame's layer takes
// H times fewer rows per thread.
std::string program_struct(const ck_ldpc_plan& plan, const char* name, int H = 1) {
    const int32_t Z = plan.Z, Zp = (Z + 31) / 32 * 32;
    // ceil(2^32 / Z): the high word of (qr0 + shift) * magic is the wrap bit.
    const unsigned long long magic = ((1ull << 32) + static_cast<unsigned long long>(Z) - 1) / static_cast<unsigned long long>(Z);
    std::string s;
    s += "struct ";
    s += name;
    s += " {\n";
    s += "    static constexpr bool kSpecialised = true;\n";
    add(s, "    static constexpr int kParts = %lld;\n", H);
    s += "    template <class St>\n";
    s += "    __device__ __forceinline__ static void iteration(const St& st, const uint32_t base4_in, const uint32_t qr0_in,\n";
    s += "                                                     const float scale, const float offset, const int bar,\n";
    s += "                                                     const int T, const uint32_t part_in) {\n";
    // Opaque copies of the thread's offsets, taken anew each iteration: the
    // columns and state addresses derived from them are then computed where
    // they are used instead of being hoisted out of the iteration loop and
    // held (or spilled) across it.
    s += "        uint32_t base4, qr0, part;\n";
    s += "        asm volatile(\"mov.b32 %0, %1;\" : \"=r\"(base4) : \"r\"(base4_in));\n";
    s += "        asm volatile(\"mov.b32 %0, %1;\" : \"=r\"(qr0) : \"r\"(qr0_in));\n";
    s += "        asm volatile(\"mov.b32 %0, %1;\" : \"=r\"(part) : \"r\"(part_in));\n";
    // Each row's message state in device memory is loaded one row ahead
    // (the thread's own rows: no other thread writes them, so the load may
    // cross a barrier), which hides its L2 latency behind the previous row's
    // arithmetic.  The padding lanes of a Z that is not a multiple of 32 load
    // from row 0 of their base row and never use it.
    const bool pad = Zp != Z;
    auto row_of = [&](int32_t b) {
        std::string r = std::to_string(static_cast<long long>(b) * Z) + "u + ";
        return r + (pad ? "(qr0 < " + std::to_string(Z) + "u ? qr0 : 0u)" : std::string("qr0"));
    };
    // Each part's chain of rows, layer by layer.
    std::vector<std::vector<std::vector<int32_t>>> parts(H);
    std::vector<std::vector<int32_t>> chain(H);
    for (int h = 0; h < H; ++h)
        for (int32_t l = 0; l < plan.L; ++l) {
            parts[h].push_back(layer_part(plan, l, H, h));
            chain[h].insert(chain[h].end(), parts[h].back().begin(), parts[h].back().end());
        }
    if (H == 1) {
        if (!chain[0].empty()) s += "        uint4 next = st.pre(" + row_of(chain[0][0]) + ");\n";
    } else {
        s += "        uint4 next = make_uint4(0u, 0u, 0u, 0u);\n";
        for (int h = 0; h < H; ++h)
            if (!chain[h].empty()) {
                add(s, "        if (part == %lldu) next = st.pre(", h);
                s += row_of(chain[h][0]) + ");\n";
            }
    }
    std::vector<size_t> pos(H, 0);  // position in each part's chain
    auto emit_row = [&](int h, int32_t b, const char* ind) {
        const int32_t e0 = plan.h_eptr[b], deg = plan.h_eptr[b + 1] - e0;
        const size_t at = pos[h]++;
        s += ind;
        s += "{\n";
        s += ind;
        s += "    const uint4 cur = st.take(next, " + row_of(b) + ");\n";
        if (at + 1 < chain[h].size()) {
            s += ind;
            s += "    next = st.pre(" + row_of(chain[h][at + 1]) + ");\n";
        }
        if (pad) {
            s += ind;
            add(s, "    if (qr0 < %lldu) {\n", Z);
        }
        s += ind;
        add(s, "    uint32_t c[%lld];\n", deg);
        for (int32_t e = 0; e < deg; ++e) {
            const int32_t first = plan.h_blk[2 * (e0 + e)];    // j Z + shift
            const int32_t end = plan.h_blk[2 * (e0 + e) + 1];  // (j + 1) Z
            const long long shift = Z - (end - first);
            s += ind;
            if (shift == 0) {
                add(s, "    c[%lld] = base4 + %lldu;\n", e, 4ll * first);
            } else {
                add(s, "    c[%lld] = wrapped_base(base4, qr0, %lluu, %lluull, ", e,
                    static_cast<long long>(magic), static_cast<long long>(magic * static_cast<unsigned long long>(shift)));
                add(s, "%lluu) + %lldu;\n", static_cast<long long>((0x100000000ull - 4ull * Z) & 0xffffffffull),
                    4ll * first);
            }
        }
        // The row's state: its record at b Z + qr0, or (per-edge state) the
        // messages of its circulants e0.. at byte 4 (e0 Z + qr0) + 4 Z e.
        s += ind;
        add(s, "    st.template row_cols<%lld, %lldu>(c, cur, ", deg, 4ll * Z);
        add(s, "%lldu + qr0, %lldu + 4u * qr0, scale, offset);\n", static_cast<long long>(b) * Z,
            4ll * e0 * Z);
        if (pad) {
            s += ind;
            s += "    }\n";
        }
        s += ind;
        s += "}\n";
    };
    for (int32_t l = 0; l < plan.L; ++l) {
        add(s, "        // layer %lld\n", l);
        if (H == 1) {
            for (int32_t b : parts[0][l]) emit_row(0, b, "        ");
        } else {
            for (int h = 0; h < H; ++h) {
                add(s, h == 0 ? "        if (part == %lldu) {\n" : "        } else if (part == %lldu) {\n", h);
                for (int32_t b : parts[h][l]) emit_row(h, b, "            ");
            }
            s += "        }\n";
        }
        s += "        ck::group_sync(bar, T);\n";
    }
    s += "    }\n";
    // The syndrome test over the same rows: per base row the parity of the
    // sign bits (the posterior holds no -0 and only positive NaNs, so the
    // sign bit is "< 0"), ORed over a round of base rows, one group OR per
    // round, stopping at the first unsatisfied round.  The first round is
    // one base row (an unconverged frame usually fails there), the others
    // eight (a converged frame pays for few group ORs).  With H parts, part
    // h takes every H-th row of a round.
    s += "    __device__ __forceinline__ static bool syndrome(const uint32_t base4_in, const uint32_t qr0_in,\n";
    s += "                                                    const int bar, const int T, const uint32_t part_in) {\n";
    s += "        uint32_t base4, qr0, part;\n";
    s += "        asm volatile(\"mov.b32 %0, %1;\" : \"=r\"(base4) : \"r\"(base4_in));\n";
    s += "        asm volatile(\"mov.b32 %0, %1;\" : \"=r\"(qr0) : \"r\"(qr0_in));\n";
    s += "        asm volatile(\"mov.b32 %0, %1;\" : \"=r\"(part) : \"r\"(part_in));\n";
    s += "        uint32_t bad = 0u;\n";
    auto emit_parity = [&](int32_t b, const char* ind) {
        const int32_t e0 = plan.h_eptr[b], deg = plan.h_eptr[b + 1] - e0;
        s += ind;
        s += "{\n";
        s += ind;
        s += "    uint32_t x = 0u;\n";
        if (pad) {
            s += ind;
            add(s, "    if (qr0 < %lldu) {\n", Z);
        }
        for (int32_t e = 0; e < deg; ++e) {
            const int32_t first = plan.h_blk[2 * (e0 + e)];
            const int32_t end = plan.h_blk[2 * (e0 + e) + 1];
            const long long shift = Z - (end - first);
            s += ind;
            if (shift == 0) {
                add(s, "    x ^= __float_as_uint(ld_shared_f32(base4 + %lldu));\n", 4ll * first);
            } else {
                add(s, "    x ^= __float_as_uint(ld_shared_f32(wrapped_base(base4, qr0, %lluu, %lluull, ",
                    static_cast<long long>(magic), static_cast<long long>(magic * static_cast<unsigned long long>(shift)));
                add(s, "%lluu) + %lldu));\n", static_cast<long long>((0x100000000ull - 4ull * Z) & 0xffffffffull),
                    4ll * first);
            }
        }
        if (pad) {
            s += ind;
            s += "    }\n";
        }
        s += ind;
        s += "    bad |= x >> 31;\n";
        s += ind;
        s += "}\n";
    };
    int32_t round_start = 0;
    for (int32_t b = 0; b < plan.mb; ++b) {
        if (b == 0 || b % 8 == 0 || b + 1 == plan.mb) {
            // rows round_start .. b form a round
            if (H == 1) {
                for (int32_t r = round_start; r <= b; ++r) emit_parity(r, "        ");
            } else {
                for (int h = 0; h < H; ++h) {
                    add(s, h == 0 ? "        if (part == %lldu) {\n" : "        } else if (part == %lldu) {\n", h);
                    for (int32_t r = round_start + h; r <= b; r += H) emit_parity(r, "            ");
                }
                s += "        }\n";
            }
            s += "        if (ck::group_any(static_cast<int>(bad), bar, T)) return false;\n";
            if (b + 1 < plan.mb) s += "        bad = 0u;\n";
            round_start = b + 1;
        }
    }
    s += "        return true;\n    }\n};\n";
    return s;
}

// The plain decoder of one code: one kernel per message-state placement
// (r0 records in device memory, r1 records in shared memory, r2 one
// message per edge in shared memory).
std::string program_source(const ck_ldpc_plan& plan, int dmax) {
    std::string s = "#include \"ck_ldpc_minsum.cuh\"\nusing namespace ck::ldpc;\nnamespace {\n";
    s += program_struct(plan, "CodeProgram");
    s += "}  // namespace\n";
    for (int r = 0; r < 3; ++r) {
        // A minimum of one block per SM, stated: without it ptxas held some of
        // these kernels to 40 registers and spilled.
        add(s, "extern \"C\" __global__ void __launch_bounds__(%lld, 1) ck_ldpc_code_r%lld(const __grid_constant__ Params p) {\n",
            max_block_threads(true, dmax), r);
        s += r == 2 ? "    decode_body<EdgeMinSumState" : "    decode_body<MinSumState";
        add(s, ", true, %lld, true, ", dmax);
        s += r ? "true" : "false";
        s += ", true, CodeProgram>(p);\n}\n";
    }
    return s;
}

// The mixed decoder of n batches; batch c runs its code's program with
// parts[c] threads per row slot when parts[c] > 0, else the table loop;
// edges[c]: its program keeps one message per edge in shared memory
// (MixedCode::r_smem == 2).
std::string mixed_program_source(const ck_ldpc_plan* const* plans, const int* parts, const int* edges, int n,
                                 int dmax) {
    std::string s = "#include \"ck_ldpc_mixed.cuh\"\nusing namespace ck::ldpc;\nnamespace {\n";
    // A code may fill several batches (one per constellation): one program
    // and one call site per distinct (plan, parts), its batches as cases of
    // the same branch.
    std::vector<int> first(n);
    std::vector<bool> special(n);
    for (int c = 0; c < n; ++c) {
        special[c] = parts[c] > 0;
        first[c] = c;
        for (int u = 0; u < c; ++u)
            if (plans[u] == plans[c] && parts[u] == parts[c] && edges[u] == edges[c]) {
                first[c] = u;
                break;
            }
        if (first[c] == c && special[c])
            s += program_struct(*plans[c], ("CodeProgram" + std::to_string(c)).c_str(), parts[c]);
    }
    s += "struct CodeDispatch {\n";
    s += "    template <int DMAX>\n";
    s += "    __device__ __forceinline__ static void run(int c, const MixedCode& K, unsigned char* smem,\n";
    s += "                                               const int32_t* s_layer, const int32_t* s_eptr,\n";
    s += "                                               const int2* s_blk, int g, int tid) {\n";
    s += "        switch (c) {\n";
    for (int c = 0; c < n; ++c) {
        if (first[c] != c) continue;
        for (int d = c; d < n; ++d)
            if (first[d] == c) add(s, "            case %lld:\n", d);
        if (special[c] && edges[c]) {
            const std::string prog = "CodeProgram" + std::to_string(c);
            s += "                mixed_frames<DMAX, true, true, " + prog + ", true>(K, smem, s_layer, s_eptr, s_blk, g, tid);\n";
        } else if (special[c]) {
            const std::string prog = "CodeProgram" + std::to_string(c);
            s += "                if (K.r_smem)\n";
            s += "                    mixed_frames<DMAX, true, true, " + prog + ">(K, smem, s_layer, s_eptr, s_blk, g, tid);\n";
            s += "                else\n";
            s += "                    mixed_frames<DMAX, false, true, " + prog + ">(K, smem, s_layer, s_eptr, s_blk, g, tid);\n";
        } else {
            s += "                TableDispatch::run<DMAX>(c, K, smem, s_layer, s_eptr, s_blk, g, tid);\n";
        }
        s += "                break;\n";
    }
    s += "            default:\n                break;\n        }\n    }\n};\n}  // namespace\n";
    add(s, "extern \"C\" __global__ void __launch_bounds__(kMixedThreads, 1) ck_ldpc_mixed_code(const __grid_constant__ MixedParams p) {\n    mixed_body<%lld, CodeDispatch>(p);\n}\n", dmax);
    return s;
}

// Compiles `src` and loads `names` from it; returns false with `why` set
// when that fails.
bool compile_load(const std::string& src, int device, const char* const* names, int count, cudaLibrary_t* lib,
                  const void** kernels, std::string* why) {
    const Nvrtc& nv = nvrtc();
    if (!nv.create) {
        *why = nv.why;
        return false;
    }
    void* prog = nullptr;
    if (nv.create(&prog, src.c_str(), "ck_ldpc_code.cu", ck_jit_header_count, ck_jit_header_sources,
                  ck_jit_header_names) != 0) {
        *why = "nvrtcCreateProgram failed";
        return false;
    }
    int major = 0, minor = 0;
    (void)cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
    (void)cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
    const std::string arch = "-arch=sm_" + std::to_string(major * 10 + minor) + "a";
    const char* opts[] = {arch.c_str(), "-std=c++17", "-fmad=false"};
    bool ok = false;
    if (nv.compile(prog, 3, opts) != 0) {
        size_t n = 0;
        nv.log_size(prog, &n);
        std::string log(n, '\0');
        if (n) nv.log(prog, &log[0]);
        *why = "NVRTC compilation failed: " + log.substr(0, 2000);
    } else {
        size_t n = 0;
        nv.cubin_size(prog, &n);
        std::string cubin(n, '\0');
        nv.cubin(prog, &cubin[0]);
        cudaError_t ce = cudaLibraryLoadData(lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
        for (int i = 0; i < count && ce == cudaSuccess; ++i) {
            cudaKernel_t k = nullptr;
            ce = cudaLibraryGetKernel(&k, *lib, names[i]);
            kernels[i] = reinterpret_cast<const void*>(k);
        }
        if (ce != cudaSuccess) {
            (void)cudaGetLastError();
            if (*lib) (void)cudaLibraryUnload(*lib);
            *lib = nullptr;
            *why = std::string("loading the specialised kernels failed: ") + cudaGetErrorString(ce);
        } else {
            ok = true;
        }
    }
    nv.destroy(&prog);
    return ok;
}

int effective_mode(int32_t mode) {
    if (mode == CK_LDPC_SPECIALISE_AUTO) {
        const char* env = getenv("COMMKIT_GB300_SPECIALISE");
        if (env && env[0] == '0') return CK_LDPC_SPECIALISE_OFF;
    }
    return mode;
}

// Mixed kernels compiled so far, by (degree bound, plan ids and whether each
// code is specialised).
struct MixedJit {
    cudaLibrary_t lib = nullptr;
    const void* kernel = nullptr;
    std::string why;
};
std::mutex g_mixed_mu;
std::map<std::vector<uint64_t>, MixedJit> g_mixed;

}  // namespace

std::string specialised_source(const ck_ldpc_plan& plan, int dmax) { return program_source(plan, dmax); }

std::string mixed_source(const ck_ldpc_plan* const* plans, const int* parts, const int* edges, int n, int dmax) {
    return mixed_program_source(plans, parts, edges, n, dmax);
}

int specialised_kernel(const ck_ldpc_plan* plan, int dmax, int place, const void** out) {
    *out = nullptr;
    const int mode = effective_mode(plan->jit_mode);
    if (mode == CK_LDPC_SPECIALISE_OFF) return CK_OK;
    std::lock_guard<std::mutex> lock(plan->jit_mu);
    ck_ldpc_plan::Jit& j = plan->jit;
    if (!j.tried) {  // a plan's degree bound never changes, so one compilation serves it
        j.tried = true;
        j.dmax = dmax;
        static const char* const names[] = {"ck_ldpc_code_r0", "ck_ldpc_code_r1", "ck_ldpc_code_r2"};
        if (!compile_load(program_source(*plan, dmax), plan->device, names, 3, &j.lib, j.kernel, &j.why))
            j.lib = nullptr;
    }
    if (!j.lib) {
        if (mode == CK_LDPC_SPECIALISE_ON)
            return ck::fail(CK_ERR_UNSUPPORTED, "code-specialised decoder unavailable: %s", j.why.c_str());
        return CK_OK;
    }
    *out = j.kernel[place];
    return CK_OK;
}

int specialised_kernel_ready(const ck_ldpc_plan* plan, int place, const void** out) {
    *out = nullptr;
    const int mode = effective_mode(plan->jit_mode);
    if (mode == CK_LDPC_SPECIALISE_OFF) return CK_OK;
    std::lock_guard<std::mutex> lock(plan->jit_mu);
    const ck_ldpc_plan::Jit& j = plan->jit;
    if (j.tried && j.lib) {
        *out = j.kernel[place];
        return CK_OK;
    }
    if (mode == CK_LDPC_SPECIALISE_ON)
        return ck::fail(CK_ERR_UNSUPPORTED,
                        j.tried ? "code-specialised decoder unavailable: %s"
                                : "the code-specialised decoder is not compiled yet%s: decode once through "
                                  "ck_ldpc_decode first",
                        j.why.c_str());
    return CK_OK;
}

int mixed_specialised_kernel(const ck_ldpc_plan* const* plans, const int32_t* T, const int* edges, int n,
                             int dmax, const void** out) {
    *out = nullptr;
    int parts[CK_LDPC_MAX_MIXED] = {};
    int edge[CK_LDPC_MAX_MIXED] = {};
    if (n < 1 || n > CK_LDPC_MAX_MIXED) return CK_OK;
    bool any = false, required = false;
    std::vector<uint64_t> key{static_cast<uint64_t>(dmax)};
    for (int c = 0; c < n; ++c) {
        const int mode = effective_mode(plans[c]->jit_mode);
        if (mode == CK_LDPC_SPECIALISE_OFF) return CK_OK;  // any code opting out keeps the table kernel
        required |= mode == CK_LDPC_SPECIALISE_ON;
        // One or two threads per row slot (threads per frame Zp or 2 Zp) run
        // the code's program; other shapes run the table loop.
        const int32_t Zp = (plans[c]->Z + 31) / 32 * 32;
        parts[c] = T[c] == Zp ? 1 : (T[c] == 2 * Zp ? 2 : 0);
        edge[c] = parts[c] == 1 && edges[c] ? 1 : 0;  // per-edge state with one thread per row slot only
        any |= parts[c] > 0;
        key.push_back(plans[c]->id);
        key.push_back(static_cast<uint64_t>(parts[c]) | (static_cast<uint64_t>(edge[c]) << 8));
    }
    if (!any) return CK_OK;
    std::lock_guard<std::mutex> lock(g_mixed_mu);
    auto it = g_mixed.find(key);
    if (it == g_mixed.end()) {
        MixedJit mj;
        static const char* const names[] = {"ck_ldpc_mixed_code"};
        const void* k = nullptr;
        const int dev = plans[0]->device;
        if (compile_load(mixed_program_source(plans, parts, edge, n, dmax), dev, names, 1, &mj.lib, &k, &mj.why))
            mj.kernel = k;
        it = g_mixed.emplace(key, std::move(mj)).first;
    }
    if (!it->second.kernel) {
        if (required)
            return ck::fail(CK_ERR_UNSUPPORTED, "code-specialised mixed decoder unavailable: %s",
                            it->second.why.c_str());
        return CK_OK;
    }
    *out = it->second.kernel;
    return CK_OK;
}

void forget_plan_kernels(const ck_ldpc_plan* plan) {
    std::lock_guard<std::mutex> lock(g_mixed_mu);
    for (auto it = g_mixed.begin(); it != g_mixed.end();) {
        bool uses = false;
        for (size_t i = 1; i + 1 < it->first.size(); i += 2) uses |= it->first[i] == plan->id;
        if (!uses) {
            ++it;
            continue;
        }
        if (it->second.lib) {
            ck::forget_kernel(it->second.kernel);
            (void)cudaLibraryUnload(it->second.lib);
        }
        it = g_mixed.erase(it);
    }
    if (plan->jit.lib) {
        for (const void* k : plan->jit.kernel) ck::forget_kernel(k);
        (void)cudaLibraryUnload(plan->jit.lib);
    }
}

}  // namespace ldpc
}  // namespace ck
