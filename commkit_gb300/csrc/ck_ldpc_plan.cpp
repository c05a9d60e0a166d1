// Host side of the layered LDPC decoder: the first-fit layer schedule and
// the decoding plan (schedule validation, recovery of the circulant
// structure of quasi-cyclic codes, device tables).
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <numeric>
#include <vector>

#include "ck_ldpc_internal.h"

// ---------------------------------------------------------------------------
// First-fit schedule: restates LDPCCode._schedule and _first_fit
// (commkit/coding/ldpc.py:283-296, 422-442).
// ---------------------------------------------------------------------------

extern "C" int ck_ldpc_schedule(const int32_t* checks, const int32_t* variables, int64_t E,
                                int32_t m, int32_t N, int32_t* row_ptr, int32_t* cols,
                                int32_t* layer_ptr, int32_t* num_layers) {
    ck::clear_error();
    if (!checks || !variables || !row_ptr || !cols || !layer_ptr || !num_layers)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
    if (m < 1 || N < 1 || E < 1 || E >= (int64_t(1) << 31))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "bad sizes m=%d N=%d E=%lld", m, N,
                        static_cast<long long>(E));
    // Rows in natural order: the edges are sorted by (row, column).
    std::vector<int64_t> ptr(static_cast<size_t>(m) + 1, 0);
    for (int64_t e = 0; e < E; ++e) {
        const int32_t r = checks[e];
        const int32_t c = variables[e];
        if (r < 0 || r >= m || c < 0 || c >= N)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "edge %lld out of range", static_cast<long long>(e));
        if (e > 0 && (checks[e - 1] > r || (checks[e - 1] == r && variables[e - 1] >= c)))
            return ck::fail(CK_ERR_INVALID_ARGUMENT,
                            "edges must be sorted by (row, column) without duplicates");
        ++ptr[static_cast<size_t>(r) + 1];
    }
    for (int32_t r = 0; r < m; ++r) ptr[r + 1] += ptr[r];

    // Layers used by each variable, as a bit set of `words` 64-bit words.
    size_t words = 1;
    std::vector<uint64_t> masks(static_cast<size_t>(N) * words, 0);
    std::vector<int32_t> color(static_cast<size_t>(m));
    std::vector<uint64_t> used;
    int32_t layers = 0;
    for (int32_t r = 0; r < m; ++r) {
        used.assign(words, 0);
        for (int64_t e = ptr[r]; e < ptr[r + 1]; ++e) {
            const uint64_t* mv = &masks[static_cast<size_t>(variables[e]) * words];
            for (size_t w = 0; w < words; ++w) used[w] |= mv[w];
        }
        // Lowest layer not in `used`.
        int32_t c = -1;
        for (size_t w = 0; w < words && c < 0; ++w) {
            if (~used[w]) c = static_cast<int32_t>(w * 64 + __builtin_ctzll(~used[w]));
        }
        if (c < 0) c = static_cast<int32_t>(words * 64);
        if (static_cast<size_t>(c) >= words * 64) {
            // Grow every mask by one word.
            const size_t nw = words + 1;
            std::vector<uint64_t> grown(static_cast<size_t>(N) * nw, 0);
            for (int32_t v = 0; v < N; ++v)
                memcpy(&grown[static_cast<size_t>(v) * nw], &masks[static_cast<size_t>(v) * words],
                       words * sizeof(uint64_t));
            masks.swap(grown);
            words = nw;
        }
        for (int64_t e = ptr[r]; e < ptr[r + 1]; ++e)
            masks[static_cast<size_t>(variables[e]) * words + static_cast<size_t>(c / 64)] |=
                uint64_t(1) << (c % 64);
        color[r] = c;
        layers = std::max(layers, c + 1);
    }
    // Stable grouping of the rows by layer.
    std::vector<int32_t> count(static_cast<size_t>(layers) + 1, 0);
    for (int32_t r = 0; r < m; ++r) ++count[color[r] + 1];
    for (int32_t l = 0; l < layers; ++l) count[l + 1] += count[l];
    std::vector<int32_t> order(static_cast<size_t>(m));
    {
        std::vector<int32_t> next(count.begin(), count.end() - 1);
        for (int32_t r = 0; r < m; ++r) order[next[color[r]]++] = r;
    }
    row_ptr[0] = 0;
    int64_t out = 0;
    for (int32_t i = 0; i < m; ++i) {
        const int32_t r = order[i];
        for (int64_t e = ptr[r]; e < ptr[r + 1]; ++e) cols[out++] = variables[e];
        row_ptr[i + 1] = static_cast<int32_t>(out);
    }
    for (int32_t l = 0; l <= layers; ++l) layer_ptr[l] = count[l];
    *num_layers = layers;
    return CK_OK;
}

// ---------------------------------------------------------------------------
// Plan
// ---------------------------------------------------------------------------

namespace {

// The circulant structure of a schedule for lifting Z, if it has one: every
// layer is a run of whole base rows (Z consecutive schedule rows whose row
// r has, at edge e, the column j_e Z + (o_e + r) mod Z for one j_e and
// shift o_e), with the block columns j_e strictly increasing along a row.
bool try_qc(const int32_t* row_ptr, const int32_t* cols, const int32_t* layer_ptr, int32_t m,
            int32_t N, int32_t L, int32_t Z, ck_ldpc_plan* plan) {
    if (Z < 2 || m % Z || N % Z) return false;
    for (int32_t l = 0; l < L; ++l)
        if ((layer_ptr[l + 1] - layer_ptr[l]) % Z) return false;
    const int32_t mb = m / Z;
    std::vector<int32_t> eptr(1, 0);
    std::vector<int32_t> blk_col, blk_shift;
    for (int32_t b = 0; b < mb; ++b) {
        const int32_t r0 = b * Z;
        const int32_t e0 = row_ptr[r0];
        const int32_t deg = row_ptr[r0 + 1] - e0;
        for (int32_t e = 0; e < deg; ++e) {
            const int32_t c = cols[e0 + e];
            const int32_t j = c / Z;
            if (e > 0 && j <= blk_col.back() / Z) return false;
            blk_col.push_back(j * Z);
            blk_shift.push_back(c % Z);
        }
        for (int32_t r = 1; r < Z; ++r) {
            const int32_t er = row_ptr[r0 + r];
            if (row_ptr[r0 + r + 1] - er != deg) return false;
            for (int32_t e = 0; e < deg; ++e) {
                const int32_t c = cols[er + e];
                const int32_t want_o = (blk_shift[eptr.back() + e] + r) % Z;
                if (c != blk_col[eptr.back() + e] + want_o) return false;
            }
        }
        eptr.push_back(static_cast<int32_t>(blk_col.size()));
    }
    plan->qc = true;
    plan->Z = Z;
    plan->mb = mb;
    plan->nb = N / Z;
    plan->nnzb = static_cast<int32_t>(blk_col.size());
    plan->h_layer.assign(static_cast<size_t>(L) + 1, 0);
    for (int32_t l = 0; l <= L; ++l) plan->h_layer[l] = layer_ptr[l] / Z;
    plan->h_eptr = eptr;
    plan->h_blk.resize(blk_col.size() * 2);
    // Per circulant: (j Z + shift, (j + 1) Z), so that row r's column is
    // r + first, wrapped back by Z once it reaches the block's end.
    for (size_t i = 0; i < blk_col.size(); ++i) {
        plan->h_blk[2 * i] = blk_col[i] + blk_shift[i];
        plan->h_blk[2 * i + 1] = blk_col[i] + Z;
    }
    return true;
}

int upload(const std::vector<int32_t>& h, int32_t** d) {
    *d = nullptr;
    if (h.empty()) return CK_OK;
    CK_CUDA(cudaMalloc(d, h.size() * sizeof(int32_t)));
    CK_CUDA(cudaMemcpy(*d, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    return CK_OK;
}

}  // namespace

namespace {

// Checks a schedule and fills the host side of `plan` (sizes, degree bound,
// circulant structure); touches no device.
int plan_host(const int32_t* row_ptr, const int32_t* cols, const int32_t* layer_ptr, int32_t m, int32_t N,
              int32_t L, ck_ldpc_plan* plan) {
    if (!row_ptr || !cols || !layer_ptr)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "row_ptr, cols and layer_ptr are required");
    if (m < 1 || N < 1 || L < 1)
        return ck::fail(CK_ERR_INVALID_ARGUMENT,
                        "row_ptr and layer_ptr need at least 2 entries (m=%d, L=%d)", m, L);
    if (row_ptr[0] != 0) return ck::fail(CK_ERR_INVALID_ARGUMENT, "row_ptr[0] must be 0");
    int32_t max_deg = 0;
    for (int32_t r = 0; r < m; ++r) {
        const int32_t d = row_ptr[r + 1] - row_ptr[r];
        if (d < 2)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "row %d has %d edges; every check needs >= 2",
                            r, d);
        max_deg = std::max(max_deg, d);
    }
    const int32_t E = row_ptr[m];
    for (int32_t e = 0; e < E; ++e)
        if (cols[e] < 0 || cols[e] >= N)
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "cols[%d] = %d out of [0, %d)", e, cols[e], N);
    if (layer_ptr[0] != 0 || layer_ptr[L] != m)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "layer_ptr must run from 0 to m");
    for (int32_t l = 0; l < L; ++l)
        if (layer_ptr[l + 1] <= layer_ptr[l])
            return ck::fail(CK_ERR_INVALID_ARGUMENT, "layer %d is empty or decreasing", l);
    // Rows of a layer must share no variable: the decoder updates them at once.
    {
        std::vector<int32_t> owner(static_cast<size_t>(N), -1);
        for (int32_t l = 0; l < L; ++l)
            for (int32_t r = layer_ptr[l]; r < layer_ptr[l + 1]; ++r)
                for (int32_t e = row_ptr[r]; e < row_ptr[r + 1]; ++e) {
                    if (owner[cols[e]] == l)
                        return ck::fail(CK_ERR_INVALID_ARGUMENT,
                                        "rows of layer %d share variable %d", l, cols[e]);
                    owner[cols[e]] = l;
                }
    }
    // Edges of a row in increasing column order (as LDPCCode stores them).
    for (int32_t r = 0; r < m; ++r)
        for (int32_t e = row_ptr[r] + 1; e < row_ptr[r + 1]; ++e)
            if (cols[e] <= cols[e - 1])
                return ck::fail(CK_ERR_INVALID_ARGUMENT,
                                "the columns of row %d must be increasing", r);
    plan->m = m;
    plan->N = N;
    plan->E = E;
    plan->L = L;
    plan->max_deg = max_deg;
    int32_t max_layer_rows = 0;
    for (int32_t l = 0; l < L; ++l)
        max_layer_rows = std::max(max_layer_rows, layer_ptr[l + 1] - layer_ptr[l]);
    plan->max_layer_rows = max_layer_rows;

    // Lifting: the largest Z dividing N and every layer's row count for
    // which the circulant pattern holds.
    int32_t g = N;
    for (int32_t l = 0; l < L; ++l) g = std::gcd(g, layer_ptr[l + 1] - layer_ptr[l]);
    for (int32_t Z = g; Z >= 2 && !plan->qc; --Z) {
        if (g % Z) continue;
        if (m / Z > ck::kMaxBaseRows) break;
        try_qc(row_ptr, cols, layer_ptr, m, N, L, Z, plan);
    }
    if (plan->qc && plan->nnzb > ck::kMaxBlocks) plan->qc = false;
    return CK_OK;
}

}  // namespace

extern "C" int ck_ldpc_plan_create(const int32_t* row_ptr, const int32_t* cols,
                                   const int32_t* layer_ptr, int32_t m, int32_t N, int32_t L,
                                   ck_ldpc_plan** out) {
    ck::clear_error();
    if (!out) return ck::fail(CK_ERR_INVALID_ARGUMENT, "plan is NULL");
    *out = nullptr;
    static std::atomic<uint64_t> next_id{1};
    ck_ldpc_plan* plan = new ck_ldpc_plan();
    plan->id = next_id.fetch_add(1);
    int status = plan_host(row_ptr, cols, layer_ptr, m, N, L, plan);
    if (status == CK_OK) status = ck::cuda_check(cudaGetDevice(&plan->device), "cudaGetDevice");
    if (status != CK_OK) {
        delete plan;
        return status;
    }
    if (plan->qc) {
        status = upload(plan->h_layer, &plan->d_layer);
        if (status == CK_OK) status = upload(plan->h_eptr, &plan->d_eptr);
        if (status == CK_OK) status = upload(plan->h_blk, &plan->d_blk);
    } else {
        plan->h_layer.assign(layer_ptr, layer_ptr + L + 1);
        std::vector<int32_t> rp(row_ptr, row_ptr + m + 1), cc(cols, cols + plan->E);
        status = upload(plan->h_layer, &plan->d_layer);
        if (status == CK_OK) status = upload(rp, &plan->d_eptr);
        if (status == CK_OK) status = upload(cc, &plan->d_cols);
    }
    if (status != CK_OK) {
        ck_ldpc_plan_destroy(plan);
        return status;
    }
    plan->divZ = ck::FastDiv::make(static_cast<uint32_t>(plan->qc ? plan->Z : 1));
    *out = plan;
    return CK_OK;
}

extern "C" int ck_ldpc_specialised_source(const int32_t* row_ptr, const int32_t* cols,
                                          const int32_t* layer_ptr, int32_t m, int32_t N, int32_t L,
                                          int32_t form, char* out, size_t capacity, size_t* length) {
    ck::clear_error();
    if (!length) return ck::fail(CK_ERR_INVALID_ARGUMENT, "length is NULL");
    if (form < 0 || form > 3) return ck::fail(CK_ERR_INVALID_ARGUMENT, "form must be 0, 1, 2 or 3");
    ck_ldpc_plan plan;
    CK_TRY(plan_host(row_ptr, cols, layer_ptr, m, N, L, &plan));
    if (!plan.qc) return ck::fail(CK_ERR_UNSUPPORTED, "the schedule has no circulant structure");
    if (plan.max_deg > ck::ldpc::kPackedDegree)
        return ck::fail(CK_ERR_UNSUPPORTED,
                        "rows of %d edges: codes with rows above %d edges run the any-degree kernels, "
                        "which have no code-specialised form", plan.max_deg, ck::ldpc::kPackedDegree);
    const int dmax = ck::ldpc::kernel_dmax(true, plan.max_deg);
    const ck_ldpc_plan* plans[1] = {&plan};
    const int parts[1] = {form == 2 ? 2 : 1};  // form 2: two threads per row slot, else one
    const int edges[1] = {form == 3 ? 1 : 0};  // form 3: one message per edge in shared memory
    const std::string src = form == 0 ? ck::ldpc::specialised_source(plan, dmax)
                                      : ck::ldpc::mixed_source(plans, parts, edges, 1, dmax);
    *length = src.size();
    if (out && capacity > 0) {
        const size_t n = std::min(capacity - 1, src.size());
        memcpy(out, src.data(), n);
        out[n] = '\0';
    }
    return CK_OK;
}

extern "C" int ck_ldpc_plan_destroy(ck_ldpc_plan* plan) {
    if (!plan) return CK_OK;
    int dev = -1;
    (void)cudaGetDevice(&dev);
    if (dev != plan->device) (void)cudaSetDevice(plan->device);
    if (plan->d_layer) (void)cudaFree(plan->d_layer);
    if (plan->d_eptr) (void)cudaFree(plan->d_eptr);
    if (plan->d_blk) (void)cudaFree(plan->d_blk);
    if (plan->d_cols) (void)cudaFree(plan->d_cols);
    ck::ldpc::forget_plan_kernels(plan);
    if (dev >= 0 && dev != plan->device) (void)cudaSetDevice(dev);
    delete plan;
    return CK_OK;
}

extern "C" int ck_ldpc_plan_get_info(const ck_ldpc_plan* plan, ck_ldpc_plan_info* info) {
    if (!plan || !info) return ck::fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
    info->quasi_cyclic = plan->qc ? 1 : 0;
    info->lifting = plan->qc ? plan->Z : 0;
    info->base_rows = plan->qc ? plan->mb : 0;
    info->base_cols = plan->qc ? plan->nb : 0;
    info->blocks = plan->qc ? plan->nnzb : 0;
    info->num_checks = plan->m;
    info->num_variables = plan->N;
    info->num_edges = plan->E;
    info->num_layers = plan->L;
    info->max_row_degree = plan->max_deg;
    info->device = plan->device;
    return CK_OK;
}

extern "C" int ck_ldpc_plan_set_launch(ck_ldpc_plan* plan, const ck_ldpc_launch* launch) {
    ck::clear_error();
    if (!plan || !launch) return ck::fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
    const int32_t T = launch->threads_per_frame, G = launch->frames_per_block;
    if (T != 0 && (T < 32 || T > 1024 || T % 32))
        return ck::fail(CK_ERR_INVALID_ARGUMENT,
                        "threads_per_frame must be 0 or a multiple of 32 in [32, 1024], got %d", T);
    if (G < 0 || (T > 0 && G > 0 && T * G > 1024))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "frames_per_block %d too large", G);
    if (T > 32 && G > ck::kMaxNamedGroups)
        return ck::fail(CK_ERR_INVALID_ARGUMENT,
                        "at most %d multi-warp frames per block (named barriers)",
                        ck::kMaxNamedGroups);
    if (launch->placement < CK_LDPC_PLACE_AUTO || launch->placement > CK_LDPC_PLACE_EDGES)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "unknown placement %d", launch->placement);
    plan->launch = *launch;
    return CK_OK;
}

extern "C" int ck_ldpc_plan_set_specialise(ck_ldpc_plan* plan, int32_t mode) {
    ck::clear_error();
    if (!plan) return ck::fail(CK_ERR_INVALID_ARGUMENT, "NULL plan");
    if (mode != CK_LDPC_SPECIALISE_AUTO && mode != CK_LDPC_SPECIALISE_OFF && mode != CK_LDPC_SPECIALISE_ON)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "unknown specialisation mode %d", mode);
    plan->jit_mode = mode;
    return CK_OK;
}

extern "C" int ck_ldpc_plan_get_specialise(const ck_ldpc_plan* plan, int32_t* mode, int32_t* state) {
    ck::clear_error();
    if (!plan || !mode || !state) return ck::fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lock(plan->jit_mu);
    *mode = plan->jit_mode;
    *state = !plan->jit.tried ? 0 : (plan->jit.lib ? 1 : -1);
    if (*state < 0) (void)ck::fail(CK_ERR_UNSUPPORTED, "%s", plan->jit.why.c_str());
    return CK_OK;
}

extern "C" int ck_ldpc_plan_get_launch(const ck_ldpc_plan* plan, ck_ldpc_launch* launch) {
    if (!plan || !launch) return ck::fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
    *launch = plan->launch;
    return CK_OK;
}
