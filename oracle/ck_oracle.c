/*
 * CPU oracle for the coded-modulation receiver back end.  TEST
 * INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU
 * baseline of the benchmark load this library to check (or time) the CUDA
 * path; the product never links or calls it.
 *
 * A plain-C restatement of the reference's CPU loops, in IEEE float32 with
 * no contraction (compiled with -ffp-contract=off, no fast-math), so that
 * every float operation rounds once, as numpy's float32 scalar operations do
 * when the reference's Numba kernels run interpreted:
 *
 *   oracle_ldpc_layered      commkit/coding/_numba_loops.py:43-68 (min_sum_row),
 *                            :97-106 (satisfied), :109-147 (ldpc_layered)
 *   oracle_ldpc_layered_sp   commkit/coding/_numba_loops.py:37-40 (phi),
 *                            :71-94 (sum_product_row)
 *   oracle_llr_sep_maxlog    commkit/mapping/_numba_llr.py:179-235
 *                            (axis_maxlog, llr_separable_maxlog_kernel)
 *   oracle_llr_separable     commkit/mapping/_numba_llr.py:35-92, 127-176
 *                            (prepare_exp, log_half_sum, bit_llr, axis_llrs,
 *                            llr_separable_kernel)
 *   oracle_llr_points        commkit/mapping/_numba_llr.py:35-81, 95-124
 *                            (the same steps over every point, llr_kernel)
 *
 * Codewords (and symbols) are independent, so the loops over them run on
 * OpenMP threads; each codeword's arithmetic is sequential and in the
 * reference's order, so the thread count never changes a result.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static void set_threads(int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Layered LDPC decoding                                                    */
/* ------------------------------------------------------------------------ */

/* _numba_loops.py:43-68: one check row by scaled/offset min-sum, in place. */
static void min_sum_row(float* a, float* r, const int32_t* cols, int32_t e0, int32_t e1,
                        float scale, float offset) {
    float min1 = INFINITY, min2 = INFINITY;
    int32_t idx = -1;
    int neg = 0;
    for (int32_t e = e0; e < e1; ++e) {
        const float q = a[cols[e]] - r[e];
        neg ^= (q < 0.0f);
        const float mag = fabsf(q);
        if (mag < min1) {
            min2 = min1;
            min1 = mag;
            idx = e;
        } else if (mag < min2) {
            min2 = mag;
        }
    }
    /* Python's max(v, 0) keeps v unless 0 > v. */
    float m1 = scale * min1;
    m1 = m1 - offset;
    if (0.0f > m1) m1 = 0.0f;
    float m2 = scale * min2;
    m2 = m2 - offset;
    if (0.0f > m2) m2 = 0.0f;
    for (int32_t e = e0; e < e1; ++e) {
        const int32_t c = cols[e];
        const float q = a[c] - r[e];
        const float mag = (e == idx) ? m2 : m1;
        const float rn = (neg ^ (q < 0.0f)) ? -mag : mag;
        a[c] = q + rn;
        r[e] = rn;
    }
}

/* _numba_loops.py:37-40: -log tanh(x/2) with x clipped to [1e-7, 30]. */
static float phi(float x) {
    const float lo = 1e-7f, hi = 30.0f;
    x = x < lo ? lo : x;
    x = x > hi ? hi : x;
    return -logf(tanhf(0.5f * x));
}

/* _numba_loops.py:71-94: one check row by sum-product (phi form). */
static void sum_product_row(float* a, float* r, const int32_t* cols, int32_t e0, int32_t e1) {
    float total = 0.0f;
    int neg = 0;
    for (int32_t e = e0; e < e1; ++e) {
        const int32_t c = cols[e];
        const float q = a[c] - r[e];
        neg ^= (q < 0.0f);
        const float p = phi(fabsf(q));
        total = total + p;
        a[c] = q;
        r[e] = p;
    }
    for (int32_t e = e0; e < e1; ++e) {
        const int32_t c = cols[e];
        const float q = a[c];
        const float mag = phi(total - r[e]);
        const float rn = (neg ^ (q < 0.0f)) ? -mag : mag;
        a[c] = q + rn;
        r[e] = rn;
    }
}

/* _numba_loops.py:97-106: every check satisfied by the hard decisions. */
static int satisfied(const float* a, const int32_t* row_ptr, const int32_t* cols, int32_t m) {
    for (int32_t row = 0; row < m; ++row) {
        int parity = 0;
        for (int32_t e = row_ptr[row]; e < row_ptr[row + 1]; ++e) parity ^= (a[cols[e]] < 0.0f);
        if (parity) return 0;
    }
    return 1;
}

/*
 * _numba_loops.py:109-147.  app (B, N) float32 in place; rows of the CSR
 * (row_ptr, cols) in schedule order (rows grouped by layer); rule 0 is
 * min-sum, 1 sum-product.  iters (B,) int32 and valid (B,) uint8 out.
 */
int oracle_ldpc_layered(float* app, int64_t B, int32_t N, const int32_t* row_ptr,
                        const int32_t* cols, int32_t m, int32_t rule, float scale,
                        float offset, int32_t max_iterations, int32_t early_stop,
                        int32_t* iters, uint8_t* valid, int threads) {
    if (B < 0 || N < 1 || m < 1 || max_iterations < 0) return 1;
    const int32_t E = row_ptr[m];
    set_threads(threads);
    int failed = 0;
#pragma omp parallel
    {
        float* r = (float*)malloc(sizeof(float) * (size_t)(E > 0 ? E : 1));
        if (!r) {
#pragma omp atomic write
            failed = 1;
        }
#pragma omp for schedule(dynamic, 1)
        for (int64_t b = 0; b < B; ++b) {
            if (!r) continue;
            float* a = app + b * (int64_t)N;
            memset(r, 0, sizeof(float) * (size_t)E);
            int32_t it = 0;
            int ok = early_stop && satisfied(a, row_ptr, cols, m);
            while (!ok && it < max_iterations) {
                for (int32_t row = 0; row < m; ++row) {
                    if (rule == 1)
                        sum_product_row(a, r, cols, row_ptr[row], row_ptr[row + 1]);
                    else
                        min_sum_row(a, r, cols, row_ptr[row], row_ptr[row + 1], scale, offset);
                }
                ++it;
                if (early_stop) ok = satisfied(a, row_ptr, cols, m);
            }
            if (!early_stop) ok = satisfied(a, row_ptr, cols, m);
            iters[b] = it;
            valid[b] = ok ? 1 : 0;
        }
        free(r);
    }
    return failed ? 2 : 0;
}

/* ------------------------------------------------------------------------ */
/* LLR demapping                                                            */
/* ------------------------------------------------------------------------ */

/* _numba_llr.py:179-210: closed-form max-log LLRs of one axis into out[pos[b]]. */
static void axis_maxlog(float x, const float* lev, const int32_t* lab, const int32_t* lo,
                        const int32_t* hi, const int32_t* pos, int32_t L, int32_t kb,
                        float inv_s2, float* out) {
    const float q = (x - lev[0]) / (lev[1] - lev[0]);
    const float qr = rintf(q);
    int64_t s;
    /* int() of a float beyond the clamp range only matters through the clamp. */
    if (qr < 0.0f) s = 0;
    else if (qr > (float)(L - 1)) s = L - 1;
    else s = (int64_t)qr;
    float t = x - lev[s];
    const int64_t s2 = t > 0.0f ? s + 1 : s - 1;
    if (s2 >= 0 && s2 < L) {
        const float t2 = x - lev[s2];
        if (t2 * t2 < t * t) {
            s = s2;
            t = t2;
        }
    }
    const float m_own = -(t * t) * inv_s2;
    for (int32_t b = 0; b < kb; ++b) {
        float m_other = -3.0e38f;
        int32_t j = lo[b * L + s];
        if (j >= 0) {
            const float u = x - lev[j];
            const float v = -(u * u) * inv_s2;
            if (v > m_other) m_other = v;
        }
        j = hi[b * L + s];
        if (j >= 0) {
            const float u = x - lev[j];
            const float v = -(u * u) * inv_s2;
            if (v > m_other) m_other = v;
        }
        if ((lab[s] >> (kb - 1 - b)) & 1)
            out[pos[b]] = m_other - m_own;
        else
            out[pos[b]] = m_own - m_other;
    }
}

/*
 * _numba_llr.py:213-235.  x (n,) complex64 as interleaved float pairs; per
 * axis: levels (L,), packed labels (L,), lo/hi (k_a, L), positions (k_a,);
 * out (n, k) float32.
 */
int oracle_llr_sep_maxlog(const float* x, int64_t n, int64_t frame_len, const float* inv_s2,
                          const float* lev_re, const int32_t* lab_re, const int32_t* lo_re,
                          const int32_t* hi_re, const int32_t* pos_re, int32_t L_re,
                          int32_t k_re, const float* lev_im, const int32_t* lab_im,
                          const int32_t* lo_im, const int32_t* hi_im, const int32_t* pos_im,
                          int32_t L_im, int32_t k_im, float* out, int threads) {
    if (n < 0 || L_re < 2 || L_im < 2 || frame_len < 1) return 1;
    const int32_t k = k_re + k_im;
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const float s2 = inv_s2[i / frame_len];
        axis_maxlog(x[2 * i], lev_re, lab_re, lo_re, hi_re, pos_re, L_re, k_re, s2, out + i * k);
        axis_maxlog(x[2 * i + 1], lev_im, lab_im, lo_im, hi_im, pos_im, L_im, k_im, s2,
                    out + i * k);
    }
    return 0;
}

#define ORACLE_EXACT_FLOOR 1e-26f
#define ORACLE_MAX_LEVELS 256

/*
 * _numba_llr.py:84-92 with :35-81: the LLRs of one axis's bits from the
 * metrics of its L levels.  Halves of bit b are the levels whose label bit
 * b (MSB first over the axis's k_a bits) is 0 and 1, in ascending level
 * order, as commkit/mapping/_demap.py:71-79 (_half_indices) lists them.
 */
static void axis_levels(float x, const float* lev, const float* logp, const int32_t* lab,
                        const int32_t* pos, int32_t L, int32_t kb, float inv_s2, int exact,
                        float* out) {
    float metric[ORACLE_MAX_LEVELS];
    float e[ORACLE_MAX_LEVELS];
    for (int32_t j = 0; j < L; ++j) {
        const float d = x - lev[j];
        metric[j] = -(d * d) * inv_s2 + logp[j];
    }
    float peak = 0.0f;
    if (exact) {
        peak = metric[0];
        for (int32_t j = 1; j < L; ++j)
            if (metric[j] > peak) peak = metric[j];
        for (int32_t j = 0; j < L; ++j) e[j] = expf(metric[j] - peak);
    }
    for (int32_t b = 0; b < kb; ++b) {
        const int shift = kb - 1 - b;
        float res[2];
        for (int v = 0; v < 2; ++v) {
            if (!exact) {
                /* bit_llr's max over the half, started at its first level. */
                int first = 1;
                float p = 0.0f;
                for (int32_t j = 0; j < L; ++j) {
                    if (((lab[j] >> shift) & 1) != v) continue;
                    if (first || metric[j] > p) p = metric[j];
                    first = 0;
                }
                res[v] = p;
                continue;
            }
            /* log_half_sum */
            float s = 0.0f;
            for (int32_t j = 0; j < L; ++j)
                if (((lab[j] >> shift) & 1) == v) s = s + e[j];
            if (s >= ORACLE_EXACT_FLOOR) {
                res[v] = logf(s);
                continue;
            }
            int first = 1;
            float p = 0.0f;
            for (int32_t j = 0; j < L; ++j) {
                if (((lab[j] >> shift) & 1) != v) continue;
                if (first || metric[j] > p) p = metric[j];
                first = 0;
            }
            s = 0.0f;
            for (int32_t j = 0; j < L; ++j)
                if (((lab[j] >> shift) & 1) == v) s = s + expf(metric[j] - p);
            res[v] = logf(s) + (p - peak);
        }
        out[pos[b]] = res[0] - res[1];
    }
}

/*
 * _numba_llr.py:127-176.  Per axis: levels (L,), log prior (L,), packed
 * labels (L,), positions (k_a,).  exact 0: max-log, 1: log-sum-exp.
 * inv_s2 holds one value per frame of frame_len symbols.
 */
int oracle_llr_separable(const float* x, int64_t n, int64_t frame_len, const float* inv_s2,
                         const float* lev_re, const float* logp_re, const int32_t* lab_re,
                         const int32_t* pos_re, int32_t L_re, int32_t k_re,
                         const float* lev_im, const float* logp_im, const int32_t* lab_im,
                         const int32_t* pos_im, int32_t L_im, int32_t k_im, int32_t exact,
                         float* out, int threads) {
    if (n < 0 || L_re < 1 || L_im < 1 || L_re > ORACLE_MAX_LEVELS || L_im > ORACLE_MAX_LEVELS ||
        frame_len < 1)
        return 1;
    const int32_t k = k_re + k_im;
    set_threads(threads);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const float s2 = inv_s2[i / frame_len];
        axis_levels(x[2 * i], lev_re, logp_re, lab_re, pos_re, L_re, k_re, s2, exact, out + i * k);
        axis_levels(x[2 * i + 1], lev_im, logp_im, lab_im, pos_im, L_im, k_im, s2, exact,
                    out + i * k);
    }
    return 0;
}

/*
 * _numba_llr.py:95-124 with :35-81: LLRs from the metrics of all M points,
 * -(dr*dr + di*di) * inv_s2 + log_pmf[m].  Halves of bit b are the points
 * whose label bit b (MSB first over k bits) is 0 and 1, in ascending point
 * order (commkit/mapping/_demap.py:71-79).  x (n, 2) and pts (M, 2) are
 * interleaved float32 (complex64); inv_s2 holds one value per frame.
 */
static void points_llrs(float xr, float xi, const float* pts, const float* logp,
                        const int32_t* lab, int32_t M, int32_t k, float inv_s2, int exact,
                        float* metric, float* e, float* out) {
    for (int32_t m = 0; m < M; ++m) {
        const float dr = xr - pts[2 * m];
        const float di = xi - pts[2 * m + 1];
        metric[m] = -(dr * dr + di * di) * inv_s2 + logp[m];
    }
    float peak = 0.0f;
    if (exact) {
        peak = metric[0];
        for (int32_t m = 1; m < M; ++m)
            if (metric[m] > peak) peak = metric[m];
        for (int32_t m = 0; m < M; ++m) e[m] = expf(metric[m] - peak);
    }
    for (int32_t b = 0; b < k; ++b) {
        const int shift = k - 1 - b;
        float res[2];
        for (int v = 0; v < 2; ++v) {
            int first = 1;
            float p = 0.0f;
            for (int32_t m = 0; m < M; ++m) {
                if (((lab[m] >> shift) & 1) != v) continue;
                if (first || metric[m] > p) p = metric[m];
                first = 0;
            }
            if (!exact) {
                res[v] = p;
                continue;
            }
            float s = 0.0f;
            for (int32_t m = 0; m < M; ++m)
                if (((lab[m] >> shift) & 1) == v) s = s + e[m];
            if (s >= ORACLE_EXACT_FLOOR) {
                res[v] = logf(s);
                continue;
            }
            s = 0.0f;
            for (int32_t m = 0; m < M; ++m)
                if (((lab[m] >> shift) & 1) == v) s = s + expf(metric[m] - p);
            res[v] = logf(s) + (p - peak);
        }
        out[b] = res[0] - res[1];
    }
}

int oracle_llr_points(const float* x, int64_t n, int64_t frame_len, const float* inv_s2,
                      const float* pts, const float* logp, const int32_t* lab, int32_t M,
                      int32_t k, int32_t exact, float* out, int threads) {
    if (n < 0 || M < 1 || k < 1 || k > 30 || frame_len < 1) return 1;
    set_threads(threads);
    int failed = 0;
#pragma omp parallel
    {
        float* metric = (float*)malloc(sizeof(float) * (size_t)M);
        float* e = (float*)malloc(sizeof(float) * (size_t)M);
        if (!metric || !e) {
#pragma omp atomic write
            failed = 1;
        }
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            if (!metric || !e) continue;
            points_llrs(x[2 * i], x[2 * i + 1], pts, logp, lab, M, k, inv_s2[i / frame_len], exact,
                        metric, e, out + i * k);
        }
        free(metric);
        free(e);
    }
    return failed ? 2 : 0;
}
