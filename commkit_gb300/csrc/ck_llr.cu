// Soft LLR demapping of separable (Gray square) QAM on sm_103a: the C-ABI
// entry points (argument checks and dispatch on the bits per axis).  The
// kernels are in ck_llr_kernels.cuh.
#include <stdint.h>

#include "ck_llr_points.cuh"

namespace ck {
namespace llr {

int g_num_sms = 0;


int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return 148;
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            (void)cudaGetLastError();
            return 148;
        }
        g_num_sms = v;
    }
    return g_num_sms;
}

template <class AX>
int check_axis(const AX* a, const char* name) {
    if (!a) return ck::fail(CK_ERR_INVALID_ARGUMENT, "the %s axis is NULL", name);
    if (a->k < 1 || a->k > CK_LLR_MAX_K)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "bits of the %s axis must be in [1, %d], got %d",
                        name, CK_LLR_MAX_K, a->k);
    if (!a->levels || !a->labels || !a->pos)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "a table of the %s axis is NULL", name);
    return CK_OK;
}


#define CK_LLR_EXTERN(KA)                                                                  \
    extern template int launch_ka<KA, 0, ck_axis_maxlog>(                                \
        const void*, uint32_t, const ck_axis_maxlog&, const ck_axis_maxlog&,             \
        const NoiseScale&, float*, cudaStream_t);                                        \
    extern template int launch_ka<KA, 1, ck_axis_levels>(                                \
        const void*, uint32_t, const ck_axis_levels&, const ck_axis_levels&,             \
        const NoiseScale&, float*, cudaStream_t);                                        \
    extern template int launch_ka<KA, 2, ck_axis_levels>(                                \
        const void*, uint32_t, const ck_axis_levels&, const ck_axis_levels&,             \
        const NoiseScale&, float*, cudaStream_t);
CK_LLR_EXTERN(1)
CK_LLR_EXTERN(2)
CK_LLR_EXTERN(3)
CK_LLR_EXTERN(4)
CK_LLR_EXTERN(5)
CK_LLR_EXTERN(6)
#undef CK_LLR_EXTERN

namespace points {
#define CK_LLR_POINTS_EXTERN(K)                                                               \
    extern template int launch_points<K>(const float2*, uint32_t, const Table&, const NoiseScale&, \
                                         bool, float*, cudaStream_t);
CK_LLR_POINTS_EXTERN(1) CK_LLR_POINTS_EXTERN(2) CK_LLR_POINTS_EXTERN(3) CK_LLR_POINTS_EXTERN(4)
CK_LLR_POINTS_EXTERN(5) CK_LLR_POINTS_EXTERN(6) CK_LLR_POINTS_EXTERN(7) CK_LLR_POINTS_EXTERN(8)
CK_LLR_POINTS_EXTERN(9) CK_LLR_POINTS_EXTERN(10) CK_LLR_POINTS_EXTERN(11) CK_LLR_POINTS_EXTERN(12)
CK_LLR_POINTS_EXTERN(13) CK_LLR_POINTS_EXTERN(14) CK_LLR_POINTS_EXTERN(15) CK_LLR_POINTS_EXTERN(16)
#undef CK_LLR_POINTS_EXTERN
}  // namespace points

namespace {

template <int METHOD, class AX>
int launch(const void* x, int64_t n, const AX* re, const AX* im, const NoiseScale& noise,
           float* out, void* stream) {
    ck::clear_error();
    CK_TRY(check_axis(re, "re"));
    CK_TRY(check_axis(im, "im"));
    if (n < 0 || n >= (int64_t(1) << 31))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "at most 2**31 - 1 symbols per call, got %lld",
                        static_cast<long long>(n));
    if (re->k + im->k > CK_LLR_MAX_K)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "bits per symbol must be at most %d, got %d",
                        CK_LLR_MAX_K, re->k + im->k);
    const int lmin = METHOD == 0 ? 2 : 1;
    if (re->L < lmin || im->L < lmin)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "each axis needs at least %d levels", lmin);
    if (re->k != im->k || re->L != (1 << re->k) || im->L != (1 << im->k))
        return ck::fail(CK_ERR_UNSUPPORTED,
                        "the kernels take square lattices with 2**k levels per axis "
                        "(re: L=%d k=%d, im: L=%d k=%d)",
                        re->L, re->k, im->L, im->k);
    if (n == 0) return CK_OK;
    if (!x || !out) return ck::fail(CK_ERR_INVALID_ARGUMENT, "x or out is NULL");
    if (reinterpret_cast<uintptr_t>(x) % 8 != 0 || reinterpret_cast<uintptr_t>(out) % 4 != 0)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "x must be 8-byte and out 4-byte aligned");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t nn = static_cast<uint32_t>(n);
    switch (re->k) {
        case 1: return launch_ka<1, METHOD>(x, nn, *re, *im, noise, out, s);
        case 2: return launch_ka<2, METHOD>(x, nn, *re, *im, noise, out, s);
        case 3: return launch_ka<3, METHOD>(x, nn, *re, *im, noise, out, s);
        case 4: return launch_ka<4, METHOD>(x, nn, *re, *im, noise, out, s);
        case 5: return launch_ka<5, METHOD>(x, nn, *re, *im, noise, out, s);
        case 6: return launch_ka<6, METHOD>(x, nn, *re, *im, noise, out, s);
        default:
            return ck::fail(CK_ERR_UNSUPPORTED,
                            "square QAM up to 4096 points (6 bits per axis), got %d bits per axis",
                            re->k);
    }
}

NoiseScale scalar_noise(float inv_s2) {
    NoiseScale s;
    s.frames = nullptr;
    s.value = inv_s2;
    s.frame_len = ck::FastDiv::make(1);
    return s;
}

int frame_noise(int64_t n, int64_t frame_len, const float* inv_s2, NoiseScale* s) {
    if (frame_len < 1 || frame_len >= (int64_t(1) << 31))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "frame_len must be in [1, 2**31), got %lld",
                        static_cast<long long>(frame_len));
    if (!inv_s2 && n > 0) return ck::fail(CK_ERR_INVALID_ARGUMENT, "inv_s2 is NULL");
    s->frames = inv_s2;
    s->value = 0.0f;
    s->frame_len = ck::FastDiv::make(static_cast<uint32_t>(frame_len));
    return CK_OK;
}

int launch_points(const void* x, int64_t n, const void* pts, const float* log_pmf,
                  const int32_t* labels, int32_t M, int32_t k, int32_t exact, const NoiseScale& noise,
                  float* out, void* stream) {
    if (k < 1 || k > CK_LLR_MAX_K)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "bits per symbol must be in [1, %d], got %d",
                        CK_LLR_MAX_K, k);
    if (M < 1) return ck::fail(CK_ERR_INVALID_ARGUMENT, "points must be non-empty, got M=%d", M);
    if (n < 0 || n >= (int64_t(1) << 31))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "at most 2**31 - 1 symbols per call, got %lld",
                        static_cast<long long>(n));
    if (n == 0) return CK_OK;
    if (!x || !out || !pts || !log_pmf || !labels)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "an array is NULL");
    if (reinterpret_cast<uintptr_t>(x) % 8 != 0 || reinterpret_cast<uintptr_t>(pts) % 8 != 0 ||
        reinterpret_cast<uintptr_t>(out) % 4 != 0)
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "x and points must be 8-byte and out 4-byte aligned");
    const points::Table t{static_cast<const float2*>(pts), log_pmf, labels, M};
    const float2* xs = static_cast<const float2*>(x);
    const uint32_t nn = static_cast<uint32_t>(n);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool ex = exact != 0;
    switch (k) {
#define CK_CASE(K) \
    case K: return points::launch_points<K>(xs, nn, t, noise, ex, out, s);
        CK_CASE(1) CK_CASE(2) CK_CASE(3) CK_CASE(4) CK_CASE(5) CK_CASE(6) CK_CASE(7) CK_CASE(8)
        CK_CASE(9) CK_CASE(10) CK_CASE(11) CK_CASE(12) CK_CASE(13) CK_CASE(14) CK_CASE(15) CK_CASE(16)
#undef CK_CASE
        default: return ck::fail(CK_ERR_INVALID_ARGUMENT, "bad k");
    }
}

int check_lo_hi(const ck_axis_maxlog* a) {
    if (a && (!a->lo || !a->hi))
        return ck::fail(CK_ERR_INVALID_ARGUMENT, "lo/hi tables are NULL");
    return CK_OK;
}

}  // namespace
}  // namespace llr
}  // namespace ck

using ck::llr::launch;
using ck::llr::scalar_noise;
using ck::llr::frame_noise;
using ck::llr::check_lo_hi;
using ck::llr::launch_points;
using ck::llr::NoiseScale;

extern "C" int ck_llr_separable_maxlog(const void* x, int64_t n, const ck_axis_maxlog* re,
                                       const ck_axis_maxlog* im, float inv_s2, float* out,
                                       void* stream) {
    CK_TRY(check_lo_hi(re));
    CK_TRY(check_lo_hi(im));
    return launch<0>(x, n, re, im, scalar_noise(inv_s2), out, stream);
}

extern "C" int ck_llr_separable(const void* x, int64_t n, const ck_axis_levels* re,
                                const ck_axis_levels* im, float inv_s2, int32_t exact,
                                float* out, void* stream) {
    if (re && !re->logp) return ck::fail(CK_ERR_INVALID_ARGUMENT, "re log prior is NULL");
    if (im && !im->logp) return ck::fail(CK_ERR_INVALID_ARGUMENT, "im log prior is NULL");
    return exact ? launch<2>(x, n, re, im, scalar_noise(inv_s2), out, stream)
                 : launch<1>(x, n, re, im, scalar_noise(inv_s2), out, stream);
}

extern "C" int ck_llr_separable_maxlog_frames(const void* x, int64_t n, int64_t frame_len,
                                              const float* inv_s2, const ck_axis_maxlog* re,
                                              const ck_axis_maxlog* im, float* out,
                                              void* stream) {
    NoiseScale s;
    CK_TRY(frame_noise(n, frame_len, inv_s2, &s));
    CK_TRY(check_lo_hi(re));
    CK_TRY(check_lo_hi(im));
    return launch<0>(x, n, re, im, s, out, stream);
}

extern "C" int ck_llr_separable_frames(const void* x, int64_t n, int64_t frame_len,
                                       const float* inv_s2, const ck_axis_levels* re,
                                       const ck_axis_levels* im, int32_t exact, float* out,
                                       void* stream) {
    NoiseScale s;
    CK_TRY(frame_noise(n, frame_len, inv_s2, &s));
    if (re && !re->logp) return ck::fail(CK_ERR_INVALID_ARGUMENT, "re log prior is NULL");
    if (im && !im->logp) return ck::fail(CK_ERR_INVALID_ARGUMENT, "im log prior is NULL");
    return exact ? launch<2>(x, n, re, im, s, out, stream)
                 : launch<1>(x, n, re, im, s, out, stream);
}

extern "C" int ck_llr_points(const void* x, int64_t n, const void* points, const float* log_pmf,
                             const int32_t* labels, int32_t M, int32_t k, float inv_s2,
                             int32_t exact, float* out, void* stream) {
    ck::clear_error();
    return launch_points(x, n, points, log_pmf, labels, M, k, exact, scalar_noise(inv_s2), out,
                         stream);
}

extern "C" int ck_llr_points_frames(const void* x, int64_t n, int64_t frame_len,
                                    const float* inv_s2, const void* points,
                                    const float* log_pmf, const int32_t* labels, int32_t M,
                                    int32_t k, int32_t exact, float* out, void* stream) {
    ck::clear_error();
    NoiseScale s;
    CK_TRY(frame_noise(n, frame_len, inv_s2, &s));
    return launch_points(x, n, points, log_pmf, labels, M, k, exact, s, out, stream);
}
