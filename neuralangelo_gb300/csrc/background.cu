// Background NeRF input encoding and density head for the fused training step.
//
// gbsdf_bg_encode  : BackgroundNeRF.encode (projects/neuralangelo/utils/modules.py:286-301)
//   of the background samples of every ray (points c + d t, camera.py:314-320, at the
//   distances of Model.sample_dists_background, model.py:269-273): [x/|x|, 1/|x|] and
//   its Fourier code (nerf_util.py:134-147: sin and cos of 2^k pi q, channel-major,
//   sin block before cos block), as fp16 rows (optionally hi + lo pairs) of the first
//   MLP layer's input; and the
//   colour MLP's input tail (modules.py:277-281): SH(d) of degree 3, the per-image
//   appearance code, then a constant-1 column (the bias column of the weight-gradient
//   GEMM).
// gbsdf_bg_density : the density output of the last point-wise layer,
//   softplus(w . h + b) (modules.py:272, torch softplus, beta 1, threshold 20), one warp
//   per row.

#include "common.cuh"
#include "dense.cuh"

namespace gbsdf {

namespace {

constexpr int BG_ENC_COLS = 84;     // 4 + 8 x 10 levels
constexpr int BG_LEVELS = 10;

// real spherical-harmonic basis up to degree 3 (spherical_harmonics.py:47-84)
__device__ __forceinline__ void sh16(float dx, float dy, float dz, float* o) {
    const float xx = dx * dx, yy = dy * dy, zz = dz * dz;
    o[0] = 0.28209479177387814f;
    o[1] = -0.4886025119029199f * dy;
    o[2] = 0.4886025119029199f * dz;
    o[3] = -0.4886025119029199f * dx;
    o[4] = 1.0925484305920792f * dx * dy;
    o[5] = -1.0925484305920792f * dy * dz;
    o[6] = 0.31539156525252005f * (2.0f * zz - xx - yy);
    o[7] = -1.0925484305920792f * dx * dz;
    o[8] = 0.5462742152960396f * (xx - yy);
    o[9] = -0.5900435899266435f * dy * (3.0f * xx - yy);
    o[10] = 2.890611442640554f * dx * dy * dz;
    o[11] = -0.4570457994644658f * dy * (4.0f * zz - xx - yy);
    o[12] = 0.3731763325901154f * dz * (2.0f * zz - 3.0f * xx - 3.0f * yy);
    o[13] = -0.4570457994644658f * dx * (4.0f * zz - xx - yy);
    o[14] = 1.445305721320277f * dz * (xx - yy);
    o[15] = -0.5900435899266435f * dx * (xx - 3.0f * yy);
}

// One thread per background sample s = r * NB + j.
__global__ void k_bg_encode(int64_t R, int NB, const float* __restrict__ center, const float* __restrict__ ray_unit,
                            const float* __restrict__ dists, const float* __restrict__ app_table,
                            const int32_t* __restrict__ app_idx, int app_dim, __half* __restrict__ X,
                            __half* __restrict__ X_lo, int ldx, int x_cols, __half* __restrict__ T,
                            __half* __restrict__ T_lo, int ldt, int t_cols) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= R * NB) return;
    const int64_t r = s / NB;
    // The point, its normalisation and the phases are formed in double precision: at the
    // highest frequency (2^9 pi) an FP32 rounding of q alone moves the phase by ~2e-4,
    // which the first layers' weight gradients amplify past 1e-3.  Each phase is reduced
    // to [-pi, pi] in double and only then evaluated in FP32 (|error| ~1e-7).
    const double t = dists[s];
    double p[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) p[i] = (double)center[3 * r + i] + (double)ray_unit[3 * r + i] * t;
    const double nrm = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    const double q[4] = {p[0] / nrm, p[1] / nrm, p[2] / nrm, 1.0 / nrm};
    // row: q (4) | per channel c: sin(q_c f_k) k < 10, cos(q_c f_k) k < 10 | 1 | zeros
    float buf[96];
#pragma unroll
    for (int c = 0; c < 4; ++c) buf[c] = (float)q[c];
    constexpr double kTwoPi = 6.283185307179586476925;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        // 2^k pi as the reference builds it in float32 (2^k times float32(pi), exact)
        const double base = q[c] * (double)3.14159265358979323846f;
#pragma unroll
        for (int k = 0; k < BG_LEVELS; ++k) {
            const double ph = ldexp(base, k);
            const float red = (float)(ph - kTwoPi * rint(ph * (1.0 / kTwoPi)));
            float sv, cv;
            sincosf(red, &sv, &cv);
            buf[4 + 20 * c + k] = sv;
            buf[4 + 20 * c + BG_LEVELS + k] = cv;
        }
    }
    buf[BG_ENC_COLS] = 1.0f;                      // the bias column
#pragma unroll
    for (int c = BG_ENC_COLS + 1; c < 96; ++c) buf[c] = 0.0f;
    __half* xr = X + s * (int64_t)ldx;
#pragma unroll
    for (int g = 0; g < 12; ++g)
        if (8 * g < x_cols) store_half8(xr + 8 * g, buf + 8 * g);
    const float zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int c0 = 96; c0 < x_cols; c0 += 8) store_half8(xr + c0, zero8);
    if (X_lo) {
        __half* xl = X_lo + s * (int64_t)ldx;
#pragma unroll
        for (int g = 0; g < 12; ++g)
            if (8 * g < x_cols) store_half8_lo(xl + 8 * g, buf + 8 * g);
        for (int c0 = 96; c0 < x_cols; c0 += 8) store_half8(xl + c0, zero8);
    }
    // colour-input tail: SH(d) 16 | app | 1 | zeros
    float o[16];
    sh16(ray_unit[3 * r], ray_unit[3 * r + 1], ray_unit[3 * r + 2], o);
    __half* tr = T + s * (int64_t)ldt;
    __half* tl = T_lo ? T_lo + s * (int64_t)ldt : nullptr;
    const float* a = (app_table && app_dim > 0) ? app_table + (int64_t)app_idx[r] * app_dim : nullptr;
    for (int c0 = 0; c0 < t_cols; c0 += 8) {
        float v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int c = c0 + i;
            float x = 0.0f;
            if (c < 16) {
#pragma unroll
                for (int k = 0; k < 16; ++k)
                    if (k == c) x = o[k];
            } else if (c < 16 + app_dim) {
                x = a ? a[c - 16] : 0.0f;
            } else if (c == 16 + app_dim) {
                x = 1.0f;
            }
            v[i] = x;
        }
        store_half8(tr + c0, v);
        if (tl) store_half8_lo(tl + c0, v);
    }
}

// sigma = softplus(h . w + b), one warp per row; lane j owns columns [8j, 8j + 8) of H <= 256
__global__ void __launch_bounds__(256) k_bg_density(int64_t M, const __half* __restrict__ Hm,
                                                    const __half* __restrict__ Hm_lo, int ldh, int H,
                                                    const float* __restrict__ w, const float* __restrict__ bias,
                                                    float* __restrict__ sigma) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float b = bias[0];
    float wl[8];
    const bool act = 8 * lane < H;
#pragma unroll
    for (int i = 0; i < 8; ++i) wl[i] = act ? w[8 * lane + i] : 0.0f;
    for (int64_t r = warp; r < M; r += nwarps) {
        float acc = 0.0f;
        if (act) {
            float h[8];
            if (Hm_lo) {                               // the low half first (smaller addends)
                load_half8(Hm_lo + r * (int64_t)ldh + 8 * lane, h);
#pragma unroll
                for (int i = 0; i < 8; ++i) acc = fmaf(h[i], wl[i], acc);
            }
            load_half8(Hm + r * (int64_t)ldh + 8 * lane, h);
#pragma unroll
            for (int i = 0; i < 8; ++i) acc = fmaf(h[i], wl[i], acc);
        }
        acc = warp_sum(acc);
        if (lane == 0) {
            const float z = acc + b;
            sigma[r] = z > 20.0f ? z : log1pf(expf(z));
        }
    }
}

}  // namespace
}  // namespace gbsdf

using namespace gbsdf;

extern "C" int gbsdf_bg_encode(int64_t R, int32_t NB, const float* center, const float* ray_unit,
                               const float* dists, const float* app_table, const int32_t* app_idx, int32_t app_dim,
                               void* X, void* X_lo, int32_t ldx, int32_t x_cols, void* T, void* T_lo, int32_t ldt,
                               int32_t t_cols, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(R >= 0 && NB >= 0, "negative sizes");
    if (R == 0 || NB == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(center && ray_unit && dists && X && T, "NULL pointer");
    GBSDF_CHECK_ARG(x_cols % 8 == 0 && x_cols > BG_ENC_COLS && ldx >= x_cols && ldx % 8 == 0,
                    "encoding columns %d (needs > 84, multiple of 8)", x_cols);
    GBSDF_CHECK_ARG(app_dim >= 0 && t_cols % 8 == 0 && t_cols >= 17 + app_dim && ldt >= t_cols && ldt % 8 == 0,
                    "colour-input tail of %d columns for app_dim %d", t_cols, app_dim);
    GBSDF_CHECK_ARG(app_dim == 0 || (app_table && app_idx), "appearance table / index missing");
    GBSDF_CHECK_ARG(aligned(X, 16) && aligned(T, 16), "X / T must be 16-byte aligned");
    GBSDF_CHECK_ARG((!X_lo || aligned(X_lo, 16)) && (!T_lo || aligned(T_lo, 16)), "X_lo / T_lo alignment");
    const int64_t n = R * NB;
    k_bg_encode<<<(unsigned)((n + 127) / 128), 128, 0, as_stream(stream)>>>(
        R, NB, center, ray_unit, dists, app_table, app_idx, app_dim, (__half*)X, (__half*)X_lo, ldx, x_cols,
        (__half*)T, (__half*)T_lo, ldt, t_cols);
    return launch_status("bg_encode");
}

extern "C" int gbsdf_bg_density(int64_t M, const void* Hm, const void* Hm_lo, int32_t ldh, int32_t H, const float* w,
                                const float* b, float* sigma, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(M >= 0, "M < 0");
    if (M == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(Hm && w && b && sigma, "NULL pointer");
    GBSDF_CHECK_ARG(H % 8 == 0 && H <= 256 && ldh >= H && ldh % 8 == 0 && aligned(Hm, 16), "hidden width %d", H);
    GBSDF_CHECK_ARG(!Hm_lo || aligned(Hm_lo, 16), "H_lo alignment");
    int64_t blocks = (M + 7) / 8;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_bg_density<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(M, (const __half*)Hm, (const __half*)Hm_lo, ldh, H,
                                                                   w, b, sigma);
    return launch_status("bg_density");
}
