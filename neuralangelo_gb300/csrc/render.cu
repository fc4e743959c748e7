// NeuS alpha and front-to-back compositing weights, plain FP32 drop-in ops.
//
// gbsdf_neus_alpha_*      : Model.compute_neus_alphas + _get_iter_cos
//                           (projects/neuralangelo/model.py:275-298)
// gbsdf_composite_weights*: render.alpha_compositing_weights
//                           (projects/nerf/utils/render.py:87-99)
#include "common.cuh"

namespace gbsdf {

// iter_cos = -(relu(-c/2 + 1/2) (1 - a) + relu(-c) a),  a = min(progress / anneal_end, 1)
__device__ __forceinline__ float iter_cos_fwd(float c, float a) {
    return -(fmaxf(-c * 0.5f + 0.5f, 0.0f) * (1.0f - a) + fmaxf(-c, 0.0f) * a);
}
// d iter_cos / d c (relu' = 1 for a strictly positive argument, as torch)
__device__ __forceinline__ float iter_cos_grad(float c, float a) {
    return (c < 1.0f ? 0.5f * (1.0f - a) : 0.0f) + (c < 0.0f ? a : 0.0f);
}

struct AlphaTerms {
    float ic, intv, ep, en, P, Q, alpha_raw;
};

__device__ __forceinline__ AlphaTerms alpha_terms(float sdf, float cosv, float intv, float inv_s, float a) {
    AlphaTerms t;
    t.ic = iter_cos_fwd(cosv, a);
    t.intv = intv;
    t.ep = sdf - t.ic * intv * 0.5f;
    t.en = sdf + t.ic * intv * 0.5f;
    t.P = sigmoidf_(t.ep * inv_s);
    t.Q = sigmoidf_(t.en * inv_s);
    t.alpha_raw = (t.P - t.Q) / (t.P + 1e-5f);
    return t;
}

__global__ void k_neus_alpha_fwd(int64_t R, int64_t N, const float* __restrict__ ray, const float* __restrict__ sdf,
                                 const float* __restrict__ grad, const float* __restrict__ dists,
                                 const float* __restrict__ far, const float* __restrict__ s_var, float a,
                                 float* __restrict__ alpha) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= R * N) return;
    const int64_t r = i / N, n = i % N;
    const float inv_s = expf(*s_var);
    const float cosv = ray[3 * r] * grad[3 * i] + ray[3 * r + 1] * grad[3 * i + 1] + ray[3 * r + 2] * grad[3 * i + 2];
    const float dnext = (n + 1 < N) ? dists[i + 1] : far[r];
    const AlphaTerms t = alpha_terms(sdf[i], cosv, dnext - dists[i], inv_s, a);
    alpha[i] = fminf(fmaxf(t.alpha_raw, 0.0f), 1.0f);
}

__global__ void k_neus_alpha_bwd(int64_t R, int64_t N, const float* __restrict__ ray, const float* __restrict__ sdf,
                                 const float* __restrict__ grad, const float* __restrict__ dists,
                                 const float* __restrict__ far, const float* __restrict__ s_var, float a,
                                 const float* __restrict__ d_alpha, float* __restrict__ d_sdf,
                                 float* __restrict__ d_grad, float* __restrict__ d_s_var) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float ds = 0.0f;
    if (i < R * N) {
        const int64_t r = i / N, n = i % N;
        const float inv_s = expf(*s_var);
        const float rx = ray[3 * r], ry = ray[3 * r + 1], rz = ray[3 * r + 2];
        const float cosv = rx * grad[3 * i] + ry * grad[3 * i + 1] + rz * grad[3 * i + 2];
        const float dnext = (n + 1 < N) ? dists[i + 1] : far[r];
        const AlphaTerms t = alpha_terms(sdf[i], cosv, dnext - dists[i], inv_s, a);
        // clamp(0, 1) passes the gradient on the closed interval (torch clamp_backward)
        float g = (t.alpha_raw >= 0.0f && t.alpha_raw <= 1.0f) ? d_alpha[i] : 0.0f;
        const float den = t.P + 1e-5f;
        const float dP = g * (t.Q + 1e-5f) / (den * den);
        const float dQ = -g / den;
        const float dep = dP * t.P * (1.0f - t.P);   // d/d(ep*inv_s)
        const float den_ = dQ * t.Q * (1.0f - t.Q);
        const float d_ep = dep * inv_s, d_en = den_ * inv_s;
        ds = (dep * t.ep + den_ * t.en) * inv_s;       // d/ds_var through inv_s = exp(s_var)
        const float d_sdf_v = d_ep + d_en;
        const float d_ic = (d_en - d_ep) * t.intv * 0.5f;
        const float d_cos = d_ic * iter_cos_grad(cosv, a);
        d_sdf[i] = d_sdf_v;
        d_grad[3 * i] = d_cos * rx;
        d_grad[3 * i + 1] = d_cos * ry;
        d_grad[3 * i + 2] = d_cos * rz;
    }
    ds = warp_sum(ds);
    if ((threadIdx.x & 31) == 0 && ds != 0.0f) atomicAdd(d_s_var, ds);
}

// One warp per ray, 32 samples per chunk; transmittance T_i = prod_{j<i} (1 - a_j)
// by a multiplicative warp scan carried across chunks.
__global__ void k_weights_fwd(int64_t R, int64_t N, const float* __restrict__ alpha, float* __restrict__ w) {
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= R) return;
    float carry = 1.0f;
    for (int64_t base = 0; base < N; base += 32) {
        const int64_t n = base + lane;
        const float a = n < N ? alpha[r * N + n] : 0.0f;
        float p = 1.0f - a;   // inclusive product scan
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float q = __shfl_up_sync(0xffffffffu, p, o);
            if (lane >= o) p *= q;
        }
        float excl = __shfl_up_sync(0xffffffffu, p, 1);
        if (lane == 0) excl = 1.0f;
        if (n < N) w[r * N + n] = a * (carry * excl);
        carry *= __shfl_sync(0xffffffffu, p, 31);
    }
}

// dL/da_k = T_k (dw_k - S_{k+1}),  S_k = dw_k a_k + (1 - a_k) S_{k+1},  S_N = 0
// (derivation without division by 1 - a_k, stable at a = 1).  T is recomputed
// chunk by chunk into d_alpha first, then the reverse pass overwrites it.
__global__ void k_weights_bwd(int64_t R, int64_t N, const float* __restrict__ alpha, const float* __restrict__ dw,
                              float* __restrict__ d_alpha) {
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= R) return;
    float carry = 1.0f;
    for (int64_t base = 0; base < N; base += 32) {
        const int64_t n = base + lane;
        const float a = n < N ? alpha[r * N + n] : 0.0f;
        float p = 1.0f - a;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float q = __shfl_up_sync(0xffffffffu, p, o);
            if (lane >= o) p *= q;
        }
        float excl = __shfl_up_sync(0xffffffffu, p, 1);
        if (lane == 0) excl = 1.0f;
        if (n < N) d_alpha[r * N + n] = carry * excl;   // T_n
        carry *= __shfl_sync(0xffffffffu, p, 31);
    }
    __syncwarp();
    float S = 0.0f;   // S_{first sample of the next chunk}
    const int64_t last = ((N + 31) / 32 - 1) * 32;
    for (int64_t base = last; base >= 0; base -= 32) {
        const int64_t n = base + lane;
        const float a = n < N ? alpha[r * N + n] : 0.0f;
        const float g = n < N ? dw[r * N + n] : 0.0f;
        float A = g * a, B = 1.0f - a;   // map s -> A + B s, composed right-to-left
        if (n >= N) { A = 0.0f; B = 1.0f; }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float A2 = __shfl_down_sync(0xffffffffu, A, o);
            const float B2 = __shfl_down_sync(0xffffffffu, B, o);
            if (lane + o < 32) {
                A = A + B * A2;
                B = B * B2;
            }
        }
        const float Sk = A + B * S;                                   // S_n
        float Snext = __shfl_down_sync(0xffffffffu, Sk, 1);          // S_{n+1}
        if (lane == 31) Snext = S;
        if (n < N) {
            const float T = d_alpha[r * N + n];
            d_alpha[r * N + n] = T * (g - Snext);
        }
        S = __shfl_sync(0xffffffffu, Sk, 0);
    }
}

}  // namespace gbsdf

using namespace gbsdf;

static float anneal_ratio(float progress, float anneal_end) {
    const float a = progress / anneal_end;
    return a < 1.0f ? a : 1.0f;
}

extern "C" int gbsdf_neus_alpha_fwd(int64_t R, int64_t N, const float* ray_unit, const float* sdf, const float* grad,
                                    const float* dists, const float* far, const float* s_var, float progress,
                                    float anneal_end, float* alpha, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(R >= 0 && N >= 0, "negative size");
    if (R * N == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(ray_unit && sdf && grad && dists && far && s_var && alpha, "NULL pointer");
    GBSDF_CHECK_ARG(anneal_end > 0.0f, "anneal_end must be > 0");
    const int64_t tot = R * N;
    k_neus_alpha_fwd<<<(unsigned)((tot + 255) / 256), 256, 0, as_stream(stream)>>>(
        R, N, ray_unit, sdf, grad, dists, far, s_var, anneal_ratio(progress, anneal_end), alpha);
    return launch_status("neus_alpha_fwd");
}

extern "C" int gbsdf_neus_alpha_bwd(int64_t R, int64_t N, const float* ray_unit, const float* sdf, const float* grad,
                                    const float* dists, const float* far, const float* s_var, float progress,
                                    float anneal_end, const float* d_alpha, float* d_sdf, float* d_grad,
                                    float* d_s_var, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(R >= 0 && N >= 0, "negative size");
    if (R * N == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(ray_unit && sdf && grad && dists && far && s_var && d_alpha && d_sdf && d_grad && d_s_var,
                    "NULL pointer");
    GBSDF_CHECK_ARG(anneal_end > 0.0f, "anneal_end must be > 0");
    const int64_t tot = R * N;
    k_neus_alpha_bwd<<<(unsigned)((tot + 255) / 256), 256, 0, as_stream(stream)>>>(
        R, N, ray_unit, sdf, grad, dists, far, s_var, anneal_ratio(progress, anneal_end), d_alpha, d_sdf, d_grad,
        d_s_var);
    return launch_status("neus_alpha_bwd");
}

extern "C" int gbsdf_composite_weights_fwd(int64_t R, int64_t N, const float* alpha, float* weights, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(R >= 0 && N >= 0, "negative size");
    if (R * N == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(alpha && weights, "NULL pointer");
    const int64_t threads = R * 32;
    k_weights_fwd<<<(unsigned)((threads + 255) / 256), 256, 0, as_stream(stream)>>>(R, N, alpha, weights);
    return launch_status("composite_weights_fwd");
}

extern "C" int gbsdf_composite_weights_bwd(int64_t R, int64_t N, const float* alpha, const float* d_weights,
                                           float* d_alpha, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(R >= 0 && N >= 0, "negative size");
    if (R * N == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(alpha && d_weights && d_alpha, "NULL pointer");
    GBSDF_CHECK_ARG(d_alpha != alpha && d_alpha != d_weights, "d_alpha must not alias the inputs");
    const int64_t threads = R * 32;
    k_weights_bwd<<<(unsigned)((threads + 255) / 256), 256, 0, as_stream(stream)>>>(R, N, alpha, d_weights, d_alpha);
    return launch_status("composite_weights_bwd");
}
