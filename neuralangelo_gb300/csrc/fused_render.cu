// Fused per-ray rendering forward + backward, the colour head, and the
// appearance-embedding gradient of the fused training step.
//
// gbsdf_render_fused : NeuS alpha (projects/neuralangelo/model.py:275-298),
//   front-to-back compositing with FP32 log-space transmittance
//   (projects/nerf/utils/render.py:87-112) of the object samples followed by the
//   background NeRF's (model.py:129-141, render.py:68-84), L1 colour x3, eikonal and curvature
//   losses (projects/neuralangelo/trainer.py:40-52, utils/misc.py:74-89) and the
//   analytic backward of all of it, one warp per ray.
// gbsdf_rgb_head_*   : last colour layer 256 -> 3 + sigmoid (modules.py:215,
//   nerf_util.py:187-196) forward and backward.
// gbsdf_app_grad     : gradient of the per-image appearance embedding
//   (model.py:215-230 gathers Embedding(idx) per ray).
#include "dense.cuh"

namespace gbsdf {

constexpr int RENDER_WARPS = 8;
constexpr int MAX_RAY_SAMPLES = 512;

__device__ __forceinline__ float iter_cos_f(float c, float a) {
    return -(fmaxf(-c * 0.5f + 0.5f, 0.0f) * (1.0f - a) + fmaxf(-c, 0.0f) * a);
}
__device__ __forceinline__ float iter_cos_g(float c, float a) {
    return (c < 1.0f ? 0.5f * (1.0f - a) : 0.0f) + (c < 0.0f ? a : 0.0f);
}
__device__ __forceinline__ float signf_(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

__global__ void __launch_bounds__(RENDER_WARPS * 32) k_render_fused(gbsdf_render_args p) {
    __shared__ float s_alpha[RENDER_WARPS][MAX_RAY_SAMPLES];
    __shared__ float s_T[RENDER_WARPS][MAX_RAY_SAMPLES];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r = (int64_t)blockIdx.x * RENDER_WARPS + wib;
    if (r >= p.R) return;
    const int64_t beg = p.S > 0 ? r * p.S : p.ray_offsets[r];
    const int64_t end = p.S > 0 ? beg + p.S : p.ray_offsets[r + 1];
    const int n = (int)(end - beg);
    const int nb = p.n_bg;                     // background samples follow the object samples
    const int ntot = n + nb;
    // the loss scale, anneal ratio and curvature weight: device scalars when given
    const float loss_scale = p.dyn ? p.dyn[0] : p.loss_scale;
    const float anneal = p.dyn ? p.dyn[1] : p.anneal;
    const float w_curv = p.dyn ? p.dyn[2] : p.w_curv;
    if (ntot > MAX_RAY_SAMPLES) {   // longer rays do not fit the per-warp buffers: report, skip
        if (lane == 0 && p.err) atomicCAS(p.err, 0, 2);
        return;
    }
    float* sa = s_alpha[wib];
    float* sT = s_T[wib];
    const float inv_s = expf(p.s_var[0]);
    const float rx = p.ray_unit[3 * r], ry = p.ray_unit[3 * r + 1], rz = p.ray_unit[3 * r + 2];
    const bool inside = !(p.outside && p.outside[r]);
    const float far = p.far[r];

    // ---------------- forward: alpha, log-space transmittance, colour ----------------
    float carry = 0.0f;   // sum of log(1 - alpha) over earlier chunks
    float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
    float op = 0.0f, gc0 = 0.0f, gc1 = 0.0f, gc2 = 0.0f, dc = 0.0f;   // evaluation composites
    float eik_sum = 0.0f, curv_sum = 0.0f;
    for (int base = 0; base < ntot; base += 32) {
        const int k = base + lane;
        float a = 0.0f, la = 0.0f;
        if (k >= n && k < ntot) {
            // background sample: alpha = 1 - exp(-sigma dt), log(1 - alpha) = -sigma dt
            const int64_t q = r * nb + (k - n);
            const float dnext = (k + 1 < ntot) ? p.bg_dists[q + 1] : 1e10f;
            la = -(p.bg_sigma[q] * (dnext - p.bg_dists[q]));
            a = -expm1f(la);
        }
        if (k < n) {
            const int64_t s = beg + k;
            const float gx = p.grad[3 * s], gy = p.grad[3 * s + 1], gz = p.grad[3 * s + 2];
            const float cosv = rx * gx + ry * gy + rz * gz;
            const float dnext = (k + 1 < n) ? p.dists[s + 1] : far;
            const float intv = dnext - p.dists[s];
            const float ic = iter_cos_f(cosv, anneal);
            const float sdf = p.sdf[s];
            const float P = 1.0f / (1.0f + expf(-(sdf - ic * intv * 0.5f) * inv_s));
            const float Q = 1.0f / (1.0f + expf(-(sdf + ic * intv * 0.5f) * inv_s));
            a = fminf(fmaxf((P - Q) / (P + 1e-5f), 0.0f), 1.0f);
            la = log1pf(-a);
            if (inside && !p.forward_only) {       // losses: training only (hess may be NULL otherwise)
                const float e = sqrtf(gx * gx + gy * gy + gz * gz) - 1.0f;
                const float ev = e * e;
                if (isfinite(ev)) eik_sum += ev;
                const float lap = fabsf(p.hess[3 * s] + p.hess[3 * s + 1] + p.hess[3 * s + 2]);
                if (isfinite(lap)) curv_sum += lap;
            }
        }
        // inclusive prefix sum of log(1 - alpha) across the warp (-inf once alpha = 1)
        float incl = la;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        float excl = __shfl_up_sync(0xffffffffu, incl, 1);
        if (lane == 0) excl = 0.0f;
        const float T = expf(carry + excl);   // prod_{j<k} (1 - a_j)
        if (k < ntot) {
            sa[k] = a;
            sT[k] = T;
            const float w = a * T;
            const float* cp;
            if (k < n) {
                const int64_t s = beg + k;
                if (p.weights) p.weights[s] = w;
                cp = p.rgbs + 3 * s;
                op += w;
                gc0 = fmaf(w, p.grad[3 * s], gc0);
                gc1 = fmaf(w, p.grad[3 * s + 1], gc1);
                gc2 = fmaf(w, p.grad[3 * s + 2], gc2);
                dc = fmaf(w, p.dists[s], dc);
            } else {
                const int64_t q = r * nb + (k - n);
                if (p.bg_weights) p.bg_weights[q] = w;
                cp = p.bg_rgbs + 3 * q;
                dc = fmaf(w, p.bg_dists[q], dc);
            }
            c0 = fmaf(w, cp[0], c0);
            c1 = fmaf(w, cp[1], c1);
            c2 = fmaf(w, cp[2], c2);
        }
        carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    c0 = warp_sum(c0);
    c1 = warp_sum(c1);
    c2 = warp_sum(c2);
    eik_sum = warp_sum(eik_sum);
    curv_sum = warp_sum(curv_sum);
    if (p.out_opacity || p.out_gradient || p.out_dist) {
        op = warp_sum(op);
        gc0 = warp_sum(gc0);
        gc1 = warp_sum(gc1);
        gc2 = warp_sum(gc2);
        dc = warp_sum(dc);
        if (lane == 0) {
            if (p.out_opacity) p.out_opacity[r] = op;
            if (p.out_gradient) {
                p.out_gradient[3 * r] = gc0;
                p.out_gradient[3 * r + 1] = gc1;
                p.out_gradient[3 * r + 2] = gc2;
            }
            if (p.out_dist) p.out_dist[r] = dc;
        }
    }
    if (p.forward_only) {
        if (lane == 0) {
            p.rgb[3 * r] = c0;
            p.rgb[3 * r + 1] = c1;
            p.rgb[3 * r + 2] = c2;
        }
        return;
    }
    const float t0 = p.target[3 * r], t1 = p.target[3 * r + 1], t2 = p.target[3 * r + 2];
    if (lane == 0) {
        p.rgb[3 * r] = c0;
        p.rgb[3 * r + 1] = c1;
        p.rgb[3 * r + 2] = c2;
        const double l1 = (double)fabsf(c0 - t0) + (double)fabsf(c1 - t1) + (double)fabsf(c2 - t2);
        atomicAdd(&p.loss_sums[0], l1);
        atomicAdd(&p.loss_sums[1], (double)eik_sum);
        atomicAdd(&p.loss_sums[2], (double)curv_sum);
    }
    __syncwarp();
    // d L / d rgb (L1Loss mean x 3, loss-scaled)
    const float gsc = loss_scale * p.w_render * p.l1_scale;
    const float dr0 = gsc * signf_(c0 - t0), dr1 = gsc * signf_(c1 - t1), dr2 = gsc * signf_(c2 - t2);
    const float eik_c = loss_scale * p.w_eik * p.mean_scale * 2.0f;
    const float curv_c = loss_scale * w_curv * p.mean_scale;

    // ---------------- backward (reverse chunks) ----------------
    float Snext = 0.0f;    // S of the first sample after the current chunk
    float ds_acc = 0.0f;
    const int last = ((ntot + 31) / 32 - 1) * 32;
    for (int base = last; base >= 0; base -= 32) {
        const int k = base + lane;
        const bool live = k < ntot;
        float a = 0.0f, T = 0.0f, dw = 0.0f;
        int64_t s = beg + k;
        const int64_t q = r * nb + (k - n);      // background index when k >= n
        if (live) {
            a = sa[k];
            T = sT[k];
            const float* cp = k < n ? p.rgbs + 3 * s : p.bg_rgbs + 3 * q;
            float* dcp = k < n ? p.d_rgbs + 3 * s : p.d_bg_rgbs + 3 * q;
            dw = dr0 * cp[0] + dr1 * cp[1] + dr2 * cp[2];
            const float w = a * T;
            dcp[0] = dr0 * w;
            dcp[1] = dr1 * w;
            dcp[2] = dr2 * w;
        }
        // S_k = dw_k a_k + (1 - a_k) S_{k+1}: suffix scan of affine maps
        float A = live ? dw * a : 0.0f, B = live ? 1.0f - a : 1.0f;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float A2 = __shfl_down_sync(0xffffffffu, A, o);
            const float B2 = __shfl_down_sync(0xffffffffu, B, o);
            if (lane + o < 32) {
                A = A + B * A2;
                B = B * B2;
            }
        }
        const float Sk = A + B * Snext;
        float Sk1 = __shfl_down_sync(0xffffffffu, Sk, 1);
        if (lane == 31) Sk1 = Snext;
        if (live && k >= n) {
            // background: d sigma = d alpha dt (1 - alpha); softplus' = 1 - exp(-sigma)
            const float d_alpha = T * (dw - Sk1);
            const float dnext = (k + 1 < ntot) ? p.bg_dists[q + 1] : 1e10f;
            const float dt = dnext - p.bg_dists[q];
            const float sig = p.bg_sigma[q];
            const float d_sig = d_alpha * dt * expf(-sig * dt);
            const float d_pre = d_sig * -expm1f(-sig);
            reinterpret_cast<__half*>(p.d_bg_pre)[q * (int64_t)p.ld_d_bg_pre] = __float2half_rn(d_pre);
        } else if (live) {
            float d_alpha = T * (dw - Sk1);
            // NeuS alpha backward (recomputed terms)
            const float gx = p.grad[3 * s], gy = p.grad[3 * s + 1], gz = p.grad[3 * s + 2];
            const float cosv = rx * gx + ry * gy + rz * gz;
            const float dnext = (k + 1 < n) ? p.dists[s + 1] : far;
            const float intv = dnext - p.dists[s];
            const float ic = iter_cos_f(cosv, anneal);
            const float sdf = p.sdf[s];
            const float ep = sdf - ic * intv * 0.5f, en = sdf + ic * intv * 0.5f;
            const float P = 1.0f / (1.0f + expf(-ep * inv_s));
            const float Q = 1.0f / (1.0f + expf(-en * inv_s));
            const float raw = (P - Q) / (P + 1e-5f);
            if (!(raw >= 0.0f && raw <= 1.0f)) d_alpha = 0.0f;
            const float den = P + 1e-5f;
            const float dP = d_alpha * (Q + 1e-5f) / (den * den);
            const float dQ = -d_alpha / den;
            const float dep = dP * P * (1.0f - P), den_ = dQ * Q * (1.0f - Q);
            ds_acc += (dep * ep + den_ * en) * inv_s;
            const float d_sdf = (dep + den_) * inv_s;
            const float d_cos = (den_ - dep) * inv_s * intv * 0.5f * iter_cos_g(cosv, anneal);
            float dgx = d_cos * rx, dgy = d_cos * ry, dgz = d_cos * rz;
            float dh = 0.0f;
            if (inside) {
                const float len = sqrtf(gx * gx + gy * gy + gz * gz);
                const float e = len - 1.0f;
                if (isfinite(e * e) && len > 0.0f) {
                    const float c = eik_c * e / len;
                    dgx += c * gx; dgy += c * gy; dgz += c * gz;
                }
                const float lap = p.hess[3 * s] + p.hess[3 * s + 1] + p.hess[3 * s + 2];
                if (isfinite(lap)) dh = curv_c * signf_(lap);
            }
            p.d_sdf[s] = d_sdf;
            p.d_grad[3 * s] = dgx;
            p.d_grad[3 * s + 1] = dgy;
            p.d_grad[3 * s + 2] = dgz;
            p.d_hess[3 * s] = dh;
            p.d_hess[3 * s + 1] = dh;
            p.d_hess[3 * s + 2] = dh;
        }
        Snext = __shfl_sync(0xffffffffu, Sk, 0);
    }
    ds_acc = warp_sum(ds_acc);
    if (lane == 0 && ds_acc != 0.0f) atomicAdd(p.d_s_var, ds_acc);
}


// rgbs = sigmoid(Y W^T + b) for the 3 colour channels; one thread per row (cheaper here than a
// warp per row, which needs three warp reductions per row); W [3, H]
__global__ void k_rgb_head_fwd(int64_t Ns, const __half* __restrict__ Y, int ldy, int H, const float* __restrict__ W,
                               const float* __restrict__ b, float* __restrict__ rgbs) {
    __shared__ float w_s[3 * 256];
    for (int i = threadIdx.x; i < 3 * H; i += blockDim.x) w_s[(i / H) * 256 + i % H] = W[i];
    __syncthreads();
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= Ns) return;
    float a0 = b[0], a1 = b[1], a2 = b[2];
    const __half* y = Y + s * ldy;
    for (int j = 0; j < H; j += 8) {
        const uint4 u = *reinterpret_cast<const uint4*>(y + j);
        const __half2* h = reinterpret_cast<const __half2*>(&u);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 f = __half22float2(h[i]);
            const int c = j + 2 * i;
            a0 = fmaf(w_s[c], f.x, fmaf(w_s[c + 1], f.y, a0));
            a1 = fmaf(w_s[256 + c], f.x, fmaf(w_s[256 + c + 1], f.y, a1));
            a2 = fmaf(w_s[512 + c], f.x, fmaf(w_s[512 + c + 1], f.y, a2));
        }
    }
    rgbs[3 * s] = sigmoidf_(a0);
    rgbs[3 * s + 1] = sigmoidf_(a1);
    rgbs[3 * s + 2] = sigmoidf_(a2);
}

// d_pre = d_rgb * rgb (1 - rgb);  dZ = (d_pre W) * [Y > 0];  d_b += d_pre;  d_W += d_pre^T Y.
// One warp per row at a time, the next row's loads issued before this row's work (two rows
// in flight per warp): lane j owns hidden columns [8j, 8j + 8) (H <= 256), so every row's
// activations and gradients move as coalesced 512-byte accesses; W [3, H] sits in shared
// memory.  The head's weight gradient is accumulated per lane (3 x 8 registers), summed over
// the block in shared memory and added to d_W once per block (the grid holds only as many
// blocks as are resident, so each of the 3 x H addresses takes one atomic per block).
constexpr int HEAD_BWD_BLOCKS_PER_SM = 3;
__device__ __forceinline__ void head_row_load(int64_t s, int64_t Ns, const __half* __restrict__ Y, int ldy, int c0,
                                              bool act, const float* __restrict__ rgbs,
                                              const float* __restrict__ d_rgbs, uint4& u, float* g) {
    const bool live = s < Ns;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float r = live ? rgbs[3 * s + k] : 0.0f;
        g[k] = live ? d_rgbs[3 * s + k] * r * (1.0f - r) : 0.0f;
    }
    u = (live && act) ? *reinterpret_cast<const uint4*>(Y + s * ldy + c0) : make_uint4(0, 0, 0, 0);
}

__global__ void __launch_bounds__(256, HEAD_BWD_BLOCKS_PER_SM) k_rgb_head_bwd(int64_t Ns, const __half* __restrict__ Y, int ldy, int H,
                                                         const float* __restrict__ W, const float* __restrict__ rgbs,
                                                         const float* __restrict__ d_rgbs, __half* __restrict__ d_pre,
                                                         __half* __restrict__ dZ, __half* __restrict__ dZlo,
                                                         float* __restrict__ d_b, float* __restrict__ d_W) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int c0 = lane * 8;
    const bool act = c0 < H;
    __shared__ __align__(16) float w_s[3][256];
    __shared__ float dw_s[3 * 256 + 3];                 // the block's d_W, then its d_b
    for (int i = threadIdx.x; i < 3 * 256; i += blockDim.x) {
        const int k = i >> 8, c = i & 255;
        w_s[k][c] = c < H ? W[k * H + c] : 0.0f;
    }
    for (int i = threadIdx.x; i < 3 * 256 + 3; i += blockDim.x) dw_s[i] = 0.0f;
    __syncthreads();
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    float dw[3][8];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int i = 0; i < 8; ++i) dw[k][i] = 0.0f;
    uint4 un;
    float gn[3];
    head_row_load(w0, Ns, Y, ldy, c0, act, rgbs, d_rgbs, un, gn);
    for (int64_t s = w0; s < Ns; s += nw) {
        const uint4 u = un;
        const float g0 = gn[0], g1 = gn[1], g2 = gn[2];
        head_row_load(s + nw, Ns, Y, ldy, c0, act, rgbs, d_rgbs, un, gn);
        if (lane == 0) {
            if (d_pre) {
                __half2 hp[4] = {__floats2half2_rn(g0, g1), __floats2half2_rn(g2, 0.f), __floats2half2_rn(0.f, 0.f),
                                 __floats2half2_rn(0.f, 0.f)};
                *reinterpret_cast<uint4*>(d_pre + s * 8) = *reinterpret_cast<const uint4*>(hp);
            }
            s0 += g0;
            s1 += g1;
            s2 += g2;
        }
        if (act) {
            const __half2* h = reinterpret_cast<const __half2*>(&u);
            __half2 o[4], ol[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float2 f = __half22float2(h[i]);
                const int c = 2 * i;
                const float2 wa = *reinterpret_cast<const float2*>(&w_s[0][c0 + c]);
                const float2 wb = *reinterpret_cast<const float2*>(&w_s[1][c0 + c]);
                const float2 wc = *reinterpret_cast<const float2*>(&w_s[2][c0 + c]);
                dw[0][c] = fmaf(g0, f.x, dw[0][c]);
                dw[1][c] = fmaf(g1, f.x, dw[1][c]);
                dw[2][c] = fmaf(g2, f.x, dw[2][c]);
                dw[0][c + 1] = fmaf(g0, f.y, dw[0][c + 1]);
                dw[1][c + 1] = fmaf(g1, f.y, dw[1][c + 1]);
                dw[2][c + 1] = fmaf(g2, f.y, dw[2][c + 1]);
                const float v0 = f.x > 0.0f ? g0 * wa.x + g1 * wb.x + g2 * wc.x : 0.0f;
                const float v1 = f.y > 0.0f ? g0 * wa.y + g1 * wb.y + g2 * wc.y : 0.0f;
                o[i] = __floats2half2_rn(v0, v1);
                const float2 r = __half22float2(o[i]);
                ol[i] = __floats2half2_rn(v0 - r.x, v1 - r.y);
            }
            *reinterpret_cast<uint4*>(dZ + s * H + c0) = *reinterpret_cast<const uint4*>(o);
            if (dZlo) *reinterpret_cast<uint4*>(dZlo + s * H + c0) = *reinterpret_cast<const uint4*>(ol);
        }
    }
    if (lane == 0) {
        atomicAdd(&dw_s[3 * 256], s0);
        atomicAdd(&dw_s[3 * 256 + 1], s1);
        atomicAdd(&dw_s[3 * 256 + 2], s2);
    }
    if (d_W && act) {
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int i = 0; i < 8; ++i) atomicAdd(&dw_s[k * 256 + c0 + i], dw[k][i]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * 256 + 3; i += blockDim.x) {
        const float v = dw_s[i];
        if (v == 0.0f) continue;
        if (i >= 3 * 256) atomicAdd(d_b + (i - 3 * 256), v);
        else if (d_W && (i & 255) < H) atomicAdd(d_W + (i >> 8) * H + (i & 255), v);
    }
}

static unsigned head_blocks(int64_t Ns) {
    // eight 256-thread blocks per SM, or fewer when there are fewer rows than warps
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (int64_t)(sms > 0 ? sms : 1) * 8;
    const int64_t need = (Ns + 7) / 8;
    return (unsigned)(need < want ? (need > 0 ? need : 1) : want);
}

// d_app[img(r)] += sum over ray r's samples of d_xc[s, col0:col0+D]; one warp per ray
// D <= 32: lane = (row offset, dimension) with Dp = D rounded up to a power of two, so a
// warp load covers 32 / Dp consecutive rows' D contiguous columns (coalesced); the row
// lanes are then summed with shuffles.  Wider codes loop over the dimensions.
__global__ void k_app_grad(int64_t R, int S, const int64_t* __restrict__ offs, const int* __restrict__ app_idx,
                           const float* __restrict__ d_xc, int ld, int col0, int D, float* __restrict__ d_app) {
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= R) return;
    const int64_t beg = S > 0 ? r * S : offs[r];
    const int64_t end = S > 0 ? beg + S : offs[r + 1];
    if (D <= 32) {
        int Dp = 1;
        while (Dp < D) Dp <<= 1;
        const int per = 32 / Dp, d = lane % Dp, ro = lane / Dp;
        float acc0 = 0.0f, acc1 = 0.0f;
        if (d < D) {
            const float* col = d_xc + col0 + d;
            int64_t s = beg + ro;
            for (; s + per < end; s += 2 * per) {
                acc0 += col[s * ld];
                acc1 += col[(s + per) * ld];
            }
            if (s < end) acc0 += col[s * ld];
        }
        float acc = acc0 + acc1;
        for (int off = Dp; off < 32; off <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
        if (ro == 0 && d < D && acc != 0.0f) atomicAdd(&d_app[(int64_t)app_idx[r] * D + d], acc);
        return;
    }
    for (int d = 0; d < D; ++d) {
        float acc = 0.0f;
        for (int64_t s = beg + lane; s < end; s += 32) acc += d_xc[s * ld + col0 + d];
        acc = warp_sum(acc);
        if (lane == 0 && acc != 0.0f) atomicAdd(&d_app[(int64_t)app_idx[r] * D + d], acc);
    }
}

}  // namespace gbsdf

using namespace gbsdf;

extern "C" size_t gbsdf_render_args_size(void) { return sizeof(gbsdf_render_args); }

extern "C" int gbsdf_render_fused(const gbsdf_render_args* a, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(a != nullptr, "args NULL");
    const gbsdf_render_args& p = *a;
    GBSDF_CHECK_ARG(p.R >= 0, "R < 0");
    if (p.R == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(p.S > 0 || p.ray_offsets, "need S > 0 or ray_offsets");
    GBSDF_CHECK_ARG(p.S <= MAX_RAY_SAMPLES, "S=%d exceeds %d samples per ray", p.S, MAX_RAY_SAMPLES);
    GBSDF_CHECK_ARG(p.ray_unit && p.dists && p.far && p.s_var && p.sdf && p.grad && p.rgbs && p.rgb, "NULL pointer");
    GBSDF_CHECK_ARG(p.forward_only || (p.target && p.hess && p.d_rgbs && p.d_sdf && p.d_grad && p.d_hess &&
                                       p.d_s_var && p.loss_sums),
                    "NULL pointer (training outputs)");
    GBSDF_CHECK_ARG(p.n_bg >= 0 && p.n_bg <= MAX_RAY_SAMPLES, "n_bg %d", p.n_bg);
    GBSDF_CHECK_ARG(p.S == 0 || p.S + p.n_bg <= MAX_RAY_SAMPLES, "S + n_bg = %d exceeds %d samples per ray",
                    p.S + p.n_bg, MAX_RAY_SAMPLES);
    if (p.n_bg > 0) {
        GBSDF_CHECK_ARG(p.bg_dists && p.bg_sigma && p.bg_rgbs, "background sample pointers");
        GBSDF_CHECK_ARG(p.forward_only || (p.d_bg_rgbs && p.d_bg_pre && p.ld_d_bg_pre >= 1),
                        "background gradient pointers");
    }
    const unsigned blocks = (unsigned)((p.R + RENDER_WARPS - 1) / RENDER_WARPS);
    k_render_fused<<<blocks, RENDER_WARPS * 32, 0, as_stream(stream)>>>(p);
    return launch_status("render_fused");
}

extern "C" int gbsdf_rgb_head_fwd(int64_t Ns, const void* Y, int ldy, int H, const float* W, const float* b,
                                  float* rgbs, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(Ns >= 0, "Ns < 0");
    if (Ns == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(Y && W && b && rgbs, "NULL pointer");
    GBSDF_CHECK_ARG(H % 8 == 0 && H <= 256 && H > 0, "hidden width %d", H);
    GBSDF_CHECK_ARG(ldy % 8 == 0 && ldy >= H && aligned(Y, 16), "Y layout");
    k_rgb_head_fwd<<<(unsigned)((Ns + 255) / 256), 256, 0, as_stream(stream)>>>(Ns, (const __half*)Y, ldy, H, W, b,
                                                                                  rgbs);
    return launch_status("rgb_head_fwd");
}

extern "C" int gbsdf_rgb_head_bwd(int64_t Ns, const void* Y, int ldy, int H, const float* W, const float* rgbs,
                                  const float* d_rgbs, void* d_pre, void* dZ, void* dZ_lo, float* d_b, float* d_W,
                                  void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(Ns >= 0, "Ns < 0");
    if (Ns == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(Y && W && rgbs && d_rgbs && dZ && d_b, "NULL pointer");
    GBSDF_CHECK_ARG(H % 8 == 0 && H <= 256 && H > 0, "hidden width %d", H);
    GBSDF_CHECK_ARG(ldy % 8 == 0 && ldy >= H && aligned(Y, 16) && aligned(dZ, 16), "layout");
    GBSDF_CHECK_ARG(!d_pre || aligned(d_pre, 16), "d_pre alignment");
    GBSDF_CHECK_ARG(!dZ_lo || aligned(dZ_lo, 16), "dZ_lo alignment");
    unsigned blocks = head_blocks(Ns);
    {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const unsigned resident = (unsigned)((sms > 0 ? sms : 1) * HEAD_BWD_BLOCKS_PER_SM);
        if (blocks > resident) blocks = resident;
    }
    k_rgb_head_bwd<<<blocks, 256, 0, as_stream(stream)>>>(
        Ns, (const __half*)Y, ldy, H, W, rgbs, d_rgbs, (__half*)d_pre, (__half*)dZ, (__half*)dZ_lo, d_b, d_W);
    return launch_status("rgb_head_bwd");
}

extern "C" int gbsdf_app_grad(int64_t R, int32_t S, const int64_t* ray_offsets, const int32_t* app_idx,
                              const void* d_xc, int ld_dxc, int col0, int app_dim, float* d_app, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(R >= 0, "R < 0");
    if (R == 0 || app_dim == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(app_idx && d_xc && d_app && (S > 0 || ray_offsets), "NULL pointer");
    const int64_t threads = R * 32;
    k_app_grad<<<(unsigned)((threads + 255) / 256), 256, 0, as_stream(stream)>>>(
        R, S, ray_offsets, app_idx, (const float*)d_xc, ld_dxc, col0, app_dim, d_app);
    return launch_status("app_grad");
}

extern "C" size_t gbsdf_render_workspace_size(int64_t R, int32_t S, int32_t n_bg) {
    (void)R; (void)S; (void)n_bg;
    return 0;
}
