// Hierarchical importance sampler of the object field (the no-grad pre-pass
// that places the training samples along each ray).
//
// Reference path: Model.sample_dists_all / sample_dists_hierarchical
// (projects/neuralangelo/model.py:232-267), nerf_util.sample_dists and
// sample_dists_from_pdf (projects/nerf/utils/nerf_util.py:20-68) and
// render.alpha_compositing_weights (projects/nerf/utils/render.py:87-99).
//
// Layout: per-ray sample lists are rows of a [R, ld] float32 array (distances,
// and their SDF values when a later round needs them).  One warp owns one ray:
// it stages the row in shared memory, sorts the concatenation of the list and
// the previous round's fine samples by rank (the reference concatenates and
// sorts, model.py:240-247), computes the NeuS interval weights with an FP32
// product scan, the normalised CDF with an FP32 sum scan, and inverts the CDF
// at the n_fine stratified midpoints.  The SDF of the new points is evaluated
// between rounds by the field kernel (gbsdf_sdf_points).
#include "common.cuh"

namespace gbsdf {

constexpr int SAMPLER_WARPS = 8;
constexpr int kMaxPerLane = (GBSDF_SAMPLER_MAX_LIST - 1 + 31) / 32;   // intervals per lane
static_assert(kMaxPerLane <= 16, "per-lane CDF chunk kept in registers");

__global__ void __launch_bounds__(256) k_sampler_coarse(gbsdf_sampler_args p, int n, const float* u, int ldu,
                                                        const float* near, const float* far, float* pts) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= p.R * n) return;
    const int64_t r = i / n;
    const int k = (int)(i % n);
    const float uk = u ? u[r * ldu + k] : 0.5f;
    // nerf_util.py:31-37: rands = u + k ; dists = rands / n * (far - near) + near
    const float rands = __fadd_rn(uk, (float)k);
    const float nr = near[r], fr = far[r];
    const float d = __fadd_rn(__fmul_rn(__fdiv_rn(rands, (float)n), __fsub_rn(fr, nr)), nr);
    p.dists[r * p.ld + k] = d;
    if (pts) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
            pts[3 * i + c] = __fadd_rn(p.center[3 * r + c], __fmul_rn(p.ray_unit[3 * r + c], d));
    }
}

__device__ __forceinline__ float sigmoid_f32(float x) { return 1.0f / (1.0f + expf(-x)); }

// torch.linspace(0, 1, steps) element i, float32 (start + step i below the middle,
// end - step (steps - 1 - i) above it)
__device__ __forceinline__ float linspace01(int i, int steps) {
    const float step = __fdiv_rn(1.0f, (float)(steps - 1));
    return i < steps / 2 ? __fmul_rn(step, (float)i) : __fsub_rn(1.0f, __fmul_rn(step, (float)(steps - 1 - i)));
}

// Warp-wide exclusive scan of per-lane chunk totals (mul = product, else sum).
template <bool MUL>
__device__ __forceinline__ float warp_exclusive(float v, int lane) {
    float inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc = MUL ? inc * y : inc + y;
    }
    const float ex = __shfl_up_sync(0xffffffffu, inc, 1);
    return lane == 0 ? (MUL ? 1.0f : 0.0f) : ex;
}

__global__ void __launch_bounds__(SAMPLER_WARPS * 32) k_sampler_round(gbsdf_sampler_args p) {
    extern __shared__ float sm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t r = blockIdx.x * (int64_t)SAMPLER_WARPS + wib;
    const int cap = p.n_list + p.n_merge;               // list length after the merge
    float* sd = sm + (size_t)wib * 5 * cap;             // staged distances
    float* ss = sd + cap;                               // staged SDF values
    float* md = ss + cap;                               // merged distances
    float* ms = md + cap;                               // merged SDF values
    float* cdf = ms + cap;                              // [n] CDF, then scratch
    if (r >= p.R) return;
    const bool with_s = p.sdfs != nullptr;
    float* rowd = p.dists + r * p.ld;
    float* rows = with_s ? p.sdfs + r * p.ld : nullptr;
    for (int i = lane; i < p.n_list; i += 32) {
        sd[i] = rowd[i];
        if (with_s) ss[i] = rows[i];
    }
    if (lane < p.n_merge) {
        sd[p.n_list + lane] = p.merge_d[r * p.n_merge + lane];
        if (with_s) ss[p.n_list + lane] = p.merge_s[r * p.n_merge + lane];
    }
    __syncwarp();
    int n = p.n_list;
    const float* d = sd;
    const float* s = ss;
    if (p.n_merge > 0) {
        // rank sort of the concatenation (ties keep their concatenation order)
        n = cap;
        for (int i = lane; i < n; i += 32) {
            const float x = sd[i];
            int pos = 0;
            for (int j = 0; j < n; ++j) {
                const float y = sd[j];
                pos += (y < x) || (y == x && j < i);
            }
            md[pos] = x;
            if (with_s) ms[pos] = ss[i];
        }
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
            rowd[i] = md[i];
            if (with_s) rows[i] = ms[i];
        }
        d = md;
        s = ms;
    }
    if (p.n_fine == 0 || n < 2) {
        if (p.n_fine > 0 && lane < p.n_fine) {   // one bin: every fine sample on it (nerf_util.py:57-66)
            const float v = n > 0 ? d[0] : 0.0f;
            p.fine_d[r * p.n_fine + lane] = v;
            if (p.fine_pts)
                for (int c = 0; c < 3; ++c)
                    p.fine_pts[3 * (r * p.n_fine + lane) + c] =
                        __fadd_rn(p.center[3 * r + c], __fmul_rn(p.ray_unit[3 * r + c], v));
        }
        return;
    }
    // ---- NeuS interval alphas (model.py:251-264), one per interval i in [0, n-1)
    const int m = n - 1;
    const int per = (m + 31) / 32;                      // consecutive intervals per lane
    const int i0 = lane * per, i1 = min(i0 + per, m);
    const float inv_s = p.inv_s;
    // alpha_i in cdf[i] (scratch), then the visibility product scan
    float prod = 1.0f;
    for (int i = i0; i < i1; ++i) {
        const float pd = d[i], nd = d[i + 1], ps = s[i], ns = s[i + 1];
        const float mid = (ps + ns) * 0.5f;
        float cosv = (ns - ps) / (nd - pd + 1e-5f);
        if (p.robust) {
            const float pc = i > 0 ? (s[i] - s[i - 1]) / (d[i] - d[i - 1] + 1e-5f) : 0.0f;
            cosv = fminf(pc, cosv);
        }
        const float iv = nd - pd;
        const float est_prev = mid - cosv * iv * 0.5f;
        const float est_next = mid + cosv * iv * 0.5f;
        const float pc_ = sigmoid_f32(est_prev * inv_s), nc_ = sigmoid_f32(est_next * inv_s);
        const float a = fminf(fmaxf((pc_ - nc_) / (pc_ + 1e-5f), 0.0f), 1.0f);
        cdf[i] = a;
        prod *= (1.0f - a);
    }
    // weights w_i = alpha_i * prod_{j<i} (1 - alpha_j)   (render.py:94-98, FP32)
    float vis = warp_exclusive<true>(prod, lane);
    float wsum = 0.0f;
    for (int i = i0; i < i1; ++i) {
        const float a = cdf[i];
        const float w = a * vis;
        vis *= (1.0f - a);
        cdf[i] = w;
        wsum += w;
    }
    const float denom = fmaxf(warp_sum(wsum), 1e-12f);  // F.normalize(p=1, eps=1e-12)
    // cdf = [0, cumsum(pdf)] over n entries (nerf_util.py:53-55).  A lane's chunk is
    // moved to registers first: its last CDF entry overwrites the next lane's first weight.
    float pdfv[kMaxPerLane];
    const int cnt = i1 - i0;
    float csum = 0.0f;
#pragma unroll
    for (int k = 0; k < kMaxPerLane; ++k) {
        pdfv[k] = k < cnt ? __fdiv_rn(cdf[i0 + k], denom) : 0.0f;
        csum += pdfv[k];
    }
    float run = warp_exclusive<false>(csum, lane);
    __syncwarp();
    if (lane == 0) cdf[0] = 0.0f;
#pragma unroll
    for (int k = 0; k < kMaxPerLane; ++k) {
        if (k < cnt) {
            run += pdfv[k];
            cdf[i0 + k + 1] = run;
        }
    }
    __syncwarp();
    // ---- inverse-CDF sampling at the stratified midpoints (nerf_util.py:56-67)
    for (int k = lane; k < p.n_fine; k += 32) {
        const float u = 0.5f * (linspace01(k, p.n_fine + 1) + linspace01(k + 1, p.n_fine + 1));
        int lo = 0, hi = n;                             // searchsorted(right=True): #cdf <= u
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (cdf[mid] <= u) lo = mid + 1; else hi = mid;
        }
        const int idx = lo;
        const int low = max(idx - 1, 0), high = min(idx, n - 1);
        const float c0 = cdf[low], c1 = cdf[high];
        const float t = (u - c0) / (c1 - c0 + 1e-8f);
        const float b0 = d[low], b1 = d[high];
        const float v = b0 + t * (b1 - b0);
        p.fine_d[r * p.n_fine + k] = v;
        if (p.fine_pts)
            for (int c = 0; c < 3; ++c)
                p.fine_pts[3 * (r * p.n_fine + k) + c] =
                    __fadd_rn(p.center[3 * r + c], __fmul_rn(p.ray_unit[3 * r + c], v));
    }
}

static int check_sampler(const gbsdf_sampler_args& p) {
    GBSDF_CHECK_ARG(p.R >= 0, "R < 0");
    GBSDF_CHECK_ARG(p.dists && p.center && p.ray_unit, "NULL pointer");
    GBSDF_CHECK_ARG(p.n_list >= 0 && p.n_merge >= 0 && p.n_merge <= 32, "n_merge %d (0..32)", p.n_merge);
    GBSDF_CHECK_ARG(p.n_fine >= 0 && p.n_fine <= 32 * 32, "n_fine %d", p.n_fine);
    GBSDF_CHECK_ARG(p.ld >= p.n_list + p.n_merge, "row stride %d below the merged list length", p.ld);
    GBSDF_CHECK_ARG(p.n_list + p.n_merge <= GBSDF_SAMPLER_MAX_LIST, "list of %d samples exceeds %d",
                    p.n_list + p.n_merge, GBSDF_SAMPLER_MAX_LIST);
    GBSDF_CHECK_ARG(p.n_merge == 0 || p.merge_d, "merge_d NULL");
    GBSDF_CHECK_ARG(p.n_merge == 0 || !p.sdfs || p.merge_s, "merge_s NULL while sdfs are kept");
    GBSDF_CHECK_ARG(p.n_fine == 0 || p.fine_d, "fine_d NULL");
    GBSDF_CHECK_ARG(p.n_fine == 0 || p.sdfs, "drawing fine samples needs the SDF values");
    return GBSDF_OK;
}

}  // namespace gbsdf

using namespace gbsdf;

extern "C" int gbsdf_sampler_coarse(const gbsdf_sampler_args* args, int n, const float* u, int ldu,
                                    const float* near, const float* far, float* pts, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(args && near && far, "NULL pointer");
    const gbsdf_sampler_args& p = *args;
    GBSDF_CHECK_ARG(p.R >= 0 && p.dists && p.center && p.ray_unit, "bad sampler arguments");
    GBSDF_CHECK_ARG(n >= 1 && n <= p.ld, "n %d vs row stride %d", n, p.ld);
    GBSDF_CHECK_ARG(!u || ldu >= n, "ldu %d < n %d", ldu, n);
    const int64_t items = p.R * n;
    if (items == 0) return GBSDF_OK;
    k_sampler_coarse<<<(unsigned)((items + 255) / 256), 256, 0, as_stream(stream)>>>(p, n, u, ldu, near, far, pts);
    return launch_status("sampler_coarse");
}

extern "C" int gbsdf_sampler_round(const gbsdf_sampler_args* args, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(args != nullptr, "NULL args");
    const gbsdf_sampler_args& p = *args;
    if (int st = check_sampler(p)) return st;
    if (p.R == 0) return GBSDF_OK;
    const int cap = p.n_list + p.n_merge;
    const size_t smem = (size_t)SAMPLER_WARPS * 5 * (cap > 0 ? cap : 1) * sizeof(float);
    allow_max_smem(k_sampler_round);
    const int64_t blocks = (p.R + SAMPLER_WARPS - 1) / SAMPLER_WARPS;
    k_sampler_round<<<(unsigned)blocks, SAMPLER_WARPS * 32, smem, as_stream(stream)>>>(p);
    return launch_status("sampler_round");
}

extern "C" size_t gbsdf_sampler_args_size(void) { return sizeof(gbsdf_sampler_args); }
