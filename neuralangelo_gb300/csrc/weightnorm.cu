// Gradients of the weight-normalised linears, and of the plain parameters that only need the
// loss scale taken off, in one launch for a whole list of layers.
//
// The reference wraps the SDF and colour MLP linears in torch.nn.utils.weight_norm (dim 0;
// projects/neuralangelo/utils/mlp.py:42-43, projects/nerf/utils/nerf_util.py:177-178):
// W = g v / ||v||, the norm taken over each output row.  The fused step yields the gradient of
// the effective weight W (times the loss scale); autograd through the weight norm is, for
// output row r with n = ||v_r|| and s = 1 / loss scale,
//     dg_r  = s sum_j dW_rj v_rj / n
//     dv_rj = (g_r / n) (s dW_rj - v_rj dg_r / n)
//     db_r  = s db_r.
// A plain entry (v == NULL) adds s dW into the weight's gradient and s db into the bias's.
//
// One warp per output row: two warp sums (||v_r||^2 and dW_r . v_r), then one pass writing
// dv_r.  Replaces the per-layer autograd graphs (norm, quotient, product and their backward)
// and the separate unscale and accumulate kernels.  gbsdf_weightnorm_fwd below forms the
// weights' working copies the same way, in place of the per-layer weight-norm forward, cast,
// transpose and reorder kernels.
#include "common.cuh"

namespace gbsdf {
namespace {

struct WnParams {
    gbsdf_weightnorm_layer L[GBSDF_WN_MAX_LAYERS];
    int64_t row0[GBSDF_WN_MAX_LAYERS + 1];   // first global row of each entry; row0[n] = total
    int n;
    const float* scale_dev;                   // device scalar (dynamic loss scaling) or NULL
    float scale;
};

__device__ __forceinline__ float wn_warp_sum(float v) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(256) k_weightnorm_bwd(const __grid_constant__ WnParams p) {
    const int64_t grow = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (grow >= p.row0[p.n]) return;
    int l = 0;
    while (grow >= p.row0[l + 1]) ++l;
    const gbsdf_weightnorm_layer& L = p.L[l];
    const int64_t r = grow - p.row0[l];
    const int64_t cols = L.cols;
    const float s = p.scale_dev ? *p.scale_dev : p.scale;
    const float* dW = L.dW + r * L.ld_dw;
    float* dv = L.dv + r * cols;
    if (L.v == nullptr) {
        for (int64_t j = lane; j < cols; j += 32) {
            const float x = s * dW[j];
            dv[j] = L.acc_v ? dv[j] + x : x;
        }
    } else {
        const float* v = L.v + r * cols;
        float n2 = 0.0f, dot = 0.0f;
        for (int64_t j = lane; j < cols; j += 32) {
            const float vv = v[j];
            n2 = fmaf(vv, vv, n2);
            dot = fmaf(dW[j], vv, dot);
        }
        n2 = wn_warp_sum(n2);
        dot = wn_warp_sum(dot);
        const float n = sqrtf(n2);
        const float dg = s * dot / n;
        const float a = L.g[r] / n, b = dg / n;
        for (int64_t j = lane; j < cols; j += 32) {
            const float x = a * (s * dW[j] - v[j] * b);
            dv[j] = L.acc_v ? dv[j] + x : x;
        }
        if (lane == 0) L.dg[r] = L.acc_g ? L.dg[r] + dg : dg;
    }
    if (lane == 0 && L.db && L.dbias) {
        const float x = s * L.db[r * L.ld_db];
        L.dbias[r] = L.acc_b ? L.dbias[r] + x : x;
    }
}

// ---------------------------------------------------------------------------
// The forward counterpart: the fp16 (and fp32) working copies of the effective weights that the
// fused step's kernels read, W = g v / ||v|| (or a plain weight), one column segment per entry,
// written row-major, as an fp16 hi + lo pair, transposed, or in FP32.  The product is formed as
// torch's weight norm forms it: v * (g / ||v||).
struct WnPackParams {
    gbsdf_weightnorm_pack E[GBSDF_WN_MAX_LAYERS];
    int64_t row0[GBSDF_WN_MAX_LAYERS + 1];
    int n;
};

__global__ void __launch_bounds__(256) k_weightnorm_fwd(const __grid_constant__ WnPackParams p) {
    const int64_t grow = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (grow >= p.row0[p.n]) return;
    int l = 0;
    while (grow >= p.row0[l + 1]) ++l;
    const gbsdf_weightnorm_pack& E = p.E[l];
    const int64_t r = grow - p.row0[l];
    const float* v = E.v + r * E.ld_src;
    float scale = 1.0f;
    if (E.g) {
        float n2 = 0.0f;
        for (int64_t j = lane; j < E.cols; j += 32) n2 = fmaf(v[j], v[j], n2);
        scale = E.g[r] / sqrtf(wn_warp_sum(n2));
    }
    __half* d16 = reinterpret_cast<__half*>(E.dst16);
    __half* d16lo = reinterpret_cast<__half*>(E.dst16_lo);
    __half* d16t = reinterpret_cast<__half*>(E.dst16T);
    for (int64_t j = lane; j < E.ncols; j += 32) {
        const float w = v[E.col0 + j] * scale;
        const __half h = __float2half_rn(w);
        if (d16) d16[r * E.ld16 + j] = h;
        if (d16lo) d16lo[r * E.ld16 + j] = __float2half_rn(w - __half2float(h));
        if (d16t) d16t[j * E.ldT + r] = h;
        if (E.dst32) E.dst32[r * E.ld32 + j] = w;
    }
}

}  // namespace
}  // namespace gbsdf

using namespace gbsdf;

extern "C" int gbsdf_weightnorm_fwd(int32_t n, const gbsdf_weightnorm_pack* entries, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(n >= 0 && n <= GBSDF_WN_MAX_LAYERS, "n %d (0 to %d entries)", n, GBSDF_WN_MAX_LAYERS);
    GBSDF_CHECK_ARG(n == 0 || entries != nullptr, "NULL entries");
    WnPackParams p{};
    p.n = n;
    int64_t rows = 0;
    for (int i = 0; i < n; ++i) {
        const gbsdf_weightnorm_pack& E = entries[i];
        GBSDF_CHECK_ARG(E.rows >= 0 && E.cols > 0 && E.col0 >= 0 && E.ncols >= 0 && E.col0 + E.ncols <= E.cols,
                        "entry %d: rows %lld, cols %lld, segment [%lld, %lld)", i, (long long)E.rows,
                        (long long)E.cols, (long long)E.col0, (long long)(E.col0 + E.ncols));
        GBSDF_CHECK_ARG(E.v, "entry %d: NULL v", i);
        GBSDF_CHECK_ARG(E.ld_src >= E.cols || E.rows <= 1, "entry %d: ld_src %lld < cols", i, (long long)E.ld_src);
        GBSDF_CHECK_ARG(E.dst16 || E.dst16T || E.dst32, "entry %d: no destination", i);
        GBSDF_CHECK_ARG(!E.dst16_lo || E.dst16, "entry %d: dst16_lo needs dst16", i);
        GBSDF_CHECK_ARG(!E.dst16 || E.ld16 >= E.ncols || E.rows <= 1, "entry %d: ld16", i);
        GBSDF_CHECK_ARG(!E.dst16T || E.ldT >= E.rows, "entry %d: ldT %lld < rows", i, (long long)E.ldT);
        GBSDF_CHECK_ARG(!E.dst32 || E.ld32 >= E.ncols || E.rows <= 1, "entry %d: ld32", i);
        p.E[i] = E;
        p.row0[i] = rows;
        rows += E.rows;
    }
    p.row0[n] = rows;
    if (rows == 0) return GBSDF_OK;
    k_weightnorm_fwd<<<(unsigned)((rows + 7) / 8), 256, 0, as_stream(stream)>>>(p);
    return launch_status("weightnorm_fwd");
}

extern "C" size_t gbsdf_weightnorm_pack_size(void) { return sizeof(gbsdf_weightnorm_pack); }

extern "C" int gbsdf_weightnorm_bwd(int32_t n, const gbsdf_weightnorm_layer* layers, const float* scale_dev,
                                    float scale, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(n >= 0 && n <= GBSDF_WN_MAX_LAYERS, "n %d (0 to %d entries)", n, GBSDF_WN_MAX_LAYERS);
    GBSDF_CHECK_ARG(n == 0 || layers != nullptr, "NULL layers");
    WnParams p{};
    p.n = n;
    p.scale_dev = scale_dev;
    p.scale = scale;
    int64_t rows = 0;
    for (int i = 0; i < n; ++i) {
        const gbsdf_weightnorm_layer& L = layers[i];
        GBSDF_CHECK_ARG(L.rows >= 0 && L.cols > 0, "entry %d: rows %lld, cols %lld", i, (long long)L.rows,
                        (long long)L.cols);
        GBSDF_CHECK_ARG(L.dW && L.dv, "entry %d: NULL dW or dv", i);
        GBSDF_CHECK_ARG(L.ld_dw >= L.cols || L.rows <= 1, "entry %d: ld_dw %lld < cols %lld", i, (long long)L.ld_dw,
                        (long long)L.cols);
        GBSDF_CHECK_ARG(!L.v || (L.g && L.dg), "entry %d: weight norm needs g and dg", i);
        GBSDF_CHECK_ARG(!L.db || !L.dbias || L.ld_db >= 1 || L.rows <= 1, "entry %d: ld_db %lld", i,
                        (long long)L.ld_db);
        p.L[i] = L;
        p.row0[i] = rows;
        rows += L.rows;
    }
    p.row0[n] = rows;
    if (rows == 0) return GBSDF_OK;
    const int64_t blocks = (rows + 7) / 8;
    k_weightnorm_bwd<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(p);
    return launch_status("weightnorm_bwd");
}

extern "C" size_t gbsdf_weightnorm_layer_size(void) { return sizeof(gbsdf_weightnorm_layer); }
