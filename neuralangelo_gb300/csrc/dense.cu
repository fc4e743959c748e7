// Generic fused dense layer on tcgen05:  Y = epi(X * W^T + b ; G)
//
// Forward layers:  epi = relu / softplus(beta) / identity
// Backward (dX):   X = dZ, W = W^T of the forward layer, epi multiplies by the
//                  derivative of the previous layer's activation read from G
//                  (G = that layer's stored output): relu' = [G > 0],
//                  softplus' = 1 - exp(-beta G).
// These are the colour-MLP layers of NeuralRGB (projects/neuralangelo/utils/
// modules.py:199-220 via projects/nerf/utils/nerf_util.py:158-196) and the SDF
// feature layer (utils/mlp.py:55-69), forward and input-gradient.
#include "dense.cuh"

namespace gbsdf {

enum DenseEpi : int {
    EPI_IDENTITY = 0,
    EPI_RELU = 1,
    EPI_SOFTPLUS = 2,
    EPI_DRELU = 3,      // y = acc * [G > 0]
    EPI_DSOFTPLUS = 4,  // y = acc * (1 - exp(-beta * G))
};

struct DenseParams {
    int64_t M;
    int K;
    int N_total;
    int n_split;
    const __half* X;
    const __half* Xlo;   // optional low half of X (X = hi + lo), same layout; doubles the MMAs
    int ldx;
    const __half* W;
    const float* bias;
    const __half* G;
    int ldg;
    void* Y;
    void* Ylo;           // optional fp16 low half of the output (Y = hi + lo)
    int ldy;
    int y_f32;
    int epi;
    float beta;
    int* err;
};

// 16 warps: four per TMEM lane quadrant, each reading a quarter of the tile's
// columns, so enough warps are in flight to hide the tcgen05.ld and MUFU latency
// of the epilogue.  The epilogue kind is a template parameter.
constexpr int DENSE_WARPS = 16;
constexpr int DENSE_TPB = DENSE_WARPS * 32;

template <int N_TILE, int EPI>
__global__ void __launch_bounds__(DENSE_TPB, 1) k_dense(DenseParams p) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* w_s = smem;                                              // [N_TILE x K]
    uint8_t* a_s = w_s + (size_t)N_TILE * p.K * 2;                    // [128 x K]
    uint8_t* a2_s = a_s + (size_t)TILE_M * p.K * 2;                   // [128 x K] low half, when Xlo
    float* bias_s = reinterpret_cast<float*>(a2_s + (p.Xlo ? (size_t)TILE_M * p.K * 2 : 0));
    uint64_t* mbar = reinterpret_cast<uint64_t*>(bias_s + N_TILE);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ns = blockIdx.x % p.n_split;
    const int group = blockIdx.x / p.n_split, ngroups = gridDim.x / p.n_split;
    const int n0 = ns * N_TILE;

    // resident weight slice and bias
    stage_rows_kmajor(w_s, p.W, n0, p.N_total, p.K, p.K, tid, DENSE_TPB, N_TILE);
    for (int i = tid; i < N_TILE; i += DENSE_TPB) bias_s[i] = p.bias ? p.bias[n0 + i] : 0.0f;
    if (tid == 0) {
        umma::mbar_init(mbar, 1);
        umma::fence_mbar_init();
    }
    if (warp == 0) {
        umma::tmem_alloc(tslot, N_TILE);
        umma::tmem_relinquish();
    }
    cp_async_wait_all();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = umma::idesc_f16(TILE_M, N_TILE);
    const uint32_t a_addr = umma::smem_u32(a_s), w_addr = umma::smem_u32(w_s), a2_addr = umma::smem_u32(a2_s);
    const int64_t ntiles = (p.M + TILE_M - 1) / TILE_M;
    uint32_t phase = 0;
    bool ok = true;

    const float inv_beta = 1.0f / p.beta;
    const int q = warp & 3;                 // TMEM lane quadrant of this warp
    const int part = warp >> 2;             // which quarter of the columns this warp reads
    const int row = q * 32 + lane;
    constexpr int COLS_PER_WARP = N_TILE / 4;
    constexpr int CHUNK = COLS_PER_WARP < 32 ? COLS_PER_WARP : 32;

    // Software pipeline: the A tile of tile t+1 is loaded (cp.async) while the
    // epilogue of tile t reads TMEM; A's shared memory is free as soon as tile t's
    // MMAs have completed.
    auto stage = [&](int64_t t) {
        stage_rows_kmajor(a_s, p.X, t * TILE_M, p.M, p.ldx, p.K, tid, DENSE_TPB);
        if (p.Xlo) stage_rows_kmajor(a2_s, p.Xlo, t * TILE_M, p.M, p.ldx, p.K, tid, DENSE_TPB);
    };
    auto issue = [&]() {
        if (tid == 0) {
            umma::fence_after_sync();
            // the low half first: small addends keep their bits in the FP32 accumulator
            if (p.Xlo) issue_tile_mma(tmem, a2_addr, w_addr, p.K, idesc);
            issue_tile_mma(tmem, a_addr, w_addr, p.K, idesc, p.Xlo != nullptr);
            umma::mma_commit(mbar);
        }
    };
    int64_t t = group;
    if (t < ntiles) {
        stage(t);
        cp_async_wait_all();
        umma::fence_proxy_async_smem();
    }
    __syncthreads();
    if (t < ntiles) issue();
    for (; t < ntiles; t += ngroups) {
        const int64_t m0 = t * TILE_M;
        ok = __syncthreads_and(umma::mbar_wait(mbar, phase));
        phase ^= 1u;
        if (!ok) {
            flag_timeout(p.err, 1);
            break;
        }
        umma::fence_after_sync();
        const int64_t tn = t + ngroups;
        if (tn < ntiles) stage(tn);                 // overlaps the epilogue below
        const int64_t grow = m0 + row;
        const bool live = grow < p.M;
#pragma unroll 1
        for (int c0 = part * COLS_PER_WARP; c0 < (part + 1) * COLS_PER_WARP; c0 += CHUNK) {
            float v[CHUNK];
            if constexpr (CHUNK == 32) umma::tmem_ld32(umma::taddr(tmem, q * 32, c0), v);
            else umma::tmem_ld16(umma::taddr(tmem, q * 32, c0), v);
            if (live) {
                if constexpr (EPI == EPI_DRELU || EPI == EPI_DSOFTPLUS) {
                    const __half* gp = p.G + grow * (int64_t)p.ldg + n0 + c0;
#pragma unroll
                    for (int j = 0; j < CHUNK; j += 8) {
                        float g[8];
                        load_half8(gp + j, g);
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            if constexpr (EPI == EPI_DRELU) v[j + i] = g[i] > 0.0f ? v[j + i] : 0.0f;
                            else v[j + i] *= 1.0f - __expf(-p.beta * g[i]);
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < CHUNK; ++j) {
                        const float z = v[j] + bias_s[c0 + j];
                        if constexpr (EPI == EPI_RELU) v[j] = fmaxf(z, 0.0f);
                        else if constexpr (EPI == EPI_SOFTPLUS) v[j] = softplus_fast_h(z, p.beta, inv_beta);
                        else v[j] = z;
                    }
                }
                if (p.y_f32) {
                    float* yp = reinterpret_cast<float*>(p.Y) + grow * (int64_t)p.ldy + n0 + c0;
#pragma unroll
                    for (int j = 0; j < CHUNK; j += 4) *reinterpret_cast<float4*>(yp + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
                } else {
                    __half* yp = reinterpret_cast<__half*>(p.Y) + grow * (int64_t)p.ldy + n0 + c0;
#pragma unroll
                    for (int j = 0; j < CHUNK; j += 8) store_half8(yp + j, v + j);
                    if (p.Ylo) {
                        __half* lp = reinterpret_cast<__half*>(p.Ylo) + grow * (int64_t)p.ldy + n0 + c0;
#pragma unroll
                        for (int j = 0; j < CHUNK; j += 8) {
                            float lo[8];
#pragma unroll
                            for (int i = 0; i < 8; ++i) lo[i] = v[j + i] - __half2float(__float2half_rn(v[j + i]));
                            store_half8(lp + j, lo);
                        }
                    }
                }
            }
        }
        umma::fence_before_sync();
        if (tn < ntiles) {
            cp_async_wait_all();
            umma::fence_proxy_async_smem();
        }
        __syncthreads();
        if (tn < ntiles) issue();
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, N_TILE);
}

static int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

static size_t dense_smem(int n_tile, int K, bool split) {
    return (size_t)n_tile * K * 2 + (split ? 2 : 1) * (size_t)TILE_M * K * 2 + n_tile * 4 + 16;
}

template <int N_TILE, int EPI>
static int launch_dense(const DenseParams& p, cudaStream_t s) {
    const size_t smem = dense_smem(N_TILE, p.K, p.Xlo != nullptr);
    if (smem > 227 * 1024) {
        set_error("dense layer K=%d N_TILE=%d needs %zu B of shared memory", p.K, N_TILE, smem);
        return GBSDF_ERR_UNSUPPORTED;
    }
    cudaFuncSetAttribute(k_dense<N_TILE, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int64_t ntiles = (p.M + TILE_M - 1) / TILE_M;
    int64_t groups = sm_count() / p.n_split;
    if (groups < 1) groups = 1;
    if (groups > ntiles) groups = ntiles;
    k_dense<N_TILE, EPI><<<(unsigned)(groups * p.n_split), DENSE_TPB, smem, s>>>(p);
    return launch_status("dense");
}

template <int N_TILE>
static int launch_dense_epi(const DenseParams& p, cudaStream_t s) {
    switch (p.epi) {
        case EPI_IDENTITY: return launch_dense<N_TILE, EPI_IDENTITY>(p, s);
        case EPI_RELU: return launch_dense<N_TILE, EPI_RELU>(p, s);
        case EPI_SOFTPLUS: return launch_dense<N_TILE, EPI_SOFTPLUS>(p, s);
        case EPI_DRELU: return launch_dense<N_TILE, EPI_DRELU>(p, s);
        default: return launch_dense<N_TILE, EPI_DSOFTPLUS>(p, s);
    }
}

int dense_launch(const DenseParams& p, int n_tile, cudaStream_t s) {
    switch (n_tile) {
        case 64: return launch_dense_epi<64>(p, s);
        case 128: return launch_dense_epi<128>(p, s);
        case 256: return launch_dense_epi<256>(p, s);
        default: set_error("unsupported n_tile %d", n_tile); return GBSDF_ERR_UNSUPPORTED;
    }
}

}  // namespace gbsdf

using namespace gbsdf;

// Y[:, 0:N] = epi(X[:, 0:K] * W^T + b ; G), fp16 in/out, fp32 accumulate.
// K multiple of 16 (<= 320), N multiple of 64; leading dimensions multiples of 8.
extern "C" int gbsdf_dense(int64_t M, int K, int N, const void* X, const void* Xlo, int ldx, const void* W,
                           const float* bias, const void* G, int ldg, void* Y, void* Ylo, int ldy, int y_f32, int epi,
                           float beta, int* err, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(M >= 0 && K > 0 && N > 0, "bad sizes");
    if (M == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(X && W && Y, "NULL pointer");
    GBSDF_CHECK_ARG(K % 16 == 0 && K <= 320, "K=%d must be a multiple of 16 and <= 320", K);
    GBSDF_CHECK_ARG(N % 64 == 0 && N <= 512, "N=%d must be a multiple of 64 and <= 512", N);
    GBSDF_CHECK_ARG(ldx % 8 == 0 && ldy % 8 == 0 && ldx >= K && ldy >= N, "leading dimensions");
    GBSDF_CHECK_ARG(aligned(X, 16) && aligned(W, 16) && aligned(Y, 16), "X, W, Y must be 16-byte aligned");
    GBSDF_CHECK_ARG(epi >= 0 && epi <= 4, "bad epilogue %d", epi);
    if (epi == EPI_DRELU || epi == EPI_DSOFTPLUS) {
        GBSDF_CHECK_ARG(G != nullptr && ldg % 8 == 0 && ldg >= N && aligned(G, 16), "gate matrix G");
    }
    DenseParams p;
    p.M = M; p.K = K; p.N_total = N;
    GBSDF_CHECK_ARG(!Xlo || aligned(Xlo, 16), "Xlo alignment");
    GBSDF_CHECK_ARG(!Ylo || (aligned(Ylo, 16) && !y_f32), "Ylo needs fp16 output, 16-byte aligned");
    p.X = (const __half*)X; p.Xlo = (const __half*)Xlo; p.ldx = ldx; p.W = (const __half*)W; p.bias = bias;
    p.G = (const __half*)G; p.ldg = ldg; p.Y = Y; p.Ylo = Ylo; p.ldy = ldy; p.y_f32 = y_f32 ? 1 : 0; p.epi = epi;
    p.beta = beta; p.err = err;
    // largest N tile whose weight slice + A tile fit in shared memory
    int n_tile = 256;
    while (n_tile > 64 && (dense_smem(n_tile, K, Xlo != nullptr) + 2048 > 227 * 1024 || N % n_tile != 0))
        n_tile >>= 1;
    p.n_split = N / n_tile;
    return dense_launch(p, n_tile, as_stream(stream));
}
