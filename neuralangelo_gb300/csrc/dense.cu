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
#include "tma.cuh"

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
    int nslots;          // A-chunk slots of the shared-memory ring
    int nslots_req;      // tuning: requested slots (0 = as many as fit)
    int tma_store;       // fp16 output written back through shared memory and TMA
};

// Warp-specialised pipeline (one persistent CTA per SM):
//   warp 16 (producer)  one lane streams the A tiles in 64-column K chunks into a ring
//                       of shared-memory slots, one TMA box per chunk (128-byte swizzle,
//                       rows past M zero-filled), completing on full[slot]'s byte count;
//   warp 17 (MMA)       one lane issues the tcgen05.mma of each chunk into one of two
//                       TMEM accumulators, frees the slot with tcgen05.commit ->
//                       empty[slot] and signals a finished tile on tfull[buf];
//   warps 0-15          the epilogue: four warps per TMEM lane quadrant, each reading a
//                       quarter of the columns of the finished accumulator, then
//                       tempty[buf] so the MMA warp can reuse it.
// The weight slice [N_TILE x K] stays resident.  Tile t+1's MMAs run while tile t's
// epilogue drains the other accumulator, and the loads run ahead of both.  With a
// low operand half (Xlo) its chunks come first: small addends keep their bits in
// the FP32 accumulator.  Every wait is bounded; a timed-out wait sets *err and the
// roles leave their loops.
constexpr int DENSE_EPI_WARPS = 16;
constexpr int DENSE_TPB = (DENSE_EPI_WARPS + 2) * 32;
constexpr int KCH = 64;                                   // A columns per chunk
constexpr int CHUNK_BYTES = TILE_M * KCH * 2;             // 16 KB
constexpr int MAX_SLOTS = 6;
constexpr int MIN_SLOTS = 3;
constexpr int STAGE_BYTES = DENSE_EPI_WARPS * 32 * 32 * 2;  // per-warp output staging of the TMA store

template <int N_TILE, int EPI>
__global__ void __launch_bounds__(DENSE_TPB, 1) k_dense(const __grid_constant__ CUtensorMap tm_x,
                                                        const __grid_constant__ CUtensorMap tm_xlo,
                                                        const __grid_constant__ CUtensorMap tm_y,
                                                        const __grid_constant__ CUtensorMap tm_ylo, DenseParams p) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int K = p.K, nslots = p.nslots;
    uint8_t* w_s = smem;                                              // [N_TILE x K]
    uint8_t* ring = w_s + (size_t)N_TILE * K * 2;                     // nslots x [128 x 64]
    uint8_t* stage_s = ring + (size_t)nslots * CHUNK_BYTES;              // 16 x [32 x 32] fp16, when tma_store
    float* bias_s = reinterpret_cast<float*>(stage_s + (p.tma_store ? STAGE_BYTES : 0));
    uint64_t* full = reinterpret_cast<uint64_t*>(bias_s + N_TILE);   // [MAX_SLOTS]
    uint64_t* empty = full + MAX_SLOTS;                               // [MAX_SLOTS]
    uint64_t* tfull = empty + MAX_SLOTS;                              // [2]
    uint64_t* tempty = tfull + 2;                                     // [2]
    uint32_t* tslot = reinterpret_cast<uint32_t*>(tempty + 2);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ns = blockIdx.x % p.n_split;
    const int group = blockIdx.x / p.n_split, ngroups = gridDim.x / p.n_split;
    const int n0 = ns * N_TILE;

    // resident weight slice and bias (all threads)
    stage_rows_kmajor(w_s, p.W, n0, p.N_total, K, K, tid, DENSE_TPB, N_TILE);
    for (int i = tid; i < N_TILE; i += DENSE_TPB) bias_s[i] = p.bias ? p.bias[n0 + i] : 0.0f;
    if (tid == 0) {
        for (int i = 0; i < nslots; ++i) {
            umma::mbar_init(&full[i], 1);
            umma::mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            umma::mbar_init(&tfull[i], 1);
            umma::mbar_init(&tempty[i], DENSE_EPI_WARPS);
        }
        umma::fence_mbar_init();
    }
    if (warp == 0) {
        umma::tmem_alloc(tslot, 2 * N_TILE);
        umma::tmem_relinquish();
    }
    cp_async_wait_all();
    umma::fence_proxy_async_smem();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    const int64_t ntiles = (p.M + TILE_M - 1) / TILE_M;
    const int nk = (K + KCH - 1) / KCH;                 // chunks per operand half
    const int nchunks = p.Xlo ? 2 * nk : nk;

    if (warp == DENSE_EPI_WARPS) {
        // ---------------- producer: one TMA box (64 columns x 128 rows, 128-byte swizzle) per chunk ----------------
        if (lane == 0) {
            uint32_t n = 0;
            bool ok = true;
            for (int64_t t = group; t < ntiles && ok; t += ngroups) {
                for (int c = 0; c < nchunks; ++c, ++n) {
                    const uint32_t slot = n % (uint32_t)nslots, use = n / (uint32_t)nslots;
                    if (use > 0 && !umma::mbar_wait(&empty[slot], (use - 1) & 1u)) {
                        ok = false;
                        break;
                    }
                    const bool lo = p.Xlo && c < nk;
                    const int kidx = p.Xlo ? (lo ? c : c - nk) : c;
                    umma::mbar_arrive_expect_tx(&full[slot], CHUNK_BYTES);
                    umma::tma_load_2d(ring + (size_t)slot * CHUNK_BYTES, lo ? (const void*)&tm_xlo : (const void*)&tm_x,
                                      kidx * KCH, (int)(t * TILE_M), &full[slot]);
                }
            }
            if (!ok) flag_timeout(p.err, 1);
        }
        __syncwarp();
    } else if (warp == DENSE_EPI_WARPS + 1) {
        // ---------------- MMA issue ----------------
        if (lane == 0) {
            const uint32_t idesc = umma::idesc_f16(TILE_M, N_TILE);
            const uint32_t w_addr = umma::smem_u32(w_s), r_addr = umma::smem_u32(ring);
            uint32_t n = 0;
            bool ok = true;
            int i = 0;
            for (int64_t t = group; t < ntiles && ok; t += ngroups, ++i) {
                const int buf = i & 1;
                const uint32_t ub = (uint32_t)(i >> 1);
                if (ub > 0 && !umma::mbar_wait(&tempty[buf], (ub - 1) & 1u)) {
                    ok = false;
                    break;
                }
                umma::fence_after_sync();
                const uint32_t d_tmem = tmem + (uint32_t)(buf * N_TILE);
                for (int c = 0; c < nchunks; ++c, ++n) {
                    const uint32_t slot = n % (uint32_t)nslots, use = n / (uint32_t)nslots;
                    if (!umma::mbar_wait(&full[slot], use & 1u)) {
                        ok = false;
                        break;
                    }
                    umma::fence_after_sync();
                    const int kidx = p.Xlo ? (c < nk ? c : c - nk) : c;
                    const int col0 = kidx * KCH, kc = min(KCH, K - col0);
                    for (int j = 0; j < kc / 16; ++j) {
                        const uint64_t ad = umma::make_desc_sw128(r_addr + slot * CHUNK_BYTES + j * 32u);
                        const uint64_t bd = umma::make_desc(w_addr + (uint32_t)(col0 / 16 + j) * 256u, 128u,
                                                            (uint32_t)K * 16u);
                        umma::mma_f16(d_tmem, ad, bd, idesc, (c > 0 || j > 0) ? 1u : 0u);
                    }
                    umma::mma_commit(&empty[slot]);
                }
                if (!ok) break;
                umma::mma_commit(&tfull[buf]);
            }
            if (!ok) flag_timeout(p.err, 1);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue ----------------
        const SoftplusK spk = softplus_k(p.beta);
        const int q = warp & 3;                 // TMEM lane quadrant of this warp
        const int part = warp >> 2;             // which quarter of the columns this warp reads
        const int row = q * 32 + lane;
        constexpr int COLS_PER_WARP = N_TILE / 4;
        constexpr int CHUNK = COLS_PER_WARP < 32 ? COLS_PER_WARP : 32;
        int i = 0;
        for (int64_t t = group; t < ntiles; t += ngroups, ++i) {
            const int buf = i & 1;
            if (!umma::mbar_wait(&tfull[buf], (uint32_t)(i >> 1) & 1u)) {
                if (lane == 0) flag_timeout(p.err, 1);
                break;
            }
            umma::fence_after_sync();
            const int64_t grow = t * TILE_M + row;
            const bool live = grow < p.M;
            const uint32_t tcol = (uint32_t)(buf * N_TILE);
#pragma unroll 1
            for (int c0 = part * COLS_PER_WARP; c0 < (part + 1) * COLS_PER_WARP; c0 += CHUNK) {
                float v[CHUNK];
                if constexpr (CHUNK == 32) umma::tmem_ld32(umma::taddr(tmem, q * 32, tcol + c0), v);
                else umma::tmem_ld16(umma::taddr(tmem, q * 32, tcol + c0), v);
                if (live) {
                    if constexpr (EPI == EPI_DRELU || EPI == EPI_DSOFTPLUS) {
                        const __half* gp = p.G + grow * (int64_t)p.ldg + n0 + c0;
#pragma unroll
                        for (int j = 0; j < CHUNK; j += 8) {
                            float g[8];
                            load_half8(gp + j, g);
#pragma unroll
                            for (int k = 0; k < 8; ++k) {
                                if constexpr (EPI == EPI_DRELU) v[j + k] = g[k] > 0.0f ? v[j + k] : 0.0f;
                                else v[j + k] *= 1.0f - ex2_ftz(-g[k] * spk.c1);
                            }
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < CHUNK; ++j) {
                            const float z = v[j] + bias_s[c0 + j];
                            if constexpr (EPI == EPI_RELU) v[j] = fmaxf(z, 0.0f);
                            else if constexpr (EPI == EPI_SOFTPLUS) v[j] = softplus_fast_h(z, spk);
                            else v[j] = z;
                        }
                    }
                    if (p.tma_store) {
                        // handled below, for the whole warp
                    } else if (p.y_f32) {
                        float* yp = reinterpret_cast<float*>(p.Y) + grow * (int64_t)p.ldy + n0 + c0;
#pragma unroll
                        for (int j = 0; j < CHUNK; j += 4)
                            *reinterpret_cast<float4*>(yp + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
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
                                for (int k = 0; k < 8; ++k) lo[k] = v[j + k] - __half2float(__float2half_rn(v[j + k]));
                                store_half8(lp + j, lo);
                            }
                        }
                    }
                }
                if constexpr (CHUNK == 32) {
                    if (p.tma_store) {
                        // coalesced write-back: the warp's block goes through a 2 KB staging
                        // buffer of 64-byte rows (64-byte swizzle: 16-byte chunk j of row r at
                        // chunk j ^ ((r >> 1) & 3)) and leaves as TMA stores; rows past M are
                        // clipped by the TMA unit.  fp16: one 32 x 32 box (then, with a low
                        // half, a second box of the residuals into Ylo); fp32: two 32 x 16 boxes.
                        uint8_t* stg = stage_s + warp * (32 * 32 * 2);
                        const int halves = (p.y_f32 || p.Ylo) ? 2 : 1;
                        for (int hh = 0; hh < halves; ++hh) {
                            if (lane == 0) umma::bulk_wait_read0();      // the previous store has read it
                            __syncwarp();
#pragma unroll
                            for (int j = 0; j < 4; ++j) {
                                uint4 u;
                                if (p.y_f32) {
                                    const float* f = v + 16 * hh + 4 * j;
                                    u = make_uint4(__float_as_uint(f[0]), __float_as_uint(f[1]), __float_as_uint(f[2]),
                                                   __float_as_uint(f[3]));
                                } else {
                                    __half2 h[4];
#pragma unroll
                                    for (int k = 0; k < 4; ++k) {
                                        float a = v[8 * j + 2 * k], b = v[8 * j + 2 * k + 1];
                                        if (hh == 1) {             // the low half: fp16 residuals
                                            a -= __half2float(__float2half_rn(a));
                                            b -= __half2float(__float2half_rn(b));
                                        }
                                        h[k] = __floats2half2_rn(a, b);
                                    }
                                    u = *reinterpret_cast<const uint4*>(h);
                                }
                                *reinterpret_cast<uint4*>(stg + lane * 64 + ((j ^ ((lane >> 1) & 3)) * 16)) = u;
                            }
                            umma::fence_proxy_async_smem();
                            __syncwarp();
                            if (lane == 0) {
                                if (p.y_f32)
                                    umma::tma_store_2d(&tm_y, n0 + c0 + 16 * hh, (int)(t * TILE_M) + q * 32, stg);
                                else
                                    umma::tma_store_2d(hh ? &tm_ylo : &tm_y, n0 + c0, (int)(t * TILE_M) + q * 32, stg);
                                umma::bulk_commit();
                            }
                        }
                    }
                }
            }
            umma::fence_before_sync();
            __syncwarp();
            if (lane == 0) umma::mbar_arrive(&tempty[buf]);
        }
    }
    if (p.tma_store && warp < DENSE_EPI_WARPS && lane == 0) umma::bulk_wait0();
    __syncthreads();
    umma::fence_after_sync();
    if (warp == 0) umma::tmem_dealloc(tmem, 2 * N_TILE);
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

constexpr size_t DENSE_SMEM_MAX = 227 * 1024;

// shared memory of a launch with `slots` ring slots (and the output staging when `stage`)
static size_t dense_smem_slots(int n_tile, int K, int slots, bool stage) {
    return (size_t)n_tile * K * 2 + (size_t)slots * CHUNK_BYTES + (stage ? STAGE_BYTES : 0) + n_tile * 4 +
           (2 * MAX_SLOTS + 4) * 8 + 16;
}
static size_t dense_smem(int n_tile, int K, bool stage) { return dense_smem_slots(n_tile, K, MIN_SLOTS, stage); }
static int dense_slots(int n_tile, int K, bool stage) {
    int s = MAX_SLOTS;
    while (s > MIN_SLOTS && dense_smem_slots(n_tile, K, s, stage) > DENSE_SMEM_MAX) --s;
    return s;
}

// TMA map of an fp16 matrix [rows x cols] with row stride ld elements: boxes of
// 64 columns x 128 rows, 128-byte swizzle, out-of-range elements read as zero
static int a_tensor_map(CUtensorMap* map, const void* base, int64_t rows, int cols, int ld) {
    return tensor_map_2d(map, false, base, rows, cols, ld, KCH, TILE_M, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, "input");
}

// TMA map of the output [rows x cols] (row stride ld elements): boxes of 64-byte rows x 32 rows
// (32 fp16 or 16 fp32 columns), 64-byte swizzle
static int y_tensor_map(CUtensorMap* map, void* base, int64_t rows, int cols, int ld, bool f32) {
    return tensor_map_2d(map, f32, base, rows, cols, ld, f32 ? 16 : 32, 32, CU_TENSOR_MAP_SWIZZLE_64B,
                         CU_TENSOR_MAP_L2_PROMOTION_NONE, "output");
}

template <int N_TILE, int EPI>
static int launch_dense(DenseParams p, cudaStream_t s) {
    // the TMA write-back needs 32-column chunks, 16-byte row strides and the staging buffers
    // next to at least MIN_SLOTS ring slots
    p.tma_store = (N_TILE / 4 >= 32 && aligned(p.Y, 16) && p.ldy % (p.y_f32 ? 4 : 8) == 0 &&
                   dense_smem_slots(N_TILE, p.K, MIN_SLOTS, true) <= DENSE_SMEM_MAX) ? 1 : 0;
    p.nslots = dense_slots(N_TILE, p.K, p.tma_store != 0);
    if (p.nslots_req >= MIN_SLOTS && p.nslots_req < p.nslots) p.nslots = p.nslots_req;
    const size_t smem = dense_smem_slots(N_TILE, p.K, p.nslots, p.tma_store != 0);
    if (smem > DENSE_SMEM_MAX) {
        set_error("dense layer K=%d N_TILE=%d needs %zu B of shared memory", p.K, N_TILE, smem);
        return GBSDF_ERR_UNSUPPORTED;
    }
    allow_max_smem(k_dense<N_TILE, EPI>);
    const int64_t ntiles = (p.M + TILE_M - 1) / TILE_M;
    int64_t groups = sm_count() / p.n_split;
    if (groups < 1) groups = 1;
    if (groups > ntiles) groups = ntiles;
    CUtensorMap tm_x, tm_xlo, tm_y, tm_ylo;
    if (int st = a_tensor_map(&tm_x, p.X, p.M, p.K, p.ldx)) return st;
    if (int st = a_tensor_map(&tm_xlo, p.Xlo ? p.Xlo : p.X, p.M, p.K, p.ldx)) return st;
    if (p.tma_store) {
        if (int st = y_tensor_map(&tm_y, p.Y, p.M, p.N_total, p.ldy, p.y_f32 != 0)) return st;
    } else {
        tm_y = tm_x;                                       // unused
    }
    if (p.tma_store && p.Ylo) {
        if (int st = y_tensor_map(&tm_ylo, p.Ylo, p.M, p.N_total, p.ldy, false)) return st;
    } else {
        tm_ylo = tm_y;                                     // unused
    }
    k_dense<N_TILE, EPI><<<(unsigned)(groups * p.n_split), DENSE_TPB, smem, s>>>(tm_x, tm_xlo, tm_y, tm_ylo, p);
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

namespace gbsdf {
// launch shapes chosen by a tuner, per (K, N); read by gbsdf_dense
struct DenseTune {
    int K, N, n_tile, nslots;
};
static DenseTune g_dense_tune[32];
static int g_dense_tune_n = 0;
static const DenseTune* dense_tune_find(int K, int N) {
    for (int i = 0; i < g_dense_tune_n; ++i)
        if (g_dense_tune[i].K == K && g_dense_tune[i].N == N) return &g_dense_tune[i];
    return nullptr;
}
}  // namespace gbsdf

using namespace gbsdf;

extern "C" int gbsdf_dense_tune(int K, int N, int n_tile, int nslots) {
    clear_error();
    GBSDF_CHECK_ARG(n_tile == 0 || n_tile == 64 || n_tile == 128 || n_tile == 256, "n_tile %d", n_tile);
    GBSDF_CHECK_ARG(nslots == 0 || (nslots >= MIN_SLOTS && nslots <= MAX_SLOTS), "nslots %d", nslots);
    for (int i = 0; i < g_dense_tune_n; ++i) {
        if (g_dense_tune[i].K == K && g_dense_tune[i].N == N) {
            g_dense_tune[i].n_tile = n_tile;
            g_dense_tune[i].nslots = nslots;
            return GBSDF_OK;
        }
    }
    GBSDF_CHECK_ARG(g_dense_tune_n < 32, "dense tuning table full");
    g_dense_tune[g_dense_tune_n++] = DenseTune{K, N, n_tile, nslots};
    return GBSDF_OK;
}

// Y[:, 0:N] = epi(X[:, 0:K] * W^T + b ; G), fp16 in/out, fp32 accumulate.
// K multiple of 16 (<= 320), N multiple of 64; leading dimensions multiples of 8.
extern "C" int gbsdf_dense(int64_t M, int K, int N, const void* X, const void* Xlo, int ldx, const void* W,
                           const float* bias, const void* G, int ldg, void* Y, void* Ylo, int ldy, int y_f32, int epi,
                           float beta, int* err, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(M >= 0 && K > 0 && N > 0, "bad sizes");
    if (M == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(X && W && Y, "NULL pointer");
    GBSDF_CHECK_ARG(K % 16 == 0 && K <= 512, "K=%d must be a multiple of 16 and <= 512", K);
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
    // N tiles of 128 columns (two CTAs share each 128-row tile of X: the second read
    // comes from L2): the resident weight slice of a 256-wide layer then leaves room for
    // six ring slots and the TMA write-back (1.5 tiles of X in flight); 256-column tiles
    // measured 10 % slower over the colour MLP, eight slots slower still
    int n_tile = 128;
    while (n_tile > 64 && (dense_smem(n_tile, K, Xlo != nullptr) > DENSE_SMEM_MAX || N % n_tile != 0))
        n_tile >>= 1;
    p.nslots_req = 0;
    if (const DenseTune* t = dense_tune_find(K, N)) {
        if (t->n_tile > 0 && N % t->n_tile == 0 && dense_smem(t->n_tile, K, Xlo != nullptr) <= DENSE_SMEM_MAX)
            n_tile = t->n_tile;
        p.nslots_req = t->nslots;
    }
    p.n_split = N / n_tile;
    return dense_launch(p, n_tile, as_stream(stream));
}

extern "C" size_t gbsdf_dense_workspace_size(int64_t M, int K, int N) {
    (void)M; (void)K; (void)N;
    return 0;
}
