// Weight gradients of the dense layers on tcgen05:
//     dW[N, K] (+)= (dZ + dZ_lo)[:, :N]^T X[:, :K]
// a contraction over millions of sample rows into a small FP32 matrix.  These are the
// torch.nn.Linear weight gradients of the colour MLP (projects/nerf/utils/nerf_util.py:
// 187-196), the SDF feature layer (projects/neuralangelo/utils/mlp.py:55-69), the
// background NeRF (projects/neuralangelo/utils/modules.py:268-284) and, for more than
// 64 encoder columns, SDF layer 0; the bias gradient is the column of X that holds
// a constant 1.
//
// Layout: dZ and X are row-major fp16 (sample rows).  Both MMA operands are read
// MN-major straight from the TMA boxes: the MMA's M is 128 rows of dW (columns of
// dZ), its N up to 256 columns of X, its K 16 sample rows.  One CTA owns a block of
// 128 dW rows and a contiguous range of sample rows:
//   warp 0 (one lane)  TMA: per stage of 64 sample rows, the dZ block (two 64-column
//                      boxes, 128-byte swizzle), its optional lo half, and every
//                      64-column box of X;
//   warp 1 (one lane)  MMA: per stage, 4 K-steps into the TMEM accumulator [128 x K],
//                      the lo half first (small addends keep their bits in FP32);
//   warps 2-5          epilogue once, after the last stage: TMEM -> registers ->
//                      FP32 atomics into dW (CTAs of other row ranges add into the
//                      same rows).
// The CTAs of one row range (dW rows 0-127, 128-255, ...) are neighbours in the grid,
// so the repeated reads of each X box come from L2.
// Every wait is bounded; a timed-out wait sets *err and the roles leave their loops.
#include "dense.cuh"
#include "tma.cuh"

namespace gbsdf {
namespace {

constexpr int WG_ROWS = 64;                  // sample rows per stage (4 MMA K-steps)
constexpr int WG_NB = 128;                   // dW rows per CTA (the MMA's M)
constexpr int WG_THREADS = 192;              // TMA warp, MMA warp, 4 epilogue warps
constexpr int WG_MAX_STAGES = 4;
constexpr uint32_t WG_BOX = WG_ROWS * 128;   // one 64-column x 64-row fp16 box: 8 KB
constexpr size_t WG_SMEM_MAX = 227 * 1024;
constexpr size_t WG_BAR_BYTES = (2 * WG_MAX_STAGES + 2) * 8;

struct WgradParams {
    int64_t M;              // sample rows
    int N, K;               // dW is [N, K]
    int kb;                 // 64-column boxes of X (K rounded up to 64)
    int n_blocks;           // ceil(N / 128)
    int64_t rows_per_cta;   // sample rows of one CTA, a multiple of WG_ROWS
    int nst;                // pipeline stages
    int has_lo;             // dZ_lo present
    uint32_t stage_bytes;
    uint32_t tmem_cols;
    float* dW;
    int ldw;
    int* err;
};

__global__ void __launch_bounds__(WG_THREADS, 1) k_wgrad(const __grid_constant__ CUtensorMap tm_z,
                                                         const __grid_constant__ CUtensorMap tm_zlo,
                                                         const __grid_constant__ CUtensorMap tm_x, WgradParams p) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)p.nst * p.stage_bytes);
    uint64_t* empty = full + WG_MAX_STAGES;
    uint64_t* done = empty + WG_MAX_STAGES;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nblk = blockIdx.x % p.n_blocks;
    const int64_t r_begin = (int64_t)(blockIdx.x / p.n_blocks) * p.rows_per_cta;
    int64_t r_end = r_begin + p.rows_per_cta;
    if (r_end > p.M) r_end = p.M;
    const int nsteps = r_end > r_begin ? (int)((r_end - r_begin + WG_ROWS - 1) / WG_ROWS) : 0;
    const int n0 = nblk * WG_NB;
    const int kpad = p.kb * 64;

    if (tid == 0) {
        for (int i = 0; i < p.nst; ++i) {
            umma::mbar_init(&full[i], 1);
            umma::mbar_init(&empty[i], 1);
        }
        umma::mbar_init(done, 1);
        umma::fence_mbar_init();
    }
    if (warp == 1) {
        umma::tmem_alloc(tslot, p.tmem_cols);
        umma::tmem_relinquish();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;

    if (warp == 0) {
        // ---------------- producer ----------------
        if (lane == 0) {
            bool ok = true;
            for (int i = 0; i < nsteps; ++i) {
                const int slot = i % p.nst;
                const uint32_t use = (uint32_t)(i / p.nst);
                if (use > 0 && !umma::mbar_wait(&empty[slot], (use - 1) & 1u)) {
                    ok = false;
                    break;
                }
                uint8_t* st = smem + (size_t)slot * p.stage_bytes;
                const int row = (int)(r_begin + (int64_t)i * WG_ROWS);
                umma::mbar_arrive_expect_tx(&full[slot], p.stage_bytes);
                umma::tma_load_2d(st, &tm_z, n0, row, &full[slot]);
                umma::tma_load_2d(st + WG_BOX, &tm_z, n0 + 64, row, &full[slot]);
                uint8_t* b = st + 2 * WG_BOX;
                if (p.has_lo) {
                    umma::tma_load_2d(b, &tm_zlo, n0, row, &full[slot]);
                    umma::tma_load_2d(b + WG_BOX, &tm_zlo, n0 + 64, row, &full[slot]);
                    b += 2 * WG_BOX;
                }
                for (int j = 0; j < p.kb; ++j) umma::tma_load_2d(b + j * WG_BOX, &tm_x, 64 * j, row, &full[slot]);
            }
            if (!ok) flag_timeout(p.err, 1);
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---------------- MMA issue ----------------
        if (lane == 0) {
            bool ok = true;
            for (int i = 0; i < nsteps; ++i) {
                const int slot = i % p.nst;
                const uint32_t use = (uint32_t)(i / p.nst);
                if (!umma::mbar_wait(&full[slot], use & 1u)) {
                    ok = false;
                    break;
                }
                umma::fence_after_sync();
                const uint32_t sa = umma::smem_u32(smem + (size_t)slot * p.stage_bytes);
                const uint32_t sal = sa + 2 * WG_BOX;
                const uint32_t sb = sa + (p.has_lo ? 4 : 2) * WG_BOX;
                for (int c = 0; c < kpad; c += 256) {
                    const int nc = kpad - c < 256 ? kpad - c : 256;
                    const uint32_t idesc = umma::idesc_f16_mn(WG_NB, (uint32_t)nc);
                    const uint32_t d = tmem + (uint32_t)c;
                    for (int ks = 0; ks < WG_ROWS / 16; ++ks) {
                        const uint64_t bd = umma::make_desc_sw128_mn(sb + (uint32_t)(c / 64) * WG_BOX + ks * 2048u,
                                                                     WG_BOX, 1024u);
                        uint32_t acc = (i > 0 || ks > 0) ? 1u : 0u;
                        if (p.has_lo) {
                            umma::mma_f16(d, umma::make_desc_sw128_mn(sal + ks * 2048u, WG_BOX, 1024u), bd, idesc,
                                          acc);
                            acc = 1u;
                        }
                        umma::mma_f16(d, umma::make_desc_sw128_mn(sa + ks * 2048u, WG_BOX, 1024u), bd, idesc, acc);
                    }
                }
                umma::mma_commit(&empty[slot]);       // the stage's buffers are free once these complete
            }
            umma::mma_commit(done);
            if (!ok) flag_timeout(p.err, 1);
        }
        __syncwarp();
    } else if (nsteps > 0) {
        // ---------------- epilogue: TMEM lane quadrant (warp % 4) = 32 rows of the dW block ----------------
        const int q = warp & 3;
        const bool ok = umma::mbar_wait(done, 0);
        if (!ok) {
            if (lane == 0) flag_timeout(p.err, 1);
        } else {
            umma::fence_after_sync();
            const int n = n0 + q * 32 + lane;
            float* dst = p.dW + (int64_t)n * p.ldw;
            for (int c = 0; c < p.K; c += 32) {
                float v[32];
                umma::tmem_ld32(umma::taddr(tmem, q * 32, (uint32_t)c), v);
                if (n < p.N) {
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (c + j < p.K && v[j] != 0.0f) atomicAdd(dst + c + j, v[j]);
                }
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (warp == 1) umma::tmem_dealloc(tmem, p.tmem_cols);
}

int sm_count_wg() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace
}  // namespace gbsdf

using namespace gbsdf;

// dW[N, K] (row stride ldw) = (accumulate ? dW : 0) + (dZ + dZ_lo)[:, :N]^T X[:, :K].
// dZ [M, ldz] and dZ_lo (optional, same strides) and X [M, ldx] are fp16 row-major.
extern "C" int gbsdf_wgrad(int64_t M, int N, int K, const void* dZ, const void* dZ_lo, int ldz, const void* X,
                           int ldx, float* dW, int ldw, int accumulate, int* err, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(M >= 0 && N > 0 && K > 0, "bad sizes");
    GBSDF_CHECK_ARG(dZ && X && dW, "NULL pointer");
    GBSDF_CHECK_ARG(N <= 512 && K <= 512, "N=%d, K=%d: at most 512 each", N, K);
    GBSDF_CHECK_ARG(ldz >= N && ldx >= K && ldw >= K, "leading dimensions");
    GBSDF_CHECK_ARG(ldz % 8 == 0 && ldx % 8 == 0, "fp16 row strides must be multiples of 8 elements");
    GBSDF_CHECK_ARG(aligned(dZ, 16) && aligned(X, 16) && (!dZ_lo || aligned(dZ_lo, 16)),
                    "dZ, dZ_lo and X must be 16-byte aligned");
    GBSDF_CHECK_ARG(M < ((int64_t)1 << 31), "M=%lld exceeds the TMA coordinate range", (long long)M);
    cudaStream_t s = as_stream(stream);
    if (!accumulate) {
        if (cudaMemset2DAsync(dW, (size_t)ldw * 4, 0, (size_t)K * 4, (size_t)N, s) != cudaSuccess) {
            set_error("clearing dW failed");
            return GBSDF_ERR_CUDA;
        }
    }
    if (M == 0) return GBSDF_OK;
    WgradParams p;
    p.M = M; p.N = N; p.K = K;
    p.kb = (K + 63) / 64;
    p.n_blocks = (N + WG_NB - 1) / WG_NB;
    p.has_lo = dZ_lo ? 1 : 0;
    p.stage_bytes = (uint32_t)(2 + 2 * p.has_lo + p.kb) * WG_BOX;
    p.nst = WG_MAX_STAGES;
    while (p.nst > 2 && (size_t)p.nst * p.stage_bytes + WG_BAR_BYTES > WG_SMEM_MAX) --p.nst;
    const size_t smem = (size_t)p.nst * p.stage_bytes + WG_BAR_BYTES;
    if (smem > WG_SMEM_MAX) {
        set_error("weight gradient K=%d needs %zu B of shared memory", K, smem);
        return GBSDF_ERR_UNSUPPORTED;
    }
    const int kpad = p.kb * 64;
    p.tmem_cols = kpad <= 32 ? 32 : kpad <= 64 ? 64 : kpad <= 128 ? 128 : kpad <= 256 ? 256 : 512;
    // one CTA per SM: the SMs are shared out between the dW row blocks, each CTA taking a
    // contiguous range of whole stages
    int64_t splits = sm_count_wg() / p.n_blocks;
    if (splits < 1) splits = 1;
    const int64_t stages = (M + WG_ROWS - 1) / WG_ROWS;
    if (splits > stages) splits = stages;
    p.rows_per_cta = (stages + splits - 1) / splits * WG_ROWS;
    splits = (M + p.rows_per_cta - 1) / p.rows_per_cta;
    p.dW = dW; p.ldw = ldw; p.err = err;
    CUtensorMap tm_z, tm_zlo, tm_x;
    const CUtensorMapL2promotion l2 = CU_TENSOR_MAP_L2_PROMOTION_L2_256B;
    if (int st = tensor_map_2d(&tm_z, false, dZ, M, N, ldz, 64, WG_ROWS, CU_TENSOR_MAP_SWIZZLE_128B, l2, "dZ"))
        return st;
    if (dZ_lo) {
        if (int st = tensor_map_2d(&tm_zlo, false, dZ_lo, M, N, ldz, 64, WG_ROWS, CU_TENSOR_MAP_SWIZZLE_128B, l2,
                                   "dZ_lo"))
            return st;
    } else {
        tm_zlo = tm_z;                                   // unused
    }
    if (int st = tensor_map_2d(&tm_x, false, X, M, K, ldx, 64, WG_ROWS, CU_TENSOR_MAP_SWIZZLE_128B, l2, "X"))
        return st;
    allow_max_smem(k_wgrad);
    k_wgrad<<<(unsigned)(splits * p.n_blocks), WG_THREADS, smem, s>>>(tm_z, tm_zlo, tm_x, p);
    return launch_status("wgrad");
}
