// Persistent tcgen05 tile engine for the width-256 MLP layers.
//
// One CTA (256 threads) per SM walks 128-row tiles of a row-major fp16 matrix X
// [M x K].  The weight slice W [N_TILE x K] (K-major) stays resident in shared
// memory for the whole launch; each tile is staged with cp.async into the
// no-swizzle K-major core-matrix layout, multiplied by one elected thread with
// tcgen05.mma (fp16 x fp16 -> fp32 in TMEM), and read back by all eight warps
// with tcgen05.ld for a fused epilogue.  N-splits (blockIdx.x % n_split) let
// two CTAs share a tile when K x N does not fit one CTA's shared memory.
#pragma once

#include "common.cuh"
#include "umma.cuh"

namespace gbsdf {

constexpr int TILE_M = 128;
constexpr int DENSE_THREADS = 256;

// Tile staging: chunk c (16 bytes = 8 fp16 of one row) of a [128 x K] tile goes
// to byte c*16 of the K-major core-matrix layout when c enumerates
// (row group, K chunk, row in group) -- see umma.cuh.  Rows at or beyond
// `rows` are zero-filled.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(umma::smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most N of this thread's committed cp.async groups are still pending
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Walk (row group, K chunk) in nested loops so no integer division is needed.
// dst_k > K: the tile's rows are dst_k columns wide and only the first K are written
__device__ __forceinline__ void stage_rows_kmajor(uint8_t* tile, const __half* src, int64_t row0, int64_t rows,
                                                  int ld, int K, int tid, int nthreads, int nrows = TILE_M,
                                                  int dst_k = 0) {
    const int KC = K >> 3;
    const size_t group_bytes = (size_t)(dst_k > K ? dst_k : K) * 16;    // one 8-row group
    const int per_group = 8 * KC;                 // chunks of one 8-row group
    // each thread starts at chunk tid and strides by nthreads; decompose once, then advance
    int c = tid;
    int rg = 0, rem = c;
    while (rem >= per_group) { rem -= per_group; ++rg; }
    const int total = nrows * KC;
    for (; c < total; c += nthreads) {
        const int r_lo = rem & 7;
        const int kc = rem >> 3;
        const int r = rg * 8 + r_lo;
        uint8_t* dst = tile + rg * group_bytes + (size_t)rem * 16;
        const int64_t gr = row0 + r;
        if (gr < rows) {
            cp_async16(dst, src + gr * (int64_t)ld + kc * 8);
        } else {
            *reinterpret_cast<uint4*>(dst) = make_uint4(0, 0, 0, 0);
        }
        rem += nthreads;
        while (rem >= per_group) { rem -= per_group; ++rg; }
    }
}

// issue the K/16 MMAs of one tile: D = A * B^T (A: 128 x K, B: N x K, both K-major)
__device__ __forceinline__ void issue_tile_mma(uint32_t d_tmem, uint32_t a_saddr, uint32_t b_saddr, int K,
                                               uint32_t idesc, bool accumulate_first = false) {
    const uint32_t sbo = (uint32_t)K * 16u;
    for (int ks = 0; ks < K / 16; ++ks) {
        const uint64_t ad = umma::make_desc(a_saddr + ks * 256u, 128u, sbo);
        const uint64_t bd = umma::make_desc(b_saddr + ks * 256u, 128u, sbo);
        umma::mma_f16(d_tmem, ad, bd, idesc, (ks > 0 || accumulate_first) ? 1u : 0u);
    }
}

// the same with different row widths of the A and B tiles (a K-column prefix of a wider tile)
__device__ __forceinline__ void issue_tile_mma_strided(uint32_t d_tmem, uint32_t a_saddr, int a_kcols,
                                                       uint32_t b_saddr, int b_kcols, int K, uint32_t idesc,
                                                       bool accumulate_first = false) {
    const uint32_t sbo_a = (uint32_t)a_kcols * 16u, sbo_b = (uint32_t)b_kcols * 16u;
    for (int ks = 0; ks < K / 16; ++ks) {
        const uint64_t ad = umma::make_desc(a_saddr + ks * 256u, 128u, sbo_a);
        const uint64_t bd = umma::make_desc(b_saddr + ks * 256u, 128u, sbo_b);
        umma::mma_f16(d_tmem, ad, bd, idesc, (ks > 0 || accumulate_first) ? 1u : 0u);
    }
}

__device__ __forceinline__ void store_half8(__half* dst, const float* v) {
    __half2 h[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = __floats2half2_rn(v[2 * i], v[2 * i + 1]);
    *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(h);
}
// the fp16 residual v - fp16(v) of eight values: with store_half8's hi half, hi + lo
// carries an FP32 value to ~2^-22 relative (the low half of an activation pair)
__device__ __forceinline__ void store_half8_lo(__half* dst, const float* v) {
    float lo[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) lo[i] = v[i] - __half2float(__float2half_rn(v[i]));
    store_half8(dst, lo);
}
__device__ __forceinline__ void load_half8(const __half* src, float* v) {
    const uint4 u = *reinterpret_cast<const uint4*>(src);
    const __half2* h = reinterpret_cast<const __half2*>(&u);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float2 f = __half22float2(h[i]);
        v[2 * i] = f.x;
        v[2 * i + 1] = f.y;
    }
}

// report a timed-out wait through a device flag the host reads after the launch
__device__ __forceinline__ void flag_timeout(int* err, int code) {
    if (err) atomicCAS(err, 0, code);
}

}  // namespace gbsdf
