// Fused neural-SDF field kernels (hash grid + SDF layer 0 + head + numerical
// gradient taps) on tcgen05, forward and backward.
//
// Reference path: NeuralSDF.forward / sdf / compute_gradients (6 taps)
// (projects/neuralangelo/utils/modules.py:68-95, 131-156), MLPforNeuralSDF
// layer 0 + SDF head (utils/mlp.py:55-69), the outside overwrite
// (projects/neuralangelo/model.py:163) and the input of NeuralRGB
// (modules.py:209-220: x, SH(view dir), normalize(gradient), feature, appearance).
//
// Tile = 18 samples x 7 evaluations (centre + 6 taps) = 126 rows (+2 dead rows)
// of a 128-row tcgen05 tile.  Row r holds evaluation e = r / 18 of sample r % 18:
// e = 0 centre, 1 +x, 2 -x, 3 +y, 4 -y, 5 +z, 6 -z.  With 4 taps (the tetrahedral
// stencil, modules.py:157-175) a tile is 25 samples x 5 evaluations = 125 rows.  The hash-grid features of
// the active levels are gathered straight into the shared-memory A tile
// (fp16, K-major core-matrix layout); W0's encoding columns are resident; the
// three position columns, bias, softplus and the SDF head run in fp32 in the
// epilogue, so SDF values and the tap differences keep fp32 accuracy.
#include "dense.cuh"
#include "tma.cuh"

namespace gbsdf {

// Evaluations of one sample (the centre, then the taps) and samples per 128-row tile:
// 6 taps (modules.py:132-156): 18 samples x 7 = 126 rows; 4 taps (modules.py:157-175):
// 25 samples x 5 = 125 rows.
template <int TAPS>
struct TapTile {
    static_assert(TAPS == 6 || TAPS == 4, "4 or 6 taps");
    static constexpr int EVALS = TAPS + 1;
    static constexpr int SPT = TAPS == 6 ? 18 : 25;
    static constexpr int ROWS = SPT * EVALS;
    // the backward's double-buffered d f per evaluation row (+4 floats of slack), rounded up to
    // 4 floats so the d_h0c rows after it stay 16-byte aligned (cp.async and float4 accesses)
    static constexpr int DF_FLOATS = (2 * ROWS + 4 + 3) / 4 * 4;
};
constexpr int FWD_SDF_FLOATS = 128;   // forward's per-evaluation SDF values (<= 126) + padding
constexpr int FIELD_THREADS = 256;
constexpr int HID = 256;         // SDF hidden width (base.yaml:41)

typedef gbsdf_field_args FieldParams;   // layout and field meanings: include/gbsdf.h

// ray of sample s (32-bit division: the launchers keep the sample count below 2^32)
__device__ __forceinline__ int ray_of(const FieldParams& p, int64_t s) {
    return p.S > 0 ? (int)((uint32_t)s / (uint32_t)p.S) : p.sample_ray[s];
}

// float32 centre point c + d t (camera.py:314-320: one multiply, one add)
__device__ __forceinline__ void sample_point_of_ray(const FieldParams& p, int64_t s, int r, float* x) {
    const float t = p.dists[s];
#pragma unroll
    for (int i = 0; i < 3; ++i) x[i] = __fadd_rn(p.center[3 * r + i], __fmul_rn(p.ray_unit[3 * r + i], t));
}
__device__ __forceinline__ void sample_point(const FieldParams& p, int64_t s, float* x) {
    sample_point_of_ray(p, s, ray_of(p, s), x);
}

// evaluation position: the reference adds a float32 tap vector to the point.
// 6 taps: e = 1..6 -> +x, -x, +y, -y, +z, -z by eps (modules.py:135-143).
// 4 taps: e = 1..4 -> k1 (1,-1,-1), k2 (-1,-1,1), k3 (-1,1,-1), k4 (1,1,1) times the
// displacement eps / sqrt(3), which the caller passes as `eps` (modules.py:158-166).
template <int TAPS>
__device__ __forceinline__ void eval_point(const float* c, int e, float eps, float* x) {
    x[0] = c[0]; x[1] = c[1]; x[2] = c[2];
    if (e == 0) return;
    if constexpr (TAPS == 6) {
        const int d = (e - 1) >> 1;
        x[d] = (e & 1) ? __fadd_rn(x[d], eps) : __fsub_rn(x[d], eps);
    } else {
        const bool px = e == 1 || e == 4, py = e == 3 || e == 4, pz = e == 2 || e == 4;
        x[0] = px ? __fadd_rn(x[0], eps) : __fsub_rn(x[0], eps);
        x[1] = py ? __fadd_rn(x[1], eps) : __fsub_rn(x[1], eps);
        x[2] = pz ? __fadd_rn(x[2], eps) : __fsub_rn(x[2], eps);
    }
}

// Gather the active levels of one (row, level) pair into the A tile.
template <int F>
__device__ __forceinline__ void gather_level(const FieldParams& p, const float* xu, int l, float* out) {
    const LevelDesc d = level_desc(p.grid, l);
    uint32_t bx, by, bz;
    float fx, fy, fz;
    grid_pos(d.scale, xu[0], bx, fx);
    grid_pos(d.scale, xu[1], by, fy);
    grid_pos(d.scale, xu[2], bz, fz);
#pragma unroll
    for (int f = 0; f < F; ++f) out[f] = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint32_t idx = grid_index(d, bx + (c & 1), by + ((c >> 1) & 1), bz + ((c >> 2) & 1));
        const float w = corner_weight(c, fx, fy, fz);
        const __half* row = (const __half*)p.table + (d.offset + idx) * F;
        float v[F];
        if constexpr (F == 8) {
            load_half8(row, v);
        } else if constexpr (F == 4) {
            const uint2 u = __ldg(reinterpret_cast<const uint2*>(row));
            const __half2* h = reinterpret_cast<const __half2*>(&u);
            const float2 a = __half22float2(h[0]), b = __half22float2(h[1]);
            v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
        } else {
#pragma unroll
            for (int f = 0; f < F; ++f) v[f] = __half2float(row[f]);
        }
#pragma unroll
        for (int f = 0; f < F; ++f) out[f] = fmaf(w, v[f], out[f]);
    }
}

template <int F>
__device__ __forceinline__ void write_half_row(uint8_t* dst, const float* v) {
    if constexpr (F == 8) {
        store_half8(reinterpret_cast<__half*>(dst), v);
    } else if constexpr (F == 4) {
        __half2 h[2] = {__floats2half2_rn(v[0], v[1]), __floats2half2_rn(v[2], v[3])};
        *reinterpret_cast<uint2*>(dst) = *reinterpret_cast<const uint2*>(h);
    } else {
#pragma unroll
        for (int f = 0; f < F; ++f) reinterpret_cast<__half*>(dst)[f] = __float2half_rn(v[f]);
    }
}

// The features go in as an fp16 pair (hi + lo, ~2^-22 relative): the +eps and
// -eps taps of a sample differ by tiny amounts, and independent fp16 rounding
// of their features would dominate the pre-activation differences that the
// table gradient is made of.
template <int F>
__device__ __forceinline__ void write_tile_features(uint8_t* a_s, uint8_t* a2_s, int row, int l, int K0,
                                                    const float* v) {
    const uint32_t off = umma::kmajor_offset(row, l * F, K0);
    float lo[F];
#pragma unroll
    for (int f = 0; f < F; ++f) lo[f] = v[f] - __half2float(__float2half_rn(v[f]));
    write_half_row<F>(a_s + off, v);
    write_half_row<F>(a2_s + off, lo);
}

// Deterministic mode: each contribution as a 64-bit fixed-point integer with DET_FRAC_BITS
// fraction bits, added with integer atomics.  Integer addition is associative, so the sums
// do not depend on the order the atomics land in: two runs give bit-identical results.
constexpr int DET_FRAC_BITS = 48;
template <int F>
__device__ __forceinline__ void scatter_add_fixed(unsigned long long* dst, const float* v) {
#pragma unroll
    for (int f = 0; f < F; ++f)
        if (v[f] != 0.0f) atomicAdd(dst + f, (unsigned long long)__float2ll_rn(v[f] * 0x1p48f));
}

__global__ void k_fixed_to_table(int64_t n, const unsigned long long* __restrict__ fix, float* __restrict__ d_table) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long q = (long long)fix[i];
    if (q != 0) d_table[i] += (float)((double)q * 0x1p-48);
}

template <int F>
__device__ __forceinline__ void scatter_add(float* dst, const float* v) {
    if constexpr (F == 8) {
        atomicAdd(reinterpret_cast<float4*>(dst), make_float4(v[0], v[1], v[2], v[3]));
        atomicAdd(reinterpret_cast<float4*>(dst) + 1, make_float4(v[4], v[5], v[6], v[7]));
    } else if constexpr (F == 4) {
        atomicAdd(reinterpret_cast<float4*>(dst), make_float4(v[0], v[1], v[2], v[3]));
    } else {
#pragma unroll
        for (int f = 0; f < F; ++f) atomicAdd(dst + f, v[f]);
    }
}

// ---------------------------------------------------------------------------
// hash-grid gather and table-gradient scatter as their own kernels: one thread
// per (row, level) / (sample, level, corner) keeps thousands of independent
// loads and atomics in flight, which the tensor-core kernels (one CTA of eight
// warps per SM) cannot.

// x0ext row t*126 + r (r = e*18 + sl) of every tile: the features of level l in
// columns [l F, l F + F) as fp16 hi and, at K0 + 16 + l F, the fp16 residual lo;
// the level-0 thread also writes the 16-column tail after the hi features and
// zeroes the padding columns.  Rows of samples past the end are zeros.
// Six blocks per SM (at most 40 registers): the gather waits on L2 latency, and the
// extra resident warps keep more corner loads in flight.
template <int F, int TAPS>
__global__ void __launch_bounds__(256, 6) k_field_gather(FieldParams p, int64_t ntiles) {
    constexpr int EVALS = TapTile<TAPS>::EVALS, SPT = TapTile<TAPS>::SPT;
    const int A = p.active, K0 = p.K0, KX = 2 * K0 + 16;
    // 32-bit index arithmetic: the launcher checks rows * A < 2^32
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t rows = (uint32_t)(ntiles * (SPT * EVALS));
    if (i >= rows * (uint32_t)A) return;
    // thread order (tile, sample, evaluation, level): the 7 evaluations of a sample are
    // neighbouring threads, so at coarse levels (same cell for all taps) their corner
    // rows come from L1; the output row is t * 126 + e * 18 + sl
    const uint32_t q = i / (uint32_t)A;
    const int l = (int)(i - q * (uint32_t)A);
    const uint32_t se = q / EVALS;                   // tile-major sample slot
    const int e = (int)(q - se * EVALS);
    const int64_t t = se / SPT;
    const int sl = (int)(se - (uint32_t)t * SPT);
    const uint32_t grow = (uint32_t)t * (SPT * EVALS) + e * SPT + sl;
    const int64_t s = t * SPT + sl;
    __half* dst = (__half*)p.x0ext + (int64_t)grow * KX;     // 64-bit: rows * KX can exceed 2^32
    float v[F], lo[F];
    float x[3] = {0.f, 0.f, 0.f};
    const bool live = s < p.Ns;
    if (live) {
        float c[3], xu[3];
        sample_point(p, s, c);
        eval_point<TAPS>(c, e, p.eps, x);
#pragma unroll
        for (int k = 0; k < 3; ++k) xu[k] = to_unit(x[k]);
        gather_level<F>(p, xu, l, v);
    } else {
#pragma unroll
        for (int f = 0; f < F; ++f) v[f] = 0.0f;
    }
#pragma unroll
    for (int f = 0; f < F; ++f) lo[f] = v[f] - __half2float(__float2half_rn(v[f]));
    write_half_row<F>(reinterpret_cast<uint8_t*>(dst + l * F), v);
    write_half_row<F>(reinterpret_cast<uint8_t*>(dst + K0 + 16 + l * F), lo);
    if (l == 0) {
        // tail (multiplied by w0b's position and bias columns in the forward MMA):
        // x hi, 1, x lo, 1, x hi, zeros -- w0x x + b0 as fp16 hi/lo products
        float tail[16] = {0.f};
        if (live) {
            tail[0] = x[0]; tail[1] = x[1]; tail[2] = x[2]; tail[3] = 1.0f;
            for (int k = 0; k < 3; ++k) tail[4 + k] = x[k] - __half2float(__float2half_rn(x[k]));
            tail[7] = 1.0f;
            tail[8] = x[0]; tail[9] = x[1]; tail[10] = x[2];
        }
        store_half8(dst + K0, tail);
        store_half8(dst + K0 + 8, tail + 8);
        for (int c0 = A * F; c0 < K0; ++c0) {
            dst[c0] = __float2half_rn(0.0f);
            dst[K0 + 16 + c0] = __float2half_rn(0.0f);
        }
    }
}

// Table gradient of one (sample, level) over the sample's 7 evaluations: each
// evaluation's grid position is computed and its corners are accumulated in
// registers, merging consecutive evaluations that hit the same entry of a corner
// (the taps are eps apart: at coarse levels all 7 usually share the cell) before the
// vector atomics.  The 8 corners go in passes of CPT (the positions and d_enc rows
// are read again per pass, from L1): fewer accumulator registers, more resident warps.
constexpr int SCATTER_CPT = 2;

template <int F, int CPT, int TAPS, bool DET>
__global__ void __launch_bounds__(256, CPT >= 8 ? 2 : (CPT == 4 ? 3 : 4)) k_field_scatter(FieldParams p) {
    constexpr int EVALS = TapTile<TAPS>::EVALS, SPT = TapTile<TAPS>::SPT;
    const int A = p.active, K0 = p.K0;
    // 32-bit index arithmetic: the launcher checks Ns * active * 8 < 2^32
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)p.Ns * (uint32_t)A) return;
    const uint32_t s32 = i / (uint32_t)A;
    const int l = (int)(i - s32 * (uint32_t)A);
    const int64_t s = s32;
    const int64_t t = s32 / SPT;
    const int sl = (int)(s32 - (uint32_t)t * SPT);
    float c[3];
    sample_point(p, s, c);
    const LevelDesc d = level_desc(p.grid, l);
    float* base = p.d_table + d.offset * F;
    unsigned long long* fbase = DET ? p.d_table_fix + d.offset * F : nullptr;
    const float gscale = p.d_table_scale_dev ? *p.d_table_scale_dev : (p.d_table_scale != 0.0f ? p.d_table_scale : 1.0f);
    bool nonfinite = false;
    const int lane = threadIdx.x & 31;
    // Final flush.  With 8 active levels the lanes l, l + 8, l + 16, l + 24 of a warp hold
    // level l of four consecutive samples, which at coarse levels often end in the same
    // cell.  Two xor-shuffle steps merge equal entries: two lanes merge only when both
    // still own their sums, the lower lane absorbing the upper one's, so every
    // contribution is written exactly once.  Only whole live warps take part (Ns * 8 a
    // multiple of 32), so no lane has left the kernel.
    const bool grouped = A == 8 && (((uint32_t)p.Ns * 8u) & 31u) == 0u;
#pragma unroll 1
    for (int c0 = 0; c0 < 8; c0 += CPT) {
        uint32_t pidx[CPT];
        float pacc[CPT][F];
#pragma unroll
        for (int cc = 0; cc < CPT; ++cc) {
            pidx[cc] = 0xffffffffu;
#pragma unroll
            for (int f = 0; f < F; ++f) pacc[cc][f] = 0.0f;
        }
#pragma unroll 1
        for (int e = 0; e < EVALS; ++e) {
            float x[3], xu[3];
            eval_point<TAPS>(c, e, p.eps, x);
#pragma unroll
            for (int k = 0; k < 3; ++k) xu[k] = to_unit(x[k]);
            uint32_t bx, by, bz;
            float fx, fy, fz;
            grid_pos(d.scale, xu[0], bx, fx);
            grid_pos(d.scale, xu[1], by, fy);
            grid_pos(d.scale, xu[2], bz, fz);
            const float* dv = p.d_enc + (t * (SPT * EVALS) + e * SPT + sl) * (int64_t)K0 + l * F;
            float g[F];
            if constexpr (F % 4 == 0) {
#pragma unroll
                for (int f = 0; f < F; f += 4) {
                    const float4 q4 = __ldg(reinterpret_cast<const float4*>(dv + f));
                    g[f] = q4.x; g[f + 1] = q4.y; g[f + 2] = q4.z; g[f + 3] = q4.w;
                }
            } else {
#pragma unroll
                for (int f = 0; f < F; ++f) g[f] = __ldg(dv + f);
            }
            if (c0 == 0) {
#pragma unroll
                for (int f = 0; f < F; ++f) nonfinite |= !isfinite(g[f]);
            }
#pragma unroll
            for (int cc = 0; cc < CPT; ++cc) {
                const int corner = c0 + cc;
                const uint32_t idx =
                    grid_index(d, bx + (corner & 1), by + ((corner >> 1) & 1), bz + ((corner >> 2) & 1));
                const float w = corner_weight(corner, fx, fy, fz) * gscale;
                if (idx != pidx[cc]) {
                    if (pidx[cc] != 0xffffffffu) {
                        if constexpr (DET) scatter_add_fixed<F>(fbase + (uint64_t)pidx[cc] * F, pacc[cc]);
                        else scatter_add<F>(base + (uint64_t)pidx[cc] * F, pacc[cc]);
                    }
                    pidx[cc] = idx;
#pragma unroll
                    for (int f = 0; f < F; ++f) pacc[cc][f] = 0.0f;
                }
#pragma unroll
                for (int f = 0; f < F; ++f) pacc[cc][f] = fmaf(w, g[f], pacc[cc][f]);
            }
        }
#pragma unroll
        for (int cc = 0; cc < CPT; ++cc) {
            bool mine = true;
            if (grouped) {
#pragma unroll
                for (int off = 8; off <= 16; off <<= 1) {
                    const uint32_t other_idx = __shfl_xor_sync(0xffffffffu, pidx[cc], off);
                    const bool other_mine = __shfl_xor_sync(0xffffffffu, mine ? 1 : 0, off) != 0;
                    float other[F];
#pragma unroll
                    for (int f = 0; f < F; ++f) other[f] = __shfl_xor_sync(0xffffffffu, pacc[cc][f], off);
                    if (mine && other_mine && other_idx == pidx[cc]) {
                        if ((lane & off) == 0) {
#pragma unroll
                            for (int f = 0; f < F; ++f) pacc[cc][f] += other[f];
                        } else {
                            mine = false;
                        }
                    }
                }
            }
            if (mine) {
                if constexpr (DET) scatter_add_fixed<F>(fbase + (uint64_t)pidx[cc] * F, pacc[cc]);
                else scatter_add<F>(base + (uint64_t)pidx[cc] * F, pacc[cc]);
            }
        }
    }
    if (nonfinite && p.found_inf) *p.found_inf = 1.0f;     // any writer stores the same value
}

// ---------------------------------------------------------------------------
// forward

// Two CTAs per SM: one CTA's epilogue overlaps the other's staging, MMAs and
// per-sample phase.  The pre-activation comes out of the MMA complete: the A
// tile is x0ext's [features hi | tail] columns and B = w0b = [W0e | position and
// bias columns], so the epilogue reads W0x x + b0 + W0e f from TMEM and adds
// nothing; the fp16 residual of the features is a second MMA over the W0e prefix.
constexpr int FWD_CTAS_PER_SM = 2;
constexpr int FWD_APP_MAX = 28;        // appearance-code columns the forward's prefetch holds
// One sample's per-ray inputs of the forward's per-sample phase, prefetched into a ring of
// four tiles in shared memory (see k_field_fwd)
struct FwdSample {
    int r;                       // ray; -1 past the last sample
    int out;                     // the ray's `outside` flag
    int appi;                    // appearance-code row
    float c[3];                  // sample point c + d t
    float dv[3];                 // ray direction
    float app[FWD_APP_MAX];      // appearance code
};
constexpr int FWD_RING = 4;
// the colour-input tail is at most 48 columns with 23 fixed ones (check_fwd): app_dim <= 25
static_assert(FWD_APP_MAX >= 48 - 23, "the prefetch record holds every appearance column");

template <int F, int TAPS>
__global__ void __launch_bounds__(FIELD_THREADS, FWD_CTAS_PER_SM) k_field_fwd(FieldParams p,
                                                                             const __grid_constant__ CUtensorMap tm_xhi,
                                                                             const __grid_constant__ CUtensorMap tm_xlo) {
    constexpr int EVALS = TapTile<TAPS>::EVALS, SPT = TapTile<TAPS>::SPT;
    extern __shared__ __align__(1024) uint8_t smem[];
    const int K0 = p.K0;
    const int KB = K0 + 16;                                     // features hi + tail
    const int KX = 2 * K0 + 16;                                 // x0ext row width
    uint8_t* w_s = smem;                                        // [256 x KB]  w0b
    uint8_t* a_s = w_s + HID * KB * 2;                          // [128 x KB]  features hi | tail
    uint8_t* a2_s = a_s + TILE_M * KB * 2;                      // [128 x K0]  features lo
    float* wh_s = reinterpret_cast<float*>(a2_s + TILE_M * K0 * 2);   // [256]
    float* part_s = wh_s + HID;                                 // [2][128] partial head sums
    float* sdf_s = part_s + 2 * TILE_M;                         // [7][18]
    // the mbarrier 8-byte aligned whatever the tile's row count: 128 floats past sdf_s
    // (125 or 126 evaluation rows + padding)
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sdf_s + FWD_SDF_FLOATS);
    uint64_t* mbar_a = mbar + 1;                                // the A tile's TMA loads
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 2);
    FwdSample* ring = reinterpret_cast<FwdSample*>(mbar + 3);  // [FWD_RING][SPT]

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    stage_rows_kmajor(w_s, (const __half*)p.w0b, 0, HID, KB, KB, tid, FIELD_THREADS, HID);
    for (int i = tid; i < HID; i += FIELD_THREADS) wh_s[i] = p.whead[i];
    if (tid == 0) {
        umma::mbar_init(mbar, 1);
        umma::mbar_init(mbar_a, 1);
        umma::fence_mbar_init();
    }
    if (warp == 0) {
        umma::tmem_alloc(tslot, HID);
        umma::tmem_relinquish();
    }
    cp_async_wait_all();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = umma::idesc_f16(TILE_M, HID);
    const uint32_t a_addr = umma::smem_u32(a_s), w_addr = umma::smem_u32(w_s), a2_addr = umma::smem_u32(a2_s);
    const float bhead = p.bhead[0];
    const int64_t ntiles = (p.Ns + SPT - 1) / SPT;
    const int q = warp & 3, half = warp >> 2;
    const int row = q * 32 + lane;
    const int e_row = row / SPT, sl_row = row % SPT;
    uint32_t phase = 0;

    // features of a tile, gathered by k_field_gather into x0ext, loaded by TMA (thread 0, one
    // box per 8-row group and part, straight into the core-matrix layout; rows past the end
    // arrive as zeros); the next tile's load overlaps this tile's epilogue (A is free once its
    // MMAs completed)
    // (a timed-out tile ends the loop at its top, before its load_a: no load is left in flight)
    (void)KX;
    auto load_a = [&](int64_t tt) {
        umma::mbar_arrive_expect_tx(mbar_a, (uint32_t)(TILE_M * (KB + K0) * 2));
        const int row0 = (int)(tt * (SPT * EVALS));
#pragma unroll 1
        for (int g = 0; g < TILE_M / 8; ++g) {
            umma::tma_load_3d(a_s + g * KB * 16, &tm_xhi, 0, row0 + 8 * g, 0, mbar_a);
            umma::tma_load_3d(a2_s + g * K0 * 16, &tm_xlo, 0, row0 + 8 * g, 0, mbar_a);
        }
    };
    auto issue = [&](uint32_t phase_a) {           // the k-th call waits for the k-th load: phase k & 1
        if (tid == 0) {
            if (!umma::mbar_wait(mbar_a, phase_a)) flag_timeout(p.err, 1);   // the A tile's TMA loads
            umma::fence_after_sync();
            // smallest terms first: the tensor core's FP32 accumulation drops low
            // bits of addends much smaller than the running sum, so the fp16
            // residuals go in before the hi features and the large position/bias tail
            issue_tile_mma_strided(tmem, a2_addr, K0, w_addr, KB, K0, idesc);
            issue_tile_mma(tmem, a_addr, w_addr, KB, idesc, true);
            umma::mma_commit(mbar);
        }
    };
    // The per-sample phase reads per-ray inputs (flags, direction, centre, appearance code)
    // behind one or two dependent global loads.  They are prefetched into a ring of FWD_RING
    // tiles by the threads that have no sample of their own in that phase, one load level per
    // tile: the ray index three tiles ahead, the per-ray values two tiles ahead, the appearance
    // row one tile ahead; each level lands before the next reads it (a CTA barrier apart).
    const bool want_xc = p.xc != nullptr;
    const bool want_app = want_xc && p.app_table && p.app_dim > 0;
    auto slot = [&](int k) { return ring + (k & (FWD_RING - 1)) * SPT; };
    auto tile_of = [&](int k) { return (int64_t)blockIdx.x + (int64_t)k * gridDim.x; };
    auto pre_ray = [&](int k, int js) {
        const int64_t tk = tile_of(k), ss = tk * SPT + js;
        slot(k)[js].r = (tk < ntiles && ss < p.Ns) ? ray_of(p, ss) : -1;
    };
    auto pre_vals = [&](int k, int js) {
        FwdSample& e = slot(k)[js];
        const int r = e.r;
        if (r < 0) return;
        e.out = p.outside && p.outside[r];
        if (want_xc) {
            const int64_t ss = tile_of(k) * SPT + js;
            sample_point_of_ray(p, ss, r, e.c);
#pragma unroll
            for (int i = 0; i < 3; ++i) e.dv[i] = p.ray_unit[3 * r + i];
        }
        if (want_app) e.appi = p.app_idx[r];
    };
    auto pre_app = [&](int k, int js) {
        FwdSample& e = slot(k)[js];
        if (e.r < 0 || !want_app) return;
        const float* a = p.app_table + (int64_t)e.appi * p.app_dim;
        for (int i0 = 0; i0 < p.app_dim; i0 += 8) {
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = i0 + j < p.app_dim ? a[i0 + j] : 0.0f;
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (i0 + j < p.app_dim) e.app[i0 + j] = v[j];
        }
    };
    constexpr int LD0 = (SPT * 6 + 31) / 32 * 32;    // first loader thread
    static_assert(LD0 + 3 * SPT <= FIELD_THREADS, "the forward's prefetch loaders fit the CTA");
    if (tid < SPT) {
        pre_ray(0, tid);
        pre_ray(1, tid);
        pre_ray(2, tid);
    }
    __syncthreads();
    if (tid < SPT) {
        pre_vals(0, tid);
        pre_vals(1, tid);
    }
    __syncthreads();
    if (tid < SPT) pre_app(0, tid);
    int64_t t = blockIdx.x;
    if (t < ntiles && tid == 0) load_a(t);
    __syncthreads();
    if (t < ntiles) issue(0u);
    for (int it = 0; t < ntiles; t += gridDim.x, ++it) {
        const int64_t s0 = t * SPT;
        const bool ok = __syncthreads_and(umma::mbar_wait(mbar, phase));
        phase ^= 1u;
        if (!ok) {
            flag_timeout(p.err, 1);
            break;
        }
        umma::fence_after_sync();
        const int64_t tn = t + gridDim.x;
        if (tn < ntiles && tid == 0) load_a(tn);
        // epilogue: h = softplus(pre) ; partial head dot ; centre rows keep h in h0c
        const int64_t s = s0 + sl_row;
        const bool keep = row < SPT * EVALS && s < p.Ns && e_row == 0;
        float part4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const SoftplusK spk = softplus_k(p.beta);
#pragma unroll 1
        for (int c0 = half * 128; c0 < half * 128 + 128; c0 += 32) {
            float v[32];
            umma::tmem_ld32(umma::taddr(tmem, q * 32, c0), v);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const float h = softplus_fast_h(v[j], spk);
                v[j] = h;
                part4[j & 3] = fmaf(wh_s[c0 + j], h, part4[j & 3]);
            }
            if (keep) {
                const int64_t off = s * (int64_t)(p.ld_h0c > 0 ? p.ld_h0c : HID) + c0;
                __half* dst = (__half*)p.h0c + off;
#pragma unroll
                for (int j = 0; j < 32; j += 8) store_half8(dst + j, v + j);
                if (p.h0c_lo) {
                    __half* lo = (__half*)p.h0c_lo + off;
#pragma unroll
                    for (int j = 0; j < 32; j += 8) store_half8_lo(lo + j, v + j);
                }
            }
        }
        part_s[half * TILE_M + row] = (part4[0] + part4[1]) + (part4[2] + part4[3]);
        umma::fence_before_sync();
        __syncthreads();
        if (tid < SPT * EVALS) {
            sdf_s[tid] = part_s[tid] + part_s[TILE_M + tid] + bhead;
        }
        __syncthreads();
        // per-sample: gradient, Hessian diagonal, outside overwrite, colour-input columns;
        // six threads per sample, each storing one 8-column chunk of the colour-input tail
        // (the first of them also the SDF, gradient and Hessian)
        if (tid >= LD0 && tid < LD0 + 3 * SPT) {
            const int li = tid - LD0, st = li / SPT, js = li - st * SPT;
            if (st == 0) pre_ray(it + 3, js);
            else if (st == 1) pre_vals(it + 2, js);
            else pre_app(it + 1, js);
        }
        if (tid < SPT * 6) {
            const int js = tid / 6, kc8 = tid - 6 * js;
            const int64_t ss = s0 + js;
            const FwdSample& e = slot(it)[js];
            if (ss < p.Ns) {
                const int r = e.r;
                const bool out = e.out != 0;
                const float fc = out ? p.outside_val : sdf_s[js];
                float g[3], hh[3];
                if constexpr (TAPS == 6) {
                    // g_d = (f+ - f-) / (2 eps); H_dd = (f+ + f- - 2 f) / eps^2 (modules.py:144-155)
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        const float fp = sdf_s[(1 + 2 * d) * SPT + js], fm = sdf_s[(2 + 2 * d) * SPT + js];
                        g[d] = __fdiv_rn(__fsub_rn(fp, fm), p.two_eps);
                        hh[d] = __fdiv_rn(__fsub_rn(__fadd_rn(fp, fm), __fmul_rn(2.0f, fc)), p.eps2);
                    }
                } else {
                    // g = (k1 f1 + k2 f2 + k3 f3 + k4 f4) / (4 e); H_xx = ((f1 + f2 + f3 + f4) / 2 - 2 f) / e^2,
                    // every diagonal entry H_xx / 3 (modules.py:167-174); two_eps = 4 e, eps2 = e^2
                    const float f1 = sdf_s[SPT + js], f2 = sdf_s[2 * SPT + js];
                    const float f3 = sdf_s[3 * SPT + js], f4 = sdf_s[4 * SPT + js];
                    const float sx = __fadd_rn(__fsub_rn(__fsub_rn(f1, f2), f3), f4);
                    const float sy = __fadd_rn(__fadd_rn(__fsub_rn(-f1, f2), f3), f4);
                    const float sz = __fadd_rn(__fsub_rn(__fadd_rn(-f1, f2), f3), f4);
                    g[0] = __fdiv_rn(sx, p.two_eps);
                    g[1] = __fdiv_rn(sy, p.two_eps);
                    g[2] = __fdiv_rn(sz, p.two_eps);
                    const float sum = __fadd_rn(__fadd_rn(__fadd_rn(f1, f2), f3), f4);
                    const float hxx = __fdiv_rn(__fsub_rn(__fmul_rn(sum, 0.5f), __fmul_rn(2.0f, fc)), p.eps2);
                    hh[0] = hh[1] = hh[2] = __fdiv_rn(hxx, 3.0f);
                }
                if (kc8 == 0) {
                    p.sdf[ss] = fc;
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        p.grad[3 * ss + d] = g[d];
                        p.hess[3 * ss + d] = hh[d];
                    }
                }
                if (p.xc && 8 * kc8 < p.ldxc - HID) {
                    // NeuralRGB input tail (modules.py:209-213): x, SH(d), normalize(g), app
                    const float* c = e.c;
                    const float dx = e.dv[0], dy = e.dv[1], dz = e.dv[2];
                    const float xx = dx * dx, yy = dy * dy, zz = dz * dz;
                    float col[22];
                    col[0] = c[0]; col[1] = c[1]; col[2] = c[2];
                    // real spherical-harmonic basis, degree <= 3 (spherical_harmonics.py:47-84)
                    col[3] = 0.28209479177387814f;
                    col[4] = -0.4886025119029199f * dy;
                    col[5] = 0.4886025119029199f * dz;
                    col[6] = -0.4886025119029199f * dx;
                    col[7] = 1.0925484305920792f * dx * dy;
                    col[8] = -1.0925484305920792f * dy * dz;
                    col[9] = 0.31539156525252005f * (2.0f * zz - xx - yy);
                    col[10] = -1.0925484305920792f * dx * dz;
                    col[11] = 0.5462742152960396f * (xx - yy);
                    col[12] = -0.5900435899266435f * dy * (3.0f * xx - yy);
                    col[13] = 2.890611442640554f * dx * dy * dz;
                    col[14] = -0.4570457994644658f * dy * (4.0f * zz - xx - yy);
                    col[15] = 0.3731763325901154f * dz * (2.0f * zz - 3.0f * xx - 3.0f * yy);
                    col[16] = -0.4570457994644658f * dx * (4.0f * zz - xx - yy);
                    col[17] = 1.445305721320277f * dz * (xx - yy);
                    col[18] = -0.5900435899266435f * dx * (xx - 3.0f * yy);
                    const float nrm = fmaxf(sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]), 1e-12f);
                    col[19] = g[0] / nrm; col[20] = g[1] / nrm; col[21] = g[2] / nrm;
                    // this thread's 8 columns k = 8 kc8 + i: the 22 computed ones picked with
                    // compile-time indices (col[] stays in registers), the appearance code read
                    // straight from the table, and the last (padding) column a constant 1: the
                    // colour layer-0 weight gradient dZ^T xc then carries the bias gradient there
                    const float* a = want_app ? e.app : nullptr;
                    (void)r;
                    __half* dst = (__half*)p.xc + ss * (int64_t)p.ldxc + HID;
                    const int ncol = p.ldxc - HID;
                    float o8[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int k = 8 * kc8 + i;
                        float val = 0.0f;
#pragma unroll
                        for (int cc = 0; cc < 22; ++cc)
                            if (cc == k) val = col[cc];
                        if (a && k >= 22 && k - 22 < p.app_dim) val = a[k - 22];
                        if (k == ncol - 1) val = 1.0f;
                        o8[i] = val;
                    }
                    store_half8(dst + 8 * kc8, o8);
                    if (p.xc_lo) store_half8_lo((__half*)p.xc_lo + ss * (int64_t)p.ldxc + HID + 8 * kc8, o8);
                }
            }
        }
        __syncthreads();
        if (tn < ntiles) issue((uint32_t)(it + 1) & 1u);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, HID);
}

// ---------------------------------------------------------------------------
// backward

// One 128-row tile (18 samples x 7 evaluations) per iteration:
//   MMA1 recomputes the pre-activations (A = x0ext's features hi | tail, B = w0b;
//        plus the features lo against the W0e prefix), exactly as the forward;
//   the epilogue forms d_pre = (d f w_head + [centre] d_h0c) softplus'(pre) and the
//        head-weight gradient, writes d_pre as an fp16 hi + lo pair into TMEM (the A
//        operand of MMA2) and its hi half to shared memory: the A operand of the in-kernel
//        layer-0 weight gradient (DW below), or staging for the global d_pre0 rows;
//   MMA2 d_enc = d_pre W0e (A from TMEM, B = the W0e part of MMA1's w0b tile read
//        MN-major) goes to global for k_field_scatter.
// The +eps and -eps taps of a sample carry large, nearly cancelling d_pre, so a
// single fp16 rounding of d_pre would dominate the table-gradient error: hence the pair.
// TMEM without DW (512 columns, one CTA per SM): [0, 256) MMA1's accumulator, reused
// for MMA2's [128 x K0] result; [256, 384) d_pre hi, [384, 512) d_pre lo.
// d_pre0 (without DW) and d_enc leave through a 4 KB staging buffer per warp and TMA stores
// (one thread per row would touch 32 cache lines per store instruction); a tile has
// 126 rows, so the last lane quadrant stores a 30-row box.
constexpr size_t BWD_SMEM_FLOOR = 120 * 1024;   // > half an SM's shared memory: one CTA per SM
constexpr int BWD_THREADS = 512;                 // 16 warps: 4 lane quadrants x 4 quarters of the hidden units
constexpr int BWD_STAGE_BYTES = 4096;            // per warp: 32 rows x 128 bytes
constexpr int DH0_LD = HID + 4;                  // d_h0c rows in shared memory, padded against bank conflicts

// DW (K0 <= 64, the caller passes d_w0): the layer-0 weight gradient dW0 = d_pre^T [x hi |
// tail] + d_pre^T x lo is accumulated here instead of through d_pre0 and a separate GEMM.
//   * d_pre's hi/lo pair is written over MMA1's accumulator in place (chunk c: hi in
//     columns [16c, 16c + 8), lo in [16c + 8, 16c + 16)), which frees TMEM for MMA2's
//     result at 256 and two dW0 accumulators (hidden halves, K0 + 16 columns each) after it.
//   * The dW0 MMAs read both operands MN-major: A = the d_pre hi rows of the staging
//     buffers (128-byte swizzle atoms of 64 hidden units x 8 rows), B = the tile's x0ext rows.
//   * The feature tile is double-buffered: the next tile's load may not overwrite what
//     dW0 reads.  dW0 goes before MMA2, so MMA2's completion also frees the staging rows.
//   * The lo feature rows are K0 + 16 columns wide, the last 16 zero, so that the lo dW0
//     MMAs have the hi MMAs' shape (MMAs into one accumulator are ordered when their
//     shapes agree).
//   * MMA1 of the next tile is issued as soon as MMA2 has completed (D1 is free then),
//     under the d_enc epilogue.
//   * Each CTA adds its dW0 into d_w0 with atomics at the end.
template <int F, bool DW, int TAPS>
__global__ void __launch_bounds__(BWD_THREADS, 1) k_field_bwd(FieldParams p,
                                                             const __grid_constant__ CUtensorMap tm_pre32,
                                                             const __grid_constant__ CUtensorMap tm_pre30,
                                                             const __grid_constant__ CUtensorMap tm_enc32,
                                                             const __grid_constant__ CUtensorMap tm_enc30,
                                                             const __grid_constant__ CUtensorMap tm_plo32,
                                                             const __grid_constant__ CUtensorMap tm_plo30,
                                                             const __grid_constant__ CUtensorMap tm_xhi,
                                                             const __grid_constant__ CUtensorMap tm_xlo) {
    constexpr int EVALS = TapTile<TAPS>::EVALS, SPT = TapTile<TAPS>::SPT, TILE_ROWS = TapTile<TAPS>::ROWS;
    extern __shared__ __align__(1024) uint8_t smem[];
    const int K0 = p.K0;
    const int KB = K0 + 16;                                     // features hi + tail
    uint8_t* stage_s = smem;                                    // [16 warps][4 KB] TMA store staging
    uint8_t* w_s = stage_s + (BWD_THREADS / 32) * BWD_STAGE_BYTES;   // [256 x KB]  w0b: B of MMA1
    uint8_t* a_s0 = w_s + HID * KB * 2;                         // [128 x KB]  features hi | tail
    const int KL = DW ? KB : K0;                                // lo row width (DW: zero-padded)
    uint8_t* a3_s0 = a_s0 + TILE_M * KB * 2;                    // [128 x KL]  features lo
    uint8_t* a_s1 = DW ? a3_s0 + TILE_M * KL * 2 : a_s0;        // the second buffer (DW)
    uint8_t* a3_s1 = DW ? a_s1 + TILE_M * KB * 2 : a3_s0;
    float* wh_s = reinterpret_cast<float*>(a3_s1 + TILE_M * KL * 2);   // [256] head weights
    float* dwh_s = wh_s + HID;                                  // [256] d_whead accumulator
    float* df_s = dwh_s + HID;                                  // [2][7][18] d f per evaluation, double-buffered
    float* dh0_s = df_s + TapTile<TAPS>::DF_FLOATS;              // [SPT][DH0_LD] d_h0c of the tile's samples
    uint64_t* mbar = reinterpret_cast<uint64_t*>(dh0_s + SPT * DH0_LD);
    uint64_t* mbar_lo = mbar + 1;                               // DW: the lo-half dW0 MMAs of a tile
    uint64_t* mbar_a = mbar + 2;                                // the A tile's TMA loads
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 3);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    stage_rows_kmajor(w_s, (const __half*)p.w0b, 0, HID, KB, KB, tid, BWD_THREADS, HID);
    for (int i = tid; i < HID; i += BWD_THREADS) {
        wh_s[i] = p.whead[i];
        dwh_s[i] = 0.0f;
    }
    if (DW) {
        // the zero columns [K0, K0 + 16) of both lo tiles: 16 row groups x 256 bytes each
        for (int i = tid; i < 2 * (TILE_M / 8) * 16; i += BWD_THREADS) {
            uint8_t* base = (i >> 8) ? a3_s1 : a3_s0;
            *reinterpret_cast<uint4*>(base + ((i >> 4) & 15) * (KL * 16) + K0 * 16 + (i & 15) * 16) =
                make_uint4(0, 0, 0, 0);
        }
    }
    if (tid == 0) {
        umma::mbar_init(mbar, 1);
        umma::mbar_init(mbar_lo, 1);
        umma::mbar_init(mbar_a, 1);
        umma::fence_mbar_init();
    }
    if (warp == 0) {
        umma::tmem_alloc(tslot, 512);
        umma::tmem_relinquish();
    }
    cp_async_wait_all();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    // d_pre hi/lo of hidden units [16c, 16c + 16): separate TMEM regions, or in place (DW)
    auto t_hi = [&](int c) { return DW ? tmem + 16u * c : tmem + HID + 8u * c; };
    auto t_lo = [&](int c) { return DW ? tmem + 16u * c + 8u : tmem + HID + HID / 2 + 8u * c; };
    const uint32_t t_enc = DW ? tmem + HID : tmem;              // MMA2's result
    const uint32_t t_dw = tmem + HID + K0;                      // DW: dW0 of hidden half h at + h KB
    const uint32_t idesc1 = umma::idesc_f16(TILE_M, HID);
    const uint32_t idesc2 = umma::idesc_f16_bmn(TILE_M, K0);
    const uint32_t w_addr = umma::smem_u32(w_s);
    // MMA2's and dW0's descriptors are built once per tile: a K = 16 step only moves the start
    // address (bits 0-13, in 16-byte units, below 2^14 for any shared-memory address), so each
    // MMA adds a multiple of a per-tile step
    auto desc_step = [](uint32_t bytes) { return (uint64_t)(bytes >> 4); };
    // feature buffer b (0, or 1 with DW): selects, not arrays, which would go to local memory
    auto a_buf = [&](int b) { return b ? a_s1 : a_s0; };
    auto a3_buf = [&](int b) { return b ? a3_s1 : a3_s0; };
    auto a_addr = [&](int b) { return umma::smem_u32(a_buf(b)); };
    auto a3_addr = [&](int b) { return umma::smem_u32(a3_buf(b)); };
    bool dw_first = true;                                       // the CTA's first dW0 MMA initialises
    const int64_t ntiles = (p.Ns + SPT - 1) / SPT;
    const int q = warp & 3, part = warp >> 2;                   // lane quadrant, quarter of the hidden units
    const int row = q * 32 + lane;
    const int e_row = row / SPT, sl_row = row % SPT;
    uint32_t phase = 0, phase_lo = 0;
    float dbh = 0.0f;
    bool ok = true;

    // the prologue runs on warp 1 (lane = sample of the tile), apart from warp 0's MMA issuer
    static_assert(TapTile<TAPS>::SPT <= 32, "the prologue's samples fit one warp");
    const int pl = tid - 32;
    const bool pl_on = pl >= 0 && pl < SPT;
    // per-sample output gradients -> d f of each evaluation (modules.py:144-156), for
    // the next tile while this one is in flight, in three steps that keep the global
    // loads and the arithmetic off the tile's critical path: the per-sample loads at the
    // top of the tile, then, while MMA2 runs, the per-ray `outside` flag and the arithmetic
    // into df_s[buf]
    struct PrologueIn {
        float g[3], dg[3], dh[3], n[3], dsdf;
        int r;
        bool out;
    };
    auto prologue_load = [&](int64_t tt, PrologueIn& in) {
        const int64_t s = tt * SPT + pl;
        if (pl_on && s < p.Ns) {
            in.r = ray_of(p, s);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                in.g[d] = p.grad[3 * s + d];
                in.dg[d] = p.d_grad[3 * s + d];
                in.dh[d] = p.d_hess[3 * s + d];
            }
            // normals = g / max(|g|, 1e-12) feed the colour MLP (model.py:167)
            const float* dn = p.d_xc + s * (int64_t)p.ld_dxc + p.normal_col;
            in.n[0] = dn[0]; in.n[1] = dn[1]; in.n[2] = dn[2];
            in.dsdf = p.d_sdf[s];
        }
    };
    auto prologue_ray = [&](int64_t tt, PrologueIn& in) {
        const int64_t s = tt * SPT + pl;
        if (pl_on && s < p.Ns) in.out = p.outside && p.outside[in.r];
    };
    auto prologue_finish = [&](int64_t tt, const PrologueIn& in, int buf) {
        if (pl_on) {
            const int64_t s = tt * SPT + pl;
            float* dfb = df_s + buf * (EVALS * SPT);
            float df[EVALS];
#pragma unroll
            for (int e = 0; e < EVALS; ++e) df[e] = 0.0f;
            if (s < p.Ns) {
                const float g0 = in.g[0], g1 = in.g[1], g2 = in.g[2];
                const float n0 = in.n[0], n1 = in.n[1], n2 = in.n[2];
                float dg[3] = {in.dg[0], in.dg[1], in.dg[2]};
                const float len = sqrtf(g0 * g0 + g1 * g1 + g2 * g2);
                if (len > 1e-12f) {
                    const float inv = 1.0f / len;
                    const float u0 = g0 * inv, u1 = g1 * inv, u2 = g2 * inv;
                    const float dot = u0 * n0 + u1 * n1 + u2 * n2;
                    dg[0] += (n0 - u0 * dot) * inv;
                    dg[1] += (n1 - u1 * dot) * inv;
                    dg[2] += (n2 - u2 * dot) * inv;
                } else {
                    dg[0] += n0 * 1e12f; dg[1] += n1 * 1e12f; dg[2] += n2 * 1e12f;
                }
                float hsum = 0.0f;
                if constexpr (TAPS == 6) {
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        const float a = dg[d] / p.two_eps, b = in.dh[d] / p.eps2;
                        df[1 + 2 * d] = a + b;
                        df[2 + 2 * d] = -a + b;
                        hsum += b;
                    }
                } else {
                    // d H_xx = (dH_x + dH_y + dH_z) / 3; tap i: k_i . dg / (4 e) + d H_xx / (2 e^2)
                    const float dhxx = (in.dh[0] + in.dh[1] + in.dh[2]) / 3.0f;
                    const float b = 0.5f * dhxx / p.eps2;
                    const float ax = dg[0] / p.two_eps, ay = dg[1] / p.two_eps, az = dg[2] / p.two_eps;
                    df[1] = ax - ay - az + b;
                    df[2] = -ax - ay + az + b;
                    df[3] = -ax + ay - az + b;
                    df[4] = ax + ay + az + b;
                    hsum = dhxx / p.eps2;
                }
                // the centre feeds alpha and the Hessian only where it was not overwritten
                df[0] = in.out ? 0.0f : (in.dsdf - 2.0f * hsum);
            }
#pragma unroll
            for (int e = 0; e < EVALS; ++e) {
                dfb[e * SPT + pl] = df[e];
                dbh += df[e];
            }
        }
    };
    // encoder features of a tile, streamed back from the forward's x0ext rows (rows
    // 126-127 of a tile read the next tile's first rows or zeros; their MMA results
    // are never used) by TMA: one thread, one box per 8-row group and part, straight into
    // the core-matrix layout (rows past the end, and the lo part's zero columns, arrive
    // as zeros); 512 threads' cp.async copies of the same bytes cost them ~2k clocks a tile
    bool a_pending = false;                         // (thread 0, which issues and waits for these loads)
    auto load_a = [&](int64_t tt, int buf) {
        a_pending = true;
        umma::mbar_arrive_expect_tx(mbar_a, (uint32_t)(TILE_M * (KB + KL) * 2));
        const int row0 = (int)(tt * (SPT * EVALS));
#pragma unroll 1
        for (int g = 0; g < TILE_M / 8; ++g) {
            umma::tma_load_3d(a_buf(buf) + g * KB * 16, &tm_xhi, 0, row0 + 8 * g, 0, mbar_a);
            umma::tma_load_3d(a3_buf(buf) + g * KL * 16, &tm_xlo, 0, row0 + 8 * g, 0, mbar_a);
        }
    };
    uint32_t phase_a = 0;
    auto stage_dh0 = [&](int64_t tt) {             // one cp.async group
        for (int c = tid; c < SPT * (HID / 4); c += BWD_THREADS) {
            const int js = c / (HID / 4), k4 = c - js * (HID / 4);
            const int64_t ss = tt * SPT + js;
            float* dst = dh0_s + js * DH0_LD + 4 * k4;
            if (ss < p.Ns) cp_async16(dst, p.d_h0c + ss * HID + 4 * k4);
            else *reinterpret_cast<float4*>(dst) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        cp_async_commit();
    };
    auto issue1 = [&](int buf) {                   // warp 0 converged: every call follows a CTA barrier
        if (warp == 0) {
            if (umma::elect_one()) {
                if (!umma::mbar_wait(mbar_a, phase_a)) flag_timeout(p.err, 1);   // the A tile's TMA loads
                a_pending = false;
                umma::fence_after_sync();
                issue_tile_mma_strided(tmem, a3_addr(buf), KL, w_addr, KB, K0, idesc1);   // residuals first
                issue_tile_mma(tmem, a_addr(buf), w_addr, KB, idesc1, true);
                umma::mma_commit(mbar);
            }
            __syncwarp();
            phase_a ^= 1u;
        }
    };
    int64_t t = blockIdx.x;
    PrologueIn pin;
    if (t < ntiles) {
        prologue_load(t, pin);
        prologue_ray(t, pin);
        prologue_finish(t, pin, 0);
        if (tid == 0) load_a(t, 0);
        stage_dh0(t);
        cp_async_wait_all();
        umma::fence_proxy_async_smem();
    }
    __syncthreads();
    if (t < ntiles) issue1(0);
    int it = 0;
    // MMA completions: one thread polls the mbarrier and the CTA barrier (a lane shuffle for the
    // per-warp lo wait) hands on its result
    for (; t < ntiles && ok; t += gridDim.x, ++it) {
        const int64_t s0 = t * SPT;
        cp_async_wait_group<0>();                    // this tile's d_h0c rows
        ok = __syncthreads_and(tid == 0 ? umma::mbar_wait(mbar, phase) : true);   // one poller
        phase ^= 1u;
        if (!ok) {
            flag_timeout(p.err, 1);
            break;
        }
        const int64_t tn = t + gridDim.x;
        const int cb = DW ? (it & 1) : 0, nb = DW ? ((it + 1) & 1) : 0;   // this tile's / the next tile's A
        umma::fence_after_sync();
        // the next tile's A tile, under the d_pre epilogue: MMA1 of tile t has completed, and with DW
        // it goes to the other buffer, whose last readers (the previous tile's lo dW0 MMAs) completed
        // before MMA1(t).  (Issued after MMA2 instead, its writes slowed the shared-memory-bound dW0
        // MMAs.)
        if (tn < ntiles && tid == 0) load_a(tn, nb);
        if (tn < ntiles) prologue_load(tn, pin);     // consumed under MMA2
        // (2) d_pre = (d f * w_head + [centre] d_h0c) * softplus'(pre) -> TMEM (hi, lo) and d_pre0
        uint8_t* stg = stage_s + warp * BWD_STAGE_BYTES;
        const CUtensorMap* tm_pre = q == 3 ? &tm_pre30 : &tm_pre32;
        const CUtensorMap* tm_enc = q == 3 ? &tm_enc30 : &tm_enc32;
        const int y0 = (int)(t * TILE_ROWS) + q * 32;
        if (lane == 0) umma::bulk_wait_read0();      // the previous tile's d_enc store has read the buffer
        __syncwarp();
        {
            // dead rows (past Ns, and rows 126-127) get d f = 0 and no d_h0c: their
            // pre-activations are finite, so their d_pre and head terms come out 0
            const int64_t s = s0 + sl_row;
            const bool live = row < SPT * EVALS && s < p.Ns;
            const float df = live ? df_s[(it & 1) * (EVALS * SPT) + row] : 0.0f;
            const bool centre = live && e_row == 0;
            const SoftplusK spk = softplus_k(p.beta);
            // the next chunk's TMEM load is in flight while this chunk is processed
            uint32_t rn[16];
            umma::tmem_ld16_nowait(umma::taddr(tmem, q * 32, part * 64), rn);
            umma::tmem_ld_wait16(rn);
#pragma unroll 1
            for (int c0 = part * 64; c0 < part * 64 + 64; c0 += 16) {
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(rn[j]);
                const bool more = c0 + 16 < part * 64 + 64;
                if (more) umma::tmem_ld16_nowait(umma::taddr(tmem, q * 32, c0 + 16), rn);
                float dh0[16];
                if (centre) {
                    const float4* src = reinterpret_cast<const float4*>(dh0_s + sl_row * DH0_LD + c0);
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float4 f = src[j];
                        dh0[4 * j] = f.x; dh0[4 * j + 1] = f.y; dh0[4 * j + 2] = f.z; dh0[4 * j + 3] = f.w;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j) dh0[j] = 0.0f;
                }
                float hc[16];   // d f * h per column: d w_head = sum over rows
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    float hval, sg;
                    softplus_fast(v[j], spk, hval, sg);
                    v[j] = fmaf(df, wh_s[c0 + j], dh0[j]) * sg;
                    hc[j] = df * hval;
                }
                {
                    const float colsum = warp_column_sum16(hc, lane);
                    if (lane < 16 && colsum != 0.0f) atomicAdd(&dwh_s[c0 + lane], colsum);
                }
                uint32_t hi[8], lo[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const __half2 h2 = __floats2half2_rn(v[2 * i], v[2 * i + 1]);
                    const float2 b = __half22float2(h2);
                    const __half2 l2 = __floats2half2_rn(v[2 * i] - b.x, v[2 * i + 1] - b.y);
                    hi[i] = *reinterpret_cast<const uint32_t*>(&h2);
                    lo[i] = *reinterpret_cast<const uint32_t*>(&l2);
                }
                if (more) umma::tmem_ld_wait16(rn);
                umma::tmem_st8(umma::taddr(t_hi(c0 >> 4), q * 32, 0), hi);
                umma::tmem_st8(umma::taddr(t_lo(c0 >> 4), q * 32, 0), lo);
                // d_pre0 (hi) into the staging rows; dead samples store zeros (their x0ext
                // rows are zero too).  128-byte swizzle: 16-byte unit u of row r sits at u ^ (r & 7)
                const int u = (c0 - part * 64) >> 3;
                *reinterpret_cast<uint4*>(stg + lane * 128 + ((u ^ (lane & 7)) * 16)) =
                    make_uint4(hi[0], hi[1], hi[2], hi[3]);
                *reinterpret_cast<uint4*>(stg + lane * 128 + (((u + 1) ^ (lane & 7)) * 16)) =
                    make_uint4(hi[4], hi[5], hi[6], hi[7]);
            }
        }
        umma::fence_proxy_async_smem();
        __syncwarp();
        if (!DW && lane == 0) {
            umma::tma_store_2d(tm_pre, part * 64, y0, stg);
            umma::bulk_commit();
        }
        umma::tmem_wait_st();
        if (!DW && p.d_pre0_lo) {
            // d_pre's lo half to d_pre0_lo through the same staging rows, read back from TMEM
            // once the hi store has read them (the layer-0 weight gradient needs the pair)
            if (lane == 0) umma::bulk_wait_read0();
            __syncwarp();
#pragma unroll 1
            for (int c0 = part * 64; c0 < part * 64 + 64; c0 += 16) {
                float f[8];
                umma::tmem_ld8(umma::taddr(t_lo(c0 >> 4), q * 32, 0), f);
                const int u = (c0 - part * 64) >> 3;
                *reinterpret_cast<uint4*>(stg + lane * 128 + ((u ^ (lane & 7)) * 16)) =
                    make_uint4(__float_as_uint(f[0]), __float_as_uint(f[1]), __float_as_uint(f[2]),
                               __float_as_uint(f[3]));
                *reinterpret_cast<uint4*>(stg + lane * 128 + (((u + 1) ^ (lane & 7)) * 16)) =
                    make_uint4(__float_as_uint(f[4]), __float_as_uint(f[5]), __float_as_uint(f[6]),
                               __float_as_uint(f[7]));
            }
            umma::fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                umma::tma_store_2d(q == 3 ? &tm_plo30 : &tm_plo32, part * 64, y0, stg);
                umma::bulk_commit();
            }
        }
        umma::fence_before_sync();
        __syncthreads();
        // (3) d_enc = d_pre * W0e  (MMA2: A = d_pre [128 x 256] in TMEM; B = W0e read
        // MN-major from MMA1's w0b tile: the core matrix of hidden rows 8g..8g+7 and
        // feature columns 8c..8c+7 sits at g * KB * 16 + c * 128 bytes)
        {
            // descriptor bases from converged code (warp-uniform values); the elected lane adds
            // constant multiples of row_step per MMA
            const uint64_t row_step = desc_step(2u * KB * 16u);   // 16 rows (dW0's B) / 16 hidden units (MMA2's B)
            const uint64_t d_stage = umma::make_desc_sw128_mn(umma::smem_u32(stage_s), 16384u, 1024u);
            const uint32_t id_dw = umma::idesc_f16_mn(TILE_M, KB);
            const uint64_t d_w = umma::make_desc(w_addr, (uint32_t)KB * 16u, 128u);
            const uint64_t bx = umma::make_desc(a_addr(cb), KB * 16u, 128u);
            const uint64_t bx3 = umma::make_desc(a3_addr(cb), KB * 16u, 128u);
            if (warp == 0 && umma::elect_one()) {      // (warp 0 reconverges below)
                // MMA2 and (DW) the two dW0 hidden halves go out in turn, each accumulator in its own order
                umma::fence_after_sync();
#pragma unroll
                for (int i = 0; i < 2 * (HID / 16); ++i) {   // d_pre lo chunks first (smaller addends), then hi
                    const int ks = i & (HID / 16 - 1);
                    umma::mma_f16_ta(t_enc, i < HID / 16 ? t_lo(ks) : t_hi(ks), d_w + ks * row_step, idesc2,
                                     i > 0 ? 1u : 0u);
                    if (DW && i < 2 * (TILE_M / 16)) {
                        // dW0[h] += d_pre^T [x hi | tail] (i < 8), then += d_pre^T [x lo | 0].
                        // A (hidden half h = staging parts 2h, 2h + 1): atoms of 64 units x 8 rows, next
                        // 64 units 16 KB on, next 8 rows 1 KB on; B (the tile's rows, MN-major): next 8
                        // rows KB*16 bytes on, next 8 features 128 bytes on.
                        const int k8 = i & (TILE_M / 16 - 1);
                        const uint64_t bd = (i < TILE_M / 16 ? bx : bx3) + k8 * row_step;
                        const uint32_t acc0 = (dw_first && i == 0) ? 0u : 1u;
#pragma unroll
                        for (int h = 0; h < 2; ++h)
                            umma::mma_f16(t_dw + (uint32_t)(h * KB), d_stage + desc_step(h * 32768 + k8 * 2048), bd,
                                          id_dw, acc0);
                    }
                }
                umma::mma_commit(mbar);
            }
        }
        if (warp == 0) __syncwarp();                 // the issuing lane rejoins its warp before the barrier
        if constexpr (DW) dw_first = false;
        if (tn < ntiles) {
            // the next tile's d_h0c rows, issued while every thread waits for MMA2 (copies landing
            // under the d_pre epilogue stretch it)
            stage_dh0(tn);                           // every warp has read this tile's d_h0c rows
            prologue_ray(tn, pin);
            prologue_finish(tn, pin, (it + 1) & 1);  // the other df buffer, under the MMAs
        }
        ok = __syncthreads_and(tid == 0 ? umma::mbar_wait(mbar, phase) : true);   // one poller
        phase ^= 1u;
        if (!ok) {
            flag_timeout(p.err, 1);
            break;
        }
        umma::fence_after_sync();
        if constexpr (DW) {
            // dW0[h] += d_pre lo^T [x hi | tail]: the hi MMAs have completed with MMA2, so the
            // staging rows take d_pre's lo half, read back from TMEM before the next tile's MMA1
            // overwrites it.  The +eps / -eps taps carry large, nearly cancelling d_pre, and a
            // single fp16 rounding of d_pre in dW0 would leave ~1e-3 of it behind.
#pragma unroll 1
            for (int c0 = part * 64; c0 < part * 64 + 64; c0 += 16) {
                float f[8];
                umma::tmem_ld8(umma::taddr(t_lo(c0 >> 4), q * 32, 0), f);
                const int u = (c0 - part * 64) >> 3;
                *reinterpret_cast<uint4*>(stg + lane * 128 + ((u ^ (lane & 7)) * 16)) =
                    make_uint4(__float_as_uint(f[0]), __float_as_uint(f[1]), __float_as_uint(f[2]),
                               __float_as_uint(f[3]));
                *reinterpret_cast<uint4*>(stg + lane * 128 + (((u + 1) ^ (lane & 7)) * 16)) =
                    make_uint4(__float_as_uint(f[4]), __float_as_uint(f[5]), __float_as_uint(f[6]),
                               __float_as_uint(f[7]));
            }
            umma::fence_proxy_async_smem();
            umma::fence_before_sync();
            __syncthreads();
            const uint64_t row_step = desc_step(2u * KB * 16u);
            const uint64_t d_stage = umma::make_desc_sw128_mn(umma::smem_u32(stage_s), 16384u, 1024u);
            const uint32_t id_dw = umma::idesc_f16_mn(TILE_M, KB);
            const uint64_t bx = umma::make_desc(a_addr(cb), KB * 16u, 128u);
            if (warp == 0 && umma::elect_one()) {
                umma::fence_after_sync();
#pragma unroll
                for (int ks = 0; ks < TILE_M / 16; ++ks)     // the two hidden halves' chains in turn
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        umma::mma_f16(t_dw + (uint32_t)(h * KB), d_stage + desc_step(h * 32768 + ks * 2048),
                                      bx + ks * row_step, id_dw, 1u);
                umma::mma_commit(mbar_lo);
            }
            if (warp == 0) __syncwarp();
        }
        if (DW && tn < ntiles) issue1(nb);           // D1 is free: MMA2 has read d_pre
        // (4) d_enc rows to global for k_field_scatter: 16-column chunks dealt in turn
        // to the four warps of a lane quadrant (K0 <= 128: at most two per warp, one
        // 2 KB half of the staging buffer each; 64-byte swizzle: unit j of row r at j ^ ((r >> 1) & 3))
        if (lane == 0) umma::bulk_wait_read0();      // the d_pre0 store (or, DW, dW0's MMAs) has read it
        if constexpr (DW) {
            // the lo dW0 MMAs read the staging rows: wait for them before d_enc goes through
            // (a timed-out wait skips this warp's stores; the tile's closing barrier ends the loop)
            ok = __shfl_sync(0xffffffffu, lane == 0 ? (int)umma::mbar_wait(mbar_lo, phase_lo) : 0, 0) != 0;
            phase_lo ^= 1u;
            if (!ok && lane == 0) flag_timeout(p.err, 1);
        }
        __syncwarp();
        for (int c0 = part * 16, i = 0; ok && c0 < K0; c0 += 64, ++i) {
            float v[16];
            umma::tmem_ld16(umma::taddr(t_enc, q * 32, c0), v);
            uint8_t* eb = stg + i * 2048;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                *reinterpret_cast<float4*>(eb + lane * 64 + ((j ^ ((lane >> 1) & 3)) * 16)) =
                    make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            umma::fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                umma::tma_store_2d(tm_enc, c0, y0, eb);
                umma::bulk_commit();
            }
        }
        umma::fence_before_sync();
        ok = __syncthreads_and(ok);   // the TMEM accumulator of tile t read; tile tn's A tile and d f in place
        if (ok && !DW && tn < ntiles) issue1(nb);
    }
    cp_async_wait_all();
    if (tid == 0 && a_pending && !umma::mbar_wait(mbar_a, phase_a)) flag_timeout(p.err, 1);   // a load left in flight
    if (lane == 0) umma::bulk_wait0();               // this warp's TMA stores have completed
    umma::fence_before_sync();
    __syncthreads();
    if constexpr (DW) {
        // the CTA's dW0 (complete: the last tile's lo MMAs were waited for): warps with part 2h, 2h + 1
        // read hidden half h, one half of its KB columns each
        if (!dw_first && ok) {
            umma::fence_after_sync();
            const int h = part >> 1, half_cols = KB / 2, cbeg = (part & 1) * half_cols;
            float* dst = p.d_w0 + (int64_t)(h * 128 + q * 32 + lane) * KB;
            for (int c = cbeg; c < cbeg + half_cols; c += 8) {
                float v[8];
                umma::tmem_ld8(umma::taddr(t_dw + (uint32_t)(h * KB), q * 32, c), v);
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (v[j] != 0.0f) atomicAdd(dst + c + j, v[j]);
            }
        }
        umma::fence_before_sync();
        __syncthreads();
    }
    for (int i = tid; i < HID; i += BWD_THREADS)
        if (dwh_s[i] != 0.0f) atomicAdd(&p.d_whead[i], dwh_s[i]);
    dbh = warp_sum(dbh);
    if (lane == 0 && dbh != 0.0f) atomicAdd(p.d_bhead, dbh);
    if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// SDF-only evaluation at arbitrary points or on a lattice block (forward only):
// NeuralSDF.sdf (modules.py:73-74) for mesh extraction (mesh.py:33-35, with the
// sign flip of scripts/extract_mesh.py:85) and for the sampler's no-grad
// evaluations (model.py:238, 245).  Tile = 128 points, one evaluation each.

struct SdfPointsArgs {
    int64_t M;
    const float* pts;          // [M, 3] or NULL for lattice mode
    const float* ax;           // lattice axes: x [nx], y [ny], z [nz]
    const float* ay;
    const float* az;
    int nx, ny, nz;
    float sign;                // +1, or -1 for the mesh's negated field
    float* out;                // [M]
};

template <int F>
__global__ void __launch_bounds__(FIELD_THREADS, 1) k_sdf_points(FieldParams p, SdfPointsArgs q) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int K0 = p.K0;
    uint8_t* w_s = smem;
    uint8_t* a_s = w_s + HID * K0 * 2;
    uint8_t* a2_s = a_s + TILE_M * K0 * 2;
    float* w0x_s = reinterpret_cast<float*>(a2_s + TILE_M * K0 * 2);
    float* b0_s = w0x_s + HID * 3;
    float* wh_s = b0_s + HID;
    float* part_s = wh_s + HID;                                 // [2][128]
    uint64_t* mbar = reinterpret_cast<uint64_t*>(part_s + 2 * TILE_M);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    stage_rows_kmajor(w_s, (const __half*)p.w0e, 0, HID, K0, K0, tid, FIELD_THREADS, HID);
    for (int i = tid; i < HID * 3; i += FIELD_THREADS) w0x_s[i] = p.w0x[i];
    for (int i = tid; i < HID; i += FIELD_THREADS) {
        b0_s[i] = p.b0[i];
        wh_s[i] = p.whead[i];
    }
    for (int i = tid; i < 2 * TILE_M * K0 / 8; i += FIELD_THREADS)
        reinterpret_cast<uint4*>(a_s)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        umma::mbar_init(mbar, 1);
        umma::fence_mbar_init();
    }
    if (warp == 0) {
        umma::tmem_alloc(tslot, HID);
        umma::tmem_relinquish();
    }
    cp_async_wait_all();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = umma::idesc_f16(TILE_M, HID);
    const uint32_t a_addr = umma::smem_u32(a_s), a2_addr = umma::smem_u32(a2_s), w_addr = umma::smem_u32(w_s);
    const float bhead = p.bhead[0];
    const SoftplusK spk = softplus_k(p.beta);
    const int64_t ntiles = (q.M + TILE_M - 1) / TILE_M;
    const int qd = warp & 3, half = warp >> 2;
    const int row = qd * 32 + lane;
    uint32_t phase = 0;
    auto point = [&](int64_t m, float* x) {
        if (q.pts) {
            x[0] = q.pts[3 * m]; x[1] = q.pts[3 * m + 1]; x[2] = q.pts[3 * m + 2];
        } else {
            const int k = (int)(m % q.nz), j = (int)((m / q.nz) % q.ny), i = (int)(m / ((int64_t)q.ny * q.nz));
            x[0] = q.ax[i]; x[1] = q.ay[j]; x[2] = q.az[k];
        }
    };
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t m0 = t * TILE_M;
        for (int i = tid; i < TILE_M * p.active; i += FIELD_THREADS) {
            const int r = i / p.active, l = i % p.active;
            const int64_t m = m0 + r;
            float v[F];
            if (m < q.M) {
                float x[3], xu[3];
                point(m, x);
#pragma unroll
                for (int k = 0; k < 3; ++k) xu[k] = to_unit(x[k]);
                gather_level<F>(p, xu, l, v);
            } else {
#pragma unroll
                for (int f = 0; f < F; ++f) v[f] = 0.0f;
            }
            write_tile_features<F>(a_s, a2_s, r, l, K0, v);
        }
        umma::fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after_sync();
            issue_tile_mma(tmem, a2_addr, w_addr, K0, idesc);          // residuals first
            issue_tile_mma(tmem, a_addr, w_addr, K0, idesc, true);
            umma::mma_commit(mbar);
        }
        const bool ok = __syncthreads_and(umma::mbar_wait(mbar, phase));
        phase ^= 1u;
        if (!ok) {
            flag_timeout(p.err, 1);
            break;
        }
        umma::fence_after_sync();
        const int64_t m = m0 + row;
        float x[3] = {0.f, 0.f, 0.f};
        if (m < q.M) point(m, x);
        float part4[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
        for (int c0 = half * 128; c0 < half * 128 + 128; c0 += 32) {
            float v[32];
            umma::tmem_ld32(umma::taddr(tmem, qd * 32, c0), v);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int n = c0 + j;
                const float z = v[j] + w0x_s[3 * n] * x[0] + w0x_s[3 * n + 1] * x[1] + w0x_s[3 * n + 2] * x[2] + b0_s[n];
                part4[j & 3] = fmaf(wh_s[n], softplus_fast_h(z, spk), part4[j & 3]);
            }
        }
        part_s[half * TILE_M + row] = (part4[0] + part4[1]) + (part4[2] + part4[3]);
        umma::fence_before_sync();
        __syncthreads();
        if (tid < TILE_M && m0 + tid < q.M) q.out[m0 + tid] = q.sign * (part_s[tid] + part_s[TILE_M + tid] + bhead);
        __syncthreads();
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, HID);
}

static int num_sms() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

template <int TAPS>
static size_t fwd_smem(int K0) {
    const size_t KB = (size_t)K0 + 16;
    return (size_t)HID * KB * 2 + (size_t)TILE_M * (KB + K0) * 2 +
           (HID + 2 * TILE_M + FWD_SDF_FLOATS) * 4 + 24 +
           (size_t)FWD_RING * TapTile<TAPS>::SPT * sizeof(FwdSample);
}
template <int TAPS>
static size_t bwd_smem(int K0, bool dw) {
    const size_t KB = (size_t)K0 + 16;
    const size_t need = (size_t)(BWD_THREADS / 32) * BWD_STAGE_BYTES + (size_t)HID * KB * 2 +
                        (size_t)TILE_M * (KB + (dw ? KB : K0)) * 2 * (dw ? 2 : 1) +
                        (2 * HID + TapTile<TAPS>::DF_FLOATS + TapTile<TAPS>::SPT * DH0_LD) * 4 + 32;
    return need > BWD_SMEM_FLOOR ? need : BWD_SMEM_FLOOR;
}

// The field's four kernels, in step order.  `which`: bit 0 the hash-grid gather,
// bit 1 the MLP forward, bit 2 the MLP backward, bit 3 the table-gradient scatter.
enum FieldKernels : int { FK_GATHER = 1, FK_MLP_FWD = 2, FK_MLP_BWD = 4, FK_SCATTER = 8 };

// TMA maps of the x0ext rows as the field MLP's A tiles (8-row groups in the core-matrix layout):
// features hi | tail (K0 + 16 columns), and features lo into a tile lo_cols wide (K0, or K0 + 16
// whose last two chunks lie past the tensor and arrive as zeros)
static int x0ext_maps(const FieldParams& p, int64_t rows, int lo_cols, CUtensorMap* hi, CUtensorMap* lo) {
    const int KX = 2 * p.K0 + 16;
    if (rows <= 0) rows = 1;                          // (no tile is loaded)
    if (int st = tensor_map_kmajor_groups(hi, p.x0ext, rows, (p.K0 + 16) / 8, KX, (p.K0 + 16) / 8, "x0ext hi"))
        return st;
    return tensor_map_kmajor_groups(lo, (const __half*)p.x0ext + p.K0 + 16, rows, p.K0 / 8, KX, lo_cols / 8,
                                    "x0ext lo");
}

template <int F, int TAPS>
static int launch_field(const FieldParams& p, int which, cudaStream_t s) {
    constexpr int EVALS = TapTile<TAPS>::EVALS, SPT = TapTile<TAPS>::SPT, TILE_ROWS = TapTile<TAPS>::ROWS;
    constexpr int LAST_BOX = TILE_ROWS - 96;          // rows of a tile's last 32-row lane quadrant
    const int64_t ntiles = (p.Ns + SPT - 1) / SPT;
    // largest thread index: gather ntiles * rows per tile * active, scatter Ns * active * 8
    const int64_t gather_items = ntiles * (SPT * EVALS) * (int64_t)p.active;
    const int64_t scatter_items = p.Ns * (int64_t)p.active * 8;
    if ((gather_items > scatter_items ? gather_items : scatter_items) >= ((int64_t)1 << 32)) {
        set_error("%lld samples x %d levels exceed the 32-bit index range of one launch", (long long)p.Ns,
                  p.active);
        return GBSDF_ERR_UNSUPPORTED;
    }
    if (which & FK_GATHER) {
        const int64_t items = ntiles * (SPT * EVALS) * p.active;
        k_field_gather<F, TAPS><<<(unsigned)((items + 255) / 256), 256, 0, s>>>(p, ntiles);
        if (int st = launch_status("field gather")) return st;
    }
    if (which & FK_MLP_FWD) {
        const size_t smem = fwd_smem<TAPS>(p.K0);
        if (smem > 227 * 1024) {
            set_error("field forward needs %zu B of shared memory", smem);
            return GBSDF_ERR_UNSUPPORTED;
        }
        // p.fwd_ctas (a tuning choice): resident CTAs per SM to launch, 1 or 2 (0 = 2)
        int64_t grid = num_sms() * (p.fwd_ctas == 1 ? 1 : FWD_CTAS_PER_SM);
        if (grid > ntiles) grid = ntiles;
        CUtensorMap tm_xhi, tm_xlo;
        if (int st = x0ext_maps(p, ntiles * TILE_ROWS, p.K0, &tm_xhi, &tm_xlo)) return st;
        allow_max_smem(k_field_fwd<F, TAPS>);
        k_field_fwd<F, TAPS><<<(unsigned)grid, FIELD_THREADS, smem, s>>>(p, tm_xhi, tm_xlo);
        if (int st = launch_status("field forward")) return st;
    }
    if (which & FK_MLP_BWD) {
        const bool dw = p.d_w0 != nullptr;
        const size_t smem = bwd_smem<TAPS>(p.K0, dw);
        if (smem > 227 * 1024) {
            set_error("field backward needs %zu B of shared memory", smem);
            return GBSDF_ERR_UNSUPPORTED;
        }
        // d_pre0 [rows, 256] fp16 (without d_w0) and d_enc [rows, K0] fp32 as TMA store targets
        // (rows = tiles x 126 or 125); with d_w0 the d_pre0 maps are never used and describe
        // d_enc's memory.  The '30' maps are the last lane quadrant's LAST_BOX-row boxes.
        const int64_t rows = ntiles * TILE_ROWS;
        if (rows >= ((int64_t)1 << 31)) {
            set_error("%lld backward rows exceed the TMA coordinate range", (long long)rows);
            return GBSDF_ERR_UNSUPPORTED;
        }
        CUtensorMap tm_pre32, tm_pre30, tm_enc32, tm_enc30, tm_plo32, tm_plo30;
        const CUtensorMapL2promotion l2n = CU_TENSOR_MAP_L2_PROMOTION_NONE;
        if (!dw) {
            if (int st = tensor_map_2d(&tm_pre32, false, p.d_pre0, rows, HID, HID, 64, 32,
                                       CU_TENSOR_MAP_SWIZZLE_128B, l2n, "d_pre0"))
                return st;
            if (int st = tensor_map_2d(&tm_pre30, false, p.d_pre0, rows, HID, HID, 64, LAST_BOX,
                                       CU_TENSOR_MAP_SWIZZLE_128B, l2n, "d_pre0"))
                return st;
        }
        if (int st = tensor_map_2d(&tm_enc32, true, p.d_enc, rows, p.K0, p.K0, 16, 32, CU_TENSOR_MAP_SWIZZLE_64B, l2n,
                                   "d_enc"))
            return st;
        if (int st = tensor_map_2d(&tm_enc30, true, p.d_enc, rows, p.K0, p.K0, 16, LAST_BOX, CU_TENSOR_MAP_SWIZZLE_64B, l2n,
                                   "d_enc"))
            return st;
        if (dw) tm_pre32 = tm_pre30 = tm_enc32;
        if (!dw && p.d_pre0_lo) {
            if (int st = tensor_map_2d(&tm_plo32, false, p.d_pre0_lo, rows, HID, HID, 64, 32,
                                       CU_TENSOR_MAP_SWIZZLE_128B, l2n, "d_pre0_lo"))
                return st;
            if (int st = tensor_map_2d(&tm_plo30, false, p.d_pre0_lo, rows, HID, HID, 64, LAST_BOX,
                                       CU_TENSOR_MAP_SWIZZLE_128B, l2n, "d_pre0_lo"))
                return st;
        } else {
            tm_plo32 = tm_plo30 = tm_pre32;              // unused
        }
        CUtensorMap tm_xhi, tm_xlo;
        if (int st = x0ext_maps(p, rows, dw ? p.K0 + 16 : p.K0, &tm_xhi, &tm_xlo)) return st;
        int64_t grid = num_sms();
        if (grid > ntiles) grid = ntiles;
        if (dw) {
            allow_max_smem(k_field_bwd<F, true, TAPS>);
            k_field_bwd<F, true, TAPS><<<(unsigned)grid, BWD_THREADS, smem, s>>>(p, tm_pre32, tm_pre30, tm_enc32, tm_enc30,
                                                                             tm_plo32, tm_plo30, tm_xhi, tm_xlo);
        } else {
            allow_max_smem(k_field_bwd<F, false, TAPS>);
            k_field_bwd<F, false, TAPS><<<(unsigned)grid, BWD_THREADS, smem, s>>>(p, tm_pre32, tm_pre30, tm_enc32, tm_enc30,
                                                                              tm_plo32, tm_plo30, tm_xhi, tm_xlo);
        }
        if (int st = launch_status("field backward")) return st;
    }
    if (which & FK_SCATTER) {
        const int64_t items = p.Ns * p.active;
        if (p.d_table_fix) {
            // deterministic mode: integer accumulation into the caller's buffer, then into d_table
            const int64_t n = (int64_t)p.grid.offset[p.grid.n_levels] * F;
            if (cudaMemsetAsync(p.d_table_fix, 0, (size_t)n * 8, s) != cudaSuccess) {
                set_error("clearing d_table_fix failed");
                return GBSDF_ERR_CUDA;
            }
            k_field_scatter<F, SCATTER_CPT, TAPS, true><<<(unsigned)((items + 255) / 256), 256, 0, s>>>(p);
            if (int st = launch_status("field scatter (deterministic)")) return st;
            k_fixed_to_table<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, p.d_table_fix, p.d_table);
        } else {
            // p.scatter_cpt (a tuning choice, 8-feature fields): table corners per pass, 2, 4 or 8 (0 = 2)
            const unsigned blocks = (unsigned)((items + 255) / 256);
            if (F == 8 && p.scatter_cpt == 4)
                k_field_scatter<F, 4, TAPS, false><<<blocks, 256, 0, s>>>(p);
            else if (F == 8 && p.scatter_cpt == 8)
                k_field_scatter<F, 8, TAPS, false><<<blocks, 256, 0, s>>>(p);
            else
                k_field_scatter<F, SCATTER_CPT, TAPS, false><<<blocks, 256, 0, s>>>(p);
        }
        if (int st = launch_status("field scatter")) return st;
    }
    return GBSDF_OK;
}

static int check_field_weights(const FieldParams& p) {
    GBSDF_CHECK_ARG(p.active >= 1 && p.active <= p.grid.n_levels, "active levels %d", p.active);
    const int F = p.grid.n_features;
    GBSDF_CHECK_ARG(F == 2 || F == 4 || F == 8, "n_features %d unsupported by the fused field", F);
    GBSDF_CHECK_ARG(p.K0 % 16 == 0 && p.K0 >= p.active * F && p.K0 <= 128, "K0 %d", p.K0);
    GBSDF_CHECK_ARG(p.table && p.w0e && p.w0x && p.b0 && p.whead && p.bhead, "NULL weight pointer");
    GBSDF_CHECK_ARG(aligned(p.table, 16) && aligned(p.w0e, 16), "table / w0e alignment");
    return GBSDF_OK;
}

static int check_field(const FieldParams& p) {
    GBSDF_CHECK_ARG(p.Ns >= 0, "Ns < 0");
    GBSDF_CHECK_ARG(p.taps == 0 || p.taps == 4 || p.taps == 6, "taps %d (4 or 6; 0 means 6)", p.taps);
    GBSDF_CHECK_ARG(p.scatter_cpt == 0 || p.scatter_cpt == 2 || p.scatter_cpt == 4 || p.scatter_cpt == 8,
                    "scatter_cpt %d (2, 4 or 8; 0 = 2)", p.scatter_cpt);
    GBSDF_CHECK_ARG(p.fwd_ctas >= 0 && p.fwd_ctas <= 2, "fwd_ctas %d (1 or 2; 0 = 2)", p.fwd_ctas);
    if (int st = check_field_weights(p)) return st;
    GBSDF_CHECK_ARG(p.S > 0 || p.sample_ray, "need S > 0 or sample_ray");
    GBSDF_CHECK_ARG(p.center && p.ray_unit && p.dists, "NULL ray pointer");
    return GBSDF_OK;
}

}  // namespace gbsdf

using namespace gbsdf;

extern "C" size_t gbsdf_field_args_size(void) { return sizeof(gbsdf_field_args); }

template <int TAPS>
static int field_dispatch_taps(const FieldParams& p, int which, void* stream) {
    switch (p.grid.n_features) {
        case 2: return launch_field<2, TAPS>(p, which, as_stream(stream));
        case 4: return launch_field<4, TAPS>(p, which, as_stream(stream));
        default: return launch_field<8, TAPS>(p, which, as_stream(stream));
    }
}
static int field_dispatch(const FieldParams& p, int which, void* stream) {
    return p.taps == 4 ? field_dispatch_taps<4>(p, which, stream) : field_dispatch_taps<6>(p, which, stream);
}

static int check_fwd(const FieldParams& p, int which) {
    if (int st = check_field(p)) return st;
    GBSDF_CHECK_ARG(p.x0ext && aligned(p.x0ext, 16), "x0ext missing or misaligned (16 bytes: its rows are loaded by TMA)");
    if (which & FK_MLP_FWD) {
        GBSDF_CHECK_ARG(p.sdf && p.grad && p.hess && p.h0c, "NULL output");
        GBSDF_CHECK_ARG(p.w0b && aligned(p.w0b, 16), "w0b (fp16 [256, K0 + 16]) missing or misaligned");
        GBSDF_CHECK_ARG(p.ld_h0c == 0 || (p.ld_h0c >= HID && p.ld_h0c % 8 == 0), "ld_h0c %d", p.ld_h0c);
        GBSDF_CHECK_ARG(!p.xc || (p.ldxc % 16 == 0 && p.ldxc - HID >= 23 + p.app_dim && p.ldxc - HID <= 48),
                        "xc leading dimension %d (needs 256 + 23 + app_dim <= ldxc <= 304, multiple of 16)", p.ldxc);
        GBSDF_CHECK_ARG(!p.xc || p.app_dim == 0 || (p.app_table && p.app_idx), "appearance table / index missing");
        GBSDF_CHECK_ARG(!p.h0c_lo || aligned(p.h0c_lo, 16), "h0c_lo misaligned");
        GBSDF_CHECK_ARG(!p.xc_lo || (p.xc && aligned(p.xc_lo, 16)), "xc_lo needs xc and 16-byte alignment");
    }
    return GBSDF_OK;
}

static int check_bwd(const FieldParams& p, int which) {
    if (int st = check_field(p)) return st;
    GBSDF_CHECK_ARG(p.d_enc && aligned(p.d_enc, 16), "d_enc missing or misaligned");
    if (which & FK_MLP_BWD) {
        GBSDF_CHECK_ARG(p.w0b && aligned(p.w0b, 16), "w0b (fp16 [256, K0 + 16]) missing or misaligned");
        GBSDF_CHECK_ARG(p.grad && p.d_sdf && p.d_grad && p.d_hess && p.d_xc && p.d_h0c && p.x0ext && p.d_whead &&
                            p.d_bhead,
                        "NULL pointer");
        GBSDF_CHECK_ARG(p.d_w0 || (p.d_pre0 && aligned(p.d_pre0, 16)), "d_pre0 missing or misaligned (no d_w0)");
        GBSDF_CHECK_ARG(!p.d_w0 || p.K0 <= 64, "d_w0 needs K0 <= 64 (K0 %d): pass d_pre0 instead", p.K0);
        GBSDF_CHECK_ARG(aligned(p.d_h0c, 16), "d_h0c alignment");
        GBSDF_CHECK_ARG(!p.d_pre0_lo || aligned(p.d_pre0_lo, 16), "d_pre0_lo alignment");
        GBSDF_CHECK_ARG(aligned(p.x0ext, 16), "x0ext misaligned (16 bytes: its rows are loaded by TMA)");
    }
    if (which & FK_SCATTER) {
        GBSDF_CHECK_ARG(p.d_table && aligned(p.d_table, 16), "d_table missing or misaligned");
        GBSDF_CHECK_ARG(!p.d_table_fix || aligned(p.d_table_fix, 16), "d_table_fix misaligned");
    }
    return GBSDF_OK;
}

static int field_call(const gbsdf_field_args* params, int which, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(params != nullptr, "params NULL");
    const FieldParams& p = *params;
    const bool fwd = (which & (FK_GATHER | FK_MLP_FWD)) != 0;
    if (int st = fwd ? check_fwd(p, which) : check_bwd(p, which)) return st;
    if (p.Ns == 0) return GBSDF_OK;
    return field_dispatch(p, which, stream);
}

extern "C" int gbsdf_field_fwd(const gbsdf_field_args* params, void* stream) {
    return field_call(params, FK_GATHER | FK_MLP_FWD, stream);
}
extern "C" int gbsdf_field_bwd(const gbsdf_field_args* params, void* stream) {
    return field_call(params, FK_MLP_BWD | FK_SCATTER, stream);
}
extern "C" int gbsdf_field_encode(const gbsdf_field_args* params, void* stream) {
    return field_call(params, FK_GATHER, stream);
}
extern "C" int gbsdf_field_mlp_fwd(const gbsdf_field_args* params, void* stream) {
    return field_call(params, FK_MLP_FWD, stream);
}
extern "C" int gbsdf_field_mlp_bwd(const gbsdf_field_args* params, void* stream) {
    return field_call(params, FK_MLP_BWD, stream);
}
extern "C" int gbsdf_field_scatter(const gbsdf_field_args* params, void* stream) {
    return field_call(params, FK_SCATTER, stream);
}

extern "C" int gbsdf_field_workspace_size(int64_t Ns, int32_t K0, int32_t taps, int32_t deterministic,
                                          const gbsdf_grid* grid, gbsdf_field_workspace* out) {
    clear_error();
    GBSDF_CHECK_ARG(out != nullptr && Ns >= 0, "bad arguments");
    GBSDF_CHECK_ARG(K0 % 16 == 0 && K0 >= 16 && K0 <= 128, "K0 %d", K0);
    GBSDF_CHECK_ARG(taps == 0 || taps == 4 || taps == 6, "taps %d", taps);
    GBSDF_CHECK_ARG(!deterministic || grid != nullptr, "the deterministic scatter's size needs the grid");
    const int spt = taps == 4 ? TapTile<4>::SPT : TapTile<6>::SPT;
    const int rows_per_tile = taps == 4 ? TapTile<4>::ROWS : TapTile<6>::ROWS;
    const int64_t rows = (Ns + spt - 1) / spt * rows_per_tile;
    out->rows = rows;
    out->x0ext_bytes = (size_t)rows * (2 * K0 + 16) * 2;
    out->d_enc_bytes = (size_t)rows * K0 * 4;
    out->d_w0_bytes = K0 <= 64 ? (size_t)HID * (K0 + 16) * 4 : 0;
    out->d_pre0_bytes = K0 > 64 ? (size_t)rows * HID * 2 : 0;
    out->d_table_fix_bytes = deterministic ? (size_t)grid->offset[grid->n_levels] * grid->n_features * 8 : 0;
    return GBSDF_OK;
}

extern "C" int gbsdf_sdf_points(const gbsdf_field_args* params, int64_t M, const float* pts, const float* ax,
                                const float* ay, const float* az, int nx, int ny, int nz, float sign, float* out,
                                void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(params != nullptr && out != nullptr, "NULL pointer");
    const FieldParams& p = *params;
    if (int st = check_field_weights(p)) return st;
    GBSDF_CHECK_ARG(M >= 0, "M < 0");
    if (M == 0) return GBSDF_OK;
    SdfPointsArgs q;
    q.M = M; q.pts = pts; q.ax = ax; q.ay = ay; q.az = az; q.nx = nx; q.ny = ny; q.nz = nz; q.sign = sign; q.out = out;
    if (!pts) {
        GBSDF_CHECK_ARG(ax && ay && az && nx > 0 && ny > 0 && nz > 0 && (int64_t)nx * ny * nz == M,
                        "lattice mode needs axes with nx*ny*nz == M");
    }
    const size_t smem = (size_t)HID * p.K0 * 2 + 2 * (size_t)TILE_M * p.K0 * 2 + (HID * 5 + 2 * TILE_M) * 4 + 16;
    GBSDF_CHECK_ARG(smem <= 227 * 1024, "K0 too large");
    const int64_t ntiles = (M + TILE_M - 1) / TILE_M;
    int64_t grid = num_sms();
    if (grid > ntiles) grid = ntiles;
    cudaStream_t s = as_stream(stream);
    switch (p.grid.n_features) {
        case 2:
            allow_max_smem(k_sdf_points<2>);
            k_sdf_points<2><<<(unsigned)grid, FIELD_THREADS, smem, s>>>(p, q);
            break;
        case 4:
            allow_max_smem(k_sdf_points<4>);
            k_sdf_points<4><<<(unsigned)grid, FIELD_THREADS, smem, s>>>(p, q);
            break;
        default:
            allow_max_smem(k_sdf_points<8>);
            k_sdf_points<8><<<(unsigned)grid, FIELD_THREADS, smem, s>>>(p, q);
            break;
    }
    return launch_status("sdf_points");
}
