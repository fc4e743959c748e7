// Shared device helpers for the gbsdf kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/gbsdf.h"

namespace gbsdf {

// ---------------------------------------------------------------------------
// error reporting (thread-local message, defined in capi.cu)
void set_error(const char* fmt, ...);
void clear_error();

#define GBSDF_CHECK_ARG(cond, ...)            \
    do {                                      \
        if (!(cond)) {                        \
            ::gbsdf::set_error(__VA_ARGS__);  \
            return GBSDF_ERR_ARG;             \
        }                                     \
    } while (0)

int launch_status(const char* what);   // checks cudaGetLastError after a launch

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

// Lets kernel k take up to the device's opt-in maximum of dynamic shared memory per
// block.  Always the same ceiling, never the current launch's size: a per-launch value
// would leave the attribute at the last launch's size, below what an earlier launch of
// the same kernel recorded in a CUDA graph asks for when that node is launched on its
// own (as a profiler does with graph nodes).
template <typename Kernel>
inline void allow_max_smem(Kernel k) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

// ---------------------------------------------------------------------------
// hash-grid level arithmetic, shared by every kernel that evaluates the field.
// Follows tiny-cuda-nn's HashGrid (the encoder behind modules.py:42-50):
// position p = fma(scale, x, 0.5); corner = floor(p); frac = p - corner; the
// corner index is dense (x + y*res + z*res^2) or the XOR prime hash, modulo the
// level size.  The per-level scale arrives precomputed in gbsdf_grid.scale.

struct LevelDesc {
    float scale;
    uint32_t res;
    uint32_t size;
    uint32_t hashed;
    uint64_t offset;
};

__device__ __forceinline__ LevelDesc level_desc(const gbsdf_grid& g, int l) {
    LevelDesc d;
    d.scale = g.scale[l];
    d.res = g.resolution[l];
    d.size = g.size[l];
    d.hashed = g.hashed[l];
    d.offset = g.offset[l];
    return d;
}

__device__ __forceinline__ void grid_pos(float scale, float x, uint32_t& base, float& frac) {
    const float p = __fmaf_rn(scale, x, 0.5f);
    const float f = floorf(p);
    base = (uint32_t)(int)f;
    frac = __fsub_rn(p, f);
}

// Same result as idx % size without a division in the common cases: a hashed
// level's size is the power of two 2^log2_hashmap_size (it is hashed exactly when
// res^3 exceeds that), and a dense index of an in-range corner is already below
// the level size (size >= res^3).
__device__ __forceinline__ uint32_t grid_index(const LevelDesc& d, uint32_t cx, uint32_t cy, uint32_t cz) {
    if (d.hashed) {
        const uint32_t idx = (cx * 1u) ^ (cy * 2654435761u) ^ (cz * 805459861u);
        return (d.size & (d.size - 1u)) == 0u ? (idx & (d.size - 1u)) : idx % d.size;
    }
    const uint32_t idx = cx + cy * d.res + cz * (d.res * d.res);
    return idx < d.size ? idx : idx % d.size;
}

// Corner c (0..7) selects +1 in dimension d when bit d of c is set.
__device__ __forceinline__ float corner_weight(int c, float fx, float fy, float fz) {
    const float wx = (c & 1) ? fx : __fsub_rn(1.0f, fx);
    const float wy = (c & 2) ? fy : __fsub_rn(1.0f, fy);
    const float wz = (c & 4) ? fz : __fsub_rn(1.0f, fz);
    return __fmul_rn(__fmul_rn(wx, wy), wz);
}

// Normalisation of a world point into the grid's unit cube, as NeuralSDF.encode
// does it (modules.py:82-83): (p - vmin) / (vmax - vmin) with range [-2, 2].
__device__ __forceinline__ float to_unit(float p) { return __fmul_rn(__fadd_rn(p, 2.0f), 0.25f); }

// ---------------------------------------------------------------------------
// numerics shared with the reference's activations

// torch.nn.functional.softplus(x, beta, threshold=20)
__device__ __forceinline__ float softplus_beta(float x, float beta) {
    const float bx = x * beta;
    return bx > 20.0f ? x : log1pf(expf(bx)) / beta;
}
// d softplus / dx = sigmoid(beta*x) (1 above the threshold)
__device__ __forceinline__ float softplus_grad(float x, float beta) {
    const float bx = x * beta;
    return bx > 20.0f ? 1.0f : 1.0f / (1.0f + expf(-bx));
}
__device__ __forceinline__ float sigmoidf_(float x) { return 1.0f / (1.0f + expf(-x)); }

// MUFU approximations with subnormals flushed to zero (PTX ex2/lg2/rcp .approx.ftz):
// the fused FP16 path's activations never need subnormal precision, and the flushing
// forms take no range fix-ups around the MUFU op.
__device__ __forceinline__ float ex2_ftz(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2_ftz(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_ftz(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Fast-path softplus(beta) and its derivative for the fused FP16 kernels, from one
// exponential by change of base (e^x = 2^(x log2 e), ln y = log2(y) ln 2):
// t = beta z log2(e), e = 2^t, softplus = log2(1 + e) ln(2) / beta, d/dz = e / (1 + e).
// Above torch's threshold (beta z > 20) softplus is z; t is capped at 64 so that e
// stays finite there (and d/dz rounds to 1).  Checked against torch's softplus (CUDA's
// expf / log1pf) to 1e-5 relative, with a ~2e-8 absolute floor where 1 + e is near 1.
struct SoftplusK {
    float c1;      // beta log2(e)
    float c2;      // ln(2) / beta
    float tthr;    // 20 log2(e): the threshold in units of t
};
__device__ __forceinline__ SoftplusK softplus_k(float beta) {
    SoftplusK k;
    k.c1 = beta * 1.4426950408889634f;
    k.c2 = 0.6931471805599453f / beta;
    k.tthr = 20.0f * 1.4426950408889634f;
    return k;
}
__device__ __forceinline__ void softplus_fast(float z, const SoftplusK& k, float& h, float& dh) {
    const float t = fminf(z * k.c1, 64.0f);
    const float e = ex2_ftz(t);
    const float one_e = 1.0f + e;
    dh = e * rcp_ftz(one_e);
    const float hl = lg2_ftz(one_e) * k.c2;
    h = t > k.tthr ? z : hl;
}
__device__ __forceinline__ float softplus_fast_h(float z, const SoftplusK& k) {
    const float t = fminf(z * k.c1, 64.0f);
    const float hl = lg2_ftz(1.0f + ex2_ftz(t)) * k.c2;
    return t > k.tthr ? z : hl;
}

// Column sums of a 32 x 32 block held one row per lane (v[j] = element (lane, j)):
// recursive-halving exchange, 31 shuffles in total; lane j returns the sum of column j.
__device__ __forceinline__ float warp_column_sum32(float* v, int lane) {
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
        const bool upper = (lane & h) != 0;
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const float send = upper ? v[i] : v[i + h];
            const float keep = upper ? v[i + h] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
        }
    }
    return v[0];
}

// Column sums of a 32 x 16 block held one row per lane (v[j] = element (lane, j)):
// four halving exchanges leave lane L with column L % 16 summed over the 16 lanes
// that share L's bit 4; one more exchange adds the other half.  Lanes L and L + 16
// both return the sum of column L % 16 (15 + 1 shuffles).
__device__ __forceinline__ float warp_column_sum16(float* v, int lane) {
#pragma unroll
    for (int h = 8; h >= 1; h >>= 1) {
        const bool upper = (lane & h) != 0;
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const float send = upper ? v[i] : v[i + h];
            const float keep = upper ? v[i + h] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
        }
    }
    return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 16);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace gbsdf
