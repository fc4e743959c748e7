// Multi-resolution hash-grid encoding, forward / backward / index dump.
//
// Replaces tcnn.Encoding (projects/neuralangelo/utils/modules.py:42-50 built,
// :84-86 called).  One thread per (point, level): blockIdx.y is the level, so a
// warp's 32 points share a level and their corner loads hit the same level
// slice of the table (coarse levels stay resident in L2).  Table rows of F
// features are read as one 8/16/32-byte vector; backward scatters with
// vector float atomics (sm_90+ atomicAdd(float4*/float2*)).
#include "common.cuh"

namespace gbsdf {

template <int F, typename TT>
struct RowLoad;

template <>
struct RowLoad<8, float> {
    __device__ static void load(const float* p, float* v) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(p));
        const float4 b = __ldg(reinterpret_cast<const float4*>(p) + 1);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    }
};
template <>
struct RowLoad<4, float> {
    __device__ static void load(const float* p, float* v) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(p));
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    }
};
template <>
struct RowLoad<2, float> {
    __device__ static void load(const float* p, float* v) {
        const float2 a = __ldg(reinterpret_cast<const float2*>(p));
        v[0] = a.x; v[1] = a.y;
    }
};
template <>
struct RowLoad<1, float> {
    __device__ static void load(const float* p, float* v) { v[0] = __ldg(p); }
};
template <>
struct RowLoad<8, __half> {
    __device__ static void load(const __half* p, float* v) {
        const uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
        const __half2* h = reinterpret_cast<const __half2*>(&a);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 f = __half22float2(h[i]);
            v[2 * i] = f.x; v[2 * i + 1] = f.y;
        }
    }
};
template <>
struct RowLoad<4, __half> {
    __device__ static void load(const __half* p, float* v) {
        const uint2 a = __ldg(reinterpret_cast<const uint2*>(p));
        const __half2* h = reinterpret_cast<const __half2*>(&a);
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const float2 f = __half22float2(h[i]);
            v[2 * i] = f.x; v[2 * i + 1] = f.y;
        }
    }
};
template <>
struct RowLoad<2, __half> {
    __device__ static void load(const __half* p, float* v) {
        const float2 f = __half22float2(*reinterpret_cast<const __half2*>(p));
        v[0] = f.x; v[1] = f.y;
    }
};
template <>
struct RowLoad<1, __half> {
    __device__ static void load(const __half* p, float* v) { v[0] = __half2float(p[0]); }
};

template <int F>
__device__ __forceinline__ void scatter_row(float* p, const float* v) {
    if constexpr (F == 8) {
        atomicAdd(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
        atomicAdd(reinterpret_cast<float4*>(p) + 1, make_float4(v[4], v[5], v[6], v[7]));
    } else if constexpr (F == 4) {
        atomicAdd(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
    } else if constexpr (F == 2) {
        atomicAdd(reinterpret_cast<float2*>(p), make_float2(v[0], v[1]));
    } else {
        atomicAdd(p, v[0]);
    }
}

template <typename TO>
__device__ __forceinline__ TO cvt_out(float v);
template <>
__device__ __forceinline__ float cvt_out<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half cvt_out<__half>(float v) { return __float2half_rn(v); }

template <int F, typename TT, typename TO>
__global__ void __launch_bounds__(256) k_hashgrid_fwd(gbsdf_grid g, int active, const float* __restrict__ x,
                                                      int64_t M, const TT* __restrict__ table,
                                                      TO* __restrict__ out) {
    const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int l = blockIdx.y;
    if (m >= M) return;
    TO* o = out + m * (int64_t)(g.n_levels * F) + l * F;
    float acc[F];
#pragma unroll
    for (int f = 0; f < F; ++f) acc[f] = 0.0f;
    if (l < active) {
        const LevelDesc d = level_desc(g, l);
        uint32_t bx, by, bz;
        float fx, fy, fz;
        grid_pos(d.scale, x[3 * m + 0], bx, fx);
        grid_pos(d.scale, x[3 * m + 1], by, fy);
        grid_pos(d.scale, x[3 * m + 2], bz, fz);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const uint32_t idx = grid_index(d, bx + (c & 1), by + ((c >> 1) & 1), bz + ((c >> 2) & 1));
            const float w = corner_weight(c, fx, fy, fz);
            float v[F];
            RowLoad<F, TT>::load(table + (d.offset + idx) * F, v);
#pragma unroll
            for (int f = 0; f < F; ++f) acc[f] = fmaf(w, v[f], acc[f]);
        }
    }
#pragma unroll
    for (int f = 0; f < F; ++f) o[f] = cvt_out<TO>(acc[f]);
}

template <int F>
__global__ void __launch_bounds__(256) k_hashgrid_bwd(gbsdf_grid g, int active, const float* __restrict__ x,
                                                      int64_t M, const float* __restrict__ d_out,
                                                      float* __restrict__ d_table) {
    const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int l = blockIdx.y;
    if (m >= M || l >= active) return;
    const float* dpt = d_out + m * (int64_t)(g.n_levels * F) + l * F;
    float dv[F];
    bool any = false;
#pragma unroll
    for (int f = 0; f < F; ++f) {
        dv[f] = dpt[f];
        any |= (dv[f] != 0.0f);
    }
    if (!any) return;
    const LevelDesc d = level_desc(g, l);
    uint32_t bx, by, bz;
    float fx, fy, fz;
    grid_pos(d.scale, x[3 * m + 0], bx, fx);
    grid_pos(d.scale, x[3 * m + 1], by, fy);
    grid_pos(d.scale, x[3 * m + 2], bz, fz);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint32_t idx = grid_index(d, bx + (c & 1), by + ((c >> 1) & 1), bz + ((c >> 2) & 1));
        const float w = corner_weight(c, fx, fy, fz);
        float v[F];
#pragma unroll
        for (int f = 0; f < F; ++f) v[f] = w * dv[f];
        scatter_row<F>(d_table + (d.offset + idx) * F, v);
    }
}

__global__ void k_hashgrid_indices(gbsdf_grid g, int active, const float* __restrict__ x, int64_t M,
                                   int64_t* __restrict__ out) {
    const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int l = blockIdx.y;
    if (m >= M) return;
    const LevelDesc d = level_desc(g, l);
    uint32_t bx, by, bz;
    float fx, fy, fz;
    grid_pos(d.scale, x[3 * m + 0], bx, fx);
    grid_pos(d.scale, x[3 * m + 1], by, fy);
    grid_pos(d.scale, x[3 * m + 2], bz, fz);
    for (int c = 0; c < 8; ++c) {
        const uint32_t idx = grid_index(d, bx + (c & 1), by + ((c >> 1) & 1), bz + ((c >> 2) & 1));
        out[(m * active + l) * 8 + c] = (int64_t)(d.offset + idx);
    }
}

static int check_grid(const gbsdf_grid* g, int active) {
    GBSDF_CHECK_ARG(g != nullptr, "grid is NULL");
    GBSDF_CHECK_ARG(g->n_levels >= 1 && g->n_levels <= GBSDF_MAX_LEVELS, "n_levels %d out of range", g->n_levels);
    GBSDF_CHECK_ARG(active >= 0 && active <= g->n_levels, "active_levels %d not in [0, %d]", active, g->n_levels);
    const int F = g->n_features;
    GBSDF_CHECK_ARG(F == 1 || F == 2 || F == 4 || F == 8, "n_features %d unsupported (1, 2, 4, 8)", F);
    return GBSDF_OK;
}

template <int F>
static void launch_fwd(const gbsdf_grid* g, int active, const float* x, int64_t M, const void* table, int tdt,
                       void* out, int odt, cudaStream_t s) {
    dim3 grid((unsigned)((M + 255) / 256), (unsigned)g->n_levels);
    if (tdt == GBSDF_F32 && odt == GBSDF_F32)
        k_hashgrid_fwd<F, float, float><<<grid, 256, 0, s>>>(*g, active, x, M, (const float*)table, (float*)out);
    else if (tdt == GBSDF_F32 && odt == GBSDF_F16)
        k_hashgrid_fwd<F, float, __half><<<grid, 256, 0, s>>>(*g, active, x, M, (const float*)table, (__half*)out);
    else if (tdt == GBSDF_F16 && odt == GBSDF_F32)
        k_hashgrid_fwd<F, __half, float><<<grid, 256, 0, s>>>(*g, active, x, M, (const __half*)table, (float*)out);
    else
        k_hashgrid_fwd<F, __half, __half><<<grid, 256, 0, s>>>(*g, active, x, M, (const __half*)table, (__half*)out);
}

}  // namespace gbsdf

using namespace gbsdf;

extern "C" int gbsdf_hashgrid_fwd(const gbsdf_grid* g, int active, const float* x, int64_t M, const void* table,
                                  int table_dtype, void* out, int out_dtype, void* stream) {
    clear_error();
    if (int st = check_grid(g, active)) return st;
    GBSDF_CHECK_ARG(M >= 0, "M < 0");
    if (M == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(x && table && out, "NULL pointer");
    GBSDF_CHECK_ARG(table_dtype == GBSDF_F32 || table_dtype == GBSDF_F16, "bad table dtype");
    GBSDF_CHECK_ARG(out_dtype == GBSDF_F32 || out_dtype == GBSDF_F16, "bad out dtype");
    GBSDF_CHECK_ARG(aligned(table, 16) && aligned(x, 4), "table must be 16-byte aligned");
    GBSDF_CHECK_ARG((M + 255) / 256 < (int64_t)INT32_MAX, "M too large");
    cudaStream_t s = as_stream(stream);
    switch (g->n_features) {
        case 1: launch_fwd<1>(g, active, x, M, table, table_dtype, out, out_dtype, s); break;
        case 2: launch_fwd<2>(g, active, x, M, table, table_dtype, out, out_dtype, s); break;
        case 4: launch_fwd<4>(g, active, x, M, table, table_dtype, out, out_dtype, s); break;
        default: launch_fwd<8>(g, active, x, M, table, table_dtype, out, out_dtype, s); break;
    }
    return launch_status("hashgrid_fwd");
}

extern "C" int gbsdf_hashgrid_bwd(const gbsdf_grid* g, int active, const float* x, int64_t M, const float* d_out,
                                  float* d_table, void* stream) {
    clear_error();
    if (int st = check_grid(g, active)) return st;
    GBSDF_CHECK_ARG(M >= 0, "M < 0");
    if (M == 0 || active == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(x && d_out && d_table, "NULL pointer");
    GBSDF_CHECK_ARG(aligned(d_table, 16), "d_table must be 16-byte aligned");
    cudaStream_t s = as_stream(stream);
    dim3 grid((unsigned)((M + 255) / 256), (unsigned)active);
    switch (g->n_features) {
        case 1: k_hashgrid_bwd<1><<<grid, 256, 0, s>>>(*g, active, x, M, d_out, d_table); break;
        case 2: k_hashgrid_bwd<2><<<grid, 256, 0, s>>>(*g, active, x, M, d_out, d_table); break;
        case 4: k_hashgrid_bwd<4><<<grid, 256, 0, s>>>(*g, active, x, M, d_out, d_table); break;
        default: k_hashgrid_bwd<8><<<grid, 256, 0, s>>>(*g, active, x, M, d_out, d_table); break;
    }
    return launch_status("hashgrid_bwd");
}

extern "C" int gbsdf_hashgrid_indices(const gbsdf_grid* g, int active, const float* x, int64_t M, int64_t* indices,
                                      void* stream) {
    clear_error();
    if (int st = check_grid(g, active)) return st;
    GBSDF_CHECK_ARG(M >= 0, "M < 0");
    if (M == 0 || active == 0) return GBSDF_OK;
    GBSDF_CHECK_ARG(x && indices, "NULL pointer");
    dim3 grid((unsigned)((M + 255) / 256), (unsigned)active);
    k_hashgrid_indices<<<grid, 256, 0, as_stream(stream)>>>(*g, active, x, M, indices);
    return launch_status("hashgrid_indices");
}
