// Exclusive int64 scan with caller workspace (block scans, recursive on the block
// sums), shared by the mesh kernels.  Everything here has internal linkage, so
// each translation unit that includes it gets its own copy.
#pragma once

#include "common.cuh"

namespace gbsdf {
namespace {

constexpr int SCAN_T = 1024;

static __global__ void k_scan_block(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                             int64_t* __restrict__ block_sums) {
    __shared__ int64_t s[SCAN_T];
    const int64_t i = blockIdx.x * (int64_t)SCAN_T + threadIdx.x;
    const int64_t v = i < n ? in[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < SCAN_T; o <<= 1) {
        const int64_t t = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;          // exclusive
    if (threadIdx.x == SCAN_T - 1) block_sums[blockIdx.x] = s[threadIdx.x];
}

static __global__ void k_scan_add(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ offs) {
    const int64_t i = blockIdx.x * (int64_t)SCAN_T + threadIdx.x;
    if (i < n) out[i] += offs[blockIdx.x];
}

static size_t scan_ws_elems(int64_t n) {
    size_t tot = 0;
    while (n > 1) {
        const int64_t nb = (n + SCAN_T - 1) / SCAN_T;
        tot += 2 * (size_t)nb;
        n = nb;
    }
    return tot + 2;
}

// out[i] = sum_{j<i} in[j]; total (optional) = sum of all, written on the device
static void exclusive_scan(const int64_t* in, int64_t* out, int64_t n, int64_t* ws, int64_t* total,
                           cudaStream_t s) {
    if (n <= 0) return;
    const int64_t nb = (n + SCAN_T - 1) / SCAN_T;
    int64_t* sums = ws;
    int64_t* sums_scan = ws + nb;
    k_scan_block<<<(unsigned)nb, SCAN_T, 0, s>>>(in, out, n, sums);
    if (nb > 1) {
        exclusive_scan(sums, sums_scan, nb, ws + 2 * nb, total, s);
        k_scan_add<<<(unsigned)nb, SCAN_T, 0, s>>>(out, n, sums_scan);
    } else if (total) {
        cudaMemcpyAsync(total, sums, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
    }
}

}  // namespace
}  // namespace gbsdf
