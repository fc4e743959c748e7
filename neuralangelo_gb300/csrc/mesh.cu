// GPU marching cubes for block-wise mesh extraction.
//
// Reference path: projects/neuralangelo/utils/mesh.py
//   marching_cubes (:119-133)           -> PyMCubes on the CPU, then V * intv + xyz[0,0,0]
//   filter_points_outside_bounding_sphere (:136-148)
// Here one block volume [nx, ny, nz] (float32, x-major, already negated as
// scripts/extract_mesh.py:85 does) goes through count -> exclusive scan -> emit
// on the device:
//   1. crossing edges (grid edge (i,j,k,axis) whose end values straddle iso)
//      -> vertex numbers in global edge order ((i*ny + j)*nz + k)*3 + axis;
//   2. cube configurations -> triangle counts -> triangle offsets in x-major
//      cube order;
//   3. vertices (double: t = (iso - v0) / (v1 - v0), index-space position,
//      * intv + origin) and faces from the case table;
//   4. the unit-sphere filter: keep |v| < 1, keep faces whose vertices are all
//      kept, re-index by exclusive scans.
// The case table follows the canonical triangulation stated in oracle/mc.c
// (face walks with positive corners separated on ambiguous faces, loops fanned
// from their smallest edge id); it is generated on the host at first use.
#include <mutex>

#include "common.cuh"
#include "scan.cuh"

namespace gbsdf {

// ---------------------------------------------------------------------------
// case table (host generation)

struct McTable {
    int8_t tri[256][16][3];   // edge ids, -1 padded
    int8_t count[256];
};

static int mc_edge_of_pair(int ca, int cb) {
    const int d = ca ^ cb;
    const int axis = d == 1 ? 0 : (d == 2 ? 1 : 2);
    const int lo = ca & cb;
    // the two remaining axes, ascending, give the bits of the edge's rank
    int others[2], m = 0;
    for (int ax = 0; ax < 3; ++ax)
        if (ax != axis) others[m++] = ax;
    const int r = ((lo >> others[0]) & 1) | (((lo >> others[1]) & 1) << 1);
    return axis * 4 + r;
}

static void mc_build_table(McTable& t) {
    // counter-clockwise corner cycle of every face as seen from outside the cube
    int cycles[6][4];
    for (int f = 0; f < 6; ++f) {
        const int n = f >> 1, side = f & 1, u = (n + 1) % 3, w = (n + 2) % 3;
        static const int uv[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
        for (int k = 0; k < 4; ++k) {
            const int q = side ? k : (4 - k) & 3;
            cycles[f][k] = (side << n) | (uv[q][0] << u) | (uv[q][1] << w);
        }
    }
    for (int cfg = 0; cfg < 256; ++cfg) {
        int succ[12];
        for (int e = 0; e < 12; ++e) succ[e] = -1;
        for (int f = 0; f < 6; ++f) {
            const int* cy = cycles[f];
            bool pos[4];
            for (int k = 0; k < 4; ++k) pos[k] = (cfg >> cy[k]) & 1;
            for (int k = 0; k < 4; ++k) {
                if (!pos[k] || pos[(k + 1) & 3]) continue;       // not an exit
                int j = k;
                while (pos[j]) j = (j + 3) & 3;                   // walk back over the positive run
                succ[mc_edge_of_pair(cy[k], cy[(k + 1) & 3])] = mc_edge_of_pair(cy[j], cy[(j + 1) & 3]);
            }
        }
        bool seen[12] = {false};
        int nt = 0;
        for (int e = 0; e < 12; ++e) {
            if (succ[e] < 0 || seen[e]) continue;
            int loop[12], m = 0;
            for (int x = e; !seen[x]; x = succ[x]) {
                seen[x] = true;
                loop[m++] = x;
            }
            for (int i = 1; i + 1 < m; ++i) {
                t.tri[cfg][nt][0] = (int8_t)loop[0];
                t.tri[cfg][nt][1] = (int8_t)loop[i + 1];
                t.tri[cfg][nt][2] = (int8_t)loop[i];
                ++nt;
            }
        }
        t.count[cfg] = (int8_t)nt;
        for (int k = nt; k < 16; ++k) t.tri[cfg][k][0] = t.tri[cfg][k][1] = t.tri[cfg][k][2] = -1;
    }
}

static const McTable& mc_table() {
    static McTable t;
    static std::once_flag once;
    std::call_once(once, [] { mc_build_table(t); });
    return t;
}

__constant__ int8_t c_tri[256][16][3];
__constant__ int8_t c_count[256];

static int upload_table_once() {
    // constant memory is per device: upload on every device the first time it is used
    static bool done[64] = {false};
    static std::mutex mu;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 0 && dev < 64 && done[dev]) return GBSDF_OK;
    const McTable& t = mc_table();
    if (cudaMemcpyToSymbol(c_tri, t.tri, sizeof(t.tri)) != cudaSuccess ||
        cudaMemcpyToSymbol(c_count, t.count, sizeof(t.count)) != cudaSuccess) {
        set_error("uploading the marching-cubes table failed: %s", cudaGetErrorString(cudaGetLastError()));
        return GBSDF_ERR_CUDA;
    }
    if (dev >= 0 && dev < 64) done[dev] = true;
    return GBSDF_OK;
}

__device__ __forceinline__ void edge_lo_corner(int e, int& a, int& dx, int& dy, int& dz) {
    a = e >> 2;
    const int r = e & 3;
    // the two other axes ascending take the bits of r
    if (a == 0) { dx = 0; dy = r & 1; dz = r >> 1; }
    else if (a == 1) { dx = r & 1; dy = 0; dz = r >> 1; }
    else { dx = r & 1; dy = r >> 1; dz = 0; }
}

// ---------------------------------------------------------------------------
// marching-cubes kernels

struct McDims {
    int nx, ny, nz;
};

__device__ __forceinline__ int64_t vol_index(const McDims& d, int i, int j, int k) {
    return ((int64_t)i * d.ny + j) * d.nz + k;
}

__global__ void k_mc_edges(const float* __restrict__ vol, McDims d, double iso, int64_t* __restrict__ flag) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t ne = (int64_t)d.nx * d.ny * d.nz * 3;
    if (g >= ne) return;
    const int a = (int)(g % 3);
    const int64_t p = g / 3;
    const int k = (int)(p % d.nz), j = (int)((p / d.nz) % d.ny), i = (int)(p / ((int64_t)d.ny * d.nz));
    const int i1 = i + (a == 0), j1 = j + (a == 1), k1 = k + (a == 2);
    int64_t f = 0;
    if (i1 < d.nx && j1 < d.ny && k1 < d.nz) {
        const bool p0 = (double)vol[vol_index(d, i, j, k)] > iso;
        const bool p1 = (double)vol[vol_index(d, i1, j1, k1)] > iso;
        f = p0 != p1;
    }
    flag[g] = f;
}

__global__ void k_mc_cubes(const float* __restrict__ vol, McDims d, double iso, int64_t* __restrict__ tri_count) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nc = (int64_t)(d.nx - 1) * (d.ny - 1) * (d.nz - 1);
    if (c >= nc) return;
    const int k = (int)(c % (d.nz - 1)), j = (int)((c / (d.nz - 1)) % (d.ny - 1)),
              i = (int)(c / ((int64_t)(d.ny - 1) * (d.nz - 1)));
    int cfg = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q)
        if ((double)vol[vol_index(d, i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1))] > iso) cfg |= 1 << q;
    tri_count[c] = c_count[cfg];
}

__global__ void k_mc_vertices(const float* __restrict__ vol, McDims d, double iso, const int64_t* __restrict__ flag,
                              const int64_t* __restrict__ vidx, double ox, double oy, double oz, double intv,
                              double* __restrict__ V) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t ne = (int64_t)d.nx * d.ny * d.nz * 3;
    if (g >= ne || !flag[g]) return;
    const int a = (int)(g % 3);
    const int64_t p = g / 3;
    const int k = (int)(p % d.nz), j = (int)((p / d.nz) % d.ny), i = (int)(p / ((int64_t)d.ny * d.nz));
    const double v0 = vol[vol_index(d, i, j, k)];
    const double v1 = vol[vol_index(d, i + (a == 0), j + (a == 1), k + (a == 2))];
    const double t = __ddiv_rn(__dsub_rn(iso, v0), __dsub_rn(v1, v0));
    double idx[3] = {(double)i, (double)j, (double)k};
    idx[a] = __dadd_rn(idx[a], t);
    const double org[3] = {ox, oy, oz};
    const int64_t v = vidx[g];
#pragma unroll
    for (int q = 0; q < 3; ++q) V[3 * v + q] = __dadd_rn(__dmul_rn(idx[q], intv), org[q]);
}

__global__ void k_mc_faces(const float* __restrict__ vol, McDims d, double iso, const int64_t* __restrict__ tri_off,
                           const int64_t* __restrict__ vidx, int64_t* __restrict__ F) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nc = (int64_t)(d.nx - 1) * (d.ny - 1) * (d.nz - 1);
    if (c >= nc) return;
    const int k = (int)(c % (d.nz - 1)), j = (int)((c / (d.nz - 1)) % (d.ny - 1)),
              i = (int)(c / ((int64_t)(d.ny - 1) * (d.nz - 1)));
    int cfg = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q)
        if ((double)vol[vol_index(d, i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1))] > iso) cfg |= 1 << q;
    const int nt = c_count[cfg];
    int64_t o = tri_off[c];
    for (int t = 0; t < nt; ++t, ++o) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            int a, dx, dy, dz;
            edge_lo_corner(c_tri[cfg][t][q], a, dx, dy, dz);
            const int64_t g = vol_index(d, i + dx, j + dy, k + dz) * 3 + a;
            F[3 * o + q] = vidx[g];
        }
    }
}

// unit-sphere filter (mesh.py:136-148)
__global__ void k_keep_vertices(const double* __restrict__ V, const int64_t* __restrict__ nv, int64_t* __restrict__ keep,
                                int64_t cap) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= cap) return;
    int64_t k = 0;
    if (v < *nv) {
        const double x = V[3 * v], y = V[3 * v + 1], z = V[3 * v + 2];
        k = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z))) < 1.0;
    }
    keep[v] = k;
}

__global__ void k_keep_faces(const int64_t* __restrict__ F, const int64_t* __restrict__ nf,
                             const int64_t* __restrict__ vkeep, int64_t* __restrict__ fkeep, int64_t cap) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= cap) return;
    int64_t k = 0;
    if (f < *nf) k = vkeep[F[3 * f]] && vkeep[F[3 * f + 1]] && vkeep[F[3 * f + 2]];
    fkeep[f] = k;
}

__global__ void k_compact(const double* __restrict__ V, const int64_t* __restrict__ vkeep,
                          const int64_t* __restrict__ vnew, int64_t vcap, const int64_t* __restrict__ F,
                          const int64_t* __restrict__ fkeep, const int64_t* __restrict__ fnew, int64_t fcap,
                          double* __restrict__ Vout, int64_t* __restrict__ Fout) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < vcap && vkeep[i]) {
        const int64_t o = vnew[i];
        Vout[3 * o] = V[3 * i];
        Vout[3 * o + 1] = V[3 * i + 1];
        Vout[3 * o + 2] = V[3 * i + 2];
    }
    if (i < fcap && fkeep[i]) {
        const int64_t o = fnew[i];
#pragma unroll
        for (int q = 0; q < 3; ++q) Fout[3 * o + q] = vnew[F[3 * i + q]];
    }
}

__global__ void k_counts(const int64_t* __restrict__ vnew, const int64_t* __restrict__ vkeep, int64_t vcap,
                         const int64_t* __restrict__ fnew, const int64_t* __restrict__ fkeep, int64_t fcap,
                         int64_t* __restrict__ counts) {
    counts[0] = vcap > 0 ? vnew[vcap - 1] + vkeep[vcap - 1] : 0;
    counts[1] = fcap > 0 ? fnew[fcap - 1] + fkeep[fcap - 1] : 0;
}

struct McWorkspace {
    int64_t* eflag;   // [ne]
    int64_t* vidx;    // [ne]
    int64_t* tcount;  // [nc]
    int64_t* toff;    // [nc]
    int64_t* raw_n;   // [2] vertices, faces before the filter
    double* Vraw;     // [vcap, 3]
    int64_t* Fraw;    // [fcap, 3]
    int64_t* vkeep;   // [vcap]
    int64_t* vnew;    // [vcap]
    int64_t* fkeep;   // [fcap]
    int64_t* fnew;    // [fcap]
    int64_t* scan;    // scan scratch
};

static size_t align256(size_t b) { return (b + 255) / 256 * 256; }

static size_t mc_layout(int nx, int ny, int nz, int64_t vcap, int64_t fcap, uint8_t* base, McWorkspace* w) {
    const int64_t ne = (int64_t)nx * ny * nz * 3;
    const int64_t nc = (int64_t)(nx - 1) * (ny - 1) * (nz - 1);
    int64_t mx = ne > nc ? ne : nc;
    if (vcap > mx) mx = vcap;
    if (fcap > mx) mx = fcap;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        uint8_t* p = base ? base + off : nullptr;
        off += align256(bytes);
        return p;
    };
    McWorkspace t;
    t.eflag = (int64_t*)take(8 * (size_t)ne);
    t.vidx = (int64_t*)take(8 * (size_t)ne);
    t.tcount = (int64_t*)take(8 * (size_t)nc);
    t.toff = (int64_t*)take(8 * (size_t)nc);
    t.raw_n = (int64_t*)take(16);
    t.Vraw = (double*)take(24 * (size_t)vcap);
    t.Fraw = (int64_t*)take(24 * (size_t)fcap);
    t.vkeep = (int64_t*)take(8 * (size_t)vcap);
    t.vnew = (int64_t*)take(8 * (size_t)vcap);
    t.fkeep = (int64_t*)take(8 * (size_t)fcap);
    t.fnew = (int64_t*)take(8 * (size_t)fcap);
    t.scan = (int64_t*)take(8 * scan_ws_elems(mx));
    if (w) *w = t;
    return off;
}

// worst-case output sizes of one block: one vertex per grid edge, five triangles per cube
static int64_t mc_vcap(int nx, int ny, int nz) { return (int64_t)nx * ny * nz * 3; }
static int64_t mc_fcap(int nx, int ny, int nz) { return 5 * (int64_t)(nx - 1) * (ny - 1) * (nz - 1); }

static int mc_run(const float* vol, int nx, int ny, int nz, double iso, const double* origin, double intv,
                  const McWorkspace& w, double* V, int64_t* F, int64_t* counts, cudaStream_t s) {
    const McDims d{nx, ny, nz};
    const int64_t ne = (int64_t)nx * ny * nz * 3;
    const int64_t nc = (int64_t)(nx - 1) * (ny - 1) * (nz - 1);
    const int64_t vcap = mc_vcap(nx, ny, nz), fcap = mc_fcap(nx, ny, nz);
    const int T = 256;
    k_mc_edges<<<(unsigned)((ne + T - 1) / T), T, 0, s>>>(vol, d, iso, w.eflag);
    exclusive_scan(w.eflag, w.vidx, ne, w.scan, nullptr, s);
    k_mc_cubes<<<(unsigned)((nc + T - 1) / T), T, 0, s>>>(vol, d, iso, w.tcount);
    exclusive_scan(w.tcount, w.toff, nc, w.scan, nullptr, s);
    // counts before the filter: last offset + last count
    k_counts<<<1, 1, 0, s>>>(w.vidx, w.eflag, ne, w.toff, w.tcount, nc, w.raw_n);
    k_mc_vertices<<<(unsigned)((ne + T - 1) / T), T, 0, s>>>(vol, d, iso, w.eflag, w.vidx, origin[0], origin[1],
                                                              origin[2], intv, w.Vraw);
    k_mc_faces<<<(unsigned)((nc + T - 1) / T), T, 0, s>>>(vol, d, iso, w.toff, w.vidx, w.Fraw);
    k_keep_vertices<<<(unsigned)((vcap + T - 1) / T), T, 0, s>>>(w.Vraw, w.raw_n, w.vkeep, vcap);
    exclusive_scan(w.vkeep, w.vnew, vcap, w.scan, nullptr, s);
    k_keep_faces<<<(unsigned)((fcap + T - 1) / T), T, 0, s>>>(w.Fraw, w.raw_n + 1, w.vkeep, w.fkeep, fcap);
    exclusive_scan(w.fkeep, w.fnew, fcap, w.scan, nullptr, s);
    const int64_t mx = vcap > fcap ? vcap : fcap;
    k_compact<<<(unsigned)((mx + T - 1) / T), T, 0, s>>>(w.Vraw, w.vkeep, w.vnew, vcap, w.Fraw, w.fkeep, w.fnew, fcap,
                                                         V, F);
    k_counts<<<1, 1, 0, s>>>(w.vnew, w.vkeep, vcap, w.fnew, w.fkeep, fcap, counts);
    return launch_status("marching_cubes");
}

}  // namespace gbsdf

using namespace gbsdf;

extern "C" int gbsdf_mc_table(int32_t* tri, int32_t* count) {
    clear_error();
    GBSDF_CHECK_ARG(tri && count, "NULL pointer");
    const McTable& t = mc_table();
    for (int c = 0; c < 256; ++c) {
        count[c] = t.count[c];
        for (int k = 0; k < 16; ++k)
            for (int q = 0; q < 3; ++q) tri[(c * 16 + k) * 3 + q] = t.tri[c][k][q];
    }
    return GBSDF_OK;
}

extern "C" size_t gbsdf_mc_workspace_size(int nx, int ny, int nz) {
    if (nx < 2 || ny < 2 || nz < 2) return 0;
    return mc_layout(nx, ny, nz, mc_vcap(nx, ny, nz), mc_fcap(nx, ny, nz), nullptr, nullptr);
}

extern "C" int gbsdf_mc_block(const float* vol, int nx, int ny, int nz, double iso, const double* origin, double intv,
                              void* workspace, size_t ws_bytes, double* V, int64_t V_cap, int64_t* F, int64_t F_cap,
                              int64_t* counts, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(vol && origin && V && F && counts, "NULL pointer");
    GBSDF_CHECK_ARG(nx >= 2 && ny >= 2 && nz >= 2, "block must have at least 2 points per axis");
    GBSDF_CHECK_ARG((int64_t)nx * ny * nz <= (int64_t)1 << 28, "block too large");
    GBSDF_CHECK_ARG(V_cap >= mc_vcap(nx, ny, nz) && F_cap >= mc_fcap(nx, ny, nz),
                    "output capacity below the worst case (3 nx ny nz vertices, 5 (nx-1)(ny-1)(nz-1) faces)");
    const size_t need = gbsdf_mc_workspace_size(nx, ny, nz);
    GBSDF_CHECK_ARG(workspace && ws_bytes >= need, "workspace of %zu bytes needed", need);
    GBSDF_CHECK_ARG(aligned(workspace, 256), "workspace must be 256-byte aligned");
    if (int st = upload_table_once()) return st;
    McWorkspace w;
    mc_layout(nx, ny, nz, mc_vcap(nx, ny, nz), mc_fcap(nx, ny, nz), (uint8_t*)workspace, &w);
    return mc_run(vol, nx, ny, nz, iso, origin, intv, w, V, F, counts, as_stream(stream));
}

// ---------------------------------------------------------------------------
// Marching cubes without any device allocation.
//
// Some callers cannot allocate device memory: a host application that owns the
// whole device budget and forbids allocations after start-up (a renderer or an
// engine plugin with a fixed pool), or a caller in a latency-critical loop where
// cudaMalloc / cudaFree could synchronise the device.  For them this variant
// keeps its scratch in a file-scope __device__ array of fixed size, enough for
// blocks of up to 33 x 33 x 33 lattice points (32^3 cubes).  The array exists on
// every device that loads this library, for the life of the process
// (12.5 MiB).  Host code may not take the array's name as a device address, so
// the device address is looked up with cudaGetSymbolAddress once per device, on
// the first call made with that device current; make that first call before any
// stream capture.  Every call reuses the same array: two calls whose kernels
// overlap on the GPU (different streams, or several host threads) race, so
// serialise them.  Every scratch element is written before it is read in a
// call, so nothing carries over from the previous call.

constexpr int kNoAllocMaxPoints = 33;
constexpr size_t kNoAllocScratchBytes = 13119488;   // gbsdf_mc_workspace_size(33, 33, 33)

static __device__ __align__(256) uint8_t g_mc_scratch[kNoAllocScratchBytes];

static int noalloc_scratch(void** out) {
    static void* addr[64] = {nullptr};
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        set_error("no current CUDA device");
        return GBSDF_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_mc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error("cudaGetSymbolAddress of the marching-cubes scratch failed: %s", cudaGetErrorString(e));
            return GBSDF_ERR_CUDA;
        }
        addr[dev] = p;
    }
    *out = addr[dev];
    return GBSDF_OK;
}

extern "C" int gbsdf_mc_block_noalloc(const float* vol, int nx, int ny, int nz, double iso, const double* origin,
                                      double intv, double* V, int64_t V_cap, int64_t* F, int64_t F_cap,
                                      int64_t* counts, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(vol && origin && V && F && counts, "NULL pointer");
    GBSDF_CHECK_ARG(nx >= 2 && ny >= 2 && nz >= 2, "block must have at least 2 points per axis");
    GBSDF_CHECK_ARG(nx <= kNoAllocMaxPoints && ny <= kNoAllocMaxPoints && nz <= kNoAllocMaxPoints,
                    "block %d x %d x %d exceeds the allocation-free limit of %d points per axis "
                    "(use gbsdf_mc_block with a caller workspace for larger blocks)",
                    nx, ny, nz, kNoAllocMaxPoints);
    GBSDF_CHECK_ARG(V_cap >= mc_vcap(nx, ny, nz) && F_cap >= mc_fcap(nx, ny, nz),
                    "output capacity below the worst case (3 nx ny nz vertices, 5 (nx-1)(ny-1)(nz-1) faces)");
    if (gbsdf_mc_workspace_size(nx, ny, nz) > kNoAllocScratchBytes) {
        set_error("internal: scratch layout larger than the static array");
        return GBSDF_ERR_UNSUPPORTED;
    }
    if (int st = upload_table_once()) return st;
    void* scratch = nullptr;
    if (int st = noalloc_scratch(&scratch)) return st;
    McWorkspace w;
    mc_layout(nx, ny, nz, mc_vcap(nx, ny, nz), mc_fcap(nx, ny, nz), (uint8_t*)scratch, &w);
    return mc_run(vol, nx, ny, nz, iso, origin, intv, w, V, F, counts, as_stream(stream));
}
