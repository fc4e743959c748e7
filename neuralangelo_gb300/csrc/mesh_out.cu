// Mesh output stage on the GPU: vertex welding, the centre/scale transform and
// degenerate-face removal, the steps between marching cubes and the PLY file.
//
// Reference behaviour (restated; trimesh is a third-party dependency, unpinned):
//  * projects/neuralangelo/utils/mesh.py:121-129 builds a trimesh.Trimesh per block,
//    whose default processing merges vertices whose coordinates round to the same
//    integers at 8 decimal digits (round-half-even of v * 1e8): every group keeps its
//    first occurrence and the faces are re-indexed to it.  The blocks are then concatenated without welding (:43-46).
//  * projects/neuralangelo/scripts/extract_mesh.py:96-97 applies
//    vertices * sphere_radius + sphere_center (two roundings) and keeps the
//    non-degenerate faces: with a = v1 - v0, b = v2 - v0 and 2A = |a x b|, the two
//    triangle heights 2A / |a| and 2A / |b| (0 where that edge is no longer than the
//    tolerance) must both exceed the height (the merge tolerance, 1e-8).  Faces that
//    repeat a vertex index have zero area and go with them.
//  All float64 arithmetic below is written with explicit round-to-nearest intrinsics
//  (no fused multiply-add), so it matches numpy's operation by operation.
//
// gbsdf_mesh_finalize does: optional weld (in input coordinates) -> transform ->
// re-index and drop degenerate faces (in output coordinates) -> compact.  Every
// vertex that survives the weld is kept, referenced or not, as trimesh's
// update_faces keeps them.  Welding uses a bounded-probe hash table over the
// quantised coordinates; a probe sequence that runs past the table raises the
// error flag instead of looping.

#include "common.cuh"
#include "scan.cuh"

namespace gbsdf {

namespace {

struct Key {
    long long x, y, z;
};

__device__ __forceinline__ Key quantise(const double* v, double mult) {
    Key k;
    k.x = __double2ll_rn(__dmul_rn(v[0], mult));
    k.y = __double2ll_rn(__dmul_rn(v[1], mult));
    k.z = __double2ll_rn(__dmul_rn(v[2], mult));
    return k;
}

__device__ __forceinline__ bool same(const Key& a, const Key& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// splitmix64 finaliser over a mix of the three coordinates
__device__ __forceinline__ uint64_t key_hash(const Key& k) {
    uint64_t h = (uint64_t)k.x * 0x9E3779B97F4A7C15ull ^ (uint64_t)k.y * 0xC2B2AE3D27D4EB4Full ^
                 (uint64_t)k.z * 0x165667B19E3779F9ull;
    h ^= h >> 30;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 27;
    h *= 0x94D049BB133111EBull;
    h ^= h >> 31;
    return h;
}

__global__ void k_quantise(const double* __restrict__ V, int64_t nv, double mult, Key* __restrict__ keys) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nv) keys[i] = quantise(V + 3 * i, mult);
}

__global__ void k_fill64(long long* __restrict__ a, int64_t n, long long v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

// slot of vertex i's key: the first slot on its probe sequence that is empty (claimed
// by i) or holds an equal key.  cap is a power of two >= 2 nv, so every sequence meets
// a free slot or its key within cap probes; running past cap sets the error flag.
__global__ void k_hash_insert(const Key* __restrict__ keys, int64_t nv, long long* __restrict__ slot_owner,
                              uint64_t cap, int64_t* __restrict__ slot_of, int* err) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const Key k = keys[i];
    uint64_t h = key_hash(k) & (cap - 1);
    for (uint64_t probe = 0; probe < cap; ++probe) {
        const unsigned long long cur =
            atomicCAS(reinterpret_cast<unsigned long long*>(&slot_owner[h]), ~0ull, (unsigned long long)i);
        if (cur == ~0ull || same(keys[cur], k)) {
            slot_of[i] = (int64_t)h;
            return;
        }
        h = (h + 1) & (cap - 1);
    }
    slot_of[i] = -1;
    if (err) atomicExch(err, 3);
}

// first occurrence of each key: atomic minimum of the vertex indices sharing its slot
__global__ void k_hash_first(const int64_t* __restrict__ slot_of, int64_t nv, long long* __restrict__ slot_first) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nv && slot_of[i] >= 0) atomicMin(&slot_first[slot_of[i]], (long long)i);
}

__global__ void k_reps(const int64_t* __restrict__ slot_of, const long long* __restrict__ slot_first, int64_t nv,
                       int64_t* __restrict__ rep, int64_t* __restrict__ is_rep) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int64_t r = slot_of[i] >= 0 ? (int64_t)slot_first[slot_of[i]] : i;
    rep[i] = r;
    is_rep[i] = r == i ? 1 : 0;
}

__global__ void k_identity(int64_t nv, int64_t* __restrict__ rep, int64_t* __restrict__ is_rep) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nv) {
        rep[i] = i;
        is_rep[i] = 1;
    }
}

struct Xform {
    double scale, ox, oy, oz;
};

__device__ __forceinline__ void xform(const double* v, const Xform& t, double* o) {
    o[0] = __dadd_rn(__dmul_rn(v[0], t.scale), t.ox);
    o[1] = __dadd_rn(__dmul_rn(v[1], t.scale), t.oy);
    o[2] = __dadd_rn(__dmul_rn(v[2], t.scale), t.oz);
}

__device__ __forceinline__ double norm3(const double* x) {
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x[0], x[0]), __dmul_rn(x[1], x[1])), __dmul_rn(x[2], x[2])));
}

__global__ void k_write_vertices(const double* __restrict__ V, int64_t nv, const int64_t* __restrict__ is_rep,
                                 const int64_t* __restrict__ new_idx, Xform t, double* __restrict__ Vout) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nv && is_rep[i]) xform(V + 3 * i, t, Vout + 3 * new_idx[i]);
}

// re-index a face through the weld and test it in output coordinates: min_side < 0
// keeps every face, 0 drops faces that repeat a vertex index, > 0 adds the height test
__global__ void k_faces(const int64_t* __restrict__ F, int64_t nf, int64_t nv, const int64_t* __restrict__ rep,
                        const int64_t* __restrict__ new_idx, const double* __restrict__ Vout, double min_side,
                        int64_t* __restrict__ Fmapped, int64_t* __restrict__ keep, int* err) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= nf) return;
    int64_t m[3];
    bool ok = true;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int64_t v = F[3 * f + c];
        if (v < 0 || v >= nv) {
            ok = false;
            m[c] = 0;
            if (err) atomicExch(err, 4);
        } else {
            m[c] = new_idx[rep[v]];
        }
        Fmapped[3 * f + c] = m[c];
    }
    if (ok && min_side >= 0.0) ok = m[0] != m[1] && m[1] != m[2] && m[0] != m[2];
    if (ok && min_side > 0.0) {
        const double* p0 = Vout + 3 * m[0];
        const double* p1 = Vout + 3 * m[1];
        const double* p2 = Vout + 3 * m[2];
        double ea[3], eb[3], cr[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            ea[k] = __dsub_rn(p1[k], p0[k]);
            eb[k] = __dsub_rn(p2[k], p0[k]);
        }
        cr[0] = __dsub_rn(__dmul_rn(ea[1], eb[2]), __dmul_rn(ea[2], eb[1]));
        cr[1] = __dsub_rn(__dmul_rn(ea[2], eb[0]), __dmul_rn(ea[0], eb[2]));
        cr[2] = __dsub_rn(__dmul_rn(ea[0], eb[1]), __dmul_rn(ea[1], eb[0]));
        const double two_area = __dmul_rn(__dmul_rn(norm3(cr), 0.5), 2.0);
        const double la = norm3(ea), lb = norm3(eb);
        const double ha = la > min_side ? __ddiv_rn(two_area, la) : 0.0;
        const double hb = lb > min_side ? __ddiv_rn(two_area, lb) : 0.0;
        ok = ha > min_side && hb > min_side;
    }
    keep[f] = ok ? 1 : 0;
}

__global__ void k_compact_faces(const int64_t* __restrict__ Fmapped, const int64_t* __restrict__ keep,
                                const int64_t* __restrict__ fnew, int64_t nf, int64_t* __restrict__ Fout) {
    const int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f < nf && keep[f]) {
        const int64_t o = fnew[f];
#pragma unroll
        for (int c = 0; c < 3; ++c) Fout[3 * o + c] = Fmapped[3 * f + c];
    }
}

__global__ void k_final_counts(const int64_t* __restrict__ is_rep, const int64_t* __restrict__ new_idx, int64_t nv,
                               const int64_t* __restrict__ keep, const int64_t* __restrict__ fnew, int64_t nf,
                               int64_t* __restrict__ counts) {
    counts[0] = nv > 0 ? new_idx[nv - 1] + is_rep[nv - 1] : 0;
    counts[1] = nf > 0 ? fnew[nf - 1] + keep[nf - 1] : 0;
}

uint64_t hash_cap(int64_t nv) {
    uint64_t c = 16;
    while (c < 2 * (uint64_t)(nv > 0 ? nv : 1)) c <<= 1;
    return c;
}

size_t a256(size_t b) { return (b + 255) / 256 * 256; }

struct FinalizeWs {
    Key* keys;
    long long* slot_owner;
    long long* slot_first;
    int64_t *slot_of, *rep, *is_rep, *new_idx;
    int64_t *Fmapped, *keep, *fnew;
    int64_t* scan;
};

size_t finalize_layout(int64_t nv, int64_t nf, uint8_t* base, FinalizeWs* w) {
    const uint64_t cap = hash_cap(nv);
    const int64_t mx = nv > nf ? nv : nf;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        uint8_t* p = base ? base + off : nullptr;
        off += a256(bytes);
        return p;
    };
    FinalizeWs t;
    t.keys = (Key*)take(sizeof(Key) * (size_t)nv);
    t.slot_owner = (long long*)take(8 * cap);
    t.slot_first = (long long*)take(8 * cap);
    t.slot_of = (int64_t*)take(8 * (size_t)nv);
    t.rep = (int64_t*)take(8 * (size_t)nv);
    t.is_rep = (int64_t*)take(8 * (size_t)nv);
    t.new_idx = (int64_t*)take(8 * (size_t)nv);
    t.Fmapped = (int64_t*)take(24 * (size_t)nf);
    t.keep = (int64_t*)take(8 * (size_t)nf);
    t.fnew = (int64_t*)take(8 * (size_t)nf);
    t.scan = (int64_t*)take(8 * scan_ws_elems(mx > 0 ? mx : 1));
    if (w) *w = t;
    return off;
}

}  // namespace
}  // namespace gbsdf

using namespace gbsdf;

extern "C" size_t gbsdf_mesh_finalize_workspace_size(int64_t nv, int64_t nf) {
    if (nv < 0 || nf < 0) return 0;
    return finalize_layout(nv, nf, nullptr, nullptr);
}

extern "C" int gbsdf_mesh_finalize(const double* V, int64_t nv, const int64_t* F, int64_t nf, int weld,
                                   double weld_mult, double scale, const double* offset, double min_side,
                                   void* workspace, size_t workspace_bytes, double* V_out, int64_t* F_out,
                                   int64_t* counts, int* err, void* stream) {
    clear_error();
    GBSDF_CHECK_ARG(nv >= 0 && nf >= 0, "negative sizes");
    GBSDF_CHECK_ARG(counts != nullptr, "counts NULL");
    GBSDF_CHECK_ARG((nv == 0 || (V && V_out)) && (nf == 0 || (F && F_out)), "NULL mesh pointer");
    GBSDF_CHECK_ARG(!weld || weld_mult > 0.0, "weld multiplier %g must be positive", weld_mult);
    const size_t need = finalize_layout(nv, nf, nullptr, nullptr);
    GBSDF_CHECK_ARG(workspace && workspace_bytes >= need, "workspace: %zu bytes needed", need);
    GBSDF_CHECK_ARG(aligned(workspace, 256), "workspace must be 256-byte aligned");
    cudaStream_t s = as_stream(stream);
    FinalizeWs w;
    finalize_layout(nv, nf, (uint8_t*)workspace, &w);
    const int T = 256;
    Xform t;
    t.scale = scale;
    t.ox = offset ? offset[0] : 0.0;
    t.oy = offset ? offset[1] : 0.0;
    t.oz = offset ? offset[2] : 0.0;
    if (nv > 0) {
        const unsigned gv = (unsigned)((nv + T - 1) / T);
        if (weld) {
            const uint64_t cap = hash_cap(nv);
            const unsigned gc = (unsigned)((cap + T - 1) / T);
            k_quantise<<<gv, T, 0, s>>>(V, nv, weld_mult, w.keys);
            k_fill64<<<gc, T, 0, s>>>(w.slot_owner, (int64_t)cap, -1ll);
            k_fill64<<<gc, T, 0, s>>>(w.slot_first, (int64_t)cap, (long long)INT64_MAX);
            k_hash_insert<<<gv, T, 0, s>>>(w.keys, nv, w.slot_owner, cap, w.slot_of, err);
            k_hash_first<<<gv, T, 0, s>>>(w.slot_of, nv, w.slot_first);
            k_reps<<<gv, T, 0, s>>>(w.slot_of, w.slot_first, nv, w.rep, w.is_rep);
        } else {
            k_identity<<<gv, T, 0, s>>>(nv, w.rep, w.is_rep);
        }
        exclusive_scan(w.is_rep, w.new_idx, nv, w.scan, nullptr, s);
        k_write_vertices<<<gv, T, 0, s>>>(V, nv, w.is_rep, w.new_idx, t, V_out);
    }
    if (nf > 0) {
        const unsigned gf = (unsigned)((nf + T - 1) / T);
        k_faces<<<gf, T, 0, s>>>(F, nf, nv, w.rep, w.new_idx, V_out, min_side, w.Fmapped, w.keep, err);
        exclusive_scan(w.keep, w.fnew, nf, w.scan, nullptr, s);
        k_compact_faces<<<gf, T, 0, s>>>(w.Fmapped, w.keep, w.fnew, nf, F_out);
    }
    k_final_counts<<<1, 1, 0, s>>>(w.is_rep, w.new_idx, nv, w.keep, w.fnew, nf, counts);
    return launch_status("mesh finalize");
}
