/*
 * CPU marching cubes + sphere filter + block concatenation (oracle).
 *
 * TEST INFRASTRUCTURE ONLY -- the checker for the GPU mesh extraction.
 *
 * Restates the mesh path of projects/neuralangelo/utils/mesh.py:
 *   marching_cubes (mesh.py:119-133): iso-surface at 0 of one block volume,
 *     vertices V in index space, V * intv + xyz[0,0,0];
 *   filter_points_outside_bounding_sphere (mesh.py:136-148): keep vertices with
 *     |v| < 1, keep faces whose three vertices are kept, re-index;
 *   extract_mesh (mesh.py:25-49): blocks in LatticeGrid order, concatenated
 *     without welding (vertex indices offset by the earlier blocks' counts).
 * The per-cube triangulation is the third-party PyMCubes package's job in the
 * reference (requirements.txt:23, unpinned, absent here), so this file states its
 * own canonical triangulation and is "parity unpinned" against PyMCubes:
 *
 *   corner c = (c&1, c>>1&1, c>>2&1); edge e: axis a = e/4, the other two axes
 *   (ascending) take the bits of e%4; a corner is positive when v > iso.
 *   On each face, walked counter-clockwise as seen from outside the cube, a cut
 *   segment runs from every "exit" crossing (positive -> non-positive) to the
 *   "entry" crossing that precedes the run of positive corners ending there, so
 *   positive corners of ambiguous faces are separated; both cubes sharing a face
 *   cut it identically, so the surface is crack-free.  Segments link into loops
 *   (each crossing edge starts one segment and ends one); loops are listed by
 *   their smallest edge id and fanned from it as (v0, v[i+1], v[i]), which turns
 *   triangle normals towards the non-positive side.
 *   Vertex of a crossing edge: t = (iso - v0) / (v1 - v0) in double, from the
 *   lower corner along the edge axis.  Vertices are numbered by global edge id
 *   ((i*ny + j)*nz + k)*3 + axis; triangles by cube (x-major), then loop order.
 *
 * Build: oracle/build_oracle.py (gcc -O2 -shared -fPIC -ffp-contract=off).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static void edge_corners(int e, int* c0, int* c1) {
    const int a = e / 4, r = e % 4;
    int lo;
    if (a == 0) lo = ((r & 1) << 1) | ((r >> 1) << 2);
    else if (a == 1) lo = (r & 1) | ((r >> 1) << 2);
    else lo = (r & 1) | ((r >> 1) << 1);
    *c0 = lo;
    *c1 = lo | (1 << a);
}

static int edge_between(int ca, int cb) {
    const int d = ca ^ cb;
    const int a = d == 1 ? 0 : (d == 2 ? 1 : 2);
    const int lo = ca & cb;
    int r;
    if (a == 0) r = ((lo >> 1) & 1) | (((lo >> 2) & 1) << 1);
    else if (a == 1) r = (lo & 1) | (((lo >> 2) & 1) << 1);
    else r = (lo & 1) | (((lo >> 1) & 1) << 1);
    return a * 4 + r;
}

/* the four corners of face f (axis n = f/2, side s = f%2) counter-clockwise from outside */
static void face_cycle(int f, int* cyc) {
    const int n = f / 2, s = f % 2;
    const int u = (n + 1) % 3, w = (n + 2) % 3;
    const int uv[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
    for (int k = 0; k < 4; ++k) {
        const int kk = s ? k : (4 - k) % 4;   /* reversed on the low side */
        const int cu = uv[kk][0], cw = uv[kk][1];
        cyc[k] = (s << n) | (cu << u) | (cw << w);
    }
}

/* triangles of one cube configuration: returns the count, tri[3*t + i] = edge ids */
static int cube_triangles(int config, int* tri) {
    int next[12];
    for (int e = 0; e < 12; ++e) next[e] = -1;
    for (int f = 0; f < 6; ++f) {
        int cyc[4];
        face_cycle(f, cyc);
        int pos[4];
        for (int k = 0; k < 4; ++k) pos[k] = (config >> cyc[k]) & 1;
        for (int k = 0; k < 4; ++k) {
            if (pos[k] && !pos[(k + 1) % 4]) {               /* exit after corner k */
                int j = k;
                while (pos[j]) j = (j + 3) % 4;               /* first non-positive corner going back */
                const int from = edge_between(cyc[k], cyc[(k + 1) % 4]);
                const int to = edge_between(cyc[j], cyc[(j + 1) % 4]);
                next[from] = to;
            }
        }
    }
    int visited[12] = {0};
    int nt = 0;
    for (int e = 0; e < 12; ++e) {
        if (next[e] < 0 || visited[e]) continue;
        int loop[12], m = 0, x = e;
        while (!visited[x]) {
            visited[x] = 1;
            loop[m++] = x;
            x = next[x];
        }
        for (int i = 1; i + 1 < m; ++i) {
            tri[3 * nt + 0] = loop[0];
            tri[3 * nt + 1] = loop[i + 1];
            tri[3 * nt + 2] = loop[i];
            ++nt;
        }
    }
    return nt;
}

/* exported for the table comparison against the GPU library */
int mc_oracle_cube(int config, int* tri) { return cube_triangles(config, tri); }

/*
 * One block: vol [nx][ny][nz] float32 (x-major), iso, origin (float32, promoted to
 * double), intv (double).  Outputs are caller-allocated with capacity hints; the
 * function returns the number of vertices after the sphere filter in *nv and faces
 * in *nf.  Vertex world positions: index-space position * intv + origin (double),
 * then |v| < 1 kept (mesh.py:123, 139).
 * Capacities: V_cap vertices (3 doubles each), F_cap faces (3 int64 each).
 * Returns 0 on success, -1 when a capacity is exceeded.
 */
int mc_oracle_block(const float* vol, int nx, int ny, int nz, double iso, const float* origin, double intv,
                    double* V, int64_t V_cap, int64_t* F, int64_t F_cap, int64_t* nv_out, int64_t* nf_out) {
    const int64_t nedges = (int64_t)nx * ny * nz * 3;
    int64_t* vidx = (int64_t*)malloc(sizeof(int64_t) * (size_t)nedges);
    if (!vidx) return -1;
    /* pass 1: crossing edges in global edge order -> vertex index */
    int64_t nv = 0;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k)
                for (int a = 0; a < 3; ++a) {
                    const int64_t g = (((int64_t)i * ny + j) * nz + k) * 3 + a;
                    vidx[g] = -1;
                    const int i1 = i + (a == 0), j1 = j + (a == 1), k1 = k + (a == 2);
                    if (i1 >= nx || j1 >= ny || k1 >= nz) continue;
                    const double v0 = vol[((int64_t)i * ny + j) * nz + k];
                    const double v1 = vol[((int64_t)i1 * ny + j1) * nz + k1];
                    const int p0 = v0 > iso, p1 = v1 > iso;
                    if (p0 == p1) continue;
                    if (nv >= V_cap) {
                        free(vidx);
                        return -1;
                    }
                    const double t = (iso - v0) / (v1 - v0);
                    double idx[3] = {(double)i, (double)j, (double)k};
                    idx[a] = idx[a] + t;
                    for (int d = 0; d < 3; ++d) V[3 * nv + d] = idx[d] * intv + (double)origin[d];
                    vidx[g] = nv++;
                }
    /* pass 2: triangles per cube, x-major */
    int64_t nf = 0;
    int tri[3 * 16];
    for (int i = 0; i + 1 < nx; ++i)
        for (int j = 0; j + 1 < ny; ++j)
            for (int k = 0; k + 1 < nz; ++k) {
                int config = 0;
                for (int c = 0; c < 8; ++c) {
                    const int64_t o = ((int64_t)(i + (c & 1)) * ny + (j + ((c >> 1) & 1))) * nz + (k + ((c >> 2) & 1));
                    if ((double)vol[o] > iso) config |= 1 << c;
                }
                if (config == 0 || config == 255) continue;
                const int nt = cube_triangles(config, tri);
                for (int t = 0; t < nt; ++t) {
                    if (nf >= F_cap) {
                        free(vidx);
                        return -1;
                    }
                    for (int q = 0; q < 3; ++q) {
                        int c0, c1;
                        edge_corners(tri[3 * t + q], &c0, &c1);
                        const int a = tri[3 * t + q] / 4;
                        const int64_t g = (((int64_t)(i + (c0 & 1)) * ny + (j + ((c0 >> 1) & 1))) * nz +
                                           (k + ((c0 >> 2) & 1))) * 3 + a;
                        F[3 * nf + q] = vidx[g];
                    }
                    ++nf;
                }
            }
    free(vidx);
    /* sphere filter (mesh.py:136-148): keep |v| < 1 */
    int64_t* remap = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nv > 0 ? nv : 1));
    if (!remap) return -1;
    int64_t kept = 0;
    for (int64_t v = 0; v < nv; ++v) {
        const double x = V[3 * v], y = V[3 * v + 1], z = V[3 * v + 2];
        const double n = sqrt(x * x + y * y + z * z);
        if (n < 1.0) {
            remap[v] = kept;
            if (kept != v) {
                V[3 * kept] = x;
                V[3 * kept + 1] = y;
                V[3 * kept + 2] = z;
            }
            ++kept;
        } else {
            remap[v] = -1;
        }
    }
    int64_t fk = 0;
    for (int64_t f = 0; f < nf; ++f) {
        const int64_t a = remap[F[3 * f]], b = remap[F[3 * f + 1]], c = remap[F[3 * f + 2]];
        if (a < 0 || b < 0 || c < 0) continue;
        F[3 * fk] = a;
        F[3 * fk + 1] = b;
        F[3 * fk + 2] = c;
        ++fk;
    }
    free(remap);
    *nv_out = kept;
    *nf_out = fk;
    return 0;
}
