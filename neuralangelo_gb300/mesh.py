"""Block-wise SDF lattice evaluation and GPU marching cubes (mesh extraction).

Mirrors projects/neuralangelo/utils/mesh.py: ``extract_mesh(sdf_func, bounds,
intv, block_res)`` walks the LatticeGrid blocks (:68-101) in order, evaluates
the SDF on each (block_res + 1)^3 lattice block, runs marching cubes at iso 0
and the unit-sphere filter (:119-148) and concatenates the blocks without
welding (:43-46).  ``sdf_func`` is either a FieldSDF (the fused lattice kernel
of libgbsdf; sign -1 as scripts/extract_mesh.py:85) or any callable taking an
[nx, ny, nz, 3] CUDA tensor and returning [nx, ny, nz, 1] like the reference's.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .fused import pack_sdf, sdf_weight_args

c_i32, c_i64, c_vp, c_dbl, c_sz = ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_double, ctypes.c_size_t
_lib.register("gbsdf_mc_block", [c_vp, c_i32, c_i32, c_i32, c_dbl, c_vp, c_dbl, c_vp, c_sz, c_vp, c_i64, c_vp, c_i64,
                                 c_vp, c_vp])
_lib.register("gbsdf_mc_table", [c_vp, c_vp])
_lib.register("gbsdf_mc_block_noalloc", [c_vp, c_i32, c_i32, c_i32, c_dbl, c_vp, c_dbl, c_vp, c_i64, c_vp, c_i64,
                                         c_vp, c_vp])

_lib.register("gbsdf_mesh_finalize", [c_vp, c_i64, c_vp, c_i64, c_i32, c_dbl, c_dbl, c_vp, c_dbl, c_vp, c_sz, c_vp,
                                      c_vp, c_vp, c_vp, c_vp])

NOALLOC_MAX_POINTS = 33
MERGE_DIGITS = 8          # trimesh's merge tolerance, 1e-8
MERGE_TOL = 1e-8


def marching_cubes_noalloc(vol, origin, intv, V, F, counts, iso=0.0):
    """gbsdf_mc_block_noalloc: marching cubes of one block (<= 33 points per axis) using
    the library's fixed device scratch, for callers that must not allocate device
    memory.  V [>= 3 nx ny nz, 3] float64, F [>= 5 (nx-1)(ny-1)(nz-1), 3] int64 and
    counts [2] int64 are caller-owned device buffers; returns the filled views."""
    nx, ny, nz = vol.shape
    org = (ctypes.c_double * 3)(*[float(o) for o in origin])
    _lib.call("gbsdf_mc_block_noalloc", c_vp(vol.data_ptr()), nx, ny, nz, float(iso), org, float(intv),
              c_vp(V.data_ptr()), V.shape[0], c_vp(F.data_ptr()), F.shape[0], c_vp(counts.data_ptr()),
              _lib.stream_ptr(vol.device))
    nv, nf = counts.tolist()
    return V[:nv], F[:nf]


def _ws_size(nx, ny, nz):
    lib = _lib.load()
    lib.gbsdf_mc_workspace_size.restype = c_sz
    lib.gbsdf_mc_workspace_size.argtypes = [c_i32, c_i32, c_i32]
    return int(lib.gbsdf_mc_workspace_size(nx, ny, nz))


def mc_table():
    """Case table of the library: ([256,16,3] int32, [256] int32); host-only call."""
    tri = np.zeros((256, 16, 3), np.int32)
    cnt = np.zeros(256, np.int32)
    _lib.call("gbsdf_mc_table", tri.ctypes.data_as(c_vp), cnt.ctypes.data_as(c_vp))
    return tri, cnt


class FieldSDF:
    """SDF of a NeuralSDF evaluated by the fused lattice kernel (FP16 table and
    weights, FP32 head); ``sign`` = -1 gives the negated field the mesh extraction
    uses (scripts/extract_mesh.py:85)."""

    def __init__(self, neural_sdf, sign=-1.0):
        self.sdf = neural_sdf
        self.sign = float(sign)
        self.pk, self.A, self.K0 = pack_sdf(neural_sdf)
        self.args = sdf_weight_args(neural_sdf, self.pk, self.A, self.K0)

    def points(self, pts):
        pts = pts.reshape(-1, 3).contiguous().float()
        out = torch.empty(pts.shape[0], device=pts.device, dtype=torch.float32)
        _lib.call("gbsdf_sdf_points", ctypes.byref(self.args), pts.shape[0], c_vp(pts.data_ptr()), None, None, None,
                  0, 0, 0, ctypes.c_float(self.sign), c_vp(out.data_ptr()), _lib.stream_ptr(pts.device))
        return out

    def lattice(self, xs, ys, zs):
        """xs, ys, zs: float32 CUDA axis tensors -> [nx, ny, nz] float32."""
        nx, ny, nz = len(xs), len(ys), len(zs)
        out = torch.empty(nx, ny, nz, device=xs.device, dtype=torch.float32)
        _lib.call("gbsdf_sdf_points", ctypes.byref(self.args), nx * ny * nz, None, c_vp(xs.data_ptr()),
                  c_vp(ys.data_ptr()), c_vp(zs.data_ptr()), nx, ny, nz, ctypes.c_float(self.sign),
                  c_vp(out.data_ptr()), _lib.stream_ptr(xs.device))
        return out


class MarchingCubes:
    """GPU marching cubes + sphere filter for blocks up to ``max_points`` per axis;
    device buffers (workspace and worst-case outputs) are allocated once."""

    def __init__(self, max_points, device="cuda"):
        n = max_points
        self.n = n
        self.ws = torch.empty(_ws_size(n, n, n), dtype=torch.uint8, device=device)
        self.V = torch.empty(3 * n ** 3, 3, dtype=torch.float64, device=device)
        self.F = torch.empty(5 * (n - 1) ** 3, 3, dtype=torch.int64, device=device)
        self.counts = torch.zeros(2, dtype=torch.int64, device=device)

    def __call__(self, vol, origin, intv, iso=0.0):
        nx, ny, nz = vol.shape
        if max(nx, ny, nz) > self.n:
            raise ValueError("block larger than the MarchingCubes capacity")
        vol = vol.contiguous().float()
        org = (ctypes.c_double * 3)(*[float(o) for o in origin])
        _lib.call("gbsdf_mc_block", c_vp(vol.data_ptr()), nx, ny, nz, float(iso), org, float(intv),
                  c_vp(self.ws.data_ptr()), self.ws.numel(), c_vp(self.V.data_ptr()), self.V.shape[0],
                  c_vp(self.F.data_ptr()), self.F.shape[0], c_vp(self.counts.data_ptr()),
                  _lib.stream_ptr(vol.device))
        nv, nf = self.counts.tolist()
        return self.V[:nv], self.F[:nf]


class Mesh:
    """Minimal stand-in for the trimesh.Trimesh the reference returns: vertices
    [nv,3] float64 and faces [nf,3] int64 (numpy)."""

    def __init__(self, vertices, faces, colors=None):
        self.vertices = vertices
        self.faces = faces
        self.colors = colors            # uint8 [nv, 3] for a textured mesh


def finalize_mesh(V, F, weld=False, digits=MERGE_DIGITS, scale=1.0, offset=(0.0, 0.0, 0.0), min_side=MERGE_TOL):
    """gbsdf_mesh_finalize on device tensors V [nv,3] float64, F [nf,3] int64:
    optional weld (coordinates equal at ``digits`` decimals, first occurrence kept)
    -> V * scale + offset -> faces re-indexed, degenerate ones dropped (min_side > 0:
    both heights 2A/|v1-v0|, 2A/|v2-v0| must exceed it; 0: only repeated indices;
    < 0: none).  Returns (V', F') device tensors."""
    _lib.require_cuda(V, F)
    V = V.contiguous().to(torch.float64)
    F = F.contiguous().to(torch.int64)
    nv, nf = V.shape[0], F.shape[0]
    lib = _lib.load()
    lib.gbsdf_mesh_finalize_workspace_size.restype = c_sz
    lib.gbsdf_mesh_finalize_workspace_size.argtypes = [c_i64, c_i64]
    ws = torch.empty(int(lib.gbsdf_mesh_finalize_workspace_size(nv, nf)) + 256, dtype=torch.uint8, device=V.device)
    pad = (-ws.data_ptr()) % 256
    Vo = torch.empty(max(nv, 1), 3, dtype=torch.float64, device=V.device)
    Fo = torch.empty(max(nf, 1), 3, dtype=torch.int64, device=V.device)
    counts = torch.zeros(2, dtype=torch.int64, device=V.device)
    err = torch.zeros(1, dtype=torch.int32, device=V.device)
    off = (c_dbl * 3)(*[float(o) for o in offset])
    _lib.call("gbsdf_mesh_finalize", c_vp(V.data_ptr()), nv, c_vp(F.data_ptr()), nf, 1 if weld else 0,
              float(10 ** digits), float(scale), off, float(min_side), c_vp(ws.data_ptr() + pad), ws.numel() - pad,
              c_vp(Vo.data_ptr()), c_vp(Fo.data_ptr()), c_vp(counts.data_ptr()), c_vp(err.data_ptr()),
              _lib.stream_ptr(V.device))
    if int(err.item()) != 0:
        raise RuntimeError(f"gbsdf_mesh_finalize reported device error {int(err.item())}")
    nv2, nf2 = counts.tolist()
    return Vo[:nv2], Fo[:nf2]


def write_ply(path, vertices, faces, colors=None):
    """Binary little-endian PLY with the element layout of the reference's export
    (trimesh, scripts/extract_mesh.py:100): float32 x y z [uchar red green blue alpha],
    faces as a uchar count and three int32 indices."""
    V = np.asarray(vertices, np.float64).reshape(-1, 3)
    F = np.asarray(faces, np.int64).reshape(-1, 3)
    vdt = [("xyz", "<f4", (3,))]
    if colors is not None:
        C = np.asarray(colors, np.uint8).reshape(len(V), -1)
        if C.shape[1] == 3:
            C = np.concatenate([C, np.full((len(V), 1), 255, np.uint8)], axis=1)
        vdt.append(("rgba", "u1", (4,)))
    vrec = np.empty(len(V), dtype=vdt)
    vrec["xyz"] = V.astype(np.float32)
    if colors is not None:
        vrec["rgba"] = C
    frec = np.empty(len(F), dtype=[("n", "u1"), ("idx", "<i4", (3,))])
    frec["n"] = 3
    frec["idx"] = F.astype(np.int32)
    head = ["ply", "format binary_little_endian 1.0", "comment gbsdf mesh export", f"element vertex {len(V)}",
            "property float x", "property float y", "property float z"]
    if colors is not None:
        head += ["property uchar red", "property uchar green", "property uchar blue", "property uchar alpha"]
    head += [f"element face {len(F)}", "property list uchar int vertex_indices", "end_header"]
    with open(path, "wb") as fh:
        fh.write(("\n".join(head) + "\n").encode("ascii"))
        fh.write(vrec.tobytes())
        fh.write(frec.tobytes())


def read_ply(path):
    """The files write_ply makes: (vertices float32 [nv,3], faces int64 [nf,3], rgba or None)."""
    with open(path, "rb") as fh:
        data = fh.read()
    end = data.index(b"end_header\n") + len(b"end_header\n")
    lines = data[:end].decode("ascii").split("\n")
    if lines[0] != "ply" or lines[1] != "format binary_little_endian 1.0":
        raise ValueError("not a binary little-endian PLY")
    nv = int(next(ln.split()[2] for ln in lines if ln.startswith("element vertex")))
    nf = int(next(ln.split()[2] for ln in lines if ln.startswith("element face")))
    has_rgba = "property uchar red" in lines
    vdt = [("xyz", "<f4", (3,))] + ([("rgba", "u1", (4,))] if has_rgba else [])
    vrec = np.frombuffer(data, dtype=vdt, count=nv, offset=end)
    frec = np.frombuffer(data, dtype=[("n", "u1"), ("idx", "<i4", (3,))], count=nf,
                         offset=end + vrec.nbytes)
    if nf and not np.all(frec["n"] == 3):
        raise ValueError("only triangle faces are supported")
    return vrec["xyz"].copy(), frec["idx"].astype(np.int64), (vrec["rgba"].copy() if has_rgba else None)


def export_mesh(mesh, path, sphere_radius=1.0, sphere_center=(0.0, 0.0, 0.0), device="cuda"):
    """scripts/extract_mesh.py:96-100 on the GPU: vertices * sphere_radius +
    sphere_center, drop the degenerate faces (trimesh's tolerance 1e-8), write the
    PLY.  Returns the exported Mesh."""
    V = torch.as_tensor(np.asarray(mesh.vertices, np.float64), device=device).reshape(-1, 3)
    F = torch.as_tensor(np.asarray(mesh.faces, np.int64), device=device).reshape(-1, 3)
    Vo, Fo = finalize_mesh(V, F, weld=False, scale=sphere_radius, offset=sphere_center, min_side=MERGE_TOL)
    out = Mesh(Vo.cpu().numpy(), Fo.cpu().numpy(), getattr(mesh, "colors", None))
    write_ply(path, out.vertices, out.faces, colors=out.colors)
    return out


def largest_component(V, F, C=None):
    """filter_largest_cc (mesh.py:151-158) on one block's mesh: (V, F, C) of the component
    of largest area.  Components as trimesh's ``split(only_watertight=False)`` defines them:
    faces are joined by the edges that exactly two faces share (its face adjacency), and
    every component counts, whatever its size.  Of equal areas the component holding the
    lowest face index wins.  The kept vertices stay in index order (as trimesh's submesh
    takes them) and the faces are re-indexed from 0, in ascending face order.  Host code,
    as the reference's is (numpy + scipy); C is per-vertex colours or None."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    V = np.asarray(V)
    F = np.asarray(F, np.int64).reshape(-1, 3)
    if len(F) == 0 or len(V) == 0:
        return V[:0], F[:0], (None if C is None else np.asarray(C)[:0])
    nf = len(F)
    e = np.sort(F[:, [0, 1, 1, 2, 2, 0]].reshape(-1, 2), axis=1)          # 3 edges per face
    key = e[:, 0] * np.int64(len(V)) + e[:, 1]
    order = np.argsort(key, kind="stable")
    ks = key[order]
    start = np.flatnonzero(np.r_[True, ks[1:] != ks[:-1]])
    count = np.diff(np.r_[start, len(ks)])
    pair = start[count == 2]                                               # edges of exactly two faces
    fa, fb = order[pair] // 3, order[pair + 1] // 3
    graph = coo_matrix((np.ones(len(fa), np.int8), (fa, fb)), shape=(nf, nf))
    n_comp, labels = connected_components(graph, directed=False)
    # scipy numbers components in order of their lowest node: label order = lowest face order
    T = V[F].astype(np.float64)
    area = 0.5 * np.linalg.norm(np.cross(T[:, 1] - T[:, 0], T[:, 2] - T[:, 0]), axis=1)
    keep = int(np.argmax(np.bincount(labels, weights=area, minlength=n_comp)))
    Fk = F[labels == keep]
    used, inv = np.unique(Fk.reshape(-1), return_inverse=True)
    return V[used], inv.reshape(-1, 3).astype(np.int64), (None if C is None else np.asarray(C)[used])


def lattice_axes(bounds, intv, device):
    """LatticeGrid axes: torch.arange(min, max, intv) in float32 (mesh.py:74-76)."""
    return [torch.arange(lo, hi, intv).to(device) for lo, hi in bounds]


def extract_mesh(sdf_func, bounds, intv, block_res=64, texture_func=None, filter_lcc=False, device="cuda",
                 merge_vertices=False):
    """extract_mesh of the reference (mesh.py:25-49) on the GPU; returns a Mesh.
    merge_vertices=True also runs the per-block vertex merge that the reference's
    trimesh.Trimesh(V, F) applies (mesh.py:124-126: coordinates equal at 8 decimals),
    keeping every face as trimesh does there.  texture_func (points [n,3] numpy -> uint8
    colours [n,3], e.g. ``inference.extract_texture`` bound to a model) colours each
    block's vertices, as marching_cubes does before its sphere filter (mesh.py:121-128).
    filter_lcc=True keeps each block's largest connected component (mesh.py:130, ``largest_component``)."""
    axes = lattice_axes(bounds, intv, device)
    nblk = [int(np.ceil(len(a) / block_res)) for a in axes]
    mc = MarchingCubes(block_res + 1, device)
    Vs, Fs, Cs, off = [], [], [], 0
    for bx in range(nblk[0]):
        for by in range(nblk[1]):
            for bz in range(nblk[2]):
                sl = [slice(b * block_res, b * block_res + block_res + 1) for b in (bx, by, bz)]
                xs, ys, zs = axes[0][sl[0]], axes[1][sl[1]], axes[2][sl[2]]
                if min(len(xs), len(ys), len(zs)) < 2:
                    continue
                if isinstance(sdf_func, FieldSDF):
                    vol = sdf_func.lattice(xs, ys, zs)
                else:
                    X, Y, Z = torch.meshgrid(xs, ys, zs, indexing="ij")
                    vol = sdf_func(torch.stack([X, Y, Z], dim=-1))[..., 0]
                origin = (float(xs[0]), float(ys[0]), float(zs[0]))
                V, F = mc(vol, origin, intv)
                if V.shape[0] == 0:
                    continue
                if merge_vertices or filter_lcc:
                    # the reference's trimesh.Trimesh(V, F) merges equal vertices before split():
                    # without the weld, vertices that several edges emit at an exact-zero lattice
                    # value would cut face adjacency and could change the component kept
                    V, F = finalize_mesh(V, F, weld=True, min_side=-1.0)
                Vb, Fb = V.cpu().numpy(), F.cpu().numpy()
                Cb = np.asarray(texture_func(Vb), np.uint8).reshape(-1, 3) if texture_func is not None else None
                if filter_lcc:
                    Vb, Fb, Cb = largest_component(Vb, Fb, Cb)
                    if len(Vb) == 0:
                        continue
                Vs.append(Vb)
                Fs.append(Fb + off)
                if Cb is not None:
                    Cs.append(Cb)
                off += Vb.shape[0]
    if not Vs:
        return Mesh(np.zeros((0, 3)), np.zeros((0, 3), np.int64),
                    np.zeros((0, 3), np.uint8) if texture_func is not None else None)
    return Mesh(np.concatenate(Vs), np.concatenate(Fs), np.concatenate(Cs) if Cs else None)
