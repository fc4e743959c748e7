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

NOALLOC_MAX_POINTS = 33


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

    def __init__(self, vertices, faces):
        self.vertices = vertices
        self.faces = faces


def lattice_axes(bounds, intv, device):
    """LatticeGrid axes: torch.arange(min, max, intv) in float32 (mesh.py:74-76)."""
    return [torch.arange(lo, hi, intv).to(device) for lo, hi in bounds]


def extract_mesh(sdf_func, bounds, intv, block_res=64, texture_func=None, filter_lcc=False, device="cuda"):
    """extract_mesh of the reference (mesh.py:25-49) on the GPU; returns a Mesh."""
    if texture_func is not None or filter_lcc:
        raise NotImplementedError("texture and largest-component filtering are outside this path")
    axes = lattice_axes(bounds, intv, device)
    nblk = [int(np.ceil(len(a) / block_res)) for a in axes]
    mc = MarchingCubes(block_res + 1, device)
    Vs, Fs, off = [], [], 0
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
                Vs.append(V.cpu().numpy())
                Fs.append(F.cpu().numpy() + off)
                off += V.shape[0]
    if not Vs:
        return Mesh(np.zeros((0, 3)), np.zeros((0, 3), np.int64))
    return Mesh(np.concatenate(Vs), np.concatenate(Fs))
