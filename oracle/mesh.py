"""Python side of the CPU marching-cubes oracle (oracle/mc.c).

TEST INFRASTRUCTURE ONLY.  extract_mesh_blocks follows
projects/neuralangelo/utils/mesh.py:25-49 (LatticeGrid :68-101) for the block
walk, the block overlap and the concatenation order.
"""
import ctypes

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_oracle.build())
        _lib.mc_oracle_block.restype = ctypes.c_int
        _lib.mc_oracle_cube.restype = ctypes.c_int
    return _lib


def cube_table():
    """[256, 16, 3] edge ids (-1 padded) and [256] triangle counts of the canonical triangulation."""
    tri = (ctypes.c_int * 48)()
    tab = -np.ones((256, 16, 3), np.int32)
    cnt = np.zeros(256, np.int32)
    for c in range(256):
        n = lib().mc_oracle_cube(c, tri)
        cnt[c] = n
        tab[c, :n] = np.array(tri[:3 * n]).reshape(n, 3)
    return tab, cnt


def marching_cubes_block(vol, origin, intv, iso=0.0):
    """vol [nx,ny,nz] float32 -> (V [nv,3] float64, F [nf,3] int64), sphere-filtered (mesh.py:119-148)."""
    vol = np.ascontiguousarray(vol, np.float32)
    nx, ny, nz = vol.shape
    cap_v = 3 * nx * ny * nz + 16
    cap_f = 5 * max(nx - 1, 1) * max(ny - 1, 1) * max(nz - 1, 1) + 16
    V = np.empty((cap_v, 3), np.float64)
    F = np.empty((cap_f, 3), np.int64)
    nv, nf = ctypes.c_int64(0), ctypes.c_int64(0)
    org = np.ascontiguousarray(origin, np.float32)
    st = lib().mc_oracle_block(vol.ctypes.data_as(ctypes.c_void_p), nx, ny, nz, ctypes.c_double(iso),
                               org.ctypes.data_as(ctypes.c_void_p), ctypes.c_double(intv),
                               V.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(cap_v),
                               F.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(cap_f),
                               ctypes.byref(nv), ctypes.byref(nf))
    assert st == 0
    return V[:nv.value].copy(), F[:nf.value].copy()


def lattice_axes(bounds, intv):
    """LatticeGrid axes: torch.arange(min, max, intv) in float32 (mesh.py:74-76)."""
    import torch
    return [torch.arange(lo, hi, intv).numpy() for lo, hi in bounds]


def block_slices(n_points, block_res):
    """Index ranges [b*B, b*B + B] inclusive (mesh.py:86-96)."""
    nb = int(np.ceil(n_points / block_res))
    return [(b * block_res, min(b * block_res + block_res + 1, n_points)) for b in range(nb)]


def extract_mesh_blocks(sdf_volume_fn, bounds, intv, block_res, iso=0.0, merge_vertices=False, filter_lcc=False):
    """sdf_volume_fn(xs, ys, zs) -> float32 [len(xs), len(ys), len(zs)] (already negated
    as extract_mesh.py:85 does).  Returns the concatenated (V, F) over blocks in order;
    merge_vertices applies trimesh's per-block merge (mesh.py:124-126, see mesh_out.py),
    filter_lcc its per-block largest component (mesh.py:130,151-158)."""
    from oracle import mesh_out
    ax = lattice_axes(bounds, intv)
    sx, sy, sz = (block_slices(len(a), block_res) for a in ax)
    Vs, Fs, off = [], [], 0
    for (x0, x1) in sx:
        for (y0, y1) in sy:
            for (z0, z1) in sz:
                xs, ys, zs = ax[0][x0:x1], ax[1][y0:y1], ax[2][z0:z1]
                vol = sdf_volume_fn(xs, ys, zs)
                V, F = marching_cubes_block(vol, np.array([xs[0], ys[0], zs[0]], np.float32), intv, iso)
                if V.shape[0] == 0:
                    continue
                if merge_vertices:
                    V, F = mesh_out.merge_vertices(V, F)
                if filter_lcc:
                    V, F = mesh_out.largest_component(V, F)
                    if V.shape[0] == 0:
                        continue
                Vs.append(V)
                Fs.append(F + off)
                off += V.shape[0]
    if not Vs:
        return np.zeros((0, 3)), np.zeros((0, 3), np.int64)
    return np.concatenate(Vs), np.concatenate(Fs)
