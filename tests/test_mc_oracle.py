"""Properties of the CPU marching-cubes oracle (oracle/mc.c): crack-free,
consistently oriented surfaces with normals towards the non-positive side,
vertices on the iso-surface, and the reference's block/sphere-filter rules
(projects/neuralangelo/utils/mesh.py:25-49, 68-148)."""
from collections import Counter

import numpy as np
import pytest

from oracle import mesh as om


def directed_edges(F):
    c = Counter()
    for f in F:
        for a, b in ((f[0], f[1]), (f[1], f[2]), (f[2], f[0])):
            c[(int(a), int(b))] += 1
    return c


def watertight(F):
    de = directed_edges(F)
    return all(de[(b, a)] == v for (a, b), v in de.items())


def grid(n, intv):
    g = (np.arange(n) - (n - 1) / 2) * intv
    return np.meshgrid(g, g, g, indexing='ij')


def test_table_covers_every_crossing_edge():
    tab, cnt = om.cube_table()
    assert cnt[0] == 0 and cnt[255] == 0 and cnt.max() <= 5
    for c in range(256):
        used = sorted(set(tab[c, :cnt[c]].reshape(-1).tolist()))
        cross = []
        for e in range(12):
            a, r = e // 4, e % 4
            lo = [((r & 1) << 1) | ((r >> 1) << 2), (r & 1) | ((r >> 1) << 2), (r & 1) | ((r >> 1) << 1)][a]
            if ((c >> lo) & 1) != ((c >> (lo | (1 << a))) & 1):
                cross.append(e)
        assert used == cross, c


@pytest.mark.parametrize("shape", ["sphere", "torus", "noise"])
def test_surface_is_watertight_and_oriented(shape):
    n, intv = 36, 0.03
    X, Y, Z = grid(n, intv)
    if shape == "sphere":
        vol = 0.4 - np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    elif shape == "torus":
        vol = 0.12 - np.sqrt((np.sqrt(X ** 2 + Y ** 2) - 0.3) ** 2 + Z ** 2)
    else:
        vol = np.random.default_rng(0).normal(size=X.shape)
        vol[[0, -1]] = vol[:, [0, -1]] = vol[:, :, [0, -1]] = -5
    vol = vol.astype(np.float32)
    V, F = om.marching_cubes_block(vol, np.full(3, -(n - 1) / 2 * intv, np.float32), intv)
    assert F.shape[0] > 0
    assert watertight(F)
    if shape == "sphere":
        c = V[F].mean(1)
        nrm = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
        assert np.all(np.sum(nrm * c, 1) > 0)          # outward: towards the non-positive side
        r = np.linalg.norm(V, axis=1)
        assert np.all(np.abs(r - 0.4) < 0.01)


def test_vertices_interpolate_linearly():
    # a linear field: vertices sit exactly on its zero plane
    n, intv = 8, 0.1
    X, Y, Z = grid(n, intv)
    vol = (0.3 * X - 0.2 * Y + 0.1 * Z + 0.01).astype(np.float32)
    V, F = om.marching_cubes_block(vol, np.full(3, -(n - 1) / 2 * intv, np.float32), intv)
    assert np.max(np.abs(0.3 * V[:, 0] - 0.2 * V[:, 1] + 0.1 * V[:, 2] + 0.01)) < 1e-6


def test_sphere_filter_and_empty_block():
    n, intv = 10, 0.5          # coordinates reach 2.25: most vertices lie outside |v| < 1
    X, Y, Z = grid(n, intv)
    vol = (1.5 - np.sqrt(X ** 2 + Y ** 2 + Z ** 2)).astype(np.float32)
    V, F = om.marching_cubes_block(vol, np.full(3, -(n - 1) / 2 * intv, np.float32), intv)
    assert V.shape[0] == 0 and F.shape[0] == 0     # everything beyond the unit sphere is dropped
    V, F = om.marching_cubes_block(-np.ones((5, 5, 5), np.float32), np.zeros(3, np.float32), 0.1)
    assert V.shape == (0, 3) and F.shape == (0, 3)


def test_blocks_follow_lattice_grid():
    # 2/res spacing over [-1, 1): 64 points per axis, blocks of 16 -> 4 blocks, the last one 16 points
    ax = om.lattice_axes([(-1, 1)] * 3, 2.0 / 64)
    assert len(ax[0]) == 64 and ax[0][0] == -1.0 and ax[0].dtype == np.float32
    sl = om.block_slices(64, 16)
    assert sl == [(0, 17), (16, 33), (32, 49), (48, 64)]


def test_library_case_table_equals_oracle():
    """The library's table generator (host-only call) against the oracle's per-cube routine."""
    from neuralangelo_gb300.build import build
    from neuralangelo_gb300.mesh import mc_table
    build()
    t1, c1 = mc_table()
    t2, c2 = om.cube_table()
    assert np.array_equal(c1, c2) and np.array_equal(t1, t2)
