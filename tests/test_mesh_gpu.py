"""GPU mesh extraction (lattice SDF kernel + marching cubes + sphere filter)
against the CPU oracle on the same SDF values: connectivity bit-exact, vertices
equal to 1e-12 (both use the same double arithmetic)."""
import numpy as np
import pytest
import torch

from neuralangelo_gb300 import mesh as gm
from neuralangelo_gb300.workloads import shapes_union
from oracle import mesh as om

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def volume(kind, n, intv, seed=0):
    g = (np.arange(n) - (n - 1) / 2) * intv
    X, Y, Z = np.meshgrid(g, g, g, indexing='ij')
    if kind == "sphere":
        v = 0.4 - np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    elif kind == "noise":
        v = np.random.default_rng(seed).normal(size=X.shape)
    elif kind == "shapes":
        pts = torch.from_numpy(np.stack([X, Y, Z], -1)).float()
        v = -shapes_union(seed)(pts).numpy()
    else:
        v = -np.ones_like(X)
    return v.astype(np.float32)


@pytest.mark.parametrize("kind,n", [("sphere", 40), ("noise", 33), ("shapes", 64), ("empty", 9), ("noise", 2)])
def test_gpu_marching_cubes_matches_oracle(kind, n):
    intv = 1.6 / max(n, 2)
    vol = volume(kind, n, intv)
    origin = np.full(3, -(n - 1) / 2 * intv, np.float32)
    Vr, Fr = om.marching_cubes_block(vol, origin, intv)
    mc = gm.MarchingCubes(max(n, 2), DEV)
    V, F = mc(torch.from_numpy(vol).to(DEV), [float(o) for o in origin], intv)
    V, F = V.cpu().numpy(), F.cpu().numpy()
    assert F.shape == Fr.shape and np.array_equal(F, Fr)
    assert V.shape == Vr.shape and np.allclose(V, Vr, rtol=0, atol=1e-12)


def test_sphere_filter_drops_outside_vertices():
    n, intv = 12, 0.4            # coordinates up to 2.2: the filter keeps only |v| < 1
    g = (np.arange(n) - (n - 1) / 2) * intv
    X, Y, Z = np.meshgrid(g, g, g, indexing='ij')
    vol = (1.2 - np.sqrt(X ** 2 + Y ** 2 + Z ** 2)).astype(np.float32)
    origin = np.full(3, -(n - 1) / 2 * intv, np.float32)
    Vr, Fr = om.marching_cubes_block(vol, origin, intv)
    V, F = gm.MarchingCubes(n, DEV)(torch.from_numpy(vol).to(DEV), [float(o) for o in origin], intv)
    assert np.array_equal(F.cpu().numpy(), Fr) and V.shape[0] == Vr.shape[0]
    if V.shape[0]:
        assert np.all(np.linalg.norm(V.cpu().numpy(), axis=1) < 1.0)


def small_field():
    from tests.test_fused_gpu import build
    m = build()
    return m.neural_sdf


def test_lattice_sdf_matches_plain_field():
    sdf = small_field()
    f = gm.FieldSDF(sdf, sign=-1.0)
    ax = gm.lattice_axes([(-1, 1)] * 3, 2.0 / 40, DEV)
    vol = f.lattice(ax[0][:17], ax[1][5:30], ax[2][:9])
    X, Y, Z = torch.meshgrid(ax[0][:17], ax[1][5:30], ax[2][:9], indexing="ij")
    with torch.no_grad():
        ref = -sdf.sdf(torch.stack([X, Y, Z], -1))[..., 0]
    e = ((vol - ref).norm() / ref.norm()).item()
    assert e < 1e-4, e
    pts = torch.rand(1000, 3, device=DEV) * 2 - 1
    with torch.no_grad():
        ref_p = sdf.sdf(pts)[:, 0]
    e2 = ((gm.FieldSDF(sdf, sign=1.0).points(pts) - ref_p).norm() / ref_p.norm()).item()
    assert e2 < 1e-4, e2


def test_extract_mesh_blocks_match_oracle_on_same_values():
    sdf = small_field()
    f = gm.FieldSDF(sdf, sign=-1.0)
    bounds, intv, block = [(-1, 1)] * 3, 2.0 / 48, 16
    mesh = gm.extract_mesh(f, bounds, intv, block_res=block, device=DEV)

    def vol_fn(xs, ys, zs):
        return f.lattice(torch.from_numpy(xs).to(DEV), torch.from_numpy(ys).to(DEV),
                         torch.from_numpy(zs).to(DEV)).cpu().numpy()

    Vr, Fr = om.extract_mesh_blocks(vol_fn, bounds, intv, block)
    assert mesh.faces.shape[0] > 100
    assert np.array_equal(mesh.faces, Fr)                         # connectivity: bit-exact
    assert np.allclose(mesh.vertices, Vr, rtol=0, atol=1e-12)
    # geometric init: the zero level set is close to the sphere of radius 0.5
    r = np.linalg.norm(mesh.vertices, axis=1)
    assert abs(np.median(r) - 0.5) < 0.05


def test_extract_mesh_with_callable_like_reference():
    target = shapes_union(1)
    bounds, intv = [(-1, 1)] * 3, 2.0 / 32
    mesh = gm.extract_mesh(lambda x: -target(x)[..., None], bounds, intv, block_res=8, device=DEV)

    def vol_fn(xs, ys, zs):   # the same CUDA evaluation the GPU path makes, so both see identical values
        X, Y, Z = torch.meshgrid(*[torch.from_numpy(a).to(DEV) for a in (xs, ys, zs)], indexing='ij')
        return -target(torch.stack([X, Y, Z], -1)).cpu().numpy()

    Vr, Fr = om.extract_mesh_blocks(vol_fn, bounds, intv, 8)
    assert np.array_equal(mesh.faces, Fr)
    assert np.allclose(mesh.vertices, Vr, rtol=0, atol=1e-12)
