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


def test_fitted_shapes_field_512_lattice_matches_oracle_block_by_block():
    """Mesh extraction from a trained-shape field: the full field (L16 F8 T2^22, 8 active
    levels) fitted to a seeded union of 3 spheres and 2 boxes, a 512^3 lattice in 128^3
    blocks (mesh.py:25-49, scripts/extract_mesh.py:76-99).  Every block's triangles are
    bit-exact against the C marching cubes on the same GPU-evaluated SDF values, vertices
    equal to 1e-12 (the same double arithmetic), and the surface lies on the target shapes."""
    from neuralangelo_gb300.config import field_config
    from neuralangelo_gb300.model import FieldModel
    from neuralangelo_gb300.workloads import fit_sdf, full_field_iteration, init_field_params
    torch.manual_seed(1)
    model = FieldModel(field_config("full")).to(DEV)
    init_field_params(model, 1)
    model.schedule(full_field_iteration(8))
    target = shapes_union(7)
    loss = fit_sdf(model.neural_sdf, target, steps=300)
    f = gm.FieldSDF(model.neural_sdf, sign=-1.0)
    bounds, intv, block = [(-1, 1)] * 3, 2.0 / 512, 128
    mesh = gm.extract_mesh(f, bounds, intv, block_res=block, device=DEV)

    def vol_fn(xs, ys, zs):
        return f.lattice(torch.from_numpy(xs).to(DEV), torch.from_numpy(ys).to(DEV),
                         torch.from_numpy(zs).to(DEV)).cpu().numpy()

    Vr, Fr = om.extract_mesh_blocks(vol_fn, bounds, intv, block)
    with torch.no_grad():
        dist = target(torch.from_numpy(mesh.vertices).to(DEV)).abs()
    print(f"\nfit L1 {loss:.4f}; {mesh.vertices.shape[0]} vertices, {mesh.faces.shape[0]} faces; "
          f"distance to the shapes: median {float(dist.median()):.4f}")
    assert mesh.faces.shape[0] > 100000
    assert np.array_equal(mesh.faces, Fr)                         # connectivity: bit-exact
    assert np.allclose(mesh.vertices, Vr, rtol=0, atol=1e-12)
    assert float(dist.median()) < 0.02                            # the field learned the shapes


# ---------------------------------------------------------------------------- output stage

def planted_mesh(nv, nf, seed):
    """Random mesh with exact and near duplicate vertices (some within the 8-digit merge,
    some just outside it) and degenerate faces of every kind."""
    rng = np.random.default_rng(seed)
    V = rng.uniform(-1, 1, size=(nv, 3))
    dup = rng.choice(nv, size=nv // 5, replace=False)
    src = rng.choice(nv, size=nv // 5)
    V[dup] = V[src] + rng.choice([0.0, 2e-9, -3e-9, 2e-8], size=(nv // 5, 1)) * rng.integers(0, 2, (nv // 5, 3))
    F = rng.integers(0, nv, size=(nf, 3))
    k = nf // 10
    F[:k, 1] = F[:k, 0]                                        # repeated index
    a, b = F[k:2 * k, 0], F[k:2 * k, 1]
    V[F[k:2 * k, 2]] = 0.5 * (V[a] + V[b])                     # (nearly) collinear
    return V, F


@pytest.mark.parametrize("weld", [False, True])
@pytest.mark.parametrize("min_side", [-1.0, 0.0, 1e-8, 1e-3])
def test_finalize_matches_oracle(weld, min_side):
    from oracle import mesh_out as mo
    V, F = planted_mesh(5000, 9000, seed=3)
    scale, offset = 1.7, (0.25, -3.0, 1e-3)
    Vg, Fg = gm.finalize_mesh(torch.from_numpy(V).to(DEV), torch.from_numpy(F).to(DEV), weld=weld, scale=scale,
                              offset=offset, min_side=min_side)
    Vr, Fr = mo.finalize(V, F, weld=weld, scale=scale, offset=offset, height=min_side)
    assert np.array_equal(Vg.cpu().numpy(), Vr)                  # same float64 operations
    assert np.array_equal(Fg.cpu().numpy(), Fr)
    if weld:
        assert len(Vr) < len(V)
    if min_side >= 0:
        assert len(Fr) < len(F)


def test_finalize_weld_at_scale():
    """A million vertices with 30 % duplicates: the hash-table weld against the oracle."""
    from oracle import mesh_out as mo
    rng = np.random.default_rng(5)
    base = rng.integers(-4000, 4000, size=(700_000, 3)) * 1e-4
    V = base[rng.integers(0, len(base), size=1_000_000)]
    F = rng.integers(0, len(V), size=(1_500_000, 3))
    Vg, Fg = gm.finalize_mesh(torch.from_numpy(V).to(DEV), torch.from_numpy(F).to(DEV), weld=True, min_side=0.0)
    Vr, Fr = mo.finalize(V, F, weld=True, height=0.0)
    assert np.array_equal(Vg.cpu().numpy(), Vr) and np.array_equal(Fg.cpu().numpy(), Fr)


def test_finalize_empty_and_bad_index():
    e = torch.zeros(0, 3, dtype=torch.float64, device=DEV)
    Vg, Fg = gm.finalize_mesh(e, torch.zeros(0, 3, dtype=torch.int64, device=DEV), weld=True)
    assert Vg.shape[0] == 0 and Fg.shape[0] == 0
    V = torch.rand(4, 3, dtype=torch.float64, device=DEV)
    F = torch.tensor([[0, 1, 4]], dtype=torch.int64, device=DEV)     # index 4 of 4 vertices
    with pytest.raises(RuntimeError, match="device error 4"):
        gm.finalize_mesh(V, F)


def test_extract_mesh_block_merge_matches_oracle():
    """A field that is exactly zero on lattice points (|x| - 0.5 on the 2/32 lattice, at
    (+-0.5, 0, 0) and its permutations).  A corner counts as positive only when
    v > 0, so each such corner has five positive neighbours and marching cubes emits
    five vertices on it, which the reference's per-block trimesh merge joins."""
    bounds, intv, block = [(-1, 1)] * 3, 2.0 / 32, 8

    def sdf(x):
        return torch.sqrt((x * x).sum(-1, keepdim=True)) - 0.5

    def vol_fn(xs, ys, zs):
        X, Y, Z = torch.meshgrid(*[torch.from_numpy(a).to(DEV) for a in (xs, ys, zs)], indexing='ij')
        return sdf(torch.stack([X, Y, Z], -1))[..., 0].cpu().numpy()

    plain = gm.extract_mesh(sdf, bounds, intv, block_res=block, device=DEV)
    merged = gm.extract_mesh(sdf, bounds, intv, block_res=block, device=DEV, merge_vertices=True)
    Vr, Fr = om.extract_mesh_blocks(vol_fn, bounds, intv, block, merge_vertices=True)
    assert len(merged.vertices) < len(plain.vertices)
    assert np.array_equal(merged.faces, Fr)
    assert np.allclose(merged.vertices, Vr, rtol=0, atol=1e-12)


def test_extract_mesh_largest_component_matches_oracle():
    """filter_lcc (mesh.py:130,151-158): ten small spheres, several per block and some cut
    by the block faces; each block keeps its largest piece, colours follow their vertices
    (on the CPU oracle this drops 662 of 1800 faces)."""
    def target(x):
        g = torch.Generator().manual_seed(11)
        cs = torch.rand(10, 3, generator=g) * 1.4 - 0.7
        rs = 0.06 + 0.1 * torch.rand(10, generator=g)
        return ((x[..., None, :] - cs.to(x)).norm(dim=-1) - rs.to(x)).min(dim=-1).values

    bounds, intv, block = [(-1, 1)] * 3, 2.0 / 40, 16

    def sdf(x):
        return -target(x)[..., None]

    def vol_fn(xs, ys, zs):
        X, Y, Z = torch.meshgrid(*[torch.from_numpy(a).to(DEV) for a in (xs, ys, zs)], indexing='ij')
        return -target(torch.stack([X, Y, Z], -1)).cpu().numpy()

    def colour(v):
        return (np.abs(v) * 200).astype(np.uint8)

    full = gm.extract_mesh(sdf, bounds, intv, block_res=block, device=DEV)
    lcc = gm.extract_mesh(sdf, bounds, intv, block_res=block, device=DEV, filter_lcc=True, texture_func=colour)
    Vr, Fr = om.extract_mesh_blocks(vol_fn, bounds, intv, block, filter_lcc=True)
    assert 0 < len(lcc.faces) < len(full.faces)
    assert np.array_equal(lcc.faces, Fr)
    assert np.allclose(lcc.vertices, Vr, rtol=0, atol=1e-12)
    assert np.array_equal(lcc.colors, colour(lcc.vertices))


def test_export_mesh_writes_the_oracle_mesh(tmp_path):
    from oracle import mesh_out as mo
    target = shapes_union(2)
    mesh = gm.extract_mesh(lambda x: -target(x)[..., None], [(-1, 1)] * 3, 2.0 / 40, block_res=16, device=DEV)
    radius, center = 2.5, (0.1, -0.2, 3.0)
    out = gm.export_mesh(mesh, tmp_path / "mesh.ply", sphere_radius=radius, sphere_center=center, device=DEV)
    Vr, Fr = mo.finalize(mesh.vertices, mesh.faces, scale=radius, offset=center)
    assert np.array_equal(out.vertices, Vr) and np.array_equal(out.faces, Fr)
    V, F, C = gm.read_ply(tmp_path / "mesh.ply")
    assert C is None and np.array_equal(F, Fr) and np.array_equal(V, Vr.astype(np.float32))
