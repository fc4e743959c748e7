"""The mesh output stage's oracle (per-block vertex merge, transform, degenerate
faces) on known answers, and the PLY writer/reader round trip; CPU only."""
import numpy as np

from neuralangelo_gb300 import mesh as gm
from oracle import mesh_out as mo


def test_merge_keeps_first_occurrence_and_reindexes():
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 0, 0], [0, 0, 1], [1 + 4e-9, 0, 0], [0, 1, 6e-9]], float)
    F = np.array([[0, 1, 2], [3, 4, 0], [5, 6, 4]])
    V2, F2 = mo.merge_vertices(V, F)
    # vertices 1, 3 and 5 share an 8-digit key (4e-9 rounds away); 6 has its own (6e-9 -> 1e-8)
    k = np.rint(V * 1e8).astype(np.int64)
    assert len(np.unique(k, axis=0)) == len(V2)
    assert np.array_equal(V2[0], V[0]) and np.array_equal(V2[1], V[1]) and np.array_equal(V2[2], V[2])
    assert np.array_equal(F2[0], [0, 1, 2]) and F2[1, 0] == 1 and F2[2, 0] == 1


def test_merge_rounds_half_to_even():
    # at 0 digits the products are exact: 0.5 -> 0, 1.5 -> 2, 2.5 -> 2
    V = np.array([[0.5, 0, 0], [0, 0, 0], [1.5, 0, 0], [2, 0, 0], [2.5, 0, 0]])
    V2, F2 = mo.merge_vertices(V, np.zeros((0, 3), np.int64), digits=0)
    assert len(V2) == 2 and np.array_equal(V2, V[[0, 2]])


def test_degenerate_faces():
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [2, 0, 0], [0.5, 1e-9, 0], [0, 0, 1e-9]], float)
    F = np.array([[0, 1, 2],      # fine
                  [0, 1, 3],      # collinear: zero area
                  [0, 0, 2],      # repeated index
                  [0, 1, 4],      # height 1e-9 over the unit edge
                  [0, 5, 1]])     # edge v1 - v0 of length 1e-9: its height counts as 0
    assert list(mo.nondegenerate(V, F)) == [True, False, False, False, False]
    assert list(mo.nondegenerate(V, F, 0.0)) == [True, True, False, True, True]
    assert list(mo.nondegenerate(V, F, -1.0)) == [True] * 5


def test_finalize_transforms_then_tests_in_output_coordinates():
    V = np.array([[0, 0, 0], [1e-5, 0, 0], [0, 1e-5, 0]], float)
    F = np.array([[0, 1, 2]])
    # heights 1e-5 pass; scaled by 1e-4 they are 1e-9 and the face goes
    assert len(mo.finalize(V, F)[1]) == 1
    V2, F2 = mo.finalize(V, F, scale=1e-4, offset=(1, 2, 3))
    assert len(F2) == 0 and np.array_equal(V2, V * 1e-4 + np.array([1.0, 2.0, 3.0]))


def test_ply_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    V = rng.normal(size=(50, 3))
    F = rng.integers(0, 50, size=(80, 3))
    C = rng.integers(0, 256, size=(50, 3)).astype(np.uint8)
    p = tmp_path / "m.ply"
    gm.write_ply(p, V, F, colors=C)
    V2, F2, C2 = gm.read_ply(p)
    assert np.array_equal(V2, V.astype(np.float32)) and np.array_equal(F2, F)
    assert np.array_equal(C2[:, :3], C) and np.all(C2[:, 3] == 255)
    head = open(p, "rb").read(300).split(b"end_header")[0].decode()
    assert "format binary_little_endian 1.0" in head and "property list uchar int vertex_indices" in head
    gm.write_ply(p, V, F)
    V3, F3, C3 = gm.read_ply(p)
    assert C3 is None and np.array_equal(F3, F)
    # file size: header + 12 B per vertex + 13 B per face
    hdr_len = open(p, "rb").read().index(b"end_header\n") + len(b"end_header\n")
    assert p.stat().st_size == hdr_len + 12 * 50 + 13 * 80


def test_largest_component_known_answers():
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0],            # a: one triangle
                  [1, 1, 0],                                    # b: shares only vertex 1 with a
                  [3, 0, 0], [5, 0, 0], [3, 2, 0], [5, 2, 0],   # c: two triangles over one edge
                  [3, 1, 1]], float)                            # d: a third face on c's shared edge
    F = np.array([[0, 1, 2], [1, 3, 2], [4, 5, 6], [5, 7, 6], [5, 6, 8]])
    # faces 0 and 1 share edge (1, 2): one component of area 1.  Faces 2, 3 and 4 all hold
    # edge (5, 6): three owners, so trimesh's adjacency skips it and they stay apart
    # (areas 2, 2 and sqrt(3)); of the two of area 2 the lower face index, 2, wins
    V2, F2 = mo.largest_component(V, F)
    assert np.array_equal(V2, V[[4, 5, 6]]) and np.array_equal(F2, [[0, 1, 2]])
    V3, F3, _ = gm.largest_component(V, F)
    assert np.array_equal(V3, V2) and np.array_equal(F3, F2)
    # without face 4, faces 2 and 3 join over (5, 6): area 4 beats faces 0 + 1 (area 1)
    V4, F4 = mo.largest_component(V, F[:4])
    assert np.array_equal(V4, V[[4, 5, 6, 7]]) and np.array_equal(F4, [[0, 1, 2], [1, 3, 2]])


def test_largest_component_ties_vertex_contact_and_empty():
    # two unit triangles touching at one vertex: two components of equal area; the one
    # holding the lowest face index wins
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [2, 0, 0], [1, 1, 0]], float)
    F = np.array([[1, 3, 4], [0, 1, 2]])
    for fn in (mo.largest_component, lambda v, f: gm.largest_component(v, f)[:2]):
        V2, F2 = fn(V, F)
        assert np.array_equal(V2, V[[1, 3, 4]]) and np.array_equal(F2, [[0, 1, 2]])
    V0, F0, C0 = gm.largest_component(V[:0], np.zeros((0, 3), np.int64), np.zeros((0, 3), np.uint8))
    assert V0.shape == (0, 3) and F0.shape == (0, 3) and C0.shape == (0, 3)


def test_largest_component_matches_oracle_on_marching_cubes():
    """Blocks of three spheres (one cut by the block edge) through the marching-cubes oracle;
    colours follow their vertices."""
    from oracle import mesh as om
    n = 40
    ax = np.linspace(-0.95, 0.95, n, dtype=np.float32)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    rng = np.random.default_rng(3)
    for trial in range(3):
        cs = rng.uniform(-0.6, 0.6, (3, 3))
        rs = rng.uniform(0.12, 0.3, 3)
        d = np.min([np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - r for c, r in zip(cs, rs)], axis=0)
        V, F = om.marching_cubes_block(-d.astype(np.float32), ax[[0, 0, 0]], float(ax[1] - ax[0]))
        assert len(F) > 0
        C = (np.arange(len(V) * 3) % 251).astype(np.uint8).reshape(-1, 3)
        Vr, Fr = mo.largest_component(V, F)
        Vg, Fg, Cg = gm.largest_component(V, F, C)
        assert np.array_equal(Vg, Vr) and np.array_equal(Fg, Fr)
        assert 0 < len(Fr) < len(F)
        idx = np.array([np.flatnonzero((V == v).all(axis=1))[0] for v in Vg[:50]])
        assert np.array_equal(Cg[:50], C[idx])
