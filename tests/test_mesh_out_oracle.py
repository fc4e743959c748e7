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
