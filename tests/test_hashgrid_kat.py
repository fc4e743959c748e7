"""Known-answer tests for the hash-grid restatement (oracle/hashgrid.py).

The hash grid comes from the third-party tiny-cuda-nn package (used at
projects/neuralangelo/utils/modules.py:42-50,85); the reference holds no tests
for it, so these values are worked out by hand from the published scheme:
dense index x + y*res + z*res^2 while res^3 fits the level, else
(x*1) ^ (y*2654435761) ^ (z*805459861) mod 2^32 mod T.
"""
import numpy as np

from oracle import hashgrid as hg


def test_layout_full_field():
    # L=16, F=8, T=2^22, 32 -> 2048 (growth 64^(1/15)); level 5 lands on scale 127.000015
    # (log2 of the float32 growth rounds up), so it is 129^3, not 128^3.
    g = float(np.exp((np.log(2048) - np.log(32)) / 15))
    lay = hg.level_layout(16, 8, 22, 32, g)
    assert list(lay['resolution'][:8]) == [32, 43, 56, 74, 98, 129, 169, 223]
    assert list(lay['size'][:6]) == [32 ** 3, 79512, 56 ** 3, 405224, 98 ** 3, 2146696]
    assert all(s == 1 << 22 for s in lay['size'][6:])
    assert list(lay['hashed']) == [False] * 6 + [True] * 10
    assert lay['n_entries'] == 45724048


def test_layout_small_field():
    lay = hg.level_layout(8, 4, 16, 16, 1.5)
    assert list(lay['resolution']) == [16, 24, 36, 54, 81, 122, 183, 274]
    assert list(lay['size']) == [4096, 13824, 46656] + [65536] * 5
    assert lay['n_entries'] == 392256
    assert lay['scale'][0] == np.float32(15.0)


def test_dense_index_by_hand():
    lay = hg.level_layout(8, 4, 16, 16, 1.5)
    # level 0: scale 15, res 16.  x = (0.3, 0.5, 0.9) -> p = 15x + 0.5 = (5.0, 8.0, 14.0)
    x = np.array([[0.3, 0.5, 0.9]], np.float32)
    idx, w = hg.level_corners(x, lay, 0)
    p = 15 * x.astype(np.float64)[0] + 0.5
    base = np.floor(p.astype(np.float32)).astype(int)
    for c in range(8):
        cx, cy, cz = base + np.array([(c >> d) & 1 for d in range(3)])
        assert idx[0, c] == cx + 16 * cy + 256 * cz
    assert abs(w.sum() - 1.0) < 1e-12


def test_hashed_index_by_hand():
    lay = hg.level_layout(8, 4, 16, 16, 1.5)
    # level 3 is hashed (54^3 > 65536). corner (7, 11, 13):
    pg = np.array([[7, 11, 13]], np.uint32)
    want = ((7 * 1) ^ ((11 * 2654435761) % 2 ** 32) ^ ((13 * 805459861) % 2 ** 32)) % 65536
    assert hg.corner_index(pg, 54, 65536, True)[0] == want
    # wrap-around of the 32-bit product: y = 2^20 -> (2^20 * 2654435761) mod 2^32
    pg = np.array([[0, 1 << 20, 0]], np.uint32)
    want = ((1 << 20) * 2654435761 % 2 ** 32) % 65536
    assert hg.corner_index(pg, 54, 65536, True)[0] == want


def test_encode_interpolates_linear_table():
    # A table whose entries are an affine function of the dense corner coordinates is
    # reproduced exactly by trilinear interpolation (dense level only).
    lay = hg.level_layout(1, 1, 16, 16, 1.5)
    res = 16
    ijk = np.stack(np.meshgrid(np.arange(res), np.arange(res), np.arange(res), indexing='ij'), -1).reshape(-1, 3)
    flat = ijk[:, 0] + res * ijk[:, 1] + res * res * ijk[:, 2]
    table = np.zeros((lay['n_entries'], 1))
    table[flat, 0] = 2.0 * ijk[:, 0] - 3.0 * ijk[:, 1] + 0.5 * ijk[:, 2]
    rng = np.random.default_rng(0)
    x = rng.uniform(0.05, 0.9, size=(64, 3)).astype(np.float32)
    out = hg.encode(x, table, lay)
    p = (15.0 * x.astype(np.float64) + 0.5).astype(np.float32).astype(np.float64)
    np.testing.assert_allclose(out[:, 0], 2 * p[:, 0] - 3 * p[:, 1] + 0.5 * p[:, 2], rtol=1e-6, atol=1e-5)


def test_backward_is_adjoint_of_forward():
    lay = hg.level_layout(4, 2, 10, 8, 1.7)
    rng = np.random.default_rng(1)
    x = rng.uniform(0, 1, size=(50, 3)).astype(np.float32)
    t = rng.normal(size=(lay['n_entries'], 2))
    d = rng.normal(size=(50, 8))
    lhs = np.sum(hg.encode(x, t, lay) * d)
    rhs = np.sum(hg.encode_backward(x, d, lay) * t)
    assert abs(lhs - rhs) < 1e-9 * max(1.0, abs(lhs))
