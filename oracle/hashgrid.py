"""numpy restatement of the multi-resolution hash-grid encoding (oracle).

TEST INFRASTRUCTURE ONLY -- the checker, never the product path.

The reference builds this encoder at projects/neuralangelo/utils/modules.py:42-50
(``tcnn.Encoding(3, dict(otype="HashGrid", ...))``) and calls it at
modules.py:84-86 on points normalised to [0,1] (modules.py:82-83).  The
encoder lives in the third-party tiny-cuda-nn package (requirements.txt:3,
un-vendored, unpinned).  This file restates its published algorithm:

* level l uses scale_l = 2^(l*log2(per_level_scale)) * base_resolution - 1 and
  resolution_l = ceil(scale_l) + 1;
* a level holds min(resolution_l^3 rounded up to a multiple of 8, 2^log2T)
  entries; it is dense (index = x + y*res + z*res^2) while resolution_l^3 fits
  in that size, otherwise spatially hashed (XOR of coord*prime with primes
  1, 2654435761, 805459861, uint32 wrap-around), the index taken modulo the
  level size;
* position in grid units p = scale_l * x + 0.5 (one fused multiply-add),
  corner = floor(p), fraction = p - floor(p), trilinear weights;
* output is level-major: out[:, l*F + f].

Everything that decides an index (scales, floor, hash) is done in float32 /
uint32 exactly as the CUDA kernels do it, so indices are compared bit-exactly.
Interpolation is done in float64 on the float32 fractions.
"""
import numpy as np

PRIMES = (np.uint32(1), np.uint32(2654435761), np.uint32(805459861))


def level_layout(n_levels, n_features, log2_hashmap_size, base_resolution, per_level_scale):
    """Per-level scale / resolution / size / offset, following tcnn's grid setup.

    The per-level scale is evaluated once in double precision from the float32
    per_level_scale and rounded to float32; the CUDA path receives exactly these
    float32 values, so both sides floor the same numbers.
    """
    pls32 = np.float32(per_level_scale)
    log2_pls = np.float32(np.log2(np.float64(pls32)))
    hashmap_size = 1 << int(log2_hashmap_size)
    scales, resolutions, sizes, offsets, hashed = [], [], [], [0], []
    for l in range(n_levels):
        e = np.float32(np.float32(l) * log2_pls)
        s = np.float32(np.float32(np.exp2(np.float64(e))) * np.float32(base_resolution)) - np.float32(1.0)
        s = np.float32(s)
        res = int(np.ceil(np.float64(s))) + 1
        dense = res ** 3
        size = min(((dense + 7) // 8) * 8, hashmap_size)
        scales.append(s)
        resolutions.append(res)
        sizes.append(size)
        hashed.append(bool(res ** 3 > size))
        offsets.append(offsets[-1] + size)
    return dict(scale=np.array(scales, np.float32), resolution=np.array(resolutions, np.int64),
                size=np.array(sizes, np.int64), offset=np.array(offsets, np.int64),
                hashed=np.array(hashed), n_levels=n_levels, n_features=n_features,
                n_entries=offsets[-1])


def _fma32(a, b, c):
    """float32 fused multiply-add fmaf(a, b, c).  The product of two float32
    values is exact in float64 and, for grid positions of order 1e-3..1e4, so is
    its sum with 0.5; one rounding to float32 then equals fmaf."""
    return (np.float64(a) * np.asarray(b, dtype=np.float64) + np.float64(c)).astype(np.float32)


def corner_index(pos_grid, res, size, hashed):
    """pos_grid: uint32 [M,3] corner coordinates -> uint32 [M] entry index in the level."""
    pg = pos_grid.astype(np.uint32)
    if hashed:
        h = (pg[:, 0] * PRIMES[0]) ^ (pg[:, 1] * PRIMES[1]) ^ (pg[:, 2] * PRIMES[2])
        return (h % np.uint32(size)).astype(np.uint32)
    r = np.uint32(res)
    idx = pg[:, 0] + pg[:, 1] * r + pg[:, 2] * (r * r)
    return (idx % np.uint32(size)).astype(np.uint32)


def level_corners(x, layout, l):
    """Corner indices [M,8] (uint32) and trilinear weights [M,8] (float64) at level l.

    Corner c selects coordinate floor(p_d) + ((c >> d) & 1) in dimension d.
    """
    x = np.asarray(x, dtype=np.float32)
    s = layout['scale'][l]
    p = _fma32(s, x, np.float32(0.5))            # [M,3] float32
    fl = np.floor(p).astype(np.float32)
    frac = (p - fl).astype(np.float32)            # exact in float32
    base = fl.astype(np.int64).astype(np.uint32)  # (uint32)(int)floor, wraps for negatives
    res = int(layout['resolution'][l])
    size = int(layout['size'][l])
    hashed = bool(layout['hashed'][l])
    M = x.shape[0]
    idx = np.empty((M, 8), np.uint32)
    w = np.empty((M, 8), np.float64)
    f64 = frac.astype(np.float64)
    for c in range(8):
        bits = np.array([(c >> d) & 1 for d in range(3)], np.uint32)
        pg = base + bits[None, :]
        idx[:, c] = corner_index(pg, res, size, hashed)
        wc = np.ones(M, np.float64)
        for d in range(3):
            wc *= f64[:, d] if bits[d] else (1.0 - f64[:, d])
        w[:, c] = wc
    return idx, w


def encode(x, table, layout, active_levels=None):
    """Forward: x [M,3] in grid-normalised coordinates, table [n_entries, F] -> [M, L*F] float64.

    Levels >= active_levels are zero (coarse-to-fine mask, modules.py:91-93,109-113).
    """
    L, F = layout['n_levels'], layout['n_features']
    active = L if active_levels is None else active_levels
    table = np.asarray(table, dtype=np.float64).reshape(-1, F)
    M = np.asarray(x).shape[0]
    out = np.zeros((M, L * F), np.float64)
    for l in range(min(active, L)):
        idx, w = level_corners(x, layout, l)
        rows = table[layout['offset'][l] + idx.astype(np.int64)]   # [M,8,F]
        out[:, l * F:(l + 1) * F] = np.einsum('mc,mcf->mf', w, rows)
    return out


def encode_backward(x, d_out, layout, active_levels=None):
    """Backward: d_out [M, L*F] -> d_table [n_entries, F] (float64 scatter-add)."""
    L, F = layout['n_levels'], layout['n_features']
    active = L if active_levels is None else active_levels
    d_out = np.asarray(d_out, dtype=np.float64)
    grad = np.zeros((layout['n_entries'], F), np.float64)
    for l in range(min(active, L)):
        idx, w = level_corners(x, layout, l)
        g = w[:, :, None] * d_out[:, None, l * F:(l + 1) * F]     # [M,8,F]
        np.add.at(grad, layout['offset'][l] + idx.astype(np.int64).reshape(-1), g.reshape(-1, F))
    return grad


def all_indices(x, layout, active_levels=None):
    """Absolute entry indices [M, L_active, 8] (int64) for index parity tests."""
    L = layout['n_levels']
    active = L if active_levels is None else active_levels
    out = []
    for l in range(min(active, L)):
        idx, _ = level_corners(x, layout, l)
        out.append(layout['offset'][l] + idx.astype(np.int64))
    return np.stack(out, axis=1)
