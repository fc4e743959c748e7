"""numpy restatement of the mesh output stage: per-block vertex merge, the
centre/scale transform and degenerate-face removal.

TEST INFRASTRUCTURE ONLY (the checker for gbsdf_mesh_finalize).

The reference hands these steps to trimesh, a third-party package that is not
vendored (requirements.txt, unpinned) and is absent here, so this file restates
its documented behaviour and parity with trimesh itself is unpinned:

* projects/neuralangelo/utils/mesh.py:121-129: every block becomes a
  ``trimesh.Trimesh(V, F)``, whose default processing merges vertices whose
  coordinates round (half to even) to the same integers at 8 decimal digits,
  keeping the first occurrence of each group and re-indexing the faces to it.
  The blocks are then concatenated without a merge (:43-46).
* projects/neuralangelo/scripts/extract_mesh.py:96-97: ``vertices * radius +
  center``, then ``update_faces(nondegenerate_faces())``: with a = v1 - v0,
  b = v2 - v0 and 2A = |a x b|, a face stays when both triangle heights 2A / |a|
  and 2A / |b| (taken as 0 when that edge is not longer than the tolerance)
  exceed the tolerance (trimesh's merge tolerance, 1e-8).  Every vertex is kept,
  referenced or not.
* projects/neuralangelo/utils/mesh.py:151-158 (``filter_largest_cc``, per block after
  the sphere filter, :130): ``mesh.split(only_watertight=False)`` then the component
  of largest area.  trimesh joins two faces when they share an edge that exactly two
  faces share (its face adjacency: sorted edge rows grouped, groups of two kept),
  keeps components of any size, and lists them by label (scipy numbers components in
  order of their lowest face); ``argmax`` takes the first of equal areas.  A
  component becomes a submesh: its vertices in index order, re-indexed from 0.
"""
import numpy as np

MERGE_DIGITS = 8
MERGE_TOL = 1e-8


def merge_vertices(V, F, digits=MERGE_DIGITS):
    """(V', F'): vertices equal after rounding to ``digits`` decimals merged into their
    first occurrence (order of first occurrence kept), faces re-indexed."""
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    keys = np.rint(V * float(10 ** digits)).astype(np.int64)
    first = {}
    rep = np.empty(len(V), np.int64)
    for i, k in enumerate(map(tuple, keys)):
        rep[i] = first.setdefault(k, i)
    is_rep = rep == np.arange(len(V))
    new_idx = np.cumsum(is_rep) - is_rep
    vmap = new_idx[rep]
    return V[is_rep], vmap[F] if len(F) else F.reshape(0, 3)


def transform(V, scale=1.0, offset=(0.0, 0.0, 0.0)):
    """V * scale + offset, two roundings (extract_mesh.py:96)."""
    return np.asarray(V, np.float64) * float(scale) + np.asarray(offset, np.float64)


def nondegenerate(V, F, height=MERGE_TOL):
    """Mask of faces whose two heights over the edges v1 - v0 and v2 - v0 both exceed
    ``height``; faces repeating a vertex index are degenerate too.  height 0 drops
    only those, a negative height keeps every face."""
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int64)
    if len(F) == 0:
        return np.zeros(0, bool)
    if height < 0:                       # trimesh's per-block merge keeps every face
        return np.ones(len(F), bool)
    distinct = (F[:, 0] != F[:, 1]) & (F[:, 1] != F[:, 2]) & (F[:, 0] != F[:, 2])
    if height == 0:
        return distinct
    t = V[F]
    a = t[:, 1] - t[:, 0]
    b = t[:, 2] - t[:, 0]
    cr = np.empty_like(a)
    cr[:, 0] = a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1]
    cr[:, 1] = a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2]
    cr[:, 2] = a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]

    def norm(x):
        return np.sqrt((x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) + x[:, 2] * x[:, 2])

    two_area = (norm(cr) * 0.5) * 2.0
    la, lb = norm(a), norm(b)
    with np.errstate(divide="ignore", invalid="ignore"):
        ha = np.where(la > height, two_area / np.where(la > 0, la, 1.0), 0.0)
        hb = np.where(lb > height, two_area / np.where(lb > 0, lb, 1.0), 0.0)
    return distinct & (ha > height) & (hb > height)


def finalize(V, F, weld=False, digits=MERGE_DIGITS, scale=1.0, offset=(0.0, 0.0, 0.0), height=MERGE_TOL):
    """The output stage in the order gbsdf_mesh_finalize runs it: weld (input
    coordinates) -> transform -> drop degenerate faces (output coordinates)."""
    V = np.asarray(V, np.float64).reshape(-1, 3)
    F = np.asarray(F, np.int64).reshape(-1, 3)
    if weld:
        V, F = merge_vertices(V, F, digits)
    V = transform(V, scale, offset)
    keep = nondegenerate(V, F, height)
    return V, F[keep]


def largest_component(V, F):
    """(V', F') of the largest-area component of (V, F), by a pure-Python union-find over
    faces joined through edges that exactly two faces share; faces in ascending order."""
    V = np.asarray(V, np.float64)
    F = [tuple(int(i) for i in f) for f in np.asarray(F, np.int64).reshape(-1, 3)]
    if not F or len(V) == 0:
        return V[:0], np.zeros((0, 3), np.int64)
    owners = {}
    for fi, (a, b, c) in enumerate(F):
        for u, v in ((a, b), (b, c), (c, a)):
            owners.setdefault((min(u, v), max(u, v)), []).append(fi)
    parent = list(range(len(F)))

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for fl in owners.values():
        if len(fl) == 2:
            ra, rb = find(fl[0]), find(fl[1])
            if ra != rb:
                parent[max(ra, rb)] = min(ra, rb)        # the root is the component's lowest face
    area = {}
    for fi, (a, b, c) in enumerate(F):
        e1, e2 = V[b] - V[a], V[c] - V[a]
        cx = e1[1] * e2[2] - e1[2] * e2[1]
        cy = e1[2] * e2[0] - e1[0] * e2[2]
        cz = e1[0] * e2[1] - e1[1] * e2[0]
        r = find(fi)
        area[r] = area.get(r, 0.0) + 0.5 * float(np.sqrt(cx * cx + cy * cy + cz * cz))
    best = max(sorted(area), key=lambda r: area[r])    # sorted roots = lowest-face order; first max
    keep = [f for fi, f in enumerate(F) if find(fi) == best]
    used = sorted({i for f in keep for i in f})
    remap = {v: k for k, v in enumerate(used)}
    return V[used], np.array([[remap[i] for i in f] for f in keep], np.int64).reshape(-1, 3)
