"""Seeded synthetic inputs with the benchmark shapes (no datasets are used).

Rays come from cameras on a radius-3 sphere aimed at the origin with seeded
jitter (all rays hit the unit sphere unless ``miss_frac`` > 0); sample
distances are stratified in the unit-sphere interval [near, far]
(projects/nerf/utils/nerf_util.py:20-38 with stratified=True); target colours
are U[0,1].  Bounds follow Model.get_dist_bounds (projects/neuralangelo/model.py:207-213).
"""
import math

import torch


def sphere_bounds(center, ray_unit):
    """intersect_with_sphere (nerf_util.py:199-205) + get_dist_bounds (model.py:207-213)."""
    ctc = (center * center).sum(-1, keepdim=True)
    ctv = (center * ray_unit).sum(-1, keepdim=True)
    disc = ctv ** 2 - (ctc - 1.0)
    near = (-ctv - disc.sqrt()).clamp(min=0)
    far = -ctv + disc.sqrt()
    outside = near.isnan()
    near = torch.where(outside, torch.ones_like(near), near)
    far = torch.where(outside, torch.full_like(far, 1.2), far)
    return near, far, outside


def make_rays(R, N, seed=0, miss_frac=0.0, n_images=0, device="cpu", n_bg=0, miss_perpendicular=False):
    """Dense batch.  The first miss_frac of the rays miss the unit sphere: aimed straight
    away from it (the reference's bounds then give far < 0, its quirk), or, with
    miss_perpendicular, across it (outside: near 1, far 1.2, as a background needs)."""
    g = torch.Generator().manual_seed(seed)
    c = torch.randn(R, 3, generator=g)
    c = 3.0 * c / c.norm(dim=-1, keepdim=True)
    d = -c + 0.3 * torch.randn(R, 3, generator=g)
    n_miss = int(round(miss_frac * R))
    if n_miss:
        if miss_perpendicular:
            side = torch.linalg.cross(c[:n_miss], torch.tensor([[0.3, -0.5, 0.8]]).expand(n_miss, 3), dim=-1)
            d[:n_miss] = side
        else:
            d[:n_miss] = c[:n_miss]
    d = d / d.norm(dim=-1, keepdim=True)
    near, far, outside = sphere_bounds(c, d)
    u = torch.rand(R, N, generator=g)
    dists = (torch.arange(N, dtype=torch.float32)[None] + u) / N * (far - near) + near
    target = torch.rand(R, 3, generator=g)
    app_idx = torch.randint(0, max(n_images, 1), (R,), generator=g)
    b = dict(center=c, ray_unit=d, dists=dists, far=far, outside=outside, target=target, app_idx=app_idx)
    if n_bg:
        b["dists_bg"] = background_dists(far, n_bg, torch.rand(R, n_bg, generator=g))
    return {k: v.to(device) for k, v in b.items()}


def background_dists(far, n, u=None):
    """Model.sample_dists_background (model.py:269-273): inverse distances stratified
    from 1 down to 0 (nerf_util.py:20-38 with dist_range (1, 0)), dists = far / (inv +
    1e-5); u [R, n] in [0, 1), or 0.5 when not stratified.  far [R, 1] -> [R, n]."""
    R = far.shape[0]
    if u is None:
        u = torch.full((R, n), 0.5, device=far.device)
    inv = (u + torch.arange(n, dtype=torch.float32, device=far.device)[None]) / n * (0.0 - 1.0) + 1.0
    return far / (inv + 1e-5)


def make_ragged_rays(R, seed=0, zero_frac=0.3, lo=16, hi=256, n_images=0, device="cpu", n_bg=0):
    """Ragged batch after sphere culling and importance sampling: a ``zero_frac`` share of
    the rays miss the unit sphere and keep no samples; every other ray gets a count
    uniform in [lo, hi] of stratified samples in its [near, far].  Ray r owns the flat
    samples [ray_offsets[r], ray_offsets[r+1]); ``sample_ray`` maps a sample to its ray."""
    g = torch.Generator().manual_seed(seed)
    c = torch.randn(R, 3, generator=g)
    c = 3.0 * c / c.norm(dim=-1, keepdim=True)
    d = -c + 0.3 * torch.randn(R, 3, generator=g)
    miss = torch.rand(R, generator=g) < zero_frac
    side = torch.linalg.cross(c, torch.randn(R, 3, generator=g), dim=-1)   # perpendicular: misses the sphere
    d = torch.where(miss[:, None], side, d)
    d = d / d.norm(dim=-1, keepdim=True)
    near, far, outside = sphere_bounds(c, d)
    counts = torch.randint(lo, hi + 1, (R,), generator=g)
    counts = torch.where(outside[:, 0], torch.zeros_like(counts), counts)
    offs = torch.zeros(R + 1, dtype=torch.int64)
    offs[1:] = torch.cumsum(counts, 0)
    Ns = int(offs[-1])
    sample_ray = torch.repeat_interleave(torch.arange(R), counts)
    k = torch.arange(Ns) - offs[:-1][sample_ray]                 # index within the ray
    u = torch.rand(Ns, generator=g)
    n = counts[sample_ray].float()
    dists = (k.float() + u) / n * (far[sample_ray, 0] - near[sample_ray, 0]) + near[sample_ray, 0]
    target = torch.rand(R, 3, generator=g)
    app_idx = torch.randint(0, max(n_images, 1), (R,), generator=g)
    b = dict(center=c, ray_unit=d, dists=dists, far=far, outside=outside, target=target, app_idx=app_idx,
             ray_offsets=offs, sample_ray=sample_ray.to(torch.int32), near=near)
    if n_bg:
        b["dists_bg"] = background_dists(far, n_bg, torch.rand(R, n_bg, generator=g))
    return {k_: v.to(device) for k_, v in b.items()}


def padded(batch, S=128, seed=0):
    """The rays of a ragged batch in the reference's dense [R, S] layout: every ray,
    misses included, gets S stratified samples in [near, far] (model.py:232-236, 163)."""
    near, far = batch['near'], batch['far']
    R = near.shape[0]
    g = torch.Generator().manual_seed(seed)
    u = torch.rand(R, S, generator=g).to(near.device)
    dists = (torch.arange(S, dtype=torch.float32, device=near.device)[None] + u) / S * (far - near) + near
    keep = ('center', 'ray_unit', 'far', 'outside', 'target', 'app_idx')
    out = {k: batch[k] for k in keep}
    out['dists'] = dists
    return out


def init_field_params(model, seed=0, enc_perturb=1e-2):
    """Reference initialisation (geometric init already applied by the modules) plus a
    seeded N(0, enc_perturb) on SDF layer 0's encoding columns: geometric init zeroes
    them (mlp.py:74-75), which would make every table gradient exactly zero."""
    g = torch.Generator().manual_seed(seed)
    with torch.no_grad():
        lin0 = model.neural_sdf.mlp.linears[0]
        v = lin0.weight_v
        pert = torch.randn(v.shape[0], v.shape[1] - 3, generator=g) * enc_perturb
        v[:, 3:] = pert.to(v)
        lin0.weight_g.copy_(v.norm(dim=1, keepdim=True))
        if model.appear_embed is not None:
            model.appear_embed.weight.copy_(torch.randn(model.appear_embed.weight.shape, generator=g))
    return model


def full_field_iteration(active_levels=8, warm_up_end=5000, step=5000):
    """The training iteration at which ``active_levels`` levels are annealed in (modules.py:97-100)."""
    return warm_up_end + active_levels * step


def flops_per_sample(cfg, active_levels):
    """Algorithmic FLOPs of one sample's forward+backward (3x forward MACs x 2), counting
    only active encoding columns: centre layer0 + feature layer + 6 taps x layer0 + colour MLP."""
    H = cfg.sdf.mlp.hidden_dim
    k0 = 3 + active_levels * cfg.sdf.encoding.hashgrid.dim
    centre = k0 * H + H + H * H
    taps = 6 * (k0 * H + H)
    dims = [6 + 16 + H + (cfg.appear_embed.dim if cfg.appear_embed.enabled else 0)]
    dims += [cfg.rgb.mlp.hidden_dim] * cfg.rgb.mlp.num_layers + [3]
    rgb = sum(a * b for a, b in zip(dims[:-1], dims[1:]))
    return 2 * 3 * (centre + taps + rgb)


def encoder_bytes_per_sample(active_levels, F, table_bytes, evals=7):
    """Algorithmic encoder bytes of one sample's forward+backward: every evaluation
    reads 8 corners x F features per active level and read-modify-writes the same
    FP32 gradient entries (4 B read + 4 B write)."""
    return evals * active_levels * 8 * F * (table_bytes + 8)


def pct(x):
    return round(100.0 * x, 2)


def median(v):
    v = sorted(v)
    n = len(v)
    return v[n // 2] if n % 2 else 0.5 * (v[n // 2 - 1] + v[n // 2])


_ = math


def shapes_union(seed=0, n_spheres=3, n_boxes=2):
    """Seeded union of spheres and axis-aligned boxes (radii / half-sizes 0.1-0.4) inside
    [-1, 1]^3 as an analytic signed distance (negative inside).  Returns a callable
    on [..., 3] tensors."""
    g = torch.Generator().manual_seed(seed)
    sph = [((torch.rand(3, generator=g) * 2 - 1) * 0.5, 0.1 + 0.3 * float(torch.rand(1, generator=g)))
           for _ in range(n_spheres)]
    box = [((torch.rand(3, generator=g) * 2 - 1) * 0.5, 0.1 + 0.3 * torch.rand(3, generator=g))
           for _ in range(n_boxes)]

    def sdf(x):
        d = None
        for c, r in sph:
            v = (x - c.to(x)).norm(dim=-1) - r
            d = v if d is None else torch.minimum(d, v)
        for c, h in box:
            q = (x - c.to(x)).abs() - h.to(x)
            v = q.clamp(min=0).norm(dim=-1) + q.max(dim=-1).values.clamp(max=0)
            d = torch.minimum(d, v)
        return d
    return sdf


def fit_sdf(neural_sdf, target, steps=300, batch=65536, lr=1e-3, seed=0):
    """Fit a NeuralSDF (plain FP32 path) to an analytic SDF with Adam on L1, points
    uniform in [-1, 1]^3 plus a jittered copy of them."""
    dev = neural_sdf.tcnn_encoding.params.device
    g = torch.Generator(device=dev).manual_seed(seed)
    opt = torch.optim.Adam(neural_sdf.parameters(), lr=lr)
    loss = torch.zeros(())
    for _ in range(steps):
        x = torch.rand(batch, 3, device=dev, generator=g) * 2 - 1
        pts = torch.cat([x, x + 0.02 * torch.randn(batch, 3, device=dev, generator=g)])
        with torch.no_grad():
            tgt = target(pts)
        loss = (neural_sdf.sdf(pts)[:, 0] - tgt).abs().mean()
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
    return float(loss)
