"""float64 restatement of the hierarchical importance sampler.

TEST INFRASTRUCTURE ONLY -- the checker, never the product path.

Follows the reference's no-grad sampling pre-pass of the object field:
  Model.sample_dists_all           projects/neuralangelo/model.py:232-248
  Model.sample_dists_hierarchical  projects/neuralangelo/model.py:250-267
  nerf_util.sample_dists           projects/nerf/utils/nerf_util.py:20-38
  nerf_util.sample_dists_from_pdf  projects/nerf/utils/nerf_util.py:41-68
  render.alpha_compositing_weights projects/nerf/utils/render.py:87-99
Rays are [R] (the reference's batch dimension B = 1 folded away); distances are
[R, N]; ``sdf_fn`` maps points [M, 3] to SDF values [M].  The stratified
uniforms are an input (the reference draws them with torch.rand inside
sample_dists), so CPU and GPU runs can share them.
"""
import torch


def stratified_dists(near, far, n, u=None):
    """nerf_util.sample_dists (:20-38): (u + i) / n * (far - near) + near, u = 0.5 when
    not stratified.  near, far [R, 1]; u [R, n] or None -> [R, n]."""
    R = near.shape[0]
    if u is None:
        u = torch.full((R, n), 0.5, dtype=near.dtype)
    rands = u + torch.arange(n, dtype=near.dtype)[None]
    return rands / n * (far - near) + near


def points_at(center, ray_unit, dists):
    """camera.get_3D_points_from_dist (camera.py:314-320): center + ray_unit * dists."""
    return center[:, None, :] + ray_unit[:, None, :] * dists[..., None]


def compositing_weights(alphas):
    """render.alpha_compositing_weights (render.py:87-99)."""
    front = torch.cat([torch.zeros_like(alphas[:, :1]), alphas[:, :-1]], dim=1)
    return alphas * torch.cumprod(1 - front, dim=1)


def pdf_dists(bins, weights, n_fine):
    """nerf_util.sample_dists_from_pdf (:41-68).  bins [R, N], weights [R, N-1] -> [R, n_fine]."""
    pdf = weights / weights.abs().sum(dim=-1, keepdim=True).clamp(min=1e-12)     # F.normalize(p=1)
    cdf = torch.cat([torch.zeros_like(pdf[:, :1]), pdf.cumsum(dim=-1)], dim=-1)    # [R, N]
    grid = torch.linspace(0, 1, n_fine + 1, dtype=bins.dtype)
    unif = (0.5 * (grid[:-1] + grid[1:])).repeat(bins.shape[0], 1)                # [R, n_fine]
    idx = torch.searchsorted(cdf.contiguous(), unif.contiguous(), right=True)
    low = (idx - 1).clamp(min=0)
    high = idx.clamp(max=cdf.shape[-1] - 1)
    d0, d1 = bins.gather(1, low), bins.gather(1, high)
    c0, c1 = cdf.gather(1, low), cdf.gather(1, high)
    t = (unif - c0) / (c1 - c0 + 1e-8)
    return d0 + t * (d1 - d0)


def hierarchical_dists(dists, sdfs, inv_s, n_fine, robust=True, eps=1e-5):
    """Model.sample_dists_hierarchical (model.py:250-267).  dists, sdfs [R, N] -> [R, n_fine]."""
    prev_s, next_s = sdfs[:, :-1], sdfs[:, 1:]
    prev_d, next_d = dists[:, :-1], dists[:, 1:]
    mid = (prev_s + next_s) * 0.5
    cos_val = (next_s - prev_s) / (next_d - prev_d + 1e-5)
    if robust:
        prev_cos = torch.cat([torch.zeros_like(cos_val[:, :1]), cos_val[:, :-1]], dim=-1)
        cos_val = torch.minimum(prev_cos, cos_val)
    intv = next_d - prev_d
    est_prev = mid - cos_val * intv * 0.5
    est_next = mid + cos_val * intv * 0.5
    prev_cdf = torch.sigmoid(est_prev * inv_s)
    next_cdf = torch.sigmoid(est_next * inv_s)
    alphas = ((prev_cdf - next_cdf) / (prev_cdf + eps)).clamp(0.0, 1.0)
    weights = compositing_weights(alphas)
    return pdf_dists(dists, weights, n_fine)


def merge(dists, sdfs, fine_d, fine_s=None):
    """Concatenate and sort along the ray (model.py:240-247); sdfs follow their distances."""
    d = torch.cat([dists, fine_d], dim=1)
    d_sorted, idx = d.sort(dim=1, stable=True)
    if fine_s is None:
        return d_sorted, None
    s = torch.cat([sdfs, fine_s], dim=1).gather(1, idx)
    return d_sorted, s


def sample_dists_all(center, ray_unit, near, far, sdf_fn, n_coarse=64, n_fine=16, n_hierarchy=4, u=None,
                     trace=None):
    """Model.sample_dists_all (model.py:232-248) -> dists [R, n_coarse + n_hierarchy * n_fine].

    ``trace`` (a list) collects (dists, sdfs, fine) per round for diagnostics."""
    dists = stratified_dists(near, far, n_coarse, u)
    sdfs = None
    if n_hierarchy > 0:
        sdfs = sdf_fn(points_at(center, ray_unit, dists).reshape(-1, 3)).reshape(dists.shape)
    for h in range(n_hierarchy):
        fine = hierarchical_dists(dists, sdfs, 64 * 2 ** h, n_fine)
        if trace is not None:
            trace.append((dists, sdfs, fine))
        if h != n_hierarchy - 1:
            fs = sdf_fn(points_at(center, ray_unit, fine).reshape(-1, 3)).reshape(fine.shape)
            dists, sdfs = merge(dists, sdfs, fine, fs)
        else:
            dists, _ = merge(dists, None, fine)
    return dists
