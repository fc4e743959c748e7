"""Generate the golden fixtures for the field / rendering / loss path.

Runs the REFERENCE's own modules -- NeuralSDF and NeuralRGB
(projects/neuralangelo/utils/modules.py), MLPforNeuralSDF (utils/mlp.py),
Model.compute_neus_alphas / _get_iter_cos (projects/neuralangelo/model.py:275-298),
render.alpha_compositing_weights / composite (projects/nerf/utils/render.py:87-112),
misc.eikonal_loss / curvature_loss (projects/neuralangelo/utils/misc.py:74-89) --
in float64 on the CPU, with the oracle's numpy hash-grid encoder injected as
``tinycudann.Encoding`` (tiny-cuda-nn is not installed here).  The render loss
restates trainer.py:43 (L1 * 3) because trainer.py imports wandb.

Usage (needs the reference checkout; writes tests/golden/*.npz):
    python tests/golden/make_golden.py /root/reference
"""
import os
import sys
import types
import warnings

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.dont_write_bytecode = True
warnings.filterwarnings("ignore")

from oracle import field as of          # noqa: E402
from oracle import hashgrid as hg       # noqa: E402


class AttrDict(dict):
    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e


def to_attr(d):
    if isinstance(d, dict):
        return AttrDict({k: to_attr(v) for k, v in d.items()})
    return d


class StubEncoding(torch.nn.Module):
    """tinycudann.Encoding stand-in: the oracle's hash-grid, float64, flat ``params``."""

    def __init__(self, n_input_dims, encoding_config):
        super().__init__()
        c = encoding_config
        self.layout = hg.level_layout(c['n_levels'], c['n_features_per_level'], c['log2_hashmap_size'],
                                      c['base_resolution'], c['per_level_scale'])
        self.params = torch.nn.Parameter(torch.zeros(self.layout['n_entries'] * c['n_features_per_level'],
                                                     dtype=torch.float64))

    def forward(self, x):
        return of.hashgrid(x, self.params, self.layout, None)


def install_stub():
    mod = types.ModuleType("tinycudann")
    mod.Encoding = StubEncoding
    sys.modules["tinycudann"] = mod


def ref_configs(L, Fd, min_logres, max_logres, dict_size, hidden, rgb_hidden, rgb_layers, taps, active):
    cfg_sdf = to_attr(dict(
        mlp=dict(num_layers=1, hidden_dim=hidden, skip=[], activ="softplus", activ_params=dict(beta=100),
                 geometric_init=True, weight_norm=True, out_bias=0.5, inside_out=False),
        encoding=dict(type="hashgrid", levels=L,
                      hashgrid=dict(min_logres=min_logres, max_logres=max_logres, dict_size=dict_size, dim=Fd,
                                    range=[-2, 2]),
                      coarse2fine=dict(enabled=True, init_active_level=active, step=5000)),
        gradient=dict(mode="numerical", taps=taps)))
    cfg_rgb = to_attr(dict(
        mlp=dict(num_layers=rgb_layers, hidden_dim=rgb_hidden, skip=[], activ="relu_", activ_params={},
                 weight_norm=True),
        mode="idr", encoding_view=dict(type="spherical", levels=3)))
    return cfg_sdf, cfg_rgb


def make_rays(R, N, seed, n_miss=1):
    """Cameras on a radius-3 sphere aimed at the origin (seeded jitter); the first
    n_miss rays are aimed away so they miss the unit sphere."""
    g = torch.Generator().manual_seed(seed)
    c = torch.randn(R, 3, generator=g, dtype=torch.float64)
    c = 3.0 * c / c.norm(dim=-1, keepdim=True)
    d = -c + 0.3 * torch.randn(R, 3, generator=g, dtype=torch.float64)
    d[:n_miss] = c[:n_miss]
    d = d / d.norm(dim=-1, keepdim=True)
    near, far, outside = of.dist_bounds(c, d)
    u = torch.rand(R, N, generator=g, dtype=torch.float64)
    dists = (torch.arange(N, dtype=torch.float64)[None] + u) / N * (far - near) + near   # nerf_util.py:20-38
    target = torch.rand(R, 3, generator=g, dtype=torch.float64)
    return dict(center=c, ray_unit=d, dists=dists, far=far, outside=outside, target=target)


def run_case(ref, name, L, Fd, min_logres, max_logres, dict_size, hidden, rgb_hidden, rgb_layers, taps,
             active, anneal, app_dim, n_images, R, N, w_eik, w_curv, progress, seed):
    modules, render, misc, Model = ref
    cfg_sdf, cfg_rgb = ref_configs(L, Fd, min_logres, max_logres, dict_size, hidden, rgb_hidden, rgb_layers,
                                   taps, active)
    torch.manual_seed(seed)
    sdf_mod = modules.NeuralSDF(cfg_sdf).double()
    app_cfg = to_attr(dict(enabled=app_dim > 0, dim=app_dim))
    rgb_mod = modules.NeuralRGB(cfg_rgb, feat_dim=hidden, appear_embed=app_cfg).double()
    # Coarse-to-fine state (modules.py:97-107) at an iteration giving `anneal` levels.
    sdf_mod.warm_up_end = 5000
    it = 5000 + anneal * 5000
    sdf_mod.set_active_levels(it)
    sdf_mod.set_normal_epsilon()
    assert sdf_mod.anneal_levels == anneal
    ocfg = of.make_config(n_levels=L, n_features=Fd, log2_hashmap_size=dict_size, base_resolution=2 ** min_logres,
                          max_resolution=2 ** max_logres, active_levels=sdf_mod.active_levels, sdf_hidden=hidden,
                          rgb_hidden=rgb_hidden, rgb_layers=rgb_layers, app_dim=app_dim, n_images=n_images,
                          taps=taps)
    params, layout = of.init_params(ocfg, seed=seed, table_scale=1e-1)
    # copy the oracle-initialised parameters into the reference modules
    with torch.no_grad():
        sdf_mod.tcnn_encoding.params.copy_(params['table'])
        for i in range(2):
            lin = sdf_mod.mlp.linears[i]
            lin.weight_v.copy_(params[f'sdf.l{i}.v'])
            lin.weight_g.copy_(params[f'sdf.l{i}.g'])
            lin.bias.copy_(params[f'sdf.l{i}.b'])
        sdf_mod.mlp.linear_sdf.weight.copy_(params['sdf.head.w'])
        sdf_mod.mlp.linear_sdf.bias.copy_(params['sdf.head.b'])
        for i, lin in enumerate(rgb_mod.mlp.linears):
            lin.weight_v.copy_(params[f'rgb.l{i}.v'])
            lin.weight_g.copy_(params[f'rgb.l{i}.g'])
            lin.bias.copy_(params[f'rgb.l{i}.b'])
    s_var = torch.nn.Parameter(params['s_var'].clone())
    app_table = torch.nn.Parameter(params['app'].clone()) if app_dim else None
    batch = make_rays(R, N, seed)
    app_idx = torch.randint(0, max(n_images, 1), (R,), generator=torch.Generator().manual_seed(seed + 1))

    # --- the reference's own forward (model.py:158-190, 124-156; trainer.py:40-52) ---
    fake = types.SimpleNamespace(s_var=s_var, anneal_end=0.1)
    fake._get_iter_cos = lambda true_cos, progress=1.: Model._get_iter_cos(fake, true_cos, progress)
    center = batch['center'][None]                     # [B=1,R,3]
    ray_unit = batch['ray_unit'][None]
    dists = batch['dists'][None, ..., None]            # [1,R,N,1]
    far = batch['far'][None]                           # [1,R,1]
    outside = batch['outside'][None]                   # [1,R,1]
    points = center[..., None, :] + ray_unit[..., None, :] * dists
    sdfs, feats = sdf_mod.forward(points)
    sdfs[outside[..., None].expand_as(sdfs)] = 1000.
    rays_unit = ray_unit[..., None, :].expand_as(points).contiguous()
    gradients, hessians = sdf_mod.compute_gradients(points, training=True, sdf=sdfs)
    normals = torch.nn.functional.normalize(gradients, dim=-1)
    app = None
    if app_dim:
        app = app_table[app_idx][None, :, None, :].expand(1, R, N, app_dim)
    rgbs = rgb_mod.forward(points, normals, rays_unit, feats, app=app)
    alphas = Model.compute_neus_alphas(fake, ray_unit, sdfs, gradients, dists, dist_far=far[..., None],
                                       progress=progress)
    weights = render.alpha_compositing_weights(alphas)
    rgb = render.composite(rgbs, weights)
    l_render = torch.nn.L1Loss()(rgb, batch['target'][None]) * 3
    l_eik = misc.eikonal_loss(gradients, outside=outside)
    loss = l_render + w_eik * l_eik
    l_curv = torch.zeros((), dtype=torch.float64)
    if w_curv:
        l_curv = misc.curvature_loss(hessians, outside=outside)
        loss = loss + w_curv * l_curv
    loss.backward()

    out = dict(
        # inputs
        center=batch['center'], ray_unit=batch['ray_unit'], dists=batch['dists'], far=batch['far'],
        outside=batch['outside'], target=batch['target'], app_idx=app_idx.numpy(),
        cfg=np.array([L, Fd, dict_size, 2 ** min_logres, 2 ** max_logres, hidden, rgb_hidden, rgb_layers, taps,
                      sdf_mod.active_levels, anneal, app_dim, n_images]),
        scalars=np.array([sdf_mod.normal_eps, progress, w_eik, w_curv, sdf_mod.growth_rate]),
        # outputs of the reference modules
        sdf=sdfs[0, ..., 0].detach(), feat=feats[0].detach(), grads=gradients[0].detach(),
        hess=hessians[0].detach(), rgbs=rgbs[0].detach(), alphas=alphas[0].detach(),
        weights=weights[0, ..., 0].detach(), rgb=rgb[0].detach(),
        losses=torch.stack([loss, l_render, l_eik, l_curv]).detach(),
        # gradients from the reference's autograd
        g_table=sdf_mod.tcnn_encoding.params.grad, g_s_var=s_var.grad,
        g_head_w=sdf_mod.mlp.linear_sdf.weight.grad, g_head_b=sdf_mod.mlp.linear_sdf.bias.grad,
    )
    for k, v in params.items():
        out['p_' + k] = v
    for i in range(2):
        lin = sdf_mod.mlp.linears[i]
        out[f'g_sdf.l{i}.v'], out[f'g_sdf.l{i}.g'], out[f'g_sdf.l{i}.b'] = lin.weight_v.grad, lin.weight_g.grad, \
            lin.bias.grad
    for i, lin in enumerate(rgb_mod.mlp.linears):
        out[f'g_rgb.l{i}.v'], out[f'g_rgb.l{i}.g'], out[f'g_rgb.l{i}.b'] = lin.weight_v.grad, lin.weight_g.grad, \
            lin.bias.grad
    if app_dim:
        out['g_app'] = app_table.grad
    out = {k: (v.detach().numpy() if torch.is_tensor(v) else np.asarray(v)) for k, v in out.items()}
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items() if k.startswith('g_')})


def main(ref_root):
    sys.path.insert(0, ref_root)
    install_stub()
    from projects.neuralangelo.utils import modules, misc
    from projects.nerf.utils import render
    from projects.neuralangelo.model import Model
    ref = (modules, render, misc, Model)
    # C1-shaped (16 levels hashed above a small table, app embedding, 6 taps, curvature)
    run_case(ref, "field_c1_small", L=8, Fd=4, min_logres=4, max_logres=7, dict_size=10, hidden=32,
             rgb_hidden=32, rgb_layers=4, taps=6, active=4, anneal=6, app_dim=4, n_images=3,
             R=6, N=16, w_eik=0.1, w_curv=5e-4 / 1.3459 ** 5, progress=0.09, seed=1)
    # C0-shaped (all levels active, no appearance embedding, no curvature)
    run_case(ref, "field_c0_small", L=6, Fd=2, min_logres=3, max_logres=6, dict_size=10, hidden=32,
             rgb_hidden=16, rgb_layers=2, taps=6, active=6, anneal=6, app_dim=0, n_images=0,
             R=5, N=12, w_eik=0.1, w_curv=0.0, progress=1.0, seed=2)
    # 4-tap variant (modules.py:157-175)
    run_case(ref, "field_taps4_small", L=6, Fd=2, min_logres=3, max_logres=6, dict_size=10, hidden=16,
             rgb_hidden=16, rgb_layers=2, taps=4, active=4, anneal=3, app_dim=0, n_images=0,
             R=4, N=8, w_eik=0.1, w_curv=5e-4, progress=0.05, seed=3)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the neuralangelo reference checkout>")
    main(sys.argv[1])
