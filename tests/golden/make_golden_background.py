"""Generate the golden fixture for the background NeRF and its compositing.

Runs the REFERENCE's own BackgroundNeRF (projects/neuralangelo/utils/modules.py:232-311,
through MLPwithSkipConnection and positional_encoding of projects/nerf/utils/nerf_util.py),
nerf_util.sample_dists with the background's inverse-distance range
(Model.sample_dists_background, projects/neuralangelo/model.py:269-273, restated
because it is a method of the full Model), render.volume_rendering_alphas_dist,
alpha_compositing_weights and composite (projects/nerf/utils/render.py:68-112) in
float64 on the CPU, with object samples (seeded alphas and colours) composited in
front of the background samples as Model.render_rays does (model.py:129-141).  The
loss is the L1 colour term x 3 (trainer.py:43).  Widths are reduced (hidden 32,
colour hidden 16) to keep the fixture small; the structure is the reference's.

Usage (needs the reference checkout; writes tests/golden/background.npz):
    python tests/golden/make_golden_background.py /root/reference
"""
import os
import sys
import warnings

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.dont_write_bytecode = True
warnings.filterwarnings("ignore")

from oracle import field as of          # noqa: E402
from tests.golden.make_golden import install_stub, to_attr   # noqa: E402

R, NO, NB, H, HRGB, APP, NIMG, SEED = 12, 20, 32, 32, 16, 8, 5, 17


def main(ref_root):
    sys.path.insert(0, ref_root)
    install_stub()
    from projects.neuralangelo.utils import modules
    from projects.nerf.utils import nerf_util, render
    cfg_bg = to_attr(dict(
        enabled=True, white=False, view_dep=True,
        mlp=dict(num_layers=8, hidden_dim=H, skip=[4], num_layers_rgb=2, hidden_dim_rgb=HRGB, skip_rgb=[],
                 activ="relu", activ_params={}, activ_density="softplus", activ_density_params={}),
        encoding=dict(type="fourier", levels=10), encoding_view=dict(type="spherical", levels=3)))
    app_cfg = to_attr(dict(enabled=True, dim=APP))
    bg = modules.BackgroundNeRF(cfg_bg, appear_embed=app_cfg).double()
    ocfg = of.make_config(app_dim=APP, n_images=NIMG, bg_enabled=True, bg_hidden=H, bg_hidden_rgb=HRGB,
                          n_levels=4, n_features=2, log2_hashmap_size=8, base_resolution=4, max_resolution=16,
                          sdf_hidden=16, rgb_hidden=16, rgb_layers=1)
    params, _ = of.init_params(ocfg, seed=SEED)
    with torch.no_grad():
        for i, lin in enumerate(bg.mlp_feat.linears):
            lin.weight.copy_(params[f'bg.l{i}.w'])
            lin.bias.copy_(params[f'bg.l{i}.b'])
        for i, lin in enumerate(bg.mlp_rgb.linears):
            lin.weight.copy_(params[f'bg.rgb.l{i}.w'])
            lin.bias.copy_(params[f'bg.rgb.l{i}.b'])
    app_bg = torch.nn.Parameter(params['app_bg'].clone())

    g = torch.Generator().manual_seed(SEED)
    c = torch.randn(R, 3, generator=g, dtype=torch.float64)
    c = 3.0 * c / c.norm(dim=-1, keepdim=True)
    d = -c + 0.6 * torch.randn(R, 3, generator=g, dtype=torch.float64)
    d = d / d.norm(dim=-1, keepdim=True)
    near, far, outside = of.dist_bounds(c, d)
    app_idx = torch.randint(0, NIMG, (R,), generator=g)
    target = torch.rand(R, 3, generator=g, dtype=torch.float64)
    obj_alpha = (torch.rand(R, NO, generator=g, dtype=torch.float64) * 0.08).requires_grad_(True)
    obj_rgbs = torch.rand(R, NO, 3, generator=g, dtype=torch.float64).requires_grad_(True)
    # Model.sample_dists_background: inverse distances from 1 down to 0, stratified
    torch.manual_seed(SEED)
    inv = nerf_util.sample_dists((1, R), dist_range=(1, 0), intvs=NB, stratified=True, device="cpu").double()
    dists_bg = far[None, :, None, :] / (inv + 1e-5)                                  # [1,R,NB,1]
    points = c[None, :, None, :] + d[None, :, None, :] * dists_bg                    # camera.py:314-320
    rays_unit = d[None, :, None, :].expand_as(points)
    app_out = app_bg[app_idx][None, :, None, :].expand(1, R, NB, APP)
    rgbs_bg, dens = bg.forward(points, rays_unit, app_out)
    alphas_bg = render.volume_rendering_alphas_dist(dens, dists_bg)
    rgbs = torch.cat([obj_rgbs[None], rgbs_bg], dim=2)
    alphas = torch.cat([obj_alpha[None], alphas_bg], dim=2)
    weights = render.alpha_compositing_weights(alphas)
    rgb = render.composite(rgbs, weights)[0]
    loss = torch.nn.functional.l1_loss(rgb, target) * 3
    loss.backward()
    out = dict(center=c, ray_unit=d, far=far, app_idx=app_idx, target=target, dists_bg=dists_bg[0, :, :, 0],
               obj_alpha=obj_alpha.detach(), obj_rgbs=obj_rgbs.detach(), rgbs_bg=rgbs_bg[0].detach(),
               density=dens[0].detach(), alphas_bg=alphas_bg[0].detach(), rgb=rgb.detach(),
               loss=loss.detach(), d_obj_alpha=obj_alpha.grad, d_obj_rgbs=obj_rgbs.grad, d_app_bg=app_bg.grad,
               app_bg=params['app_bg'])
    for i, lin in enumerate(bg.mlp_feat.linears):
        out[f'bg.l{i}.w'], out[f'bg.l{i}.b'] = params[f'bg.l{i}.w'], params[f'bg.l{i}.b']
        out[f'd_bg.l{i}.w'], out[f'd_bg.l{i}.b'] = lin.weight.grad, lin.bias.grad
    for i, lin in enumerate(bg.mlp_rgb.linears):
        out[f'bg.rgb.l{i}.w'], out[f'bg.rgb.l{i}.b'] = params[f'bg.rgb.l{i}.w'], params[f'bg.rgb.l{i}.b']
        out[f'd_bg.rgb.l{i}.w'], out[f'd_bg.rgb.l{i}.b'] = lin.weight.grad, lin.bias.grad
    meta = np.array([R, NO, NB, H, HRGB, APP, NIMG])
    np.savez_compressed(os.path.join(HERE, "background.npz"), meta=meta,
                        **{k: v.detach().numpy() if torch.is_tensor(v) else v for k, v in out.items()})
    print("wrote background.npz", {k: tuple(v.shape) for k, v in out.items() if torch.is_tensor(v)}.get('rgbs_bg'))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the neuralangelo reference checkout>")
    main(sys.argv[1])
