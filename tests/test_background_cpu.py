"""The package's plain BackgroundNeRF module (torch, the reference's structure) against
the reference's own module through the golden fixture; CPU, float64."""
import numpy as np
import torch

from neuralangelo_gb300.config import background_config, to_attr
from neuralangelo_gb300.modules import BackgroundNeRF
from neuralangelo_gb300 import render
from neuralangelo_gb300.workloads import background_dists
from tests import golden_io


def test_plain_background_module_matches_reference_golden():
    z = np.load(golden_io.GOLDEN + "/background.npz")
    R, NO, NB, H, HRGB, APP, NIMG = [int(v) for v in z['meta']]
    bg = BackgroundNeRF(background_config(hidden=H, hidden_rgb=HRGB), to_attr(dict(enabled=True, dim=APP))).double()
    with torch.no_grad():
        for i, lin in enumerate(bg.mlp_feat.linears):
            lin.weight.copy_(torch.from_numpy(z[f'bg.l{i}.w']))
            lin.bias.copy_(torch.from_numpy(z[f'bg.l{i}.b']))
        for i, lin in enumerate(bg.mlp_rgb.linears):
            lin.weight.copy_(torch.from_numpy(z[f'bg.rgb.l{i}.w']))
            lin.bias.copy_(torch.from_numpy(z[f'bg.rgb.l{i}.b']))
    c, d = torch.from_numpy(z['center']), torch.from_numpy(z['ray_unit'])
    dists = torch.from_numpy(z['dists_bg'])
    pts = c[:, None, :] + d[:, None, :] * dists[..., None]
    app = torch.from_numpy(z['app_bg'])[torch.from_numpy(z['app_idx'])][:, None, :].expand(R, NB, APP)
    rgbs, dens = bg(pts, d[:, None, :].expand_as(pts), app)
    assert np.allclose(rgbs.detach().numpy(), z['rgbs_bg'], rtol=1e-10, atol=1e-12)
    assert np.allclose(dens.detach().numpy(), z['density'], rtol=1e-10, atol=1e-12)
    alphas = render.volume_rendering_alphas_dist(dens, dists)
    assert np.allclose(alphas.detach().numpy(), z['alphas_bg'], rtol=1e-10, atol=1e-12)


def test_background_dists_follow_inverse_depth_sampling():
    far = torch.tensor([[2.0], [3.5]])
    d = background_dists(far, 32)                 # u = 0.5: inverse depth 1 - (k + 0.5)/32
    inv = 1 - (torch.arange(32) + 0.5) / 32
    assert torch.allclose(d, far / (inv + 1e-5))
    assert torch.all(d[:, 1:] > d[:, :-1]) and torch.all(d[:, 0] >= far[:, 0])
