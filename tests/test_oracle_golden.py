"""Pin the oracle restatement (oracle/field.py) against golden vectors produced by
the reference's own modules (tests/golden/make_golden.py)."""
import numpy as np
import pytest
import torch

from oracle import field as of
from oracle import hashgrid as hg
from tests import golden_io


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", golden_io.CASES)
def test_oracle_matches_reference_modules(name):
    g = golden_io.load(name)
    cfg, z = g['cfg'], g['z']
    params = {k: v.clone().requires_grad_(True) for k, v in g['params'].items()}
    layout = hg.level_layout(cfg['n_levels'], cfg['n_features'], cfg['log2_hashmap_size'],
                             cfg['base_resolution'], cfg['per_level_scale'])
    assert abs(of.normal_eps(cfg, g['anneal']) - g['eps']) < 1e-15
    out = of.render_step(params, cfg, layout, g['batch'], g['eps'], g['progress'], g['w_eik'], g['w_curv'])
    out['loss'].backward()
    for key in ('sdf', 'feat', 'grads', 'hess', 'rgbs', 'alphas', 'weights', 'rgb'):
        ref = z[key]
        mine = out[key].detach().numpy()
        if key == 'hess':   # rays outside the sphere carry ~1e8 values (masked in the loss)
            m = ~z['outside'][:, 0]
            ref, mine = ref[m], mine[m]
        assert rel(mine, ref) < 1e-12, key
    losses = [out['loss'], out['l_render'], out['l_eik'], out['l_curv'] if out['l_curv'] is not None else 0.0]
    np.testing.assert_allclose([float(v) for v in losses], z['losses'], rtol=1e-12, atol=1e-15)
    assert rel(params['table'].grad, z['g_table']) < 1e-10
    assert rel(params['s_var'].grad, z['g_s_var']) < 1e-10
    assert rel(params['sdf.head.w'].grad, z['g_head_w']) < 1e-10
    for k in z:
        if k.startswith('g_sdf.') or k.startswith('g_rgb.'):
            assert rel(params[k[2:]].grad, z[k]) < 1e-10, k
    if 'g_app' in z:
        assert rel(params['app'].grad, z['g_app']) < 1e-10
    assert np.linalg.norm(z['g_table']) > 0   # the perturbed encoding columns make the table gradient live


def test_background_oracle_matches_reference_golden():
    """Background NeRF (modules.py:232-311), its alphas (render.py:68-84) and the
    compositing behind object samples (model.py:129-141), forward and the L1 loss
    gradients, against the reference's own modules run in float64
    (tests/golden/make_golden_background.py)."""
    z = np.load(golden_io.GOLDEN + "/background.npz")
    R, NO, NB, H, HRGB, APP, NIMG = [int(v) for v in z['meta']]
    cfg = of.make_config(app_dim=APP, n_images=NIMG, bg_enabled=True, bg_hidden=H, bg_hidden_rgb=HRGB)
    p = {k: torch.from_numpy(z[k]).requires_grad_(True) for k in z.files
         if k.startswith('bg.') or k == 'app_bg'}
    t = {k: torch.from_numpy(z[k]) for k in ('center', 'ray_unit', 'far', 'app_idx', 'target', 'dists_bg')}
    obj_a = torch.from_numpy(z['obj_alpha']).requires_grad_(True)
    obj_c = torch.from_numpy(z['obj_rgbs']).requires_grad_(True)
    rgbs_bg, alphas_bg = of.background_branch(p, cfg, t['center'], t['ray_unit'], t['dists_bg'], t['app_idx'])
    w = of.compositing_weights(torch.cat([obj_a, alphas_bg], dim=1))
    rgb = (torch.cat([obj_c, rgbs_bg], dim=1) * w[..., None]).sum(dim=1)
    loss = (rgb - t['target']).abs().mean() * 3
    loss.backward()
    close = dict(rtol=1e-10, atol=1e-12)
    assert np.allclose(rgbs_bg.detach().numpy(), z['rgbs_bg'], **close)
    assert np.allclose(alphas_bg.detach().numpy(), z['alphas_bg'], **close)
    assert np.allclose(rgb.detach().numpy(), z['rgb'], **close)
    assert np.allclose(float(loss), float(z['loss']), **close)
    assert np.allclose(obj_a.grad.numpy(), z['d_obj_alpha'], **close)
    assert np.allclose(obj_c.grad.numpy(), z['d_obj_rgbs'], **close)
    assert np.allclose(p['app_bg'].grad.numpy(), z['d_app_bg'], **close)
    for k, v in p.items():
        if k.startswith('bg.'):
            assert np.allclose(v.grad.numpy(), z['d_' + k], **close), k
