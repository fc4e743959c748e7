"""Evaluation rendering (Model.render_rays / render_image with training off) and
textured-mesh colours against the float64 oracle."""
import functools

import numpy as np
import pytest
import torch

from neuralangelo_gb300 import mesh as gm
from neuralangelo_gb300.fused import FusedField
from neuralangelo_gb300.inference import Inference, extract_texture
from neuralangelo_gb300.workloads import make_rays
from oracle import field as of
from tests import params_io
from tests.test_background_gpu import build, oracle_run

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_cfg(model):
    c = model.cfg
    hg = c.sdf.encoding.hashgrid
    b = c.background.mlp
    cfg = of.make_config(n_levels=c.sdf.encoding.levels, n_features=hg.dim, log2_hashmap_size=hg.dict_size,
                         base_resolution=2 ** hg.min_logres, per_level_scale=model.neural_sdf.growth_rate,
                         active_levels=model.neural_sdf.active_levels, sdf_hidden=256,
                         rgb_hidden=c.rgb.mlp.hidden_dim, rgb_layers=c.rgb.mlp.num_layers,
                         app_dim=c.appear_embed.dim, n_images=c.appear_embed.num_images,
                         bg_enabled=model.with_background, bg_hidden=b.hidden_dim, bg_hidden_rgb=b.hidden_dim_rgb)
    from oracle import hashgrid as hgo
    layout = hgo.level_layout(cfg['n_levels'], cfg['n_features'], cfg['log2_hashmap_size'],
                              cfg['base_resolution'], cfg['per_level_scale'])
    return cfg, layout


def test_eval_render_matches_oracle():
    model = build()
    batch = make_rays(24, 48, seed=9, miss_frac=0.25, n_images=10, device=DEV, n_bg=32, miss_perpendicular=True)
    batch.pop('target')
    ev = FusedField(model).render(batch)
    torch.cuda.synchronize()
    cfg, layout = oracle_cfg(model)
    p = {k: v.double() for k, v in params_io.model_to_oracle(model, True).items() if v is not None}
    bt = {k: (v.double().cpu() if v.is_floating_point() else v.cpu()) for k, v in batch.items()}
    with torch.no_grad():
        ref = of.render_eval(p, cfg, layout, bt, model.neural_sdf.normal_eps, model.progress)
    errs = {k: rel(ev[k].cpu(), ref[k]) for k in ('rgb', 'opacity', 'gradient', 'dist')}
    print("\neval render:", {k: f"{v:.1e}" for k, v in errs.items()})
    for k, e in errs.items():
        assert e < 1e-4, (k, e)


def test_render_image_maps():
    model = build(seed=2)
    # camera at distance 3 on +z looking at the origin (world-to-camera [R|t])
    R = torch.diag(torch.tensor([1.0, -1.0, -1.0]))
    pose = torch.cat([R, torch.tensor([[0.0], [0.0], [3.0]])], dim=1).to(DEV)
    H, W = 12, 16
    intr = torch.tensor([[14.0, 0.0, W / 2], [0.0, 14.0, H / 2], [0.0, 0.0, 1.0]], device=DEV)
    maps = Inference(model, chunk=64).render_image(pose, intr, H, W, image_idx=3)
    assert maps['rgb_map'].shape == (3, H, W) and maps['normal_map'].shape == (3, H, W)
    assert maps['opacity_map'].shape == (1, H, W) and maps['depth_map'].shape == (1, H, W)
    for v in maps.values():
        assert torch.isfinite(v).all()
    op = maps['opacity_map'][0]
    assert float(op[H // 2, W // 2]) > 0.5                 # the geometric-init sphere covers the centre
    dep = maps['depth_map'][0][op > 0.9]
    assert dep.numel() and torch.all((dep > 2.0) & (dep < 3.2))   # the sphere of radius 0.5 at distance 3


def test_extract_texture_matches_oracle():
    model = build(seed=4)
    rng = np.random.default_rng(0)
    v = rng.normal(size=(300, 3))
    pts = 0.5 * v / np.linalg.norm(v, axis=1, keepdims=True)
    col = extract_texture(pts, model)
    cfg, layout = oracle_cfg(model)
    p = {k: v.double() for k, v in params_io.model_to_oracle(model, False).items() if v is not None}
    x = torch.from_numpy(pts).double()[None]
    with torch.no_grad():
        sdf, feat = of.neural_sdf(p, cfg, layout, x, with_feat=True)
        grads, _ = of.compute_gradients(p, cfg, layout, x, model.neural_sdf.normal_eps, sdf, training=False)
        n = torch.nn.functional.normalize(grads, dim=-1)
        app = torch.zeros(1, x.shape[1], cfg['app_dim'], dtype=torch.float64)
        rgb = of.neural_rgb(p, cfg, x, n, -n, feat, app)[0].numpy()
    want = (rgb * 255).astype(np.uint8)
    assert col.shape == (300, 3) and col.dtype == np.uint8
    assert np.abs(col.astype(int) - want.astype(int)).max() <= 1


def test_textured_mesh_export(tmp_path):
    model = build(seed=4)
    f = gm.FieldSDF(model.neural_sdf, sign=-1.0)
    mesh = gm.extract_mesh(f, [(-1, 1)] * 3, 2.0 / 32, block_res=16, device=DEV,
                           texture_func=functools.partial(extract_texture, model=model))
    assert mesh.colors is not None and mesh.colors.shape == (len(mesh.vertices), 3)
    out = gm.export_mesh(mesh, tmp_path / "tex.ply", device=DEV)
    V, F, C = gm.read_ply(tmp_path / "tex.ply")
    assert np.array_equal(C[:, :3], out.colors) and len(F) == len(out.faces)
