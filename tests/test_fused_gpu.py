"""Fused FP16 step (tcgen05 kernels, C ABI) against the float64 oracle and the
plain FP32 drop-in.

Gates (the field's accuracy targets), against the float64 oracle evaluated on the
same fp16-rounded parameters: SDF relative error <= 1e-4, and every gradient tensor
-- the table and each MLP weight on its own -- within 1e-3.  With the curvature
term on, the table gradient is a second difference over the taps whose float32
conditioning is above 1e-3: there the gate is 1.25x the float32 reference
arithmetic's own error on the same tensor."""
import numpy as np
import pytest
import torch

from neuralangelo_gb300.config import field_config
from neuralangelo_gb300.fused import CapturedStep, FusedField
from neuralangelo_gb300.model import FieldModel
from neuralangelo_gb300.workloads import full_field_iteration, init_field_params, make_ragged_rays, make_rays
from oracle import field as of
from tests import params_io

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def build(log2T=14, n_images=10, seed=0, table_range=0.05, rgb_layers=4, rgb_hidden=256, small=False, active=8,
          taps=6):
    cfg = field_config("small" if small else "full")
    cfg.sdf.encoding.hashgrid.dict_size = log2T
    cfg.sdf.gradient.taps = taps
    if not small:
        cfg.appear_embed.num_images = n_images
        cfg.rgb.mlp.num_layers = rgb_layers
        cfg.rgb.mlp.hidden_dim = rgb_hidden
    torch.manual_seed(seed)
    model = FieldModel(cfg).to(DEV)
    init_field_params(model, seed)
    model.schedule(full_field_iteration(active))
    with torch.no_grad():
        model.neural_sdf.tcnn_encoding.params.uniform_(-table_range, table_range)
    return model


def oracle_run(model, batch, fp16, effective=False, retain=False, fp16_storage=False, dtype=torch.float64):
    c = model.cfg
    hg = c.sdf.encoding.hashgrid
    ocfg = of.make_config(n_levels=c.sdf.encoding.levels, n_features=hg.dim, log2_hashmap_size=hg.dict_size,
                          base_resolution=2 ** hg.min_logres, per_level_scale=model.neural_sdf.growth_rate,
                          active_levels=model.neural_sdf.active_levels, sdf_hidden=256,
                          rgb_hidden=c.rgb.mlp.hidden_dim, rgb_layers=c.rgb.mlp.num_layers,
                          app_dim=c.appear_embed.dim if c.appear_embed.enabled else 0,
                          n_images=c.appear_embed.num_images if c.appear_embed.enabled else 0,
                          taps=c.sdf.gradient.taps)
    ocfg['fp16_storage'] = fp16_storage
    from oracle import hashgrid as hgo
    layout = hgo.level_layout(ocfg['n_levels'], ocfg['n_features'], ocfg['log2_hashmap_size'],
                              ocfg['base_resolution'], ocfg['per_level_scale'])
    p = {k: (v.to(dtype).clone().requires_grad_(True) if v is not None else None)
         for k, v in params_io.model_to_oracle(model, fp16, effective).items()}
    b = {k: (v if isinstance(v, list) else v.to(dtype).cpu() if v.is_floating_point() else v.cpu())
         for k, v in batch.items()}
    if 'ray_offsets' in b:
        out = of.render_step_ragged(p, ocfg, layout, b, model.neural_sdf.normal_eps, model.progress, 0.1,
                                    model.w_curv)
    else:
        out = of.render_step(p, ocfg, layout, b, model.neural_sdf.normal_eps, model.progress, 0.1, model.w_curv,
                             retain=retain)
    out['loss'].backward()
    return out, {k: (v.grad if v is not None else None) for k, v in p.items()}


def fused_gates(ff):
    """The colour MLP's ReLU gates of the last fused step, [Ns, H] per hidden layer: the
    backward's [y > 0] on the stored fp16 hi half."""
    Hc = ff.Hc
    return [(y[:, :Hc] > 0).cpu() for y in ff.ws['ys']]


def gate_consistent(model, batch, ff, **kw):
    """The float64 oracle with the colour MLP's ReLU gates taken from the fused step.  A
    ReLU gate is discontinuous: a pre-activation within rounding of zero lands on either
    side in two valid computations (float32 against float64, one float32 summation order
    against another), and every gradient upstream of that layer moves with it.  Fed the
    fused step's gates, the oracle checks the rest of the arithmetic across them."""
    b = dict(batch)
    b['rgb_gates'] = fused_gates(ff)
    return oracle_run(model, b, fp16=True, effective=True, **kw)


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
    tgt = batch['target'].cpu().double()
    flips = int(((rgb_mine.double() - tgt).sign() != (out_q['rgb'].detach() - tgt).sign()).sum())
    margin = float((out_q['rgb'].detach() - tgt).abs().min())
    print(f"\nsdf {e_sdf:.2e} table {e_tab:.2e} rgb {e_rgb:.2e} loss {e_loss:.2e} all-params {allp:.2e} "
          f"L1-sign flips {flips} min |rgb - target| {margin:.1e}")
    print("vs fp16-weight oracle", {k: f"{v:.1e}" for k, v in worst.items()})
    print({k: f"{v:.1e}" for k, v in diag.items()})
    assert e_sdf < 1e-4                      # SDF gate
    assert e_tab < 1e-3                      # table-gradient gate
    assert e_rgb < 1e-4
    assert e_loss < 1e-5
    assert allp < 1e-3
    for k, e in worst.items():               # every gradient tensor on its own
        assert e < 1e-3, (k, e)


def test_single_fp16_activations_miss_the_gate_that_pairs_meet():
    """The same step with the activations stored as single fp16 values: the next layer's
    pre-activations move by the fp16 rounding and single weight gradients leave the 1e-3
    band, which the hi + lo pairs of the default step close."""
    model = build()
    batch = make_rays(48, 32, seed=3, miss_frac=0.1, n_images=10, device=DEV)
    errs = {}
    _, g_e = oracle_run(model, batch, fp16=True, effective=True)
    for pairs in (True, False):
        ff = FusedField(model, activation_pairs=pairs)
        model.zero_grad(set_to_none=True)
        ff.step(batch)
        torch.cuda.synchronize()
        errs[pairs] = max(rel(dW.double().cpu(), g_e[n + '.v']) for n, (dW, db) in ff.eff_grads.items())
    print(f"\nworst MLP weight-gradient error: pairs {errs[True]:.1e}, single fp16 {errs[False]:.1e}")
    assert errs[True] < 1e-3 and errs[False] > 2 * errs[True]


@pytest.mark.parametrize("active", [10, 16])
def test_fused_more_levels_matches_oracle(active):
    """10 active levels (80 encoder columns: some warps store two d_enc chunks) and all 16
    (128 columns: the largest shared-memory and TMEM footprint of the field kernels)."""
    model = build(active=active)
    assert model.neural_sdf.active_levels == active
    R, S = 32, 32
    batch = make_rays(R, S, seed=4, miss_frac=0.1, n_images=10, device=DEV)
    ff = FusedField(model)
    model.zero_grad(set_to_none=True)
    res = ff.step(batch)
    torch.cuda.synchronize()
    assert ff.check_device_errors() == 0
    assert ff.K0 == 16 * ((active * 8 + 15) // 16)       # packed at the step
    mine = fused_grads(model)
    out_q, g_q = oracle_run(model, batch, fp16=True)
    inside = ~batch['outside'][:, 0].cpu()
    e_sdf = rel(ff.ws['sdf'].reshape(R, S).cpu()[inside], out_q['sdf'].detach()[inside])
    e_tab = rel(mine['table'], g_q['table'])
    e_rgb = rel(res['rgb'].cpu(), out_q['rgb'].detach())
    print(f"\n{active} levels: sdf {e_sdf:.2e} table {e_tab:.2e} rgb {e_rgb:.2e}")
    assert e_sdf < 1e-4 and e_tab < 1e-3 and e_rgb < 1e-4


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


def test_combined_field_entry_points_match_split_calls(monkeypatch):
    """gbsdf_field_fwd / gbsdf_field_bwd (two kernels each) give the step that the four
    single-kernel calls give."""
    from neuralangelo_gb300 import _lib
    model = build()
    batch = make_rays(32, 32, seed=2, n_images=10, device=DEV)
    ff = FusedField(model)
    model.zero_grad(set_to_none=True)
    a = ff.step(batch)['loss']
    g1 = {k: v.clone() for k, v in fused_grads(model).items()}
    real = _lib.call
    seen = []

    def combined(name, *args):
        if name in ("gbsdf_field_encode", "gbsdf_field_scatter"):
            return None                                  # part of the combined call below
        name = {"gbsdf_field_mlp_fwd": "gbsdf_field_fwd", "gbsdf_field_mlp_bwd": "gbsdf_field_bwd"}.get(name, name)
        seen.append(name)
        return real(name, *args)

    monkeypatch.setattr(_lib, "call", combined)
    model.zero_grad(set_to_none=True)
    b = ff.step(batch)['loss']
    torch.cuda.synchronize()
    assert "gbsdf_field_fwd" in seen and "gbsdf_field_bwd" in seen
    assert abs(a - b) < 1e-6 * abs(a)
    g2 = fused_grads(model)
    for k in ('table', 'sdf.l0.v', 'sdf.head.w', 'rgb.l0.v'):
        assert rel(g2[k].cpu(), g1[k].cpu()) < 1e-5, k          # atomics reorder only


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


def test_fused_ragged_matches_oracle():
    """Ragged batch (30% of the rays culled to zero samples, the rest 2..40 samples):
    the same gates as the dense step against the float64 oracle run ray by ray."""
    model = build()
    batch = make_ragged_rays(40, seed=4, zero_frac=0.3, lo=2, hi=40, n_images=10, device=DEV)
    ff = FusedField(model)
    model.zero_grad(set_to_none=True)
    res = ff.step(batch)
    torch.cuda.synchronize()
    assert ff.check_device_errors() == 0
    mine = fused_grads(model)
    out_q, g_q = oracle_run(model, batch, fp16=True)
    live = ~batch['outside'][batch['sample_ray'].long(), 0].cpu()
    e_sdf = rel(ff.ws['sdf'].cpu()[live], out_q['sdf'].detach()[live])
    e_tab = rel(mine['table'], g_q['table'])
    e_rgb = rel(res['rgb'].cpu(), out_q['rgb'].detach())
    e_loss = abs(res['loss'] - float(out_q['loss'])) / abs(float(out_q['loss']))
    print(f"\nragged: sdf {e_sdf:.2e} table {e_tab:.2e} rgb {e_rgb:.2e} loss {e_loss:.2e}")
    assert e_sdf < 1e-4 and e_tab < 1e-3 and e_rgb < 1e-4 and e_loss < 1e-5
    # every weight and embedding gradient on its own, against the oracle that takes the fused
    # step's ReLU gates (see gate_consistent); the distance to the plain oracle is printed
    _, g_e = oracle_run(model, batch, fp16=True, effective=True)
    _, g_g = gate_consistent(model, batch, ff)
    e_w = {n: rel(dW.double().cpu(), g_g[n + '.v']) for n, (dW, db) in ff.eff_grads.items()}
    e_w.update({k: rel(mine[k], g_g[k]) for k in ('sdf.head.w', 's_var', 'app')})
    e_plain = {n: rel(dW.double().cpu(), g_e[n + '.v']) for n, (dW, db) in ff.eff_grads.items()}
    print("gate-consistent oracle:", {k: f"{v:.1e}" for k, v in e_w.items()})
    print("oracle with its own ReLU gates:", {k: f"{v:.1e}" for k, v in e_plain.items()})
    for k, e in e_w.items():
        assert e < 1e-3, (k, e)
    # a culled ray renders black: its colour is exactly zero
    counts = (batch['ray_offsets'][1:] - batch['ray_offsets'][:-1]).cpu()
    assert torch.all(res['rgb'].cpu()[counts == 0] == 0)


def test_ragged_layout_of_a_dense_batch_equals_dense():
    """The ragged entry points given a dense batch in ragged form (every ray S samples)
    reproduce the dense path: same loss, same gradients up to atomic reordering."""
    model = build()
    dense = make_rays(64, 24, seed=6, miss_frac=0.1, n_images=10, device=DEV)
    ff = FusedField(model)
    model.zero_grad(set_to_none=True)
    a = ff.step(dense)
    g_dense = {k: v.clone() for k, v in fused_grads(model).items()}
    rag = dict(dense)
    rag['dists'] = dense['dists'].reshape(-1)
    rag['ray_offsets'] = torch.arange(65, device=DEV, dtype=torch.int64) * 24
    rag['sample_ray'] = torch.arange(64, device=DEV, dtype=torch.int32).repeat_interleave(24)
    ff2 = FusedField(model)
    model.zero_grad(set_to_none=True)
    b = ff2.step(rag)
    g_rag = fused_grads(model)
    assert abs(a['loss'] - b['loss']) <= 1e-6 * abs(a['loss'])
    assert torch.equal(ff.ws['sdf'], ff2.ws['sdf'])
    for k in ('table', 'sdf.l0.v', 'rgb.l0.v', 's_var', 'app'):
        assert rel(g_rag[k], g_dense[k]) < 1e-5, k


def test_captured_graph_step_matches_eager():
    """The whole ragged step (gradient zeroing, forward, backward) captured in one CUDA
    graph: replays reproduce the eager step, also after new inputs are copied in."""
    model = build()
    batch = make_ragged_rays(48, seed=8, zero_frac=0.3, lo=4, hi=48, n_images=10, device=DEV)
    ff = FusedField(model)
    model.zero_grad(set_to_none=True)
    a = ff.step(batch)
    g_eager = {k: v.clone() for k, v in fused_grads(model).items()}
    cap = CapturedStep(ff, batch)
    for _ in range(2):                         # replays do not accumulate
        cap.replay()
    torch.cuda.synchronize()
    assert abs(cap.losses()['loss'] - a['loss']) <= 1e-6 * abs(a['loss'])
    g = fused_grads(model)
    for k in ('table', 'sdf.l0.v', 'sdf.l1.v', 'rgb.l0.v', 's_var', 'app'):
        assert rel(g[k], g_eager[k]) < 1e-5, k
    b2 = dict(batch)
    b2['target'] = torch.rand_like(batch['target'])
    cap.replay(b2)
    torch.cuda.synchronize()
    l_graph = cap.losses()['loss']
    g_graph = {k: v.clone() for k, v in fused_grads(model).items()}
    model.zero_grad(set_to_none=False)
    l_eager = ff.step(b2)['loss']
    assert abs(l_graph - l_eager) <= 1e-6 * abs(l_eager)
    g2 = fused_grads(model)
    for k in ('table', 'rgb.l4.v', 's_var'):
        assert rel(g_graph[k], g2[k]) < 1e-5, k


def test_c2_accuracy_report_512_rays():
    """Mixed-precision accuracy on the full field (L16 F8 T=2^22, 8 active levels, colour
    MLP 4x256, 100 images) for a 512-ray x 128-sample subset against the float64 oracle
    on the same fp16 parameters.

    SDF <= 1e-4 and colour <= 1e-4 (relative); each MLP weight and bias gradient <= 1e-3.
    The table gradient of the numerical curvature loss is a second difference over the
    taps, (df+ + df- - 2 df0) / eps^2, which amplifies FP32 rounding by up to 1/eps^2:
    the reference's own arithmetic run in float32 on these inputs misses float64 by
    ~1.5e-3.  Gates: with the curvature term each gradient tensor is within 1e-3 or
    1.25x of the float32 error on that tensor; without it, the table meets 1e-3."""
    model = build(log2T=22, n_images=100, table_range=1e-2)
    batch = make_rays(512, 128, seed=11, miss_frac=0.05, n_images=100, device=DEV)
    ff = FusedField(model)
    model.zero_grad(set_to_none=True)
    res = ff.step(batch)
    torch.cuda.synchronize()
    assert ff.check_device_errors() == 0
    mine = fused_grads(model)
    out_q, g_q = oracle_run(model, batch, fp16=True)
    _, g_32 = oracle_run(model, batch, fp16=True, dtype=torch.float32)
    inside = ~batch['outside'][:, 0].cpu()
    e_sdf = rel(ff.ws['sdf'].reshape(512, 128).cpu()[inside], out_q['sdf'].detach()[inside])
    e_rgb = rel(res['rgb'].cpu(), out_q['rgb'].detach())
    e_tab = rel(mine['table'], g_q['table'])
    e_tab32 = rel(g_32['table'], g_q['table'])
    eff_curv = {n: (dW.clone(), db.clone()) for n, (dW, db) in ff.eff_grads.items()}
    _, g_ec = oracle_run(model, batch, fp16=True, effective=True)
    _, g_ec32 = oracle_run(model, batch, fp16=True, effective=True, dtype=torch.float32)
    # the float32 reference arithmetic's error through the curvature term swings between two
    # equally valid fp16 roundings of the same FP32 weights (the step's copies and torch's): the
    # yardstick is the larger of the two
    with params_io.torch_rounded_weights():
        _, g_qt = oracle_run(model, batch, fp16=True)
        _, g_32t = oracle_run(model, batch, fp16=True, dtype=torch.float32)
        _, g_ect = oracle_run(model, batch, fp16=True, effective=True)
        _, g_ect32 = oracle_run(model, batch, fp16=True, effective=True, dtype=torch.float32)
    e_tab32 = max(e_tab32, rel(g_32t['table'], g_qt['table']))
    # the same step without the curvature term
    model.w_curv = 0.0
    model.zero_grad(set_to_none=True)
    ff.step(batch)
    torch.cuda.synchronize()
    mine0 = fused_grads(model)
    _, g_q0 = oracle_run(model, batch, fp16=True)
    e_tab0 = rel(mine0['table'], g_q0['table'])
    print(f"\nC2 512 rays: sdf {e_sdf:.2e} colour {e_rgb:.2e} table-grad {e_tab:.2e} "
          f"(float32 reference arithmetic {e_tab32:.2e}; without curvature {e_tab0:.2e})")
    # MLP weight gradients (effective, weight-norm space) against the float64 oracle on
    # the same fp16 weights, curvature off as in the step just taken
    _, g_e = oracle_run(model, batch, fp16=True, effective=True)
    e_w = {n: rel(dW.double().cpu(), g_e[n + '.v']) for n, (dW, db) in ff.eff_grads.items()}
    e_b = {n: rel(db.double().cpu(), g_e[n + '.b']) for n, (dW, db) in ff.eff_grads.items()}
    allp = rel(np.concatenate([ff.eff_grads[n][0].double().cpu().reshape(-1) for n in ff.eff_grads]),
               np.concatenate([g_e[n + '.v'].reshape(-1) for n in ff.eff_grads]))
    print("C2 MLP weight gradients:", {k: f"{v:.1e}" for k, v in e_w.items()}, f"all MLP weights {allp:.2e}")
    print("C2 MLP bias gradients:", {k: f"{v:.1e}" for k, v in e_b.items()})
    # with the curvature term on: each MLP weight gradient against the same float64 oracle,
    # gated at 1e-3 or 1.25x the float32 reference arithmetic's error on that tensor
    e_wc = {n: rel(dW.double().cpu(), g_ec[n + '.v']) for n, (dW, db) in eff_curv.items()}
    e_wc32 = {n: max(rel(g_ec32[n + '.v'], g_ec[n + '.v']), rel(g_ect32[n + '.v'], g_ect[n + '.v']))
              for n in eff_curv}
    print("C2 MLP weight gradients, curvature on:", {k: f"{v:.1e}" for k, v in e_wc.items()},
          "float32 reference:", {k: f"{v:.1e}" for k, v in e_wc32.items()})
    # every tensor on its own (the activations are stored as fp16 hi + lo pairs)
    for k, e in list(e_w.items()) + list(e_b.items()):
        assert e < 1e-3, (k, e)
    for k, e in e_wc.items():
        assert e < max(1e-3, 1.25 * e_wc32[k]), (k, e, e_wc32[k])
    assert allp < 1e-3
    assert e_sdf < 1e-4 and e_rgb < 1e-4
    assert e_tab < 1.25 * e_tab32
    assert e_tab0 < 1e-3


def test_in_kernel_layer0_weight_gradient_matches_gemm_path():
    """K0 <= 64: the backward kernel's own dW0 (TMEM accumulators, per-CTA atomics) against the
    d_pre0 rows + k_wgrad path on the same step; every other gradient must agree as well."""
    model = build(seed=5)
    batch = make_rays(96, 64, seed=12, miss_frac=0.2, n_images=10, device=DEV)
    grads = []
    for fused in (True, False):
        ff = FusedField(model, fused_w0_grad=fused)
        model.zero_grad(set_to_none=True)
        ff.step(batch)
        torch.cuda.synchronize()
        assert ff.check_device_errors() == 0
        assert (ff.ws['d_w0'] is not None) == fused and (ff.ws['d_pre0'] is None) == fused
        grads.append({k: v.clone() for k, v in params_io.model_grads(model).items() if v is not None})
    a, b = grads
    errs = {k: rel(a[k].cpu(), b[k].cpu()) for k in b}
    print("\nin-kernel dW0 vs GEMM:", {k: f"{v:.1e}" for k, v in errs.items()})
    # the same fp16 products summed in another order (FP32 both ways)
    for k, e in errs.items():
        assert e < 1e-5, (k, e)


def test_captured_step_follows_the_schedule():
    """A captured step replayed after model.schedule(): the anneal ratio and curvature weight
    come from a device buffer refreshed at every replay (the replay equals an eager step at
    the new iteration), and a change of active levels / normal epsilon re-captures."""
    model = build()
    batch = make_rays(32, 24, seed=9, miss_frac=0.1, n_images=10, device=DEV)
    model.schedule(2000)                                  # warm-up: w_curv ramps with the iteration
    ff = FusedField(model)
    cap = CapturedStep(ff, batch)
    model.zero_grad(set_to_none=False)
    l_2000 = ff.step(batch)['loss']
    model.schedule(3000)
    assert ff.schedule_key() == cap.key
    cap.replay()
    torch.cuda.synchronize()
    l_graph = cap.losses()['loss']
    g_graph = {k: v.clone() for k, v in fused_grads(model).items()}
    model.zero_grad(set_to_none=False)
    l_eager = ff.step(batch)['loss']
    g_eager = fused_grads(model)
    print(f"\nloss at 2000 {l_2000:.6e}, at 3000: graph {l_graph:.6e} eager {l_eager:.6e}")
    assert abs(l_2000 - l_eager) > 1e-4 * abs(l_eager)     # the schedule moved the loss
    assert abs(l_graph - l_eager) <= 1e-6 * abs(l_eager)
    for k in ('table', 'sdf.l0.v', 'rgb.l0.v', 's_var'):
        assert rel(g_graph[k], g_eager[k]) < 1e-5, k
    # coarse-to-fine: more active levels (and a new epsilon) -> the replay captures again
    model.schedule(full_field_iteration(8))
    assert ff.schedule_key() != cap.key
    cap.replay()
    torch.cuda.synchronize()
    assert cap.recaptures == 1
    l_graph = cap.losses()['loss']
    g_graph = {k: v.clone() for k, v in fused_grads(model).items()}
    model.zero_grad(set_to_none=False)
    l_eager = ff.step(batch)['loss']
    g_eager = fused_grads(model)
    assert abs(l_graph - l_eager) <= 1e-6 * abs(l_eager)
    for k in ('table', 'sdf.l0.v', 'rgb.l0.v'):
        assert rel(g_graph[k], g_eager[k]) < 1e-5, k


def test_dynamic_loss_scale_inside_the_graph():
    """GradScaler's rule on the device, replay by replay: an overflowing scale halves until the
    gradients are finite, growth_interval clean steps double it; an inf planted in an input
    between replays raises found_inf and halves the scale; gradients of clean steps match an
    eager step at the default scale."""
    model = build()
    batch = make_rays(32, 16, seed=1, n_images=10, device=DEV)
    ref = FusedField(model)
    model.zero_grad(set_to_none=True)
    ref.step(batch)
    g_ref = {k: v.clone() for k, v in fused_grads(model).items()}
    ff = FusedField(model, loss_scale=2.0 ** 40, growth_interval=3)
    cap = CapturedStep(ff, batch, warmup=0)
    scale, tracker, seen = 2.0 ** 40, 0, []
    for _ in range(30):
        cap.replay()
        inf = ff.found_inf()
        new = ff.current_loss_scale()
        seen.append((scale, inf))
        # GradScaler.update: back off on overflow, grow after growth_interval clean steps
        if inf:
            want, tracker = scale * 0.5, 0
        else:
            tracker += 1
            want = scale * 2.0 if tracker == 3 else scale
            tracker = 0 if tracker == 3 else tracker
        assert new == want, (seen, new, want)
        if not inf:
            g = fused_grads(model)
            for k in ('table', 'sdf.l0.v', 'rgb.l4.v', 's_var'):
                assert torch.isfinite(g[k]).all() and rel(g[k], g_ref[k]) < 1e-3, k
        scale = new
    flags = [f for _, f in seen]
    assert flags[0] and not all(flags) and any(not f for f in flags[-6:])
    print("\nscale / found_inf per replay:", [(int(round(torch.log2(torch.tensor(s)).item())), f) for s, f in seen])
    # an inf in an input (an appearance code used by the batch) between replays
    img = int(batch['app_idx'][0])
    while ff.found_inf():
        cap.replay()
    before = ff.current_loss_scale()
    with torch.no_grad():
        saved = model.appear_embed.weight[img].clone()
        model.appear_embed.weight[img, 0] = float('inf')
    cap.replay()
    assert ff.found_inf() and ff.current_loss_scale() == before * 0.5
    with torch.no_grad():
        model.appear_embed.weight[img] = saved
    cap.replay()
    assert not ff.found_inf()


@pytest.mark.parametrize("ragged", [False, True])
def test_fused_4_taps_matches_oracle(ragged):
    """The tetrahedral 4-tap stencil (modules.py:157-175, the reference's default
    configuration, projects/neuralangelo/configs/base.yaml:68): 25 samples of 5 evaluations
    per tile.  Same gates as the 6-tap step: SDF <= 1e-4, colour <= 1e-4, loss <= 1e-5,
    every gradient tensor <= 1e-3 against the float64 oracle on the same fp16 parameters
    (table: curvature off; with curvature, <= 1.25x the float32 reference's own error)."""
    model = build(taps=4)
    if ragged:
        batch = make_ragged_rays(40, seed=4, zero_frac=0.3, lo=2, hi=40, n_images=10, device=DEV)
    else:
        batch = make_rays(48, 32, seed=3, miss_frac=0.1, n_images=10, device=DEV)
    ff = FusedField(model)
    assert ff.taps == 4 and ff.tile_rows == 125
    model.zero_grad(set_to_none=True)
    res = ff.step(batch)
    torch.cuda.synchronize()
    assert ff.check_device_errors() == 0
    mine = fused_grads(model)
    out_q, g_q = oracle_run(model, batch, fp16=True)
    _, g_32 = oracle_run(model, batch, fp16=True, dtype=torch.float32)
    if ragged:
        live = ~batch['outside'][batch['sample_ray'].long(), 0].cpu()
        sdf_mine = ff.ws['sdf'].cpu()
    else:
        live = (~batch['outside'][:, 0].cpu())[:, None].expand(48, 32)
        sdf_mine = ff.ws['sdf'].reshape(48, 32).cpu()
    e_sdf = rel(sdf_mine[live], out_q['sdf'].detach()[live])
    e_rgb = rel(res['rgb'].cpu(), out_q['rgb'].detach())
    e_loss = abs(res['loss'] - float(out_q['loss'])) / abs(float(out_q['loss']))
    e_tab, e_tab32 = rel(mine['table'], g_q['table']), rel(g_32['table'], g_q['table'])
    _, g_e = oracle_run(model, batch, fp16=True, effective=True)
    _, g_g = gate_consistent(model, batch, ff)
    e_w = {n: rel(dW.double().cpu(), g_g[n + '.v']) for n, (dW, db) in ff.eff_grads.items()}
    e_w.update({k: rel(mine[k], g_g[k]) for k in ('sdf.head.w', 's_var', 'app')})
    e_plain = {n: rel(dW.double().cpu(), g_e[n + '.v']) for n, (dW, db) in ff.eff_grads.items()}
    model.w_curv = 0.0
    model.zero_grad(set_to_none=True)
    ff.step(batch)
    torch.cuda.synchronize()
    _, g_q0 = oracle_run(model, batch, fp16=True)
    e_tab0 = rel(fused_grads(model)['table'], g_q0['table'])
    print(f"\n4 taps{' ragged' if ragged else ''}: sdf {e_sdf:.2e} rgb {e_rgb:.2e} loss {e_loss:.2e} "
          f"table {e_tab:.2e} (float32 reference {e_tab32:.2e}; without curvature {e_tab0:.2e})")
    print("gate-consistent oracle:", {k: f"{v:.1e}" for k, v in e_w.items()})
    print("oracle with its own ReLU gates:", {k: f"{v:.1e}" for k, v in e_plain.items()})
    assert e_sdf < 1e-4 and e_rgb < 1e-4 and e_loss < 1e-5
    assert e_tab0 < 1e-3 and e_tab < max(1e-3, 1.25 * e_tab32)
    for k, e in e_w.items():
        assert e < 1e-3, (k, e)


def test_fused_4_taps_matches_plain():
    """4 taps: the fused step against the plain FP32 drop-in (NeuralSDF.compute_gradients
    with the tetrahedral stencil) on the same FP32 masters."""
    model = build(taps=4, log2T=16, table_range=1e-2)
    batch = make_rays(128, 64, seed=5, n_images=10, device=DEV)
    model.zero_grad(set_to_none=True)
    out = model.render_step(batch)
    out['loss'].backward()
    ref = {k: v.clone() for k, v in fused_grads(model).items()}
    ref_loss = float(out['loss'])
    model.zero_grad(set_to_none=True)
    res = FusedField(model).step(batch)
    torch.cuda.synchronize()
    mine = fused_grads(model)
    assert abs(res['loss'] - ref_loss) < 2e-3 * abs(ref_loss)
    for k in ('table', 'sdf.l0.v', 'sdf.l1.v', 'rgb.l0.v', 's_var'):
        assert rel(mine[k], ref[k]) < 2e-2, k


def test_deterministic_table_scatter():
    """The fixed-point table scatter: two runs give bit-identical table gradients, and they
    agree with the FP32-atomics path up to its summation order."""
    model = build()
    batch = make_rays(64, 32, seed=2, miss_frac=0.1, n_images=10, device=DEV)
    tabs = []
    for det in (True, True, False):
        ff = FusedField(model, deterministic_table=det)
        model.zero_grad(set_to_none=True)
        ff.step(batch)
        torch.cuda.synchronize()
        tabs.append(model.neural_sdf.tcnn_encoding.params.grad.clone())
    assert torch.equal(tabs[0], tabs[1])
    e = rel(tabs[0].cpu(), tabs[2].cpu())
    print(f"\ndeterministic vs atomics: {e:.1e}")
    assert e < 1e-6
