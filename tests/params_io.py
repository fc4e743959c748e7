"""Move parameters between the package's FieldModel and the oracle's dict layout."""
import numpy as np
import torch

from neuralangelo_gb300.config import field_config, rgb_config, sdf_config, to_attr
from neuralangelo_gb300.model import FieldModel


def model_from_golden(g, device, table_dtype=torch.float32):
    """FieldModel configured like a golden case, with the golden parameters loaded."""
    c = g['cfg']
    L, Fd = c['n_levels'], c['n_features']
    min_logres = int(round(np.log2(c['base_resolution'])))
    sdf = sdf_config(levels=L, dim=Fd, dict_size=c['log2_hashmap_size'], min_logres=min_logres,
                     max_logres=None, per_level_scale=c['per_level_scale'], hidden=c['sdf_hidden'],
                     taps=c['taps'])
    rgb = rgb_config(layers=c['rgb_layers'], hidden=c['rgb_hidden'])
    cfg = field_config("small")
    cfg.sdf, cfg.rgb = sdf, rgb
    cfg.appear_embed = to_attr(dict(enabled=c['app_dim'] > 0, dim=c['app_dim'], num_images=c['n_images']))
    model = FieldModel(cfg, table_dtype=table_dtype).to(device)
    load_oracle_params(model, g['params'])
    sdfm = model.neural_sdf
    sdfm.active_levels = c['active_levels']
    sdfm.anneal_levels = g['anneal']
    sdfm.set_normal_epsilon()
    assert abs(sdfm.normal_eps - g['eps']) < 1e-15
    model.progress = g['progress']
    model.w_curv = g['w_curv']
    cfg.loss_weight.eikonal = g['w_eik']
    return model


def load_oracle_params(model, p):
    with torch.no_grad():
        s = model.neural_sdf
        s.tcnn_encoding.params.copy_(p['table'].to(s.tcnn_encoding.params.dtype))
        for i in range(2):
            lin = s.mlp.linears[i]
            lin.weight_v.copy_(p[f'sdf.l{i}.v'])
            lin.weight_g.copy_(p[f'sdf.l{i}.g'])
            lin.bias.copy_(p[f'sdf.l{i}.b'])
        s.mlp.linear_sdf.weight.copy_(p['sdf.head.w'])
        s.mlp.linear_sdf.bias.copy_(p['sdf.head.b'])
        for i, lin in enumerate(model.neural_rgb.mlp.linears):
            lin.weight_v.copy_(p[f'rgb.l{i}.v'])
            lin.weight_g.copy_(p[f'rgb.l{i}.g'])
            lin.bias.copy_(p[f'rgb.l{i}.b'])
        model.s_var.copy_(p['s_var'])
        if model.appear_embed is not None:
            model.appear_embed.weight.copy_(p['app'])


def model_grads(model):
    """Gradients of a FieldModel in the oracle's naming."""
    s = model.neural_sdf
    g = {'table': s.tcnn_encoding.params.grad, 'sdf.head.w': s.mlp.linear_sdf.weight.grad,
         'sdf.head.b': s.mlp.linear_sdf.bias.grad, 's_var': model.s_var.grad}
    for i in range(2):
        lin = s.mlp.linears[i]
        g[f'sdf.l{i}.v'], g[f'sdf.l{i}.g'], g[f'sdf.l{i}.b'] = lin.weight_v.grad, lin.weight_g.grad, lin.bias.grad
    for i, lin in enumerate(model.neural_rgb.mlp.linears):
        g[f'rgb.l{i}.v'], g[f'rgb.l{i}.g'], g[f'rgb.l{i}.b'] = lin.weight_v.grad, lin.weight_g.grad, lin.bias.grad
    if model.appear_embed is not None:
        g['app'] = model.appear_embed.weight.grad
    if getattr(model, 'with_background', False):
        bgm = model.background_nerf
        for pre, lins in (('bg', bgm.mlp_feat.linears), ('bg.rgb', bgm.mlp_rgb.linears)):
            for i, lin in enumerate(lins):
                g[f'{pre}.l{i}.w'], g[f'{pre}.l{i}.b'] = lin.weight.grad, lin.bias.grad
        if model.appear_embed_outside is not None:
            g['app_bg'] = model.appear_embed_outside.weight.grad
    return {k: (v.detach().double().cpu() if v is not None else None) for k, v in g.items()}


def batch_to(batch, device, dtype=torch.float32):
    out = {}
    for k, v in batch.items():
        if v.dtype in (torch.float64, torch.float32):
            out[k] = v.to(device=device, dtype=dtype)
        else:
            out[k] = v.to(device)
    return out


def step_weight_copies(model):
    """The MLP weight copies exactly as the fused step forms them from the FP32 masters (weight
    norm and rounding in gbsdf_weightnorm_fwd, a deterministic kernel), or None when the model
    is not on a GPU or not a configuration the fused step takes."""
    if not next(model.parameters()).is_cuda:
        return None
    from neuralangelo_gb300.fused import FusedField
    try:
        ff = FusedField(model)
    except (ValueError, NotImplementedError):
        return None
    ff._pack()
    return ff.pk


class torch_rounded_weights:
    """Within this block, model_to_oracle rounds torch's own FP32 weights to fp16 instead of
    taking the step's copies: the other of two equally valid roundings of the same masters."""

    def __enter__(self):
        global step_weight_copies
        self._saved, step_weight_copies = step_weight_copies, (lambda model: None)
        return self

    def __exit__(self, *exc):
        global step_weight_copies
        step_weight_copies = self._saved
        return False


def model_to_oracle(model, fp16_weights=False, effective=False):
    """FieldModel parameters -> the oracle's float64 dict.  With fp16_weights the
    table and the MLP weight matrices are first rounded to fp16 the way the fused
    step uses them (weight norm applied in fp32, then rounded; biases, SDF head,
    s_var and the appearance table stay fp32): on a GPU the step's own copies, since
    an FP32 weight one bit off rounds to a neighbouring fp16 value now and then, and a
    ReLU gate can follow it."""
    s = model.neural_sdf
    p = {}
    pk = step_weight_copies(model) if fp16_weights else None

    def q(t):
        return t.detach().half().double().cpu() if fp16_weights else t.detach().double().cpu()

    p['table'] = q(s.tcnn_encoding.params)
    def vg(lin, W):
        if effective:
            return W.double().cpu(), None
        if fp16_weights:
            return W.double().cpu(), W.double().norm(dim=1, keepdim=True).cpu()
        return lin.weight_v.detach().double().cpu(), lin.weight_g.detach().double().cpu()

    for i in range(2):
        lin = s.mlp.linears[i]
        W = lin.weight.detach()
        if fp16_weights and i == 0:
            W = torch.cat([W[:, :3], W[:, 3:].half().float()], dim=1)    # position columns stay fp32
            if pk is not None:                  # the step's copies over the active columns
                n = s.active_levels * s.tcnn_encoding.layout.n_features
                W[:, :3] = pk['w0x']
                W[:, 3:3 + n] = pk['w0e'][:, :n].float()
        elif fp16_weights:
            W = pk['w1'].float() if pk is not None else W.half().float()
        p[f'sdf.l{i}.v'], p[f'sdf.l{i}.g'] = vg(lin, W)
        p[f'sdf.l{i}.b'] = lin.bias.detach().double().cpu()
    p['sdf.head.w'] = s.mlp.linear_sdf.weight.detach().double().cpu()
    p['sdf.head.b'] = s.mlp.linear_sdf.bias.detach().double().cpu()
    lins = model.neural_rgb.mlp.linears
    for i, lin in enumerate(lins):
        W = lin.weight.detach()
        if fp16_weights and pk is not None:
            if i == 0:                          # undo the step's column order [feat | x, SH, n, app | 0]
                wc0, sh, nt = pk['wc'][0].float(), 16, W.shape[1] - 256
                W = torch.cat([wc0[:, 256:256 + 6 + sh], wc0[:, :256], wc0[:, 256 + 6 + sh:256 + nt]], dim=1)
            elif i == len(lins) - 1:
                W = pk['wl'].clone()
            else:
                W = pk['wc'][i].float()
        elif fp16_weights and i != len(lins) - 1:
            W = W.half().float()
        p[f'rgb.l{i}.v'], p[f'rgb.l{i}.g'] = vg(lin, W)
        p[f'rgb.l{i}.b'] = lin.bias.detach().double().cpu()
    p['s_var'] = model.s_var.detach().double().cpu()
    if model.appear_embed is not None:
        p['app'] = model.appear_embed.weight.detach().double().cpu()
    if getattr(model, 'with_background', False):
        # the fused step rounds every background matrix to fp16 except the density row of
        # layer 7 and the colour head, which stay FP32
        bgm = model.background_nerf
        for pre, lins in (('bg', bgm.mlp_feat.linears), ('bg.rgb', bgm.mlp_rgb.linears)):
            for i, lin in enumerate(lins):
                W = lin.weight.detach()
                if fp16_weights:
                    if pre == 'bg' and i == len(lins) - 1:
                        W = torch.cat([W[:1], W[1:].half().float()], dim=0)
                    elif not (pre == 'bg.rgb' and i == len(lins) - 1):
                        W = W.half().float()
                p[f'{pre}.l{i}.w'] = W.double().cpu()
                p[f'{pre}.l{i}.b'] = lin.bias.detach().double().cpu()
        if model.appear_embed_outside is not None:
            p['app_bg'] = model.appear_embed_outside.weight.detach().double().cpu()
    return p
