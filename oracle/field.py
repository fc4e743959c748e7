"""float64 torch restatement of the neural-SDF field, NeuS rendering and losses.

TEST INFRASTRUCTURE ONLY -- the checker, never the product path.

Each function states the reference lines it follows.  Parameters travel as a
plain dict of tensors (layout described in ``init_params``); autograd in
float64 provides the reference gradients.  The hash-grid encoder is the numpy
restatement in ``oracle/hashgrid.py`` wrapped as an autograd function.
"""
import math

import numpy as np
import torch
import torch.nn.functional as F

from . import hashgrid as hg


# ---------------------------------------------------------------------------
# configuration (plain dict; mirrors projects/neuralangelo/configs/base.yaml:38-115)

def make_config(n_levels=16, n_features=8, log2_hashmap_size=22, base_resolution=32,
                per_level_scale=None, max_resolution=2048, active_levels=None,
                sdf_hidden=256, rgb_hidden=256, rgb_layers=4, app_dim=0, n_images=0,
                softplus_beta=100.0, out_bias=0.5, inside_out=False, s_var_init=3.0,
                anneal_end=0.1, taps=6, vol_range=(-2.0, 2.0), sh_levels=3, f32_positions=False,
                bg_enabled=False, bg_layers=8, bg_hidden=256, bg_skip=(4,), bg_layers_rgb=2, bg_hidden_rgb=128,
                bg_levels=10, bg_view_levels=3):
    if per_level_scale is None:
        # modules.py:39-41
        per_level_scale = float(np.exp((np.log(max_resolution) - np.log(base_resolution)) / (n_levels - 1)))
    return dict(n_levels=n_levels, n_features=n_features, log2_hashmap_size=log2_hashmap_size,
                base_resolution=base_resolution, per_level_scale=per_level_scale,
                active_levels=n_levels if active_levels is None else active_levels,
                sdf_hidden=sdf_hidden, rgb_hidden=rgb_hidden, rgb_layers=rgb_layers, app_dim=app_dim,
                n_images=n_images, softplus_beta=softplus_beta, out_bias=out_bias, inside_out=inside_out,
                s_var_init=s_var_init, anneal_end=anneal_end, taps=taps, vol_range=vol_range,
                sh_levels=sh_levels, f32_positions=f32_positions, bg_enabled=bg_enabled, bg_layers=bg_layers,
                bg_hidden=bg_hidden, bg_skip=tuple(bg_skip), bg_layers_rgb=bg_layers_rgb,
                bg_hidden_rgb=bg_hidden_rgb, bg_levels=bg_levels, bg_view_levels=bg_view_levels)


def eps_resolutions(cfg):
    """modules.py:52-54: resolutions[l] = floor(r_min * growth^l) + 1 (used only for eps)."""
    g = cfg['per_level_scale']
    return [int(np.floor(cfg['base_resolution'] * g ** lv).astype(int)) + 1 for lv in range(cfg['n_levels'])]


def normal_eps(cfg, anneal_levels):
    """modules.py:102-107: eps = 1 / resolutions[anneal_levels - 1]."""
    return 1.0 / eps_resolutions(cfg)[anneal_levels - 1]


# ---------------------------------------------------------------------------
# hash-grid encoder as a float64 autograd function

class _HashGridFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, table, layout, active):
        xn = x.detach().to(torch.float32).cpu().numpy()
        out = hg.encode(xn, table.detach().cpu().numpy(), layout, active)
        ctx.save_for_backward(x)
        ctx.layout, ctx.active, ctx.dtype = layout, active, table.dtype
        return torch.from_numpy(out).to(table.dtype)

    @staticmethod
    def backward(ctx, d_out):
        (x,) = ctx.saved_tensors
        g = hg.encode_backward(x.detach().to(torch.float32).cpu().numpy(),
                               d_out.detach().cpu().numpy(), ctx.layout, ctx.active)
        return None, torch.from_numpy(g.reshape(-1)).to(ctx.dtype), None, None


def hashgrid(x01, table, layout, active=None):
    """x01 [...,3] in [0,1] -> [..., L*F]; the table gradient flows, dx does not
    (numerical-gradient mode never asks for it)."""
    shp = x01.shape[:-1]
    out = _HashGridFn.apply(x01.reshape(-1, 3), table, layout, active)
    return out.reshape(*shp, out.shape[-1])


# ---------------------------------------------------------------------------
# parameters

def weight_norm(v, g):
    """torch.nn.utils.weight_norm(dim=0): W = g * v / ||v||_row (mlp.py:42-43, nerf_util.py:177-178).
    g = None takes v as the effective weight (gradients then are dL/dW)."""
    if g is None:
        return v
    return v * (g / v.norm(dim=1, keepdim=True))


def rgb_layer_dims(cfg):
    """modules.py:186-202: input = [x 3, SH 16, normal 3, feat, app] -> hidden*layers -> 3."""
    sh = (cfg['sh_levels'] + 1) ** 2
    d_in = 6 + sh + cfg['sdf_hidden'] + cfg['app_dim']
    return [d_in] + [cfg['rgb_hidden']] * cfg['rgb_layers'] + [3]


def init_params(cfg, seed=0, enc_perturb=1e-2, table_scale=1e-4, dtype=torch.float64):
    """Seeded parameters with the reference's initialisation.

    Geometric init (mlp.py:71-84) zeroes the encoding columns of SDF layer 0, so
    the table gradient would be exactly zero; a seeded N(0, enc_perturb) is
    added to those columns so table-gradient parity is meaningful.
    Layout (all float64 unless dtype says otherwise):
      table [n_entries*F] ~ U(-table_scale, table_scale)
      sdf.l0.{v,g,b}: v [H, 3+L*F]; sdf.l1.{v,g,b}: v [H,H]; sdf.head.{w,b}: w [1,H]
      rgb.l{i}.{v,g,b} for each colour layer; s_var (scalar); app [n_images, app_dim]
    """
    gen = torch.Generator().manual_seed(seed)
    L, Fd = cfg['n_levels'], cfg['n_features']
    layout = hg.level_layout(L, Fd, cfg['log2_hashmap_size'], cfg['base_resolution'], cfg['per_level_scale'])
    H = cfg['sdf_hidden']
    p = {}
    p['table'] = (torch.rand(layout['n_entries'] * Fd, generator=gen, dtype=torch.float64) * 2 - 1) * table_scale
    d0 = 3 + L * Fd
    # layer 0: N(0, sqrt(2/k_out)), encoding columns zero (mlp.py:72-75), then perturbed
    v0 = torch.randn(H, d0, generator=gen, dtype=torch.float64) * math.sqrt(2.0 / H)
    v0[:, 3:] = torch.randn(H, d0 - 3, generator=gen, dtype=torch.float64) * enc_perturb
    v1 = torch.randn(H, H, generator=gen, dtype=torch.float64) * math.sqrt(2.0 / H)
    for name, v in (('sdf.l0', v0), ('sdf.l1', v1)):
        p[name + '.v'] = v
        p[name + '.g'] = v.norm(dim=1, keepdim=True).clone()   # weight_norm init: g = ||v||
        p[name + '.b'] = torch.zeros(H, dtype=torch.float64)
    # SDF head: N(sqrt(pi/k_in), 1e-4), bias -out_bias (mlp.py:79-84)
    sgn = -1.0 if cfg['inside_out'] else 1.0
    p['sdf.head.w'] = sgn * (math.sqrt(math.pi / H) + 1e-4 * torch.randn(1, H, generator=gen, dtype=torch.float64))
    p['sdf.head.b'] = sgn * torch.full((1,), -cfg['out_bias'], dtype=torch.float64)
    dims = rgb_layer_dims(cfg)
    for i, (k_in, k_out) in enumerate(zip(dims[:-1], dims[1:])):
        bound = 1.0 / math.sqrt(k_in)                  # torch.nn.Linear default init
        v = (torch.rand(k_out, k_in, generator=gen, dtype=torch.float64) * 2 - 1) * bound
        b = (torch.rand(k_out, generator=gen, dtype=torch.float64) * 2 - 1) * bound
        if i == len(dims) - 2:
            b = torch.zeros_like(b)                    # nerf_util.py:182-183
        p[f'rgb.l{i}.v'] = v
        p[f'rgb.l{i}.g'] = v.norm(dim=1, keepdim=True).clone()
        p[f'rgb.l{i}.b'] = b
    p['s_var'] = torch.tensor(cfg['s_var_init'], dtype=torch.float64)
    if cfg['app_dim'] > 0:
        p['app'] = torch.randn(cfg['n_images'], cfg['app_dim'], generator=gen, dtype=torch.float64)
    if cfg.get('bg_enabled'):
        # BackgroundNeRF (modules.py:232-266): torch.nn.Linear default init, no weight
        # norm, last-layer biases zero (nerf_util.py:182-183)
        for pre, dims, skip in (('bg', bg_feat_dims(cfg), cfg['bg_skip']), ('bg.rgb', bg_rgb_dims(cfg), ())):
            for i, (k_in, k_out) in enumerate(zip(dims[:-1], dims[1:])):
                k_in = k_in + (dims[0] if i in skip else 0)
                bound = 1.0 / math.sqrt(k_in)
                p[f'{pre}.l{i}.w'] = (torch.rand(k_out, k_in, generator=gen, dtype=torch.float64) * 2 - 1) * bound
                b = (torch.rand(k_out, generator=gen, dtype=torch.float64) * 2 - 1) * bound
                p[f'{pre}.l{i}.b'] = torch.zeros_like(b) if i == len(dims) - 2 else b
        if cfg['app_dim'] > 0:
            p['app_bg'] = torch.randn(cfg['n_images'], cfg['app_dim'], generator=gen, dtype=torch.float64)
    return {k: v.to(dtype) for k, v in p.items()}, layout


def bg_feat_dims(cfg):
    """BackgroundNeRF.build_mlp (modules.py:258-261): [4 + 8 L] + [H] * (layers - 1) + [H + 1]."""
    return [4 + 8 * cfg['bg_levels']] + [cfg['bg_hidden']] * (cfg['bg_layers'] - 1) + [cfg['bg_hidden'] + 1]


def bg_rgb_dims(cfg):
    """modules.py:238-240, 263-264: [H + SH + app] + [H_rgb] * (layers_rgb - 1) + [3]."""
    d_in = cfg['bg_hidden'] + (cfg['bg_view_levels'] + 1) ** 2 + cfg['app_dim']
    return [d_in] + [cfg['bg_hidden_rgb']] * (cfg['bg_layers_rgb'] - 1) + [3]


def positional_encoding(x, num_freq_bases):
    """nerf_util.py:134-147; the frequencies 2^k pi are float32 as the reference builds them."""
    freq = (2 ** torch.arange(num_freq_bases, dtype=torch.float32) * np.pi).to(x.dtype)
    spectrum = x[..., None] * freq
    enc = torch.stack([spectrum.sin(), spectrum.cos()], dim=-2)
    return enc.reshape(*x.shape[:-1], -1)


def bg_encode(cfg, pts):
    """BackgroundNeRF.encode (modules.py:286-301): [x/|x|, 1/|x|] and its Fourier code."""
    norm = pts.norm(dim=-1, keepdim=True)
    q = torch.cat([pts / norm, 1.0 / norm], dim=-1)
    return torch.cat([q, positional_encoding(q, cfg['bg_levels'])], dim=-1)


def background(p, cfg, pts, rays_unit, app_out=None):
    """BackgroundNeRF.forward (modules.py:268-284) -> (rgb [...,3], density [...])."""
    x = bg_encode(cfg, pts)
    h = x
    n = cfg['bg_layers']
    for i in range(n):                                        # MLPwithSkipConnection (nerf_util.py:187-196)
        if i in cfg['bg_skip']:
            h = torch.cat([h, x], dim=-1)
        h = h @ p[f'bg.l{i}.w'].t() + p[f'bg.l{i}.b']
        if i != n - 1:
            h = torch.relu(h)
    density, feat = F.softplus(h[..., 0]), torch.relu(h[..., 1:])
    parts = [feat, spherical_harmonics(rays_unit)]
    if app_out is not None:
        parts.append(app_out)
    g = torch.cat(parts, dim=-1)
    m = cfg['bg_layers_rgb']
    for i in range(m):
        g = g @ p[f'bg.rgb.l{i}.w'].t() + p[f'bg.rgb.l{i}.b']
        if i != m - 1:
            g = torch.relu(g)
    return torch.sigmoid(g), density


def volume_alphas(density, dists, dist_far=1e10):
    """render.py:68-84: 1 - exp(-density * interval), the last interval to dist_far."""
    d = torch.cat([dists, torch.full_like(dists[..., :1], dist_far)], dim=-1)
    return 1 - torch.exp(-(density * (d[..., 1:] - d[..., :-1])))


def background_branch(p, cfg, center, ray_unit, dists_bg, app_idx=None):
    """Model.render_rays_background (model.py:192-205) on precomputed distances
    (sample_dists_background, model.py:269-273): (rgbs [R,Nb,3], alphas [R,Nb])."""
    pts = center[:, None, :] + ray_unit[:, None, :] * dists_bg[..., None]
    rays = ray_unit[:, None, :].expand_as(pts)
    app_out = None
    if cfg['app_dim'] > 0 and 'app_bg' in p:
        app_out = p['app_bg'][app_idx][:, None, :].expand(pts.shape[0], pts.shape[1], cfg['app_dim'])
    rgbs, dens = background(p, cfg, pts, rays, app_out)
    return rgbs, volume_alphas(dens, dists_bg)


# ---------------------------------------------------------------------------
# field

def softplus(x, beta):
    """torch.nn.functional.softplus(beta, threshold=20) (misc.py:92-107 via base.yaml:46-48)."""
    return F.softplus(x, beta=beta)


def fp16_store(t, on):
    """Forward value rounded to fp16 with an identity gradient: emulates where the fused
    FP16 kernels store an activation in fp16 (used only with fp16_storage=True)."""
    if not on:
        return t
    return t + (t.detach().half().to(t.dtype) - t.detach())


def sdf_mlp(p, cfg, enc_in, with_feat):
    """MLPforNeuralSDF.forward (mlp.py:55-69) for layer_dims [3+LF, H, H]:
    h0 = softplus(W0 in + b0); sdf = w_head h0 + b_head; feat = softplus(W1 h0 + b1)."""
    beta = cfg['softplus_beta']
    W0 = weight_norm(p['sdf.l0.v'], p['sdf.l0.g'])
    h0 = softplus(enc_in @ W0.t() + p['sdf.l0.b'], beta)
    sdf = h0 @ p['sdf.head.w'].t() + p['sdf.head.b']
    feat = None
    if with_feat:
        W1 = weight_norm(p['sdf.l1.v'], p['sdf.l1.g'])
        st = cfg.get('fp16_storage', False)
        feat = softplus(fp16_store(h0, st) @ W1.t() + p['sdf.l1.b'], beta)
    return sdf, feat


def encode(p, cfg, layout, pts):
    """NeuralSDF.encode (modules.py:76-95): normalise by the volume range, hash-grid,
    coarse-to-fine mask (implemented by not evaluating masked levels), cat [x, enc]."""
    vmin, vmax = cfg['vol_range']
    x01 = (pts - vmin) / (vmax - vmin)
    enc = hashgrid(x01, p['table'], layout, cfg['active_levels'])
    return torch.cat([pts, enc], dim=-1)


def neural_sdf(p, cfg, layout, pts, with_feat=True):
    return sdf_mlp(p, cfg, encode(p, cfg, layout, pts), with_feat)


def tap_offsets(cfg, eps):
    """Tap displacement vectors, modules.py:134-143 (6 taps) / :158-166 (4 taps)."""
    if cfg['taps'] == 6:
        return [(eps, 0, 0), (-eps, 0, 0), (0, eps, 0), (0, -eps, 0), (0, 0, eps), (0, 0, -eps)]
    e = eps / np.sqrt(3)
    return [(e, -e, -e), (-e, -e, e), (-e, e, -e), (e, e, e)]


def compute_gradients(p, cfg, layout, pts, eps, sdf_centre, training=True):
    """NeuralSDF.compute_gradients, numerical mode (modules.py:131-178).

    6 taps: g_i = (f(x+e_i) - f(x-e_i)) / 2eps; H_ii = (f+ + f- - 2 sdf) / eps^2
    where sdf is the caller's (post-overwrite) centre value (model.py:163-166).
    """
    dt = pts.dtype
    f32 = cfg.get('f32_positions', False)

    def shifted(k, sign):
        # the tap point x + sign * k, formed in float32 like the reference's float32
        # tensors (modules.py:135-143) when f32_positions, else in the oracle's dtype
        if f32:
            return (pts.float() + sign * k.float()).to(dt)
        return pts + sign * k

    if cfg['taps'] == 6:
        fs = []
        for d in range(3):
            e = torch.zeros(3, dtype=dt)
            e[d] = eps
            fs.append((neural_sdf(p, cfg, layout, shifted(e, 1), False)[0],
                       neural_sdf(p, cfg, layout, shifted(e, -1), False)[0]))
        grad = torch.cat([(fp - fm) / (2 * eps) for fp, fm in fs], dim=-1)
        hess = torch.cat([(fp + fm - 2 * sdf_centre) / (eps ** 2) for fp, fm in fs], dim=-1) if training else None
        return grad, hess
    e = eps / np.sqrt(3)
    ks = [torch.tensor(k, dtype=dt) for k in ((1, -1, -1), (-1, -1, 1), (-1, 1, -1), (1, 1, 1))]
    sd = [neural_sdf(p, cfg, layout, shifted(k * e, 1), False)[0] for k in ks]
    grad = sum(k * s for k, s in zip(ks, sd)) / (4.0 * e)
    hess = None
    if training:
        hxx = ((sd[0] + sd[1] + sd[2] + sd[3]) / 2.0 - 2 * sdf_centre) / e ** 2
        hess = torch.cat([hxx, hxx, hxx], dim=-1) / 3.0
    return grad, hess


_SH_C0 = 0.28209479177387814
_SH_C1 = 0.4886025119029199
_SH_C2 = (1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792, 0.5462742152960396)
_SH_C3 = (-0.5900435899266435, 2.890611442640554, -0.4570457994644658, 0.3731763325901154,
          -0.4570457994644658, 1.445305721320277, -0.5900435899266435)


def spherical_harmonics(d):
    """Degree-3 real SH basis (projects/neuralangelo/utils/spherical_harmonics.py:47-84).
    The coefficients are the standard real-SH normalisation constants.  The
    reference stores the basis in a tensor of the default dtype (float32,
    spherical_harmonics.py:49), so each value is rounded to float32 once."""
    x, y, z = d.unbind(-1)
    xx, yy, zz = x * x, y * y, z * z
    xy, yz, xz = x * y, y * z, x * z
    return torch.stack([
        torch.full_like(x, _SH_C0),
        -_SH_C1 * y, _SH_C1 * z, -_SH_C1 * x,
        _SH_C2[0] * xy, _SH_C2[1] * yz, _SH_C2[2] * (2.0 * zz - xx - yy), _SH_C2[3] * xz, _SH_C2[4] * (xx - yy),
        _SH_C3[0] * y * (3 * xx - yy), _SH_C3[1] * xy * z, _SH_C3[2] * y * (4 * zz - xx - yy),
        _SH_C3[3] * z * (2 * zz - 3 * xx - 3 * yy), _SH_C3[4] * x * (4 * zz - xx - yy),
        _SH_C3[5] * z * (xx - yy), _SH_C3[6] * x * (xx - 3 * yy)], dim=-1).to(torch.float32).to(d.dtype)


def neural_rgb(p, cfg, pts, normals, rays_unit, feats, app, gates=None):
    """NeuralRGB.forward (modules.py:209-220) with MLPwithSkipConnection (nerf_util.py:187-196):
    input [x, SH(d), n, feat, app], ReLU hidden layers, sigmoid output.

    gates (test diagnostics only): per hidden layer a {0, 1} tensor shaped like its output,
    used in place of the ReLU's own [h > 0].  A pre-activation within rounding of zero takes
    either side in two valid computations; feeding the gates another computation took
    compares the rest of the arithmetic across that discontinuity."""
    st = cfg.get('fp16_storage', False)
    parts = [pts, spherical_harmonics(rays_unit), normals, feats]
    if app is not None:
        parts.append(app)
    h = fp16_store(torch.cat(parts, dim=-1), st)
    n = cfg['rgb_layers'] + 1
    for i in range(n):
        W = weight_norm(p[f'rgb.l{i}.v'], p[f'rgb.l{i}.g'])
        h = h @ W.t() + p[f'rgb.l{i}.b']
        if i != n - 1:
            h = fp16_store(h * gates[i].to(h.dtype) if gates is not None else torch.relu(h), st)
    return torch.sigmoid(h)


# ---------------------------------------------------------------------------
# rendering

def intersect_with_sphere(center, ray_unit, radius=1.0):
    """nerf_util.py:199-205."""
    ctc = (center * center).sum(dim=-1, keepdim=True)
    ctv = (center * ray_unit).sum(dim=-1, keepdim=True)
    b2_minus_4ac = ctv ** 2 - (ctc - radius ** 2)
    return -ctv - b2_minus_4ac.sqrt(), -ctv + b2_minus_4ac.sqrt()


def dist_bounds(center, ray_unit):
    """Model.get_dist_bounds (model.py:207-213): near.relu_(); misses get near=1, far=1.2."""
    near, far = intersect_with_sphere(center, ray_unit)
    near = near.clamp(min=0)
    outside = near.isnan()
    near = torch.where(outside, torch.ones_like(near), near)
    far = torch.where(outside, torch.full_like(far, 1.2), far)
    return near, far, outside


def iter_cos(true_cos, progress, anneal_end):
    """Model._get_iter_cos (model.py:294-298)."""
    a = min(progress / anneal_end, 1.0)
    return -(torch.relu(-true_cos * 0.5 + 0.5) * (1.0 - a) + torch.relu(-true_cos) * a)


def neus_alphas(ray_unit, sdfs, grads, dists, far, s_var, progress, anneal_end, eps=1e-5):
    """Model.compute_neus_alphas (model.py:275-292).
    ray_unit [R,3], sdfs [R,N], grads [R,N,3], dists [R,N], far [R,1] -> alphas [R,N]."""
    inv_s = s_var.exp()
    true_cos = (ray_unit[:, None, :] * grads).sum(dim=-1)
    ic = iter_cos(true_cos, progress, anneal_end)
    d = torch.cat([dists, far], dim=1)
    intv = d[:, 1:] - d[:, :-1]
    est_prev = sdfs - ic * intv * 0.5
    est_next = sdfs + ic * intv * 0.5
    prev_cdf = torch.sigmoid(est_prev * inv_s)
    next_cdf = torch.sigmoid(est_next * inv_s)
    return ((prev_cdf - next_cdf) / (prev_cdf + eps)).clamp(0.0, 1.0)


def compositing_weights(alphas):
    """render.alpha_compositing_weights (render.py:87-99): w_i = a_i * prod_{j<i}(1 - a_j)."""
    front = torch.cat([torch.zeros_like(alphas[:, :1]), alphas[:, :-1]], dim=1)
    return alphas * torch.cumprod(1 - front, dim=1)


def eikonal_loss(grads, outside):
    """misc.py:74-80 (mean over every sample, outside rays contribute 0)."""
    err = ((grads.norm(dim=-1) - 1.0) ** 2).nan_to_num(nan=0.0, posinf=0.0, neginf=0.0)
    return (err * (~outside).to(err.dtype)).mean()


def curvature_loss(hess, outside):
    """misc.py:83-89."""
    lap = hess.sum(dim=-1).abs().nan_to_num(nan=0.0, posinf=0.0, neginf=0.0)
    return (lap * (~outside).to(lap.dtype)).mean()


def render_step(p, cfg, layout, batch, eps, progress, w_eik, w_curv, training=True, retain=False):
    """One training forward of Model.render_rays_object + render_rays + Trainer._compute_loss
    (model.py:124-190, trainer.py:40-52), with the background NeRF's samples composited
    after the object's (model.py:129-134) when cfg['bg_enabled'] and batch['dists_bg'].

    batch: center [R,3], ray_unit [R,3], dists [R,N], far [R,1], outside [R,1] (bool),
           target [R,3], app_idx [R] (or None).  Returns a dict of outputs incl. 'loss'.
    """
    c, d, dists = batch['center'], batch['ray_unit'], batch['dists']
    R, N = dists.shape
    pts = c[:, None, :] + d[:, None, :] * dists[..., None]                # camera.py:314-320
    if cfg.get('f32_positions', False):   # the points as the reference's float32 tensors hold them
        pts = (c.float()[:, None, :] + d.float()[:, None, :] * dists.float()[..., None]).to(c.dtype)
    sdf, feat = neural_sdf(p, cfg, layout, pts, with_feat=True)
    outside = batch['outside']
    out_val = 1000.0 * (-1 if cfg['inside_out'] else 1)                   # model.py:33
    sdf = torch.where(outside[:, None, :].expand_as(sdf), torch.full_like(sdf, out_val), sdf)  # model.py:163
    grads, hess = compute_gradients(p, cfg, layout, pts, eps, sdf, training)
    normals = F.normalize(grads, dim=-1)
    if retain:   # expose intermediate gradients for diagnostics
        for t in (sdf, feat, grads, hess, normals):
            t.retain_grad()
    rays = d[:, None, :].expand_as(pts)
    app = None
    if cfg['app_dim'] > 0:
        app = p['app'][batch['app_idx']][:, None, :].expand(R, N, cfg['app_dim'])
    gates = batch.get('rgb_gates')
    if gates is not None:
        gates = [g.reshape(R, N, -1) for g in gates]
    rgbs = neural_rgb(p, cfg, pts, normals, rays, feat, app, gates)
    alphas = neus_alphas(d, sdf[..., 0], grads, dists, batch['far'], p['s_var'], progress, cfg['anneal_end'])
    rgbs_all, alphas_all = rgbs, alphas
    if cfg.get('bg_enabled') and batch.get('dists_bg') is not None:     # model.py:129-134
        rgbs_bg, alphas_bg = background_branch(p, cfg, c, d, batch['dists_bg'], batch.get('app_idx'))
        rgbs_all = torch.cat([rgbs, rgbs_bg], dim=1)
        alphas_all = torch.cat([alphas, alphas_bg], dim=1)
    weights = compositing_weights(alphas_all)
    rgb = (rgbs_all * weights[..., None]).sum(dim=1)
    weights = weights[:, :N]
    l_render = (rgb - batch['target']).abs().mean() * 3.0                  # trainer.py:43
    out_mask = outside.expand(R, N)
    l_eik = eikonal_loss(grads, out_mask)
    loss = l_render + w_eik * l_eik
    l_curv = None
    if hess is not None and w_curv:
        l_curv = curvature_loss(hess, out_mask)
        loss = loss + w_curv * l_curv
    return dict(loss=loss, l_render=l_render, l_eik=l_eik, l_curv=l_curv, rgb=rgb, rgbs=rgbs,
                sdf=sdf[..., 0], feat=feat, grads=grads, hess=hess, alphas=alphas, weights=weights,
                normals=normals, sdf_full=sdf)


def render_step_ragged(p, cfg, layout, batch, eps, progress, w_eik, w_curv, mean_count=None):
    """render_step on a ragged batch: ray r owns the flat samples [ray_offsets[r],
    ray_offsets[r+1]) of ``dists`` [Ns] (the ray-major layout of the reference's
    [B, R, N] tensors with per-ray N).  Each ray is rendered exactly as
    render_rays_object + render_rays do for its own samples (model.py:124-190); a ray
    without samples composites to 0.  The loss keeps the reference's composition
    (trainer.py:40-52): L1 x 3 averaged over rays and channels, eikonal and curvature
    summed over every sample and divided by ``mean_count`` (the number of samples the
    reference's mean runs over: Ns by default, R x N for a padded batch).
    Rays with the same count are evaluated together."""
    offs = batch['ray_offsets']
    counts = (offs[1:] - offs[:-1]).tolist()
    R = len(counts)
    Ns = int(offs[-1])
    mean_count = Ns if mean_count is None else mean_count
    dt = batch['center'].dtype
    rgb_rows = [None] * R
    eik_sum = torch.zeros((), dtype=dt)
    curv_sum = torch.zeros((), dtype=dt)
    sdf_flat = [None] * R
    for n in sorted(set(counts)):
        rays = [r for r in range(R) if counts[r] == n]
        if n == 0:
            for r in rays:
                rgb_rows[r] = torch.zeros(3, dtype=dt)
                sdf_flat[r] = torch.zeros(0, dtype=dt)
            if cfg.get('bg_enabled') and batch.get('dists_bg') is not None:
                idx = torch.tensor(rays)
                rgbs_bg, alphas_bg = background_branch(
                    p, cfg, batch['center'][idx], batch['ray_unit'][idx], batch['dists_bg'][idx],
                    batch['app_idx'][idx] if batch.get('app_idx') is not None else None)
                rgb0 = (rgbs_bg * compositing_weights(alphas_bg)[..., None]).sum(dim=1)
                for j, r in enumerate(rays):
                    rgb_rows[r] = rgb0[j]
            continue
        idx = torch.tensor(rays)
        d = torch.stack([batch['dists'][offs[r]:offs[r + 1]] for r in rays])
        gates = None
        if batch.get('rgb_gates') is not None:          # flat per-sample rows -> this group's rays
            rows = torch.cat([torch.arange(int(offs[r]), int(offs[r + 1])) for r in rays])
            gates = [g[rows] for g in batch['rgb_gates']]
        sub = dict(center=batch['center'][idx], ray_unit=batch['ray_unit'][idx], dists=d,
                   far=batch['far'][idx], outside=batch['outside'][idx], target=batch['target'][idx],
                   app_idx=batch['app_idx'][idx] if batch.get('app_idx') is not None else None,
                   dists_bg=batch['dists_bg'][idx] if batch.get('dists_bg') is not None else None,
                   rgb_gates=gates)
        out = render_step(p, cfg, layout, sub, eps, progress, w_eik, w_curv)
        ins = (~sub['outside']).to(dt).expand(len(rays), n)
        eik = ((out['grads'].norm(dim=-1) - 1.0) ** 2).nan_to_num(nan=0.0, posinf=0.0, neginf=0.0)
        eik_sum = eik_sum + (eik * ins).sum()
        if out['hess'] is not None:
            lap = out['hess'].sum(dim=-1).abs().nan_to_num(nan=0.0, posinf=0.0, neginf=0.0)
            curv_sum = curv_sum + (lap * ins).sum()
        for j, r in enumerate(rays):
            rgb_rows[r] = out['rgb'][j]
            sdf_flat[r] = out['sdf'][j]
    rgb = torch.stack(rgb_rows)
    l_render = (rgb - batch['target']).abs().mean() * 3.0
    l_eik = eik_sum / mean_count
    l_curv = curv_sum / mean_count
    loss = l_render + w_eik * l_eik
    if w_curv:
        loss = loss + w_curv * l_curv
    return dict(loss=loss, l_render=l_render, l_eik=l_eik, l_curv=l_curv, rgb=rgb, sdf=torch.cat(sdf_flat))


def render_eval(p, cfg, layout, batch, eps, progress):
    """Model.render_rays + render_image with training off (model.py:90-114, 158-190):
    rgb over object and background samples, opacity and the gradient composite over the
    object samples' own weights, and the distance composite over all samples."""
    c, d, dists = batch['center'], batch['ray_unit'], batch['dists']
    R, N = dists.shape
    pts = c[:, None, :] + d[:, None, :] * dists[..., None]
    sdf, feat = neural_sdf(p, cfg, layout, pts, with_feat=True)
    out_val = 1000.0 * (-1 if cfg['inside_out'] else 1)
    sdf = torch.where(batch['outside'][:, None, :].expand_as(sdf), torch.full_like(sdf, out_val), sdf)
    grads, _ = compute_gradients(p, cfg, layout, pts, eps, sdf, training=False)
    normals = F.normalize(grads, dim=-1)
    app = None
    if cfg['app_dim'] > 0:
        app = p['app'][batch['app_idx']][:, None, :].expand(R, N, cfg['app_dim'])
    rgbs = neural_rgb(p, cfg, pts, normals, d[:, None, :].expand_as(pts), feat, app)
    alphas = neus_alphas(d, sdf[..., 0], grads, dists, batch['far'], p['s_var'], progress, cfg['anneal_end'])
    w_obj = compositing_weights(alphas)
    opacity = w_obj.sum(dim=1, keepdim=True)
    gradient = (grads * w_obj[..., None]).sum(dim=1)
    rgbs_all, alphas_all, dists_all = rgbs, alphas, dists
    if cfg.get('bg_enabled') and batch.get('dists_bg') is not None:
        rgbs_bg, alphas_bg = background_branch(p, cfg, c, d, batch['dists_bg'], batch.get('app_idx'))
        rgbs_all = torch.cat([rgbs, rgbs_bg], dim=1)
        alphas_all = torch.cat([alphas, alphas_bg], dim=1)
        dists_all = torch.cat([dists, batch['dists_bg']], dim=1)
    w = compositing_weights(alphas_all)
    return dict(rgb=(rgbs_all * w[..., None]).sum(dim=1), opacity=opacity, gradient=gradient,
                dist=(dists_all * w).sum(dim=1, keepdim=True), normals=normals, feat=feat)
