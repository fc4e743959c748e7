"""NeuralSDF / NeuralRGB with the reference's call surface (plain FP32 drop-in path).

Follows projects/neuralangelo/utils/modules.py:24-229, utils/mlp.py:18-84 and
projects/nerf/utils/nerf_util.py:158-196.  Parameter names match the
reference's state dict (``tcnn_encoding.params``, ``mlp.linears.{i}.weight_g /
weight_v / bias``, ``mlp.linear_sdf.*``) so reference checkpoints load.  The
hash grid runs on the libgbsdf CUDA kernels; the linear layers are torch
matmuls exactly as in the reference.
"""
import math
from functools import partial

import numpy as np
import torch
import torch.nn.functional as torch_F

from .config import growth_rate
from .encoding import HashGridEncoding


class WeightNormLinear(torch.nn.Module):
    """Linear layer with the reparametrisation of torch.nn.utils.weight_norm(dim=0):
    W = g * v / ||v||_row (mlp.py:42-43, nerf_util.py:177-178)."""

    def __init__(self, linear):
        super().__init__()
        self.in_features, self.out_features = linear.in_features, linear.out_features
        w = linear.weight.detach()
        self.weight_g = torch.nn.Parameter(w.norm(dim=1, keepdim=True).clone())
        self.weight_v = torch.nn.Parameter(w.clone())
        self.bias = torch.nn.Parameter(linear.bias.detach().clone())

    @property
    def weight(self):
        return self.weight_v * (self.weight_g / self.weight_v.norm(dim=1, keepdim=True))

    def forward(self, x):
        return torch_F.linear(x, self.weight, self.bias)


def get_activation(activ, **kwargs):
    """misc.py:92-107."""
    func = dict(identity=lambda x: x, relu=torch_F.relu, relu_=torch_F.relu_, softplus=torch_F.softplus,
                sigmoid=torch.sigmoid, abs=torch.abs, exp=torch.exp, silu=torch_F.silu)[activ]
    return partial(func, **kwargs)


class MLPforNeuralSDF(torch.nn.Module):
    """mlp.py:18-84: hidden layers, SDF head fed by the penultimate activation,
    geometric init (sphere of radius out_bias), weight norm on the hidden layers only."""

    def __init__(self, layer_dims, skip_connection=(), activ=None, use_weightnorm=False, geometric_init=False,
                 out_bias=0.0, invert=False):
        super().__init__()
        self.skip_connection = list(skip_connection)
        self.linears = torch.nn.ModuleList()
        pairs = list(zip(layer_dims[:-1], layer_dims[1:]))
        for li, (k_in, k_out) in enumerate(pairs):
            if li in self.skip_connection:
                k_in += layer_dims[0]
            linear = torch.nn.Linear(k_in, k_out)
            if geometric_init:
                self._geometric_init(linear, k_out, first=(li == 0),
                                     skip_dim=(layer_dims[0] if li in self.skip_connection else 0))
            if li == len(pairs) - 1:
                linear.bias.data.fill_(0.0)
            self.linears.append(WeightNormLinear(linear) if use_weightnorm else linear)
        self.linear_sdf = torch.nn.Linear(k_in, 1)
        if geometric_init:
            torch.nn.init.normal_(self.linear_sdf.weight, mean=np.sqrt(np.pi / k_in), std=0.0001)
            torch.nn.init.constant_(self.linear_sdf.bias, -out_bias)
            if invert:
                self.linear_sdf.weight.data *= -1
                self.linear_sdf.bias.data *= -1
        self.activ = activ or torch_F.relu_

    @staticmethod
    def _geometric_init(linear, k_out, first=False, skip_dim=0):
        torch.nn.init.constant_(linear.bias, 0.0)
        torch.nn.init.normal_(linear.weight, 0.0, np.sqrt(2 / k_out))
        if first:
            torch.nn.init.constant_(linear.weight[:, 3:], 0.0)
        if skip_dim:
            torch.nn.init.constant_(linear.weight[:, -skip_dim:], 0.0)

    def forward(self, inp, with_sdf=True, with_feat=True):
        feat = inp
        out = None
        n = len(self.linears)
        for li, linear in enumerate(self.linears):
            if li in self.skip_connection:
                feat = torch.cat([feat, inp], dim=-1)
            if li != n - 1 or with_feat:
                feat_activ = self.activ(linear(feat))
            if li == n - 1:
                out = [self.linear_sdf(feat) if with_sdf else None, feat_activ if with_feat else None]
            feat = feat_activ
        return out


class MLPwithSkipConnection(torch.nn.Module):
    """nerf_util.py:158-196 (the colour MLP); last-layer bias zeroed at init."""

    def __init__(self, layer_dims, skip_connection=(), activ=None, use_weightnorm=False):
        super().__init__()
        self.skip_connection = list(skip_connection)
        self.linears = torch.nn.ModuleList()
        pairs = list(zip(layer_dims[:-1], layer_dims[1:]))
        for li, (k_in, k_out) in enumerate(pairs):
            if li in self.skip_connection:
                k_in += layer_dims[0]
            linear = torch.nn.Linear(k_in, k_out)
            if li == len(pairs) - 1:
                linear.bias.data.fill_(0.0)
            self.linears.append(WeightNormLinear(linear) if use_weightnorm else linear)
        self.activ = activ or torch_F.relu_

    def forward(self, inp):
        feat = inp
        for li, linear in enumerate(self.linears):
            if li in self.skip_connection:
                feat = torch.cat([feat, inp], dim=-1)
            feat = linear(feat)
            if li != len(self.linears) - 1:
                feat = self.activ(feat)
        return feat


SH_C0 = 0.28209479177387814
SH_C1 = 0.4886025119029199
SH_C2 = (1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792, 0.5462742152960396)
SH_C3 = (-0.5900435899266435, 2.890611442640554, -0.4570457994644658, 0.3731763325901154, -0.4570457994644658,
         1.445305721320277, -0.5900435899266435)


def get_spherical_harmonics(dirs, levels=3):
    """Real SH basis up to degree 3 (spherical_harmonics.py:47-84); float32 output like the reference."""
    if levels > 3:
        raise NotImplementedError("SH degree > 3")
    x, y, z = dirs.unbind(-1)
    vals = [torch.full_like(x, SH_C0)]
    if levels >= 1:
        vals += [-SH_C1 * y, SH_C1 * z, -SH_C1 * x]
    if levels >= 2:
        xx, yy, zz, xy, yz, xz = x * x, y * y, z * z, x * y, y * z, x * z
        vals += [SH_C2[0] * xy, SH_C2[1] * yz, SH_C2[2] * (2.0 * zz - xx - yy), SH_C2[3] * xz,
                 SH_C2[4] * (xx - yy)]
    if levels >= 3:
        vals += [SH_C3[0] * y * (3 * xx - yy), SH_C3[1] * xy * z, SH_C3[2] * y * (4 * zz - xx - yy),
                 SH_C3[3] * z * (2 * zz - 3 * xx - 3 * yy), SH_C3[4] * x * (4 * zz - xx - yy),
                 SH_C3[5] * z * (xx - yy), SH_C3[6] * x * (xx - 3 * yy)]
    return torch.stack(vals, dim=-1).float()


class NeuralSDF(torch.nn.Module):
    """modules.py:24-178 with the hash grid on libgbsdf (``tcnn_encoding``)."""

    def __init__(self, cfg_sdf, table_dtype=torch.float32):
        super().__init__()
        self.cfg_sdf = cfg_sdf
        enc = cfg_sdf.encoding
        assert enc.type == "hashgrid", "only the hash-grid encoding is on this path"
        hg = enc.hashgrid
        L = enc.levels
        self.growth_rate = growth_rate(cfg_sdf)
        r_min = 2 ** hg.min_logres
        config = dict(otype="HashGrid", n_levels=L, n_features_per_level=hg.dim, log2_hashmap_size=hg.dict_size,
                      base_resolution=r_min, per_level_scale=self.growth_rate)
        self.tcnn_encoding = HashGridEncoding(3, config, dtype=table_dtype)
        # modules.py:52-54 -- used only for the numerical-gradient step
        self.resolutions = [int(np.floor(r_min * self.growth_rate ** lv).astype(int)) + 1 for lv in range(L)]
        input_dim = 3 + hg.dim * L
        m = cfg_sdf.mlp
        dims = [input_dim] + [m.hidden_dim] * m.num_layers + [m.hidden_dim]
        self.mlp = MLPforNeuralSDF(dims, skip_connection=m.skip, activ=get_activation(m.activ, **m.activ_params),
                                   use_weightnorm=m.weight_norm, geometric_init=m.geometric_init,
                                   out_bias=m.out_bias, invert=m.inside_out)
        self.warm_up_end = 0
        self.active_levels = L
        self.anneal_levels = L
        self.normal_eps = 1.0 / self.resolutions[-1]

    def forward(self, points_3D, with_sdf=True, with_feat=True):
        return self.mlp(self.encode(points_3D), with_sdf=with_sdf, with_feat=with_feat)

    def sdf(self, points_3D):
        return self.forward(points_3D, with_sdf=True, with_feat=False)[0]

    def encode(self, points_3D):
        vmin, vmax = self.cfg_sdf.encoding.hashgrid.range
        x01 = (points_3D - vmin) / (vmax - vmin)
        self.tcnn_encoding.active_levels = self.active_levels if self.cfg_sdf.encoding.coarse2fine.enabled \
            else self.tcnn_encoding.layout.n_levels
        # levels >= active_levels come back as exact zeros: the coarse-to-fine mask of modules.py:91-93
        enc = self.tcnn_encoding(x01)
        return torch.cat([points_3D, enc.to(points_3D.dtype)], dim=-1)

    def set_active_levels(self, current_iter=None):
        """modules.py:97-100."""
        c2f = self.cfg_sdf.encoding.coarse2fine
        anneal = max((current_iter - self.warm_up_end) // c2f.step, 1)
        self.anneal_levels = min(self.cfg_sdf.encoding.levels, anneal)
        self.active_levels = max(c2f.init_active_level, self.anneal_levels)

    def set_normal_epsilon(self):
        """modules.py:102-107 (uses anneal_levels, not active_levels)."""
        if self.cfg_sdf.encoding.coarse2fine.enabled:
            self.normal_eps = 1.0 / self.resolutions[self.anneal_levels - 1]
        else:
            self.normal_eps = 1.0 / self.resolutions[-1]

    def compute_gradients(self, x, training=False, sdf=None):
        """Numerical gradients, modules.py:131-178 (6 or 4 taps)."""
        taps = self.cfg_sdf.gradient.taps
        if self.cfg_sdf.gradient.mode != "numerical":
            raise NotImplementedError("analytical gradients are outside this path")
        if taps == 6:
            eps = self.normal_eps
            fs = []
            for d in range(3):
                e = torch.zeros(3, dtype=x.dtype, device=x.device)
                e[d] = eps
                fs.append((self.sdf(x + e), self.sdf(x - e)))
            gradient = torch.cat([(fp - fm) / (2 * eps) for fp, fm in fs], dim=-1)
            hessian = None
            if training:
                assert sdf is not None
                hessian = torch.cat([(fp + fm - 2 * sdf) / (eps ** 2) for fp, fm in fs], dim=-1)
            return gradient, hessian
        if taps == 4:
            eps = self.normal_eps / np.sqrt(3)
            ks = [torch.tensor(k, dtype=x.dtype, device=x.device)
                  for k in ((1, -1, -1), (-1, -1, 1), (-1, 1, -1), (1, 1, 1))]
            sd = [self.sdf(x + k * eps) for k in ks]
            gradient = sum(k * s for k, s in zip(ks, sd)) / (4.0 * eps)
            hessian = None
            if training:
                assert sdf is not None
                hxx = ((sd[0] + sd[1] + sd[2] + sd[3]) / 2.0 - 2 * sdf) / eps ** 2
                hessian = torch.cat([hxx, hxx, hxx], dim=-1) / 3.0
            return gradient, hessian
        raise ValueError("Only support 4 or 6 taps.")


class NeuralRGB(torch.nn.Module):
    """modules.py:181-229 (mode "idr": input [x, SH(d), normal, feat, app])."""

    def __init__(self, cfg_rgb, feat_dim, appear_embed):
        super().__init__()
        self.cfg_rgb = cfg_rgb
        self.cfg_appear_embed = appear_embed
        assert cfg_rgb.encoding_view.type == "spherical"
        self.sh_levels = cfg_rgb.encoding_view.levels
        view_dim = (self.sh_levels + 1) ** 2
        base = 6 if cfg_rgb.mode == "idr" else 3
        input_dim = base + view_dim + feat_dim + (appear_embed.dim if appear_embed.enabled else 0)
        m = cfg_rgb.mlp
        dims = [input_dim] + [m.hidden_dim] * m.num_layers + [3]
        self.mlp = MLPwithSkipConnection(dims, skip_connection=m.skip, activ=get_activation(m.activ, **m.activ_params),
                                         use_weightnorm=m.weight_norm)

    def forward(self, points_3D, normals, rays_unit, feats, app):
        view_enc = get_spherical_harmonics(rays_unit, self.sh_levels)
        parts = [points_3D, view_enc, normals, feats]
        if app is not None:
            parts.append(app)
        if self.cfg_rgb.mode == "no_view_dir":
            parts.remove(view_enc)
        if self.cfg_rgb.mode == "no_normal":
            parts.remove(normals)
        return self.mlp(torch.cat(parts, dim=-1)).sigmoid_()


def positional_encoding(x, num_freq_bases):
    """nerf_util.py:134-147: [sin(2^k pi x), cos(2^k pi x)] per input channel, k < L,
    laid out [..., N, 2, L] -> [..., 2 N L]."""
    freq = 2 ** torch.arange(num_freq_bases, dtype=torch.float32, device=x.device) * np.pi
    spectrum = x[..., None] * freq
    enc = torch.stack([spectrum.sin(), spectrum.cos()], dim=-2)
    return enc.view(*x.shape[:-1], -1)


class BackgroundNeRF(torch.nn.Module):
    """modules.py:232-311: points reparametrised onto the unit sphere plus inverse
    distance [x / |x|, 1 / |x|], Fourier-encoded (levels L: 4 + 8 L inputs); an
    8-layer ReLU MLP with the input concatenated again at layer 4 gives the softplus
    density (output 0) and 256 ReLU features; the view-dependent colour MLP takes
    [features, SH(d), app] -> sigmoid RGB.  No weight norm (build_mlp passes none)."""

    def __init__(self, cfg_bg, appear_embed):
        super().__init__()
        self.cfg = cfg_bg
        assert cfg_bg.encoding.type == "fourier" and cfg_bg.encoding_view.type == "spherical"
        self.levels = cfg_bg.encoding.levels
        self.sh_levels = cfg_bg.encoding_view.levels
        m = cfg_bg.mlp
        in_dim = 4 + 8 * self.levels
        view_dim = m.hidden_dim + (self.sh_levels + 1) ** 2 + (appear_embed.dim if appear_embed.enabled else 0)
        self.mlp_feat = MLPwithSkipConnection([in_dim] + [m.hidden_dim] * (m.num_layers - 1) + [m.hidden_dim + 1],
                                              skip_connection=m.skip, activ=get_activation(m.activ, **m.activ_params))
        self.activ_density = get_activation(m.activ_density, **m.activ_density_params)
        self.mlp_rgb = MLPwithSkipConnection([view_dim] + [m.hidden_dim_rgb] * (m.num_layers_rgb - 1) + [3],
                                             skip_connection=m.skip_rgb,
                                             activ=get_activation(m.activ, **m.activ_params))

    def encode(self, points_3D):
        norm = points_3D.norm(dim=-1, keepdim=True)
        pts = torch.cat([points_3D / norm, 1.0 / norm], dim=-1)
        return torch.cat([pts, positional_encoding(pts, self.levels)], dim=-1)

    def forward(self, points_3D, rays_unit, app_outside):
        out = self.mlp_feat(self.encode(points_3D))
        density, feat = self.activ_density(out[..., 0]), self.mlp_feat.activ(out[..., 1:])
        parts = [feat, get_spherical_harmonics(rays_unit, self.sh_levels)]
        if app_outside is not None:
            parts.append(app_outside)
        rgb = self.mlp_rgb(torch.cat(parts, dim=-1)).sigmoid_()
        return rgb, density
