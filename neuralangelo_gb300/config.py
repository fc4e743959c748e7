"""Configuration objects mirroring the reference's YAML keys.

The reference reads ``cfg.model.object.sdf.*`` / ``cfg.model.object.rgb.*``
(projects/neuralangelo/configs/base.yaml:38-115) by attribute access.
``AttrDict`` gives the same access without a YAML dependency, and the
``field_config`` helper builds the two field configurations used by the
benchmarks and tests:

* ``small``  -- L=8, F=4, T=2^16, base 16, growth 1.5, SDF MLP 256, colour MLP 2x128
* ``full``   -- L=16, F=8, T=2^22, 32 -> 2048, SDF MLP 256, colour MLP 4x256,
                16-dim appearance embedding over 100 images (base.yaml defaults
                with the embedding enabled)
"""
import copy

import numpy as np


class AttrDict(dict):
    """dict with attribute access (the reference uses addict/EasyDict-style configs)."""

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e

    def __setattr__(self, k, v):
        self[k] = v

    def __deepcopy__(self, memo):
        return AttrDict({k: copy.deepcopy(v, memo) for k, v in self.items()})


def to_attr(d):
    if isinstance(d, dict):
        return AttrDict({k: to_attr(v) for k, v in d.items()})
    if isinstance(d, list):
        return [to_attr(v) for v in d]
    return d


def sdf_config(levels=16, dim=8, dict_size=22, min_logres=5, max_logres=11, per_level_scale=None,
               hidden=256, init_active_level=4, c2f_step=5000, taps=6, beta=100.0):
    """cfg.model.object.sdf (base.yaml:40-68).  ``per_level_scale`` overrides the
    growth derived from min/max_logres (the small field's growth 1.5 is not a
    ratio of powers of two over 7 levels)."""
    return to_attr(dict(
        mlp=dict(num_layers=1, hidden_dim=hidden, skip=[], activ="softplus", activ_params=dict(beta=beta),
                 geometric_init=True, weight_norm=True, out_bias=0.5, inside_out=False),
        encoding=dict(type="hashgrid", levels=levels,
                      hashgrid=dict(min_logres=min_logres, max_logres=max_logres, dict_size=dict_size, dim=dim,
                                    range=[-2, 2], per_level_scale=per_level_scale),
                      coarse2fine=dict(enabled=True, init_active_level=init_active_level, step=c2f_step)),
        gradient=dict(mode="numerical", taps=taps)))


def rgb_config(layers=4, hidden=256):
    """cfg.model.object.rgb (base.yaml:69-80)."""
    return to_attr(dict(
        mlp=dict(num_layers=layers, hidden_dim=hidden, skip=[], activ="relu_", activ_params={}, weight_norm=True),
        mode="idr", encoding_view=dict(type="spherical", levels=3)))


def background_config(enabled=True, layers=8, hidden=256, skip=(4,), layers_rgb=2, hidden_rgb=128, levels=10,
                      view_levels=3, samples=32):
    """cfg.model.background (base.yaml:84-104) and render.num_samples.background."""
    return to_attr(dict(
        enabled=enabled, white=False, view_dep=True, samples=samples,
        mlp=dict(num_layers=layers, hidden_dim=hidden, skip=list(skip), num_layers_rgb=layers_rgb,
                 hidden_dim_rgb=hidden_rgb, skip_rgb=[], activ="relu", activ_params={},
                 activ_density="softplus", activ_density_params={}),
        encoding=dict(type="fourier", levels=levels),
        encoding_view=dict(type="spherical", levels=view_levels)))


def field_config(name, background=False):
    """Return AttrDict(sdf=..., rgb=..., appear_embed=..., s_var=..., background=...).
    background=True enables the background NeRF of the reference's base config."""
    if name == "small":
        sdf = sdf_config(levels=8, dim=4, dict_size=16, min_logres=4, max_logres=None, per_level_scale=1.5,
                         hidden=256)
        rgb = rgb_config(layers=2, hidden=128)
        app = dict(enabled=False, dim=0, num_images=0)
    elif name == "full":
        sdf = sdf_config()
        rgb = rgb_config()
        app = dict(enabled=True, dim=16, num_images=100)
    else:
        raise ValueError(name)
    return to_attr(dict(sdf=sdf, rgb=rgb, appear_embed=app, s_var=dict(init_val=3.0, anneal_end=0.1),
                        background=background_config(enabled=bool(background)),
                        loss_weight=dict(render=1.0, eikonal=0.1, curvature=5e-4), warm_up_end=5000,
                        max_iter=500000))


def growth_rate(cfg_sdf):
    """modules.py:39-41 (or the explicit per_level_scale)."""
    hg = cfg_sdf.encoding.hashgrid
    if hg.get("per_level_scale"):
        return float(hg.per_level_scale)
    r_min, r_max = 2 ** hg.min_logres, 2 ** hg.max_logres
    return float(np.exp((np.log(r_max) - np.log(r_min)) / (cfg_sdf.encoding.levels - 1)))
