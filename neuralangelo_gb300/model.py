"""Field model and training forward with the reference's structure (plain FP32 drop-in).

``FieldModel.render_step`` follows Model.render_rays_object + render_rays
(projects/neuralangelo/model.py:124-190; with the background NeRF of
render_rays_background, :192-205, when ``cfg.background.enabled``) and
Trainer._compute_loss (projects/neuralangelo/trainer.py:40-52).  Hash grid,
NeuS alpha and compositing weights run on libgbsdf; the MLPs are torch linears
exactly as in the reference.  ``schedule`` restates the per-iteration
coarse-to-fine / epsilon / curvature-weight updates (trainer.py:54-74).
"""
import torch
import torch.nn.functional as torch_F

from . import render
from .modules import BackgroundNeRF, NeuralRGB, NeuralSDF


class FieldModel(torch.nn.Module):
    def __init__(self, cfg, table_dtype=torch.float32):
        super().__init__()
        self.cfg = cfg
        self.neural_sdf = NeuralSDF(cfg.sdf, table_dtype=table_dtype)
        self.neural_rgb = NeuralRGB(cfg.rgb, feat_dim=cfg.sdf.mlp.hidden_dim, appear_embed=cfg.appear_embed)
        self.s_var = torch.nn.Parameter(torch.tensor(cfg.s_var.init_val, dtype=torch.float32))
        self.appear_embed = None
        if cfg.appear_embed.enabled:
            self.appear_embed = torch.nn.Embedding(cfg.appear_embed.num_images, cfg.appear_embed.dim)
        bg = cfg.get("background")
        self.with_background = bool(bg and bg.enabled)
        self.background_nerf = self.appear_embed_outside = None
        if self.with_background:
            self.background_nerf = BackgroundNeRF(bg, cfg.appear_embed)                 # model.py:60-61
            if cfg.appear_embed.enabled:                                             # model.py:51-54
                self.appear_embed_outside = torch.nn.Embedding(cfg.appear_embed.num_images, cfg.appear_embed.dim)
        self.outside_val = 1000.0 * (-1 if cfg.sdf.mlp.inside_out else 1)
        self.anneal_end = cfg.s_var.anneal_end
        self.progress = 0.0
        self.w_curv = cfg.loss_weight.curvature

    def schedule(self, iteration):
        """Trainer._start_of_iteration + get_curvature_weight (trainer.py:54-74)."""
        self.progress = iteration / self.cfg.max_iter
        sdf = self.neural_sdf
        sdf.warm_up_end = self.cfg.warm_up_end
        sdf.set_active_levels(iteration)
        sdf.set_normal_epsilon()
        w0 = self.cfg.loss_weight.curvature
        if iteration <= self.cfg.warm_up_end:
            self.w_curv = iteration / self.cfg.warm_up_end * w0
        else:
            self.w_curv = w0 / (sdf.growth_rate ** (sdf.anneal_levels - 1))

    def render_step(self, batch, with_curvature=True):
        """One training forward on a batch of rays; returns outputs and the total loss.

        batch: center [R,3], ray_unit [R,3], dists [R,N], far [R,1], outside [R,1] (bool),
               target [R,3], app_idx [R] (long, when the appearance embedding is on),
               dists_bg [R,Nb] (background sample distances, with the background NeRF).
        """
        c, d, dists = batch["center"], batch["ray_unit"], batch["dists"]
        R, N = dists.shape
        points = c[:, None, :] + d[:, None, :] * dists[..., None]             # camera.py:314-320
        sdfs, feats = self.neural_sdf(points)
        outside = batch["outside"]
        sdfs = sdfs.masked_fill(outside[:, None, :].expand_as(sdfs), self.outside_val)   # model.py:163
        rays_unit = d[:, None, :].expand_as(points).contiguous()
        gradients, hessians = self.neural_sdf.compute_gradients(points, training=True, sdf=sdfs)
        normals = torch_F.normalize(gradients, dim=-1)
        app = None
        if self.appear_embed is not None:
            app = self.appear_embed(batch["app_idx"])[:, None, :].expand(R, N, -1)
        rgbs = self.neural_rgb(points, normals, rays_unit, feats, app)
        alphas = render.compute_neus_alphas(d, sdfs[..., 0], gradients, dists, self.s_var, dist_far=batch["far"],
                                            progress=self.progress, anneal_end=self.anneal_end)
        rgbs_all, alphas_all = rgbs, alphas
        if self.with_background:                                                      # model.py:129-134, 192-205
            dists_bg = batch["dists_bg"]
            pts_bg = c[:, None, :] + d[:, None, :] * dists_bg[..., None]
            app_out = None
            if self.appear_embed_outside is not None:
                app_out = self.appear_embed_outside(batch["app_idx"])[:, None, :].expand(R, dists_bg.shape[1], -1)
            rgbs_bg, dens_bg = self.background_nerf(pts_bg, d[:, None, :].expand_as(pts_bg), app_out)
            alphas_bg = render.volume_rendering_alphas_dist(dens_bg, dists_bg)
            rgbs_all = torch.cat([rgbs, rgbs_bg], dim=1)
            alphas_all = torch.cat([alphas, alphas_bg], dim=1)
        weights = render.alpha_compositing_weights(alphas_all)
        rgb = render.composite(rgbs_all, weights)
        lw = self.cfg.loss_weight
        l_render = torch_F.l1_loss(rgb, batch["target"]) * 3                   # trainer.py:43
        inside = (~outside.expand(R, N)).float()
        eik = ((gradients.norm(dim=-1) - 1.0) ** 2).nan_to_num(nan=0.0, posinf=0.0, neginf=0.0)
        l_eik = (eik * inside).mean()                                         # misc.py:74-80
        loss = lw.render * l_render + lw.eikonal * l_eik
        l_curv = None
        if with_curvature and self.w_curv:
            lap = hessians.sum(dim=-1).abs().nan_to_num(nan=0.0, posinf=0.0, neginf=0.0)
            l_curv = (lap * inside).mean()                                    # misc.py:83-89
            loss = loss + self.w_curv * l_curv
        return dict(loss=loss, l_render=l_render, l_eik=l_eik, l_curv=l_curv, rgb=rgb, rgbs=rgbs,
                    sdf=sdfs[..., 0], feat=feats, grads=gradients, hess=hessians, alphas=alphas,
                    weights=weights[..., 0])
