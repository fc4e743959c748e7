"""Evaluation rendering and textured-mesh colours on the package's kernels.

* ``camera_rays``: camera.get_center_and_ray (projects/nerf/utils/camera.py:283-311).
* ``Inference.render_rays`` / ``render_image``: Model.inference and render_image
  (projects/neuralangelo/model.py:73-114) with training off.
  * The hierarchical sampler runs on the GPU, non-stratified (model.py:232-248).
  * The object and background fields use the fused forward kernels.
  * The render kernel runs forward only.
  * Outputs: colour, object opacity, the composite of the unnormalised gradient
    (model.py:175-178), and depth = composite distance / |ray| (model.py:106-107).
  * The normal map is -gradient R^T in camera axes (model.py:79).
* ``extract_texture``: per-vertex colours of the textured mesh (projects/neuralangelo/
  utils/mesh.py:53-65) on the plain modules.
  * It uses the SDF, features and eval-mode numerical gradient.
  * The colour MLP sees the view direction -normal and a zero appearance code.
"""
import numpy as np
import torch
import torch.nn.functional as torch_F

from .fused import FusedField
from .sampler import HierarchicalSampler, field_sdf_fn
from .workloads import background_dists, sphere_bounds


def camera_rays(pose, intr, H, W):
    """pose [3,4] world-to-camera [R|t], intr [3,3] -> center [HW,3], ray [HW,3] (depth-1
    rays, not unit), pixels row-major with centres at +0.5 (camera.py:283-311)."""
    dev = pose.device
    y = torch.arange(H, dtype=torch.float32, device=dev) + 0.5
    x = torch.arange(W, dtype=torch.float32, device=dev) + 0.5
    Y, X = torch.meshgrid(y, x, indexing="ij")
    xy = torch.stack([X, Y], dim=-1).view(-1, 2)
    grid = torch.cat([xy, torch.ones_like(xy[:, :1])], dim=-1) @ intr.float().inverse().t()     # img2cam
    R, t = pose[:, :3].float(), pose[:, 3:].float()
    pose_inv = torch.cat([R.t(), -R.t() @ t], dim=1)                                           # Pose().invert

    def cam2world(Xc):
        return torch.cat([Xc, torch.ones_like(Xc[:, :1])], dim=-1) @ pose_inv.t()

    center = cam2world(torch.zeros_like(grid))
    return center, cam2world(grid) - center


class Inference:
    """Full-image rendering of a FieldModel (object field, plus its background NeRF when the
    model has one) through the fused forward kernels, in chunks of rays."""

    def __init__(self, model, n_coarse=64, n_fine=16, n_hierarchy=4, chunk=65536):
        self.model = model
        self.ff = FusedField(model)
        self.sampler = HierarchicalSampler(n_coarse, n_fine, n_hierarchy)
        self.chunk = int(chunk)

    @torch.no_grad()
    def render_rays(self, center, ray, app_idx=None):
        """center, ray [R,3] (ray not unit) -> dict of rgb [R,3], opacity [R,1],
        gradient [R,3], depth [R,1]."""
        m = self.model
        R = center.shape[0]
        if app_idx is None:
            app_idx = torch.zeros(R, dtype=torch.int64, device=center.device)
        ray_unit = torch_F.normalize(ray, dim=-1)
        sdf_fn = field_sdf_fn(m.neural_sdf)
        parts = []
        for i in range(0, R, self.chunk):
            c, d, r = center[i:i + self.chunk], ray_unit[i:i + self.chunk], ray[i:i + self.chunk]
            near, far, outside = sphere_bounds(c, d)                                  # model.py:207-213
            dists = self.sampler(sdf_fn, c, d, near, far, u=None)
            b = dict(center=c, ray_unit=d, dists=dists, far=far, outside=outside, app_idx=app_idx[i:i + self.chunk])
            if getattr(m, "with_background", False):
                b["dists_bg"] = background_dists(far, m.cfg.background.samples)        # model.py:269-273
            ev = self.ff.render(b)
            ev["depth"] = ev["dist"] / r.norm(dim=-1, keepdim=True)
            parts.append(ev)
        out = {k: torch.cat([p[k] for p in parts]) for k in ("rgb", "opacity", "gradient", "depth")}
        self.ff.release()
        return out

    @torch.no_grad()
    def render_image(self, pose, intr, H, W, image_idx=0):
        """Model.inference for one view: rgb_map [3,H,W], opacity_map [1,H,W], depth_map
        [1,H,W], normal_map [3,H,W] (camera axes)."""
        center, ray = camera_rays(pose, intr, H, W)
        app_idx = torch.full((H * W,), int(image_idx), dtype=torch.int64, device=pose.device)
        out = self.render_rays(center, ray, app_idx)
        normal_cam = -out["gradient"] @ pose[:, :3].float().t()

        def img(x):
            return x.t().reshape(x.shape[1], H, W)

        return dict(rgb_map=img(out["rgb"]), opacity_map=img(out["opacity"]), depth_map=img(out["depth"]),
                    normal_map=img(normal_cam))


@torch.no_grad()
def extract_texture(xyz, model):
    """mesh.py:53-65: colours (uint8 [N,3]) of the points xyz [N,3] (numpy)."""
    dev = next(model.parameters()).device
    x = torch.from_numpy(np.asarray(xyz)).float().to(dev)[None, None]
    sdfs, feats = model.neural_sdf(x)
    grads, _ = model.neural_sdf.compute_gradients(x, training=False, sdf=sdfs)
    normals = torch_F.normalize(grads, dim=-1)
    app = None
    if model.appear_embed is not None:
        app = torch.zeros(1, 1, x.shape[2], model.appear_embed.embedding_dim, device=dev)
    rgbs = model.neural_rgb(x, normals, -normals, feats, app)
    return (rgbs.reshape(-1, 3).cpu().numpy() * 255).astype(np.uint8)
