"""Generate the golden fixture of the hierarchical importance sampler.

Runs the REFERENCE's own Model.sample_dists_all / sample_dists_hierarchical
(projects/neuralangelo/model.py:232-267) with nerf_util.sample_dists and
sample_dists_from_pdf (projects/nerf/utils/nerf_util.py:20-68), the ray bounds of
Model.get_dist_bounds (model.py:207-213) and render.alpha_compositing_weights, in
float64 on the CPU.  The field is an analytic SDF (a wobbly sphere of radius 0.5)
standing in for NeuralSDF.sdf, so the fixture pins the sampler alone.  The
reference's sample_dists defaults to device="cuda" (nerf_util.py:20); the
generator calls it with device="cpu" and otherwise unchanged.

Usage (needs the reference checkout; writes tests/golden/sampler.npz):
    python tests/golden/make_golden_sampler.py /root/reference
"""
import functools
import os
import sys
import types
import warnings

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.dont_write_bytecode = True
warnings.filterwarnings("ignore")


def wobbly_sphere(x):
    """Analytic SDF-like field [..., 3] -> [..., 1]."""
    r = x.norm(dim=-1, keepdim=True)
    w = torch.sin(5 * x[..., :1]) * torch.sin(5 * x[..., 1:2]) * torch.sin(5 * x[..., 2:3])
    return r - 0.5 + 0.05 * w


def main(ref_root):
    sys.path.insert(0, ref_root)
    sys.modules.setdefault("tinycudann", types.ModuleType("tinycudann"))
    torch.set_default_dtype(torch.float64)
    from projects.nerf.utils import nerf_util
    from projects.neuralangelo.model import Model

    orig = nerf_util.sample_dists
    nerf_util.sample_dists = functools.partial(orig, device="cpu")

    R, n_coarse, n_fine, n_hier, seed = 40, 64, 16, 4, 7
    g = torch.Generator().manual_seed(seed)
    c = torch.randn(R, 3, generator=g)
    c = 3.0 * c / c.norm(dim=-1, keepdim=True)
    d = -c + 0.3 * torch.randn(R, 3, generator=g)
    # three rays miss the unit sphere: aimed perpendicular to the camera direction
    d[:3] = torch.linalg.cross(c[:3], torch.tensor([[0.3, 0.5, 0.8]]).expand(3, 3))
    d = d / d.norm(dim=-1, keepdim=True)
    center, ray_unit = c[None], d[None]            # [B=1, R, 3]

    fake = types.SimpleNamespace()
    fake.cfg_render = types.SimpleNamespace(num_samples=types.SimpleNamespace(coarse=n_coarse, fine=n_fine),
                                            num_sample_hierarchy=n_hier)
    fake.neural_sdf = types.SimpleNamespace(sdf=wobbly_sphere)
    fake.sample_dists_from_pdf = functools.partial(nerf_util.sample_dists_from_pdf, intvs_fine=n_fine)  # model.py:42
    fake.sample_dists_hierarchical = lambda *a, **k: Model.sample_dists_hierarchical(fake, *a, **k)
    near, far, outside = Model.get_dist_bounds(fake, center, ray_unit)

    # per-round trace of the reference's hierarchical step
    trace = []
    orig_h = fake.sample_dists_hierarchical

    def traced(dists, sdfs, inv_s, **k):
        fine = orig_h(dists, sdfs, inv_s=inv_s, **k)
        trace.append((dists[0, ..., 0].clone(), sdfs[0, ..., 0].clone(), fine[0, ..., 0].clone(), inv_s))
        return fine
    fake.sample_dists_hierarchical = traced

    torch.manual_seed(seed)
    dists = Model.sample_dists_all(fake, center, ray_unit, near, far, stratified=True)
    torch.manual_seed(seed)
    u = torch.rand(1, R, n_coarse, 1)              # the uniforms sample_dists drew (nerf_util.py:33)
    out = dict(center=c.numpy(), ray_unit=d.numpy(), near=near[0].numpy(), far=far[0].numpy(),
               outside=outside[0].numpy(), u=u[0, ..., 0].numpy(), dists=dists[0, ..., 0].numpy(),
               sizes=np.array([n_coarse, n_fine, n_hier]))
    for h, (dd, ss, ff, inv_s) in enumerate(trace):
        out[f'round{h}_dists'] = dd.numpy()
        out[f'round{h}_sdfs'] = ss.numpy()
        out[f'round{h}_fine'] = ff.numpy()
        assert inv_s == 64 * 2 ** h
    path = os.path.join(HERE, "sampler.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the neuralangelo reference checkout>")
    main(sys.argv[1])
