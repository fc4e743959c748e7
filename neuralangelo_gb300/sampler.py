"""Hierarchical importance sampler on the GPU (the no-grad pre-pass of the object field).

``HierarchicalSampler(n_coarse, n_fine, n_hierarchy)(sdf_fn, center, ray_unit,
near, far, u)`` returns the sorted sample distances [R, n_coarse + n_hierarchy *
n_fine] of Model.sample_dists_all (projects/neuralangelo/model.py:232-248):
stratified coarse samples (nerf_util.sample_dists, nerf_util.py:20-38), then
``n_hierarchy`` rounds that draw ``n_fine`` samples each from the NeuS weights at
sharpness 64 * 2^h (model.py:250-267, nerf_util.sample_dists_from_pdf :41-68)
and sort them in.  The per-ray work runs in ``gbsdf_sampler_round``; the SDF of
new points comes from ``sdf_fn`` (points [M, 3] -> [M]), by default the fused
field kernel (``FieldSDF(neural_sdf, sign=1).points``).
"""
import ctypes

import torch

from . import _lib

c_i32, c_vp = ctypes.c_int32, ctypes.c_void_p


class SamplerArgs(ctypes.Structure):
    _fields_ = [("R", ctypes.c_int64), ("ld", c_i32), ("n_list", c_i32), ("n_merge", c_i32), ("n_fine", c_i32),
                ("inv_s", ctypes.c_float), ("robust", c_i32), ("center", c_vp), ("ray_unit", c_vp),
                ("dists", c_vp), ("sdfs", c_vp), ("merge_d", c_vp), ("merge_s", c_vp), ("fine_d", c_vp),
                ("fine_pts", c_vp)]


_lib.register("gbsdf_sampler_args_size", [])
_lib.register("gbsdf_sampler_coarse", [c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp])
_lib.register("gbsdf_sampler_round", [c_vp, c_vp])

MAX_LIST = 512


def _p(t):
    return None if t is None else t.data_ptr()


def check_struct_size():
    lib = _lib.load()
    lib.gbsdf_sampler_args_size.restype = ctypes.c_size_t
    assert lib.gbsdf_sampler_args_size() == ctypes.sizeof(SamplerArgs), "gbsdf_sampler_args layout mismatch"


class HierarchicalSampler:
    """Model.sample_dists_all (model.py:232-248) with the per-ray work on libgbsdf."""

    def __init__(self, n_coarse=64, n_fine=16, n_hierarchy=4, robust=True):
        if n_coarse + n_hierarchy * n_fine > MAX_LIST:
            raise ValueError(f"at most {MAX_LIST} samples per ray")
        if n_fine > 32:
            raise ValueError("at most 32 fine samples per round")
        check_struct_size()
        self.nc, self.nf, self.nh = int(n_coarse), int(n_fine), int(n_hierarchy)
        self.robust = bool(robust)

    @property
    def n_samples(self):
        return self.nc + self.nh * self.nf

    def __call__(self, sdf_fn, center, ray_unit, near, far, u=None, trace=None):
        """center, ray_unit [R, 3]; near, far [R, 1] (or [R]); u [R, n_coarse] stratified
        uniforms or None (0.5, the non-stratified case) -> dists [R, n_samples] float32.
        ``trace`` (a list) receives (dists, sdfs, fine) per round, for tests."""
        dev = center.device
        _lib.require_cuda(center, ray_unit, near, far, u)
        R = center.shape[0]
        N = self.n_samples
        f32 = dict(device=dev, dtype=torch.float32)
        center = center.contiguous().float()
        ray_unit = ray_unit.contiguous().float()
        near = near.reshape(-1).contiguous().float()
        far = far.reshape(-1).contiguous().float()
        if u is not None:
            u = u.contiguous().float()
        dists = torch.empty(R, N, **f32)
        if R == 0:
            return dists
        sdfs = torch.empty(R, N, **f32) if self.nh > 0 else None
        pts = torch.empty(R * self.nc, 3, **f32) if self.nh > 0 else None
        stream = _lib.stream_ptr(dev)
        a = SamplerArgs()
        a.R, a.ld = R, N
        a.center, a.ray_unit, a.dists, a.sdfs = _p(center), _p(ray_unit), _p(dists), _p(sdfs)
        a.robust = 1 if self.robust else 0
        _lib.call("gbsdf_sampler_coarse", ctypes.byref(a), self.nc, c_vp(_p(u)), self.nc if u is not None else 0,
                  c_vp(near.data_ptr()), c_vp(far.data_ptr()), c_vp(_p(pts)), stream)
        if self.nh == 0:
            return dists
        sdfs[:, :self.nc] = sdf_fn(pts).reshape(R, self.nc)
        fine_d = torch.empty(R, self.nf, **f32)
        fine_s = torch.empty(R, self.nf, **f32)
        fine_pts = torch.empty(R * self.nf, 3, **f32)
        n_list = self.nc
        for h in range(self.nh):
            a.n_list, a.n_merge = n_list, (self.nf if h > 0 else 0)
            a.n_fine, a.inv_s = self.nf, float(64 * 2 ** h)
            a.merge_d, a.merge_s = _p(fine_d), _p(fine_s)
            a.fine_d, a.fine_pts = _p(fine_d), _p(fine_pts)
            _lib.call("gbsdf_sampler_round", ctypes.byref(a), stream)
            n_list += a.n_merge
            if trace is not None:   # the (merged) list this round's weights were computed on
                trace.append((dists[:, :n_list].clone(), sdfs[:, :n_list].clone(), fine_d.clone()))
            if h != self.nh - 1:
                fine_s.copy_(sdf_fn(fine_pts).reshape(R, self.nf))
        # final merge of the last round's samples (distances only, model.py:240-241)
        a.n_list, a.n_merge, a.n_fine = n_list, self.nf, 0
        a.sdfs, a.merge_s, a.fine_d, a.fine_pts = None, None, None, None
        a.merge_d = _p(fine_d)
        _lib.call("gbsdf_sampler_round", ctypes.byref(a), stream)
        return dists


def field_sdf_fn(neural_sdf):
    """SDF of a NeuralSDF through the fused field kernel (FP16 table and weights,
    FP32 head), as the sampler's ``sdf_fn``."""
    from .mesh import FieldSDF
    f = FieldSDF(neural_sdf, sign=1.0)
    return f.points


def plain_sdf_fn(neural_sdf):
    """SDF of a NeuralSDF through the plain FP32 drop-in (libgbsdf hash grid + torch MLP),
    the evaluation the reference's sampler makes (model.py:238, 245)."""
    def fn(pts):
        with torch.no_grad():
            return neural_sdf.sdf(pts)[..., 0]
    return fn
