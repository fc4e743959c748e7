"""NeuS alpha and compositing over the libgbsdf CUDA kernels (plain FP32 drop-in).

Mirrors the reference call surface:
  compute_neus_alphas(...)          Model.compute_neus_alphas, projects/neuralangelo/model.py:275-292
  alpha_compositing_weights(alphas) projects/nerf/utils/render.py:87-99
  composite(quantities, weights)    projects/nerf/utils/render.py:102-112
  volume_rendering_alphas_dist(...) projects/nerf/utils/render.py:68-84 (background samples; torch)
Shapes follow the reference ([B,R,N] with B folded into R).
"""
import torch

from . import _lib


class _NeusAlphaFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, ray_unit, sdfs, gradients, dists, far, s_var, progress, anneal_end):
        R, N = sdfs.shape
        args = [t.contiguous().float() for t in (ray_unit, sdfs, gradients, dists, far)]
        s_var_f = s_var.detach().reshape(1).float().contiguous()
        alpha = torch.empty(R, N, device=sdfs.device, dtype=torch.float32)
        _lib.call("gbsdf_neus_alpha_fwd", R, N, *[_lib.ptr(t) for t in args], _lib.ptr(s_var_f),
                  float(progress), float(anneal_end), _lib.ptr(alpha), _lib.stream_ptr(sdfs.device))
        ctx.save_for_backward(*args, s_var_f)
        ctx.progress, ctx.anneal_end, ctx.s_shape = progress, anneal_end, s_var.shape
        return alpha

    @staticmethod
    def backward(ctx, d_alpha):
        ray, sdf, grad, dists, far, s_var = ctx.saved_tensors
        R, N = sdf.shape
        d_sdf = torch.empty_like(sdf)
        d_grad = torch.empty_like(grad)
        d_s = torch.zeros(1, device=sdf.device, dtype=torch.float32)
        _lib.call("gbsdf_neus_alpha_bwd", R, N, _lib.ptr(ray), _lib.ptr(sdf), _lib.ptr(grad), _lib.ptr(dists),
                  _lib.ptr(far), _lib.ptr(s_var), float(ctx.progress), float(ctx.anneal_end),
                  _lib.ptr(d_alpha.contiguous().float()), _lib.ptr(d_sdf), _lib.ptr(d_grad), _lib.ptr(d_s),
                  _lib.stream_ptr(sdf.device))
        return None, d_sdf, d_grad, None, None, d_s.reshape(ctx.s_shape), None, None


def compute_neus_alphas(ray_unit, sdfs, gradients, dists, s_var, dist_far=None, progress=1.0, anneal_end=0.1):
    """ray_unit [R,3], sdfs [R,N] (or [R,N,1]), gradients [R,N,3], dists [R,N] (or [R,N,1]),
    dist_far [R,1] (None -> 1e10 as the reference) -> alphas [R,N]."""
    if sdfs.dim() == 3:
        sdfs = sdfs[..., 0]
    if dists.dim() == 3:
        dists = dists[..., 0]
    R = sdfs.shape[0]
    if dist_far is None:
        dist_far = torch.full((R,), 1e10, device=sdfs.device)
    _lib.require_cuda(ray_unit, sdfs, gradients, dists, dist_far)
    return _NeusAlphaFn.apply(ray_unit.reshape(R, 3), sdfs, gradients.reshape(R, -1, 3), dists,
                              dist_far.reshape(R), s_var, progress, anneal_end)


class _WeightsFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, alphas):
        a = alphas.contiguous().float()
        R, N = a.shape
        w = torch.empty_like(a)
        _lib.call("gbsdf_composite_weights_fwd", R, N, _lib.ptr(a), _lib.ptr(w), _lib.stream_ptr(a.device))
        ctx.save_for_backward(a)
        return w

    @staticmethod
    def backward(ctx, d_w):
        (a,) = ctx.saved_tensors
        R, N = a.shape
        d_a = torch.empty_like(a)
        _lib.call("gbsdf_composite_weights_bwd", R, N, _lib.ptr(a), _lib.ptr(d_w.contiguous().float()),
                  _lib.ptr(d_a), _lib.stream_ptr(a.device))
        return d_a


def volume_rendering_alphas_dist(densities, dists, dist_far=None):
    """render.py:68-84: alpha = 1 - exp(-density * interval), the last interval running to
    dist_far (1e10 by default); densities [R,N], dists [R,N] -> alphas [R,N]."""
    if dist_far is None:
        dist_far = torch.empty_like(dists[..., :1]).fill_(1e10)
    d = torch.cat([dists, dist_far], dim=-1)
    sigma_delta = densities * (d[..., 1:] - d[..., :-1])
    return 1 - (-sigma_delta).exp()


def alpha_compositing_weights(alphas):
    """alphas [R,N] -> weights [R,N,1] (render.py:87-99)."""
    _lib.require_cuda(alphas)
    shp = alphas.shape
    w = _WeightsFn.apply(alphas.reshape(-1, shp[-1]))
    return w.reshape(*shp, 1)


def composite(quantities, weights):
    """sum_i w_i q_i over the sample axis (render.py:102-112)."""
    return (quantities * weights).sum(dim=-2)
