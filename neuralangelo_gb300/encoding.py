"""HashGridEncoding: drop-in for ``tinycudann.Encoding(3, {"otype": "HashGrid", ...})``.

The reference builds the encoder at projects/neuralangelo/utils/modules.py:42-50
and calls it at :85 on [N,3] points in [0,1]; the output is [N, L*F],
level-major (the mask at :109-113 slices the first active_levels*F columns).
This module keeps that surface -- the constructor signature, the flat
``params`` parameter (checkpoint key ``...tcnn_encoding.params``) and the
autograd behaviour (dL/dparams; no dL/dx in numerical-gradient mode) -- over
the CUDA kernels of libgbsdf.so.
"""
import ctypes

import numpy as np
import torch

from . import _lib


class GridLayout:
    """Level table computed by the library's gbsdf_grid_init (host-only call)."""

    def __init__(self, n_levels, n_features, log2_hashmap_size, base_resolution, per_level_scale):
        self.struct = _lib.GridStruct()
        _lib.call("gbsdf_grid_init", ctypes.byref(self.struct), int(n_levels), int(n_features),
                  int(log2_hashmap_size), int(base_resolution), float(per_level_scale))
        s = self.struct
        self.n_levels, self.n_features = n_levels, n_features
        self.scale = np.array(s.scale[:n_levels], np.float32)
        self.resolution = np.array(s.resolution[:n_levels], np.int64)
        self.size = np.array(s.size[:n_levels], np.int64)
        self.hashed = np.array(s.hashed[:n_levels], bool)
        self.offset = np.array(s.offset[:n_levels + 1], np.int64)
        self.n_entries = int(self.offset[-1])
        self.n_params = self.n_entries * n_features


class _HashGridFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, params, layout, active, out_dtype):
        x = x.contiguous().float()
        M = x.shape[0]
        L, F = layout.n_levels, layout.n_features
        out = torch.empty(M, L * F, device=x.device, dtype=out_dtype)
        tdt = _lib.F16 if params.dtype == torch.float16 else _lib.F32
        odt = _lib.F16 if out_dtype == torch.float16 else _lib.F32
        _lib.call("gbsdf_hashgrid_fwd", ctypes.byref(layout.struct), int(active), _lib.ptr(x), M,
                  _lib.ptr(params), tdt, _lib.ptr(out), odt, _lib.stream_ptr(x.device))
        ctx.save_for_backward(x)
        ctx.layout, ctx.active, ctx.params_shape, ctx.params_dtype = layout, active, params.shape, params.dtype
        return out

    @staticmethod
    def backward(ctx, d_out):
        (x,) = ctx.saved_tensors
        layout = ctx.layout
        d_out = d_out.contiguous().float()
        d_params = torch.zeros(ctx.params_shape, device=x.device, dtype=torch.float32)
        _lib.call("gbsdf_hashgrid_bwd", ctypes.byref(layout.struct), int(ctx.active), _lib.ptr(x), x.shape[0],
                  _lib.ptr(d_out), _lib.ptr(d_params), _lib.stream_ptr(x.device))
        return None, d_params.to(ctx.params_dtype), None, None, None


class HashGridEncoding(torch.nn.Module):
    """``tcnn.Encoding(n_input_dims=3, encoding_config)`` for otype "HashGrid".

    encoding_config keys: n_levels, n_features_per_level, log2_hashmap_size,
    base_resolution, per_level_scale (modules.py:42-49).  ``dtype`` selects the
    table precision (float32 for the plain drop-in; float16 matches tcnn's
    default half-precision parameters).  ``active_levels`` (default: all)
    skips levels the caller masks to zero anyway (modules.py:91-93), which
    leaves the output and gradients unchanged.
    """

    def __init__(self, n_input_dims, encoding_config, dtype=torch.float32, seed=1337):
        super().__init__()
        if n_input_dims != 3:
            raise ValueError("HashGridEncoding supports 3 input dimensions")
        c = encoding_config
        if c.get("otype", "HashGrid") not in ("HashGrid", "Grid"):
            raise ValueError(f"unsupported encoding otype {c.get('otype')!r}")
        self.n_input_dims = 3
        self.layout = GridLayout(c["n_levels"], c.get("n_features_per_level", 2), c.get("log2_hashmap_size", 19),
                                 c.get("base_resolution", 16), c.get("per_level_scale", 2.0))
        self.n_output_dims = self.layout.n_levels * self.layout.n_features
        self.active_levels = self.layout.n_levels
        g = torch.Generator().manual_seed(seed)
        # tcnn initialises grid parameters uniformly in [-1e-4, 1e-4]
        init = (torch.rand(self.layout.n_params, generator=g) * 2 - 1) * 1e-4
        self.params = torch.nn.Parameter(init.to(dtype))
        self.out_dtype = torch.float32

    def forward(self, x):
        if x.shape[-1] != 3:
            raise ValueError("expected [..., 3] input")
        _lib.require_cuda(x, self.params)
        shp = x.shape[:-1]
        out = _HashGridFunction.apply(x.reshape(-1, 3), self.params, self.layout, self.active_levels,
                                      self.out_dtype)
        return out.reshape(*shp, self.n_output_dims)

    def indices(self, x):
        """Absolute table-entry index per (point, active level, corner): int64 [M, A, 8]."""
        _lib.require_cuda(x)
        x = x.reshape(-1, 3).contiguous().float()
        A = self.active_levels
        out = torch.empty(x.shape[0], A, 8, dtype=torch.int64, device=x.device)
        _lib.call("gbsdf_hashgrid_indices", ctypes.byref(self.layout.struct), int(A), _lib.ptr(x), x.shape[0],
                  _lib.ptr(out), _lib.stream_ptr(x.device))
        return out


# tcnn-compatible alias so ``sys.modules["tinycudann"] = neuralangelo_gb300.encoding``
# makes the reference's ``tcnn.Encoding(3, config)`` resolve here.
Encoding = HashGridEncoding
