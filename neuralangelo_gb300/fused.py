"""Fused mixed-precision training step of the field (FP16 tensor cores, FP32 masters).

One call of ``FusedField.step(batch)`` runs the forward and backward of
Model.render_rays_object + render_rays + Trainer._compute_loss
(projects/neuralangelo/model.py:124-190, trainer.py:40-52; background off)
through the libgbsdf kernels and leaves FP32 gradients in ``.grad`` of the
FieldModel's master parameters, exactly where the plain drop-in's autograd
puts them.

Precision: the hash table and the MLP weights are used as FP16 copies of the
FP32 masters; every contraction accumulates in FP32 (tcgen05 TMEM); the SDF
head, positions, tap differences, transmittance (log space) and losses stay
FP32; the loss sums are accumulated in FP64.  Gradients are computed with a
loss scale and unscaled into FP32.  With dynamic loss scaling (the default, as the
reference's GradScaler: imaginaire/trainers/base.py:186-193,447-454) the scale lives
in a device scalar that starts at 2^15: a step whose gradients are not finite sets a
device flag (``found_inf``) and halves the scale, and growth_interval clean steps in
a row double it; the update runs on the device, inside a captured graph too.

Kernels per step (all on the current stream):
  field_fwd, dense x (1 + colour layers), rgb_head_fwd, render_fused,
  rgb_head_bwd (with the colour head's weight gradient), dense x (colour layers + 2),
  app_grad, field_bwd, and the weight gradients (tcgen05, fp16 in / fp32 out).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .dense import EPI_DRELU, EPI_DSOFTPLUS, EPI_IDENTITY, EPI_RELU, EPI_SOFTPLUS

c_i32, c_i64, c_f32, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p


class FieldArgs(ctypes.Structure):
    _fields_ = [("Ns", c_i64), ("S", c_i32), ("ld_h0c", c_i32), ("sample_ray", c_vp), ("center", c_vp),
                ("ray_unit", c_vp), ("dists", c_vp), ("outside", c_vp), ("app_idx", c_vp),
                ("grid", _lib.GridStruct), ("active", c_i32), ("K0", c_i32), ("table", c_vp), ("w0e", c_vp),
                ("w0eT", c_vp), ("w0b", c_vp), ("w0x", c_vp), ("b0", c_vp), ("whead", c_vp), ("bhead", c_vp),
                ("beta", c_f32), ("eps", c_f32), ("two_eps", c_f32), ("eps2", c_f32), ("outside_val", c_f32),
                ("d_table_scale", c_f32), ("xc", c_vp), ("ldxc", c_i32), ("app_dim", c_i32), ("app_table", c_vp),
                ("sdf", c_vp), ("grad", c_vp), ("hess", c_vp), ("h0c", c_vp), ("d_sdf", c_vp), ("d_grad", c_vp),
                ("d_hess", c_vp), ("d_xc", c_vp), ("ld_dxc", c_i32), ("normal_col", c_i32), ("d_h0c", c_vp),
                ("d_table", c_vp), ("d_pre0", c_vp), ("x0ext", c_vp), ("d_enc", c_vp), ("d_whead", c_vp),
                ("d_bhead", c_vp),
                ("err", c_vp), ("d_w0", c_vp), ("h0c_lo", c_vp), ("xc_lo", c_vp), ("d_pre0_lo", c_vp),
                ("d_table_scale_dev", c_vp), ("found_inf", c_vp),
                ("taps", c_i32), ("pad_taps", c_i32), ("d_table_fix", c_vp), ("scatter_cpt", c_i32),
                ("fwd_ctas", c_i32)]


class FieldWorkspace(ctypes.Structure):
    _fields_ = [("rows", c_i64), ("x0ext_bytes", ctypes.c_size_t), ("d_enc_bytes", ctypes.c_size_t),
                ("d_w0_bytes", ctypes.c_size_t), ("d_pre0_bytes", ctypes.c_size_t),
                ("d_table_fix_bytes", ctypes.c_size_t)]


class RenderArgs(ctypes.Structure):
    _fields_ = [("R", c_i64), ("S", c_i32), ("pad0", c_i32), ("ray_offsets", c_vp), ("ray_unit", c_vp),
                ("dists", c_vp), ("far", c_vp), ("outside", c_vp), ("target", c_vp), ("s_var", c_vp),
                ("sdf", c_vp), ("grad", c_vp), ("hess", c_vp), ("rgbs", c_vp), ("anneal", c_f32),
                ("w_render", c_f32), ("w_eik", c_f32), ("w_curv", c_f32), ("l1_scale", c_f32),
                ("mean_scale", c_f32), ("loss_scale", c_f32), ("pad1", c_i32), ("rgb", c_vp), ("weights", c_vp),
                ("d_rgbs", c_vp), ("d_sdf", c_vp), ("d_grad", c_vp), ("d_hess", c_vp), ("d_s_var", c_vp),
                ("loss_sums", c_vp), ("err", c_vp), ("n_bg", c_i32), ("ld_d_bg_pre", c_i32), ("bg_dists", c_vp),
                ("bg_sigma", c_vp), ("bg_rgbs", c_vp), ("bg_weights", c_vp), ("d_bg_rgbs", c_vp), ("d_bg_pre", c_vp),
                ("forward_only", c_i32), ("pad2", c_i32), ("out_opacity", c_vp), ("out_gradient", c_vp),
                ("out_dist", c_vp), ("dyn", c_vp)]


_lib.register("gbsdf_field_args_size", [])
_lib.register("gbsdf_render_args_size", [])
for _name in ("gbsdf_field_fwd", "gbsdf_field_bwd", "gbsdf_field_encode", "gbsdf_field_mlp_fwd",
              "gbsdf_field_mlp_bwd", "gbsdf_field_scatter"):
    _lib.register(_name, [c_vp, c_vp])
_lib.register("gbsdf_render_fused", [c_vp, c_vp])
_lib.register("gbsdf_field_workspace_size", [c_i64, c_i32, c_i32, c_i32, c_vp, c_vp])
_lib.register("gbsdf_rgb_head_fwd", [c_i64, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp])
_lib.register("gbsdf_rgb_head_bwd", [c_i64, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                     c_vp])
_lib.register("gbsdf_app_grad", [c_i64, c_i32, c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_vp, c_vp])
_lib.register("gbsdf_sdf_points", [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_f32, c_vp, c_vp])
_lib.register("gbsdf_wgrad", [c_i64, c_i32, c_i32, c_vp, c_vp, c_i32, c_vp, c_i32, c_vp, c_i32, c_i32, c_vp, c_vp])
_lib.register("gbsdf_bg_encode", [c_i64, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_i32, c_i32, c_vp,
                                  c_vp, c_i32, c_i32, c_vp])
_lib.register("gbsdf_bg_density", [c_i64, c_vp, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp])

BG_X_COLS = 96        # background input: 84 encoding columns, the ones column at 84, zeros
BG_S_COLS = 256 + BG_X_COLS    # [h4 | background input]: the skip layer's input (modules.py:258-261)


def check_struct_sizes():
    lib = _lib.load()
    lib.gbsdf_field_args_size.restype = ctypes.c_size_t
    lib.gbsdf_render_args_size.restype = ctypes.c_size_t
    assert lib.gbsdf_field_args_size() == ctypes.sizeof(FieldArgs), "gbsdf_field_args layout mismatch"
    assert lib.gbsdf_render_args_size() == ctypes.sizeof(RenderArgs), "gbsdf_render_args layout mismatch"


def _p(t):
    return None if t is None else t.data_ptr()


def _round16(n):
    return (n + 15) // 16 * 16


# dense-layer calls of a step, recorded for the launch-shape tuner (autotune.py) when a list
DENSE_CALLS = None


def _dense(X, Wt, N, K, out, bias=None, epi=EPI_IDENTITY, beta=100.0, G=None, err=None, X_lo=None, out_lo=None):
    """out[:, :N] = epi((X + X_lo)[:, :K] @ Wt[:N, :K].T + bias ; G) on the tcgen05 kernel."""
    M = X.shape[0]
    _lib.TIMER.count_bytes("gbsdf_dense", M * (K * 2 * (2 if X_lo is not None else 1) + (N * 2 if G is not None else 0)
                                               + N * out.element_size() * (2 if out_lo is not None else 1)))
    args = (X.shape[0], K, N, c_vp(X.data_ptr()), c_vp(_p(X_lo)), X.stride(0),
            c_vp(Wt.data_ptr()), c_vp(_p(bias)), c_vp(_p(G)), G.stride(0) if G is not None else 0,
            c_vp(out.data_ptr()), c_vp(_p(out_lo)), out.stride(0), 1 if out.dtype == torch.float32 else 0,
            int(epi), float(beta), c_vp(_p(err)), _lib.stream_ptr(X.device))
    if DENSE_CALLS is not None:
        DENSE_CALLS.append(args)
    _lib.call("gbsdf_dense", *args)


def _wgrad(dZ, X, N, K, dW, accumulate=False, dZ_lo=None, err=None):
    """dW[N, K] (+)= (dZ + dZ_lo)[:, :N]^T X[:, :K] (fp32 out) on the tcgen05 weight-gradient kernel."""
    _lib.TIMER.count_bytes("gbsdf_wgrad", dZ.shape[0] * (N * 2 * (2 if dZ_lo is not None else 1) + K * 2))
    _lib.call("gbsdf_wgrad", dZ.shape[0], N, K, c_vp(dZ.data_ptr()), c_vp(_p(dZ_lo)), dZ.stride(0),
              c_vp(X.data_ptr()), X.stride(0), c_vp(dW.data_ptr()), dW.stride(0), 1 if accumulate else 0,
              c_vp(_p(err)), _lib.stream_ptr(dZ.device))


class WeightNormLayer(ctypes.Structure):
    """gbsdf_weightnorm_layer (include/gbsdf.h)."""
    _fields_ = [("rows", c_i64), ("cols", c_i64), ("dW", c_vp), ("ld_dw", c_i64), ("db", c_vp), ("ld_db", c_i64),
                ("v", c_vp), ("g", c_vp), ("dv", c_vp), ("dg", c_vp), ("dbias", c_vp),
                ("acc_v", c_i32), ("acc_g", c_i32), ("acc_b", c_i32), ("pad", c_i32)]


WN_MAX_LAYERS = 16
_lib.register("gbsdf_weightnorm_bwd", [c_i32, c_vp, c_vp, c_f32, c_vp])


class _GradSink:
    """The masters' .grad tensors that gbsdf_weightnorm_bwd writes: an absent one is created
    uninitialised and overwritten (as autograd sets a fresh .grad), a present one is added into."""

    def __init__(self):
        self.seen = {}

    def __call__(self, param):
        key = id(param)
        if key not in self.seen:
            if param.grad is None:
                param.grad = torch.empty_like(param, memory_format=torch.contiguous_format)
                acc = 0
            else:
                if not param.grad.is_contiguous():
                    raise ValueError("gbsdf_weightnorm_bwd writes contiguous gradients")
                acc = 1
            self.seen[key] = (param.grad, acc)
        return self.seen[key]


def _wn_entry(sink, dW, db=None, weight=None, bias=None, v=None, g=None, rows=None):
    """One gbsdf_weightnorm_layer: the weight-norm parameters v, g (weight-norm entry) or the
    plain weight (plain entry), the bias, and the row range ``rows`` (a slice of the
    destination's rows, for gradients assembled from row blocks)."""
    if dW.dim() == 1:
        dW = dW.reshape(1, -1)
    assert dW.stride(1) == 1 and dW.dtype == torch.float32
    e = WeightNormLayer()
    e.rows, e.cols = dW.shape
    e.dW, e.ld_dw = dW.data_ptr(), dW.stride(0)
    sl = rows if rows is not None else slice(0, dW.shape[0])
    if v is not None:
        dv, e.acc_v = sink(v)
        dg, e.acc_g = sink(g)
        e.v, e.g = v.detach()[sl].data_ptr(), g.detach().reshape(-1)[sl].data_ptr()
        e.dv, e.dg = dv[sl].data_ptr(), dg.reshape(-1)[sl].data_ptr()
    else:
        dv, e.acc_v = sink(weight)
        e.dv = dv.reshape(-1, e.cols)[sl].data_ptr()
    if db is not None and bias is not None:
        db = db.reshape(-1)
        assert db.dtype == torch.float32
        dbias, e.acc_b = sink(bias)
        e.db, e.ld_db = db.data_ptr(), db.stride(0)
        e.dbias = dbias.reshape(-1)[sl].data_ptr()
    return e


class WeightNormPack(ctypes.Structure):
    """gbsdf_weightnorm_pack (include/gbsdf.h)."""
    _fields_ = [("rows", c_i64), ("cols", c_i64), ("v", c_vp), ("ld_src", c_i64), ("g", c_vp),
                ("col0", c_i64), ("ncols", c_i64), ("dst16", c_vp), ("ld16", c_i64), ("dst16_lo", c_vp),
                ("dst16T", c_vp), ("ldT", c_i64), ("dst32", c_vp), ("ld32", c_i64)]


_lib.register("gbsdf_weightnorm_fwd", [c_i32, c_vp, c_vp])


def _wsrc(lin):
    """(v, g) of a weight-normalised linear, (weight, None) of a plain one."""
    if hasattr(lin, 'weight_v'):
        return lin.weight_v.detach(), lin.weight_g.detach().reshape(-1)
    return lin.weight.detach(), None


def _pk_entry(src, g=None, col0=0, ncols=None, rows=None, dst16=None, dst16_lo=None, dst16T=None, dst32=None):
    """One gbsdf_weightnorm_pack entry: rows ``rows`` (a slice) of W = g v / ||v|| (src = v; or
    W = src when g is None), columns [col0, col0 + ncols).  Each destination is a view whose
    element (0, 0) takes (first row, col0): dst16 / dst16_lo / dst32 row-major [rows, ncols] (a
    1-D view for one column), dst16T [ncols, rows]."""
    if src.dim() == 1:
        src = src.reshape(-1, 1)
    sl = rows if rows is not None else slice(0, src.shape[0])
    part = src[sl]
    assert src.dtype == torch.float32 and src.stride(1) == 1
    e = WeightNormPack()
    e.rows, e.cols = part.shape[0], src.shape[1]
    e.v, e.ld_src = part.data_ptr(), src.stride(0)
    e.g = g[sl].data_ptr() if g is not None else None
    e.col0 = col0
    e.ncols = ncols if ncols is not None else src.shape[1] - col0

    def rowmajor(t, dt):
        assert t.dtype == dt and (t.dim() == 1 or t.stride(1) == 1)
        return t.data_ptr(), t.stride(0)
    if dst16 is not None:
        e.dst16, e.ld16 = rowmajor(dst16, torch.float16)
        if dst16_lo is not None:
            ptr, ld = rowmajor(dst16_lo, torch.float16)
            assert ld == e.ld16
            e.dst16_lo = ptr
    if dst16T is not None:
        e.dst16T, e.ldT = rowmajor(dst16T, torch.float16)
    if dst32 is not None:
        e.dst32, e.ld32 = rowmajor(dst32, torch.float32)
    return e


def _weightnorm_fwd(entries, device):
    """All pack entries in launches of up to WN_MAX_LAYERS."""
    for i in range(0, len(entries), WN_MAX_LAYERS):
        chunk = entries[i:i + WN_MAX_LAYERS]
        arr = (WeightNormPack * len(chunk))(*chunk)
        _lib.call("gbsdf_weightnorm_fwd", len(chunk), ctypes.cast(arr, c_vp), _lib.stream_ptr(device))


def _weightnorm_bwd(entries, scale, device):
    """All entries in launches of up to WN_MAX_LAYERS; scale a device scalar or a float."""
    sdev = scale.data_ptr() if torch.is_tensor(scale) else None
    sval = 0.0 if torch.is_tensor(scale) else float(scale)
    for i in range(0, len(entries), WN_MAX_LAYERS):
        chunk = entries[i:i + WN_MAX_LAYERS]
        arr = (WeightNormLayer * len(chunk))(*chunk)
        _lib.call("gbsdf_weightnorm_bwd", len(chunk), ctypes.cast(arr, c_vp), c_vp(sdev), sval,
                  _lib.stream_ptr(device))


def active_table_params(sdf):
    """Number of table parameters in the active levels: the levels are stored level-major, so
    the active ones are a prefix of the table, and no kernel reads or writes past it."""
    layout = sdf.tcnn_encoding.layout
    return int(layout.offset[sdf.active_levels]) * layout.n_features


def pack_sdf(sdf, table16=None, bufs=None, entries=None):
    """FP16 working copies of a NeuralSDF's hash table and layer-0 weights (weight norm
    applied) plus the FP32 position columns, bias and head; returns (pk, active, K0).
    An FP32 table is converted over its active levels only, into ``table16`` when given (a
    persistent buffer of the table's size; the inactive levels are left as they are).
    The layer-0 copies are written by gbsdf_weightnorm_fwd into ``bufs`` (zero-initialised
    buffers kept by the caller for this active-level count; fresh ones when None); with
    ``entries`` (a list) the pack entries are appended there for the caller's launch."""
    A = sdf.active_levels
    F = sdf.tcnn_encoding.layout.n_features
    K0 = max(16, _round16(A * F))
    H = sdf.cfg_sdf.mlp.hidden_dim
    l0 = sdf.mlp.linears[0]
    dev = l0.bias.device
    if bufs is None:
        bufs = {}
    if 'w0e' not in bufs:
        bufs['w0e'] = torch.zeros(H, K0, device=dev, dtype=torch.float16)
        bufs['w0b'] = torch.zeros(H, K0 + 16, device=dev, dtype=torch.float16)
        bufs['w0x'] = torch.zeros(H, 3, device=dev, dtype=torch.float32)
    w0e, w0b, w0x = bufs['w0e'], bufs['w0b'], bufs['w0x']
    b0 = l0.bias.detach()
    # w0b: the fp16 encoding columns, then the position columns and bias as fp16 hi/lo pairs
    # matched to the x0ext tail (x hi, 1, x lo, 1, x hi): w hi, b hi, w hi, b lo, w lo.  The
    # products sum to w0x x + b0 to ~2^-20 relative, so the pre-activation keeps FP32 accuracy.
    v, g = _wsrc(l0)
    ents = [_pk_entry(v, g, col0=3, ncols=A * F, dst16=w0e),
            _pk_entry(v, g, col0=3, ncols=A * F, dst16=w0b),
            _pk_entry(v, g, col0=0, ncols=3, dst16=w0b[:, K0:], dst16_lo=w0b[:, K0 + 8:], dst32=w0x),
            _pk_entry(v, g, col0=0, ncols=3, dst16=w0b[:, K0 + 4:]),
            _pk_entry(b0, None, dst16=w0b[:, K0 + 3], dst16_lo=w0b[:, K0 + 7])]
    if entries is not None:
        entries += ents
    else:
        _weightnorm_fwd(ents, dev)
    params = sdf.tcnn_encoding.params.detach()
    if params.dtype == torch.float16:
        table = params
    else:
        n = active_table_params(sdf)
        table = table16 if table16 is not None else torch.empty(max(n, 1), device=params.device,
                                                                dtype=torch.float16)
        table[:n].copy_(params[:n])
    pk = dict(table=table, w0e=w0e, w0b=w0b, w0x=w0x, b0=b0,
              whead=sdf.mlp.linear_sdf.weight.detach()[0],
              bhead=sdf.mlp.linear_sdf.bias.detach())
    return pk, A, K0


def sdf_weight_args(sdf, pk, A, K0, err=None):
    """A FieldArgs carrying only the SDF weights (for gbsdf_sdf_points)."""
    fa = FieldArgs()
    fa.grid = sdf.tcnn_encoding.layout.struct
    fa.active, fa.K0 = A, K0
    fa.table, fa.w0e, fa.w0b = _p(pk['table']), _p(pk['w0e']), _p(pk['w0b'])
    fa.w0x, fa.b0, fa.whead, fa.bhead = _p(pk['w0x']), _p(pk['b0']), _p(pk['whead']), _p(pk['bhead'])
    fa.beta = float(sdf.cfg_sdf.mlp.activ_params.beta)
    fa.err = _p(err)
    return fa


class FusedField:
    """Fused FP16 forward+backward over a FieldModel's FP32 master parameters."""

    def __init__(self, model, loss_scale=2.0 ** 15, split_colour_grads=False, fused_w0_grad=True,
                 activation_pairs=True, dynamic_loss_scale=True, growth_interval=2000, deterministic_table=False):
        check_struct_sizes()
        self.model = model
        # the table gradient through the order-independent fixed-point scatter (bit-identical
        # across runs; an int64 buffer of the table's size besides the FP32 gradient)
        self.deterministic = bool(deterministic_table)
        # launch shapes chosen by autotune.StepTuner (results unchanged): scatter_cpt, fwd_ctas
        self.tuning = {}
        # dynamic loss scaling: the scale, the schedule scalars and the overflow flag in one device
        # buffer (created at the first step): [0] loss scale, [1] anneal, [2] curvature weight,
        # [3] 1 / loss scale, [4] found_inf; an int32 growth tracker beside it
        self.dynamic = bool(dynamic_loss_scale)
        self.growth_interval = int(growth_interval)
        self._scal = self._growth = self._one = None
        # forward activations that feed another layer's forward stored as fp16 hi + lo pairs
        # (the SDF layer-0 output, the colour input, the colour hidden layers but the last):
        # with single fp16 storage the next layer's pre-activations move by the fp16 rounding
        # and single weight gradients miss the float64 oracle by up to ~4e-3; with the pairs
        # they agree to ~1e-7 in the oracle's own emulation.  The weight gradients read the hi
        # halves only (that costs <= 2e-4).  False: single fp16 storage (faster, less accurate).
        self.pairs = bool(activation_pairs)
        # the layer-0 weight gradient: accumulated by the backward kernel itself (K0 <= 64), or
        # (False, or K0 > 64) from the kernel's fp16 d_pre0 rows by the weight-gradient kernel
        self.fused_w0_grad = bool(fused_w0_grad)
        # carry the colour MLP's input gradients as fp16 hi+lo pairs (costs ~9% of the step and
        # leaves the weight-gradient error unchanged: that comes from fp16 storage of the
        # forward activations, whose rounding moves ReLU gates near zero)
        self.split = bool(split_colour_grads)
        self.loss_scale = float(loss_scale)
        sdf = model.neural_sdf
        cfg = model.cfg
        self.H = cfg.sdf.mlp.hidden_dim
        if self.H != 256:
            raise ValueError("the fused field is built for SDF hidden width 256")
        if cfg.sdf.gradient.taps not in (4, 6) or cfg.sdf.gradient.mode != "numerical":
            raise ValueError("the fused field implements the 6- and 4-tap numerical gradients")
        self.taps = int(cfg.sdf.gradient.taps)
        # samples per 128-row tile and rows used: 18 x 7 (6 taps) or 25 x 5 (4 taps)
        self.spt, self.tile_rows = (18, 126) if self.taps == 6 else (25, 125)
        if cfg.sdf.mlp.skip or cfg.sdf.mlp.num_layers != 1:
            raise ValueError("the fused field implements the one-hidden-layer SDF MLP of the reference config")
        rgb = cfg.rgb
        if rgb.mode != "idr" or rgb.mlp.skip or rgb.encoding_view.levels != 3:
            raise ValueError("the fused colour MLP implements mode 'idr' with SH degree 3 and no skips")
        self.Hc = rgb.mlp.hidden_dim
        if self.Hc not in (128, 256):
            raise ValueError("colour hidden width must be 128 or 256")
        self.n_rgb_hidden = rgb.mlp.num_layers
        self.app_dim = cfg.appear_embed.dim if cfg.appear_embed.enabled else 0
        self.tail = 22 + self.app_dim                  # x 3, SH 16, normal 3, app
        self.Kc0 = 256 + _round16(self.tail + 1)       # + a padding column of ones (bias gradient)
        self.F = sdf.tcnn_encoding.layout.n_features
        self.L = sdf.tcnn_encoding.layout.n_levels
        self.bg = bool(getattr(model, "with_background", False))
        if self.bg:
            cb = cfg.background
            mb = cb.mlp
            ok = (mb.num_layers == 8 and list(mb.skip) == [4] and mb.hidden_dim == 256 and mb.num_layers_rgb == 2
                  and mb.hidden_dim_rgb in (64, 128, 256) and mb.activ == "relu" and not mb.activ_params
                  and mb.activ_density == "softplus" and not mb.activ_density_params and cb.view_dep
                  and cb.encoding.type == "fourier" and cb.encoding.levels == 10
                  and cb.encoding_view.type == "spherical" and cb.encoding_view.levels == 3 and not cb.white)
            if not ok:
                raise ValueError("the fused background NeRF implements the reference's base configuration "
                                 "(8 x 256 ReLU with a skip at 4, softplus density, 10 Fourier levels, SH 3)")
            self.n_bg = int(cb.samples)
            self.Hbr = int(mb.hidden_dim_rgb)
            self.Kr0 = 256 + _round16(16 + self.app_dim + 1)   # [feat | SH 16, app, 1 | 0]
        self.ws = None
        self.err = None
        self._table16 = None          # persistent fp16 working copy of an FP32 table
        self._pkbuf = None            # persistent weight copies (per active-level count)

    # ------------------------------------------------------------------ parameters
    def _pack(self):
        """Working copies of the FP32 masters (weight norm applied) for this step: the fp16
        table over the active levels, and every MLP weight copy (fp16, transposed, reordered)
        from gbsdf_weightnorm_fwd into buffers kept across steps."""
        m = self.model
        sdf = m.neural_sdf
        params = sdf.tcnn_encoding.params
        if params.dtype != torch.float16 and (self._table16 is None or self._table16.numel() != params.numel()
                                               or self._table16.device != params.device):
            self._table16 = torch.zeros(params.numel(), device=params.device, dtype=torch.float16)
        key = (sdf.active_levels, params.device)
        if self._pkbuf is None or self._pkbuf['key'] != key:
            self._pkbuf = dict(key=key)            # zero-initialised: padding columns stay zero
        bufs = self._pkbuf
        ents = []
        pk, self.A, self.K0 = pack_sdf(sdf, self._table16, bufs, ents)
        dev = params.device
        f16 = torch.float16
        z = lambda *sh: torch.zeros(*sh, device=dev, dtype=f16)  # noqa: E731
        lins = m.neural_rgb.mlp.linears
        l1 = sdf.mlp.linears[1]
        Hc, n_hid = self.Hc, self.n_rgb_hidden
        if 'w1' not in bufs:
            bufs['w1'], bufs['w1T'] = z(*l1.bias.shape, l1.in_features), z(l1.in_features, *l1.bias.shape)
            bufs['wc'] = [z(Hc, self.Kc0)] + [z(Hc, Hc) for _ in range(1, n_hid)]
            bufs['wcT'] = [None] + [z(Hc, Hc) for _ in range(1, n_hid)]
            bufs['wc0T_feat'], bufs['wc0T_tail'] = z(256, Hc), z(64, Hc)
            bufs['wl'] = torch.zeros(lins[-1].bias.shape[0], Hc, device=dev, dtype=torch.float32)
        v, g = _wsrc(l1)
        ents.append(_pk_entry(v, g, dst16=bufs['w1'], dst16T=bufs['w1T']))
        # colour layer 0 columns reordered to [feat 256 | x 3, SH 16, n 3, app | 0] from the
        # reference's [x 3 | SH 16 | n 3 | feat 256 | app]
        sh = 16
        wc0, t_tail = bufs['wc'][0], bufs['wc0T_tail']
        v, g = _wsrc(lins[0])
        ents.append(_pk_entry(v, g, col0=6 + sh, ncols=256, dst16=wc0[:, :256], dst16T=bufs['wc0T_feat']))
        ents.append(_pk_entry(v, g, col0=0, ncols=6 + sh, dst16=wc0[:, 256:256 + 6 + sh], dst16T=t_tail[:6 + sh]))
        if self.app_dim:
            ents.append(_pk_entry(v, g, col0=6 + sh + 256, ncols=self.app_dim,
                                  dst16=wc0[:, 256 + 6 + sh:256 + 6 + sh + self.app_dim],
                                  dst16T=t_tail[6 + sh:6 + sh + self.app_dim]))
        for i in range(1, n_hid):
            v, g = _wsrc(lins[i])
            ents.append(_pk_entry(v, g, dst16=bufs['wc'][i], dst16T=bufs['wcT'][i]))
        v, g = _wsrc(lins[-1])
        ents.append(_pk_entry(v, g, dst32=bufs['wl']))
        pk['w1'], pk['w1T'], pk['b1'] = bufs['w1'], bufs['w1T'], l1.bias.detach()
        pk['wc'], pk['wcT'] = bufs['wc'], bufs['wcT']
        pk['bc'] = [lins[i].bias.detach() for i in range(n_hid)]
        pk['wc0T_feat'], pk['wc0T_tail'] = bufs['wc0T_feat'], t_tail          # [256, Hc], [64, Hc]
        pk['wl'], pk['bl'] = bufs['wl'], lins[-1].bias.detach()
        pk['s_var'] = m.s_var.detach().reshape(1)
        pk['app'] = m.appear_embed.weight.detach() if self.app_dim else None
        if self.bg:
            self._pack_background(pk, bufs, ents)
        _weightnorm_fwd(ents, dev)
        self.pk = pk

    def _pack_background(self, pk, bufs, ents):
        """Working copies of the background NeRF (no weight norm), laid out for the dense
        kernel: layer 0 padded to the 96-column input, the skip layer over [h4 | input], the
        last layer split into its 256 feature rows and the density row (modules.py:258-264);
        pack entries appended to ``ents``."""
        bgm = self.model.background_nerf
        L, Lr = bgm.mlp_feat.linears, bgm.mlp_rgb.linears
        dev = L[0].weight.device
        Hbr, Kr0 = self.Hbr, self.Kr0
        nin = 256 + 16 + self.app_dim
        z = lambda *sh: torch.zeros(*sh, device=dev, dtype=torch.float16)  # noqa: E731
        if 'bw' not in bufs:
            bufs['bw'] = [z(256, BG_X_COLS)] + [z(256, 256) for _ in range(3)] + [z(256, BG_S_COLS)] + \
                         [z(256, 256) for _ in range(3)]
            bufs['bwT'] = [None] + [z(256, 256) for _ in range(6)]
            bufs['bw7extT'] = z(256, 272)
            bufs['bwr0'], bufs['bwr0T_feat'], bufs['bwr0T_tail'] = z(Hbr, Kr0), z(256, Hbr), z(64, Hbr)
        w, wT = bufs['bw'], bufs['bwT']
        W = lambda i: L[i].weight.detach()  # noqa: E731
        ents.append(_pk_entry(W(0), ncols=84, dst16=w[0][:, :84]))
        for i in (1, 2, 3, 5, 6):
            ents.append(_pk_entry(W(i), dst16=w[i], dst16T=wT[i]))
        ents.append(_pk_entry(W(4), ncols=340, dst16=w[4][:, :340]))
        ents.append(_pk_entry(W(4), ncols=256, dst16T=wT[4]))
        # layer 7: feature rows 1-256 (row-major and transposed), the density row transposed only
        ents.append(_pk_entry(W(7), rows=slice(1, 257), dst16=w[7], dst16T=bufs['bw7extT'][:, :256]))
        ents.append(_pk_entry(W(7), rows=slice(0, 1), dst16T=bufs['bw7extT'][:, 256:257]))
        Wr0 = Lr[0].weight.detach()                                       # [feat | SH | app]: same order
        ents.append(_pk_entry(Wr0, ncols=256, dst16=bufs['bwr0'][:, :256], dst16T=bufs['bwr0T_feat']))
        ents.append(_pk_entry(Wr0, col0=256, ncols=nin - 256, dst16=bufs['bwr0'][:, 256:nin],
                              dst16T=bufs['bwr0T_tail'][:nin - 256]))
        b = [L[i].bias.detach() for i in range(7)] + [L[7].bias.detach()[1:]]
        pk['bw'], pk['bb'] = w, b
        pk['bw7d'] = W(7)[0]
        pk['bb7d'] = L[7].bias.detach()[:1]
        pk['bwT'] = wT                                                     # input-gradient operands (W^T)
        pk['bw7extT'] = bufs['bw7extT']                                    # [256, 272]
        pk['bwr0'], pk['bbr0'] = bufs['bwr0'], Lr[0].bias.detach()
        pk['bwr0T_feat'], pk['bwr0T_tail'] = bufs['bwr0T_feat'], bufs['bwr0T_tail']   # [256, Hbr], [64, Hbr]
        pk['bwr1'] = Lr[1].weight.detach()                                 # [3, Hbr]
        pk['bbr1'] = Lr[1].bias.detach()
        ae = self.model.appear_embed_outside
        pk['app_bg'] = ae.weight.detach() if ae is not None else None

    # ------------------------------------------------------------------ workspace
    def _in_kernel_w0_grad(self):
        return self.fused_w0_grad and self.K0 <= 64

    def _workspace(self, R, S, Ns, device):
        key = (R, S, Ns, self.K0, self.bg, self.pairs, self.deterministic)
        if self.ws is not None and self.ws['key'] == key:
            return self.ws
        self.ws = None                      # release the previous shape's buffers first
        # the caller-owned buffers of the field calls, sized by the library
        wsz = FieldWorkspace()
        lay = self.model.neural_sdf.tcnn_encoding.layout
        _lib.call("gbsdf_field_workspace_size", Ns, self.K0, self.taps, 1 if self.deterministic else 0,
                  ctypes.byref(lay.struct), ctypes.byref(wsz))
        rows0 = int(wsz.rows)                                        # layer-0 rows, tile-major
        assert rows0 == (Ns + self.spt - 1) // self.spt * self.tile_rows
        f16, f32 = torch.float16, torch.float32
        e = lambda *s, dt=f32: torch.empty(*s, device=device, dtype=dt)  # noqa: E731
        Hc = self.Hc
        ws = dict(key=key)
        ws.update(sdf=e(Ns), grad=e(Ns, 3), hess=e(Ns, 3), h0c=self._with_ones(e(Ns, 264, dt=f16), 256),
                  xc=e(Ns, self.Kc0, dt=f16),
                  ys=[self._with_ones(e(Ns, Hc + 8, dt=f16), Hc) for _ in range(self.n_rgb_hidden)],
                  rgbs=e(Ns, 3), rgb=e(R, 3),
                  weights=e(Ns), d_rgbs=e(Ns, 3), d_sdf=e(Ns), d_grad=e(Ns, 3), d_hess=e(Ns, 3),
                  loss_sums=torch.zeros(4, device=device, dtype=torch.float64), d_s_var=torch.zeros(1, device=device),
                  d_wl=torch.zeros(3, Hc, device=device), dzs=[e(Ns, Hc, dt=f16) for _ in range(2)],
                  dzs_lo=[e(Ns, Hc, dt=f16) for _ in range(2)] if self.split else None,
                  dzfeat=e(Ns, 256, dt=f16), dzfeat_lo=e(Ns, 256, dt=f16) if self.split else None,
                  dxc_tail=e(Ns, 64), d_h0c=e(Ns, 256),
                  # K0 <= 64: the backward kernel accumulates dW0 itself; otherwise d_pre0 -> k_wgrad
                  d_pre0=None if self._in_kernel_w0_grad() else e(rows0, 256, dt=f16),
                  d_pre0_lo=None if self._in_kernel_w0_grad() else e(rows0, 256, dt=f16),
                  d_w0=e(256, self.K0 + 16) if self._in_kernel_w0_grad() else None,
                  x0ext=e(rows0, 2 * self.K0 + 16, dt=f16), d_enc=e(rows0, self.K0),
                  d_whead=torch.zeros(256, device=device),
                  d_bhead=torch.zeros(1, device=device), d_bl=torch.zeros(3, device=device),
                  err=torch.zeros(1, device=device, dtype=torch.int32),
                  d_table_fix=(torch.empty(wsz.d_table_fix_bytes // 8, device=device, dtype=torch.int64)
                               if self.deterministic else None))
        if self.pairs:
            # low halves, with the row strides of their hi buffers (the constant-1 column's lo is 0)
            ws.update(h0c_lo=e(Ns, 264, dt=f16).zero_(), xc_lo=e(Ns, self.Kc0, dt=f16),
                      ys_lo=[e(Ns, Hc + 8, dt=f16) for _ in range(self.n_rgb_hidden - 1)])
        else:
            ws.update(h0c_lo=None, xc_lo=None, ys_lo=[None] * (self.n_rgb_hidden - 1))
        if self.bg:
            Nb = R * self.n_bg
            Hbr = self.Hbr
            ws.update(bg_S=e(Nb, BG_S_COLS, dt=f16),
                      bg_h={i: self._with_ones(e(Nb, 264, dt=f16), 256) for i in (1, 2, 3, 5, 6, 7)},
                      bg_G=e(Nb, self.Kr0, dt=f16), bg_hr=self._with_ones(e(Nb, Hbr + 8, dt=f16), Hbr),
                      bg_sigma=e(Nb), bg_rgbs=e(Nb, 3), bg_weights=e(Nb), bg_d_rgbs=e(Nb, 3),
                      bg_dZ7=torch.zeros(Nb, 272, device=device, dtype=f16), bg_dz_r=e(Nb, Hbr, dt=f16),
                      bg_dz=[e(Nb, 256, dt=f16) for _ in range(2)],
                      bg_d_tail=e(Nb, 64) if self.app_dim else None, bg_d_bl=torch.zeros(3, device=device))
            if self.pairs:
                # low halves of every background activation that feeds another layer's forward
                # (or the density head); the colour hidden layer feeds the FP32 head only
                z = lambda *sh: torch.zeros(*sh, device=device, dtype=f16)  # noqa: E731
                ws.update(bg_S_lo=z(Nb, BG_S_COLS), bg_h_lo={i: z(Nb, 264) for i in (1, 2, 3, 5, 6, 7)},
                          bg_G_lo=z(Nb, self.Kr0),
                          # the backward's input gradients too: they pass through up to eight layers
                          # (the density column of dZ7 stays a single fp16 value: its lo is 0)
                          bg_dz_r_lo=z(Nb, Hbr), bg_dZ7_lo=z(Nb, 272), bg_dz_lo=[z(Nb, 256) for _ in range(2)])
            else:
                ws.update(bg_S_lo=None, bg_h_lo={i: None for i in (1, 2, 3, 5, 6, 7)}, bg_G_lo=None,
                          bg_dz_r_lo=None, bg_dZ7_lo=None, bg_dz_lo=[None, None])
        self.ws = ws
        return ws

    @staticmethod
    def _with_ones(t, col):
        """Activation buffer [Ns, H + 8] whose column H is a constant 1 (written once): the
        weight-gradient GEMM dZ^T [y | 1] then yields the next layer's bias gradient too."""
        t[:, col:] = 0
        t[:, col] = 1
        return t

    # ------------------------------------------------------------------ step
    def render(self, batch):
        """Forward only (evaluation, Model.render_rays with training off, model.py:124-190):
        the same kernels with the render kernel's losses and backward switched off.
        Returns per-ray rgb [R,3], opacity [R,1] (object samples), gradient [R,3] (the
        weights' composite of the unnormalised object gradients) and dist [R,1] (composite
        of the distances over object and background samples).  ``target`` may be absent."""
        return self.step(batch, compute_loss=False, _evaluate=True)

    def step(self, batch, compute_loss=True, _evaluate=False, _refresh=True):
        """Forward + backward on a batch (same keys as FieldModel.render_step).

        Ragged batches pass ``ray_offsets`` [R+1] (int64) and flat ``dists`` [Ns];
        dense batches pass ``dists`` [R, S].  Returns a dict with the loss terms
        (python floats when compute_loss) and writes FP32 ``.grad`` into the model."""
        m = self.model
        sdfm = m.neural_sdf
        dev = batch['center'].device
        self._pack()
        pk = self.pk
        dists = batch['dists']
        R = batch['center'].shape[0]
        ragged = 'ray_offsets' in batch
        if ragged:
            offs = batch['ray_offsets']
            Ns = int(dists.numel())
            S = 0
            sample_ray = batch['sample_ray']
        else:
            S = dists.shape[1]
            Ns = R * S
            offs = None
            sample_ray = None
        ws = self._workspace(R, S, Ns, dev)
        scal = self._scalars(dev) if self.dynamic else None
        if scal is not None:
            if _refresh:
                self.refresh_scalars()
            scal[4:5].zero_()                                        # found_inf of this step
            torch.reciprocal(scal[0:1], out=scal[3:4])               # 1 / loss scale
        dists_f = dists.reshape(-1).contiguous().float()
        center = batch['center'].contiguous().float()
        ray_unit = batch['ray_unit'].contiguous().float()
        far = batch['far'].reshape(-1).contiguous().float()
        outside = batch['outside'].reshape(-1).to(torch.uint8).contiguous()
        target = batch['target'].contiguous().float() if 'target' in batch else None
        app_idx = batch['app_idx'].to(torch.int32).contiguous() if self.app_dim else None
        stream = _lib.stream_ptr(dev)
        eps = float(sdfm.normal_eps)
        lay = sdfm.tcnn_encoding.layout
        Hc = self.Hc
        ws['err'].zero_()

        fa = FieldArgs()
        fa.Ns, fa.S = Ns, S
        fa.sample_ray = _p(sample_ray)
        fa.center, fa.ray_unit, fa.dists, fa.outside = _p(center), _p(ray_unit), _p(dists_f), _p(outside)
        fa.app_idx = _p(app_idx)
        fa.grid = lay.struct
        fa.active, fa.K0 = self.A, self.K0
        fa.table, fa.w0e, fa.w0b = _p(pk['table']), _p(pk['w0e']), _p(pk['w0b'])
        fa.w0x, fa.b0, fa.whead, fa.bhead = _p(pk['w0x']), _p(pk['b0']), _p(pk['whead']), _p(pk['bhead'])
        fa.beta = float(m.cfg.sdf.mlp.activ_params.beta)
        fa.taps = self.taps
        if self.taps == 6:
            fa.eps = eps
            fa.two_eps = float(torch.tensor(2 * eps, dtype=torch.float32))
            fa.eps2 = float(torch.tensor(eps ** 2, dtype=torch.float32))
        else:
            # the tetrahedral stencil's displacement and denominators as the reference forms them
            # (modules.py:158-174): eps / sqrt(3) in double, then float32 scalars
            e = eps / float(np.sqrt(3.0))
            fa.eps = e
            fa.two_eps = float(torch.tensor(4.0 * e, dtype=torch.float32))
            fa.eps2 = float(torch.tensor(e ** 2, dtype=torch.float32))
        fa.outside_val = float(m.outside_val)
        fa.xc, fa.ldxc = _p(ws['xc']), self.Kc0
        fa.app_dim, fa.app_table = self.app_dim, _p(pk['app'])
        fa.sdf, fa.grad, fa.hess, fa.h0c = _p(ws['sdf']), _p(ws['grad']), _p(ws['hess']), _p(ws['h0c'])
        fa.ld_h0c = ws['h0c'].stride(0)
        fa.h0c_lo, fa.xc_lo = _p(ws['h0c_lo']), _p(ws['xc_lo'])
        fa.x0ext = _p(ws['x0ext'])
        fa.err = _p(ws['err'])
        fa.scatter_cpt = int(self.tuning.get('scatter_cpt', 0))
        fa.fwd_ctas = int(self.tuning.get('fwd_ctas', 0))
        self._fa = fa                      # the field calls' arguments of the last step (the tuner re-issues them)
        # ---------------- forward ----------------
        _lib.call("gbsdf_field_encode", ctypes.byref(fa), stream)     # = gbsdf_field_fwd in two calls
        _lib.call("gbsdf_field_mlp_fwd", ctypes.byref(fa), stream)
        # SDF feature layer, written into the colour input's first 256 columns
        _dense(ws['h0c'], pk['w1'], 256, 256, ws['xc'], bias=pk['b1'], epi=EPI_SOFTPLUS, beta=fa.beta,
               err=ws['err'], X_lo=ws['h0c_lo'], out_lo=ws['xc_lo'])
        X, Xl, K = ws['xc'], ws['xc_lo'], self.Kc0
        n_last = self.n_rgb_hidden - 1
        for i in range(self.n_rgb_hidden):
            # the last hidden layer feeds only the FP32 colour head: single fp16 storage suffices
            Yl = ws['ys_lo'][i] if i < n_last else None
            _dense(X, pk['wc'][i], Hc, K, ws['ys'][i], bias=pk['bc'][i], epi=EPI_RELU, err=ws['err'], X_lo=Xl,
                   out_lo=Yl)
            X, Xl, K = ws['ys'][i], Yl, Hc
        ylast = ws['ys'][-1]
        _lib.TIMER.count_bytes("gbsdf_rgb_head_fwd", Ns * (Hc * 2 + 12))
        _lib.call("gbsdf_rgb_head_fwd", Ns, c_vp(ylast.data_ptr()), ylast.stride(0), Hc, c_vp(pk['wl'].data_ptr()),
                  c_vp(pk['bl'].data_ptr()), c_vp(ws['rgbs'].data_ptr()), stream)
        dists_bg = None
        if self.bg:
            dists_bg = batch['dists_bg'].reshape(-1).contiguous().float()
            if dists_bg.numel() != R * self.n_bg:
                raise ValueError(f"dists_bg must hold {self.n_bg} background samples per ray")
            self._background_forward(R, center, ray_unit, dists_bg, app_idx, stream)
        # ---------------- render + losses, fwd + bwd ----------------
        lw = m.cfg.loss_weight
        n_mean = batch.get('mean_count', Ns)
        ra = RenderArgs()
        ra.R, ra.S = R, S
        ra.ray_offsets = _p(offs)
        ra.ray_unit, ra.dists, ra.far, ra.outside, ra.target = _p(ray_unit), _p(dists_f), _p(far), _p(outside), \
            _p(target)
        ra.s_var = _p(pk['s_var'])
        ra.sdf, ra.grad, ra.hess, ra.rgbs = _p(ws['sdf']), _p(ws['grad']), _p(ws['hess']), _p(ws['rgbs'])
        ra.anneal = min(m.progress / m.anneal_end, 1.0)
        ra.w_render, ra.w_eik, ra.w_curv = float(lw.render), float(lw.eikonal), float(m.w_curv or 0.0)
        ra.l1_scale = 3.0 / (3.0 * R)
        ra.mean_scale = 1.0 / n_mean
        ra.loss_scale = self.loss_scale
        ra.dyn = _p(scal)
        ra.rgb, ra.weights = _p(ws['rgb']), _p(ws['weights'])
        ra.d_rgbs, ra.d_sdf, ra.d_grad, ra.d_hess = _p(ws['d_rgbs']), _p(ws['d_sdf']), _p(ws['d_grad']), \
            _p(ws['d_hess'])
        ws['d_s_var'].zero_()
        ws['loss_sums'].zero_()
        ra.d_s_var, ra.loss_sums = _p(ws['d_s_var']), _p(ws['loss_sums'])
        ra.err = _p(ws['err'])
        if self.bg:
            ra.n_bg, ra.ld_d_bg_pre = self.n_bg, ws['bg_dZ7'].stride(0)
            ra.bg_dists, ra.bg_sigma, ra.bg_rgbs = _p(dists_bg), _p(ws['bg_sigma']), _p(ws['bg_rgbs'])
            ra.bg_weights, ra.d_bg_rgbs = _p(ws['bg_weights']), _p(ws['bg_d_rgbs'])
            ra.d_bg_pre = ws['bg_dZ7'][:, 256:].data_ptr()             # column 256: the density row of layer 7
        if _evaluate:
            ev = dict(opacity=torch.empty(R, 1, device=dev), gradient=torch.empty(R, 3, device=dev),
                      dist=torch.empty(R, 1, device=dev))
            ra.forward_only = 1
            ra.out_opacity, ra.out_gradient, ra.out_dist = _p(ev['opacity']), _p(ev['gradient']), _p(ev['dist'])
            _lib.call("gbsdf_render_fused", ctypes.byref(ra), stream)
            ev['rgb'] = ws['rgb'].clone()
            return ev
        _lib.call("gbsdf_render_fused", ctypes.byref(ra), stream)
        # ---------------- colour MLP backward ----------------
        ws['d_bl'].zero_()
        ws['d_wl'].zero_()
        dz = ws['dzs'][0]
        # Y row in, dZ row (and its lo half) out, the per-sample colour and its gradient
        _lib.TIMER.count_bytes("gbsdf_rgb_head_bwd", Ns * (Hc * 2 * (3 if self.split else 2) + 24))
        _lib.call("gbsdf_rgb_head_bwd", Ns, c_vp(ylast.data_ptr()), ylast.stride(0), Hc, c_vp(pk['wl'].data_ptr()),
                  c_vp(ws['rgbs'].data_ptr()), c_vp(ws['d_rgbs'].data_ptr()), None,
                  c_vp(dz.data_ptr()), c_vp(_p(ws['dzs_lo'][0] if self.split else None)), c_vp(ws['d_bl'].data_ptr()),
                  c_vp(ws['d_wl'].data_ptr()), stream)
        grads = {}
        dev32 = dict(device=dev, dtype=torch.float32)
        n = self.n_rgb_hidden
        # the last colour layer's weight gradient came with its backward
        grads['wl'], grads['bl'] = ws['d_wl'], ws['d_bl']
        cur = 0
        for i in range(n - 1, 0, -1):
            dzi = ws['dzs'][cur]
            gw = torch.empty(Hc, Hc + 8, **dev32)
            _wgrad(dzi, ws['ys'][i - 1], Hc, Hc + 8, gw, err=ws['err'])   # column Hc: the bias gradient
            grads[f'wc{i}'], grads[f'bc{i}'] = gw[:, :Hc], gw[:, Hc]
            nxt = ws['dzs'][1 - cur]
            _dense(dzi, pk['wcT'][i], Hc, Hc, nxt, epi=EPI_DRELU, G=ws['ys'][i - 1], err=ws['err'],
                   X_lo=ws['dzs_lo'][cur] if self.split else None,
                   out_lo=ws['dzs_lo'][1 - cur] if self.split else None)
            cur = 1 - cur
        dz0 = ws['dzs'][cur]
        dz0_lo = ws['dzs_lo'][cur] if self.split else None
        gw0 = torch.empty(Hc, self.Kc0, **dev32)
        _wgrad(dz0, ws['xc'], Hc, self.Kc0, gw0, err=ws['err'])   # last column: the bias gradient
        grads['wc0'], grads['bc0'] = gw0, gw0[:, self.Kc0 - 1]
        # input gradient of colour layer 0: feature part through softplus', tail (x, SH, n, app) as is
        _dense(dz0, pk['wc0T_feat'], 256, Hc, ws['dzfeat'], epi=EPI_DSOFTPLUS, beta=fa.beta, G=ws['xc'],
               err=ws['err'], X_lo=dz0_lo, out_lo=ws['dzfeat_lo'] if self.split else None)
        _dense(dz0, pk['wc0T_tail'], 64, Hc, ws['dxc_tail'], epi=EPI_IDENTITY, err=ws['err'], X_lo=dz0_lo)
        # SDF feature layer
        gw1 = torch.empty(256, 264, **dev32)
        _wgrad(ws['dzfeat'], ws['h0c'], 256, 264, gw1, err=ws['err'])   # column 256: the bias gradient
        grads['w1'], grads['b1'] = gw1[:, :256], gw1[:, 256]
        _dense(ws['dzfeat'], pk['w1T'], 256, 256, ws['d_h0c'], epi=EPI_IDENTITY, err=ws['err'],
               X_lo=ws['dzfeat_lo'] if self.split else None)
        if self.app_dim:
            g_app = torch.zeros_like(pk['app'])
            _lib.call("gbsdf_app_grad", R, S, c_vp(_p(offs)), c_vp(app_idx.data_ptr()),
                      c_vp(ws['dxc_tail'].data_ptr()), 64, 22, self.app_dim, c_vp(g_app.data_ptr()), stream)
            grads['app'] = g_app
        # ---------------- field backward ----------------
        # the table gradient is scattered straight into the FP32 master's .grad (accumulating, as
        # autograd does), already unscaled; an fp16 table gets a separate FP32 buffer
        table = sdfm.tcnn_encoding.params
        self._table_in_place = table.dtype == torch.float32
        if self._table_in_place:
            if table.grad is None:
                table.grad = torch.zeros_like(table)
            d_table = table.grad
        else:
            d_table = torch.zeros(table.shape, device=dev, dtype=torch.float32)
        fa.d_table_scale = 1.0 / self.loss_scale
        fa.d_table_scale_dev = scal[3:4].data_ptr() if scal is not None else None
        fa.found_inf = scal[4:5].data_ptr() if scal is not None else None
        ws['d_whead'].zero_()
        ws['d_bhead'].zero_()
        fa.d_sdf, fa.d_grad, fa.d_hess = _p(ws['d_sdf']), _p(ws['d_grad']), _p(ws['d_hess'])
        fa.d_xc, fa.ld_dxc, fa.normal_col = _p(ws['dxc_tail']), 64, 19
        fa.d_h0c = _p(ws['d_h0c'])
        fa.d_table, fa.d_pre0, fa.d_enc = _p(d_table), _p(ws['d_pre0']), _p(ws['d_enc'])
        fa.d_pre0_lo = _p(ws['d_pre0_lo'])
        fa.d_table_fix = _p(ws['d_table_fix'])
        fa.d_whead, fa.d_bhead = _p(ws['d_whead']), _p(ws['d_bhead'])
        if ws['d_w0'] is not None:
            ws['d_w0'].zero_()
        fa.d_w0 = _p(ws['d_w0'])
        _lib.call("gbsdf_field_mlp_bwd", ctypes.byref(fa), stream)    # = gbsdf_field_bwd in two calls
        _lib.call("gbsdf_field_scatter", ctypes.byref(fa), stream)
        if ws['d_w0'] is not None:
            grads['w0ext'] = ws['d_w0']                               # [256, K0 + 16], lo folded in
        else:
            gw0x = torch.empty(256, 2 * self.K0 + 16, **dev32)
            # d_pre as its hi + lo pair against every x0ext column (features hi, tail, features lo)
            _wgrad(ws['d_pre0'], ws['x0ext'], 256, 2 * self.K0 + 16, gw0x, dZ_lo=ws['d_pre0_lo'], err=ws['err'])
            grads['w0ext'] = gw0x
        grads['table'] = d_table
        if self.bg:
            grads['bg'] = self._background_backward(R, app_idx, stream)
        self._scatter_grads(grads)
        if scal is not None:
            self._check_and_update_scale(scal)
        self._loss_norm = (R, n_mean, float(lw.render), float(lw.eikonal))
        out = self.losses() if compute_loss else {}
        out['rgb'] = ws['rgb']
        return out

    # ------------------------------------------------------------------ background NeRF
    def _background_forward(self, R, center, ray_unit, dists_bg, app_idx, stream):
        """BackgroundNeRF.forward (modules.py:268-284) of the R x n_bg background samples:
        encode -> 8 ReLU layers with the input concatenated at layer 4 -> density head and
        256 features -> [features, SH(d), app] -> ReLU -> sigmoid colour."""
        ws, pk = self.ws, self.pk
        NB, Nb, Hbr, Kr0 = self.n_bg, R * self.n_bg, self.Hbr, self.Kr0
        S, G, h = ws['bg_S'], ws['bg_G'], ws['bg_h']
        Sl, Gl, hl = ws['bg_S_lo'], ws['bg_G_lo'], ws['bg_h_lo']
        X = S[:, 256:]
        Xl = Sl[:, 256:] if Sl is not None else None
        Gt = G[:, 256:]
        Gtl = Gl[:, 256:] if Gl is not None else None
        _lib.call("gbsdf_bg_encode", R, NB, c_vp(center.data_ptr()), c_vp(ray_unit.data_ptr()),
                  c_vp(dists_bg.data_ptr()), c_vp(_p(pk['app_bg'])), c_vp(_p(app_idx)), self.app_dim,
                  c_vp(X.data_ptr()), c_vp(_p(Xl)), S.stride(0), BG_X_COLS, c_vp(Gt.data_ptr()), c_vp(_p(Gtl)),
                  G.stride(0), Kr0 - 256, stream)
        err = ws['err']
        w, b = pk['bw'], pk['bb']
        _dense(X, w[0], 256, BG_X_COLS, h[1], bias=b[0], epi=EPI_RELU, err=err, X_lo=Xl, out_lo=hl[1])
        _dense(h[1], w[1], 256, 256, h[2], bias=b[1], epi=EPI_RELU, err=err, X_lo=hl[1], out_lo=hl[2])
        _dense(h[2], w[2], 256, 256, h[3], bias=b[2], epi=EPI_RELU, err=err, X_lo=hl[2], out_lo=hl[3])
        _dense(h[3], w[3], 256, 256, S, bias=b[3], epi=EPI_RELU, err=err,             # h4 into S[:, :256]
               X_lo=hl[3], out_lo=Sl)
        _dense(S, w[4], 256, BG_S_COLS, h[5], bias=b[4], epi=EPI_RELU, err=err,       # skip: [h4 | input]
               X_lo=Sl, out_lo=hl[5])
        _dense(h[5], w[5], 256, 256, h[6], bias=b[5], epi=EPI_RELU, err=err, X_lo=hl[5], out_lo=hl[6])
        _dense(h[6], w[6], 256, 256, h[7], bias=b[6], epi=EPI_RELU, err=err, X_lo=hl[6], out_lo=hl[7])
        _dense(h[7], w[7], 256, 256, G, bias=b[7], epi=EPI_RELU, err=err,             # features into G[:, :256]
               X_lo=hl[7], out_lo=Gl)
        _lib.call("gbsdf_bg_density", Nb, c_vp(h[7].data_ptr()), c_vp(_p(hl[7])), h[7].stride(0), 256,
                  c_vp(pk['bw7d'].data_ptr()), c_vp(pk['bb7d'].data_ptr()), c_vp(ws['bg_sigma'].data_ptr()), stream)
        hr = ws['bg_hr']
        _dense(G, pk['bwr0'], Hbr, Kr0, hr, bias=pk['bbr0'], epi=EPI_RELU, err=err, X_lo=Gl)
        _lib.call("gbsdf_rgb_head_fwd", Nb, c_vp(hr.data_ptr()), hr.stride(0), Hbr, c_vp(pk['bwr1'].data_ptr()),
                  c_vp(pk['bbr1'].data_ptr()), c_vp(ws['bg_rgbs'].data_ptr()), stream)

    def _background_backward(self, R, app_idx, stream):
        """Gradients of the background NeRF from the render kernel's d colour and d density
        pre-activation (column 256 of the layer-7 gradient buffer); weight gradients
        dZ^T [X | 1] (loss-scaled, FP32)."""
        ws, pk = self.ws, self.pk
        dev = ws['bg_S'].device
        dev32 = dict(device=dev, dtype=torch.float32)
        Nb, Hbr, Kr0 = R * self.n_bg, self.Hbr, self.Kr0
        S, G, h, hr = ws['bg_S'], ws['bg_G'], ws['bg_h'], ws['bg_hr']
        dZ7, dz = ws['bg_dZ7'], ws['bg_dz']
        err = ws['err']
        g = {}
        ws['bg_d_bl'].zero_()
        g['r1'] = torch.zeros(3, Hbr, **dev32)
        dzr_lo, dZ7_lo, dz_lo = ws['bg_dz_r_lo'], ws['bg_dZ7_lo'], ws['bg_dz_lo']
        _lib.call("gbsdf_rgb_head_bwd", Nb, c_vp(hr.data_ptr()), hr.stride(0), Hbr, c_vp(pk['bwr1'].data_ptr()),
                  c_vp(ws['bg_rgbs'].data_ptr()), c_vp(ws['bg_d_rgbs'].data_ptr()), None,
                  c_vp(ws['bg_dz_r'].data_ptr()), c_vp(_p(dzr_lo)), c_vp(ws['bg_d_bl'].data_ptr()),
                  c_vp(g['r1'].data_ptr()), stream)
        g['r0'] = torch.empty(Hbr, Kr0, **dev32)
        _wgrad(ws['bg_dz_r'], G, Hbr, Kr0, g['r0'], err=err)                        # bias column 256 + 16 + app
        _dense(ws['bg_dz_r'], pk['bwr0T_feat'], 256, Hbr, dZ7, epi=EPI_DRELU, G=G, err=err,   # d feature pre-act
               X_lo=dzr_lo, out_lo=dZ7_lo)
        if self.app_dim:
            _dense(ws['bg_dz_r'], pk['bwr0T_tail'], 64, Hbr, ws['bg_d_tail'], epi=EPI_IDENTITY, err=err,
                   X_lo=dzr_lo)
            g['app'] = torch.zeros_like(pk['app_bg'])
            _lib.call("gbsdf_app_grad", R, self.n_bg, None, c_vp(app_idx.data_ptr()),
                      c_vp(ws['bg_d_tail'].data_ptr()), 64, 16, self.app_dim, c_vp(g['app'].data_ptr()), stream)
        g[7] = torch.empty(272, 264, **dev32)
        _wgrad(dZ7, h[7], 272, 264, g[7], err=err)
        _dense(dZ7, pk['bw7extT'], 256, 272, dz[0], epi=EPI_DRELU, G=h[7], err=err,       # dZ6
               X_lo=dZ7_lo, out_lo=dz_lo[0])
        cur = 0
        for i, gate in ((6, h[6]), (5, h[5]), (4, S), (3, h[3]), (2, h[2]), (1, h[1])):
            X = S if i == 4 else h[i]
            g[i] = torch.empty(256, X.shape[1], **dev32)
            _wgrad(dz[cur], X, 256, X.shape[1], g[i], err=err)
            _dense(dz[cur], pk['bwT'][i], 256, 256, dz[1 - cur], epi=EPI_DRELU, G=gate, err=err,
                   X_lo=dz_lo[cur], out_lo=dz_lo[1 - cur] if i > 1 else None)
            cur = 1 - cur
        g[0] = torch.empty(256, BG_X_COLS, **dev32)
        _wgrad(dz[cur], S[:, 256:], 256, BG_X_COLS, g[0], err=err)
        return g

    def losses(self):
        """Loss terms of the last step (reads the FP64 device sums: synchronises)."""
        R, n_mean, w_r, w_e = self._loss_norm
        w_c = float(self.model.w_curv or 0.0)
        sums = self.ws['loss_sums'].tolist()
        l_render = 3.0 * sums[0] / (3.0 * R)
        l_eik = sums[1] / n_mean
        l_curv = sums[2] / n_mean
        loss = w_r * l_render + w_e * l_eik + w_c * l_curv
        return dict(loss=loss, l_render=l_render, l_eik=l_eik, l_curv=l_curv)

    def release(self):
        """Drop the workspace (its memory returns to torch's caching allocator)."""
        self.ws = None
        self.pk = None

    def check_device_errors(self):
        """Non-zero when a bounded device wait timed out or a ray was too long."""
        return int(self.ws['err'].item()) if self.ws is not None else 0

    # ------------------------------------------------------------------ gradients -> masters
    def _scatter_grads(self, g):
        """Map the effective-weight gradients onto the weight-norm parameters (W = g v / ||v||),
        take the loss scale off and accumulate into the masters' .grad: gbsdf_weightnorm_bwd,
        one launch for every layer and plain parameter of the field and the colour MLP."""
        m = self.model
        inv = self._scal[3:4] if self.dynamic else 1.0 / self.loss_scale
        sdf = m.neural_sdf
        A, F = self.A, self.F
        K0 = self.K0
        l0, l1 = sdf.mlp.linears[0], sdf.mlp.linears[1]
        lins = m.neural_rgb.mlp.linears
        dW0 = torch.zeros_like(l0.weight_v)
        gx = g['w0ext']      # columns: features hi | x,y,z hi, 1, x,y,z lo, 0 [| features lo]
        dW0[:, 3:3 + A * F] = gx[:, :A * F]
        if gx.shape[1] > K0 + 16:                      # the k_wgrad path keeps the lo columns apart
            dW0[:, 3:3 + A * F] += gx[:, K0 + 16:K0 + 16 + A * F]
        dW0[:, :3] = gx[:, K0:K0 + 3] + gx[:, K0 + 4:K0 + 7]
        db0 = gx[:, K0 + 3]
        # colour layer 0: undo the column reordering
        sh = 16
        Wc0_grad = torch.zeros(lins[0].weight_v.shape, device=dW0.device, dtype=torch.float32)
        gc0 = g['wc0']
        Wc0_grad[:, 6 + sh:6 + sh + 256] = gc0[:, :256]
        Wc0_grad[:, 0:3] = gc0[:, 256:259]
        Wc0_grad[:, 3:3 + sh] = gc0[:, 259:259 + sh]
        Wc0_grad[:, 3 + sh:6 + sh] = gc0[:, 259 + sh:262 + sh]
        if self.app_dim:
            Wc0_grad[:, 6 + sh + 256:] = gc0[:, 262 + sh:262 + sh + self.app_dim]
        eff = [(l0, dW0, db0), (l1, g['w1'], g['b1']), (lins[0], Wc0_grad, g['bc0'])]
        for i in range(1, self.n_rgb_hidden):
            eff.append((lins[i], g[f'wc{i}'], g[f'bc{i}']))
        eff.append((lins[-1], g['wl'], g['bl']))
        names = ['sdf.l0', 'sdf.l1'] + [f'rgb.l{i}' for i in range(len(eff) - 2)]
        self._eff = (names, [(dW, db) for _, dW, db in eff], inv)
        sink = _GradSink()
        ents = [_wn_entry(sink, dW, db, bias=lin.bias, v=lin.weight_v, g=lin.weight_g) for lin, dW, db in eff]
        head = sdf.mlp.linear_sdf
        ents.append(_wn_entry(sink, self.ws['d_whead'], self.ws['d_bhead'], weight=head.weight, bias=head.bias))
        ents.append(_wn_entry(sink, self.ws['d_s_var'].reshape(1, 1), weight=m.s_var))
        if self.app_dim:
            ents.append(_wn_entry(sink, g['app'], weight=m.appear_embed.weight))
        if self.bg:
            ents += self._scatter_background(g['bg'], inv, sink)
        _weightnorm_bwd(ents, inv, dW0.device)
        if not self._table_in_place:
            _acc(sdf.tcnn_encoding.params, g['table'].to(sdf.tcnn_encoding.params.dtype))

    @property
    def eff_grads(self):
        """Unscaled gradients of the effective weights and biases of the last step, per layer."""
        names, eff, inv = self._eff
        return {n: (dW * inv, db * inv) for n, (dW, db) in zip(names, eff)}

    def _scatter_background(self, g, inv, sink):
        """Background NeRF gradients (plain linears) from the packed layouts: entries of the
        gradient launch."""
        bgm = self.model.background_nerf
        L, Lr = bgm.mlp_feat.linears, bgm.mlp_rgb.linears
        eff = {}
        eff['bg.l0'] = (g[0][:, :84], g[0][:, 84])
        for i in (1, 2, 3, 5, 6):
            eff[f'bg.l{i}'] = (g[i][:, :256], g[i][:, 256])
        eff['bg.l4'] = (g[4][:, :340], g[4][:, 340])
        nin = 256 + 16 + self.app_dim
        eff['bg.rgb.l0'] = (g['r0'][:, :nin], g['r0'][:, nin])
        eff['bg.rgb.l1'] = (g['r1'], self.ws['bg_d_bl'])
        lins = {f'bg.l{i}': L[i] for i in range(8)}
        lins.update({'bg.rgb.l0': Lr[0], 'bg.rgb.l1': Lr[1]})
        # layer 7's rows come packed as [256 feature rows | density row]; the layer's order is
        # [density | features]
        g7 = g[7]
        self._bg_eff = (eff, g7, inv)
        ents = [_wn_entry(sink, dW, db, weight=lins[k].weight, bias=lins[k].bias) for k, (dW, db) in eff.items()]
        ents.append(_wn_entry(sink, g7[256:257, :256], g7[256:257, 256], weight=L[7].weight, bias=L[7].bias,
                              rows=slice(0, 1)))
        ents.append(_wn_entry(sink, g7[:256, :256], g7[:256, 256], weight=L[7].weight, bias=L[7].bias,
                              rows=slice(1, 257)))
        if self.app_dim:
            ents.append(_wn_entry(sink, g['app'], weight=self.model.appear_embed_outside.weight))
        return ents

    @property
    def bg_grads(self):
        """Unscaled gradients of the background NeRF's weights and biases of the last step."""
        eff, g7, inv = self._bg_eff
        out = {k: (dW * inv, db * inv) for k, (dW, db) in eff.items()}
        out['bg.l7'] = (torch.cat([g7[256:257, :256], g7[:256, :256]], dim=0) * inv,
                        torch.cat([g7[256:257, 256], g7[:256, 256]], dim=0) * inv)
        return out

    # ------------------------------------------------------------------ dynamic loss scaling
    def _scalars(self, device):
        if self._scal is None or self._scal.device != torch.device(device):
            self._scal = torch.zeros(8, device=device, dtype=torch.float32)
            self._scal[0] = self.loss_scale
            self._growth = torch.zeros(1, device=device, dtype=torch.int32)
            self._one = torch.ones(1, device=device, dtype=torch.float32)
            self.refresh_scalars()
        return self._scal

    def refresh_scalars(self):
        """Copy the schedule's per-iteration scalars (the anneal ratio of iter_cos and the
        curvature weight) into the device buffer the render kernel reads.  Eager steps do this
        themselves; CapturedStep.replay calls it before every replay."""
        if self._scal is None:
            return
        m = self.model
        self._scal[1].fill_(min(m.progress / m.anneal_end, 1.0))
        self._scal[2].fill_(float(m.w_curv or 0.0))

    def _check_and_update_scale(self, scal):
        """found_inf |= any non-finite master gradient (the scatter already flagged the table's);
        then the scale update of GradScaler.update: x 0.5 on overflow, x 2 after growth_interval
        clean steps in a row.  Device work only, no host synchronisation."""
        table = self.model.neural_sdf.tcnn_encoding.params
        small = [p.grad for p in self.model.parameters()
                 if p.grad is not None and p is not table and p.grad.dtype == torch.float32]
        if small:
            torch._amp_foreach_non_finite_check_and_unscale_(small, scal[4:5], self._one)
        torch._amp_update_scale_(scal[0:1], self._growth, scal[4:5], 2.0, 0.5, self.growth_interval)

    def found_inf(self):
        """True when the last step's gradients were not finite (skip that optimizer step; the
        scale has already been halved).  One device read."""
        if self.dynamic:
            return bool(self._scal[4].item() > 0) if self._scal is not None else False
        for prm in self.model.parameters():
            if prm.grad is not None and not torch.isfinite(prm.grad).all():
                return True
        return False

    def current_loss_scale(self):
        return float(self._scal[0].item()) if (self.dynamic and self._scal is not None) else self.loss_scale

    def schedule_key(self):
        """The schedule values baked into a step's launches (normal epsilon, active levels):
        a captured graph is valid while these are unchanged."""
        sdfm = self.model.neural_sdf
        return (float(sdfm.normal_eps), int(sdfm.active_levels))


def _acc(param, grad):
    grad = grad.to(param.dtype).reshape(param.shape)
    if param.grad is None:
        param.grad = grad
    else:
        param.grad.add_(grad)


class CapturedStep:
    """One training step of a FusedField -- zero the master gradients, forward,
    backward (and, with dynamic loss scaling, the overflow check and the scale update) --
    captured in a CUDA graph and replayed.  A replay clears the hash table's gradient over the
    active levels only; the inactive levels stay as the capture left them (zero), so code that
    writes into that gradient between replays must keep them zero.

    The batch is copied into static device buffers at capture time; ``replay(batch)``
    copies a new batch of the same shapes into them (host tensors are copied from
    pinned memory asynchronously) and launches the whole step as one graph.  The
    gradients land in the masters' ``.grad`` tensors, which must not be replaced
    (zero_grad(set_to_none=True) between replays would detach them from the graph).

    Schedule: the per-iteration scalars (iter_cos anneal ratio, curvature weight) are read
    from a device buffer that every replay refreshes from the model, and the loss scale is a
    device scalar; the normal epsilon and the active levels are baked into the launches, so
    replay() captures the step again when model.schedule() has changed them (every few
    thousand iterations of the coarse-to-fine schedule).
    """

    def __init__(self, fused, batch, warmup=2):
        self.fused = fused
        self.static = {k: v.clone() for k, v in batch.items() if torch.is_tensor(v)}
        self.static.update({k: v for k, v in batch.items() if not torch.is_tensor(v)})
        self.graph = None
        self.recaptures = 0
        self._capture(warmup)

    def _capture(self, warmup):
        fused, model = self.fused, self.fused.model
        dev = self.static['center'].device
        self.graph = None
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            for _ in range(warmup):
                model.zero_grad(set_to_none=False)
                fused.step(self.static, compute_loss=False)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        self.params = [p for p in model.parameters() if p.requires_grad]
        for p in self.params:
            if p.grad is None:
                p.grad = torch.zeros_like(p)
        if fused.dynamic:
            fused._scalars(dev)           # created eagerly: a scale set inside the capture would reset at replays
        fused.refresh_scalars()
        self.key = fused.schedule_key()
        self.graph = torch.cuda.CUDAGraph()
        # the table gradient is cleared over the active levels only: the warm-up above zeroed
        # all of it, the step writes nothing past the active prefix, and a change of the active
        # levels captures the step again
        table = model.neural_sdf.tcnn_encoding.params
        n_act = active_table_params(model.neural_sdf)
        with torch.cuda.graph(self.graph):
            for p in self.params:
                if p is table:
                    p.grad[:n_act].zero_()
                else:
                    p.grad.zero_()
            self.out = fused.step(self.static, compute_loss=False, _refresh=False)

    def replay(self, batch=None):
        if self.fused.schedule_key() != self.key:
            self.recaptures += 1
            self._capture(warmup=1)
        if batch is not None:
            for k, v in batch.items():
                if torch.is_tensor(v):
                    self.static[k].copy_(v, non_blocking=True)
        self.fused.refresh_scalars()
        self.graph.replay()
        return self.out

    def losses(self):
        return self.fused.losses()
