"""Host side of the weight-norm entry points (no GPU): the ctypes entries the fused step builds for
gbsdf_weightnorm_bwd / gbsdf_weightnorm_fwd carry the right shapes, strides, row offsets and
write-or-add flags, and `.grad` tensors are created once per parameter."""
import torch

from neuralangelo_gb300 import fused


def test_gradient_entries_write_fresh_grads_and_add_into_existing_ones():
    torch.manual_seed(0)
    lin = torch.nn.utils.weight_norm(torch.nn.Linear(16, 8), dim=0)
    buf = torch.zeros(8, 20)
    dW, db = buf[:, :16], buf[:, 17]               # a column slice and a strided column
    sink = fused._GradSink()
    e = fused._wn_entry(sink, dW, db, bias=lin.bias, v=lin.weight_v, g=lin.weight_g)
    assert (e.rows, e.cols, e.ld_dw, e.ld_db) == (8, 16, 20, 20)
    assert e.dW == dW.data_ptr() and e.db == db.data_ptr()
    assert (e.acc_v, e.acc_g, e.acc_b) == (0, 0, 0)          # fresh .grad tensors are written
    assert e.dv == lin.weight_v.grad.data_ptr() and e.dg == lin.weight_g.grad.data_ptr()
    assert e.dbias == lin.bias.grad.data_ptr()
    assert e.v == lin.weight_v.data_ptr() and e.g == lin.weight_g.data_ptr()
    e2 = fused._wn_entry(fused._GradSink(), dW, db, bias=lin.bias, v=lin.weight_v, g=lin.weight_g)
    assert (e2.acc_v, e2.acc_g, e2.acc_b) == (1, 1, 1)       # present ones are added into


def test_gradient_entries_from_row_blocks_share_one_grad():
    """The background's layer 7 arrives as [features | density] rows and goes back as [density |
    features]: two plain entries into one gradient tensor, created once."""
    l7 = torch.nn.Linear(4, 5)
    g7 = torch.zeros(5, 5)
    sink = fused._GradSink()
    a = fused._wn_entry(sink, g7[4:5, :4], g7[4:5, 4], weight=l7.weight, bias=l7.bias, rows=slice(0, 1))
    b = fused._wn_entry(sink, g7[:4, :4], g7[:4, 4], weight=l7.weight, bias=l7.bias, rows=slice(1, 5))
    assert a.v is None and b.v is None                        # plain entries
    assert a.acc_v == b.acc_v == 0 and a.acc_b == b.acc_b == 0
    assert a.dv == l7.weight.grad.data_ptr()
    assert b.dv == l7.weight.grad.data_ptr() + 4 * 4          # row 1 of a [5, 4] FP32 gradient
    assert b.dbias == l7.bias.grad.data_ptr() + 4
    assert (b.rows, b.cols, b.ld_dw) == (4, 4, 5)


def test_pack_entries_describe_segments_and_destinations():
    torch.manual_seed(1)
    v = torch.randn(8, 30)
    g = torch.rand(8)
    wc0 = torch.zeros(8, 48, dtype=torch.float16)
    tail_t = torch.zeros(64, 8, dtype=torch.float16)
    e = fused._pk_entry(v, g, col0=0, ncols=22, dst16=wc0[:, 16:38], dst16T=tail_t[:22])
    assert (e.rows, e.cols, e.col0, e.ncols, e.ld_src) == (8, 30, 0, 22, 30)
    assert e.g == g.data_ptr()
    assert e.dst16 == wc0.data_ptr() + 16 * 2 and e.ld16 == 48
    assert e.dst16T == tail_t.data_ptr() and e.ldT == 8
    assert e.dst16_lo is None and e.dst32 is None
    # a bias as one column with its fp16 residual two columns on, and rows from an offset
    b = torch.randn(8)
    w0b = torch.zeros(8, 80, dtype=torch.float16)
    eb = fused._pk_entry(b, None, dst16=w0b[:, 67], dst16_lo=w0b[:, 71])
    assert (eb.rows, eb.cols, eb.ncols, eb.ld_src, eb.ld16) == (8, 1, 1, 1, 80)
    assert eb.g is None and eb.dst16_lo == w0b.data_ptr() + 71 * 2
    w7 = torch.randn(5, 6)
    t7 = torch.zeros(6, 9, dtype=torch.float16)
    er = fused._pk_entry(w7, rows=slice(1, 5), dst16T=t7[:, :4])
    assert er.rows == 4 and er.v == w7.data_ptr() + 6 * 4 and er.ldT == 9


def test_active_table_prefix_follows_the_level_layout():
    """The fp16 working copy and the captured step's gradient clearing cover the active levels
    only: a level-major prefix of offset[active] entries x F features, growing with the schedule."""
    from neuralangelo_gb300.config import field_config
    from neuralangelo_gb300.model import FieldModel
    from neuralangelo_gb300.workloads import full_field_iteration
    cfg = field_config("full")
    cfg.sdf.encoding.hashgrid.dict_size = 14
    model = FieldModel(cfg)
    sdf = model.neural_sdf
    layout = sdf.tcnn_encoding.layout
    F = layout.n_features
    seen = []
    for active in (4, 8, 12, layout.n_levels):
        model.schedule(full_field_iteration(active))
        assert sdf.active_levels == active
        n = fused.active_table_params(sdf)
        assert n == int(layout.offset[active]) * F
        seen.append(n)
    assert seen == sorted(seen) and seen[-1] == sdf.tcnn_encoding.params.numel()
