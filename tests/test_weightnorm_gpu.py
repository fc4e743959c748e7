"""Weight-norm backward kernel (gbsdf_weightnorm_bwd) against torch autograd through
torch.nn.utils.weight_norm (dim 0), the parametrisation of the reference's MLP linears
(projects/neuralangelo/utils/mlp.py:42-43): the gradients of v, g and the bias from the
effective-weight gradient, with the loss scale taken off, written or accumulated."""
import pytest
import torch

from neuralangelo_gb300 import fused

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def rel(a, b):
    return float((a.double() - b.double()).norm() / b.double().norm().clamp_min(1e-300))


def weight_norm_linear(rows, cols, seed):
    torch.manual_seed(seed)
    lin = torch.nn.utils.weight_norm(torch.nn.Linear(cols, rows), dim=0).to(DEV)
    with torch.no_grad():
        lin.weight_g.mul_(torch.rand_like(lin.weight_g) + 0.5)
    return lin


def autograd_ref(lin, dW, db, s):
    """Gradients of (v, g, b) when the effective weight W = g v / ||v|| receives s dW."""
    v = lin.weight_v.detach().double().requires_grad_(True)
    g = lin.weight_g.detach().double().requires_grad_(True)
    W = v * (g / v.norm(dim=1, keepdim=True))
    dv, dg = torch.autograd.grad(W, (v, g), grad_outputs=dW.double() * s)
    return dv, dg, db.double() * s


@pytest.mark.parametrize("dynamic", [False, True])
def test_weight_norm_layers_write_then_accumulate(dynamic):
    shapes = [(256, 131), (256, 256), (256, 280), (3, 256), (272, 340)]
    lins = [weight_norm_linear(r, c, i) for i, (r, c) in enumerate(shapes)]
    torch.manual_seed(7)
    s = 1.0 / 32768.0
    scale = torch.tensor([s], device=DEV) if dynamic else s
    # dW as a column slice of a wider buffer (row stride > cols), the bias as a strided column
    bufs = [torch.randn(r, c + 9, device=DEV) * 1e3 for r, c in shapes]
    dWs = [b[:, :c] for b, (r, c) in zip(bufs, shapes)]
    dbs = [b[:, c + 3] for b, (r, c) in zip(bufs, shapes)]
    for lin in lins:
        lin.zero_grad(set_to_none=True)
    for rep in range(2):                        # first call writes fresh .grad, second adds
        sink = fused._GradSink()
        ents = [fused._wn_entry(sink, dW, db, bias=lin.bias, v=lin.weight_v, g=lin.weight_g)
                for lin, dW, db in zip(lins, dWs, dbs)]
        fused._weightnorm_bwd(ents, scale, DEV)
    torch.cuda.synchronize()
    for lin, dW, db in zip(lins, dWs, dbs):
        dv, dg, dbias = autograd_ref(lin, dW, db, s)
        assert rel(lin.weight_v.grad, 2 * dv) < 1e-5
        assert rel(lin.weight_g.grad, 2 * dg) < 1e-5
        assert rel(lin.bias.grad, 2 * dbias) < 1e-6


def test_plain_entries_and_row_blocks():
    """Plain entries (no weight norm): the head weight from a flat vector, a scalar, and one
    weight assembled from two row blocks of a packed gradient (the background's layer 7)."""
    torch.manual_seed(3)
    head = torch.nn.Linear(256, 1).to(DEV)
    s_var = torch.nn.Parameter(torch.tensor(0.3, device=DEV))
    l7 = torch.nn.Linear(256, 257).to(DEV)
    d_head, d_hb = torch.randn(256, device=DEV), torch.randn(1, device=DEV)
    d_s = torch.randn(1, 1, device=DEV)
    g7 = torch.randn(257, 257, device=DEV)       # rows: 256 features, then the density row
    s = 0.25
    sink = fused._GradSink()
    ents = [fused._wn_entry(sink, d_head, d_hb, weight=head.weight, bias=head.bias),
            fused._wn_entry(sink, d_s, weight=s_var),
            fused._wn_entry(sink, g7[256:257, :256], g7[256:257, 256], weight=l7.weight, bias=l7.bias,
                            rows=slice(0, 1)),
            fused._wn_entry(sink, g7[:256, :256], g7[:256, 256], weight=l7.weight, bias=l7.bias,
                            rows=slice(1, 257))]
    fused._weightnorm_bwd(ents, s, DEV)
    torch.cuda.synchronize()
    assert torch.equal(head.weight.grad, (d_head * s).reshape(1, -1))
    assert torch.equal(head.bias.grad, d_hb * s)
    assert torch.equal(s_var.grad.reshape(1, 1), d_s * s)
    w7 = torch.cat([g7[256:257, :256], g7[:256, :256]], dim=0) * s
    b7 = torch.cat([g7[256:257, 256], g7[:256, 256]], dim=0) * s
    assert torch.equal(l7.weight.grad, w7)
    assert torch.equal(l7.bias.grad, b7)


def test_more_entries_than_one_launch():
    """More entries than GBSDF_WN_MAX_LAYERS: the launcher splits them over several launches."""
    lins = [weight_norm_linear(64, 48, 100 + i) for i in range(fused.WN_MAX_LAYERS + 3)]
    torch.manual_seed(11)
    dWs = [torch.randn(64, 48, device=DEV) for _ in lins]
    dbs = [torch.randn(64, device=DEV) for _ in lins]
    sink = fused._GradSink()
    fused._weightnorm_bwd([fused._wn_entry(sink, dW, db, bias=lin.bias, v=lin.weight_v, g=lin.weight_g)
                           for lin, dW, db in zip(lins, dWs, dbs)], 1.0, DEV)
    torch.cuda.synchronize()
    for lin, dW, db in zip(lins, dWs, dbs):
        dv, dg, dbias = autograd_ref(lin, dW, db, 1.0)
        assert rel(lin.weight_v.grad, dv) < 1e-5
        assert rel(lin.weight_g.grad, dg) < 1e-5


def torch_pack(ff):
    """The fused step's weight copies formed with torch ops (weight norm as the module's weight
    property, casts, transposes and column reorders): what gbsdf_weightnorm_fwd must produce."""
    m = ff.model
    sdf = m.neural_sdf
    A, F, K0 = sdf.active_levels, sdf.tcnn_encoding.layout.n_features, ff.K0
    f16 = torch.float16
    with torch.no_grad():
        W0 = sdf.mlp.linears[0].weight
        H = W0.shape[0]
        w0e = torch.zeros(H, K0, device=DEV, dtype=f16)
        w0e[:, :A * F] = W0[:, 3:3 + A * F]
        w0x, b0 = W0[:, :3].contiguous(), sdf.mlp.linears[0].bias
        hi, lo = w0x.half(), (w0x - w0x.half().float()).half()
        bh, bl = b0.half(), (b0 - b0.half().float()).half()
        w0b = torch.zeros(H, K0 + 16, device=DEV, dtype=f16)
        w0b[:, :K0] = w0e
        w0b[:, K0:K0 + 3], w0b[:, K0 + 3], w0b[:, K0 + 4:K0 + 7] = hi, bh, hi
        w0b[:, K0 + 7], w0b[:, K0 + 8:K0 + 11] = bl, lo
        out = dict(w0e=w0e, w0b=w0b, w0x=w0x)
        W1 = sdf.mlp.linears[1].weight
        out['w1'], out['w1T'] = W1.half(), W1.t().half()
        lins = m.neural_rgb.mlp.linears
        Wc0, sh = lins[0].weight, 16
        tail = torch.cat([Wc0[:, 0:6 + sh], Wc0[:, 6 + sh + 256:6 + sh + 256 + ff.app_dim]], dim=1)
        wc0 = torch.zeros(ff.Hc, ff.Kc0, device=DEV, dtype=f16)
        wc0[:, :256] = Wc0[:, 6 + sh:6 + sh + 256]
        wc0[:, 256:256 + tail.shape[1]] = tail
        out['wc'] = [wc0] + [lins[i].weight.half() for i in range(1, ff.n_rgb_hidden)]
        out['wcT'] = [None] + [w.t() for w in out['wc'][1:]]
        out['wc0T_feat'] = wc0[:, :256].t()
        t = torch.zeros(64, ff.Hc, device=DEV, dtype=f16)
        t[:ff.Kc0 - 256] = wc0[:, 256:].t()
        out['wc0T_tail'] = t
        out['wl'] = lins[-1].weight
        if ff.bg:
            L = m.background_nerf.mlp_feat.linears
            Lr = m.background_nerf.mlp_rgb.linears
            w = [torch.zeros(256, fused.BG_X_COLS, device=DEV, dtype=f16)] + [None] * 7
            w[0][:, :84] = L[0].weight
            for i in (1, 2, 3, 5, 6, 7):
                w[i] = L[i].weight.half() if i != 7 else L[7].weight[1:].half()
            w[4] = torch.zeros(256, fused.BG_S_COLS, device=DEV, dtype=f16)
            w[4][:, :340] = L[4].weight
            out['bw'] = w
            out['bwT'] = [None] + [w[i].t() if i != 4 else w[4][:, :256].t() for i in range(1, 7)]
            w7 = torch.zeros(272, 256, device=DEV, dtype=f16)
            w7[:256], w7[256] = L[7].weight[1:], L[7].weight[0]
            out['bw7extT'] = w7.t()
            nin = 256 + 16 + ff.app_dim
            wr0 = torch.zeros(ff.Hbr, ff.Kr0, device=DEV, dtype=f16)
            wr0[:, :nin] = Lr[0].weight
            out['bwr0'], out['bwr0T_feat'] = wr0, wr0[:, :256].t()
            t = torch.zeros(64, ff.Hbr, device=DEV, dtype=f16)
            t[:ff.Kr0 - 256] = wr0[:, 256:].t()
            out['bwr0T_tail'] = t
    return out


def close(a, b):
    """fp16 copies agree to one fp16 rounding of W (the native norm may differ from torch's in the
    last FP32 bit); FP32 copies to FP32 rounding."""
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    rtol = 2e-3 if a.dtype == torch.float16 else 2e-6
    return torch.allclose(a.float(), b.float(), rtol=rtol, atol=1e-7)


@pytest.mark.parametrize("background", [False, True])
def test_step_pack_matches_torch(background):
    from neuralangelo_gb300.config import field_config
    from neuralangelo_gb300.model import FieldModel
    from neuralangelo_gb300.workloads import full_field_iteration, init_field_params
    cfg = field_config("full", background=background)
    cfg.sdf.encoding.hashgrid.dict_size = 14
    cfg.appear_embed.num_images = 10
    torch.manual_seed(0)
    model = FieldModel(cfg).to(DEV)
    init_field_params(model, 0)
    model.schedule(full_field_iteration(7))
    with torch.no_grad():                       # weight_g away from ||v||, so the norm matters
        for mod in model.modules():
            if hasattr(mod, 'weight_g'):
                mod.weight_g.mul_(torch.rand_like(mod.weight_g) + 0.5)
    ff = fused.FusedField(model)
    for rep in range(2):                        # the second pack reuses the buffers
        ff._pack()
        torch.cuda.synchronize()
        ref = torch_pack(ff)
        pk = ff.pk
        for k, v in ref.items():
            if isinstance(v, list):
                for i, (a, b) in enumerate(zip(pk[k], v)):
                    assert (a is None) == (b is None), (k, i)
                    assert a is None or close(a, b), (k, i)
            else:
                assert close(pk[k], v), k
        n = fused.active_table_params(model.neural_sdf)
        params = model.neural_sdf.tcnn_encoding.params
        assert torch.equal(pk['table'][:n], params[:n].detach().half())
        with torch.no_grad():                   # the next pack must see updated masters
            for prm in model.parameters():
                prm.add_(0.01 * torch.randn_like(prm))
