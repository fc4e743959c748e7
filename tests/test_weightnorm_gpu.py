"""Weight-norm backward kernel (gbsdf_weightnorm_bwd) against torch autograd through
torch.nn.utils.weight_norm (dim 0), the parametrisation of the reference's MLP linears
(projects/neuralangelo/utils/mlp.py:55-69): the gradients of v, g and the bias from the
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
