"""GPU parity of the plain FP32 drop-in path (hash grid, NeuS alpha, compositing,
full training forward+backward) against the oracle, through the C ABI."""
import numpy as np
import pytest
import torch

from oracle import field as of
from oracle import hashgrid as hg
from tests import golden_io, params_io

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


FULL = (16, 8, 22, 32, float(np.exp((np.log(2048) - np.log(32)) / 15)))
SMALL = (8, 4, 16, 16, 1.5)


def points(M, seed, lo=0.2, hi=0.8):
    rng = np.random.default_rng(seed)
    x = rng.uniform(lo, hi, size=(M, 3)).astype(np.float32)
    # points exactly on level-0 cell faces and taps straddling them
    k = min(64, M)
    x[:k, 0] = (np.arange(k) + 0.5) / 31.0
    return x


@pytest.mark.parametrize("cfg", [FULL, SMALL])
def test_hashgrid_indices_bit_exact(cfg):
    from neuralangelo_gb300.encoding import HashGridEncoding
    L, F, log2T, base, pls = cfg
    enc = HashGridEncoding(3, dict(n_levels=L, n_features_per_level=F, log2_hashmap_size=log2T,
                                   base_resolution=base, per_level_scale=pls)).to(DEV)
    x = points(20000, 0, -0.05, 1.05)
    got = enc.indices(torch.from_numpy(x).to(DEV)).cpu().numpy()
    want = hg.all_indices(x, hg.level_layout(*cfg))
    assert np.array_equal(got, want)


@pytest.mark.parametrize("cfg", [FULL, SMALL])
@pytest.mark.parametrize("table_dtype", [torch.float32, torch.float16])
def test_hashgrid_forward_backward(cfg, table_dtype):
    from neuralangelo_gb300.encoding import HashGridEncoding
    L, F, log2T, base, pls = cfg
    enc = HashGridEncoding(3, dict(n_levels=L, n_features_per_level=F, log2_hashmap_size=log2T,
                                   base_resolution=base, per_level_scale=pls), dtype=table_dtype).to(DEV)
    active = L // 2 + 1
    enc.active_levels = active
    with torch.no_grad():
        enc.params.uniform_(-0.1, 0.1)
    x = points(4000, 1)
    xt = torch.from_numpy(x).to(DEV)
    out = enc(xt)
    lay = hg.level_layout(*cfg)
    table = enc.params.detach().double().cpu().numpy()
    want = hg.encode(x, table, lay, active)
    assert rel(out.detach().cpu(), want) < 2e-6
    assert torch.all(out[:, active * F:] == 0)
    d = torch.randn(out.shape, device=DEV, generator=torch.Generator(DEV).manual_seed(3))
    (out * d).sum().backward()
    want_g = hg.encode_backward(x, d.double().cpu().numpy(), lay, active).reshape(-1)
    # autograd hands back the gradient in the parameter dtype: fp16 rounding for fp16 tables
    tol = 1e-5 if table_dtype == torch.float32 else 1e-3
    assert rel(enc.params.grad.double().cpu(), want_g) < tol


def test_hashgrid_empty_and_ragged():
    from neuralangelo_gb300.encoding import HashGridEncoding
    enc = HashGridEncoding(3, dict(n_levels=4, n_features_per_level=2, log2_hashmap_size=8,
                                   base_resolution=8, per_level_scale=2.0)).to(DEV)
    assert enc(torch.zeros(0, 3, device=DEV)).shape == (0, 8)
    x = points(37, 5)    # not a multiple of the block size; T=2^8 forces collisions
    out = enc(torch.from_numpy(x).to(DEV))
    want = hg.encode(x, enc.params.detach().double().cpu().numpy(), hg.level_layout(4, 2, 8, 8, 2.0))
    assert rel(out.detach().cpu(), want) < 2e-6


def test_alpha_and_weights_against_oracle():
    from neuralangelo_gb300 import render
    g = torch.Generator().manual_seed(0)
    R, N = 257, 70
    ray = torch.nn.functional.normalize(torch.randn(R, 3, generator=g, dtype=torch.float64), dim=-1)
    sdf = 0.3 * torch.randn(R, N, generator=g, dtype=torch.float64)
    grad = torch.randn(R, N, 3, generator=g, dtype=torch.float64)
    dists = torch.sort(torch.rand(R, N, generator=g, dtype=torch.float64) * 2 + 1, dim=1).values
    far = dists[:, -1:] + 0.1
    s_var = torch.tensor(3.0, dtype=torch.float64)
    ts = [t.clone().requires_grad_(True) for t in (sdf, grad, s_var)]
    a_ref = of.neus_alphas(ray, ts[0], ts[1], dists, far, ts[2], 0.05, 0.1)
    w_ref = of.compositing_weights(a_ref)
    gw = torch.randn(R, N, generator=g, dtype=torch.float64)
    (w_ref * gw).sum().backward()
    tc = [t.float().to(DEV).requires_grad_(True) for t in (sdf, grad, s_var)]
    a = render.compute_neus_alphas(ray.float().to(DEV), tc[0], tc[1], dists.float().to(DEV), tc[2],
                                   dist_far=far.float().to(DEV), progress=0.05, anneal_end=0.1)
    w = render.alpha_compositing_weights(a)[..., 0]
    (w * gw.float().to(DEV)).sum().backward()
    assert rel(a.detach().cpu(), a_ref.detach()) < 1e-5
    assert rel(w.detach().cpu(), w_ref.detach()) < 1e-5
    for t, r in zip(tc, ts):
        assert rel(t.grad.cpu(), r.grad) < 1e-4


def test_weights_saturated_alpha():
    from neuralangelo_gb300 import render
    a = torch.tensor([[0.2, 1.0, 0.5, 0.3], [0.0, 0.0, 0.0, 0.0]], dtype=torch.float64, requires_grad=True)
    w_ref = of.compositing_weights(a)
    gw = torch.tensor([[1.0, -2.0, 3.0, 0.5], [1.0, 1.0, 1.0, 1.0]], dtype=torch.float64)
    (w_ref * gw).sum().backward()
    ac = a.detach().float().to(DEV).requires_grad_(True)
    w = render.alpha_compositing_weights(ac)[..., 0]
    (w * gw.float().to(DEV)).sum().backward()
    np.testing.assert_allclose(w.detach().cpu(), w_ref.detach(), atol=1e-7)
    np.testing.assert_allclose(ac.grad.cpu(), a.grad, atol=1e-6)


@pytest.mark.parametrize("name", golden_io.CASES)
def test_plain_model_matches_golden(name):
    g = golden_io.load(name)
    model = params_io.model_from_golden(g, DEV)
    out = model.render_step(params_io.batch_to(g['batch'], DEV))
    out['loss'].backward()
    z = g['z']
    for key, tol in (('sdf', 1e-5), ('grads', 1e-4), ('rgbs', 1e-5), ('alphas', 1e-4), ('weights', 1e-4),
                     ('rgb', 1e-5)):
        assert rel(out[key].detach().cpu(), z[key]) < tol, key
    inside = ~z['outside'][:, 0]
    assert rel(out['hess'].detach().cpu()[inside], z['hess'][inside]) < 1e-3
    assert abs(float(out['loss']) - float(z['losses'][0])) < 1e-5 * abs(float(z['losses'][0]))
    grads = params_io.model_grads(model)
    assert rel(grads['table'], z['g_table']) < 1e-3
    assert rel(grads['s_var'], z['g_s_var']) < 1e-3
    for k in z:
        if k.startswith('g_sdf.') or k.startswith('g_rgb.'):
            assert rel(grads[k[2:]], z[k]) < 1e-3, k
