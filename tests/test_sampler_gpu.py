"""GPU hierarchical sampler (gbsdf_sampler_coarse / gbsdf_sampler_round, C ABI) against
the golden vectors of the reference's own Model.sample_dists_all
(tests/golden/make_golden_sampler.py) and the oracle (oracle/sampler.py).

Tolerances.  The kernels compute in float32, as the reference does on a GPU; the
golden vectors are float64.  Per round, a ray falls in one of three classes by
its float64 weight sum W:
  * W > 1e-2 (the ray crosses the surface): fine distances within 2e-5 of the
    ray span (far - near) of the golden ones (float32 noise measured <= 5e-6);
  * W == 0 (no surface in reach even in float64): every fine sample sits on
    the last bin, bit-exact (nerf_util.py:57-66);
  * otherwise the float32 sigmoid saturates where float64 does not, and the
    normalised weights are ill-conditioned in either precision: the fine
    distances only have to stay inside the list's range.
Sorting is index work and is checked bit-exact."""
import ctypes
import os

import numpy as np
import pytest
import torch

from neuralangelo_gb300.sampler import HierarchicalSampler, SamplerArgs, field_sdf_fn, plain_sdf_fn
from neuralangelo_gb300 import _lib
from oracle import sampler as osm

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sampler.npz")


def wobbly(x):
    r = x.norm(dim=-1)
    w = torch.sin(5 * x[..., 0]) * torch.sin(5 * x[..., 1]) * torch.sin(5 * x[..., 2])
    return r - 0.5 + 0.05 * w


def golden():
    return dict(np.load(GOLDEN))


def weight_sum64(d, s, inv_s):
    d, s = torch.from_numpy(d), torch.from_numpy(s)
    prev_s, next_s, prev_d, next_d = s[:, :-1], s[:, 1:], d[:, :-1], d[:, 1:]
    mid = (prev_s + next_s) * 0.5
    cos = (next_s - prev_s) / (next_d - prev_d + 1e-5)
    cos = torch.minimum(torch.cat([torch.zeros_like(cos[:, :1]), cos[:, :-1]], -1), cos)
    iv = next_d - prev_d
    pc, nc = torch.sigmoid((mid - cos * iv * 0.5) * inv_s), torch.sigmoid((mid + cos * iv * 0.5) * inv_s)
    a = ((pc - nc) / (pc + 1e-5)).clamp(0, 1)
    return osm.compositing_weights(a).sum(1).numpy()


def check_fine(fine, ref_fine, lists, W, span):
    good = W > 1e-2
    assert good.sum() >= 25
    err = np.abs(fine - ref_fine) / span
    assert err[good].max() < 2e-5, err[good].max()
    dead = W == 0
    if dead.any():
        assert np.array_equal(fine[dead], np.repeat(lists[dead, -1:], fine.shape[1], 1))
    lo, hi = lists.min(1, keepdims=True), lists.max(1, keepdims=True)
    assert np.all(fine >= lo) and np.all(fine <= hi)


def run_round(z, h, merge):
    """One gbsdf_sampler_round on the golden inputs of round h (float32)."""
    R = z['center'].shape[0]
    c = torch.from_numpy(z['center']).float().to(DEV)
    d = torch.from_numpy(z['ray_unit']).float().to(DEV)
    if merge:   # the list before round h's merge + round h-1's fine samples
        base_d = z[f'round{h - 1}_dists']
        base_s = z[f'round{h - 1}_sdfs']
        md = z[f'round{h - 1}_fine']
        pts = torch.from_numpy(z['center'])[:, None] + torch.from_numpy(z['ray_unit'])[:, None] * \
            torch.from_numpy(md)[..., None]
        ms = wobbly(pts).numpy()
    else:
        base_d, base_s = z[f'round{h}_dists'], z[f'round{h}_sdfs']
        md = ms = None
    n_list = base_d.shape[1]
    n_merge = 0 if md is None else md.shape[1]
    ld = n_list + n_merge
    dists = torch.zeros(R, ld, device=DEV)
    sdfs = torch.zeros(R, ld, device=DEV)
    dists[:, :n_list] = torch.from_numpy(base_d).float()
    sdfs[:, :n_list] = torch.from_numpy(base_s).float()
    fine = torch.empty(R, 16, device=DEV)
    fpts = torch.empty(R * 16, 3, device=DEV)
    mdt = torch.from_numpy(md).float().to(DEV) if md is not None else None
    mst = torch.from_numpy(ms).float().to(DEV) if ms is not None else None
    a = SamplerArgs()
    a.R, a.ld, a.n_list, a.n_merge, a.n_fine, a.inv_s, a.robust = R, ld, n_list, n_merge, 16, 64.0 * 2 ** h, 1
    a.center, a.ray_unit, a.dists, a.sdfs = c.data_ptr(), d.data_ptr(), dists.data_ptr(), sdfs.data_ptr()
    a.merge_d = mdt.data_ptr() if mdt is not None else None
    a.merge_s = mst.data_ptr() if mst is not None else None
    a.fine_d, a.fine_pts = fine.data_ptr(), fpts.data_ptr()
    _lib.call("gbsdf_sampler_round", ctypes.byref(a), _lib.stream_ptr(DEV))
    torch.cuda.synchronize()
    return dists.cpu().numpy(), sdfs.cpu().numpy(), fine.cpu().numpy(), fpts.cpu().numpy(), (mdt, mst)


@pytest.mark.parametrize("h", [0, 1, 2, 3])
def test_round_on_reference_inputs(h):
    z = golden()
    span = z['far'] - z['near']
    dl, sl, fine, fpts, _ = run_round(z, h, merge=False)
    W = weight_sum64(z[f'round{h}_dists'], z[f'round{h}_sdfs'], 64.0 * 2 ** h)
    check_fine(fine, z[f'round{h}_fine'], z[f'round{h}_dists'].astype(np.float32), W, span)
    # the points handed to the SDF evaluation are c + d t in float32
    c = z['center'].astype(np.float32)
    u = z['ray_unit'].astype(np.float32)
    ref_pts = (c[:, None] + u[:, None] * fine[..., None]).reshape(-1, 3)
    np.testing.assert_allclose(fpts, ref_pts, rtol=0, atol=1e-6)


@pytest.mark.parametrize("h", [1, 2, 3])
def test_merge_is_the_reference_sort(h):
    """Sorting round h-1's fine samples into the list gives round h's list: bit-exact
    on the float32 values, with each SDF value travelling with its distance."""
    z = golden()
    dl, sl, fine, _, (mdt, mst) = run_round(z, h, merge=True)
    ref = z[f'round{h}_dists'].astype(np.float32)
    assert np.array_equal(dl, ref)
    src_d = np.concatenate([z[f'round{h - 1}_dists'].astype(np.float32), mdt.cpu().numpy()], 1)
    src_s = np.concatenate([z[f'round{h - 1}_sdfs'].astype(np.float32), mst.cpu().numpy()], 1)
    for r in range(dl.shape[0]):
        order = np.argsort(src_d[r], kind='stable')
        assert np.array_equal(dl[r], src_d[r][order])
        assert np.array_equal(sl[r], src_s[r][order])


def test_full_sampler_matches_reference():
    z = golden()
    t = {k: torch.from_numpy(v).float().to(DEV) for k, v in z.items()}
    smp = HierarchicalSampler(64, 16, 4)
    trace = []
    d = smp(lambda p: wobbly(p), t['center'], t['ray_unit'], t['near'], t['far'], u=t['u'], trace=trace)
    d = d.cpu().numpy()
    span = z['far'] - z['near']
    assert d.shape == (40, 128)
    assert np.all(np.diff(d, axis=1) >= 0)
    Ws = np.stack([weight_sum64(z[f'round{h}_dists'], z[f'round{h}_sdfs'], 64.0 * 2 ** h) for h in range(4)])
    stable = np.all(Ws > 1e-2, 0) | np.all(Ws == 0, 0)
    assert stable.sum() >= 25
    err = np.abs(d - z['dists']) / span
    assert err[stable].max() < 1e-4, err[stable].max()
    assert np.all(d >= z['near'] - 1e-6) and np.all(d <= z['far'] + 1e-6)


def test_coarse_is_bit_exact_and_non_stratified_default():
    """Stratified coarse distances are the float32 formula of nerf_util.py:31-37 bit for bit;
    u = None is the non-stratified 0.5 case; n_hierarchy = 0 returns them unchanged."""
    z = golden()
    t = {k: torch.from_numpy(v).float() for k, v in z.items()}
    ref = osm.stratified_dists(t['near'], t['far'], 64, t['u'])
    smp = HierarchicalSampler(64, 16, 0)
    g = {k: v.to(DEV) for k, v in t.items()}
    d = smp(None, g['center'], g['ray_unit'], g['near'], g['far'], u=g['u']).cpu()
    assert torch.equal(d, ref)
    d5 = smp(None, g['center'], g['ray_unit'], g['near'], g['far']).cpu()
    assert torch.equal(d5, osm.stratified_dists(t['near'], t['far'], 64, None))


def test_empty_and_invalid():
    smp = HierarchicalSampler(64, 16, 4)
    e = torch.empty(0, 3, device=DEV)
    out = smp(None, e, e, torch.empty(0, 1, device=DEV), torch.empty(0, 1, device=DEV))
    assert out.shape == (0, 128)
    a = SamplerArgs()
    a.R, a.ld, a.n_list, a.n_merge, a.n_fine = 4, 64, 64, 16, 16
    with pytest.raises(RuntimeError, match="NULL"):
        _lib.call("gbsdf_sampler_round", ctypes.byref(a), _lib.stream_ptr(DEV))
    buf = torch.zeros(4 * 96, device=DEV)
    a.center = a.ray_unit = a.dists = a.sdfs = a.merge_d = a.merge_s = a.fine_d = buf.data_ptr()
    with pytest.raises(RuntimeError, match="row stride"):
        _lib.call("gbsdf_sampler_round", ctypes.byref(a), _lib.stream_ptr(DEV))
    with pytest.raises(ValueError):
        HierarchicalSampler(256, 32, 9)


def test_field_sampler_fused_and_plain_sdf_agree():
    """The sampler driven by the fused FP16 field kernel and by the plain FP32 field
    places nearly the same samples (they differ only by the field's fp16 weights)."""
    from neuralangelo_gb300.config import field_config
    from neuralangelo_gb300.model import FieldModel
    from neuralangelo_gb300.workloads import full_field_iteration, init_field_params, make_rays, sphere_bounds
    cfg = field_config("full")
    cfg.sdf.encoding.hashgrid.dict_size = 16
    torch.manual_seed(0)
    model = FieldModel(cfg).to(DEV)
    init_field_params(model, 0)
    model.schedule(full_field_iteration(8))
    b = make_rays(512, 1, seed=2, device=DEV)
    near, far, outside = sphere_bounds(b['center'], b['ray_unit'])
    u = torch.rand(512, 64, device=DEV, generator=torch.Generator(device=DEV).manual_seed(1))
    smp = HierarchicalSampler()
    d_fused = smp(field_sdf_fn(model.neural_sdf), b['center'], b['ray_unit'], near, far, u=u)
    d_plain = smp(plain_sdf_fn(model.neural_sdf), b['center'], b['ray_unit'], near, far, u=u)
    span = (far - near)
    assert torch.all(d_fused[:, 1:] >= d_fused[:, :-1])
    close = ((d_fused - d_plain).abs() / span < 1e-3).float().mean().item()
    assert close > 0.95, close
