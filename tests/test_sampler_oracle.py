"""Pin the sampler oracle (oracle/sampler.py) against golden vectors produced by the
reference's own Model.sample_dists_all (tests/golden/make_golden_sampler.py)."""
import os

import numpy as np
import torch

from oracle import sampler as osm

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sampler.npz")


def wobbly_sphere(x):
    r = x.norm(dim=-1)
    w = torch.sin(5 * x[..., 0]) * torch.sin(5 * x[..., 1]) * torch.sin(5 * x[..., 2])
    return r - 0.5 + 0.05 * w


def load():
    z = dict(np.load(GOLDEN))
    t = {k: torch.from_numpy(v) for k, v in z.items()}
    return z, t


def test_sampler_oracle_matches_reference():
    z, t = load()
    n_coarse, n_fine, n_hier = (int(v) for v in z['sizes'])
    trace = []
    dists = osm.sample_dists_all(t['center'], t['ray_unit'], t['near'], t['far'], wobbly_sphere, n_coarse, n_fine,
                                 n_hier, u=t['u'], trace=trace)
    assert dists.shape == (40, n_coarse + n_hier * n_fine)
    np.testing.assert_allclose(dists.numpy(), z['dists'], rtol=0, atol=1e-12)
    for h, (dd, ss, ff) in enumerate(trace):
        np.testing.assert_allclose(dd.numpy(), z[f'round{h}_dists'], rtol=0, atol=1e-12)
        np.testing.assert_allclose(ss.numpy(), z[f'round{h}_sdfs'], rtol=0, atol=1e-12)
        np.testing.assert_allclose(ff.numpy(), z[f'round{h}_fine'], rtol=0, atol=1e-12)


def test_each_round_from_the_reference_inputs():
    """One hierarchical round at a time, fed the reference's own round inputs."""
    z, t = load()
    n_fine = int(z['sizes'][1])
    for h in range(int(z['sizes'][2])):
        fine = osm.hierarchical_dists(t[f'round{h}_dists'], t[f'round{h}_sdfs'], 64 * 2 ** h, n_fine)
        np.testing.assert_allclose(fine.numpy(), z[f'round{h}_fine'], rtol=0, atol=1e-12)


def test_sampler_outputs_sorted_inside_bounds():
    z, _ = load()
    d = z['dists']
    assert np.all(np.diff(d, axis=1) >= 0)
    assert np.all(d >= z['near'] - 1e-12) and np.all(d <= z['far'] + 1e-12)
    assert z['outside'][:3].all() and not z['outside'][3:].any()


def test_zero_weights_fall_back_to_last_bin():
    """All-zero weights (a ray far from the surface): cdf stays 0, searchsorted returns N
    and every fine sample lands on the last bin (nerf_util.py:57-66)."""
    bins = torch.linspace(1.0, 2.0, 9, dtype=torch.float64)[None]
    fine = osm.pdf_dists(bins, torch.zeros(1, 8, dtype=torch.float64), 4)
    assert torch.equal(fine, torch.full((1, 4), 2.0, dtype=torch.float64))
