"""Load a golden fixture (tests/golden/*.npz) into the oracle's parameter / batch form."""
import os

import numpy as np
import torch

from oracle import field as of

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("field_c1_small", "field_c0_small", "field_taps4_small")


def load(name):
    z = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    (L, Fd, log2T, base, rmax, hidden, rgb_hidden, rgb_layers, taps, active, anneal, app_dim,
     n_images) = [int(v) for v in z['cfg']]
    eps, progress, w_eik, w_curv, growth = [float(v) for v in z['scalars']]
    cfg = of.make_config(n_levels=L, n_features=Fd, log2_hashmap_size=log2T, base_resolution=base,
                         max_resolution=rmax, active_levels=active, sdf_hidden=hidden, rgb_hidden=rgb_hidden,
                         rgb_layers=rgb_layers, app_dim=app_dim, n_images=n_images, taps=taps)
    params = {k[2:]: torch.from_numpy(v) for k, v in z.items() if k.startswith('p_')}
    batch = dict(center=torch.from_numpy(z['center']), ray_unit=torch.from_numpy(z['ray_unit']),
                 dists=torch.from_numpy(z['dists']), far=torch.from_numpy(z['far']),
                 outside=torch.from_numpy(z['outside']), target=torch.from_numpy(z['target']),
                 app_idx=torch.from_numpy(z['app_idx']))
    return dict(z=z, cfg=cfg, params=params, batch=batch, eps=eps, progress=progress, w_eik=w_eik,
                w_curv=w_curv, anneal=anneal)
