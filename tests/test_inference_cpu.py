"""Camera rays of evaluation rendering against the reference's camera.get_center_and_ray
(golden fixture tests/golden/camera.npz); CPU."""
import numpy as np
import torch

from neuralangelo_gb300.inference import camera_rays
from tests import golden_io


def test_camera_rays_match_reference_golden():
    z = np.load(golden_io.GOLDEN + "/camera.npz")
    H, W = int(z['H']), int(z['W'])
    for i in range(z['pose'].shape[0]):
        c, r = camera_rays(torch.from_numpy(z['pose'][i]), torch.from_numpy(z['intr'][i]), H, W)
        assert np.allclose(c.numpy(), z['center'][i], rtol=1e-6, atol=1e-6)
        assert np.allclose(r.numpy(), z['ray'][i], rtol=1e-5, atol=1e-6)
