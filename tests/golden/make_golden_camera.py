"""Golden fixture for the camera rays of evaluation rendering: the REFERENCE's own
camera.get_center_and_ray (projects/nerf/utils/camera.py:283-311) on two seeded poses
and intrinsics, float32 on the CPU.

Usage (needs the reference checkout; writes tests/golden/camera.npz):
    python tests/golden/make_golden_camera.py /root/reference
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    sys.path.insert(0, ref_root)
    from projects.nerf.utils import camera
    g = torch.Generator().manual_seed(3)
    poses, intrs = [], []
    for _ in range(2):
        q, _ = torch.linalg.qr(torch.randn(3, 3, generator=g))
        q = q * torch.sign(torch.det(q))
        t = torch.randn(3, 1, generator=g) * 2
        poses.append(torch.cat([q, t], dim=1))
        f = 20 + 10 * torch.rand(2, generator=g)
        intrs.append(torch.tensor([[float(f[0]), 0.0, 12.3], [0.0, float(f[1]), 7.9], [0.0, 0.0, 1.0]]))
    pose, intr = torch.stack(poses), torch.stack(intrs)
    H, W = 14, 22
    center, ray = camera.get_center_and_ray(pose, intr, (H, W))
    np.savez_compressed(os.path.join(HERE, "camera.npz"), pose=pose.numpy(), intr=intr.numpy(), H=H, W=W,
                        center=center.numpy(), ray=ray.numpy())
    print("wrote camera.npz", tuple(center.shape))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the neuralangelo reference checkout>")
    main(sys.argv[1])
