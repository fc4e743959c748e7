"""The reference's own NeuralSDF (projects/neuralangelo/utils/modules.py:24-178), imported
unmodified, with this package standing in for tiny-cuda-nn (sys.modules["tinycudann"]):
it builds on the drop-in encoder and shares the package NeuralSDF's parameter names,
shapes and checkpoints (CPU); on a GPU its forward and numerical gradients, forward and
backward, run through this library's hash-grid kernels and match the package's own.

The reference checkout is not part of this repository: set NEURALANGELO_REFERENCE to its
path (the directory holding projects/ and imaginaire/) to run these tests."""
import importlib
import os
import sys

import pytest
import torch

from neuralangelo_gb300 import encoding
from neuralangelo_gb300.config import sdf_config
from neuralangelo_gb300.modules import NeuralSDF

REF = os.environ.get("NEURALANGELO_REFERENCE")
pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF or "", "projects")),
                                reason="NEURALANGELO_REFERENCE does not name a neuralangelo checkout")


@pytest.fixture(scope="module")
def ref_modules():
    saved = sys.modules.get("tinycudann")
    sys.modules["tinycudann"] = encoding
    sys.path.insert(0, REF)
    try:
        mod = importlib.import_module("projects.neuralangelo.utils.modules")
        yield mod
    finally:
        sys.path.remove(REF)
        if saved is None:
            sys.modules.pop("tinycudann", None)
        else:
            sys.modules["tinycudann"] = saved


def configs():
    """The full field's SDF configuration (base.yaml:40-68 shapes: L16 F8, 32 -> 2048) as the
    reference reads it, and the package's own."""
    from tests.golden.make_golden import ref_configs
    ref_sdf, _ = ref_configs(16, 8, 5, 11, 14, 256, 256, 4, 6, 8)
    ours = sdf_config(levels=16, dim=8, dict_size=14, min_logres=5, max_logres=11, hidden=256, taps=6)
    return ref_sdf, ours


def test_reference_neural_sdf_builds_on_the_drop_in(ref_modules):
    ref_sdf, ours_cfg = configs()
    ref = ref_modules.NeuralSDF(ref_sdf)
    assert isinstance(ref.tcnn_encoding, encoding.HashGridEncoding)
    ours = NeuralSDF(ours_cfg)
    a, b = ref.state_dict(), ours.state_dict()
    assert sorted(a) == sorted(b)                                  # checkpoint keys
    for k in a:
        assert a[k].shape == b[k].shape, k
    ref.load_state_dict(b)                                         # the package's checkpoint loads
    assert torch.equal(ref.tcnn_encoding.params, ours.tcnn_encoding.params)


@pytest.mark.gpu
def test_reference_neural_sdf_runs_on_the_kernels(ref_modules):
    ref_sdf, ours_cfg = configs()
    torch.manual_seed(0)
    ours = NeuralSDF(ours_cfg).cuda()
    with torch.no_grad():
        ours.tcnn_encoding.params.uniform_(-1e-2, 1e-2)
    ref = ref_modules.NeuralSDF(ref_sdf).cuda()
    ref.load_state_dict(ours.state_dict())
    for m in (ref, ours):
        m.warm_up_end = 5000                      # set by the reference's trainer (trainer.py:63-74)
        m.set_active_levels(45000)
        m.set_normal_epsilon()
    x = (torch.rand(4096, 3, device="cuda") * 2 - 1) * 0.8
    outs = []
    for m in (ref, ours):
        m.zero_grad(set_to_none=True)
        sdf, feat = m(x)
        g, h = m.compute_gradients(x, training=True, sdf=sdf)
        (sdf.sum() + feat.mean() + g.norm(dim=-1).sum() + h.abs().sum()).backward()
        outs.append((sdf.detach(), g.detach(), h.detach(), m.tcnn_encoding.params.grad.clone()))
    for a, b in zip(*outs):
        assert ((a - b).norm() / b.norm().clamp_min(1e-30)).item() < 1e-5
