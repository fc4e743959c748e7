"""The launch-shape autotuner: it picks valid shapes for every tunable call of the step,
caches them per workload, and the tuned step computes what the default one does."""
import json

import pytest
import torch

from neuralangelo_gb300.autotune import StepTuner
from neuralangelo_gb300.fused import CapturedStep, FusedField
from neuralangelo_gb300.workloads import make_ragged_rays
from tests.test_fused_gpu import build, fused_grads, rel

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def test_tuned_step_matches_default(tmp_path):
    model = build()
    batch = make_ragged_rays(300, seed=3, zero_frac=0.3, lo=16, hi=128, n_images=10, device=DEV)
    ff = FusedField(model)
    model.zero_grad(set_to_none=True)
    ref_loss = ff.step(batch)['loss']
    ref = {k: v.clone() for k, v in fused_grads(model).items()}
    path = tmp_path / "tune.json"
    tuner = StepTuner(ff, reps=3, cache_path=str(path))
    choice = tuner.tune(batch)
    print("\nchoice", choice, "\ntimings", {k: {str(a): round(b, 4) for a, b in v.items()} for k, v in tuner.timings.items()})
    assert choice['scatter_cpt'] in StepTuner.SCATTER_CPT and choice['fwd_ctas'] in StepTuner.FWD_CTAS
    assert choice['dense'] and all(list(v) in [list(s) for s in StepTuner.DENSE_SHAPES] for v in choice['dense'].values())
    assert ff.tuning == {k: v for k, v in choice.items() if k != 'dense'}
    # the tuned step, eager and captured, computes the same step (atomics reorder only)
    model.zero_grad(set_to_none=True)
    loss = ff.step(batch)['loss']
    assert abs(loss - ref_loss) <= 1e-6 * abs(ref_loss)
    g = fused_grads(model)
    for k in ('table', 'sdf.l0.v', 'sdf.l1.v', 'rgb.l0.v', 's_var', 'app'):
        assert rel(g[k], ref[k]) < 1e-5, k
    cap = CapturedStep(ff, batch)
    cap.replay()
    torch.cuda.synchronize()
    assert abs(cap.losses()['loss'] - ref_loss) <= 1e-6 * abs(ref_loss)
    # the cache: a second tuner on the same workload reads the choice back without timing
    saved = json.loads(path.read_text())
    assert tuner.key(batch) in saved
    t2 = StepTuner(ff, cache_path=str(path))
    assert t2.tune(batch) == saved[tuner.key(batch)] and not t2.timings
