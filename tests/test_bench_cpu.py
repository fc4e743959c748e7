"""bench.py's roofline bookkeeping, on the CPU: every field call's DRAM traffic is read
from measured_traffic.json (figures of an ncu capture), and the MLP calls' figures agree
with the algorithmic bytes the bench divides by."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


CALLS = ("gbsdf_field_encode", "gbsdf_field_mlp_fwd", "gbsdf_field_mlp_bwd", "gbsdf_field_scatter")


def test_every_field_call_has_profiled_traffic(bench):
    for call in CALLS:
        per_sample, source, _ = bench.profiled_traffic(call)
        assert per_sample is not None and per_sample > 0, call
        assert "ncu" in source, source


def test_mlp_traffic_matches_the_algorithmic_bytes(bench):
    """The MLP calls move what they must (8 active levels of 8 features, K0 = 64):
    forward x0ext rows in, SDF/gradient/Hessian/h0c/colour tail (hi + lo pairs) out; backward x0ext rows,
    d_h0c and the output gradients in, d_enc out, the layer-0 weight gradient on chip."""
    K0, H = 64, 256
    KX = 2 * K0 + 16
    fwd = 7 * KX * 2 + 4 + 12 + 12 + ((H + 8) * 2 + 48 * 2) * 2      # h0c row and colour tail as hi + lo
    bwd = 7 * KX * 2 + H * 4 + 52 + 7 * K0 * 4
    for call, algo in (("gbsdf_field_mlp_fwd", fwd), ("gbsdf_field_mlp_bwd", bwd)):
        measured, _, _ = bench.profiled_traffic(call)
        assert abs(measured - algo) < 0.05 * algo, (call, measured, algo)


def test_unknown_call_has_no_traffic(bench):
    assert bench.profiled_traffic("gbsdf_no_such_call") == (None, None, None)
