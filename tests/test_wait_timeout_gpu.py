"""Failure detection on the GPU: a bounded mbarrier wait that nothing completes runs out
after its limit and reports it (gbsdf_selftest_wait exercises the same umma::mbar_wait
that the tensor-core kernels use); the context stays usable afterwards."""
import ctypes

import pytest
import torch

from neuralangelo_gb300 import _lib
from neuralangelo_gb300 import dense as D

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
_lib.register("gbsdf_selftest_wait", [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p])


def run(timeout_ns, arrive_first):
    st = torch.full((2,), -1, device=DEV, dtype=torch.int32)
    _lib.call("gbsdf_selftest_wait", int(timeout_ns), int(arrive_first), ctypes.c_void_p(st.data_ptr()),
              _lib.stream_ptr(DEV))
    torch.cuda.synchronize()
    return st.tolist()


@pytest.mark.parametrize("limit_ms", [1, 20])
def test_wait_that_nothing_completes_runs_out(limit_ms):
    timed_out, us = run(limit_ms * 1_000_000, arrive_first=False)
    assert timed_out == 1
    assert limit_ms * 1000 <= us < limit_ms * 1000 + 50_000      # it waited the limit, then returned
    # the context is still usable: a tensor-core kernel runs and is right
    X = torch.randn(300, 64, device=DEV).half()
    W = torch.randn(64, 64, device=DEV).half()
    Y = D.dense(X, W, out=torch.empty(300, 64, device=DEV))
    ref = X.float() @ W.float().t()
    assert ((Y.float() - ref).norm() / ref.norm()) < 2e-3


def test_completed_wait_returns_at_once():
    timed_out, us = run(1_000_000_000, arrive_first=True)
    assert timed_out == 0 and us < 1000


def test_wait_limit_is_bounded():
    with pytest.raises(RuntimeError, match="timeout"):
        run(5_000_000_000, arrive_first=False)
