"""tcgen05 weight-gradient kernel (gbsdf_wgrad) against a float64 torch reference of the
same op: dW = (accumulate ? dW : 0) + (dZ + dZ_lo)[:, :N]^T X[:, :K] on fp16 inputs.
fp16 x fp16 products are exact in FP32, so the only error is FP32 accumulation order."""
import pytest
import torch

from neuralangelo_gb300 import fused

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def ref(dZ, X, N, K, dZ_lo=None):
    z = dZ[:, :N].double()
    if dZ_lo is not None:
        z = z + dZ_lo[:, :N].double()
    return z.t() @ X[:, :K].double()


def rel(a, b):
    return float((a.double() - b).norm() / b.norm().clamp_min(1e-300))


@pytest.mark.parametrize("M,N,K,ldz,ldx", [
    (1, 256, 264, 256, 264),          # one row
    (1000, 128, 304, 128, 304),       # colour layer 0 (K not a multiple of 64)
    (70001, 256, 264, 256, 264),      # hidden layers: ragged last stage, many CTAs
    (5000, 272, 264, 272, 264),       # three dW row blocks (the background layer 7)
    (3000, 64, 96, 64, 352),          # narrow dZ, X a column slice of a wider buffer
    (20000, 256, 384, 256, 384),      # the widest X
])
def test_wgrad_matches_float64(M, N, K, ldz, ldx):
    g = torch.Generator(DEV).manual_seed(M + N + K)
    dZ = torch.randn(M, ldz, device=DEV, generator=g).half()
    Xb = torch.randn(M, ldx + 256, device=DEV, generator=g).half()
    X = Xb[:, 256:256 + ldx] if ldx < 352 else Xb[:, :ldx]
    dW = torch.full((N, K + 8), 5.0, device=DEV)
    fused._wgrad(dZ, X, N, K, dW[:, :K])
    torch.cuda.synchronize()
    R = ref(dZ, X, N, K).cpu()
    assert rel(dW[:, :K].cpu(), R) < 1e-5
    assert torch.all(dW[:, K:] == 5.0)                  # columns past K untouched


def test_wgrad_lo_half_and_accumulate():
    """dZ as an fp16 hi + lo pair reproduces an FP32 dZ far below fp16 precision, and a
    second call adds into dW."""
    M, N, K = 30000, 256, 144
    g = torch.Generator(DEV).manual_seed(5)
    Zf = torch.randn(M, N, device=DEV, generator=g) * 100.0
    hi = Zf.half()
    lo = (Zf - hi.float()).half()
    X = torch.randn(M, K, device=DEV, generator=g).half()
    dW = torch.empty(N, K, device=DEV)
    fused._wgrad(hi, X, N, K, dW, dZ_lo=lo)
    exact = (Zf.double().t() @ X.double()).cpu()
    e_pair = rel(dW.cpu(), exact)
    single = torch.empty(N, K, device=DEV)
    fused._wgrad(hi, X, N, K, single)
    e_single = rel(single.cpu(), exact)
    print(f"\npair {e_pair:.1e} single fp16 {e_single:.1e}")
    assert e_pair < 1e-5 and e_single > 10 * e_pair
    fused._wgrad(hi, X, N, K, dW, dZ_lo=lo, accumulate=True)
    assert rel(dW.cpu(), 2 * exact) < 1e-5


def test_wgrad_rejects_bad_arguments():
    dZ = torch.zeros(16, 1024, device=DEV, dtype=torch.float16)
    X = torch.zeros(16, 64, device=DEV, dtype=torch.float16)
    dW = torch.zeros(1024, 64, device=DEV)
    with pytest.raises(RuntimeError, match="at most 512"):
        fused._wgrad(dZ, X, 1024, 64, dW)
