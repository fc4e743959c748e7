"""tcgen05 dense-layer kernel against a float32 torch reference of the same op."""
import pytest
import torch

from neuralangelo_gb300 import dense as D

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def ref(X, W, b, epi, beta, G):
    z = X.float() @ W.float().t()
    if epi in (D.EPI_IDENTITY, D.EPI_RELU, D.EPI_SOFTPLUS) and b is not None:
        z = z + b
    if epi == D.EPI_RELU:
        z = torch.relu(z)
    elif epi == D.EPI_SOFTPLUS:
        z = torch.nn.functional.softplus(z, beta=beta)
    elif epi == D.EPI_DRELU:
        z = z * (G.float() > 0).float()
    elif epi == D.EPI_DSOFTPLUS:
        z = z * (1 - torch.exp(-beta * G.float()))
    return z


@pytest.mark.parametrize("M,K,N", [(128, 64, 256), (1000, 256, 256), (777, 304, 256), (300, 256, 128),
                                   (129, 32, 64), (5000, 256, 256)])
@pytest.mark.parametrize("epi", [D.EPI_IDENTITY, D.EPI_RELU, D.EPI_SOFTPLUS, D.EPI_DRELU, D.EPI_DSOFTPLUS])
def test_dense_matches_torch(M, K, N, epi):
    g = torch.Generator(DEV).manual_seed(M + K + N + epi)
    X = (torch.randn(M, K, device=DEV, generator=g) * 0.5).half()
    W = (torch.randn(N, K, device=DEV, generator=g) / K ** 0.5).half()
    b = torch.randn(N, device=DEV, generator=g) * 0.1
    G = None
    if epi == D.EPI_DRELU:
        G = torch.randn(M, N, device=DEV, generator=g).half()
    elif epi == D.EPI_DSOFTPLUS:   # a softplus output is positive
        G = (torch.rand(M, N, device=DEV, generator=g) * 0.05).half()
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    Y = D.dense(X, W, b, epi=epi, beta=100.0 if epi in (D.EPI_SOFTPLUS, D.EPI_DSOFTPLUS) else 1.0, G=G, err=err)
    torch.cuda.synchronize()
    assert int(err) == 0
    beta = 100.0 if epi in (D.EPI_SOFTPLUS, D.EPI_DSOFTPLUS) else 1.0
    R = ref(X, W, b, epi, beta, G)
    e = (Y.float() - R).norm() / R.norm().clamp_min(1e-12)
    assert e < 2e-3, float(e)


def test_dense_strided_output_and_input():
    M, K, N = 513, 256, 256
    g = torch.Generator(DEV).manual_seed(7)
    big = torch.randn(M, 320, device=DEV, generator=g).half()
    W = (torch.randn(N, K, device=DEV, generator=g) / 16).half()
    out = torch.zeros(M, 512, device=DEV, dtype=torch.float16)
    D.dense(big, W, None, epi=D.EPI_RELU, out=out[:, 256:], K=K)
    R = torch.relu(big[:, :K].float() @ W.float().t())
    assert ((out[:, 256:].float() - R).norm() / R.norm()) < 2e-3
    assert torch.all(out[:, :256] == 0)


@pytest.mark.parametrize("pad,epi", [(0, D.EPI_DRELU), (8, D.EPI_RELU)])
def test_dense_split_operand_and_output(pad, epi):
    """X = X_hi + X_lo and Y = Y_hi + Y_lo: the pair reproduces an fp32 product far below fp16
    precision.  pad 8: outputs in [M, N + 8] buffers (the activation layout of the fused step,
    written back through TMA stores of both halves)."""
    M, K, N = 700, 256, 256
    g = torch.Generator(DEV).manual_seed(11)
    Xf = torch.randn(M, K, device=DEV, generator=g)
    X_hi = Xf.half()
    X_lo = (Xf - X_hi.float()).half()
    W = (torch.randn(N, K, device=DEV, generator=g) / 16).half()
    G = torch.randn(M, N, device=DEV, generator=g).half()
    b = torch.randn(N, device=DEV, generator=g)
    hi = torch.full((M, N + pad), 7.0, device=DEV, dtype=torch.float16)
    lo = torch.full((M, N + pad), 7.0, device=DEV, dtype=torch.float16)
    if epi == D.EPI_DRELU:
        D.dense(X_hi, W, None, epi=epi, G=G, out=hi[:, :N], X_lo=X_lo, out_lo=lo[:, :N])
        R = (Xf.double() @ W.double().t()) * (G.double() > 0)
    else:
        D.dense(X_hi, W, b, epi=epi, out=hi[:, :N], X_lo=X_lo, out_lo=lo[:, :N])
        R = torch.relu(Xf.double() @ W.double().t() + b.double())
    assert torch.all(hi[:, N:] == 7) and torch.all(lo[:, N:] == 7)      # padding columns untouched
    hi, lo = hi[:, :N], lo[:, :N]
    e_pair = ((hi.double() + lo.double()) - R).norm() / R.norm()
    e_hi = (hi.double() - R).norm() / R.norm()
    assert e_pair < 1e-5, float(e_pair)
    assert e_hi > 1e-4                       # a single fp16 output is much coarser


@pytest.mark.parametrize("epi", [D.EPI_SOFTPLUS, D.EPI_DSOFTPLUS])
def test_dense_fp32_softplus_epilogues_against_cuda_math(epi):
    """The fused kernels' softplus(beta = 100) and its derivative (change of base to the
    MUFU ex2 / lg2 / rcp approximations) against torch's softplus and exp (CUDA's
    expf / log1pf) on the same FP32 pre-activations, with FP32 outputs so the FP16
    storage of the fused path does not hide the function's own error.  The
    pre-activations span the far tail (beta z ~ -40), the steep middle and torch's
    identity threshold (beta z > 20)."""
    M, K, N = 4096, 16, 128
    g = torch.Generator(DEV).manual_seed(11 + epi)
    X = (torch.randn(M, K, device=DEV, generator=g) * 0.5).half()
    W = (torch.randn(N, K, device=DEV, generator=g) * 0.08).half()
    b = torch.linspace(-0.4, 0.4, N, device=DEV)
    beta = 100.0
    G = None
    if epi == D.EPI_DSOFTPLUS:   # a softplus output: positive, from ~1e-6 up to ~0.4
        G = torch.nn.functional.softplus(torch.randn(M, N, device=DEV, generator=g) * 0.15, beta=beta).half()
    out = torch.empty(M, N, device=DEV, dtype=torch.float32)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    D.dense(X, W, b, epi=epi, beta=beta, G=G, out=out, err=err)
    torch.cuda.synchronize()
    assert int(err) == 0
    z = X.float() @ W.float().t()
    # the tensor core and torch sum the 16 products in different orders: an FP32
    # difference of order 2^-24 sum |x w| that is absolute, not relative to |z|
    zabs = X.float().abs() @ W.float().abs().t()
    if epi == D.EPI_SOFTPLUS:
        z = z + b
        assert float((z * beta).min()) < -30 and float((z * beta).max()) > 25
        R = torch.nn.functional.softplus(z, beta=beta)
        # relative 1e-5, with an absolute floor for the lg2 approximation near 1 + e = 1
        bound = 1e-5 * R.abs() + 2e-8 + 1e-6 * zabs
    else:
        R = z * (1 - torch.exp(-beta * G.float()))
        # 1 - e^(-beta g) cancels for small g: the ex2 approximation's ~2^-22 error on e
        # is then absolute, relative to |z|
        bound = 1e-5 * R.abs() + 5e-7 * z.abs() + 1e-6 * zabs
    excess = ((out - R).abs() - bound).max()
    assert float(excess) <= 0.0, float(excess)
