"""Python entry to the tcgen05 dense-layer kernel (gbsdf_dense)."""
import torch

from . import _lib

EPI_IDENTITY, EPI_RELU, EPI_SOFTPLUS, EPI_DRELU, EPI_DSOFTPLUS = range(5)


def dense(X, W, bias=None, epi=EPI_IDENTITY, beta=100.0, G=None, out=None, err=None, K=None, X_lo=None,
          out_lo=None):
    """Y = epi((X + X_lo)[:, :K] @ W.T + bias ; G) with fp16 operands on the tensor cores.

    X [M, ldx] fp16 (row stride may exceed K), W [N, K] fp16, bias [N] fp32,
    G [M, N]-shaped fp16 gate for the backward epilogues; returns Y [M, N] fp16
    or fp32 (or writes into ``out``, which may be a column slice view with row
    stride).  X_lo / out_lo carry the low fp16 halves of split operands."""
    _lib.require_cuda(X, W)
    M = X.shape[0]
    N, Kw = W.shape
    K = Kw if K is None else K
    if out is None:
        out = torch.empty(M, N, device=X.device, dtype=torch.float16)
    _lib.call("gbsdf_dense", M, K, N, _lib.ptr(X), _lib.ptr(X_lo), X.stride(0), _lib.ptr(W.contiguous()),
              _lib.ptr(bias), _lib.ptr(G), G.stride(0) if G is not None else 0, _lib.ptr(out), _lib.ptr(out_lo),
              out.stride(0), 1 if out.dtype == torch.float32 else 0, int(epi), float(beta), _lib.ptr(err),
              _lib.stream_ptr(X.device))
    return out
