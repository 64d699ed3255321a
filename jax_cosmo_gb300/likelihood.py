"""Gaussian log-likelihood (jax_cosmo/likelihood.py:9-61).

The covariance of a Limber C_ell data vector is block diagonal after permuting
(cls, ell) -> (ell, cls).  libjcg factors the per-ell n_cls x n_cls blocks by
Cholesky in float64 (``jcg_gaussian_loglike_sparse`` / ``_dense``), which gives
the value of the reference's sparse path (inverse + Schur complements) and of
its dense path (inverse or Cholesky) up to rounding.  A dense matrix that is
not block diagonal in ell (a user covariance with ell-ell correlations) is
factored as a whole with torch.linalg.cholesky.

Sign convention kept from the reference: ``-0.5 * (r^T C^-1 r - logdet C)``
(likelihood.py:61), i.e. ``+0.5 logdet``.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from jax_cosmo_gb300 import _lib

__all__ = ["gaussian_log_likelihood"]


def _t(x, device):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float64)
    return torch.as_tensor(np.asarray(x, dtype=np.float64), device=device)


def _dense_n_ell(C):
    """ell count of a (cls, ell) x (cls, ell) dense covariance, from row 0."""
    hint = getattr(C, "_jcg_n_ell", None)
    if hint is not None:
        return int(hint)
    N = C.shape[-1]
    row = C.reshape(-1, N, N)[0, 0]
    nz = torch.nonzero(row).flatten().cpu().numpy()
    if nz.size >= 2 and nz[0] == 0 and N % int(nz[1]) == 0:
        return int(nz[1])
    return N


def _loglike_blocks(r_data, mu, C, n_cls, n_ell, include_logdet, dense, alpha=None):
    """libjcg per-ell block Cholesky; also writes alpha = C^-1 (mu - data) if given."""
    device = mu.device
    B = mu.shape[0]
    wsz = ctypes.c_size_t()
    _lib.call("jcg_loglike_workspace_size", B, n_cls, n_ell, ctypes.byref(wsz))
    ws = _lib.workspace(wsz.value, device)
    out = torch.empty(B, dtype=torch.float64, device=device)
    status = torch.zeros(B, dtype=torch.int32, device=device)
    name = "jcg_gaussian_loglike_dense" if dense else "jcg_gaussian_loglike_sparse"
    _lib.call(name, _lib.ptr(r_data), _lib.ptr(mu), _lib.ptr(C), B, n_cls, n_ell,
              1 if include_logdet else 0, _lib.ptr(out), _lib.ptr(status), _lib.ptr(alpha), _lib.ptr(ws),
              ctypes.c_size_t(ws.numel()), _lib.stream_of(device))
    return out, status


def _loglike_core(data2, mu2, Cb, sparse, n_cls, n_ell, include_logdet, alpha=None):
    """[B] log-likelihoods of prepared batched operands (and C^-1 r into ``alpha``).

    Returns (out, status); status 1 marks a dense matrix that is not block
    diagonal in ell, factored as a whole.
    """
    B, N = mu2.shape
    device = mu2.device
    if sparse:
        return _loglike_blocks(data2, mu2, Cb, n_cls, n_ell, include_logdet, dense=False, alpha=alpha)
    if n_cls <= 160:
        out, status = _loglike_blocks(data2, mu2, Cb, n_cls, n_ell, include_logdet, dense=True, alpha=alpha)
    else:
        out = torch.full((B,), float("nan"), dtype=torch.float64, device=device)
        status = torch.ones(B, dtype=torch.int32, device=device)
    unstructured = (status == 1).nonzero().flatten().tolist()
    for i in unstructured:
        # not block diagonal in ell: whole-matrix Cholesky
        L = torch.linalg.cholesky(Cb[i])
        r = mu2[i] - data2[i]
        y = torch.cholesky_solve(r[:, None], L)[:, 0]
        q = torch.dot(r, y)
        ld = 2.0 * torch.log(torch.diagonal(L)).sum()
        out[i] = -0.5 * (q - ld) if include_logdet else -0.5 * q
        if alpha is not None:
            alpha[i] = y
    return out, status


def _prepare(data, mu, C, device):
    mu_t = _t(mu, device)
    data_t = _t(data, device)
    C_t = _t(C, device)
    batched = mu_t.dim() == 2
    mu2 = mu_t if batched else mu_t[None]
    data2 = data_t.expand_as(mu2) if data_t.dim() == 1 else data_t
    B, N = mu2.shape
    sparse = C_t.dim() == (4 if batched else 3)
    Cb = C_t if batched else C_t[None]
    if sparse:
        n_cls, n_ell = Cb.shape[1], Cb.shape[3]
        if Cb.shape[2] != n_cls or n_cls * n_ell != N:
            raise ValueError(f"sparse covariance {tuple(C_t.shape)} does not match data length {N}")
    else:
        if Cb.shape[1:] != (N, N):
            raise ValueError(f"covariance {tuple(C_t.shape)} does not match data length {N}")
        n_ell = _dense_n_ell(C_t.detach())
        n_cls = N // n_ell
    return batched, data2, mu2, Cb, sparse, n_cls, n_ell


def gaussian_log_likelihood(data, mu, C, include_logdet=True, inverse_method="inverse"):
    """Log-likelihood of ``data`` under N(mu, C); batched if mu is 2-D.

    Differentiable (torch.autograd) in data, mu and C.
    """
    if inverse_method not in ("inverse", "cholesky"):
        raise NotImplementedError
    device = _lib.require_cuda()
    batched, data2, mu2, Cb, sparse, n_cls, n_ell = _prepare(data, mu, C, device)
    if any(isinstance(x, torch.Tensor) and x.requires_grad for x in (data, mu, C)):
        from jax_cosmo_gb300 import autodiff

        out = autodiff.loglike_autograd(data2, mu2, Cb, include_logdet, sparse, n_cls, n_ell)
    else:
        out, _ = _loglike_core(data2.contiguous(), mu2.contiguous(), Cb.contiguous(), sparse,
                               n_cls, n_ell, include_logdet)
    return out if batched else out[0]
