"""Block-diagonal ("sparse") matrices (jax_cosmo/sparse.py).

Format (sparse.py:1-11): a 3-D array (ny, nx, ndiag) of ny x nx square blocks,
each diagonal, the vector at [i, j] being the diagonal of block (i, j).
``inv``, ``slogdet``, ``to_dense`` and every product of ``dot`` (matrix-vector,
sparse-dense, dense-sparse, sparse-sparse and the bilinear form) run in
libjcg (FP64).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from jax_cosmo_gb300 import _lib

__all__ = ["is_sparse", "check_sparse", "to_dense", "dot", "inv", "inv_batched", "slogdet", "det"]
MAX_N = 160  # JCG_SPARSE_MAX_N: block size limit of inv / slogdet


def _t(x):
    device = _lib.require_cuda()
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.asarray(x, dtype=np.float64), device=device).contiguous()


def is_sparse(sparse):
    """sparse.py:37-39"""
    return np.ndim(sparse) == 3 if not isinstance(sparse, torch.Tensor) else sparse.dim() == 3


def check_sparse(sparse, square=False):
    """sparse.py:42-49"""
    if not is_sparse(sparse):
        raise ValueError("Expected 3D array of sparse diagonals.")
    sparse = _t(sparse)
    if square and (sparse.shape[0] != sparse.shape[1]):
        raise ValueError("Expected a square matrix.")
    return sparse


def to_dense(sparse):
    """(a, b, ndiag) -> (a ndiag, b ndiag) (sparse.py:52-68)."""
    sp = check_sparse(sparse)
    n, m, nd = sp.shape
    out = torch.empty(n * nd, m * nd, dtype=torch.float64, device=sp.device)
    _lib.call("jcg_sparse_to_dense", _lib.ptr(sp), n, m, nd, _lib.ptr(out), _lib.stream_of(sp.device))
    return out


def _vec_dot(sp, v, transpose):
    n, m, nd = sp.shape
    rows = (m if transpose else n) * nd
    out = torch.empty(rows, dtype=torch.float64, device=sp.device)
    _lib.call("jcg_sparse_dot_vec", _lib.ptr(sp), n, m, nd, _lib.ptr(v.contiguous()),
              1 if transpose else 0, _lib.ptr(out), _lib.stream_of(sp.device))
    return out


def sparse_dot_vec(sparse, vec):
    return _vec_dot(_t(sparse), _t(vec), False)


def vec_dot_sparse(vec, sparse):
    return _vec_dot(_t(sparse), _t(vec), True)


def sparse_dot_dense(sparse, dense):
    """A @ D, A sparse (n, m, nd), D dense (m nd, k) -> (n nd, k) (sparse.py:164-182)."""
    sp, d = _t(sparse), _t(dense)
    n, m, nd = sp.shape
    d2 = d.reshape(m * nd, -1)
    out = torch.empty(n * nd, d2.shape[1], dtype=torch.float64, device=sp.device)
    _lib.call("jcg_sparse_dot_dense", _lib.ptr(sp), n, m, nd, _lib.ptr(d2), d2.shape[1], _lib.ptr(out),
              _lib.stream_of(sp.device))
    return out


def dense_dot_sparse(dense, sparse):
    """D @ A, D dense (r, n nd), A sparse (n, m, nd) -> (r, m nd) (sparse.py:210-233)."""
    sp, d = _t(sparse), _t(dense)
    n, m, nd = sp.shape
    d2 = d.reshape(-1, n * nd)
    out = torch.empty(d2.shape[0], m * nd, dtype=torch.float64, device=sp.device)
    _lib.call("jcg_dense_dot_sparse", _lib.ptr(d2), d2.shape[0], _lib.ptr(sp), n, m, nd, _lib.ptr(out),
              _lib.stream_of(sp.device))
    return out


def sparse_dot_sparse(sparse1, sparse2):
    """A @ B, both sparse: (n, m, nd) @ (m, p, nd) -> (n, p, nd) (sparse.py:236-260)."""
    a, b = _t(sparse1), _t(sparse2)
    n, m, nd = a.shape
    p = b.shape[1]
    out = torch.empty(n, p, nd, dtype=torch.float64, device=a.device)
    _lib.call("jcg_sparse_dot_sparse", _lib.ptr(a), n, m, p, nd, _lib.ptr(b), _lib.ptr(out),
              _lib.stream_of(a.device))
    return out


def dense_dot_sparse_dot_dense(X, Y, Z):
    """Bilinear form X @ Y @ Z with Y sparse (sparse.py:263-292)."""
    x, y, z = _t(X), _t(Y), _t(Z)
    n, m, nd = y.shape
    k = z.shape[1]
    work = torch.empty(n * nd, k, dtype=torch.float64, device=y.device)
    out = torch.empty(x.shape[0], k, dtype=torch.float64, device=y.device)
    _lib.call("jcg_dense_dot_sparse_dot_dense", _lib.ptr(x), x.shape[0], _lib.ptr(y), n, m, nd, _lib.ptr(z), k,
              _lib.ptr(work), _lib.ptr(out), _lib.stream_of(y.device))
    return out


def dot(*args):
    """A @ B (or A @ B @ C) with at least one sparse operand (sparse.py:71-137)."""
    if len(args) == 2:
        A, B = args
        a_sp, b_sp = is_sparse(A), is_sparse(B)
        A, B = _t(A), _t(B)
        Acols = A.shape[1] * A.shape[2] if a_sp else A.shape[-1]
        if not a_sp and not (1 <= A.dim() <= 2):
            raise ValueError(f"A has invalid dimension {A.dim()} (expected 1 or 2).")
        if not b_sp and not (1 <= B.dim() <= 2):
            raise ValueError(f"B has invalid dimension {B.dim()} (expected 1 or 2).")
        Brows = B.shape[0] * B.shape[2] if b_sp else B.shape[0]
        if Acols != Brows:
            raise ValueError(f"Shapes of A {tuple(A.shape)} and B {tuple(B.shape)} not compatible for dot product.")
        if a_sp and b_sp:
            return sparse_dot_sparse(A, B)
        if a_sp:
            return _vec_dot(A, B, False) if B.dim() == 1 else sparse_dot_dense(A, B)
        return _vec_dot(B, A, True) if A.dim() == 1 else dense_dot_sparse(A, B)
    if len(args) == 3:
        A, B, C = (_t(x) for x in args)
        if A.dim() != 2 or B.dim() != 3 or C.dim() != 2:
            raise ValueError("Can only handle dense @ sparse @ dense bilinear form.")
        if A.shape[1] != B.shape[0] * B.shape[2] or B.shape[1] * B.shape[2] != C.shape[0]:
            raise ValueError("Shapes not compatible for dot product.")
        return dense_dot_sparse_dot_dense(A, B, C)
    raise ValueError(f"Expected 2 or 3 input arrays but got {len(args)}.")


def inv(sparse):
    """Per-diagonal inverse (sparse.py:295-315)."""
    sp = check_sparse(sparse, square=True)
    n, _, nd = sp.shape
    out = torch.empty_like(sp)
    _lib.call("jcg_sparse_inv", _lib.ptr(sp), n, nd, _lib.ptr(out), _lib.stream_of(sp.device))
    return out


def inv_batched(sparse):
    """``inv`` of a stack [B, n, n, nd] of sparse matrices in one launch."""
    sp = _t(sparse)
    if sp.dim() != 4 or sp.shape[1] != sp.shape[2]:
        raise ValueError(f"expected [B, n, n, ndiag], got {tuple(sp.shape)}")
    B, n, _, nd = sp.shape
    out = torch.empty_like(sp)
    _lib.call("jcg_sparse_inv_batched", _lib.ptr(sp), B, n, nd, _lib.ptr(out), _lib.stream_of(sp.device))
    return out


def slogdet(sparse):
    """(sign, log|det|) (sparse.py:334-366)."""
    sp = check_sparse(sparse, square=True)
    n, _, nd = sp.shape
    sign = torch.empty((), dtype=torch.float64, device=sp.device)
    logdet = torch.empty((), dtype=torch.float64, device=sp.device)
    work = torch.empty(2 * nd, dtype=torch.float64, device=sp.device)
    _lib.call("jcg_sparse_slogdet", _lib.ptr(sp), n, nd, _lib.ptr(sign), _lib.ptr(logdet),
              _lib.ptr(work), _lib.stream_of(sp.device))
    return sign, logdet


def det(sparse):
    """sparse.py:369-389"""
    sign, logdet = slogdet(sparse)
    return sign * torch.exp(logdet)
