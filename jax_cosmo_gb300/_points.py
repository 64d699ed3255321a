"""Pointwise evaluation of the table functions through ``jcg_eval_points``."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from jax_cosmo_gb300 import _lib


def _vec(x, device):
    if x is None:
        return None
    if isinstance(x, torch.Tensor):
        t = x.detach().to(device=device, dtype=torch.float64)
    else:
        t = torch.as_tensor(np.asarray(x, dtype=np.float64), device=device)
    return torch.atleast_1d(t).reshape(-1).contiguous()


def evaluate(cosmo, what, a=None, k=None):
    """Returns [n] (single cosmology) or [B, n] of the quantity ``what``."""
    device = _lib.require_cuda()
    params = cosmo.param_tensor(device)
    B = params.shape[0]
    a_t, k_t = _vec(a, device), _vec(k, device)
    if a_t is not None and k_t is not None and a_t.numel() != k_t.numel():
        if a_t.numel() == 1:
            a_t = a_t.expand(k_t.numel()).contiguous()
        elif k_t.numel() == 1:
            k_t = k_t.expand(a_t.numel()).contiguous()
        else:
            raise ValueError("k and a must broadcast")
    n = (a_t if a_t is not None else k_t).numel()
    wsz = ctypes.c_size_t()
    _lib.call("jcg_eval_workspace_size", B, ctypes.byref(wsz))
    ws = _lib.workspace(wsz.value, device)
    out = torch.empty(B, n, dtype=torch.float64, device=device)
    what = what | (cosmo.physics_bits() << 8)
    _lib.call("jcg_eval_points", _lib.ptr(params), B, _lib.ptr(a_t), _lib.ptr(k_t), n, what,
              _lib.ptr(out), _lib.ptr(ws), ctypes.c_size_t(ws.numel()), _lib.stream_of(device))
    return out if cosmo.batch_size is not None else out[0]
