"""Eisenstein & Hu (1998) transfer function (jax_cosmo/transfer.py:10-156)."""
from __future__ import annotations

import functools

from jax_cosmo_gb300 import _lib, _points

__all__ = ["Eisenstein_Hu"]

_TYPES = {"eisenhu_osc": 0, "eisenhu": _lib.TF_NOWIGGLE}


def Eisenstein_Hu(cosmo, k, type="eisenhu_osc"):
    """T(k) on the device: "eisenhu_osc" with baryon oscillations
    (transfer.py:107-153) or "eisenhu", the zero-baryon fit (transfer.py:99-105)."""
    if type not in _TYPES:
        raise NotImplementedError(f"transfer type {type!r}")
    return _points.evaluate(cosmo, _lib.EVAL_TRANSFER | (_TYPES[type] << 8), k=k)


def partial_kw(fn, base, key, default):
    """``key`` of ``fn`` when fn is ``base`` or ``functools.partial(base, key=...)``, else None."""
    if fn is base:
        return default
    if isinstance(fn, functools.partial) and fn.func is base and not fn.args and set(fn.keywords) <= {key}:
        return fn.keywords.get(key, default)
    return None


def transfer_bits(transfer_fn):
    """libjcg physics bits of a transfer_fn: Eisenstein_Hu, or functools.partial
    of it with ``type``; anything else raises NotImplementedError."""
    t = partial_kw(transfer_fn, Eisenstein_Hu, "type", "eisenhu_osc")
    if t not in _TYPES:
        raise NotImplementedError("transfer_fn must be transfer.Eisenstein_Hu (type 'eisenhu_osc' or 'eisenhu')")
    return _TYPES[t]
