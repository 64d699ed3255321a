"""Eisenstein & Hu (1998) transfer function (jax_cosmo/transfer.py:10-156)."""
from __future__ import annotations

from jax_cosmo_gb300 import _lib, _points

__all__ = ["Eisenstein_Hu"]


def Eisenstein_Hu(cosmo, k, type="eisenhu_osc"):
    """T(k) with baryon oscillations (transfer.py:107-153), on the device."""
    if type != "eisenhu_osc":
        raise NotImplementedError("only type='eisenhu_osc' is accelerated")
    return _points.evaluate(cosmo, _lib.EVAL_TRANSFER, k=k)
