"""Matter power spectra (jax_cosmo/power.py:14-272).

``linear_matter_power`` and ``nonlinear_matter_power`` / ``halofit``
(takahashi2012) run in libjcg at (k, a) points: sigma_8 normalisation by the
reference's 7-level Romberg rule, the halofit non-linear scale by the
reference's sigma^2(R) table and interpolation rule, FP64.
"""
from __future__ import annotations

import torch

from jax_cosmo_gb300 import _lib, _points
from jax_cosmo_gb300 import transfer as tklib

__all__ = ["primordial_matter_power", "linear_matter_power", "nonlinear_matter_power", "halofit"]


def primordial_matter_power(cosmo, k):
    """k^n_s (power.py:14-18)."""
    return torch.as_tensor(k, dtype=torch.float64) ** cosmo.n_s


def linear_matter_power(cosmo, k, a=1.0, transfer_fn=tklib.Eisenstein_Hu, **kwargs):
    """power.py:21-53"""
    if transfer_fn is not tklib.Eisenstein_Hu or kwargs:
        raise NotImplementedError("only the default Eisenstein_Hu transfer is accelerated")
    return _points.evaluate(cosmo, _lib.EVAL_PLIN, a=a, k=k)


def halofit_parameters(cosmo, a):
    """(k_nl, n_eff, C) at scale factors a (power.py:86-141)."""
    return (
        _points.evaluate(cosmo, _lib.EVAL_KNL, a=a),
        _points.evaluate(cosmo, _lib.EVAL_NEFF, a=a),
        _points.evaluate(cosmo, _lib.EVAL_C, a=a),
    )


def halofit(cosmo, k, a, transfer_fn=tklib.Eisenstein_Hu, prescription="takahashi2012"):
    """Non-linear power by halofit (power.py:144-262)."""
    if prescription != "takahashi2012":
        raise NotImplementedError("only prescription='takahashi2012' is accelerated")
    if transfer_fn is not tklib.Eisenstein_Hu:
        raise NotImplementedError("only the default Eisenstein_Hu transfer is accelerated")
    return _points.evaluate(cosmo, _lib.EVAL_PNL, a=a, k=k)


def nonlinear_matter_power(cosmo, k, a=1.0, transfer_fn=tklib.Eisenstein_Hu, nonlinear_fn=halofit):
    """power.py:265-272"""
    if nonlinear_fn is not halofit:
        raise NotImplementedError("only halofit is accelerated")
    return halofit(cosmo, k, a, transfer_fn=transfer_fn)
