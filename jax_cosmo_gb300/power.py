"""Matter power spectra (jax_cosmo/power.py:14-272).

``linear_matter_power`` and ``nonlinear_matter_power`` / ``halofit``
(takahashi2012 or smith2003) run in libjcg at (k, a) points: sigma_8
normalisation by the reference's 7-level Romberg rule, the halofit non-linear
scale by the reference's sigma^2(R) table and interpolation rule, FP64.  The
transfer function is Eisenstein_Hu with type "eisenhu_osc" or "eisenhu"
(``functools.partial(Eisenstein_Hu, type="eisenhu")``).
"""
from __future__ import annotations

import functools

import torch

from jax_cosmo_gb300 import _lib, _points
from jax_cosmo_gb300 import transfer as tklib

__all__ = ["primordial_matter_power", "linear_matter_power", "nonlinear_matter_power", "halofit"]

_PRESCRIPTIONS = {"takahashi2012": _lib.PK_TAKAHASHI2012, "smith2003": _lib.PK_SMITH2003}


def primordial_matter_power(cosmo, k):
    """k^n_s (power.py:14-18)."""
    return torch.as_tensor(k, dtype=torch.float64) ** cosmo.n_s


def linear_matter_power(cosmo, k, a=1.0, transfer_fn=tklib.Eisenstein_Hu, **kwargs):
    """power.py:21-53"""
    if kwargs:
        transfer_fn = functools.partial(transfer_fn, **kwargs)
    bits = tklib.transfer_bits(transfer_fn)
    return _points.evaluate(cosmo, _lib.EVAL_PLIN | (bits << 8), a=a, k=k)


def halofit_parameters(cosmo, a, transfer_fn=tklib.Eisenstein_Hu):
    """(k_nl, n_eff, C) at scale factors a (power.py:86-141)."""
    bits = tklib.transfer_bits(transfer_fn) << 8
    return (
        _points.evaluate(cosmo, _lib.EVAL_KNL | bits, a=a),
        _points.evaluate(cosmo, _lib.EVAL_NEFF | bits, a=a),
        _points.evaluate(cosmo, _lib.EVAL_C | bits, a=a),
    )


def halofit(cosmo, k, a, transfer_fn=tklib.Eisenstein_Hu, prescription="takahashi2012"):
    """Non-linear power by halofit (power.py:144-262)."""
    if prescription not in _PRESCRIPTIONS:
        raise NotImplementedError(f"halofit prescription {prescription!r}")
    phys = tklib.transfer_bits(transfer_fn) | _PRESCRIPTIONS[prescription]
    return _points.evaluate(cosmo, _lib.EVAL_PNL | (phys << 8), a=a, k=k)


def nonlinear_matter_power(cosmo, k, a=1.0, transfer_fn=tklib.Eisenstein_Hu, nonlinear_fn=halofit):
    """power.py:265-272: nonlinear_fn(cosmo, k, a, transfer_fn=transfer_fn) for
    halofit (either prescription, via functools.partial) or linear_matter_power."""
    if nonlinear_fn is linear_matter_power:
        return linear_matter_power(cosmo, k, a, transfer_fn=transfer_fn)
    presc = tklib.partial_kw(nonlinear_fn, halofit, "prescription", "takahashi2012")
    if presc is None:
        raise NotImplementedError("nonlinear_fn must be power.halofit or power.linear_matter_power")
    return halofit(cosmo, k, a, transfer_fn=transfer_fn, prescription=presc)


def model_bits(nonlinear_fn):
    """libjcg power-model code of a nonlinear_fn (JCG_PK_*)."""
    if nonlinear_fn is linear_matter_power:
        return _lib.PK_LINEAR
    presc = tklib.partial_kw(nonlinear_fn, halofit, "prescription", "takahashi2012")
    if presc not in _PRESCRIPTIONS:
        raise NotImplementedError(
            "nonlinear_fn must be power.halofit (prescription 'takahashi2012' or 'smith2003') "
            "or power.linear_matter_power"
        )
    return _PRESCRIPTIONS[presc]
