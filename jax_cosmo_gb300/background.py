"""Background cosmology (jax_cosmo/background.py:25-512).

``radial_comoving_distance``, ``a_of_chi``, ``transverse_comoving_distance``,
``angular_diameter_distance``, ``growth_factor``, ``growth_rate``, ``H`` and
``dchioverda`` run in libjcg (FP64 RK4 tables on the reference's grids, then
the reference's interpolation rule).  The closed forms ``w``, ``f_de``, ``Esqr``, ``Omega_m_a``,
``Omega_de_a`` are one-line expressions evaluated with torch on the parameters'
device; the accelerated path evaluates them inside its kernels.
"""
from __future__ import annotations

import torch

from jax_cosmo_gb300 import _lib, _points

__all__ = ["w", "f_de", "Esqr", "H", "Omega_m_a", "Omega_de_a", "radial_comoving_distance",
           "a_of_chi", "dchioverda", "transverse_comoving_distance", "angular_diameter_distance",
           "growth_factor", "growth_rate"]


def _a(a):
    return torch.as_tensor(a, dtype=torch.float64)


def w(cosmo, a):
    """Linder w(a) = w0 + (1 - a) wa (background.py:25-53)."""
    return cosmo.w0 + (1.0 - _a(a)) * cosmo.wa


def f_de(cosmo, a):
    """background.py:56-90"""
    a = _a(a)
    return -3.0 * (1.0 + cosmo.w0 + cosmo.wa) * torch.log(a) + 3.0 * cosmo.wa * (a - 1.0)


def Esqr(cosmo, a):
    """background.py:93-126"""
    a = _a(a)
    return (cosmo.Omega_m * torch.pow(a, -3) + cosmo.Omega_k * torch.pow(a, -2)
            + cosmo.Omega_de * torch.exp(f_de(cosmo, a)))


def Omega_m_a(cosmo, a):
    """background.py:145-168"""
    a = _a(a)
    return cosmo.Omega_m * torch.pow(a, -3) / Esqr(cosmo, a)


def Omega_de_a(cosmo, a):
    """background.py:171-196"""
    a = _a(a)
    return cosmo.Omega_de * torch.exp(f_de(cosmo, a)) / Esqr(cosmo, a)


def H(cosmo, a):
    """Hubble parameter [km/s/(Mpc/h)] (background.py:129-142)."""
    return _points.evaluate(cosmo, _lib.EVAL_H, a=a)


def dchioverda(cosmo, a):
    """background.py:270-294"""
    return _points.evaluate(cosmo, _lib.EVAL_DCHI, a=a)


def radial_comoving_distance(cosmo, a, log10_amin=-3, steps=256):
    """Radial comoving distance [Mpc/h] (background.py:199-242)."""
    if (log10_amin, steps) != (-3, 256):
        raise NotImplementedError("the chi table uses the reference grid logspace(-3, 0, 256)")
    return _points.evaluate(cosmo, _lib.EVAL_CHI, a=a)


def growth_factor(cosmo, a):
    """Linear growth factor D(a), D(1) = 1: the growth ODE (background.py:371-398,
    443-488), or with a Cosmology gamma the integral of Omega_m(a)^gamma
    (background.py:515-552)."""
    return _points.evaluate(cosmo, _lib.EVAL_GROWTH, a=a)


def a_of_chi(cosmo, chi):
    """Scale factor at radial comoving distance chi [Mpc/h], by the reference's
    interpolation of the chi table (background.py:245-267)."""
    return _points.evaluate(cosmo, _lib.EVAL_A_OF_CHI, a=chi)


def transverse_comoving_distance(cosmo, a):
    """f_k(a) [Mpc/h]: chi for Omega_k = 0, R_H / sqrt|Omega_k| sinh / sin of
    sqrt|Omega_k| chi / R_H for open / closed universes (background.py:297-344)."""
    return _points.evaluate(cosmo, _lib.EVAL_TRANSVERSE, a=a)


def angular_diameter_distance(cosmo, a):
    """d_A(a) = a f_k(a) [Mpc/h] (background.py:347-368)."""
    return _points.evaluate(cosmo, _lib.EVAL_DA, a=a)


def growth_rate(cosmo, a):
    """Growth rate dlnD/dlna from the growth ODE table (background.py:401-440, 491-512),
    or Omega_m(a)^gamma with a Cosmology gamma (background.py:555-582)."""
    return _points.evaluate(cosmo, _lib.EVAL_GROWTH_RATE, a=a)
