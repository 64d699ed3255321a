"""Tracer probes (jax_cosmo/probes.py:132-281).

``WeakLensing`` and ``NumberCounts`` keep the reference's constructor, pytree
split and ``n_tracers`` / ``zmax`` / ``noise`` / ``kernel`` methods.  Their radial
kernels are computed by libjcg (FP64): the lensing efficiency integral of
probes.py:16-74 and the density kernel of probes.py:77-99.

Intrinsic alignment (``ia_bias``: the NLA model of probes.py:102-129, added to
the shear kernel before the multiplicative bias, probes.py:200-207) and the
three bias models of bias.py are on the accelerated path.  Not on it (they
raise NotImplementedError): ``delta_nz`` bins (probes.py:53-64) and non-Smail
n(z).
"""
from __future__ import annotations

import numpy as np
import torch

from jax_cosmo_gb300.jax_utils import container

__all__ = ["WeakLensing", "NumberCounts"]


def _bias_specs(bias, n):
    """Bias specs of n bins from one bias object or a list (probes.py:89-93)."""
    from jax_cosmo_gb300.bias import constant_linear_bias, des_y1_ia_bias, inverse_growth_linear_bias

    blist = bias if isinstance(bias, list) else [bias] * n
    if len(blist) != n:
        raise ValueError(f"{len(blist)} biases for {n} redshift bins")
    out = []
    for b in blist:
        if not isinstance(b, (constant_linear_bias, inverse_growth_linear_bias, des_y1_ia_bias)):
            raise NotImplementedError(f"bias model {type(b).__name__} is not on the accelerated path")
        out.append(b.spec())
    return out


class WeakLensing(container):
    """Weak lensing probe with a list of redshift bins (probes.py:132-223)."""

    def __init__(self, redshift_bins, ia_bias=None, multiplicative_bias=0.0, sigma_e=0.26, **kwargs):
        if ia_bias is None:
            ia_enabled = False
            args = (redshift_bins, multiplicative_bias)
        else:
            ia_enabled = True
            args = (redshift_bins, multiplicative_bias, ia_bias)
        if "ia_enabled" not in kwargs.keys():
            kwargs["ia_enabled"] = ia_enabled
        super(WeakLensing, self).__init__(*args, sigma_e=sigma_e, **kwargs)

    @property
    def n_tracers(self):
        return len(self.params[0])

    @property
    def zmax(self):
        return max([pz.zmax for pz in self.params[0]])

    def ia_specs(self):
        """(kind, amplitude, eta, z0) of each bin's NLA bias; kind 0 without IA."""
        if not self.config.get("ia_enabled", False):
            return [(0, 0.0, 0.0, 0.0)] * self.n_tracers
        return _bias_specs(self.params[2], self.n_tracers)

    def multiplicative_biases(self):
        m = self.params[1]
        if isinstance(m, (list, tuple)):
            return [float(x) for x in m]
        return [float(m)] * self.n_tracers

    def kernel(self, cosmo, z, ell):
        """Radial kernel of every bin at redshifts z, shape (nbins, nz) (probes.py:188-208)."""
        from jax_cosmo_gb300 import _geometry

        return _geometry.probe_kernel(self, cosmo, z, ell)

    def noise(self):
        """sigma_e^2 / n_gal per bin (probes.py:210-223)."""
        pzs = self.params[0]
        ngals = np.array([pz.gals_per_steradian for pz in pzs])
        if isinstance(self.config["sigma_e"], list):
            sigma_e = np.array([s for s in self.config["sigma_e"]])
        else:
            sigma_e = self.config["sigma_e"]
        return torch.as_tensor(sigma_e**2 / ngals, dtype=torch.float64)


class NumberCounts(container):
    """Galaxy clustering probe with a list of redshift bins (probes.py:226-281)."""

    def __init__(self, redshift_bins, bias, has_rsd=False, **kwargs):
        super(NumberCounts, self).__init__(redshift_bins, bias, has_rsd=has_rsd, **kwargs)

    @property
    def zmax(self):
        return max([pz.zmax for pz in self.params[0]])

    @property
    def n_tracers(self):
        return len(self.params[0])

    def bias_specs(self):
        """(kind, amplitude, eta, z0) of each bin's galaxy bias."""
        return _bias_specs(self.params[1], self.n_tracers)

    def kernel(self, cosmo, z, ell):
        """n(z) b(z) H(z) per bin, shape (nbins, nz) (probes.py:260-272)."""
        from jax_cosmo_gb300 import _geometry

        return _geometry.probe_kernel(self, cosmo, z, ell)

    def noise(self):
        """1 / n_gal per bin (probes.py:274-281)."""
        ngals = np.array([pz.gals_per_steradian for pz in self.params[0]])
        return torch.as_tensor(1.0 / ngals, dtype=torch.float64)
