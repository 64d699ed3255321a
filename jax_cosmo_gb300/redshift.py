"""Redshift distributions (jax_cosmo/redshift.py:15-77).

``smail_nz`` is the distribution on the accelerated path: its parameters are
passed to libjcg, which builds n(z) on the Limber and lensing grids on the
device (normalised by ``simps(pz_fn, 0, zmax, 256)``, redshift.py:27-31).
``__call__`` evaluates the normalised n(z) with torch for host-side use.
"""
from __future__ import annotations

import numpy as np
import torch

from jax_cosmo_gb300.jax_utils import container

steradian_to_arcmin2 = 11818102.86004228

__all__ = ["smail_nz", "redshift_distribution"]


def _simps(f, a, b, N):
    # scipy/integrate.py:162-199
    if N % 2 == 1:
        raise ValueError("N must be an even integer.")
    x = torch.as_tensor(np.linspace(a, b, N + 1), dtype=torch.float64)
    y = f(x)
    return (b - a) / N / 3 * torch.sum(y[0:-1:2] + 4 * y[1::2] + y[2::2], dim=0)


class redshift_distribution(container):
    def __init__(self, *args, gals_per_arcmin2=1.0, zmax=10.0, **kwargs):
        self._norm = None
        self._gals_per_arcmin2 = gals_per_arcmin2
        super(redshift_distribution, self).__init__(*args, zmax=zmax, **kwargs)

    def pz_fn(self, z):
        raise NotImplementedError

    def __call__(self, z):
        z = torch.as_tensor(z, dtype=torch.float64)
        if self._norm is None:
            self._norm = _simps(lambda t: self.pz_fn(t), 0.0, self.config["zmax"], 256)
        return self.pz_fn(z) / self._norm.to(z.device)

    @property
    def zmax(self):
        return self.config["zmax"]

    @property
    def gals_per_arcmin2(self):
        return self._gals_per_arcmin2

    @property
    def gals_per_steradian(self):
        return self._gals_per_arcmin2 * steradian_to_arcmin2

    def tree_flatten(self):
        return ((self.params, self._gals_per_arcmin2), self.config)

    @classmethod
    def tree_unflatten(cls, aux_data, children):
        args, gals_per_arcmin2 = children
        return cls(*args, gals_per_arcmin2=gals_per_arcmin2, **aux_data)


class smail_nz(redshift_distribution):
    """Smail distribution n(z) ~ z^a exp(-(z / z0)^b) (redshift.py:61-77).

    Parameters: a, b, z0; gals_per_arcmin2; zmax (default 10).
    """

    def pz_fn(self, z):
        a, b, z0 = self.params
        return z**a * torch.exp(-((z / z0) ** b))

    def device_params(self):
        a, b, z0 = self.params
        return float(a), float(b), float(z0), float(self.zmax)
