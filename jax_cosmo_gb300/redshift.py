"""Redshift distributions (jax_cosmo/redshift.py:15-171).

``smail_nz``'s parameters are passed to libjcg, which evaluates n(z) on the
Limber and lensing grids on the device.  Every other distribution (``fu_nz``,
``kde_nz``, ``systematic_shift`` and user subclasses of
``redshift_distribution`` whose ``pz_fn`` takes a torch tensor) is tabulated:
its ``pz_fn`` is evaluated with torch on the device at the exact points
libjcg lists (``jcg_geometry_nz_points``), and libjcg normalises it with
``simps(pz_fn, 0, zmax, 256)`` (redshift.py:27-31).  ``delta_nz`` single-plane
bins of WeakLensing probes take the reference's separate branch
(probes.py:53-64): the lensing ratio at the plane's redshift, no z' integral.
"""
from __future__ import annotations

import hashlib

import numpy as np
import torch

from jax_cosmo_gb300.jax_utils import container

steradian_to_arcmin2 = 11818102.86004228

__all__ = ["redshift_distribution", "smail_nz", "fu_nz", "delta_nz", "kde_nz", "systematic_shift"]


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

    def cache_key(self):
        """Identity of the tabulated n(z): class, parameters and configuration."""
        h = hashlib.sha1(type(self).__name__.encode())
        for p in self.params:
            if isinstance(p, redshift_distribution):
                h.update(repr(p.cache_key()).encode())
            elif isinstance(p, torch.Tensor):
                h.update(p.detach().cpu().numpy().astype(np.float64).tobytes())
            else:
                h.update(np.asarray(p, dtype=np.float64).tobytes())
        h.update(repr(sorted(self.config.items())).encode())
        return h.hexdigest()

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


class fu_nz(redshift_distribution):
    """Fu et al. (2008) n(z) ~ (z^a + z^(a b)) / (z^b + c) (redshift.py:80-105)."""

    def pz_fn(self, z):
        a, b, c = self.params
        return (z**a + z ** (a * b)) / (z**b + c)


class delta_nz(redshift_distribution):
    """Single plane at z0 (redshift.py:108-122); WeakLensing bins only on the accelerated path."""

    def __init__(self, *args, **kwargs):
        super(delta_nz, self).__init__(*args, **kwargs)
        self._norm = torch.tensor(1.0, dtype=torch.float64)

    def pz_fn(self, z):
        z0 = self.params[0]
        return torch.where(z == z0, 1.0, 0.0).to(torch.float64)


class kde_nz(redshift_distribution):
    """Gaussian KDE of a weighted redshift catalog, bandwidth ``bw`` (redshift.py:125-156).

    pz_fn(z) = sum_i w_i N(z; z_i, bw) / sum_i w_i, evaluated on the device in
    chunks of points.
    """

    def _kernel(self, bw, X, x):
        return (1.0 / np.sqrt(2 * np.pi) / bw) * torch.exp(-((X - x) ** 2) / (bw**2 * 2.0))

    def pz_fn(self, z):
        zcat, weight = self.params[:2]
        z = torch.as_tensor(z, dtype=torch.float64)
        X = torch.as_tensor(zcat, dtype=torch.float64).to(z.device).reshape(-1)
        w = torch.atleast_1d(torch.as_tensor(weight, dtype=torch.float64)).to(z.device)
        q = torch.sum(w)
        zf = z.reshape(-1)
        out = torch.empty_like(zf)
        step = max(1, (1 << 25) // max(1, X.shape[0]))
        for s0 in range(0, zf.numel(), step):
            k = self._kernel(self.config["bw"], X[:, None], zf[None, s0 : s0 + step])
            out[s0 : s0 + step] = (k * w[:, None]).sum(0) / q
        return out.reshape(z.shape)


class systematic_shift(redshift_distribution):
    """A parent distribution shifted by a mean bias: pz_fn(clip(z - bias, 0)) (redshift.py:159-171)."""

    def pz_fn(self, z):
        parent_pz, bias = self.params[:2]
        return parent_pz.pz_fn(torch.clamp(z - bias, min=0.0))
