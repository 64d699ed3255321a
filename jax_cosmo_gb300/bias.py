"""Galaxy bias models (jax_cosmo/bias.py:10-57).

The three models of the reference are on the accelerated path: libjcg
evaluates them per Limber node (the NumberCounts galaxy bias, probes.py:89-94,
and the WeakLensing NLA intrinsic-alignment bias, probes.py:113-117).  Their
parameters are constants of a request (gradients are taken with respect to the
Cosmology only).
"""
import torch

from jax_cosmo_gb300.jax_utils import container

__all__ = ["constant_linear_bias", "inverse_growth_linear_bias", "des_y1_ia_bias"]


def _z(z):
    return torch.as_tensor(z, dtype=torch.float64)


class constant_linear_bias(container):
    """Redshift-independent linear bias ``b`` (bias.py:10-22)."""

    def __call__(self, cosmo, z):
        z = _z(z)
        return self.params[0] * torch.ones_like(z)

    def spec(self):
        return (1, float(self.params[0]), 0.0, 0.0)


class inverse_growth_linear_bias(container):
    """Bias ``b / D(a)`` with D the growth factor (bias.py:25-39)."""

    def __call__(self, cosmo, z):
        from jax_cosmo_gb300 import background

        z = _z(z)
        return self.params[0] / background.growth_factor(cosmo, 1.0 / (1.0 + z))

    def spec(self):
        return (2, float(self.params[0]), 0.0, 0.0)


class des_y1_ia_bias(container):
    """DES Y1 intrinsic-alignment bias ``A ((1 + z) / (1 + z0))^eta`` (bias.py:42-57)."""

    def __call__(self, cosmo, z):
        A, eta, z0 = self.params
        return A * ((1.0 + _z(z)) / (1.0 + z0)) ** eta

    def spec(self):
        A, eta, z0 = self.params
        return (3, float(A), float(eta), float(z0))
