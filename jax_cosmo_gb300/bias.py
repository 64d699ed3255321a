"""Galaxy bias models (jax_cosmo/bias.py:10-22).

Only ``constant_linear_bias`` is on the accelerated path; the bias value is
passed to the NumberCounts kernel of libjcg.
"""
from jax_cosmo_gb300.jax_utils import container

__all__ = ["constant_linear_bias"]


class constant_linear_bias(container):
    """Redshift-independent linear bias ``b`` (bias.py:10-22)."""

    def __call__(self, cosmo, z):
        import torch

        b = self.params[0]
        z = torch.as_tensor(z, dtype=torch.float64)
        return b * torch.ones_like(z)
